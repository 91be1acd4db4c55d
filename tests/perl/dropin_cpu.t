#!/usr/bin/env perl
# PDL::GB300 against the reference PDL itself, on the CPU (no GPU needed):
# the descriptor of every kind of view, the shapes/types/error text of the
# library's planner against PDL's own ops, explicit broadcast ids refused,
# and install() routing PDL's subs and operators to the module.
use strict;
use warnings;
use Test::More;
use PDL;
use PDL::GB300;

# --- descriptors: a view of a sequence() parent holds, at each index, its
# own physical flat index, so offs + sum(idx * incs) must equal the value
my $par = sequence(5, 4, 3);
my @views = (
  [$par, 'whole'],
  [$par->slice('1:3,(2)'), 'slice with a dropped dim'],
  [$par->slice('-1:0,:,1'), 'reversed dim'],
  [$par->xchg(0, 2), 'xchg'],
  [$par->mv(2, 0), 'mv'],
  [$par->slice(':,1')->dummy(1, 4), 'dummy'],
  [$par->slice('0:4:2,1:3'), 'stride 2'],
  [$par->clump(2), 'clump'],
);
for my $v (@views) {
  my ($x, $what) = @$v;
  my ($type, $offs, $state, $hb, $dims, $incs) = PDL::GB300::_desc($x);
  is_deeply($dims, [$x->dims], "$what: dims");
  is($type, $x->get_datatype, "$what: type");
  my $ok = 1;
  my $n = $x->nelem;
  for my $flat (0 .. $n - 1) {
    my @idx = map { ref $_ ? $_->sclr : $_ } $x->one2nd($flat);
    my $p = $offs;
    $p += $idx[$_] * $incs->[$_] for 0 .. $#idx;
    $ok &&= $x->at(@idx) == $p;
  }
  ok($ok, "$what: offs + sum(idx * incs) addresses every element");
}
{
  my $b = sequence(4)->long;
  $b->badflag(1);
  $b->badvalue(2);
  my (undef, undef, $state, $hb) = PDL::GB300::_desc($b);
  is($state & 1, 1, 'badflag carried');
  is($hb, 1, 'per-ndarray badvalue carried');
}

# --- the planner: output dims and types equal PDL's own, error text equal
my @reduce = @PDL::GB300::REDUCE;
my @biop = @PDL::GB300::BIOP;
my @types = (byte, short, long, longlong, float, double);
my @shapes = ([7], [4, 3], [2, 3, 4], [1, 5]);
my ($nplan, $nok) = (0, 0);
for my $op (@reduce) {
  next if $op =~ /^(bandover|borover|bxorover)$/;    # integer types only, below
  for my $t (@types) {
    for my $s (@shapes) {
      my $a = ones($t, @$s);
      my $want = eval { no strict 'refs'; &{"PDL::$op"}($a) };
      next unless defined $want;
      my ($type, $dims) = PDL::GB300::_redodims($op, [$a, PDL->null], 0);
      $nplan++;
      $nok++ if $type == $want->get_datatype && "@$dims" eq join(' ', $want->dims);
    }
  }
}
for my $op (@biop) {
  for my $ta (byte, long, float, double) {
    for my $tb (short, longlong, double) {
      next if $op =~ /^(shiftleft|shiftright|or2|and2|xor)$/ && ($ta->enum > 8 || $tb->enum > 8);
      for my $p ([[3], [3]], [[4, 1], [1, 5]], [[2, 3, 1], [3, 1]]) {
        my ($a, $b) = (ones($ta, @{$p->[0]}), ones($tb, @{$p->[1]}));
        my $want = eval { no strict 'refs'; &{"PDL::$op"}($a, $b) };
        next unless defined $want;
        my ($type, $dims) = PDL::GB300::_redodims($op, [$a, $b, PDL->null], 0);
        $nplan++;
        $nok++ if $type == $want->get_datatype && "@$dims" eq join(' ', $want->dims);
      }
    }
  }
}
for my $p ([[3, 4], [3, 1]], [[5, 2, 3], [5, 1, 3]]) {
  my ($a, $b) = (sequence(@{$p->[0]}), sequence(@{$p->[1]}));
  my $want = inner($a, $b);
  my ($type, $dims) = PDL::GB300::_redodims('inner', [$a, $b, PDL->null], 0);
  $nplan++;
  $nok++ if $type == $want->get_datatype && "@$dims" eq join(' ', $want->dims);
}
ok($nplan > 400, "planner cases: $nplan");
is($nok, $nplan, 'output dims and types equal PDL\'s own');

for my $case (
  ['plus', [zeroes(4, 3), zeroes(5), PDL->null], sub { PDL::plus(zeroes(4, 3), zeroes(5)) }],
  ['sumover', [zeroes(4, 2), zeroes(3)], sub { sumover(zeroes(4, 2), zeroes(3)) }],
  ['inner', [zeroes(4, 2), zeroes(4, 3), PDL->null], sub { inner(zeroes(4, 2), zeroes(4, 3)) }],
  ['minimum_ind', [zeroes(4, 2), zeroes(3)], sub { minimum_ind(zeroes(4, 2), zeroes(3)) }],
) {
  my ($op, $pdls, $ref) = @$case;
  eval { $ref->() };
  (my $want = $@) =~ s/ at \S+ line \d+.*//s;
  eval { PDL::GB300::_redodims($op, $pdls, 0) };
  (my $got = $@) =~ s/ at \S+ line \d+.*//s;
  $want =~ s/\s+$//;
  $got =~ s/\s+$//;
  is($got, $want, "$op: the error text is PDL's");
}
{
  my $x = $par->copy;
  eval { PDL::GB300::_desc($x->broadcast(1)) };
  like($@, qr/explicit broadcast ids/, 'explicit broadcast ids refused');
}

# --- install(): PDL's subs and operators reach the module
PDL::GB300::install();
{
  no strict 'refs';
  is(\&{'PDL::sumover'}, \&PDL::GB300::sumover, 'PDL::sumover is the module\'s');
  is(\&{'PDL::plus'}, \&PDL::GB300::plus, 'PDL::plus is the module\'s');
}
if (PDL::GB300::device_count() == 0) {
  # no GPU here: the op gets to the library, which reports that
  for my $c (['sumover', sub { sequence(5)->sumover }], ['+', sub { sequence(5) + 1 }],
             ['x', sub { sequence(3, 3) x sequence(3, 3) }]) {
    eval { $c->[1]->() };
    like($@, qr/CUDA|device/i, "$c->[0] runs through libpdlgb300 (no GPU here)");
  }
}
PDL::GB300::uninstall();
{
  no strict 'refs';
  isnt(\&{'PDL::sumover'}, \&PDL::GB300::sumover, 'uninstall restores PDL\'s subs');
}
done_testing();
