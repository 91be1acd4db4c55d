package PDL::GB300;

# The PDL ops of this library's path run on the GB300: the same names,
# arguments and results as PDL's own (lib/PDL/Ufunc.pd, lib/PDL/Ops.pd,
# lib/PDL/Primitive.pd), with host data staged to the GPU per call.
#
#   use PDL; use PDL::GB300;
#   PDL::GB300::install();            # PDL::sumover, PDL::plus, ... and the
#                                     # operators (+ * x ...) now run here
#   my $g = PDL::GB300::sumover_bwd($gb, $a);   # hand-written adjoints
#
# install() replaces the subs in package PDL; PDL's operator overloads call
# those subs by name, so `$a + $b` and `$a x $b` reach this module too.

use strict;
use warnings;
use PDL::Core ();
use Scalar::Util ();
require DynaLoader;
our @ISA = ('DynaLoader');
our $VERSION = '0.2';
bootstrap PDL::GB300 $VERSION;

our %saved;    # PDL's own subs, kept by install()

# a(n); [o]b() reductions over dim 0, and the one-input sort-based functions
# (a(n) or a(n,m) in, one output)
our @REDUCE = qw(sumover dsumover prodover dprodover average daverage minimum maximum
                 minimum_ind maximum_ind cumusumover dcumusumover cumuprodover dcumuprodover
                 andover orover xorover zcover bandover borover bxorover firstnonzeroover
                 qsort qsorti medover oddmedover modeover qsortvec qsortveci);
# Inplace => 1 among them (lib/PDL/Ufunc.pd:1042,1117)
my %INPLACE = map { $_ => 1 } qw(qsort qsortvec);
# a(n); p(); [o]b()
our @PCT = qw(pctover oddpctover);
# a(); b(); [o]c(); OtherPars swap
our @BIOP = qw(plus mult minus divide gt lt le ge eq ne shiftleft shiftright or2 and2 xor);
my %CMP = map { $_ => 1 } qw(gt lt le ge eq ne);    # Comparison ops (Ops.pd:297-302)

sub _is_pdl { UNIVERSAL::isa($_[0], 'PDL') }

# More arguments than the signature has fail as the generated XS fails
# ("Usage: PDL::op(a, b=b)").
sub _usage {
  my ($op, $sig, $max, @args) = @_;
  PDL::Core::barf("Usage: PDL::$op($sig)") if @args > $max;
}

# A new output, made as PDL::PP's XS makes one (PDL_XS_PREAMBLE and
# PDL_XS_pdlinit, lib/PDL/Core/pdlperl.h:4-45): in the class of the first
# argument when that is an object (a PDL or a hash-based subclass), through
# the class's initialize unless the class is PDL itself.
sub _new_out {
  my ($first) = @_;
  my $rt = Scalar::Util::reftype($first) // '';
  if (Scalar::Util::blessed($first) && ($rt eq 'SCALAR' || $rt eq 'HASH')) {
    return ref($first) eq 'PDL' ? PDL->null : $first->initialize;
  }
  return PDL->null;
}

# The GPU path takes the real types up to double and runs ops eagerly.  A
# call with a long double or complex ndarray (no device type for either), or
# with a flowing input (the op would make a dataflow transformation,
# lib/PDL/Core/pdlapi.c:776-783), stays on PDL's own op.
my $D = PDL::Core::double()->enum;
sub _pdl_op {
  my ($op, $args) = @_;
  return undef unless grep { _is_pdl($_) && ($_->get_datatype > $D || $_->fflows) } @$args;
  no strict 'refs';
  return $saved{$op} // \&{"PDL::$op"};
}

for my $op (@REDUCE) {
  no strict 'refs';
  *{"PDL::GB300::$op"} = sub {
    if (my $f = _pdl_op($op, \@_)) { return $f->(@_) }
    _usage($op, 'a, b=b', 2, @_);
    my ($a, $b) = @_;
    if ($INPLACE{$op} && _is_pdl($a) && $a->is_inplace) {
      PDL::Core::barf("inplace input but different output given") if defined $b;
      $b = $a;
      $a->set_inplace(0);
    }
    $b = _new_out($a) unless defined $b;
    _run($op, [$a, $b], 0);
    return $b;
  };
}

for my $op (@PCT) {
  no strict 'refs';
  *{"PDL::GB300::$op"} = sub {
    if (my $f = _pdl_op($op, \@_)) { return $f->(@_) }
    _usage($op, 'a, p, b=b', 3, @_);
    my ($a, $p, $b) = @_;
    $b = _new_out($a) unless defined $b;
    _run($op, [$a, $p, $b], 0);
    return $b;
  };
}

# a(n); [o]cmin(); [o]cmax(); indx [o]cmin_ind(); indx [o]cmax_ind()
sub minmaximum {
  if (my $f = _pdl_op('minmaximum', \@_)) { return $f->(@_) }
  _usage('minmaximum', 'a, cmin=cmin, cmax=cmax, cmin_ind=cmin_ind, cmax_ind=cmax_ind', 5, @_);
  my ($a, @o) = @_;
  $o[$_] = _new_out($a) for grep { !defined $o[$_] } 0 .. 3;
  _run('minmaximum', [$a, @o], 0);
  return @o;
}

# Called as op($a, $b), op($a, $b, $swap) (the operator overloads),
# op($a, $b, $c) or op($a, $b, $c, $swap); an inplace $a is the output
# (Inplace => ['a'], lib/PDL/Ops.pd biop).
for my $op (@BIOP) {
  no strict 'refs';
  *{"PDL::GB300::$op"} = sub {
    if (my $f = _pdl_op($op, \@_)) { return $f->(@_) }
    _usage($op, 'a, b, c=c, swap=swap', 4, @_);
    my ($a, $b, @rest) = @_;
    my ($c, $swap);
    if (@rest == 1 && !_is_pdl($rest[0])) { $swap = $rest[0] }
    else { ($c, $swap) = @rest }
    if (_is_pdl($a) && $a->is_inplace) {
      PDL::Core::barf("inplace input but different output given") if defined $c;
      $c = $a;
      $a->set_inplace(0);
    }
    $c = _new_out($_[0]) unless defined $c;
    _badval_warn($a, $b, $swap ? 1 : 0) if $CMP{$op};
    _run($op, [$a, $b, $c], $swap ? 1 : 0);
    return $c;
  };
}

sub inner {
  if (my $f = _pdl_op('inner', \@_)) { return $f->(@_) }
  _usage('inner', 'a, b, c=c', 3, @_);
  my ($a, $b, $c) = @_;
  $c = _new_out($a) unless defined $c;
  _run('inner', [$a, $b, $c], 0);
  return $c;
}

# PDL::matmult's own wrapper (lib/PDL/Primitive.pd:196-210), the same
# steps: pad to 2 dims with dummies, a 1x1 operand is an elementwise
# product, dim 0 of x must equal dim 1 of y; then the contraction here.
sub matmult {
  if (my $f = _pdl_op('matmult', \@_)) { return $f->(@_) }
  my ($x, $y, $c) = @_;
  $y = PDL->topdl($y);
  $c = PDL->null unless _is_pdl($c);
  $x = $x->dummy(-1) while $x->getndims < 2;
  $y = $y->dummy(-1) while $y->getndims < 2;
  return ($c .= $x * $y)
    if ($x->dim(0) == 1 && $x->dim(1) == 1) || ($y->dim(0) == 1 && $y->dim(1) == 1);
  PDL::Core::barf(sprintf 'Dim mismatch in matmult of [%1$dx%2$d] x [%3$dx%4$d]: %1$d != %4$d',
                  $x->dim(0), $x->dim(1), $y->dim(0), $y->dim(1))
    if $y->dim(1) != $x->dim(0);
  _run('matmult', [$x, $y, $c], 0);
  return $c;
}

# ---------------------------------------------------------------- adjoints
# Gradients of a loss with respect to an op's inputs from the gradient with
# respect to its output (nothing stored from the forward pass but its
# inputs): float or double ndarrays.
sub _like { my ($x) = @_; PDL->zeroes($x->type, $x->dims) }

sub sumover_bwd { my ($gb, $a) = @_; my $ga = _like($a); _bwd('sumover_bwd', [$gb, $ga]); $ga }
sub average_bwd { my ($gb, $a) = @_; my $ga = _like($a); _bwd('average_bwd', [$gb, $ga]); $ga }

sub plus_bwd {
  my ($gc, $a, $b) = @_;
  my ($ga, $gb) = (_like($a), _like($b));
  _bwd('plus_bwd', [$gc, $ga, $gb]);
  return ($ga, $gb);
}

sub mult_bwd {
  my ($gc, $a, $b) = @_;
  my ($ga, $gb) = (_like($a), _like($b));
  _bwd('mult_bwd', [$gc, $a, $b, $ga, $gb]);
  return ($ga, $gb);
}

sub matmult_bwd {
  my ($gc, $a, $b) = @_;
  my ($ga, $gb) = (_like($a), _like($b));
  _bwd('matmult_bwd', [$gc, $a, $b, $ga, $gb]);
  return ($ga, $gb);
}

# ----------------------------------------------------------------- install

# `use PDL::GB300 'install'` (or perl -MPDL::GB300=install) installs at once.
sub import {
  my ($pkg, @args) = @_;
  for (@args) {
    if ($_ eq 'install') { install() }
    else { PDL::Core::barf("PDL::GB300: unknown import $_") }
  }
}

sub install {
  no strict 'refs';
  no warnings 'redefine';
  for my $op (@REDUCE, @PCT, @BIOP, qw(inner matmult minmaximum)) {
    $saved{$op} //= \&{"PDL::$op"};
    *{"PDL::$op"} = \&{"PDL::GB300::$op"};
  }
}

sub uninstall {
  no strict 'refs';
  no warnings 'redefine';
  *{"PDL::$_"} = $saved{$_} for keys %saved;
}

1;
