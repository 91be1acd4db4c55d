#!/bin/bash
# TEST INFRASTRUCTURE ONLY: build the reference PDL (a checker for the
# oracle and the golden fixtures; nothing in the library uses it).
#
# The reference's build needs five CPAN modules that are not installed here
# (Devel::CheckLib, File::Which and File::Map for the build; Test::Exception
# and Test::Warn for its tests).  This script writes small stand-ins of our
# own for the few functions the build calls, copies the reference tree to a
# scratch directory outside this repository (the reference tree is
# read-only), and builds it there with the reference's own Makefile.PL.
#
# Usage: oracle/build_reference_pdl.sh [SRC] [OUT]
#   SRC defaults to /root/reference, OUT to /tmp/pdl_ref.
# Afterwards: PERL5LIB=$OUT/shims:$OUT/src/blib/lib:$OUT/src/blib/arch perl -MPDL ...
set -euo pipefail
SRC=${1:-/root/reference}
OUT=${2:-/tmp/pdl_ref}
mkdir -p "$OUT/shims/Devel" "$OUT/shims/File" "$OUT/shims/Test"

cat > "$OUT/shims/Devel/CheckLib.pm" <<'PM'
package Devel::CheckLib;
# check_lib: does a program using the given header/library/function compile
# and link with the configured C compiler?
use strict; use warnings;
use Config; use File::Temp qw(tempdir);
use Exporter 'import';
our @EXPORT = qw(check_lib check_lib_or_exit assert_lib);
sub check_lib {
  my %a = @_;
  my $d = tempdir(CLEANUP => 1);
  my @h = ref $a{header} ? @{$a{header}} : grep defined, $a{header};
  my @l = ref $a{lib} ? @{$a{lib}} : grep { defined && length } $a{lib};
  my $body = $a{function} // 'return 0;';
  open my $fh, '>', "$d/t.c" or return 0;
  print $fh "#include <$_>\n" for @h;
  print $fh "int main(void) { $body }\n";
  close $fh;
  my $inc = join ' ', map "-I$_", grep { defined && length } (ref $a{incpath} ? @{$a{incpath}} : $a{incpath});
  my $libs = join ' ', map "-l$_", @l;
  my $cc = "$Config{cc} $Config{ccflags} " . ($a{ccflags} // '') . " $inc -o $d/t $d/t.c $libs 2>/dev/null";
  return system($cc) == 0 ? 1 : 0;
}
sub assert_lib { check_lib(@_) or die "library check failed\n"; 1 }
sub check_lib_or_exit { check_lib(@_) or exit 0; 1 }
1;
PM

cat > "$OUT/shims/File/Which.pm" <<'PM'
package File::Which;
# which: the first executable of that name on PATH
use strict; use warnings;
use Exporter 'import';
our @EXPORT_OK = qw(which);
sub which {
  my ($p) = @_;
  for my $d (split /:/, $ENV{PATH} // '') { return "$d/$p" if -x "$d/$p" && !-d "$d/$p"; }
  return undef;
}
1;
PM

cat > "$OUT/shims/File/Map.pm" <<'PM'
package File::Map;
# map_file: here the file's contents are read into the variable
use strict; use warnings;
use Exporter 'import';
our @EXPORT_OK = qw(map_file PROT_READ PROT_WRITE MAP_SHARED MAP_PRIVATE);
sub PROT_READ { 1 } sub PROT_WRITE { 2 } sub MAP_SHARED { 1 } sub MAP_PRIVATE { 2 }
sub map_file {
  my (undef, $file) = @_;
  open my $fh, '<:raw', $file or die "open $file: $!";
  local $/; $_[0] = <$fh>; close $fh; 1;
}
1;
PM

cat > "$OUT/shims/Test/Exception.pm" <<'PM'
package Test::Exception;
# throws_ok / lives_ok / dies_ok on top of Test::More
use strict; use warnings;
use Test::More ();
use Exporter 'import';
our @EXPORT = qw(throws_ok lives_ok dies_ok lives_and);
sub throws_ok(&$;$) {
  my ($c, $re, $name) = @_;
  eval { $c->() }; my $e = $@;
  local $Test::Builder::Level = $Test::Builder::Level + 1;
  ref $re eq 'Regexp' ? Test::More::like($e, $re, $name) : Test::More::ok(ref $e && $e->isa($re), $name);
}
sub lives_ok(&;$) { my ($c, $n) = @_; local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(eval { $c->(); 1 }, $n) or Test::More::diag($@) }
sub dies_ok(&;$) { my ($c, $n) = @_; local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(!eval { $c->(); 1 }, $n) }
sub lives_and(&;$) { my ($c, $n) = @_; eval { $c->() }; Test::More::fail($n) if $@ }
1;
PM

cat > "$OUT/shims/Test/Warn.pm" <<'PM'
package Test::Warn;
# warning_like / warnings_like / warning_is / warnings_are
use strict; use warnings;
use Test::More ();
use Exporter 'import';
our @EXPORT = qw(warning_like warnings_like warning_is warnings_are);
sub _collect { my $c = shift; my @w; local $SIG{__WARN__} = sub { push @w, $_[0] }; $c->(); @w }
sub warning_like(&$;$) { my ($c, $re, $n) = @_; my @w = _collect($c);
  local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(@w == 1 && $w[0] =~ (ref $re eq 'HASH' ? (values %$re)[0] : $re), $n) }
sub warnings_like(&$;$) { my ($c, $res, $n) = @_; my @w = _collect($c);
  $res = [$res] if ref $res ne 'ARRAY';
  local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(@w == @$res && !grep({ $w[$_] !~ $res->[$_] } 0..$#w), $n) }
sub warning_is(&$;$) { my ($c, $s, $n) = @_; my @w = _collect($c);
  local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(defined $s ? (@w == 1 && index($w[0], ref $s ? (values %$s)[0] : $s) >= 0) : !@w, $n) }
sub warnings_are(&$;$) { my ($c, $s, $n) = @_; my @w = _collect($c);
  local $Test::Builder::Level = $Test::Builder::Level + 1;
  Test::More::ok(@w == @$s, $n) }
1;
PM

rm -rf "$OUT/src"
cp -r "$SRC" "$OUT/src"
chmod -R u+w "$OUT/src"
cd "$OUT/src"
export PERL5LIB="$OUT/shims${PERL5LIB:+:$PERL5LIB}"
perl Makefile.PL > "$OUT/configure.log" 2>&1
make -j"$(nproc)" > "$OUT/make.log" 2>&1
perl -Mblib -MPDL -e 'print "PDL $PDL::VERSION pthreads=", PDL::Core::pthreads_enabled(), "\n"'
