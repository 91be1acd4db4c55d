"""TEST INFRASTRUCTURE: FastRaw files written by the reference PDL's own
writefraw (lib/PDL/IO/FastRaw.pm), for the readers' tests.

    oracle/build_reference_pdl.sh /root/reference /tmp/pdl_ref
    python tests/golden/make_fraw_fixtures.py --pdl /tmp/pdl_ref

Writes tests/golden/fraw/<name> and <name>.hdr for: a double (5,4,3)
sequence*1.5-7, a long (7,2) sequence*-3, a byte (9) sequence, a float
(6,2) with its default badvalue at two positions, and a double written
with a custom header file name."""
import argparse
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent

CODE = r'''
use strict; use PDL; use PDL::IO::FastRaw;
my $d = shift;
writefraw(sequence(double, 5, 4, 3) * 1.5 - 7, "$d/seq_double");
writefraw(sequence(long, 7, 2) * -3, "$d/seq_long");
writefraw(sequence(byte, 9), "$d/seq_byte");
my $f = sequence(float, 6, 2) / 4; $f->badflag(1); $f->set(1, 0, $f->badvalue); $f->set(4, 1, $f->badvalue);
writefraw($f, "$d/float_bad");
writefraw(sequence(double, 3, 2), "$d/own_header", {Header => "$d/own_header.h"});
'''


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pdl", default="/tmp/pdl_ref")
    a = ap.parse_args()
    pdl = Path(a.pdl)
    out = HERE / "fraw"
    out.mkdir(exist_ok=True)
    env = dict(os.environ, PERL5LIB=":".join(str(p) for p in (
        pdl / "shims", pdl / "src/blib/lib", pdl / "src/blib/arch")))
    subprocess.run(["perl", "-e", CODE, str(out)], env=env, check=True)
    for f in sorted(out.iterdir()):
        print(f.name, f.stat().st_size)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
