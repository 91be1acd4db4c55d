"""TEST INFRASTRUCTURE: time the reference PDL beside the oracle (the C port
of its loops that bench.py's reference arm runs) on the same host, on the
float32 stress workload's ops (sumover, average, cumusumover over dim 0 of
the (65536, 4096) matrix and of the 2^27 row, 1 % BAD), so the port's timing
can be read against PDL's own.

Needs the reference built by oracle/build_reference_pdl.sh (default
/tmp/pdl_ref).  Prints one JSON line: GB/s (input read once + output
written once) for PDL at PDL_AUTOPTHREAD_TARG=1 thread and =nproc, and for
the port with 1 thread and nproc threads; median of 5 runs each.

Usage: python oracle/time_reference_pdl.py [--pdl /tmp/pdl_ref] [--rows 1024]
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))
import config_inputs as CI  # noqa: E402

OPS = ["sumover", "average", "cumusumover"]


def op_bytes(op, n, rows):
    return rows * n * 8 if op == "cumusumover" else rows * n * 4 + rows * 4


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pdl", default="/tmp/pdl_ref")
    ap.add_argument("--rows", type=int, default=4096)
    args = ap.parse_args()
    c5 = CI.c5(rows=args.rows)
    mat, row = c5["mat"], c5["row"]
    nproc = os.cpu_count() or 1
    total = sum(op_bytes(op, 65536, args.rows) + op_bytes(op, 1 << 27, 1) for op in OPS)
    out = {"host": platform.machine(), "cores": nproc, "rows": args.rows,
           "workload": "sumover, average, cumusumover over dim 0: float32 (65536, rows) and a row "
                       "of 2^27, lognormal(0,4) magnitudes, random sign, 1% BAD, seed 7",
           "bytes_per_step": total}
    with tempfile.TemporaryDirectory() as td:
        for nm, arr in (("mat", mat), ("row", row)):
            Path(td, nm).write_bytes(np.ascontiguousarray(arr).tobytes())
            Path(td, nm + ".hdr").write_text(f"9\n2\n{arr.shape[1]} {arr.shape[0]}\n")
        perl = f'''use strict; use PDL; use PDL::IO::FastRaw; use Time::HiRes qw(time);
my @x = map {{ my $p = readfraw("{td}/$_"); $p->badflag(1); $p }} qw(mat row);
my @t;
for my $rep (0..5) {{
  my $t0 = time;
  for my $p (@x) {{ my $s = sumover($p); my $a = average($p); my $c = cumusumover($p); }}
  push @t, time - $t0 if $rep;
}}
@t = sort {{ $a <=> $b }} @t; print $t[2], "\\n";'''
        env = dict(os.environ, PERL5LIB=f"{args.pdl}/shims:{args.pdl}/src/blib/lib:{args.pdl}/src/blib/arch")
        for label, targ in (("pdl_1_thread", "0"), (f"pdl_{nproc}_threads", str(nproc))):
            env["PDL_AUTOPTHREAD_TARG"] = targ
            r = subprocess.run(["perl", "-e", perl], env=env, capture_output=True, text=True)
            if r.returncode:
                raise RuntimeError(r.stderr)
            out[label] = total / float(r.stdout.strip()) / 1e9
    import pdl_gb300 as P
    from oracle import oracle as O
    xs = []
    for arr in (mat, row):
        x = P.pdl(arr)
        x.badflag(1)
        xs.append(x)
    for label, nt in (("port_1_thread", 1), (f"port_{nproc}_threads", nproc)):
        ts = []
        for rep in range(6):
            t0 = time.perf_counter()
            for x in xs:
                for op in OPS:
                    O.run(op, [x], nthreads=nt)
            if rep:
                ts.append(time.perf_counter() - t0)
        out[label] = total / statistics.median(ts) / 1e9
    out["unit"] = "GB/s"
    print(json.dumps(out))


if __name__ == "__main__":
    main()
