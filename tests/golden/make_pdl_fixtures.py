"""TEST INFRASTRUCTURE: golden fixtures from the reference PDL itself, at the
configurations' full sizes.

Run where the reference can be built (oracle/build_reference_pdl.sh builds
it outside this repository):

    oracle/build_reference_pdl.sh /root/reference /tmp/pdl_ref
    python tests/golden/make_pdl_fixtures.py --pdl /tmp/pdl_ref

Each configuration's inputs come from tests/config_inputs.py (seeded numpy),
are written as FastRaw files, read by PDL's readfraw, put through PDL's own
ops (sumover, prodover, average, minimum, maximum, minimum_ind, maximum_ind,
dsumover, cumusumover, inner, matmult, and the unfused sumover($a*$b+$a)),
and the results are written back with writefraw.  Kept here: the full
results where they are small, and sampled positions plus SHA-256 digests of
the full results where they are large; each input's SHA-256 too, so a test
that regenerates the inputs can prove they are the bytes PDL saw.

Writes tests/golden/pdl_fixtures.npz and pdl_fixtures.json (manifest: PDL
version, host, threads, and per-case metadata).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import config_inputs as CI  # noqa: E402

PDL_TYPE = {np.dtype(np.float64): 10, np.dtype(np.float32): 9, np.dtype(np.int32): 4,
            np.dtype(np.int64): 6}
NP_TYPE = {10: np.float64, 9: np.float32, 4: np.int32, 6: np.int64, 8: np.int64}


def write_fraw(path: Path, arr: np.ndarray) -> None:
    """FastRaw: the data as laid out in memory plus "<type>\\n<ndims>\\n<dims>\\n"
    (PDL dims are numpy's shape reversed)."""
    arr = np.ascontiguousarray(arr)
    path.write_bytes(arr.tobytes())
    dims = list(arr.shape[::-1])
    (path.parent / (path.name + ".hdr")).write_text(
        f"{PDL_TYPE[arr.dtype]}\n{len(dims)}\n{' '.join(map(str, dims))}\n")


def read_fraw(path: Path) -> np.ndarray:
    t, nd, dims = (path.parent / (path.name + ".hdr")).read_text().split("\n")[:3]
    dims = [int(d) for d in dims.split()] if int(nd) else []
    return np.frombuffer(path.read_bytes(), dtype=NP_TYPE[int(t)]).reshape(dims[::-1])


def run_perl(pdl: Path, code: str) -> None:
    env = dict(os.environ)
    env["PERL5LIB"] = ":".join([str(pdl / "shims"), str(pdl / "src/blib/lib"),
                                str(pdl / "src/blib/arch")])
    r = subprocess.run(["perl", "-e", "use strict; use PDL; use PDL::IO::FastRaw;\n" + code],
                       env=env, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pdl", default="/tmp/pdl_ref")
    ap.add_argument("--out", default=str(HERE))
    args = ap.parse_args()
    pdl = Path(args.pdl)
    fx: dict[str, np.ndarray] = {}
    meta: dict[str, dict] = {}
    with tempfile.TemporaryDirectory() as td:
        d = Path(td)

        # ---------------- float64 (4096, 2048) family
        a = CI.c1()["a"]
        write_fraw(d / "c1a", a)
        ops = ["sumover", "dsumover", "prodover", "average", "minimum", "maximum",
               "minimum_ind", "maximum_ind", "cumusumover"]
        run_perl(pdl, f'my $a = readfraw("{d}/c1a");\n' +
                 "".join(f'writefraw({op}($a), "{d}/c1_{op}");\n' for op in ops))
        for op in ops:
            r = read_fraw(d / f"c1_{op}")
            if op == "cumusumover":
                fx["c1/cumusumover/sample"] = np.ascontiguousarray(r[::32, ::16])
                meta["c1/cumusumover"] = {"sha256": CI.sha(r), "sample": "rows ::32, positions ::16"}
            else:
                fx[f"c1/{op}"] = r
        meta["c1"] = {"input_sha256": CI.sha(a), "dims": [4096, 2048], "type": "double"}

        # ---------------- float32 (65536, 4096) + 2^27 row, 1 % BAD
        c5 = CI.c5()
        write_fraw(d / "c5m", c5["mat"])
        write_fraw(d / "c5r", c5["row"])
        code = ""
        for nm in ("c5m", "c5r"):
            code += f'{{ my $a = readfraw("{d}/{nm}"); $a->badflag(1);\n'
            for op in ("sumover", "average", "dsumover", "daverage", "cumusumover"):
                code += f'  writefraw({op}($a), "{d}/{nm}_{op}");\n'
            code += "}\n"
        run_perl(pdl, code)
        for nm, rows_step, pos_step in (("c5m", 64, 128), ("c5r", 1, 65536)):
            src = c5["mat"] if nm == "c5m" else c5["row"]
            meta[nm] = {"input_sha256": CI.sha(src), "dims": list(src.shape[::-1]),
                        "type": "float", "badflag": 1}
            for op in ("sumover", "average", "dsumover", "daverage"):
                fx[f"{nm}/{op}"] = read_fraw(d / f"{nm}_{op}").reshape(-1)
            r = read_fraw(d / f"{nm}_cumusumover").reshape(src.shape)
            fx[f"{nm}/cumusumover/sample"] = np.ascontiguousarray(r[::rows_step, ::pos_step])
            meta[f"{nm}/cumusumover"] = {"sha256": CI.sha(r),
                                         "bad_sha256": CI.sha(r == CI.F32_BAD),
                                         "sample": f"rows ::{rows_step}, positions ::{pos_step}"}
            del r
        del c5

        # ---------------- sumover(a*b + a), unfused, int32 and float32 with BAD
        for nm, gen in (("c2i", CI.c2_int32), ("c2f", CI.c2_float32_bad)):
            x = gen()
            write_fraw(d / f"{nm}a", x["a"])
            write_fraw(d / f"{nm}b", x["b"])
            bf = "$a->badflag(1); $b->badflag(1);" if nm == "c2f" else ""
            run_perl(pdl, f'my $a = readfraw("{d}/{nm}a"); my $b = readfraw("{d}/{nm}b"); {bf}\n'
                          f'writefraw(sumover($a * $b + $a), "{d}/{nm}_out");\n')
            r = read_fraw(d / f"{nm}_out")                     # numpy (8192, 512)
            fx[f"{nm}/sample"] = np.ascontiguousarray(r[::2048])
            meta[nm] = {"input_sha256": [CI.sha(x["a"]), CI.sha(x["b"])], "sha256": CI.sha(r),
                        "sample": "output rows (dim 1) ::2048"}
            if nm == "c2f":
                meta[nm]["bad_sha256"] = CI.sha(r == CI.F32_BAD)
            del x, r

        # ---------------- float64 inner (4096, 65536)
        x = CI.c3_inner()
        write_fraw(d / "c3ia", x["a"])
        write_fraw(d / "c3ib", x["b"])
        run_perl(pdl, f'writefraw(inner(readfraw("{d}/c3ia"), readfraw("{d}/c3ib")), "{d}/c3i_out");\n')
        r = read_fraw(d / "c3i_out")
        fx["c3i/sample"] = np.ascontiguousarray(r[::8])
        meta["c3i"] = {"input_sha256": [CI.sha(x["a"]), CI.sha(x["b"])], "sha256": CI.sha(r),
                       "sample": "::8", "platform": platform.machine()}
        del x, r

        # ---------------- float32 matmult, batch 16
        x = CI.c3_matmult()
        write_fraw(d / "c3ma", x["a"])
        write_fraw(d / "c3mb", x["b"])
        run_perl(pdl, f'writefraw(matmult(readfraw("{d}/c3ma"), readfraw("{d}/c3mb")), "{d}/c3m_out");\n')
        r = read_fraw(d / "c3m_out")                           # numpy (16, 2048, 2048)
        fx["c3m/sample"] = np.ascontiguousarray(r[[0, 11]][:, ::256, :])
        meta["c3m"] = {"input_sha256": [CI.sha(x["a"]), CI.sha(x["b"])], "sha256": CI.sha(r),
                       "sample": "batches [0, 11], rows (h) ::256, every w"}
        del x, r

        # ---------------- the adjoint workload's gradients, by hand in PDL (FP64)
        # L = sumover(sumover((X x W + bias)**2)) / 8192; G = dL/dZ = 2 Z / 8192
        x = CI.c4()
        for k in ("X", "W", "bias"):
            write_fraw(d / f"c4{k}", x[k])
        run_perl(pdl, f'my $X = readfraw("{d}/c4X")->double; my $W = readfraw("{d}/c4W")->double;\n'
                      f'my $b = readfraw("{d}/c4bias")->double;\n'
                      'my $G = 2 * (($X x $W) + $b) / 8192;\n'
                      f'writefraw($G x $W->transpose, "{d}/c4_gX");\n'
                      f'writefraw($X->transpose x $G, "{d}/c4_gW");\n'
                      f'writefraw($G->xchg(0, 1)->sumover, "{d}/c4_gbias");\n')
        gX, gW, gb = (read_fraw(d / f"c4_{k}") for k in ("gX", "gW", "gbias"))
        fx["c4/gX/sample"] = np.ascontiguousarray(gX[::256])     # numpy (8192, 512): rows ::256
        fx["c4/gW/sample"] = np.ascontiguousarray(gW[::8])       # numpy (512, 256): rows ::8
        fx["c4/gbias"] = gb
        meta["c4"] = {"input_sha256": [CI.sha(x[k]) for k in ("X", "W", "bias")],
                      "sha256": {"gX": CI.sha(gX), "gW": CI.sha(gW), "gbias": CI.sha(gb)},
                      "what": "dL/dX, dL/dW, dL/dbias by hand in PDL, float64",
                      "sample": "gX numpy rows ::256, gW numpy rows ::8, gbias whole"}
        del x, gX, gW, gb

    env = dict(os.environ, PERL5LIB=f"{pdl}/shims:{pdl}/src/blib/lib:{pdl}/src/blib/arch")
    ver = subprocess.run(["perl", "-MPDL", "-e",
                          'print "$PDL::VERSION ", PDL::Core::pthreads_enabled(), " ", '
                          'PDL::Core::online_cpus()'], env=env, capture_output=True, text=True).stdout
    v, pt, ncpu = ver.split()
    meta["_made_by"] = {"pdl_version": v, "pthreads_enabled": int(pt), "online_cpus": int(ncpu),
                        "host": platform.machine(), "script": "tests/golden/make_pdl_fixtures.py"}
    out = Path(args.out)
    np.savez_compressed(out / "pdl_fixtures.npz", **fx)
    (out / "pdl_fixtures.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(fx)} arrays, {(out / 'pdl_fixtures.npz').stat().st_size} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
