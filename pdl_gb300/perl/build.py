"""Build the PDL::GB300 Perl module (GB300.xs + GB300.pm) against a PDL build.

PDL::GB300 links libpdlgb300.so (built first by pdl_gb300.build) and PDL's
headers (pdl.h, pdlcore.h).  The module is written to
pdl_gb300/perl/_build/{PDL/GB300.pm, auto/PDL/GB300/GB300.so}; use it with

    PERL5LIB=<pdl lib dirs>:pdl_gb300/perl/_build perl -MPDL -MPDL::GB300 ...

Usage: python -m pdl_gb300.perl.build --pdl-lib <dir with PDL/Core/pdl.h> [--pdl-arch <dir>]
"""
from __future__ import annotations

import argparse
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
OUT = HERE / "_build"


def build(pdl_lib: Path, force: bool = False, lib: Path | None = None,
          out: Path | None = None) -> Path:
    """Compile the module; pdl_lib holds PDL/Core/pdl.h and pdlcore.h (a
    PDL install's lib or build tree's blib/lib).  lib: the libpdlgb300.so to
    link (default: the package's own, built first if missing); out: the
    module tree to write (default pdl_gb300/perl/_build)."""
    core = Path(pdl_lib) / "PDL" / "Core"
    if not (core / "pdl.h").exists():
        raise RuntimeError(f"no PDL headers under {core}")
    OUT = Path(out) if out is not None else globals()["OUT"]
    if lib is None:
        lib = PKG / "_lib" / "libpdlgb300.so"
        if not lib.exists():
            from pdl_gb300 import build as B
            B.build()
    lib = Path(lib).resolve()
    so = OUT / "auto" / "PDL" / "GB300" / "GB300.so"
    src = HERE / "GB300.xs"
    if not force and so.exists() and so.stat().st_mtime > max(src.stat().st_mtime, lib.stat().st_mtime):
        shutil.copy(HERE / "GB300.pm", OUT / "PDL" / "GB300.pm")
        return OUT
    so.parent.mkdir(parents=True, exist_ok=True)
    (OUT / "PDL").mkdir(parents=True, exist_ok=True)
    privlib = subprocess.run(["perl", "-MConfig", "-e", "print $Config{privlibexp}"],
                             capture_output=True, text=True, check=True).stdout
    c = OUT / "GB300.c"
    r = subprocess.run(["xsubpp", "-typemap", f"{privlib}/ExtUtils/typemap", str(src)],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("xsubpp failed:\n" + r.stderr)
    c.write_text(r.stdout)
    ccopts = subprocess.run(["perl", "-MExtUtils::Embed", "-e", "ccopts"],
                            capture_output=True, text=True, check=True).stdout.split()
    cmd = ["gcc", "-shared", "-fPIC", "-O2", *ccopts, "-I", str(core), "-I", str(PKG.parent / "include"),
           "-o", str(so), str(c), "-L", str(lib.parent), "-lpdlgb300",
           f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("compiling PDL::GB300 failed:\n" + r.stderr[-4000:])
    shutil.copy(HERE / "GB300.pm", OUT / "PDL" / "GB300.pm")
    return OUT


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--pdl-lib", required=True)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build(Path(a.pdl_lib), a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
