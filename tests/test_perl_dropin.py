"""PDL::GB300, the Perl module a PDL session loads, checked against the
reference PDL itself on the CPU.

* tests/perl/dropin_cpu.t: the descriptors of PDL's views, the planner's
  shapes, types and error text against PDL's own ops, explicit broadcast
  ids refused, install() routing PDL's subs and operators to the module.
* The reference's own test suite (every t/*.t of the built tree) run with
  the module installed, its compute answered by tests/perl/cpu_double.c
  (the oracle in place of the GPU), must give the same results as without
  it: this checks the glue -- views, null outputs allocated by PDL,
  supplied outputs of other types, in-place ops, bad-value flags and their
  propagation to views, headers, subclasses, read-only outputs, error
  text -- on everything PDL's tests do with these ops.  The one expected
  difference is t/pthread.t, which reads PDL's auto-pthread counters: the
  module's ops do not run on PDL's CPU threads.

Needs a build of the reference PDL (oracle/build_reference_pdl.sh writes one
to the directory PDLGB300_PDL_BUILD names, by default the script's own
default); the tests skip when there is none, or no perl/xsubpp/gcc."""
import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PDL_BUILD = Path(os.environ.get("PDLGB300_PDL_BUILD", "/tmp/pdl_ref"))
EXPECTED_DIFFERENT = {"pthread.t"}


def _pdl_lib():
    lib = PDL_BUILD / "src" / "blib" / "lib"
    return lib if (lib / "PDL" / "Core" / "pdl.h").exists() else None


@pytest.fixture(scope="module")
def pdl_lib():
    if not all(shutil.which(t) for t in ("perl", "xsubpp", "gcc")):
        pytest.skip("no perl toolchain")
    lib = _pdl_lib()
    if lib is None:
        pytest.skip(f"no reference PDL build under {PDL_BUILD} (oracle/build_reference_pdl.sh makes one)")
    return lib


def _perl5lib(lib, *more):
    return ":".join(str(p) for p in (PDL_BUILD / "shims", lib, PDL_BUILD / "src" / "blib" / "arch", *more))


def test_perl_module_against_reference_pdl(pdl_lib):
    from pdl_gb300.perl import build as PB
    out = PB.build(pdl_lib)
    env = dict(os.environ, PERL5LIB=_perl5lib(pdl_lib, out))
    r = subprocess.run(["perl", str(ROOT / "tests" / "perl" / "dropin_cpu.t")], env=env,
                       capture_output=True, text=True, timeout=600)
    lines = r.stdout.splitlines()
    bad = [l for l in lines if l.startswith("not ok")]
    assert r.returncode == 0 and not bad, r.stdout[-3000:] + r.stderr[-3000:]
    assert any(l.startswith("1..") for l in lines), r.stdout[-2000:]


@pytest.fixture(scope="module")
def glue_on_double(pdl_lib, tmp_path_factory):
    """PDL::GB300 linked against the CPU double of libpdlgb300."""
    d = tmp_path_factory.mktemp("double")
    so = d / "libpdlgb300.so"
    subprocess.run(["gcc", "-O2", "-fPIC", "-fwrapv", "-ffp-contract=off", "-std=gnu11",
                    "-I", str(ROOT / "include"), "-shared", "-o", str(so),
                    str(ROOT / "tests" / "perl" / "cpu_double.c"),
                    str(ROOT / "oracle" / "pdl_oracle.c"), "-lpthread", "-lm"], check=True)
    from pdl_gb300.perl import build as PB
    return PB.build(pdl_lib, True, lib=so, out=d / "mod")


def _run_t(t: Path, env, install: bool):
    cmd = ["perl", "-MPDL"] + (["-MPDL::GB300=install"] if install else []) + [str(t)]
    r = subprocess.run(cmd, env=env, cwd=PDL_BUILD / "src", capture_output=True, text=True,
                       timeout=300)
    failed = len(re.findall(r"^\s*not ok", r.stdout, re.M))
    return failed, r.returncode


def test_reference_suite_through_the_glue(pdl_lib, glue_on_double, tmp_path):
    tests = sorted((PDL_BUILD / "src" / "t").glob("*.t"))
    if not tests:
        pytest.skip("the PDL build has no t/ directory")
    log = tmp_path / "runs.log"
    base = dict(os.environ, PERL5LIB=_perl5lib(pdl_lib))
    glue = dict(os.environ, PERL5LIB=_perl5lib(pdl_lib, glue_on_double),
                PDLGB300_DOUBLE_LOG=str(log))
    diff = []
    for t in tests:
        want = _run_t(t, base, False)
        got = _run_t(t, glue, True)
        if got != want and t.name not in EXPECTED_DIFFERENT:
            diff.append(f"{t.name}: without the module {want}, with it {got} (failed tests, exit code)")
    assert not diff, "\n".join(diff)
    runs = {}
    for line in log.read_text().splitlines():
        op, n = line.split()
        runs[op] = runs.get(op, 0) + int(n)
    # the path's ops went through the glue
    for op in ("sumover", "prodover", "average", "minimum", "maximum", "cumusumover", "plus",
               "mult", "inner", "matmult", "qsort", "qsorti", "qsortvec", "medover", "pctover",
               "minmaximum"):
        assert runs.get(op, 0) > 0, (op, runs)
