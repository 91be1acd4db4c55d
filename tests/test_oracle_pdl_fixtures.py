"""The oracle pinned to the reference PDL itself at the configurations' full
sizes: tests/golden/pdl_fixtures.npz holds PDL 2.106's own results on the
seeded inputs of tests/config_inputs.py (made by
tests/golden/make_pdl_fixtures.py with the reference built by
oracle/build_reference_pdl.sh).  The oracle restates PDL's loops in the
same order and arithmetic, so its results must equal PDL's bit for bit:
whole results where PDL's are kept whole, SHA-256 digests of the whole
result where they are large, and sampled rows (an output depends only on its
own rows' elements, so a row subset reproduces the sampled outputs) for the
contractions."""
import json
from pathlib import Path

import numpy as np
import pytest

import config_inputs as CI
import pdl_gb300 as P
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
FX = np.load(GOLD / "pdl_fixtures.npz")
META = json.loads((GOLD / "pdl_fixtures.json").read_text())
NTH = 8


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view({8: np.uint64, 4: np.uint32, 2: np.uint16, 1: np.uint8}[a.dtype.itemsize])


def test_fixture_inputs_regenerate_exactly():
    assert CI.sha(CI.c1()["a"]) == META["c1"]["input_sha256"]
    x = CI.c2_int32()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c2i"]["input_sha256"]
    x = CI.c2_float32_bad()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c2f"]["input_sha256"]


def test_c1_family_bit_for_bit():
    a = CI.c1()["a"]
    x = P.pdl(a)
    for op in ["sumover", "dsumover", "prodover", "average", "minimum", "maximum",
               "minimum_ind", "maximum_ind"]:
        got = O.run(op, [x], nthreads=NTH)[0].numpy()
        assert np.array_equal(bits(got), bits(FX[f"c1/{op}"])), op
    c = O.run("cumusumover", [x], nthreads=NTH)[0].numpy()
    assert CI.sha(c) == META["c1/cumusumover"]["sha256"]
    assert np.array_equal(bits(c[::32, ::16]), bits(FX["c1/cumusumover/sample"]))


@pytest.mark.parametrize("which", ["c5m", "c5r"])
def test_c5_sums_bit_for_bit(which):
    c5 = CI.c5()
    src = c5["mat"] if which == "c5m" else c5["row"]
    del c5
    assert CI.sha(src) == META[which]["input_sha256"]
    x = P.pdl(src)
    x.badflag(1)
    for op in ("sumover", "average", "dsumover", "daverage"):
        got = O.run(op, [x], nthreads=NTH)[0].numpy().reshape(-1)
        assert np.array_equal(bits(got), bits(FX[f"{which}/{op}"])), op
    c = O.run("cumusumover", [x], nthreads=NTH)[0].numpy().reshape(src.shape)
    assert CI.sha(c) == META[f"{which}/cumusumover"]["sha256"]
    assert CI.sha(c == CI.F32_BAD) == META[f"{which}/cumusumover"]["bad_sha256"]


@pytest.mark.parametrize("which", ["c2i", "c2f"])
def test_c2_unfused_chain_bit_for_bit_on_sampled_rows(which):
    x = CI.c2_int32() if which == "c2i" else CI.c2_float32_bad()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META[which]["input_sha256"]
    a = np.ascontiguousarray(x["a"][::2048])              # output rows k ::2048
    pa, pb = P.pdl(a), P.pdl(x["b"])
    if which == "c2f":
        pa.badflag(1)
        pb.badflag(1)
    t = O.run("mult", [pa, pb], nthreads=NTH)[0]
    u = O.run("plus", [t, pa], nthreads=NTH)[0]
    got = O.run("sumover", [u], nthreads=NTH)[0].numpy()
    assert np.array_equal(bits(got), bits(FX[f"{which}/sample"]))


def test_c3_inner_bit_for_bit_on_sampled_rows():
    import platform
    if META["c3i"]["platform"] != platform.machine():
        pytest.skip("inner accumulates in long double: fixtures from another architecture")
    x = CI.c3_inner()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c3i"]["input_sha256"]
    a, b = np.ascontiguousarray(x["a"][::8]), np.ascontiguousarray(x["b"][::8])
    del x
    got = O.run("inner", [P.pdl(a), P.pdl(b)], nthreads=NTH)[0].numpy()
    assert np.array_equal(bits(got), bits(FX["c3i/sample"]))


def test_c3_matmult_bit_for_bit_on_sampled_rows():
    x = CI.c3_matmult()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c3m"]["input_sha256"]
    a = np.ascontiguousarray(x["a"][[0, 11]][:, ::256, :])   # batches 0, 11; rows h ::256
    got = O.run("matmult", [P.pdl(a), P.pdl(x["b"])], nthreads=NTH)[0].numpy()
    assert np.array_equal(bits(got), bits(FX["c3m/sample"]))


def test_c4_gradients_by_hand_in_pdl_are_the_fp64_gradients():
    """The fixture's gradients (written out by hand in PDL, float64) equal
    numpy's float64 evaluation of the same formulas to rounding."""
    x = CI.c4()
    assert [CI.sha(x[k]) for k in ("X", "W", "bias")] == META["c4"]["input_sha256"]
    X, W, b = (x[k].astype(np.float64) for k in ("X", "W", "bias"))
    G = 2.0 * (X @ W + b) / 8192.0
    want = {"gX": (G @ W.T)[::256], "gW": (X.T @ G)[::8], "gbias": G.sum(0)}
    for k, w in want.items():
        got = FX[f"c4/{k}/sample"] if k != "gbias" else FX["c4/gbias"]
        assert np.max(np.abs(got - w)) <= 1e-12 * np.max(np.abs(w)), k
