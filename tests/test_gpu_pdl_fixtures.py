"""The GPU against the reference PDL itself at the configurations' full
sizes: tests/golden/pdl_fixtures.npz holds PDL 2.106's results on the seeded
inputs of tests/config_inputs.py (regenerated here; their SHA-256 digests
prove they are the bytes PDL saw).

Bar: bit-exact where the GPU keeps the reference's order or the result is
order-free (minimum, maximum and their indices, prodover's early exit,
int32 sums, bad masks, exact-mode matmult); floating sums within the
reference's own bound for a sequential sum, (n+2)*eps*sum|a|, and
compensated float32 also within 4*eps32*|s| + (n+2)*eps64*sum|a| of PDL's
float64 dsumover; bf16x6 matmult within (2K+8)*2^-24*(|A||B|) of PDL's
float32 result (PDL's own error is up to K*2^-24*(|A||B|))."""
import json
from pathlib import Path

import numpy as np
import pytest

import config_inputs as CI
import pdl_gb300 as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
FX = np.load(GOLD / "pdl_fixtures.npz")
META = json.loads((GOLD / "pdl_fixtures.json").read_text())
EPS32, EPS64 = 2.0 ** -24, 2.0 ** -53


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view({8: np.uint64, 4: np.uint32}[a.dtype.itemsize])


@pytest.fixture(scope="module")
def c1():
    a = CI.c1()["a"]
    assert CI.sha(a) == META["c1"]["input_sha256"]
    return a, P.pdl(a).to_device()


@pytest.mark.parametrize("op", ["minimum", "maximum", "minimum_ind", "maximum_ind", "prodover",
                                "sumover", "dsumover", "average", "cumusumover"])
def test_c1_family_against_pdl(gpu, c1, op):
    a, x = c1
    got = getattr(P, op)(x).numpy()
    if op == "cumusumover":
        want = FX["c1/cumusumover/sample"]
        scale = np.cumsum(np.abs(a), -1)[::32, ::16]
        assert np.all(np.abs(got[::32, ::16] - want) <= (4096 + 2) * EPS64 * scale)
        return
    want = FX[f"c1/{op}"]
    if op in ("minimum", "maximum", "minimum_ind", "maximum_ind", "prodover"):
        assert np.array_equal(bits(got), bits(want))
        return
    scale = np.abs(a).sum(-1) / (4096 if op == "average" else 1)
    assert np.all(np.abs(got - want) <= (4096 + 2) * EPS64 * scale)


@pytest.mark.parametrize("which", ["c5m", "c5r"])
def test_c5_against_pdl(gpu, which):
    c5 = CI.c5()
    src = c5["mat"] if which == "c5m" else c5["row"]
    del c5
    assert CI.sha(src) == META[which]["input_sha256"]
    x = P.pdl(src)
    x.badflag(1)
    x.to_device()
    good = src != CI.F32_BAD
    absum = np.where(good, np.abs(src.astype(np.float64)), 0).sum(-1)
    cnt = good.sum(-1)
    n = src.shape[-1]
    d64 = FX[f"{which}/dsumover"]
    for op, div in (("sumover", 1), ("average", cnt)):
        g = getattr(P, op)(x).numpy().reshape(-1).astype(np.float64)
        e = FX[f"{which}/{op}"].astype(np.float64)
        assert np.all(np.abs(g - e) <= (n + 2) * EPS32 * absum / div), op
        ref64 = d64 / div
        assert np.all(np.abs(g - ref64) <= 4 * EPS32 * np.abs(ref64) + (n + 2) * EPS64 * absum / div), op
    g = P.dsumover(x).numpy().reshape(-1)
    assert np.all(np.abs(g - d64) <= (n + 2) * EPS64 * absum)
    c = P.cumusumover(x).numpy().reshape(src.shape)
    assert CI.sha(c == CI.F32_BAD) == META[f"{which}/cumusumover"]["bad_sha256"]
    rs, ps = (64, 128) if which == "c5m" else (1, 65536)
    want = FX[f"{which}/cumusumover/sample"].astype(np.float64)
    absc = np.cumsum(np.where(good, np.abs(src.astype(np.float64)), 0), -1)[::rs, ::ps]
    gs = c[::rs, ::ps].astype(np.float64)
    ok = good[::rs, ::ps]
    assert np.all(np.abs(gs - want)[ok] <= (n + 2) * EPS32 * absc[ok])


def test_c2_int32_fused_equals_pdls_unfused_chain(gpu):
    x = CI.c2_int32()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c2i"]["input_sha256"]
    a, b = P.pdl(x["a"]).to_device(), P.pdl(x["b"]).to_device()
    got = P.sumover_mult_plus(a, b, a).numpy()
    assert CI.sha(got) == META["c2i"]["sha256"]          # every element, bit for bit
    assert np.array_equal(got[::2048], FX["c2i/sample"])


def test_c2_float32_bad_fused_against_pdl(gpu):
    x = CI.c2_float32_bad()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c2f"]["input_sha256"]
    a, b = P.pdl(x["a"]), P.pdl(x["b"])
    a.badflag(1)
    b.badflag(1)
    a.to_device()
    b.to_device()
    got = P.sumover_mult_plus(a, b, a).numpy()
    assert CI.sha(got == CI.F32_BAD) == META["c2f"]["bad_sha256"]   # the bad mask, exactly
    want = FX["c2f/sample"].astype(np.float64)
    A = x["a"][::2048, 0, :].astype(np.float64)                     # (4, 256)
    B = x["b"][0].astype(np.float64)                                 # (512, 256)
    ga, gb = A != CI.F32_BAD, B != CI.F32_BAD
    scale = (np.abs(np.where(ga, A, 0))[:, None, :] *
             np.where(gb, np.abs(B), 0)[None, :, :] +
             np.where(ga, np.abs(A), 0)[:, None, :] * gb[None, :, :]).sum(-1)
    g = got[::2048].astype(np.float64)
    ok = want != CI.F32_BAD
    assert np.all(np.abs(g - want)[ok] <= (256 + 2) * 2 * EPS32 * scale[ok])


def test_c3_inner_against_pdl(gpu):
    x = CI.c3_inner()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c3i"]["input_sha256"]
    got = P.inner(P.pdl(x["a"]).to_device(), P.pdl(x["b"]).to_device()).numpy()[::8]
    scale = np.einsum("ij,ij->i", np.abs(x["a"][::8]), np.abs(x["b"][::8]))
    assert np.all(np.abs(got - FX["c3i/sample"]) <= (4096 + 2) * EPS64 * scale)


def test_c3_matmult_against_pdl(gpu):
    x = CI.c3_matmult()
    assert [CI.sha(x["a"]), CI.sha(x["b"])] == META["c3m"]["input_sha256"]
    pa, pb = P.pdl(x["a"]).to_device(), P.pdl(x["b"]).to_device()
    want = FX["c3m/sample"]
    As = x["a"][[0, 11]][:, ::256, :].astype(np.float64)
    scale = np.abs(As) @ np.abs(x["b"].astype(np.float64))
    try:
        P.set_matmult_mode(P.MATMULT_SIMT_EXACT)
        exact = P.matmult(pa, pb).numpy()[[0, 11]][:, ::256, :]
        P.set_matmult_mode(P.MATMULT_BF16X6)
        split = P.matmult(pa, pb).numpy()[[0, 11]][:, ::256, :]
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)
    assert np.array_equal(bits(exact), bits(want))                  # the reference's order
    assert np.all(np.abs(split.astype(np.float64) - want) <= (2 * 1024 + 8) * EPS32 * scale)


def test_c4_adjoints_against_gradients_by_hand_in_pdl(gpu):
    """The hand-written adjoint kernels (float32) on the adjoint workload
    against dL/dX, dL/dW, dL/dbias written out by hand in PDL (float64):
    normwise error (max |diff| / max |gradient|) within 2e-6."""
    x = CI.c4()
    assert [CI.sha(x[k]) for k in ("X", "W", "bias")] == META["c4"]["input_sha256"]
    X, W, b = (P.pdl(x[k]).to_device() for k in ("X", "W", "bias"))
    Y = P.matmult(X, W)
    Z = P.plus(Y, b)
    S = P.mult(Z, Z)
    s1 = P.sumover(S)
    gL = P.pdl(np.array(1.0 / 8192, np.float32)).to_device()
    g_s1 = P.sumover_bwd(gL, s1)
    g_S = P.sumover_bwd(g_s1, S)
    gz1, gz2 = P.mult_bwd(g_S, Z, Z)
    g_Y, g_b = P.plus_bwd(P.plus(gz1, gz2), Y, b)
    g_X, g_W = P.matmult_bwd(g_Y, X, W)
    got = {"gX": g_X.numpy()[::256], "gW": g_W.numpy()[::8], "gbias": g_b.numpy()}
    for k, g in got.items():
        want = FX[f"c4/{k}/sample"] if k != "gbias" else FX["c4/gbias"]
        nw = np.max(np.abs(g.astype(np.float64) - want)) / np.max(np.abs(want))
        assert nw <= 2e-6, (k, nw)
