"""The configurations at their full sizes on the GPU, checked against the CPU
oracle (the reference's own loops in C) on the same seeded inputs, not
against another GPU path.

* float64 (4096, 2048) uniform[-1,1) seed 1 (Ufunc family): every op of the
  family against the oracle over all 2048 rows.  minimum/maximum and their
  indices bit-exact; sums, averages and running sums within the reference's
  own bound for a sequential sum, (n+2)*eps*sum|a|; prodover bit for bit,
  the sign of each zero included (the reference stops at the first zero of
  its running product, lib/PDL/Ufunc.pd:107).
* float32 (65536, 4096) plus one row of 2^27, lognormal(0,4) magnitudes,
  random sign, 1 % BAD, seed 7 (accuracy stress): sumover, average,
  cumusumover, dsumover and dcumusumover on 64 sampled rows of the matrix
  and on the whole long row.  The oracle's float32 loop carries the
  reference's rounding error, (n+2)*eps32*sum|a|; the GPU's compensated
  float32 result is also held to the oracle's float64 loop within
  4*eps32*|s| + (n+2)*eps64*sum|a| (the compensated sum is correct to a few
  float32 ulps); bad masks bit-exact.
* float32 matmult a(t=1024, h=2048) batch 16 x b(w=2048, t=1024), N(0,1),
  seed 4: every element of every batch against an FP64 product (cuBLAS
  DGEMM through torch, whose own error is below 1e-12 here): bf16x6 within
  (K+8)*2^-24*(|A||B|) per element and 1e-6 normwise per batch; the FP32
  SIMT kernel within (K+2)*2^-24*(|A||B|); the exact kernel bit-identical
  to the oracle on 32 sampled rows of 2 batches (the reference accumulates
  t in order whatever the h and w tiles, so rows can be sampled)."""
import os

import numpy as np
import pytest

import pdl_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS32, EPS64 = 2.0 ** -24, 2.0 ** -53
F32_BAD = np.float32(-3.4028234663852886e38)
NTH = os.cpu_count() or 1


# ------------------------------------------------ float64 (4096, 2048) family

@pytest.fixture(scope="module")
def c1():
    a = np.random.default_rng(1).uniform(-1.0, 1.0, size=(2048, 4096))
    h = P.pdl(a)
    return a, h, P.pdl(a).to_device()


@pytest.mark.parametrize("op", ["minimum", "maximum", "minimum_ind", "maximum_ind",
                                "sumover", "dsumover", "average", "cumusumover", "prodover"])
def test_c1_family_against_the_oracle(gpu, c1, op):
    a, h, x = c1
    got = getattr(P, op)(x)
    exp = O.run(op, [h], nthreads=NTH)[0]
    assert got.type == exp.type and got.dims == exp.dims and got.badflag() == exp.badflag()
    g, e = got.numpy(), exp.numpy()
    if op in ("minimum", "maximum", "minimum_ind", "maximum_ind", "prodover"):
        # bit for bit (prodover: every row's running product underflows to a
        # signed zero before the end; the sign is the product's at that point)
        assert np.array_equal(g.view(np.uint64), e.view(np.uint64))
        if op == "prodover":
            assert np.all(e == 0)
        return
    absa = np.abs(a)
    scale = np.cumsum(absa, -1) if op == "cumusumover" else absa.sum(-1)
    if op == "average":
        scale = scale / 4096
    assert np.all(np.abs(g - e) <= (4096 + 2) * EPS64 * scale)


# --------------------------------- float32 (65536, 4096) + 2^27 row, 1 % BAD

def _c5():
    import config_inputs as CI
    d = CI.c5()
    return d["mat"], d["row"]


@pytest.fixture(scope="module")
def c5():
    mat, row = _c5()
    xs = []
    for a in (mat, row):
        x = P.pdl(a)
        x.badflag(1)
        xs.append(x.to_device())
    sample = np.sort(np.random.default_rng(77).choice(mat.shape[0], 64, replace=False))
    hs = []
    for a in (mat[sample], row):
        hx = P.pdl(np.ascontiguousarray(a))
        hx.badflag(1)
        hs.append(hx)
    return (mat, row), xs, hs, sample


@pytest.mark.parametrize("which", [0, 1], ids=["matrix_64_rows", "row_2e27"])
@pytest.mark.parametrize("op", ["sumover", "average", "dsumover"])
def test_c5_sums_against_the_oracle(gpu, c5, op, which):
    arrays, xs, hs, sample = c5
    a = arrays[which] if which else arrays[0][sample]
    good = a != F32_BAD
    absum = np.where(good, np.abs(a.astype(np.float64)), 0).sum(-1)
    cnt = good.sum(-1)
    n = a.shape[-1]
    g = getattr(P, op)(xs[which]).numpy().reshape(-1)
    if which == 0:
        g = g[sample]
    g = g.astype(np.float64)
    e = O.run(op, [hs[which]], nthreads=NTH)[0].numpy().reshape(-1).astype(np.float64)
    e64 = O.run("dsumover" if op != "average" else "daverage", [hs[which]],
                nthreads=NTH)[0].numpy().reshape(-1)
    div = cnt if op == "average" else 1
    if op == "dsumover":
        assert np.all(np.abs(g - e) <= (n + 2) * EPS64 * absum)
        return
    # against the oracle's float32 loop: the reference's own error bound
    assert np.all(np.abs(g - e) <= (n + 2) * EPS32 * absum / div)
    # against the oracle's float64 loop: compensated float32 is a few ulps off
    assert np.all(np.abs(g - e64) <= 4 * EPS32 * np.abs(e64) + (n + 2) * EPS64 * absum / div)


@pytest.mark.parametrize("which", [0, 1], ids=["matrix_64_rows", "row_2e27"])
def test_c5_running_sums_against_the_oracle(gpu, c5, which):
    arrays, xs, hs, sample = c5
    a = arrays[which] if which else arrays[0][sample]
    bad = a == F32_BAD
    g = P.cumusumover(xs[which]).numpy().reshape(-1, a.shape[-1])
    if which == 0:
        g = g[sample]
    e = O.run("cumusumover", [hs[which]], nthreads=NTH)[0].numpy().reshape(a.shape)
    e64 = O.run("dcumusumover", [hs[which]], nthreads=NTH)[0].numpy().reshape(a.shape)
    # bad inputs give bad outputs and nothing else does: bit-exact masks
    assert np.array_equal(g == F32_BAD, bad) and np.array_equal(e == F32_BAD, bad)
    absc = np.cumsum(np.where(bad, 0, np.abs(a.astype(np.float64))), -1)
    n = a.shape[-1]
    gd = g.astype(np.float64)[~bad]
    assert np.all(np.abs(gd - e.astype(np.float64)[~bad]) <= (n + 2) * EPS32 * absc[~bad])
    assert np.all(np.abs(gd - e64[~bad]) <= 4 * EPS32 * np.abs(e64[~bad]) + (n + 2) * EPS64 * absc[~bad])
    g64 = P.dcumusumover(xs[which]).numpy().reshape(-1, a.shape[-1])
    if which == 0:
        g64 = g64[sample]
    assert np.all(np.abs(g64[~bad] - e64[~bad]) <= (n + 2) * EPS64 * absc[~bad])


# ------------------------------------- float32 matmult, batch 16, full size

@pytest.fixture(scope="module")
def c3():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    T, H, W, NB = 1024, 2048, 2048, 16
    a = rng.standard_normal((NB, H, T)).astype(np.float32)   # PDL dims (t, h, batch)
    b = rng.standard_normal((T, W)).astype(np.float32)       # PDL dims (w, t)
    dev = torch.device("cuda", 0)
    A = torch.from_numpy(a).to(dev, torch.float64)
    B = torch.from_numpy(b).to(dev, torch.float64)
    ref = torch.matmul(A, B)                                  # (NB, H, W) FP64
    absref = torch.matmul(A.abs(), B.abs())
    return a, b, (P.pdl(a).to_device(), P.pdl(b).to_device()), ref, absref, torch


@pytest.mark.parametrize("mode,bound", [("bf16x6", 8), ("simt_fp32", 2)])
def test_c3_matmult_every_element(gpu, c3, mode, bound):
    a, b, (x, y), ref, absref, torch = c3
    P.set_matmult_mode({"bf16x6": P.MATMULT_BF16X6, "simt_fp32": P.MATMULT_SIMT_FP32}[mode])
    try:
        c = P.matmult(x, y)
        got = torch.from_numpy(c.numpy()).to(ref.device, torch.float64)
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)
    err = (got - ref).abs()
    assert not torch.isnan(got).any()
    # per element: (K + bound) * 2^-24 * (|A||B|)
    assert bool((err <= (1024 + bound) * EPS32 * absref).all())
    if mode == "bf16x6":
        normwise = (err.amax(dim=(1, 2)) / ref.abs().amax(dim=(1, 2))).max().item()
        assert normwise <= 1e-6, normwise


def test_c3_matmult_exact_mode_against_the_oracle(gpu, c3):
    a, b, (x, y), ref, absref, torch = c3
    rows = np.sort(np.random.default_rng(40).choice(2048, 32, replace=False))
    zs = [0, 11]
    P.set_matmult_mode(P.MATMULT_SIMT_EXACT)
    try:
        c = P.matmult(x, y).numpy()
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)
    hx = P.pdl(np.ascontiguousarray(a[zs][:, rows, :]))
    e = O.run("matmult", [hx, P.pdl(b)], nthreads=NTH)[0].numpy()
    assert np.array_equal(c[zs][:, rows, :].view(np.uint32), e.view(np.uint32))
