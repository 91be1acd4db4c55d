"""GPU parity at the configurations' full sizes, through size-independent
properties and checks numpy can afford at these sizes:

* float32 stress workload (65536 x 4096 plus one row of 2^27, lognormal(0,4)
  magnitudes, random sign, 1 % BAD): compensated sums and averages against
  the float64 path, running sums against the float64 running sums at
  positions spread over every chunk of the chained scan, the last running
  sum of a row equal to its sum, bad masks of the running sums bit-exact;
* float64 (4096, 2048) family: minimum/maximum and their indices bit-exact
  against numpy, sums/averages/running sums within the sequential-sum bound,
  min <= average <= max;
* fused sumover(a*b+a), int32 (256,1,8192) x (256,512,1): bit-exact against
  an exact float64 matmul (every term and partial sum is an integer below
  2^53) wrapped to int32; the float32 version with 2 % BAD: bad
  mask exact (an output is BAD iff no good pair) and values within the bound;
* float64 inner over (4096, 65536) against numpy.

The float tolerance is the reference's own error bound for a sequential sum
in the accumulating type: |got - exact| <= (n + 2) * eps * sum|terms|."""
import numpy as np
import pytest

import pdl_gb300 as P

pytestmark = pytest.mark.gpu

F32_BAD = np.float32(-3.4028234663852886e38)
EPS32, EPS64 = 2.0 ** -24, 2.0 ** -53


def _c5_inputs():
    import config_inputs as CI
    d = CI.c5()
    return d["mat"], d["row"].reshape(-1)


@pytest.fixture(scope="module")
def c5():
    mat, row = _c5_inputs()
    xs = []
    for a in (mat, row):
        x = P.pdl(a)
        x.badflag(1)
        x.to_device()
        xs.append(x)
    return mat, row.reshape(1, -1), xs


def test_c5_sums_and_averages_match_float64_path(gpu, c5):
    mat, row, xs = c5
    for a, x in zip((mat, row), xs):
        good = a != F32_BAD
        absum = np.where(good, np.abs(a.astype(np.float64)), 0).sum(-1)
        cnt = good.sum(-1)
        n = a.shape[-1]
        s32 = P.sumover(x).numpy().astype(np.float64).reshape(-1)
        s64 = P.dsumover(x).numpy().reshape(-1)
        # compensated float32: the final rounding plus second-order terms
        # (n eps32^2 sum|a|), against the float64 path's own n eps64 sum|a|
        slack = 4 * n * (EPS32 ** 2 + EPS64) * absum
        assert np.all(np.abs(s32 - s64) <= 4 * EPS32 * np.abs(s64) + slack)
        av = P.average(x).numpy().astype(np.float64).reshape(-1)
        assert np.all(np.abs(av * cnt - s64) <= 8 * EPS32 * np.abs(s64) + slack + 1e-30)
        assert P.sumover(x).badflag() and P.average(x).badflag()


def test_c5_running_sums(gpu, c5):
    mat, row, xs = c5
    rng = np.random.default_rng(70)
    for a, x in zip((mat, row), xs):
        c32 = P.cumusumover(x).numpy().reshape(a.shape)
        c64 = P.dcumusumover(x).numpy().reshape(a.shape)
        bad = a == F32_BAD
        # bad inputs give bad outputs, good inputs never do (bit-exact mask)
        assert np.array_equal(c32 == F32_BAD, bad)
        assert np.array_equal(c64 == -np.finfo(np.float64).max, bad)
        # the last good running sum of each row equals the row's sum
        s64 = P.dsumover(x).numpy().reshape(-1)
        for r in range(a.shape[0]) if a.shape[0] <= 8 else rng.choice(a.shape[0], 8, replace=False):
            last = np.flatnonzero(~bad[r])[-1]
            assert abs(c64[r, last] - s64[r]) <= 1e-9 * np.abs(a[r][~bad[r]].astype(np.float64)).sum()
        # float32 running sums against the float64 ones at positions in every
        # chunk (16384 elements) of the row, normwise to the running sum of |a|
        n = a.shape[-1]
        pos = np.unique(np.concatenate([np.arange(0, n, 16384), np.arange(16383, n, 16384),
                                        rng.integers(0, n, 20000)]))
        rows = range(a.shape[0]) if a.shape[0] <= 8 else rng.choice(a.shape[0], 8, replace=False)
        for r in rows:
            absc = np.cumsum(np.where(bad[r], 0, np.abs(a[r].astype(np.float64))))
            g = ~bad[r][pos]
            err = np.abs(c32[r, pos].astype(np.float64) - c64[r, pos])[g]
            # a wrong chunk carry would be off by a chunk's total (~absc / chunks)
            bound = 4 * EPS32 * np.abs(c64[r, pos][g]) + 4 * n * EPS32 ** 2 * absc[pos][g] + 1e-30
            assert np.all(err <= bound)


@pytest.fixture(scope="module")
def c1():
    a = np.random.default_rng(1).uniform(-1.0, 1.0, size=(2048, 4096))
    return a, P.pdl(a).to_device()


def test_c1_family_full_size(gpu, c1):
    a, x = c1
    assert np.array_equal(P.minimum(x).numpy(), a.min(-1))
    assert np.array_equal(P.maximum(x).numpy(), a.max(-1))
    assert np.array_equal(P.minimum_ind(x).numpy(), a.argmin(-1))
    assert np.array_equal(P.maximum_ind(x).numpy(), a.argmax(-1))
    absum = np.abs(a).sum(-1)
    tol = (4096 + 2) * EPS64 * absum
    s = P.sumover(x).numpy()
    assert np.all(np.abs(s - np.sum(a, -1)) <= tol)
    av = P.average(x).numpy()
    assert np.all(np.abs(av - a.mean(-1)) <= tol / 4096 + 1e-300)
    assert np.all((P.minimum(x).numpy() <= av) & (av <= P.maximum(x).numpy()))
    cs = P.cumusumover(x).numpy()
    assert np.all(np.abs(cs - np.cumsum(a, -1)) <= (4096 + 2) * EPS64 * np.cumsum(np.abs(a), -1))
    # uniform[-1,1) products of 4096 terms underflow to zero in every row
    assert np.all(P.prodover(x).numpy() == 0)


def test_c2_int32_fused_exact_full_size(gpu):
    rng = np.random.default_rng(2)
    a = rng.integers(-1000, 1001, size=(8192, 1, 256)).astype(np.int32)   # PDL (256,1,8192)
    b = rng.integers(-1000, 1001, size=(1, 512, 256)).astype(np.int32)    # PDL (256,512,1)
    x, y = P.pdl(a).to_device(), P.pdl(b).to_device()
    got = P.sumover_mult_plus(x, y, x).numpy()                            # (8192, 512)
    # |terms| <= 1000 * 1001 and 256 of them: exact in float64 (BLAS), then
    # wrapped to int32 as the reference's int32 arithmetic would
    A = a[:, 0, :].astype(np.float64)                                     # (k, i)
    B1 = b[0].astype(np.float64).T + 1                                    # (i, j)
    want = (A @ B1).astype(np.int64)
    want = ((want + 2 ** 31) % 2 ** 32 - 2 ** 31).astype(np.int32)
    assert got.dtype == np.int32 and np.array_equal(got, want)


def test_c2_float32_bad_fused_full_size(gpu):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((8192, 1, 256)).astype(np.float32)
    b = rng.standard_normal((1, 512, 256)).astype(np.float32)
    a[rng.random(a.shape) < 0.02] = F32_BAD
    b[rng.random(b.shape) < 0.02] = F32_BAD
    x, y = P.pdl(a), P.pdl(b)
    x.badflag(1)
    y.badflag(1)
    x.to_device()
    y.to_device()
    c = P.sumover_mult_plus(x, y, x)
    got = c.numpy()
    A = a[:, 0, :].astype(np.float64)                                     # (k, i)
    B = b[0].astype(np.float64).T                                         # (i, j)
    ga, gb = (A != F32_BAD).astype(np.float64), (B != F32_BAD).astype(np.float64)
    Am = np.where(ga > 0, A, 0.0)
    Bm = np.where(gb > 0, B, 0.0)
    cnt = ga @ gb
    want = Am @ Bm + Am @ gb                                              # sum over good pairs of a*b + a
    scale = np.abs(Am) @ np.abs(Bm) + np.abs(Am) @ gb
    assert c.badflag()
    assert np.array_equal(got == F32_BAD, cnt == 0)
    ok = cnt > 0
    assert np.all(np.abs(got[ok].astype(np.float64) - want[ok]) <= (256 + 2) * 2 * EPS32 * scale[ok] + 1e-30)


def test_c3_inner_float64_full_size(gpu):
    rng = np.random.default_rng(5)
    a = rng.uniform(-1.0, 1.0, size=(65536, 4096))
    b = rng.uniform(-1.0, 1.0, size=(65536, 4096))
    got = P.inner(P.pdl(a).to_device(), P.pdl(b).to_device()).numpy()
    want = np.einsum("ij,ij->i", a, b)
    scale = np.einsum("ij,ij->i", np.abs(a), np.abs(b))
    assert np.all(np.abs(got - want) <= (4096 + 2) * EPS64 * scale)


def test_rows_beyond_2_31_elements(gpu):
    """64-bit indexing: one row of 2^31 + 77 bytes (2 GiB) through a sum,
    a max index past 2^31, a minimum, and an elementwise op over all of it."""
    n = (1 << 31) + 77
    a = np.zeros(n, np.uint8)
    a[[5, 1 << 31, n - 1]] = [1, 2, 3]
    x = P.pdl(a).to_device()
    assert P.sumover(x).numpy() == 6
    assert P.maximum_ind(x).numpy() == n - 1
    a[n - 1] = 0
    y = P.pdl(a).to_device()
    assert P.maximum_ind(y).numpy() == 1 << 31
    assert P.minimum(y).numpy() == 0
    z = P.plus(y, y)                                  # byte + byte, 2^31 + 77 outputs
    zs = P.sumover(z).numpy()
    assert zs == 2 * (1 + 2)
    del x, y, z
