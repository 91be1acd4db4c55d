"""GPU parity: every op of the path through the C ABI against the oracle on
the same seeded inputs.

Bar: integer results, indices, bad masks and badflags bit-exact; float
results bit-exact where the GPU keeps the reference's order and rounding
(plus, mult, min/max, exact-mode matmult), otherwise within the stated
bound of the reference's own rounding error:
  sums / averages / running sums:  |g-e| <= (n+2) * eps * sum|a|
  products:                         |g-e| <= (n+2) * eps * |e|  (+ tiny)
  inner:                            |g-e| <= (n+2) * eps * sum|a*b|
where eps is the unit roundoff of the accumulating type (float32 results
are compared against the reference's plain float32 loop, which carries
that error; the GPU's compensated sum carries less)."""
import numpy as np
import pytest

import pdl_gb300 as P
from helpers import (FLOAT_TYPES, INT_TYPES, REAL_TYPES, assert_same, rand_array,
                     seeded, to_pdl)
from oracle import oracle as O
from pdl_gb300.ndarray import NP_DTYPES, type_code

pytestmark = pytest.mark.gpu

EPS = {"float": 2.0 ** -24, "double": 2.0 ** -53}
RED_OPS = ["sumover", "dsumover", "prodover", "dprodover", "average", "daverage",
           "minimum", "maximum", "minimum_ind", "maximum_ind", "cumusumover", "dcumusumover"]
SHAPES = [(7,), (1,), (0,), (0, 3), (5, 0), (3, 4), (17, 33, 2), (257, 5), (1500, 3),
          (4096, 12), (20000, 2)]


def _tol(op, x_np, exp, out_type):
    """(rtol, atol, scale) for float outputs."""
    n = x_np.shape[-1] if x_np.ndim else 1
    acc = "double" if op.startswith("d") or out_type == "double" else "float"
    eps = EPS[acc]
    a = np.abs(np.nan_to_num(x_np.astype(np.float64), nan=0.0, posinf=0, neginf=0))
    if op in ("sumover", "dsumover", "average", "daverage"):
        scale = a.sum(axis=-1) if a.ndim else a
        if op.endswith("average"):
            scale = scale / max(n, 1)
        return (n + 2) * eps, 1e-300, scale
    if op in ("cumusumover", "dcumusumover"):
        return (n + 2) * eps, 1e-300, np.cumsum(a, axis=-1)
    if op in ("prodover", "dprodover", "cumuprodover", "dcumuprodover"):
        return (n + 2) * eps, 1e-290 if acc == "double" else 1e-36, None
    return 0.0, 0.0, None


def _run_both(op, xs, **kw):
    fn = getattr(P, op)
    got = fn(*xs, **kw)
    exp = O.run(op, xs)[0]
    return got, exp


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", RED_OPS)
def test_reductions_all_types(gpu, op, t):
    rng = seeded((op, t))
    for shape in SHAPES:
        if op in ("prodover", "dprodover") and t in FLOAT_TYPES:
            lo, hi = -1.6, 1.6
        elif op in ("prodover", "dprodover"):
            lo, hi = -3, 3
        else:
            lo, hi = -100, 100
        a, _ = rand_array(rng, t, shape[::-1], lo, hi)
        x = to_pdl(a, t)
        got, exp = _run_both(op, [x])
        rtol, atol, scale = _tol(op, a, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
        assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} {shape}")


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", RED_OPS)
def test_reductions_bad_values(gpu, op, t):
    rng = seeded((op, t, "bad"))
    for shape in [(9, 4), (300, 7), (5000, 3), (3, 1)]:
        lo, hi = (-1.6, 1.6) if "prod" in op and t in FLOAT_TYPES else ((-3, 3) if "prod" in op else (-100, 100))
        a, bad = rand_array(rng, t, shape[::-1], lo, hi, bad_frac=0.2)
        a[0, :] = P.default_badvalue(type_code(t))  # an all-bad row
        x = to_pdl(a, t, badflag=True)
        got, exp = _run_both(op, [x])
        clean = np.where(bad | (a == P.default_badvalue(type_code(t))), 0, a)
        rtol, atol, scale = _tol(op, clean, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
        assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} bad {shape}")


@pytest.mark.parametrize("op", ["minimum", "maximum", "minimum_ind", "maximum_ind"])
@pytest.mark.parametrize("t", FLOAT_TYPES)
def test_minmax_nan_rules(gpu, op, t):
    rng = seeded(7)
    a, _ = rand_array(rng, t, (64, 333), -5, 5, special=True)
    a[3, :] = np.nan                        # all NaN: the last NaN's index
    a[4, ::2] = np.nan
    a[5, :] = 1.0                           # ties: the first index
    a[6, 10] = -0.0
    a[6, 11] = 0.0
    got, exp = _run_both(op, [to_pdl(a, t)])
    assert_same(got, exp, what=f"{op} {t}")


@pytest.mark.parametrize("t", ["double", "float", "long", "byte"])
@pytest.mark.parametrize("op", ["sumover", "minimum_ind", "cumusumover", "average", "prodover"])
def test_reductions_on_views(gpu, op, t):
    """vaffine inputs: transposed (strided n), reversed (negative incs),
    dummy (zero incs) and sliced views reach the kernels as increments."""
    rng = seeded(11)
    a, _ = rand_array(rng, t, (40, 30, 6), -3 if "prod" in op else -50, 3 if "prod" in op else 50)
    base = to_pdl(a, t)
    views = [base.xchg(0, 1), base.slice(slice(None, None, -1)), base.slice(slice(1, 29, 3), 4),
             base.dummy(1, 3), base.xchg(0, 2), base.slice(slice(None), slice(None, None, -2))]
    for v in views:
        got, exp = _run_both(op, [v])
        rtol, atol, scale = (0, 0, None)
        if exp.type in FLOAT_TYPES:
            rtol, atol, scale = _tol(op, v.numpy(), exp, exp.type)
        assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} view {v.dims}")


@pytest.mark.parametrize("op", ["sumover", "average", "minimum", "maximum_ind", "prodover",
                                "cumusumover", "dsumover"])
@pytest.mark.parametrize("t", ["double", "float", "long"])
def test_long_rows_split(gpu, op, t):
    """Few very long rows take the multi-block split (partials in scratch)."""
    rng = seeded(3)
    n = 300_000
    lo, hi = (-1.2, 1.2) if "prod" in op else (-10, 10)
    a, _ = rand_array(rng, t, (3, n), lo, hi)
    x = to_pdl(a, t)
    got, exp = _run_both(op, [x])
    rtol, atol, scale = _tol(op, a, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} split")


def test_device_resident_matches_host_staged(gpu):
    rng = seeded(5)
    a, _ = rand_array(rng, "double", (512, 1000), -1, 1)
    h = to_pdl(a, "double")
    d = to_pdl(a, "double").to_device()
    for op in ["sumover", "minimum_ind", "cumusumover"]:
        r1, r2 = getattr(P, op)(h), getattr(P, op)(d)
        assert r2.on_device
        assert np.array_equal(r1.numpy(), r2.numpy(), equal_nan=True), op


# ------------------------------------------------------------- plus / mult

BIOP_SHAPES = [((5,), (5,)), ((3, 4), (3, 1)), ((1,), (6, 2)), ((256, 1, 33), (256, 7, 1)),
               ((4, 1, 3), (1, 5, 1)), ((0, 3), (0, 1)), ((), (4,)), ((1000, 100), (1000, 100))]


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", ["plus", "mult"])
def test_biops_broadcast_exact(gpu, op, t):
    rng = seeded((op, t))
    for sa, sb in BIOP_SHAPES:
        a, _ = rand_array(rng, t, sa[::-1])
        b, _ = rand_array(rng, t, sb[::-1])
        x, y = to_pdl(a, t), to_pdl(b, t)
        for swap in (0, 1):
            got = getattr(P, op)(x, y, swap=swap)
            exp = O.run(op, [x, y], swap=swap)[0]
            assert_same(got, exp, what=f"{op} {t} {sa}x{sb} swap={swap}")


@pytest.mark.parametrize("t", ["float", "double", "long", "byte", "ulonglong"])
@pytest.mark.parametrize("op", ["plus", "mult"])
def test_biops_bad_values(gpu, op, t):
    rng = seeded(13)
    a, _ = rand_array(rng, t, (7, 50), bad_frac=0.1)
    b, _ = rand_array(rng, t, (1, 50), bad_frac=0.1)
    for fa, fb in [(1, 0), (0, 1), (1, 1)]:
        x, y = to_pdl(a, t, fa), to_pdl(b, t, fb)
        got = getattr(P, op)(x, y)
        exp = O.run(op, [x, y])[0]
        assert_same(got, exp, what=f"{op} {t} bad {fa}{fb}")


def test_biop_mixed_types_promote(gpu):
    x = P.pdl(np.array([1, 2, 250], np.uint8))
    y = P.pdl(np.array([1.5, 2.5, 3.5], np.float32))
    got, exp = P.plus(x, y), O.run("plus", [x, y])[0]
    assert_same(got, exp, what="byte+float")
    z = P.plus(x, x)  # byte arithmetic wraps
    assert z.type == "byte" and list(z.numpy()) == [2, 4, 244]


def test_biop_into_supplied_output_of_other_type(gpu):
    x = P.pdl(np.arange(6, dtype=np.int32))
    out = P.zeroes("double", 6)
    r = P.plus(x, x, out)
    assert r is out and list(out.numpy()) == [0, 2, 4, 6, 8, 10]


# -------------------------------------------------------------------- inner

@pytest.mark.parametrize("t", REAL_TYPES)
def test_inner_all_types(gpu, t):
    rng = seeded(("inner", t))
    for sa, sb in [((7,), (7,)), ((33, 5), (33,)), ((1, 4), (9, 4)), ((0,), (0,)),
                   ((3000, 6), (3000, 6)), ((20000,), (20000,))]:
        a, _ = rand_array(rng, t, sa[::-1], -20, 20)
        b, _ = rand_array(rng, t, sb[::-1], -20, 20)
        x, y = to_pdl(a, t), to_pdl(b, t)
        got, exp = P.inner(x, y), O.run("inner", [x, y])[0]
        if t in FLOAT_TYPES:
            n = max(sa[0], sb[0])
            ab = np.abs(np.broadcast_to(a.astype(np.float64), np.broadcast_shapes(a.shape, b.shape)) *
                        np.broadcast_to(b.astype(np.float64), np.broadcast_shapes(a.shape, b.shape)))
            scale = ab.sum(axis=-1) + np.abs(exp.numpy())
            assert_same(got, exp, rtol=(n + 2) * EPS[t], atol=1e-300, scale=scale, what=f"inner {t}")
        else:
            assert_same(got, exp, what=f"inner {t} {sa}")


@pytest.mark.parametrize("t", ["double", "float", "long"])
def test_inner_bad_and_views(gpu, t):
    rng = seeded(17)
    a, _ = rand_array(rng, t, (40, 64), -20, 20, bad_frac=0.01)
    b, _ = rand_array(rng, t, (40, 64), -20, 20)
    x, y = to_pdl(a, t, 1), to_pdl(b, t)
    got, exp = P.inner(x, y), O.run("inner", [x, y])[0]
    assert_same(got, exp, rtol=80 * EPS.get(t, 0), atol=1e-300,
                scale=np.abs(a.astype(np.float64) * b).sum(-1) if t in FLOAT_TYPES else None,
                what="inner bad")
    # views (transposed: strided n); values without badvalues, since a
    # badvalue read as data overflows (undefined in the reference's C)
    a, _ = rand_array(rng, t, (40, 64), -20, 20)
    xv = to_pdl(a, t).xchg(0, 1)
    yv = to_pdl(b, t).xchg(0, 1)
    got, exp = P.inner(xv, yv), O.run("inner", [xv, yv])[0]
    assert_same(got, exp, rtol=80 * EPS.get(t, 0), atol=1e-300,
                scale=np.abs(a.astype(np.float64) * b).sum(0) if t in FLOAT_TYPES else None,
                what="inner views")


# ------------------------------------------------------------------ matmult

MM_SHAPES = [((3, 4), (2, 3)), ((5, 5), (5, 5)), ((1, 7), (7, 1)), ((130, 129), (131, 130)),
             ((64, 200, 3), (150, 64)), ((17, 9, 2), (5, 17, 2)), ((8, 300), (260, 8))]


@pytest.mark.parametrize("t", REAL_TYPES)
def test_matmult_exact_all_types(gpu, t):
    """The exact SIMT kernel keeps the reference's t order and rounding
    (separately rounded product and sum): bit-identical for every type."""
    rng = seeded(("mm", t))
    P.set_matmult_mode(P.MATMULT_SIMT_EXACT)
    try:
        for sa, sb in MM_SHAPES:
            a, _ = rand_array(rng, t, sa[::-1], -8, 8)
            b, _ = rand_array(rng, t, sb[::-1], -8, 8)
            x, y = to_pdl(a, t), to_pdl(b, t)
            got, exp = P.matmult(x, y), O.run("matmult", [x, y])[0]
            assert_same(got, exp, what=f"matmult {t} {sa}x{sb}")
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)


def test_matmult_float_with_bad_uses_exact_kernel(gpu):
    rng = seeded(19)
    # float32 with the badflag set runs the exact kernel in every mode
    for sa, sb in MM_SHAPES:
        a, _ = rand_array(rng, "float", sa[::-1], -8, 8)
        b, _ = rand_array(rng, "float", sb[::-1], -8, 8)
        x, y = to_pdl(a, "float", 1), to_pdl(b, "float")
        got, exp = P.matmult(x, y), O.run("matmult", [x, y])[0]
        assert_same(got, exp, what=f"matmult float exact {sa}x{sb}")


@pytest.mark.parametrize("t", ["double", "float", "long"])
def test_matmult_bad_values(gpu, t):
    rng = seeded(23)
    a, _ = rand_array(rng, t, (20, 30), -5, 5, bad_frac=0.01)
    b, _ = rand_array(rng, t, (30, 25), -5, 5, bad_frac=0.01)
    x, y = to_pdl(a, t, 1), to_pdl(b, t, 1)
    got, exp = P.matmult(x, y), O.run("matmult", [x, y])[0]
    assert_same(got, exp, what=f"matmult bad {t}")


def test_matmult_simt_fp32_within_tolerance(gpu):
    rng = seeded(29)
    a = rng.standard_normal((300, 200)).astype(np.float32)
    b = rng.standard_normal((200, 100)).astype(np.float32)
    x, y = P.pdl(a), P.pdl(b)
    P.set_matmult_mode(P.MATMULT_SIMT_FP32)
    try:
        got = P.matmult(x, y).numpy().astype(np.float64)
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)
    ref = a.astype(np.float64) @ b.astype(np.float64)
    bound = (200 + 2) * EPS["float"] * (np.abs(a).astype(np.float64) @ np.abs(b))
    assert np.all(np.abs(got - ref) <= bound)


# ----------------------------------------------------- fused sumover(a*b+d)

def test_fused_int32_outer_exact(gpu):
    rng = seeded(31)
    a, _ = rand_array(rng, "long", (40, 1, 96), -1000, 1000)   # numpy order of dims (96,1,40)
    b, _ = rand_array(rng, "long", (1, 70, 96), -1000, 1000)
    x, y = to_pdl(a, "long"), to_pdl(b, "long")
    got = P.sumover_mult_plus(x, y, x)
    t = O.run("mult", [x, y])[0]
    u = O.run("plus", [t, x])[0]
    exp = O.run("sumover", [u])[0]
    assert_same(got, exp, what="fused int32")
    assert "outer" in P.last_launch_info()["kernel"]


@pytest.mark.parametrize("t", ["float", "double", "short", "ulong"])
def test_fused_generic_and_bad(gpu, t):
    rng = seeded(37)
    for fa, fb, fd in [(0, 0, 0), (1, 0, 0), (1, 1, 1)]:
        a, _ = rand_array(rng, t, (20, 1, 33), -50, 50, bad_frac=0.02 if fa else 0)
        b, _ = rand_array(rng, t, (1, 9, 33), -50, 50, bad_frac=0.02 if fb else 0)
        d, _ = rand_array(rng, t, (20, 1, 33), -50, 50, bad_frac=0.02 if fd else 0)
        x, y, z = to_pdl(a, t, fa), to_pdl(b, t, fb), to_pdl(d, t, fd)
        got = P.sumover_mult_plus(x, y, z)
        tt = O.run("mult", [x, y])[0]
        u = O.run("plus", [tt, z])[0]
        exp = O.run("sumover", [u])[0]
        scale = None
        if t in FLOAT_TYPES:
            un = np.abs(np.nan_to_num(u.numpy().astype(np.float64)))
            un[u.numpy() == P.default_badvalue(type_code(t))] = 0
            scale = un.sum(-1)
        assert_same(got, exp, rtol=40 * EPS.get(t, 0), atol=1e-300, scale=scale,
                    what=f"fused {t} {fa}{fb}{fd}")


# ------------------------------------------------------------ conversions

@pytest.mark.parametrize("src", REAL_TYPES)
def test_convert_matches_c_casts(gpu, src):
    rng = seeded(41)
    a, _ = rand_array(rng, src, (3, 37), -100, 100)
    x = to_pdl(a, src)
    for dst in REAL_TYPES:
        got = P.convert(x, dst).numpy()
        if np.dtype(NP_DTYPES[type_code(dst)]).kind == "u" and a.dtype.kind == "f":
            want = a.astype(np.int64).astype(NP_DTYPES[type_code(dst)])
        else:
            want = a.astype(NP_DTYPES[type_code(dst)])
        assert np.array_equal(got, want), (src, dst)


@pytest.mark.parametrize("t,n,rows", [("float", (1 << 21) + 123, 1), ("float", 9004, 5),
                                      ("double", 300_007, 2), ("long", 3 * 8192 + 4, 3),
                                      ("longlong", 70_000, 2), ("float", 65536, 40)])
@pytest.mark.parametrize("op", ["cumusumover", "dcumusumover"])
def test_chained_scan_rows(gpu, op, t, n, rows):
    """Contiguous aligned rows of 4/8-byte types run the chained single-pass
    scan: several chunks per row (look-back inside the row), a row of 257
    chunks (three look-back rounds of 128), ragged last chunks."""
    rng = seeded(n + rows)
    a, _ = rand_array(rng, t, (rows, n), -10, 10)
    x = to_pdl(a, t)
    got, exp = _run_both(op, [x])
    rtol, atol, scale = _tol(op, a, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} {rows}x{n}")


@pytest.mark.parametrize("t", ["float", "double", "long"])
@pytest.mark.parametrize("nanbad", [False, True])
def test_chained_scan_bad_values(gpu, t, nanbad):
    rng = seeded(21)
    a, bad = rand_array(rng, t, (3, 50_000), -10, 10, bad_frac=0.05)
    x = to_pdl(a, t, badflag=True)
    if nanbad:
        if t == "long":
            pytest.skip("NaN badvalue is for float types")
        arr = x.numpy().copy()
        arr[bad] = np.nan
        x = to_pdl(arr, t, badflag=True)
        x.badvalue(float("nan"))
    got, exp = _run_both("cumusumover", [x])
    clean = np.where(bad, 0, a)
    rtol, atol, scale = _tol("cumusumover", clean, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"cumusumover {t} bad nan={nanbad}")


@pytest.mark.parametrize("t,n,rows", [("float", 16_400, 3700), ("double", 8_194, 3700),
                                      ("long", 16_384, 3700)])
def test_row_block_scan_many_rows(gpu, t, n, rows):
    """Many rows of equally wide types run a block per row, the row's chunks
    in order with the carry in registers (two or more chunks per row,
    ragged row ends, 1 % BAD); float32 into float64 (dcumusumover) keeps the
    chained scan."""
    rng = seeded(n + rows + 7)
    a, bad = rand_array(rng, t, (rows, n), -10, 10, bad_frac=0.01)
    x = to_pdl(a, t, badflag=True)
    got, exp = _run_both("cumusumover", [x])
    assert P.last_launch_info()["kernel"] == "k_scan_rowblk"
    clean = np.where(bad, 0, a)
    rtol, atol, scale = _tol("cumusumover", clean, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"cumusumover {t} {rows}x{n}")
    if t == "float":
        P.dcumusumover(x)
        assert P.last_launch_info()["kernel"] == "k_scan_chain"


def test_chained_scan_unaligned_rows_fall_back(gpu):
    """Rows whose starts are not 16-byte aligned take the warp kernel."""
    rng = seeded(22)
    a, _ = rand_array(rng, "float", (4, 20_001), -10, 10)
    x = to_pdl(a, "float").slice(slice(1, None))
    got, exp = _run_both("cumusumover", [x])
    rtol, atol, scale = _tol("cumusumover", x.numpy(), exp, exp.type)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what="cumusumover unaligned")


@pytest.mark.parametrize("t", FLOAT_TYPES)
@pytest.mark.parametrize("op", ["prodover", "dprodover"])
def test_prodover_stops_at_first_zero(gpu, op, t):
    """The reference's loop breaks once the running product is zero
    (Ufunc.pd:107): inf or NaN after a zero leave it zero, a zero after an
    inf gives NaN, and the zero's sign is the running product's at the
    break.  Covers the row kernel, the split kernel and strided views."""
    dt = NP_DTYPES[type_code(t)]
    rows = np.array([[2, 0, np.nan, 5, 1],
                     [3, -0.0, -1, -2, 1],
                     [np.inf, 0, 1, 1, 1],
                     [-1, 1, 0, np.inf, -7],
                     [1, 2, 3, 4, 5],
                     [0, 0, np.nan, 0, 1]], dtype=dt)
    long = np.full((2, 300_000), 1.0, dtype=dt)
    long[0, 100_000] = -0.0
    long[0, 200_000] = np.nan
    long[1, 250_000] = 0.0
    long[1, 10] = -1.0
    long[1, 299_999] = np.inf
    for a in [rows, long, np.ascontiguousarray(rows.T)]:
        x = to_pdl(a, t)
        for v in [x, x.xchg(0, 1)] if a is not long else [x]:
            got, exp = _run_both(op, [v])
            g, e = got.numpy(), exp.numpy()
            assert np.array_equal(np.isnan(g), np.isnan(e)), f"{op} {t}: NaN\n{g}\n{e}"
            fin = ~np.isnan(e)
            np.testing.assert_allclose(g[fin], e[fin], rtol=1e-6)
            zero = fin & (e == 0)
            assert np.array_equal(np.signbit(g[zero]), np.signbit(e[zero])), f"{op} {t}: sign of 0"


@pytest.mark.parametrize("t", FLOAT_TYPES)
@pytest.mark.parametrize("op", ["prodover", "dprodover"])
def test_products_leaving_the_normal_range_are_the_references(gpu, op, t):
    """Rows whose running product overflows, underflows (to a subnormal and
    to zero), or comes back into range, with zeros, infs, NaNs and bad
    values before and after the sequential prefix (2048 or 4096 elements):
    the result is the reference's loop's, bit for bit (NaN positions
    equal, zeros' signs equal)."""
    dt = NP_DTYPES[type_code(t)]
    rng = seeded(("leave", op, t))
    big = 1e30 if t == "float" else 1e200
    rows = []
    for n in (100, 3000, 5000, 9000):
        base = rng.uniform(0.9, 1.1, n) * np.where(rng.random(n) < 0.5, -1, 1)
        for k in range(6):
            r = base.copy()
            p = int(rng.integers(0, n))
            if k == 0:
                r[p], r[min(p + 1, n - 1)] = big, big          # overflow, stays inf
            elif k == 1:
                r[p], r[min(p + 1, n - 1)] = 1 / big, 1 / big  # underflow to 0 (stops)
            elif k == 2:
                r[p] = big
                r[min(p + 3, n - 1)] = 1 / big                 # back in range
            elif k == 3:
                r[p] = 0.0
                r[min(p + 5, n - 1)] = np.inf                  # zero then inf: stays 0
            elif k == 4:
                r[p], r[min(p + 1, n - 1)] = big, big
                r[min(p + 9, n - 1)] = 0.0                     # inf then 0: NaN
            else:
                r[:] = rng.uniform(-1, 1, n)                   # drifts to a signed 0
            rows.append(r)
    width = max(len(r) for r in rows)
    for r in rows:
        a = np.ones((1, width))
        a[0, :len(r)] = r
        x = to_pdl(a.astype(dt), t)
        got, exp = _run_both(op, [x])
        g, e = got.numpy(), exp.numpy()
        what = f"{op} {t} n={len(r)}"
        assert np.array_equal(np.isnan(g), np.isnan(e)), what
        fin = ~np.isnan(e)
        bits = np.uint64 if g.dtype.itemsize == 8 else np.uint32
        if not np.isfinite(e[fin]).all() or (e[fin] == 0).any():
            assert np.array_equal(g[fin].view(bits), e[fin].view(bits)), f"{what}: {g} {e}"
        else:
            np.testing.assert_allclose(g[fin], e[fin], rtol=(width + 2) * EPS["double" if op == "dprodover" else t])
    # the same rows together, and with 5 % bad values
    a = np.ones((len(rows), width))
    for i, r in enumerate(rows):
        a[i, :len(r)] = r
    a = a.astype(dt)
    for badfrac in (0.0, 0.05):
        b = a.copy()
        if badfrac:
            b[rng.random(b.shape) < badfrac] = P.default_badvalue(type_code(t))
        x = to_pdl(b, t, badflag=bool(badfrac))
        got, exp = _run_both(op, [x])
        g, e = got.numpy(), exp.numpy()
        assert np.array_equal(np.isnan(g), np.isnan(e))
        special = ~np.isnan(e) & (~np.isfinite(e) | (e == 0))
        bits = np.uint64 if g.dtype.itemsize == 8 else np.uint32
        assert np.array_equal(g[special].view(bits), e[special].view(bits))


def test_prodover_zero_in_bad_and_integer_rows(gpu):
    rng = seeded(31)
    a, bad = rand_array(rng, "double", (4, 5000), 0.9, 1.1, bad_frac=0.1)
    a[1, 100] = 0.0
    a[1, 101] = np.nan
    a[2, 7] = 0.0
    a[2, :7] = P.default_badvalue(type_code("double"))
    x = to_pdl(a, "double", badflag=True)
    got, exp = _run_both("prodover", [x])
    assert np.array_equal(np.isnan(got.numpy()), np.isnan(exp.numpy()))
    np.testing.assert_allclose(got.numpy(), exp.numpy(), rtol=1e-9)
    ai, _ = rand_array(rng, "long", (3, 4000), -3, 3)
    ai[0, 5] = 0
    for op in ["prodover", "dprodover"]:
        got, exp = _run_both(op, [to_pdl(ai, "long")])
        if exp.type in FLOAT_TYPES:
            np.testing.assert_allclose(got.numpy(), exp.numpy(), rtol=1e-9)
        else:
            assert_same(got, exp, what=f"{op} long")


def test_float64_products_bit_exact_over_the_exponent_range(gpu):
    """float64 products are formed on the integer pipe for normal operands
    (hardware multiply for zeros, subnormals, inf, NaN and the underflow
    range): bit-identical to IEEE round-to-nearest, through mult and through
    inner with n=1 (whose output is the rounded product)."""
    rng = np.random.default_rng(41)
    n = 1 << 21
    bits = rng.integers(0, 2 ** 63, size=(4, n), dtype=np.int64).astype(np.uint64)
    bits[:, ::2] ^= np.uint64(1) << np.uint64(63)                      # both signs
    bits[1] = (bits[1] & np.uint64(0x800FFFFFFFFFFFFF)) | (
        rng.integers(1023 - 40, 1023 + 40, size=n).astype(np.uint64) << np.uint64(52))
    bits[2] &= ~np.uint64(0xFFFFFFF)                                     # short significands: ties
    bits[3] = (bits[3] & np.uint64(0x800FFFFFFFFFFFFF)) | (
        rng.integers(0, 60, size=n).astype(np.uint64) << np.uint64(52))  # near underflow, subnormal
    a = bits.view(np.float64).reshape(-1)
    b = np.roll(a, 12345)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.2250738585072014e-308,
                        1.7976931348623157e308, 1.0, -1.0])
    a = np.concatenate([a, np.repeat(special, len(special))])
    b = np.concatenate([b, np.tile(special, len(special))])
    with np.errstate(all="ignore"):
        want = a * b
    got = P.mult(P.pdl(a), P.pdl(b)).numpy()
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{(~same).sum()} products differ, e.g. {a[~same][:3]} x {b[~same][:3]}"
    got = P.inner(P.pdl(a.reshape(-1, 1)), P.pdl(b.reshape(-1, 1))).numpy().reshape(-1)
    want = want + 0.0  # the reference's tmp = 0; tmp += a*b turns -0 into +0
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"inner n=1: {(~same).sum()} products differ"


def _golden_gpu(case):
    from helpers import make_input
    ins = [make_input(s) for s in case["inputs"]]
    if case.get("view") == "xchg01":
        ins[0] = ins[0].xchg(0, 1)
    if case.get("view") == "dim1_index1":
        ins[0] = ins[0].slice(slice(None), 1)
    if "whole" in case:
        return getattr(P, case["whole"])(*ins)
    out = None
    if "out" in case:
        kind, dims = case["out"].split(":")
        dims = [int(d) for d in dims.split(",")]
        out = (P.zeroes if kind == "zeroes" else P.ones)("double", *dims)
    if case["op"] == "matmult":
        return P.matmult(ins[0], ins[1], out)
    fn = getattr(P, case["op"])
    if case.get("nout", 1) > 1:
        return fn(*ins)[case.get("pick", 0)]
    if case["op"] in P_BIOPS:
        return fn(ins[0], ins[1], out, swap=case.get("swap", 0))
    if case["op"] in P_TWO_IN:
        return fn(ins[0], ins[1], out)
    return fn(*ins, out) if out is not None else fn(*ins)


P_BIOPS = {"plus", "mult", "minus", "divide", "gt", "lt", "le", "ge", "eq", "ne",
           "shiftleft", "shiftright", "or2", "and2", "xor"}
P_TWO_IN = {"pctover", "oddpctover"}


def test_golden_vectors_on_the_gpu(gpu):
    """Every known answer from the reference's own tests, through the GPU
    library (the oracle passes the same cases in test_oracle_golden.py)."""
    from helpers import golden_cases
    from test_oracle_golden import check_result
    for case in golden_cases():
        if "expect_error" in case:
            with pytest.raises(P.PDLError, match=case["expect_error"]):
                _golden_gpu(case)
            continue
        check_result(case, _golden_gpu(case))


NEW_BIOPS = ["minus", "divide", "gt", "lt", "le", "ge", "eq", "ne"]
BIT_OPS = ["shiftleft", "shiftright", "or2", "and2", "xor"]


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", NEW_BIOPS + BIT_OPS)
def test_more_binary_ops_exact(gpu, op, t):
    """The other binary ops of Ops.pd against the oracle, bit-exact, under
    broadcasting, with swap, a supplied output and bad values.  Integer
    divisors are nonzero and shift counts in [0, 7] with non-negative
    values (elsewhere the reference's C has no defined result)."""
    rng = seeded((op, t))
    dt = np.dtype(NP_DTYPES[type_code(t)])
    for sa, sb in [((37, 5), (37, 5)), ((1, 64), (9, 64)), ((7, 1, 33), (1, 4, 33)), ((1,), (6,))]:
        a, _ = rand_array(rng, t, sa, -100, 100)
        b, _ = rand_array(rng, t, sb, -100, 100)
        if op in BIT_OPS:
            a = np.abs(a.astype(np.float64)).astype(dt)
        if op in ("shiftleft", "shiftright"):
            b = (np.abs(b.astype(np.int64)) % 8).astype(dt)
        if op == "divide" and dt.kind != "f":
            b = np.where(b == 0, 1, b).astype(dt)
        if op == "divide" and dt.kind == "f":
            b.reshape(-1)[::5] = 0  # IEEE inf / NaN
        for swap in (0, 1):
            if swap and (op in ("shiftleft", "shiftright") or (op == "divide" and dt.kind != "f")):
                continue  # the swapped operand would be a shift count / integer divisor
            x, y = to_pdl(a, t), to_pdl(b, t)
            got = getattr(P, op)(x, y, swap=swap)
            exp = O.run(op, [x, y], swap=swap)[0]
            assert_same(got, exp, what=f"{op} {t} {sa}x{sb} swap={swap}")
    # bad values propagate (bit-exact masks and badflag)
    a, _ = rand_array(rng, t, (50, 8), -100, 100, bad_frac=0.1)
    b, _ = rand_array(rng, t, (50, 8), 1, 100)
    if op in ("shiftleft", "shiftright"):
        b = (np.abs(b.astype(np.int64)) % 8).astype(dt)
    if op in BIT_OPS:
        a = np.where(a == P.default_badvalue(type_code(t)), a, np.abs(a.astype(np.float64))).astype(dt)
    x, y = to_pdl(a, t, badflag=True), to_pdl(b, t)
    got = getattr(P, op)(x, y)
    exp = O.run(op, [x, y])[0]
    assert_same(got, exp, what=f"{op} {t} bad")


@pytest.mark.parametrize("op", BIT_OPS)
def test_bit_ops_on_floats_work_in_longlong(gpu, op):
    x, y = P.pdl(np.array([1.0, 2.0, 3.0])), P.pdl(np.array([4.0, 5.0, 1.0]))
    got = getattr(P, op)(x, y)
    exp = O.run(op, [x, y])[0]
    assert got.type == "longlong"
    assert_same(got, exp, what=op)


LOGIC_OPS = ["andover", "orover", "xorover", "zcover", "firstnonzeroover"]
BITOVER_OPS = ["bandover", "borover", "bxorover"]


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", LOGIC_OPS + BITOVER_OPS)
def test_logical_and_bitwise_reductions(gpu, op, t):
    """Ufunc.pd:143-187 against the oracle, bit-exact: sparse zeros so the
    logical results vary, rows of every kernel path (warp rows, block rows,
    split long rows, strided views), bad values with all-bad rows."""
    rng = seeded((op, t, "logic"))
    for shape in [(7,), (0,), (3, 0), (33, 17), (2049, 6), (300_000, 2)]:
        a, _ = rand_array(rng, t, shape[::-1], -3, 3)
        x = to_pdl(a, t)
        got, exp = _run_both(op, [x])
        assert_same(got, exp, what=f"{op} {t} {shape}")
    a, _ = rand_array(rng, t, (30, 40, 5), -3, 3)
    got, exp = _run_both(op, [to_pdl(a, t).xchg(0, 1)])
    assert_same(got, exp, what=f"{op} {t} strided")
    a, bad = rand_array(rng, t, (12, 900), -3, 3, bad_frac=0.3)
    a[0, :] = P.default_badvalue(type_code(t))
    got, exp = _run_both(op, [to_pdl(a, t, badflag=True)])
    assert_same(got, exp, what=f"{op} {t} bad")


def test_firstnonzeroover_zero_rows_keep_the_last_zero(gpu):
    a = np.array([[0.0, -0.0, 0.0, -0.0], [0.0, 0.0, -0.0, 3.0], [np.nan, 1.0, 0.0, 0.0]])
    x = P.pdl(a)
    got, exp = _run_both("firstnonzeroover", [x])
    g, e = got.numpy(), exp.numpy()
    assert np.array_equal(np.isnan(g), np.isnan(e))
    assert np.array_equal(g[~np.isnan(g)], e[~np.isnan(e)])
    assert np.array_equal(np.signbit(g), np.signbit(e))


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", ["cumuprodover", "dcumuprodover"])
def test_running_products(gpu, op, t):
    """cumuprodover (Ufunc.pd:120-140 with *=) against the oracle: integers
    wrap exactly whatever the order; floats near 1 in magnitude (no
    underflow or overflow on the way) within (n+2) eps |p|; rows of every
    scan path (thread rows, warp rows, the chained scan over many chunks),
    bad values."""
    rng = seeded((op, t, "cumuprod"))
    dt = np.dtype(NP_DTYPES[type_code(t)])
    for shape in [(7,), (0,), (33, 17), (4100, 3), (70_000, 2)]:
        if dt.kind == "f":
            a = (rng.uniform(0.999, 1.001, size=shape[::-1]) *
                 np.where(rng.random(shape[::-1]) < 0.5, -1, 1)).astype(dt)
        else:
            a, _ = rand_array(rng, t, shape[::-1], -3, 3)
        x = to_pdl(a, t)
        got, exp = _run_both(op, [x])
        rtol, atol, scale = _tol(op, a, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
        assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} {shape}")
    a, _ = rand_array(rng, t, (9, 300), -3 if dt.kind != "f" else 0.9, 3 if dt.kind != "f" else 1.1,
                      bad_frac=0.1)
    x = to_pdl(a, t, badflag=True)
    got, exp = _run_both(op, [x])
    rtol, atol, scale = _tol(op, a, exp, exp.type) if exp.type in FLOAT_TYPES else (0, 0, None)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what=f"{op} {t} bad")
    got, exp = _run_both(op, [to_pdl(a, t, badflag=True).xchg(0, 1)])
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale if scale is None else None,
                what=f"{op} {t} strided")


def _mm4_both(x):
    got = P.minmaximum(x)
    exp = O.run("minmaximum", [x], [None] * 4)
    return got, exp


@pytest.mark.parametrize("t", REAL_TYPES)
def test_minmaximum(gpu, t):
    """minmaximum (Ufunc.pd:563-613) against the oracle, all four outputs
    bit-exact: ties keep the first index, NaN and bad elements are skipped,
    a row with nothing left (empty, all NaN, all bad) sets every output BAD
    and their bad flags; views and rows longer than a warp's stride."""
    rng = seeded(("minmaximum", t))
    dt = np.dtype(NP_DTYPES[type_code(t)])
    for shape in [(7,), (1,), (33, 17), (3, 4, 5), (2049, 6), (100_000, 2)]:
        a, _ = rand_array(rng, t, shape[::-1], -5, 5)
        x = to_pdl(a, t)
        got, exp = _mm4_both(x)
        for k in range(4):
            assert_same(got[k], exp[k], what=f"minmaximum {t} {shape} out {k}")
    for shape in [(0,), (0, 3)]:
        x = to_pdl(np.zeros(shape[::-1], dt), t)
        got, exp = _mm4_both(x)
        for k in range(4):
            assert_same(got[k], exp[k], what=f"minmaximum {t} empty {shape} out {k}")
            assert got[k].badflag()
    a, _ = rand_array(rng, t, (30, 40, 5), -5, 5)
    got, exp = _mm4_both(to_pdl(a, t).xchg(0, 1))
    for k in range(4):
        assert_same(got[k], exp[k], what=f"minmaximum {t} strided out {k}")
    a, _ = rand_array(rng, t, (12, 900), -5, 5, bad_frac=0.3)
    a[0, :] = P.default_badvalue(type_code(t))
    got, exp = _mm4_both(to_pdl(a, t, badflag=True))
    for k in range(4):
        assert_same(got[k], exp[k], what=f"minmaximum {t} bad out {k}")
    assert got[0].badflag()
    if dt.kind == "f":
        a, _ = rand_array(rng, t, (8, 333), -5, 5, special=True)
        a[3, :] = np.nan
        a[5, :] = 1.0
        a[6, 10], a[6, 11] = -0.0, 0.0
        got, exp = _mm4_both(to_pdl(a, t))
        for k in range(4):
            assert_same(got[k], exp[k], what=f"minmaximum {t} NaN out {k}")
            assert got[k].badflag()


def test_minmaximum_doc_example(gpu):
    # Ufunc.pd:597-600: [[-2,3,4],[1,0,3]] -> [-2 0] [4 3] [0 1] [2 2]
    cmin, cmax, imin, imax = P.minmaximum(P.pdl(np.array([[-2.0, 3, 4], [1, 0, 3]])))
    assert cmin.numpy().tolist() == [-2, 0] and cmax.numpy().tolist() == [4, 3]
    assert imin.numpy().tolist() == [0, 1] and imax.numpy().tolist() == [2, 2]
    assert not cmin.badflag() and imin.type == "indx"


WHOLE = [("sum", "sumover"), ("avg", "average"), ("prod", "prodover"), ("dsum", "dsumover"),
         ("davg", "daverage"), ("dprod", "dprodover"), ("zcheck", "zcover"), ("and_", "andover"),
         ("band", "bandover"), ("or_", "orover"), ("bor", "borover"), ("xorall", "xorover"),
         ("bxor", "bxorover"), ("min", "minimum"), ("max", "maximum")]


@pytest.mark.parametrize("t", ["byte", "long", "longlong", "float", "double"])
def test_whole_array_reductions(gpu, t):
    """Ufunc.pd:615-663: each whole-array function is flat then the
    reduction over dim 0; against the oracle on the flattened ndarray,
    including a view whose dims do not merge (flat makes a device copy) and
    bad values.  Sums and products of floats within the sequential bound."""
    rng = seeded(("whole", t))
    a, _ = rand_array(rng, t, (6, 5, 7), -3, 3)
    x = to_pdl(a, t)
    ab, _ = rand_array(rng, t, (40, 50), -3, 3, bad_frac=0.2)
    xb = to_pdl(ab, t, badflag=True)
    for name, op in WHOLE:
        if op in ("bandover", "borover", "bxorover") and t in ("float", "double"):
            cases = [(x, x.flat())]
        else:
            cases = [(x, x.flat()), (xb, xb.flat())]
        # a strided view: dims (7, 6) of the (7, 5, 6) ndarray at index 2 of dim 1
        v = x.slice(slice(None), 2)
        cases.append((v, P.pdl(np.ascontiguousarray(v.numpy()))))
        cases.append((x.xchg(0, 2), P.pdl(np.ascontiguousarray(x.xchg(0, 2).numpy()))))
        for src, flat in cases:
            got = getattr(P, name)(src.to_device() if src is x else src)
            exp = O.run(op, [flat.flat()])[0]
            assert got.dims == () and exp.dims == ()
            if op in ("prodover", "dprodover") and t in ("float", "double"):
                n = flat.nelem
                assert_same(got, exp, rtol=(n + 2) * EPS[t], atol=1e-300, what=f"{name} {t}")
            elif op in ("sumover", "average", "dsumover", "daverage") and t in ("float", "double"):
                n = flat.nelem
                absum = np.abs(flat.numpy().astype(np.float64)).sum()
                eps = EPS["double"] if op.startswith("d") else EPS[t]
                assert_same(got, exp, atol=(n + 2) * eps * absum, what=f"{name} {t}")
            else:
                assert_same(got, exp, what=f"{name} {t}")


SORT_OPS = ["qsort", "qsorti", "medover", "oddmedover"]


def _bits_equal(got, exp, what):
    assert got.type == exp.type and got.dims == exp.dims, what
    assert got.badflag() == exp.badflag(), what
    g, e = np.atleast_1d(got.numpy()), np.atleast_1d(exp.numpy())
    if g.dtype.kind == "f":
        # NaN produced by arithmetic has a hardware-defined payload (the
        # GPU's canonical NaN, x86's default NaN): compare NaN positions,
        # then every other element bit for bit (signed zeros included)
        gn, en = np.isnan(g), np.isnan(e)
        assert np.array_equal(gn, en), f"{what}: NaN positions differ"
        g, e = np.where(gn, 0, g), np.where(en, 0, e)
    assert np.array_equal(g.view(np.uint8), e.view(np.uint8)), (
        f"{what}: got {g.ravel()[:12]} exp {e.ravel()[:12]}")


def _sort_data(rng, t, shape, bad_frac=0.0):
    """Few distinct values (ties), and for floats NaN and both zeros."""
    a, bad = rand_array(rng, t, shape, -4, 4, bad_frac=bad_frac)
    dt = a.dtype
    if dt.kind == "f":
        a = np.round(a).astype(dt)
        flat = a.reshape(-1)
        k = max(1, flat.size // 20)
        flat[rng.integers(0, flat.size, k)] = np.nan
        flat[rng.integers(0, flat.size, k)] = -0.0
        flat[rng.integers(0, flat.size, k)] = 0.0
        if bad_frac:
            a[bad] = P.default_badvalue(type_code(str(t)))
    return a


@pytest.mark.parametrize("t", REAL_TYPES)
@pytest.mark.parametrize("op", SORT_OPS)
def test_sort_based_bit_exact(gpu, op, t):
    """Ufunc.pd:878-1112 against the oracle bit for bit: the GPU runs the
    reference's quicksort steps, so ties (qsorti's index order), NaN
    placement and the signs of zeros all agree; bad values, strided views."""
    rng = seeded(("sort", op, t))
    for shape in [(7,), (1,), (33, 17), (200, 40), (3, 1000)]:
        x = to_pdl(_sort_data(rng, t, shape[::-1]), t)
        got, exp = _run_both(op, [x])
        _bits_equal(got, exp, f"{op} {t} {shape}")
    a = _sort_data(rng, t, (12, 300), bad_frac=0.25)
    a[0, :] = P.default_badvalue(type_code(t))
    xb = to_pdl(a, t, badflag=True)
    got, exp = _run_both(op, [xb])
    _bits_equal(got, exp, f"{op} {t} bad")
    v = to_pdl(_sort_data(rng, t, (20, 30, 5)), t).xchg(0, 1)
    got, exp = _run_both(op, [v])
    _bits_equal(got, exp, f"{op} {t} strided")


@pytest.mark.parametrize("t", ["byte", "long", "longlong", "float", "double"])
@pytest.mark.parametrize("op", ["pctover", "oddpctover"])
def test_percentiles_bit_exact(gpu, op, t):
    rng = seeded(("pct", op, t))
    for n in [1, 2, 5, 25, 300]:
        a = _sort_data(rng, t, (9, n))
        x = to_pdl(a, t)
        for p in [-0.5, 0.0, 0.1, 0.23, 0.5, 0.77, 0.9, 1.0, 2.0]:
            pp = P.pdl(np.array(p))
            got = getattr(P, op)(x, pp)
            exp = O.run(op, [x, pp])[0]
            _bits_equal(got, exp, f"{op} {t} n={n} p={p}")
    # p broadcast per row, and bad values
    a = _sort_data(rng, t, (16, 50), bad_frac=0.3)
    x = to_pdl(a, t, badflag=True)
    pp = P.pdl(rng.uniform(-0.2, 1.2, size=16))
    _bits_equal(getattr(P, op)(x, pp), O.run(op, [x, pp])[0], f"{op} {t} per-row p")


@pytest.mark.parametrize("t", ["sbyte", "byte", "short", "ushort", "long", "ulong", "longlong"])
def test_modeover(gpu, t):
    rng = seeded(("mode", t))
    for shape in [(7,), (40, 33), (5, 1000)]:
        a, _ = rand_array(rng, t, shape[::-1], 0, 6)
        x = to_pdl(a, t)
        got, exp = _run_both("modeover", [x])
        _bits_equal(got, exp, f"modeover {t} {shape}")


def test_sort_based_empty_and_errors(gpu):
    with pytest.raises(P.PDLError, match="Error in medover:cannot process empty ndarray"):
        P.medover(P.zeroes("double", 0))
    with pytest.raises(P.PDLError, match="cannot process empty ndarray"):
        P.pctover(P.zeroes("double", 0, 3), 0.5)
    e = P.qsort(P.zeroes("double", 0))          # the reference returns at once
    assert e.dims == (0,)
    assert P.qsorti(P.pdl(np.array([8.0]))).numpy().tolist() == [0]


@pytest.mark.parametrize("t", ["byte", "long", "float", "double"])
@pytest.mark.parametrize("op", SORT_OPS + ["pctover", "modeover"])
def test_sort_based_long_rows(gpu, op, t):
    """Rows of 513 to 8192 elements (a block per row in shared memory) and
    beyond (the merge sort; for qsorti of (value, index) pairs): ties, NaN and
    signed zeros, distinct values (the network), bad values."""
    if op == "modeover" and t in ("float", "double"):
        return
    rng = seeded(("sortlong", op, t))
    for n in [513, 1000, 2048, 5000, 8192, 9000]:
        datas = [_sort_data(rng, t, (3, n))]
        if t in ("float", "double", "long"):
            datas.append(rng.permutation(np.arange(3 * n)).reshape(3, n).astype(NP_DTYPES[type_code(t)]))
        for a in datas:
            x = to_pdl(a, t)
            ins = [x, P.pdl(np.array(0.37))] if op == "pctover" else [x]
            got, exp = _run_both(op, ins)
            _bits_equal(got, exp, f"{op} {t} n={n}")
    if op != "modeover":
        a = _sort_data(rng, t, (4, 3000), bad_frac=0.2)
        x = to_pdl(a, t, badflag=True)
        ins = [x, P.pdl(np.array(0.37))] if op == "pctover" else [x]
        got, exp = _run_both(op, ins)
        _bits_equal(got, exp, f"{op} {t} bad n=3000")


@pytest.mark.parametrize("t", ["byte", "ushort", "long", "longlong", "float", "double"])
@pytest.mark.parametrize("op", ["qsort", "qsorti", "medover", "oddmedover", "pctover",
                                "oddpctover", "modeover"])
def test_sort_based_rows_beyond_shared_memory(gpu, op, t):
    """Rows longer than 8192 values: a merge sort (tiles of 4096 sorted in
    shared memory, then merge passes) wherever the good values hold no NaN
    and not both zeros; other rows sorted again with the reference's
    quicksort.  Ties, bad values, ragged lengths, several rows, a row of
    2^20; bit for bit against the oracle."""
    if op == "modeover" and t in ("float", "double"):
        return
    rng = seeded(("lsort", op, t))
    fl = t in ("float", "double")
    cases = []
    a, _ = rand_array(rng, t, (3, 20_001), -50, 50, bad_frac=0.0 if op == "modeover" else 0.05)
    if fl:  # ties, and zeros of one sign only
        a = np.where(a == P.default_badvalue(type_code(t)), a, np.round(a))
        a = np.where(a == 0, np.zeros_like(a), a)
    cases.append((a, op != "modeover"))
    cases.append((rand_array(rng, t, (2, 100_003), -1000, 1000)[0], False))
    if t in ("long", "float"):
        cases.append((rand_array(rng, t, (1, 1 << 20), -1e6, 1e6)[0], False))
    if fl:  # NaN in one row, both zeros in the other: the quicksort's order
        b, _ = rand_array(rng, t, (2, 9_001), -3, 3)
        b = np.round(b)
        b[0, ::97] = np.nan
        b[1, ::89] = -0.0
        b[1, 1::89] = 0.0
        cases.append((b, False))
    for a, bf in cases:
        x = to_pdl(a, t, badflag=bf)
        ins = [x, P.pdl(np.array(0.37))] if op in ("pctover", "oddpctover") else [x]
        got, exp = _run_both(op, ins)
        assert P.last_launch_info()["kernel"] == ("k_lsorti_finish" if op == "qsorti"
                                                  else "k_lsort_finish")
        _bits_equal(got, exp, f"{op} {t} {a.shape} bad={bf}")


@pytest.mark.parametrize("t", ["float", "double", "long", "ulonglong"])
def test_qsorti_long_rows_distinct_values(gpu, t):
    """qsorti of rows longer than 8192 with all good values distinct: the
    (value, index) merge sort gives the quicksort's order; bad indices
    follow in the reference's order (from the row's end backwards)."""
    rng = seeded(("lsorti", t))
    n = (1 << 20) + 77
    clean = np.stack([rng.permutation(n), rng.permutation(n)]).astype(NP_DTYPES[type_code(t)])
    marked = clean.copy()
    marked[rng.random(clean.shape) < 0.03] = P.default_badvalue(type_code(t))
    for a, bf in ((clean, False), (marked, True)):
        x = to_pdl(a, t, badflag=bf)
        got, exp = _run_both("qsorti", [x])
        assert P.last_launch_info()["kernel"] == "k_lsorti_finish"
        _bits_equal(got, exp, f"qsorti {t} bad={bf}")


@pytest.mark.parametrize("op", ["qsort", "medover", "pctover"])
def test_sort_beyond_shared_memory_edges(gpu, op):
    """The merge sort at its edges: one past the shared-memory limit, whole
    tiles, rows read with a stride (a transposed view), a strided qsort
    output."""
    rng = seeded(("lsort-edge", op))
    for shape in [(2, 8193), (3, 12288)]:
        a, _ = rand_array(rng, "double", shape, -100, 100)
        x = to_pdl(a, "double")
        ins = [x, P.pdl(np.array(0.61))] if op == "pctover" else [x]
        got, exp = _run_both(op, ins)
        _bits_equal(got, exp, f"{op} {shape}")
    a, _ = rand_array(rng, "float", (20_000, 3), -100, 100)
    v = to_pdl(a, "float").xchg(0, 1)       # 3 rows of 20000, increment 3
    ins = [v, P.pdl(np.array(0.61))] if op == "pctover" else [v]
    got, exp = _run_both(op, ins)
    assert P.last_launch_info()["kernel"] == "k_lsort_finish"
    _bits_equal(got, exp, f"{op} strided rows")


def test_row_block_scan_strided_rows(gpu):
    """The block-per-row scan over every other row of a matrix (a row
    increment of two rows), and into an output slice of a larger array."""
    rng = seeded(("rowblk", "stride"))
    a, _ = rand_array(rng, "float", (7400, 16_400), -10, 10)
    x = to_pdl(a, "float").slice(slice(None), slice(0, None, 2))   # rows 0, 2, 4, ...
    got, exp = _run_both("cumusumover", [x])
    assert P.last_launch_info()["kernel"] == "k_scan_rowblk"
    rtol, atol, scale = _tol("cumusumover", x.numpy(), exp, exp.type)
    assert_same(got, exp, rtol=rtol, atol=atol, scale=scale, what="cumusumover every other row")
    big = P.pdl(np.zeros((7400, 16_400), np.float32))
    out = big.slice(slice(None), slice(1, None, 2))
    P.cumusumover(x, out)
    assert P.last_launch_info()["kernel"] == "k_scan_rowblk"
    assert np.array_equal(out.numpy(), got.numpy())
    assert not big.numpy()[0::2].any()


@pytest.mark.parametrize("where", ["host", "device"])
def test_in_place_outputs(gpu, where):
    """An output that is one of the inputs (PDL's Inplace => 1: the binary
    ops, qsort, qsortvec), on host and device memory: the same values as a
    separate output."""
    rng = seeded(("inplace", where))
    for op in ("plus", "mult", "minus", "divide"):
        a, _ = rand_array(rng, "double", (5, 7), 1, 9)
        b, _ = rand_array(rng, "double", (5, 7), 1, 9)
        x, y = to_pdl(a, "double"), to_pdl(b, "double")
        exp = O.run(op, [x, y])[0]
        if where == "device":
            x.to_device()
            y.to_device()
        got = getattr(P, op)(x, y, out=x)
        assert got is x
        assert_same(x, exp, what=f"{op} in place ({where})")
    for op, shape in (("qsort", (9, 1000)), ("qsort", (3, 700)), ("qsortvec", (40, 3, 3))):
        a = rng.standard_normal(shape)
        x = to_pdl(a, "double")
        exp = O.run(op, [x])[0]
        if where == "device":
            x.to_device()
        got = getattr(P, op)(x, out=x)
        _bits_equal(got, exp, f"{op} in place ({where}) {shape}")
