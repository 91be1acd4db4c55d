"""Per-ndarray badvalues on the GPU against the oracle.

PDL gives every parameter of an op its own badvalue: the ndarray's own
(`has_badvalue`) or its type's default (lib/PDL/Core/pdlcore.h:197-205,
PDL_DECLARE_PARAMETER_BADVAL).  An input element is bad when it equals its
own ndarray's badvalue (or is NaN when that badvalue is NaN); an output
marked bad gets the OUTPUT's badvalue.  These tests give the inputs and the
output different, non-default badvalues (as t/bad.t:69,97,266 set them), and
plant each type's default badvalue as an ordinary good value, so a kernel
that tested against the wrong badvalue would be caught.

Bar: bit-exact for integers, indices and bad masks; float sums within
(n+2)*eps*sum|a| of the oracle, as in the other parity tests."""
import numpy as np
import pytest

import pdl_gb300 as P
from helpers import FLOAT_TYPES, assert_same, rand_array, seeded, to_pdl
from oracle import oracle as O
from pdl_gb300.ndarray import NP_DTYPES, type_code

pytestmark = pytest.mark.gpu

EPS = {"float": 2.0 ** -24, "double": 2.0 ** -53}


def _bad_input(rng, t, shape, bv, lo=-20, hi=20, frac=0.05, plant_default=True):
    """An ndarray with badflag on and badvalue bv; about frac of its elements
    are bv, and (if plant_default) a few others hold the type's default
    badvalue, which for this ndarray is an ordinary value."""
    a, _ = rand_array(rng, t, shape, lo, hi)
    a = a.copy()
    dt = np.dtype(NP_DTYPES[type_code(t)])
    bad = rng.random(shape) < frac
    a[bad] = np.nan if (isinstance(bv, float) and np.isnan(bv)) else dt.type(bv)
    if plant_default and a.size:
        flat = a.reshape(-1)
        cand = np.flatnonzero(~bad.reshape(-1))
        if cand.size:
            flat[rng.choice(cand, size=max(1, cand.size // 97), replace=False)] = \
                P.default_badvalue(type_code(t))
    x = to_pdl(a, t, badflag=True)
    x.badvalue(bv)
    return x, a, bad


def _preset_out(t, dims, bv):
    o = P.zeroes(t, *dims)
    o.badvalue(bv)
    return o


def _same_with_own_badvalue(got, exp, bv, rtol=0.0, scale=None, what=""):
    """Values equal (floats within rtol*scale) and the same elements hold the
    output's own badvalue."""
    assert got.type == exp.type and got.dims == exp.dims, what
    assert got.badflag() == exp.badflag(), f"{what}: badflag"
    g, e = got.numpy(), exp.numpy()
    if isinstance(bv, float) and np.isnan(bv):
        gb, eb = np.isnan(g), np.isnan(e)
    else:
        gb, eb = g == g.dtype.type(bv), e == e.dtype.type(bv)
    assert np.array_equal(gb, eb), f"{what}: elements holding the output badvalue differ"
    if g.dtype.kind != "f" or rtol == 0:
        assert np.array_equal(g, e, equal_nan=g.dtype.kind == "f"), f"{what}: values differ"
        return
    m = ~(gb | np.isnan(g) | np.isnan(e))
    diff = np.abs(g[m].astype(np.float64) - e[m].astype(np.float64))
    tol = rtol * np.broadcast_to(scale, g.shape)[m] + 1e-300
    ok = (g[m] == e[m]) | (diff <= tol)
    assert ok.all(), f"{what}: {np.count_nonzero(~ok)} values outside tolerance"


RED_CASES = [("long", 7, -99), ("short", -3, 12), ("ulong", 5, 77), ("byte", 9, 1),
             ("longlong", 1000, -1), ("float", 2.5, -7.0), ("float", float("nan"), 3.0),
             ("double", -1.25, 42.0), ("double", float("nan"), -2.0)]
RED_OPS = ["sumover", "dsumover", "prodover", "average", "daverage", "minimum", "maximum",
           "minimum_ind", "maximum_ind", "cumusumover", "dcumusumover", "andover", "borover",
           "firstnonzeroover"]


@pytest.mark.parametrize("t,bv_in,bv_out", RED_CASES)
@pytest.mark.parametrize("op", RED_OPS)
def test_reductions_with_own_badvalues(gpu, op, t, bv_in, bv_out):
    if op == "borover" and t in FLOAT_TYPES:
        pytest.skip("borover is an integer op")
    rng = seeded(("a19red", op, t, str(bv_in)))
    lo, hi = (-1.5, 1.5) if op.endswith("prodover") and t in FLOAT_TYPES else \
             (-3, 3) if "prod" in op else (-20, 20)
    if t in ("byte", "ulong"):
        lo = 0
    for shape in [(6, 40), (3, 5000), (2, 70000), (4, 0)]:
        # the default badvalue as a good value: where it cannot overflow
        plant = t not in FLOAT_TYPES or op in ("minimum", "maximum", "minimum_ind", "maximum_ind",
                                                "andover", "firstnonzeroover")
        x, a, bad = _bad_input(rng, t, shape, bv_in, lo, hi, plant_default=plant)
        if shape[0] > 1 and shape[1] > 0:
            a[0] = np.nan if np.isnan(float(bv_in)) else a.dtype.type(bv_in)   # an all-bad row
            bad[0] = True
            x = to_pdl(a, t, badflag=True)
            x.badvalue(bv_in)
        exp_null = O.run(op, [x])[0]
        out_t, dims = exp_null.type, exp_null.dims
        cmp_bv = bv_out
        if np.dtype(NP_DTYPES[type_code(out_t)]).kind != "f" and isinstance(bv_out, float):
            cmp_bv = int(bv_out)
        if np.dtype(NP_DTYPES[type_code(out_t)]).kind in "u" and cmp_bv < 0:
            cmp_bv = 3
        go, eo = _preset_out(out_t, dims, cmp_bv), _preset_out(out_t, dims, cmp_bv)
        got = getattr(P, op)(x.to_device(), go)
        exp = O.run(op, [x], [eo])[0]
        rtol, scale = 0.0, None
        if out_t in FLOAT_TYPES and op not in ("minimum", "maximum", "firstnonzeroover"):
            n = shape[-1]
            acc = "double" if op.startswith("d") or out_t == "double" else "float"
            clean = np.where(bad, 0, np.abs(np.nan_to_num(a.astype(np.float64))))
            scale = np.cumsum(clean, -1) if "cumu" in op else clean.sum(-1)
            if "average" in op:
                scale = scale / max(n, 1)
            rtol = (n + 2) * EPS[acc]
            if "prod" in op:
                scale, rtol = np.abs(np.nan_to_num(exp.numpy().astype(np.float64))), (n + 2) * EPS[acc]
        _same_with_own_badvalue(got, exp, cmp_bv, rtol, scale, what=f"{op} {t} bv={bv_in} {shape}")
        # a null output: the type's default badvalue marks bad outputs
        got_null = getattr(P, op)(x)
        _same_with_own_badvalue(got_null, exp_null, P.default_badvalue(type_code(out_t)), rtol,
                                scale, what=f"{op} {t} bv={bv_in} {shape} null output")


BIOP_CASES = [("long", 7, -5, 99), ("double", 0.5, float("nan"), -8.0), ("float", float("nan"), 3.0, 11.0),
              ("short", -2, 4, 6), ("byte", 3, 200, 17)]


@pytest.mark.parametrize("t,bva,bvb,bvc", BIOP_CASES)
@pytest.mark.parametrize("op", ["plus", "mult", "minus", "divide", "gt", "eq", "and2"])
def test_biops_with_three_badvalues(gpu, op, t, bva, bvb, bvc):
    if op == "and2" and t in FLOAT_TYPES:
        pytest.skip("and2 on floats is covered by the bit-op tests")
    rng = seeded(("a19biop", op, t))
    # divide: no zero divisors on either side (swap divides by a; integer
    # division by zero is undefined in the reference's C)
    lo = 1 if op == "divide" else 0 if t == "byte" else -20
    x, _, _ = _bad_input(rng, t, (5, 1, 64), bva, lo, 20)
    y, _, _ = _bad_input(rng, t, (1, 7, 64), bvb, lo, 20)
    exp_null = O.run(op, [x, y])[0]
    ot = exp_null.type
    okind = np.dtype(NP_DTYPES[type_code(ot)]).kind
    c_bv = bvc if okind == "f" else int(bvc) if not (isinstance(bvc, float) and np.isnan(bvc)) else 1
    for swap in (0, 1):
        go, eo = _preset_out(ot, exp_null.dims, c_bv), _preset_out(ot, exp_null.dims, c_bv)
        got = getattr(P, op)(x.to_device(), y.to_device(), go, swap=swap)
        exp = O.run(op, [x, y], [eo], swap=swap)[0]
        _same_with_own_badvalue(got, exp, c_bv, what=f"{op} {t} swap={swap}")
    _same_with_own_badvalue(getattr(P, op)(x, y), exp_null, P.default_badvalue(type_code(ot)),
                            what=f"{op} {t} null output")


def test_biop_mixed_types_convert_the_own_badvalue(gpu):
    """A long input with badvalue 7 promoted to double: its bad elements stay
    bad after the conversion (the converted badvalue), while a double 7.0 in
    the other input is an ordinary value."""
    rng = seeded(("a19mixed",))
    x, _, _ = _bad_input(rng, "long", (4, 33), 7)
    y, _, _ = _bad_input(rng, "double", (4, 33), float("nan"))
    yn = y.numpy().copy()
    yn[0, :5] = 7.0
    y = to_pdl(yn, "double", badflag=True)
    y.badvalue(float("nan"))
    for op in ("plus", "mult"):
        got, exp = getattr(P, op)(x.to_device(), y.to_device()), O.run(op, [x, y])[0]
        assert_same(got, exp, what=f"{op} long(bv 7) + double(bv NaN)")


@pytest.mark.parametrize("t,bva,bvb,bvc", [("double", 1.5, -2.5, 9.0), ("long", 3, -4, 100),
                                            ("float", float("nan"), 0.25, -1.0)])
def test_inner_with_three_badvalues(gpu, t, bva, bvb, bvc):
    rng = seeded(("a19inner", t))
    # (no default badvalue planted: an integer inner outside the type's
    # range is undefined in the reference's C)
    x, a, ba = _bad_input(rng, t, (50, 300), bva, -4, 4, frac=0.002, plant_default=False)
    y, b, bb = _bad_input(rng, t, (50, 300), bvb, -4, 4, frac=0.002, plant_default=False)
    ot = O.run("inner", [x, y])[0].type
    go, eo = _preset_out(ot, (50,), bvc), _preset_out(ot, (50,), bvc)
    got = P.inner(x.to_device(), y.to_device(), go)
    exp = O.run("inner", [x, y], [eo])[0]
    rtol, scale = 0.0, None
    if t in FLOAT_TYPES:
        clean = np.where(ba | bb, 0, np.abs(np.nan_to_num(a.astype(np.float64) * b)))
        rtol, scale = (300 + 2) * EPS[t], clean.sum(-1)
    _same_with_own_badvalue(got, exp, bvc, rtol, scale, what=f"inner {t}")


@pytest.mark.parametrize("t,bva,bvb,bvc", [("double", 1.5, -2.5, 9.0), ("long", 3, -4, 100),
                                            ("float", float("nan"), 0.25, -1.0)])
def test_matmult_with_three_badvalues(gpu, t, bva, bvb, bvc):
    rng = seeded(("a19mm", t))
    x, _, _ = _bad_input(rng, t, (2, 40, 30), bva, -4, 4, frac=0.004)    # dims (t=30, h=40, 2)
    y, _, _ = _bad_input(rng, t, (30, 25), bvb, -4, 4, frac=0.004)       # dims (w=25, t=30)
    exp_null = O.run("matmult", [x, y])[0]
    go, eo = _preset_out(t, exp_null.dims, bvc), _preset_out(t, exp_null.dims, bvc)
    got = P.matmult(x.to_device(), y.to_device(), go)
    exp = O.run("matmult", [x, y], [eo])[0]
    _same_with_own_badvalue(got, exp, bvc, what=f"matmult {t}")


def _chain(x, y, z):
    tt = O.run("mult", [x, y])[0]
    u = O.run("plus", [tt, z])[0]
    return O.run("sumover", [u])[0], u


@pytest.mark.parametrize("t,bvs", [("long", (7, -5, 11)), ("float", (0.5, float("nan"), -3.0)),
                                   ("double", (float("nan"), 2.0, -1.0))])
def test_fused_and_deferred_with_own_badvalues(gpu, t, bvs):
    """sumover(a*b + d) through the fused kernel and through a recorded
    expression: every leaf tested against its own badvalue, the
    intermediates against their type's default (they are null outputs in
    the eager chain)."""
    rng = seeded(("a19fused", t))
    x, _, _ = _bad_input(rng, t, (20, 1, 33), bvs[0], -30, 30, frac=0.03, plant_default=t == "long")
    y, _, _ = _bad_input(rng, t, (1, 9, 33), bvs[1], -30, 30, frac=0.03, plant_default=t == "long")
    z, _, _ = _bad_input(rng, t, (20, 1, 33), bvs[2], -30, 30, frac=0.03, plant_default=t == "long")
    exp, u = _chain(x, y, z)
    rtol, scale = 0.0, None
    if t in FLOAT_TYPES:
        un = np.abs(np.nan_to_num(u.numpy().astype(np.float64)))
        un[u.numpy() == P.default_badvalue(type_code(t))] = 0
        rtol, scale = 40 * EPS[t], un.sum(-1)
    bv_def = P.default_badvalue(type_code(t))
    xd, yd, zd = x.to_device(), y.to_device(), z.to_device()
    got = P.sumover_mult_plus(xd, yd, zd)
    _same_with_own_badvalue(got, exp, bv_def, rtol, scale, what=f"fused {t}")
    got = (P.lazy(xd) * yd + zd).sumover()
    _same_with_own_badvalue(got, exp, bv_def, rtol, scale, what=f"deferred {t}")
