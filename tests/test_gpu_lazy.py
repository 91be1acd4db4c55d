"""Fused expression reductions (pdlgb300_run_expr_reduce) against the
oracle running the same ops one by one and then the reduction: integer
types and every min/max/index/logical result bit-exact, bad masks and bad
flags exact, float sums within the sequential-sum bound of the float terms
(|got - exp| <= (n + 2) eps sum|terms|).  Also: the fused kernel is the one
that ran, long rows split over blocks, an intermediate that equals its
type's badvalue is bad for the next op as in the eager chain, and
expressions that are not fused give the eager result."""
import numpy as np
import pytest

import pdl_gb300 as P
from helpers import assert_same, rand_array, seeded, to_pdl
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = {"float": 2.0 ** -24, "double": 2.0 ** -53}
TYPES = ["long", "longlong", "float", "double"]


def _oracle(e):
    if not isinstance(e, P.Lazy):
        return e
    return O.run(e.op, [_oracle(e.a), _oracle(e.b)])[0]


def _check(e, red, what):
    got = getattr(e, red)()
    op = P.last_launch_info()["op"]
    assert op.endswith("(expr)") or op == "sumover_mult_plus", (what, op)
    ref_in = _oracle(e)
    exp = O.run(red, [ref_in])[0]
    if got.type in ("float", "double") and red in ("sumover", "average", "dsumover", "daverage"):
        v = ref_in.numpy().astype(np.float64)
        good = np.ones(v.shape, bool)
        if ref_in.badflag():
            good = v != float(P.default_badvalue(ref_in.datatype))
        n = v.shape[-1] if v.ndim else 1
        s = np.where(good, np.abs(v), 0).sum(-1)
        if red in ("average", "daverage"):
            s = s / np.maximum(good.sum(-1), 1)
        eps = EPS["double"] if red.startswith("d") or got.type == "double" else EPS["float"]
        assert_same(got, exp, rtol=1.0, atol=1e-300, scale=(n + 2) * eps * s, what=what)
    else:
        assert_same(got, exp, what=what)


@pytest.mark.parametrize("t", TYPES)
def test_smp_shape_all_reductions(gpu, t):
    """sumover(a*b + a) over an outer-product broadcast, and the other
    fused reductions over the same expression."""
    rng = seeded(("lazy", t))
    a, _ = rand_array(rng, t, (64, 1, 300), -20, 20)      # PDL (300, 1, 64)
    b, _ = rand_array(rng, t, (1, 48, 300), -20, 20)      # PDL (300, 48, 1)
    x, y = to_pdl(a, t).to_device(), to_pdl(b, t).to_device()
    e = P.lazy(x) * y + x
    for red in ["sumover", "dsumover", "average", "daverage", "minimum", "maximum",
                "minimum_ind", "maximum_ind", "andover", "orover", "xorover", "zcover"]:
        _check(e, red, f"{red} {t}")
    if t in ("long", "longlong"):
        for red in ["prodover", "bandover", "borover", "bxorover"]:
            _check(e, red, f"{red} {t}")


@pytest.mark.parametrize("n", [333, 336])
@pytest.mark.parametrize("t", TYPES)
def test_bad_values_through_the_chain(gpu, t, n):
    """n = 333: rows not 16-byte aligned (element loads); 336: aligned rows
    (16-byte loads)."""
    rng = seeded(("lazy-bad", t, n))
    a, _ = rand_array(rng, t, (40, n), -9, 9, bad_frac=0.1)
    b, _ = rand_array(rng, t, (40, n), -9, 9)
    c, _ = rand_array(rng, t, (1, n), 1, 9, bad_frac=0.05)
    x, y, z = to_pdl(a, t, badflag=True), to_pdl(b, t), to_pdl(c, t, badflag=True)
    e = (P.lazy(x) - y) * z
    for red in ["sumover", "average", "minimum", "maximum_ind", "orover"]:
        _check(e, red, f"{red} {t} bad")
        assert getattr(e, red)().badflag()
    # the comparisons feed the logical reductions (all(x > y) row by row)
    g = P.lazy(x) > y
    for red in ["andover", "orover", "sumover"]:
        _check(g, red, f"{red} {t} gt")


def test_intermediate_equal_to_badvalue_is_bad(gpu):
    # 65536 * -32768 is int32's default badvalue: with a's bad flag set the
    # eager plus sees a bad intermediate, and so must the fused chain
    a = np.array([[65536, 1, 2], [3, 65536, 5]], np.int32)
    b = np.array([[-32768, 1, 1], [1, -32768, 1]], np.int32)
    x, y = P.pdl(a), P.pdl(b)
    x.badflag(1)
    e = P.lazy(x) * y + 1
    _check(e, "sumover", "collision")
    got = e.sumover().numpy()
    # row 0: the bad product is skipped, 1*1+1 + 2*1+1 = 5; row 1: 3+1 + 5+1 = 10
    assert got.tolist() == [5, 10]


@pytest.mark.parametrize("t", ["float", "long"])
def test_long_rows_split(gpu, t):
    rng = seeded(("lazy-long", t))
    a, _ = rand_array(rng, t, (3, 300_000), -5, 5)
    b, _ = rand_array(rng, t, (3, 300_000), -5, 5)
    x, y = to_pdl(a, t).to_device(), to_pdl(b, t).to_device()
    e = P.lazy(x) * y + x
    for red in ["sumover", "maximum_ind", "orover"]:
        _check(e, red, f"{red} {t} long rows")


def test_views_and_scalars(gpu):
    rng = seeded(("lazy-views",))
    a = rng.standard_normal((30, 40, 5))
    x = P.pdl(a)
    v = x.xchg(0, 1)                                   # a strided reduced dim
    e = (P.lazy(v) * 2.0 - v) / 3.0
    _check(e, "sumover", "strided")
    _check(e, "minimum_ind", "strided")


def test_not_fused_gives_the_eager_result(gpu):
    a = np.arange(24, dtype=np.uint8).reshape(4, 6)
    x = P.pdl(a)
    e = P.lazy(x) * x + x
    got = e.sumover()
    assert not P.last_launch_info()["op"].endswith("(expr)")
    assert np.array_equal(got.numpy(), P.sumover(P.plus(P.mult(x, x), x)).numpy())


def test_generic_kernel_matches_the_tiled_kernel(gpu):
    # sumover(a*b + a) goes to the tiled sumover_mult_plus kernel; the
    # generic expression kernel gives the same integers
    from pdl_gb300.lazy import _run_fused
    rng = seeded(("lazy-smp",))
    a = rng.integers(-100, 100, size=(256, 1, 64)).astype(np.int32)
    b = rng.integers(-100, 100, size=(1, 128, 64)).astype(np.int32)
    x, y = P.pdl(a).to_device(), P.pdl(b).to_device()
    e = P.lazy(x) * y + x
    got = e.sumover()
    assert P.last_launch_info()["op"] == "sumover_mult_plus"
    leaves, nodes = e._program()
    generic = _run_fused("sumover", leaves, nodes, None)
    assert P.last_launch_info()["op"] == "sumover(expr)"
    got, generic = got.numpy(), generic.numpy()
    assert np.array_equal(got, generic)
    assert np.array_equal(got, P.sumover(P.plus(P.mult(x, y), x)).numpy())


@pytest.mark.parametrize("t", ["long", "float", "double"])
def test_programs_of_one_to_eight_nodes(gpu, t):
    """Programs of one or two nodes without bad values keep the node results
    in registers, longer ones (and bad values) in shared-memory slots: one
    to eight nodes over four leaves, node operands reaching back to every
    earlier node, against the eager chain."""
    rng = seeded(("nodes", t))
    lv = [to_pdl(rand_array(rng, t, (6, 5000), -9, 9)[0], t) for _ in range(4)]
    a, b, c, d = (P.lazy(x) for x in lv)
    n0 = a * b
    n1 = n0 + c
    n2 = d - a
    n3 = n1 * n2
    progs = [a * b, (a - b) * (a - b), n0 + c * d, n3, n3 - n0, (n3 - n0) * n2,
             ((n3 - n0) * n2) + n1, (((n3 - n0) * n2) + n1) - d]
    for k, e in enumerate(progs):
        for red in ("sumover", "minimum", "maximum_ind"):
            _check(e, red, f"{t} program {k} {red}")
