"""qsortvec / qsortveci on the GPU against the oracle (the reference's vector
quicksort, lib/PDL/Ufunc.pd:1115-1231), bit for bit: the reference's known
answers, rows sorted by the network (no two vectors equal), rows with ties,
NaN and signed zeros (the reference's own steps), vectors with bad values
(default and custom badvalues), views, broadcast planes, rows too large for
shared memory (one thread per row) and empty inputs."""
import numpy as np
import pytest

import pdl_gb300 as P
from helpers import assert_same, make_input, seeded, to_pdl
from pdl_gb300.ndarray import type_code
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NP = {"double": np.float64, "float": np.float32, "long": np.int32, "byte": np.uint8,
      "longlong": np.int64, "short": np.int16}


def both(x):
    for op in ("qsortvec", "qsortveci"):
        got = getattr(P, op)(x)
        exp = O.run(op, [x])[0]
        assert_same(got, exp, what=f"{op} {x.type} dims {x.dims}")


def test_known_answers(gpu):
    # t/ufunc.t:9-14 and t/primitive-vector.t:43-48: equal vectors keep the
    # reference's order (indices 3, 0)
    p2d = make_input({"type": "double", "data": [[1, 2], [3, 4], [1, 3], [1, 2], [3, 3]]})
    assert P.qsortveci(p2d).numpy().tolist() == [3, 0, 2, 4, 1]
    assert P.qsortvec(p2d).numpy().tolist() == [[1, 2], [1, 2], [1, 3], [3, 3], [3, 4]]
    # t/ufunc.t:49-53 with bad values
    x = make_input({"type": "double", "data": [[1, 2], [0, 500], [2, 3], [4, "BAD"], [3, 4], [3, 5]],
                    "badflag": 1})
    both(x)
    x = make_input({"type": "double", "data": [[0, 0], [-100, 0], ["BAD", 0], [100, 0]], "badflag": 1})
    both(x)
    # t/ufunc.t:79-80
    both(P.pdl(np.array([42.0, 41.0])))


@pytest.mark.parametrize("t", ["double", "float", "long", "byte", "longlong", "short"])
@pytest.mark.parametrize("m", [1, 2, 9, 64, 500, 3000])
def test_ties_and_distinct(gpu, t, m):
    rng = seeded(("qsv", t, m))
    # few values: many equal vectors (the reference's steps)
    a = rng.integers(0, 3, size=(4, m, 3))
    both(to_pdl(a.astype(NP[t]), t))
    # many values: distinct vectors (the network)
    hi = {"byte": 255, "short": 30000}.get(t, 10 ** 6)
    a = rng.integers(0, hi, size=(3, m, 2))
    both(to_pdl(a.astype(NP[t]), t))


def test_nan_and_signed_zeros(gpu):
    rng = seeded(44)
    a = rng.standard_normal((2, 300, 3))
    a[0, rng.integers(0, 300, 20), rng.integers(0, 3, 20)] = np.nan
    a[1, :, 0] = 0.0
    a[1, ::3, 0] = -0.0
    a[1, :, 1] = np.round(a[1, :, 1])
    both(P.pdl(a))
    both(P.pdl(a.astype(np.float32)))


@pytest.mark.parametrize("t", ["double", "float", "long"])
def test_bad_vectors(gpu, t):
    rng = seeded(("qsvbad", t))
    a = rng.integers(-5, 5, size=(3, 700, 2)).astype(NP[t])
    bad = rng.random(a.shape) < 0.05
    a[bad] = P.default_badvalue(type_code(t))
    x = to_pdl(a, t, True)
    both(x)
    # a custom badvalue on the input
    y = to_pdl(np.where(bad, 3, a).astype(a.dtype), t, True)
    y.badvalue(3)
    both(y)


def test_views_and_long_rows(gpu):
    rng = seeded(45)
    a = rng.standard_normal((300, 2, 5))        # PDL dims (5, 2, 300)
    x = P.pdl(a)
    both(x.xchg(0, 2))      # dims (300, 2, 5): vectors of 300 components, strided
    both(x.mv(2, 0))        # dims (300, 5, 2)
    both(x.xchg(0, 1))      # dims (2, 5, 300): 5 vectors of 2 components, strided
    # too large for shared memory: one thread per row over device scratch
    big = rng.integers(0, 4, size=(2, 20000, 8)).astype(np.float64)   # 1.28 MB of vectors a row
    both(P.pdl(big))
    big2 = rng.standard_normal((1, 30000, 8))
    both(P.pdl(big2))


def test_empty(gpu):
    for dims in ((0, 4), (3, 0)):
        x = P.zeroes("double", *dims)
        r = P.qsortvec(x)
        assert r.dims == dims
        i = P.qsortveci(x)
        assert i.dims == (dims[1],) and i.type == "indx"
