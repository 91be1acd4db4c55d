"""The oracle's vector sorts (qsortvec, qsortveci: lib/PDL/Ufunc.pd:769-851,
1115-1230) against the reference's known answers (t/ufunc.t,
t/primitive-vector.t).  CPU only: the GPU kernels for the vector sorts
are not built yet, so these pin the oracle they will be checked against."""
import numpy as np

import pdl_gb300 as P
from helpers import make_input
from oracle import oracle as O


def _vecs(rows, bad=False):
    return make_input({"type": "double", "data": rows, "badflag": int(bad)})


def test_qsortveci_order_of_equal_vectors():
    # t/ufunc.t:9-14: equal vectors [1 2] at 0 and 3 come out as 3, 0
    p2d = _vecs([[1, 2], [3, 4], [1, 3], [1, 2], [3, 3]])
    ix = O.run("qsortveci", [p2d])[0].numpy()
    assert ix.tolist() == [3, 0, 2, 4, 1]
    # t/primitive-vector.t:43-48: qsortvec, and qsortveci's rows in order
    want = [[1, 2], [1, 2], [1, 3], [3, 3], [3, 4]]
    assert O.run("qsortvec", [p2d])[0].numpy().tolist() == want
    assert p2d.numpy()[ix].tolist() == want


def test_qsortvec_cases_of_the_reference_tests():
    # t/ufunc.t:49-53 (the 2-D cases of the qsort loop)
    cases = [
        ([[1, 2], [0, 500], [2, 3], [4, 2], [3, 4], [3, 5]],
         [[0, 500], [1, 2], [2, 3], [3, 4], [3, 5], [4, 2]]),
        ([[1, 2], [0, 500], [2, 3], [4, "BAD"], [3, 4], [3, 5]],
         [[0, 500], [1, 2], [2, 3], [3, 4], [3, 5], [4, "BAD"]]),
        ([[0, 0], [-100, 0], ["BAD", 0], [100, 0]],
         [[-100, 0], [0, 0], [100, 0], ["BAD", 0]]),
    ]
    for data, want in cases:
        bad = any("BAD" in r for r in data)
        x = _vecs(data, bad)
        got = O.run("qsortvec", [x])[0].numpy()
        w = make_input({"type": "double", "data": want, "badflag": int(bad)}).numpy()
        assert np.array_equal(got, w), (data, got)
        ix = O.run("qsortveci", [x])[0].numpy()
        assert np.array_equal(x.numpy()[ix], w)


def test_trivial_vector_sorts():
    # t/ufunc.t:79-80
    # pdl(42,41)->qsortvec is pdl(42,41)->dummy(1): dims (2, 1)
    r = O.run("qsortvec", [P.pdl(np.array([42.0, 41.0]))])[0]
    assert r.dims == (2, 1) and r.numpy().tolist() == [[42, 41]]
    r = O.run("qsortveci", [P.pdl(np.array([53.0, 35.0]))])[0]
    assert r.type == "indx" and r.dims == (1,) and r.numpy().tolist() == [0]


def test_vector_sort_against_lexicographic_order():
    rng = np.random.default_rng(5)
    for m in (1, 2, 9, 64):
        a = rng.integers(0, 3, size=(4, m, 3)).astype(np.float64)   # PDL dims (3, m, 4)
        x = P.pdl(a)
        got = O.run("qsortvec", [x])[0].numpy()
        for plane, g in zip(a, got):
            assert g.tolist() == sorted(plane.tolist())
        ix = O.run("qsortveci", [x])[0].numpy()
        for plane, i in zip(a, ix):
            assert plane[i].tolist() == sorted(plane.tolist())
