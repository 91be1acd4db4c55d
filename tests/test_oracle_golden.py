"""The oracle against the reference's own known answers (CPU only).

Every case in tests/golden/reference_vectors.json is transcribed from a PDL
test file (cited per case).  Passing here pins the oracle before it is used
as the checker of the GPU path."""
import math

import numpy as np
import pytest

import pdl_gb300 as P
from helpers import _parse_data, golden_cases, make_input
from oracle import oracle as O
from pdl_gb300.ndarray import type_code

CASES = golden_cases()


def oracle_matmult(x, y, out=None):
    """PDL::matmult's Perl wrapper (lib/PDL/Primitive.pd:196-210) over the
    oracle's _matmult_int."""
    while x.ndims < 2:
        x = x.dummy(-1)
    while y.ndims < 2:
        y = y.dummy(-1)
    if y.dim(1) != x.dim(0):
        raise O.OracleError("Dim mismatch in matmult of [%dx%d] x [%dx%d]: %d != %d"
                            % (x.dim(0), x.dim(1), y.dim(0), y.dim(1), x.dim(0), y.dim(1)))
    return O.run("matmult", [x, y], [out])[0]


def run_case_oracle(case):
    ins = [make_input(s) for s in case["inputs"]]
    if case.get("view") == "xchg01":
        ins[0] = ins[0].xchg(0, 1)
    if case.get("view") == "dim1_index1":
        ins[0] = ins[0].slice(slice(None), 1)
    if "whole" in case:
        ins[0] = ins[0].flat()
    out = None
    if "out" in case:
        kind, dims = case["out"].split(":")
        dims = [int(d) for d in dims.split(",")]
        out = (P.zeroes if kind == "zeroes" else P.ones)("double", *dims)
    if case["op"] == "matmult":
        return oracle_matmult(ins[0], ins[1], out)
    outs = [out] + [None] * (case.get("nout", 1) - 1)
    return O.run(case["op"], ins, outs, swap=case.get("swap", 0))[case.get("pick", 0)]


def check_result(case, got):
    exp_t = case.get("expect_type")
    if exp_t:
        assert got.type == exp_t
    if case.get("check") == "index":
        # the reference's test: the input indexed by the result is `expect`
        src = make_input(case["inputs"][0])
        vals = src.numpy().reshape(-1)[got.numpy().reshape(-1)]
        e, bad = _parse_data(case["expect"], src.datatype)
        assert np.array_equal(vals[~bad], e[~bad])
        assert np.all(vals[bad] == P.default_badvalue(src.datatype))
        return
    g = got.numpy()
    if "expect_badflag" in case:
        assert int(got.badflag()) == case["expect_badflag"]
    if "expect_sum" in case:
        assert float(g.sum()) == case["expect_sum"]
    exp = case["expect"]
    t = got.datatype
    if exp == "BAD":
        assert g.reshape(-1)[0] == P.default_badvalue(t)
        return
    if exp == "nan":
        assert math.isnan(float(g.reshape(-1)[0]))
        return
    e, bad = _parse_data(exp, t)
    e = e.astype(np.float64)
    gf = g.astype(np.float64).reshape(e.shape)
    if bad.any():
        assert np.all(gf[bad] == float(P.default_badvalue(t)))
    m = ~bad
    atol, rtol = case.get("atol", 0.0), case.get("rtol", 0.0)
    both_nan = np.isnan(gf) & np.isnan(e)
    ok = both_nan | (np.abs(gf - e) <= atol + rtol * np.abs(e))
    assert np.all(ok[m]), f"got {gf} expected {e}"


@pytest.mark.parametrize("case", CASES, ids=[c["id"] for c in CASES])
def test_oracle_matches_reference_known_answers(case):
    if "expect_error" in case:
        with pytest.raises(O.OracleError, match=case["expect_error"]):
            run_case_oracle(case)
        return
    check_result(case, run_case_oracle(case))


def test_oracle_prodover_stops_at_zero():
    # Ufunc.pd:91,107: the product stops at the first zero, so a later NaN
    # does not turn the result into NaN.
    x = P.pdl(np.array([2.0, 0.0, np.nan, 3.0]))
    r = O.run("prodover", [x])[0].numpy()
    assert r == 0.0


def test_oracle_min_ind_ties_and_nans():
    # first index on ties; NaN only when all are NaN (then the last NaN)
    x = P.pdl(np.array([[3.0, 1.0, 1.0, 2.0], [np.nan, np.nan, np.nan, np.nan]]))
    r = O.run("minimum_ind", [x])[0].numpy()
    assert list(r) == [1, 3]


def test_oracle_average_int_division():
    x = P.pdl(np.array([[1, 2, 2], [-7, 0, 0]], dtype=np.int32))
    r = O.run("average", [x])[0]
    assert r.type == "long"
    assert list(r.numpy()) == [1, -2]  # C integer division truncates


def test_oracle_int_wraps():
    x = P.pdl(np.array([2**31 - 1, 1], dtype=np.int32))
    assert O.run("sumover", [x])[0].numpy() == -2**31


def test_oracle_threads_agree():
    rng = np.random.default_rng(0)
    a = P.pdl(rng.standard_normal((512, 2048)))
    for op in ["sumover", "minimum_ind", "cumusumover", "prodover"]:
        r1 = O.run(op, [a], nthreads=1)[0].numpy()
        r8 = O.run(op, [a], nthreads=8)[0].numpy()
        assert np.array_equal(r1, r8, equal_nan=True), op


def test_oracle_sort_functions_against_numpy():
    """Properties any correct sort satisfies, on data without NaN or mixed
    zeros: qsort is numpy's sorted row, qsorti a permutation that sorts
    the row, medover the middle value (the mean of the two middle ones
    for an even count, in the type's arithmetic), oddmedover the lower
    middle, modeover the most frequent repeated value."""
    rng = np.random.default_rng(11)
    for n in (1, 2, 7, 64, 301):
        a = rng.integers(-20, 20, size=(9, n)).astype(np.float64)
        x = P.pdl(a)
        s = np.sort(a, -1)
        assert np.array_equal(O.run("qsort", [x])[0].numpy(), s)
        ix = O.run("qsorti", [x])[0].numpy()
        assert np.array_equal(np.take_along_axis(a, ix, -1), s)
        assert all(sorted(r) == list(range(n)) for r in ix.tolist())
        lo, hi = s[:, (n - 1) // 2], s[:, n // 2]
        assert np.array_equal(O.run("medover", [x])[0].numpy(), 0.5 * (lo + hi))
        assert np.array_equal(O.run("oddmedover", [x])[0].numpy(), lo)
        xi = P.pdl(a.astype(np.int32))
        mo = O.run("modeover", [xi])[0].numpy()
        for r, m in zip(a.astype(np.int32), mo):
            vals, cnt = np.unique(r, return_counts=True)
            want = vals[np.argmax(cnt)] if cnt.max() > 1 else 0
            assert m == want
