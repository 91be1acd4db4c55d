"""The oracle against numpy on random data without bad values (CPU): the
binary ops of Ops.pd under broadcasting (integers wrap, floats are IEEE
operations in the op's type, comparisons give 0/1 in that type), and the
logical/bitwise reductions of Ufunc.pd:143-187 and minmaximum.  A second
pin of the oracle beside the reference's own known answers."""
import numpy as np
import pytest

import pdl_gb300 as P
from oracle import oracle as O

NP = {"byte": np.uint8, "short": np.int16, "long": np.int32, "longlong": np.int64,
      "float": np.float32, "double": np.float64}
BIN = {"plus": np.add, "mult": np.multiply, "minus": np.subtract,
       "gt": np.greater, "lt": np.less, "le": np.less_equal, "ge": np.greater_equal,
       "eq": np.equal, "ne": np.not_equal}


@pytest.mark.parametrize("t", list(NP))
@pytest.mark.parametrize("op", list(BIN) + ["divide", "or2", "and2", "xor", "shiftleft"])
def test_binary_ops(op, t):
    dt = np.dtype(NP[t])
    if op in ("or2", "and2", "xor", "shiftleft") and dt.kind == "f":
        pytest.skip("bit ops work in longlong for float inputs (covered by the golden vectors)")
    rng = np.random.default_rng([len(op), len(t), ord(op[0]), ord(t[0])])
    a = rng.integers(0 if op == "shiftleft" else -50, 50, size=(3, 1, 6)).astype(dt)
    b = rng.integers(0 if op == "shiftleft" else -50, 50, size=(1, 4, 6)).astype(dt)
    if op == "shiftleft":
        b = (b % 5).astype(dt)
    if op == "divide" and dt.kind != "f":
        b[b == 0] = 1
    got = O.run(op, [P.pdl(a), P.pdl(b)])[0].numpy()
    with np.errstate(all="ignore"):
        if op == "divide":
            want = (a / b).astype(dt) if dt.kind == "f" else (np.trunc(a.astype(np.float64) / b)).astype(dt)
        elif op in ("or2", "and2", "xor"):
            want = {"or2": np.bitwise_or, "and2": np.bitwise_and, "xor": np.bitwise_xor}[op](a, b)
        elif op == "shiftleft":
            # C's promotion to int (at least), then back to the type
            want = (a.astype(np.int64) << b.astype(np.int64)).astype(dt)
        else:
            want = BIN[op](a, b).astype(dt)
    assert got.dtype == dt and np.array_equal(got, want)


@pytest.mark.parametrize("t", ["byte", "long", "longlong", "double"])
def test_logical_and_bitwise_reductions(t):
    dt = np.dtype(NP[t])
    rng = np.random.default_rng(len(t))
    a = rng.integers(0, 4, size=(7, 11)).astype(dt)
    a[rng.random(a.shape) < 0.6] = 0
    a[0, :] = 0                      # all zero: zcover 1, orover 0
    a[1, :] = 3                      # none zero: andover 1
    x = P.pdl(a)
    nz = a != 0
    assert np.array_equal(O.run("andover", [x])[0].numpy(), nz.all(-1).astype(dt))
    assert np.array_equal(O.run("orover", [x])[0].numpy(), nz.any(-1).astype(dt))
    assert np.array_equal(O.run("xorover", [x])[0].numpy(), (nz.sum(-1) % 2).astype(dt))
    # zcover: every element zero (tmp = 1; tmp &= (a == 0), Ufunc.pd:146)
    assert np.array_equal(O.run("zcover", [x])[0].numpy(), (~nz).all(-1).astype(dt))
    first = np.array([r[r != 0][0] if (r != 0).any() else 0 for r in a], dtype=dt)
    assert np.array_equal(O.run("firstnonzeroover", [x])[0].numpy(), first)
    if dt.kind != "f":
        assert np.array_equal(O.run("bandover", [x])[0].numpy(), np.bitwise_and.reduce(a, -1))
        assert np.array_equal(O.run("borover", [x])[0].numpy(), np.bitwise_or.reduce(a, -1))
        assert np.array_equal(O.run("bxorover", [x])[0].numpy(), np.bitwise_xor.reduce(a, -1))


def test_minmaximum_against_numpy():
    rng = np.random.default_rng(4)
    a = rng.integers(-9, 9, size=(13, 17)).astype(np.float64)
    cmin, cmax, imin, imax = O.run("minmaximum", [P.pdl(a)], [None] * 4)
    assert np.array_equal(cmin.numpy(), a.min(-1)) and np.array_equal(cmax.numpy(), a.max(-1))
    assert np.array_equal(imin.numpy(), a.argmin(-1)) and np.array_equal(imax.numpy(), a.argmax(-1))
