"""Shared helpers: building inputs, running the GPU path and the oracle on the
same data, and comparing with the tolerances the parity bar states."""
from __future__ import annotations

import json
import zlib
from pathlib import Path

import numpy as np

import pdl_gb300 as P
from pdl_gb300 import _abi as A
from pdl_gb300.ndarray import NP_DTYPES, type_code

GOLDEN = Path(__file__).resolve().parent / "golden"

REAL_TYPES = ["sbyte", "byte", "short", "ushort", "long", "ulong", "indx",
              "ulonglong", "longlong", "float", "double"]
INT_TYPES = REAL_TYPES[:9]
FLOAT_TYPES = ["float", "double"]


def golden_cases():
    return json.loads((GOLDEN / "reference_vectors.json").read_text())["cases"]


def _parse_data(data, t):
    if isinstance(data, str) and ":" in data:
        kind, dims = data.split(":")
        dims = [int(x) for x in dims.split(",")]
        shape = tuple(dims[::-1])
        if kind == "ones":
            return np.ones(shape, dtype=NP_DTYPES[t]), np.zeros(shape, bool)
        if kind == "sequence":
            return (np.arange(int(np.prod(dims))).reshape(shape).astype(NP_DTYPES[t]),
                    np.zeros(shape, bool))
        if kind == "zeroes":
            return np.zeros(shape, dtype=NP_DTYPES[t]), np.zeros(shape, bool)
    arr = np.array(data, dtype=object)
    bad = np.vectorize(lambda v: v == "BAD", otypes=[bool])(arr) if arr.size else np.zeros(arr.shape, bool)
    vals = np.vectorize(lambda v: 0 if v == "BAD" else (float("nan") if v == "nan" else v),
                        otypes=[object])(arr) if arr.size else arr
    dt = NP_DTYPES[t]
    if np.dtype(dt).kind in "iu":
        out = np.array([int(v) for v in vals.reshape(-1)], dtype=dt).reshape(arr.shape) if arr.size \
            else np.zeros(arr.shape, dt)
    else:
        out = np.array(vals.tolist(), dtype=dt) if arr.size else np.zeros(arr.shape, dt)
    return out, bad


def make_input(spec) -> P.ndarray:
    t = type_code(spec["type"])
    arr, bad = _parse_data(spec["data"], t)
    if bad.any():
        arr = arr.copy()
        arr[bad] = P.default_badvalue(t)
    x = P.from_numpy(arr, t)
    if spec.get("badflag"):
        x.badflag(1)
    return x


def expect_array(case, like_type=None):
    t = type_code(case.get("expect_type", like_type or "double"))
    return _parse_data(case["expect"], t)


def seeded(seed):
    """A generator from an int or from a tuple of strings/ints; tuples are
    hashed with CRC-32 so the seed is the same in every process (Python's
    str hash is salted per process)."""
    if isinstance(seed, tuple):
        seed = zlib.crc32(repr(seed).encode())
    return np.random.default_rng(seed)


def rand_array(rng, t, shape, lo=-100, hi=100, bad_frac=0.0, special=False):
    """A typed numpy array; optional bad fraction (default badvalue)."""
    t = type_code(t)
    dt = np.dtype(NP_DTYPES[t])
    if dt.kind == "f":
        a = rng.uniform(lo, hi, size=shape).astype(dt)
        if special and a.size >= 4:
            flat = a.reshape(-1)
            flat[rng.integers(0, flat.size, size=max(1, flat.size // 50))] = np.nan
    else:
        info = np.iinfo(dt)
        l = max(lo, int(info.min))
        h = min(hi, int(info.max))
        a = rng.integers(l, h + 1, size=shape, dtype=np.int64).astype(dt)
    bad = np.zeros(shape, bool)
    if bad_frac > 0 and a.size:
        bad = rng.random(shape) < bad_frac
        a = a.copy()
        a[bad] = P.default_badvalue(t)
    return a, bad


def to_pdl(a, t, badflag=False):
    x = P.from_numpy(a, t)
    if badflag:
        x.badflag(1)
    return x


def values_equal(got: np.ndarray, exp: np.ndarray) -> bool:
    if got.dtype.kind == "f":
        return bool(np.array_equal(got, exp, equal_nan=True))
    return bool(np.array_equal(got, exp))


def assert_same(got: P.ndarray, exp: P.ndarray, rtol=0.0, atol=0.0, scale=None, what=""):
    """Types, dims and badflag equal; values exact (ints, indices, bad
    masks) or within |g-e| <= atol + rtol*scale for floats (scale defaults
    to |e|)."""
    assert got.type == exp.type, f"{what}: type {got.type} != {exp.type}"
    assert got.dims == exp.dims, f"{what}: dims {got.dims} != {exp.dims}"
    assert got.badflag() == exp.badflag(), f"{what}: badflag {got.badflag()} != {exp.badflag()}"
    g, e = got.numpy(), exp.numpy()
    if g.dtype.kind != "f" or (rtol == 0 and atol == 0):
        assert values_equal(g, e), f"{what}: values differ\n got {g.ravel()[:16]}\n exp {e.ravel()[:16]}"
        return
    bv = P.default_badvalue(got.datatype)
    gb, eb = g == bv, e == bv
    assert np.array_equal(gb, eb), f"{what}: bad masks differ"
    gn, en = np.isnan(g), np.isnan(e)
    assert np.array_equal(gn, en), f"{what}: NaN masks differ"
    m = ~(gb | gn)
    if scale is None:
        scale = np.abs(e)
    scale = np.broadcast_to(scale, e.shape)
    with np.errstate(invalid="ignore"):
        diff = np.abs(g.astype(np.float64) - e.astype(np.float64))
    tol = atol + rtol * np.abs(scale)
    # equal infinities differ by NaN: equality passes before the tolerance
    bad = m & ~((g == e) | (diff <= tol))
    assert not bad.any(), (f"{what}: {bad.sum()} values outside tolerance; worst diff "
                           f"{diff[m].max() if m.any() else 0} tol {tol[bad].ravel()[:4]}")
