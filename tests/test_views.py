"""View arithmetic of the mirror (no GPU): mv and clump/flat shapes and
strides as documented in lib/PDL/Core.pm:1806-1864 and Slices.pd:1563-1587.
A clump whose dims do not merge makes a copy through the library and is
covered by the GPU tests."""
import numpy as np
import pytest

import pdl_gb300 as P


def test_clump_documented_shapes():
    z = P.zeroes("double", 2, 3, 5, 7)
    assert z.clump(-1).dims == (210,)
    assert z.clump(-2).dims == (30, 7)
    assert z.clump(2).dims == (6, 5, 7)
    assert z.clump(3).dims == (30, 7)
    assert z.clump(1, 2).dims == (2, 15, 7)
    assert z.clump(9).dims == (210,)
    assert z.clump(0).dims == (1, 2, 3, 5, 7)


def test_clump_views_keep_element_order():
    a = np.arange(60.0).reshape(3, 4, 5)           # PDL dims (5, 4, 3)
    x = P.pdl(a)
    f = x.flat()
    assert f.dims == (60,) and f.incs == (1,) and f.storage is x.storage
    np.testing.assert_array_equal(f.numpy(), a.reshape(-1))
    s = x.slice(1)                                  # dims (4, 3), incs (5, 20): merge
    assert s.clump(-1).dims == (12,) and s.clump(-1).incs == (5,)
    np.testing.assert_array_equal(s.clump(-1).numpy(), a[:, :, 1].reshape(-1))
    d = x.dummy(1)                                  # a size-1 dim merges with anything
    assert d.clump(-1).incs == (1,)
    assert P.pdl(np.array(3.0)).flat().dims == (1,)
    e = P.zeroes("long", 0, 4)
    assert e.flat().dims == (0,)


def test_mv():
    x = P.zeroes("double", 4, 3, 2)
    assert x.mv(0, 2).dims == (3, 2, 4)
    assert x.mv(2, 0).dims == (2, 4, 3)
    assert x.mv(-1, 0).dims == (2, 4, 3)
    assert x.mv(0, 2).incs == (4, 12, 1)
    with pytest.raises(P.PDLError, match="out of range"):
        x.mv(0, 3)


def test_clump_list_errors():
    x = P.zeroes("double", 4, 3, 2)
    with pytest.raises(P.PDLError, match="duplicate"):
        x.clump(1, 1)
    with pytest.raises(P.PDLError, match="larger than greatest"):
        x.clump(0, 5)


def test_clump_views_against_numpy_on_random_views():
    """Random slices, exchanges and dummies: every clump that stays a view
    holds the elements of the view in PDL order (dim 0 fastest); the ones
    that need a copy are left to the GPU tests."""
    rng = np.random.default_rng(3)
    done = 0
    for _ in range(300):
        shape = tuple(int(v) for v in rng.integers(1, 5, size=int(rng.integers(1, 4))))
        a = np.arange(int(np.prod(shape)), dtype=np.float64).reshape(shape)
        x = P.pdl(a)
        if rng.random() < 0.4 and x.ndims > 1:
            i, j = (int(v) for v in rng.choice(x.ndims, 2, replace=False))
            x = x.xchg(i, j)
        if rng.random() < 0.3:
            x = x.dummy(int(rng.integers(0, x.ndims + 1)), int(rng.integers(1, 3)))
        if rng.random() < 0.3:
            k = int(rng.integers(0, x.ndims))
            specs = [slice(None)] * x.ndims
            specs[k] = slice(None, None, 2)
            x = x.slice(*specs)
        n = int(rng.integers(-x.ndims - 1, x.ndims + 2))
        try:
            c = x.clump(n)
        except P.PDLError:
            continue  # a copy: needs the device
        v = x.numpy()                              # numpy order: last PDL dim first
        nd = x.ndims
        m = nd if n == -1 else (max(nd + n + 1, 0) if n < -1 else min(n, nd))
        want = v.reshape(v.shape[: nd - m] + (-1,)) if m else v[..., None]
        assert c.numpy().shape == want.shape and np.array_equal(c.numpy(), want)
        done += 1
    assert done > 150
