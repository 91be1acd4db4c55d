"""pdlgb300_sumover_noalloc: sumover for callers that cannot let the library
allocate device memory (it keeps its split partials in a fixed device
array).  Checked through the C ABI against pdlgb300_run_sumover on two calls
in a row.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import pdl_gb300 as P
from pdl_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def _dev(arr, t):
    """A device-resident ndarray descriptor holding arr (the test allocates)."""
    x = P.from_numpy(arr, t).to_device()
    return x, x._desc(True)


def _out(t, dims):
    y = P.device_empty(t, *dims)
    return y, y._desc(True)


@pytest.mark.parametrize("t,shape", [("double", (5, 300000)), ("double", (64, 5000)),
                                     ("float", (3, 200000)), ("long", (4, 100000)),
                                     ("byte", (7, 3000))])
def test_noalloc_matches_sumover_twice(gpu, t, shape):
    L = A.lib()
    rng = np.random.default_rng(2024)
    if t in ("double", "float"):
        a = rng.uniform(-1, 1, size=shape)
    else:
        a = rng.integers(0 if t == "byte" else -1000, 200 if t == "byte" else 1000, size=shape)
    x, dx = _dev(a, t)
    ref, dref = _out(P.sumover(x).type, shape[:-1][::-1])
    A.check(L.pdlgb300_run_sumover(C.byref(dx), C.byref(dref)))
    ref.storage.fresh = "dev"
    want = ref.numpy()
    tol = None
    if t in ("double", "float"):
        eps = 2.0 ** -53 if t == "double" else 2.0 ** -24
        tol = (shape[-1] + 2) * eps * np.abs(a).sum(-1)
    for _ in range(2):  # the array keeps the last call's contents
        out, dout = _out(ref.type, shape[:-1][::-1])
        A.check(L.pdlgb300_sumover_noalloc(C.byref(dx), C.byref(dout)))
        A.check(L.pdlgb300_sync())
        out.storage.fresh = "dev"
        got = out.numpy()
        if tol is None:
            assert np.array_equal(got, want)
        else:
            assert np.all(np.abs(got.astype(np.float64) - want) <= tol)


def test_noalloc_rejects_too_many_rows_and_host_memory(gpu):
    L = A.lib()
    a = np.zeros((200000, 8))
    x, dx = _dev(a, "double")
    out, dout = _out("double", (200000,))
    e = L.pdlgb300_sumover_noalloc(C.byref(dx), C.byref(dout))
    assert e.error == A.EUSERERROR and b"limit" in e.message
    h = P.pdl(np.zeros((3, 8)))
    hd = h._desc(False)
    ho = P.pdl(np.zeros(3))._desc(False)
    e = L.pdlgb300_sumover_noalloc(C.byref(hd), C.byref(ho))
    assert e.error == A.EUSERERROR and b"device-resident" in e.message


@pytest.mark.parametrize("t,limit", [("double", 32760), ("float", 32760), ("long", 43680)])
def test_noalloc_row_limit_boundary(gpu, t, limit):
    """The documented row limit: (1 MiB - 256) / (2 * (accumulator + 8))
    rows are accepted and give sumover's result; one more row is refused."""
    L = A.lib()
    a = np.ones((limit + 1, 3))
    a[:, 1] = np.arange(limit + 1) % 7
    x, dx = _dev(a, t)
    ref = P.sumover(x).numpy()
    ok_view = P.from_numpy(a[:limit], t).to_device()
    dv = ok_view._desc(True)
    out, dout = _out(P.sumover(ok_view).type, (limit,))
    A.check(L.pdlgb300_sumover_noalloc(C.byref(dv), C.byref(dout)))
    A.check(L.pdlgb300_sync())
    out.storage.fresh = "dev"
    assert np.array_equal(out.numpy(), ref[:limit])
    big, dbig = _out(P.sumover(x).type, (limit + 1,))
    e = L.pdlgb300_sumover_noalloc(C.byref(dx), C.byref(dbig))
    assert e.error == A.EUSERERROR and f"at most {limit} rows".encode() in e.message
