"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle (pdl_oracle.c).

Used by tests/ as the parity checker and by bench.py's CPU-baseline leg and
reference arm.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from pdl_gb300 import _abi as A
from pdl_gb300.ndarray import NP_DTYPES, Storage, ndarray

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libpdloracle.so"
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "pdl_oracle.c").stat().st_mtime:
            build()
        L = C.CDLL(str(LIB))
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.c_char_p, A.PP, C.POINTER(C.c_int64), C.c_int,
                                 C.c_char_p, C.c_size_t]
        L.oracle_redodims.restype = C.c_int
        L.oracle_redodims.argtypes = [C.c_char_p, A.PP, C.c_char_p, C.c_size_t]
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_npdls.restype = C.c_int
        L.oracle_npdls.argtypes = [C.c_char_p]
        L.oracle_sumover_bwd.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
        L.oracle_average_bwd.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
        L.oracle_matmult_bwd.argtypes = [C.c_void_p] * 5 + [C.c_int64] * 6
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _host_desc(x: ndarray) -> A.Ndarray:
    return x._desc(False)


def run(op: str, inputs, outputs=None, swap: int = 0, nthreads: int = 1):
    """Run `op` on the CPU oracle.  inputs: ndarrays; outputs: list of
    ndarray or None (null).  Returns the output ndarrays (host)."""
    outputs = outputs if outputs is not None else [None]
    npdls = lib().oracle_npdls(op.encode())
    if npdls < 0:
        raise OracleError(f"unknown op {op}")
    if len(inputs) + len(outputs) != npdls:
        raise OracleError(f"{op} takes {npdls} ndarrays, got {len(inputs) + len(outputs)}")
    ds = [_host_desc(x) for x in inputs]
    keep = []
    for o in outputs:
        if o is None:
            d = A.Ndarray()
            d.state = A.NOMYDIMS
            d.badvalue.type = -1
            ds.append(d)
        else:
            ds.append(_host_desc(o))
            keep.append(o)
    arr = (A.P * len(ds))(*[C.pointer(d) for d in ds])
    other = (C.c_int64 * 1)(swap)
    msg = C.create_string_buffer(8192)
    rc = lib().oracle_run(op.encode(), arr, other, nthreads, msg, 8192)
    if rc:
        raise OracleError(msg.value.decode())
    res = []
    for k, o in enumerate(outputs):
        d = ds[len(inputs) + k]
        if o is None:
            dims = tuple(d.dims[i] for i in range(d.ndims))
            t = d.datatype
            n = int(np.prod(dims, dtype=np.int64)) if dims else 1
            it = np.dtype(NP_DTYPES[t]).itemsize
            # (copied with memmove: string_at's size overflows at 2 GiB)
            host = np.empty(max(n * it, 1), dtype=np.uint8)
            if n:
                C.memmove(host.ctypes.data, d.data, n * it)
            lib().oracle_free(d.data)
            o = ndarray(Storage(n * it, host=host), t, dims)
        o._badflag = bool(d.state & A.BADVAL)
        res.append(o)
    return res


def redodims(op: str, inputs, swap: int = 0):
    """Shapes and types of null outputs, or OracleError with PDL's text."""
    ds = [_host_desc(x) for x in inputs]
    d = A.Ndarray()
    d.state = A.NOMYDIMS
    ds.append(d)
    if swap:
        ds[0], ds[1] = ds[1], ds[0]
    arr = (A.P * len(ds))(*[C.pointer(x) for x in ds])
    msg = C.create_string_buffer(8192)
    if lib().oracle_redodims(op.encode(), arr, msg, 8192):
        raise OracleError(msg.value.decode())
    return tuple(d.dims[i] for i in range(d.ndims)), d.datatype
