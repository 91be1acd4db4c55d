"""ctypes view of include/pdlgb300.h and the loader of libpdlgb300.so.

The library is the product: if it is missing or fails to load, importing the
package raises (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

MAXDIMS = 16

# pdlgb300_datatype: PDL's own type order (lib/PDL/Types.pm)
SB, B, S, US, L, UL, IND, ULL, LL, F, D, LD, CF, CD, CLD = range(15)
NTYPES = 15

BADVAL = 0x1
NOMYDIMS = 0x2

ENONE, EUSERERROR, EFATAL = 0, 1, 2

MATMULT_SIMT_FP32, MATMULT_BF16X3, MATMULT_BF16X6, MATMULT_SIMT_EXACT = 0, 1, 2, 3
OPT_MATMULT_MODE, OPT_F32_COMPENSATED, OPT_DEBUG = 1, 2, 3


class Value(C.Union):
    _fields_ = [("A", C.c_int8), ("B", C.c_uint8), ("S", C.c_int16), ("U", C.c_uint16),
                ("L", C.c_int32), ("K", C.c_uint32), ("N", C.c_int64), ("P", C.c_uint64),
                ("Q", C.c_int64), ("F", C.c_float), ("D", C.c_double)]


class Anyval(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("value", Value)]


class Error(C.Structure):
    _fields_ = [("error", C.c_int32), ("reserved", C.c_int32), ("message", C.c_char_p)]


class Ndarray(C.Structure):
    _fields_ = [("datatype", C.c_int32), ("ndims", C.c_int32), ("state", C.c_uint32),
                ("has_badvalue", C.c_int32), ("badvalue", Anyval), ("offs", C.c_int64),
                ("data", C.c_void_p), ("ddata", C.c_void_p),
                ("dims", C.c_int64 * MAXDIMS), ("incs", C.c_int64 * MAXDIMS)]


class Vtable(C.Structure):
    _fields_ = [("name", C.c_char_p), ("npdls", C.c_int32), ("nparents", C.c_int32),
                ("ninds", C.c_int32), ("nother", C.c_int32),
                ("par_names", C.POINTER(C.c_char_p)), ("par_realdims", C.POINTER(C.c_int32)),
                ("par_flags", C.POINTER(C.c_int32)), ("par_types", C.POINTER(C.c_int32)),
                ("ind_ids", C.POINTER(C.c_int32)), ("ind_names", C.POINTER(C.c_char_p)),
                ("gentypes", C.POINTER(C.c_int32))]


class LaunchInfo(C.Structure):
    _fields_ = [("op", C.c_char * 32), ("kernel", C.c_char * 64), ("datatype", C.c_int32),
                ("nlaunches", C.c_int32), ("grid", C.c_int64), ("block", C.c_int64),
                ("rows", C.c_int64), ("n", C.c_int64), ("bytes", C.c_double),
                ("flops", C.c_double), ("kernel_ms", C.c_double), ("h2d_ms", C.c_double),
                ("d2h_ms", C.c_double), ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["op"] = self.op.decode()
        d["kernel"] = self.kernel.decode()
        return d


P = C.POINTER(Ndarray)
PP = C.POINTER(P)

# name -> (restype, argtypes)
SIGNATURES = {
    "pdlgb300_abi_version": (C.c_int32, []),
    "pdlgb300_type_size": (C.c_size_t, [C.c_int32]),
    "pdlgb300_type_name": (C.c_char_p, [C.c_int32]),
    "pdlgb300_ndarray_init": (Error, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p]),
    "pdlgb300_ndarray_null": (Error, [P]),
    "pdlgb300_get_default_badvalue": (Error, [C.c_int32, C.POINTER(Anyval)]),
    "pdlgb300_set_default_badvalue": (Error, [C.c_int32, Anyval]),
    "pdlgb300_get_vtable": (C.POINTER(Vtable), [C.c_char_p]),
    "pdlgb300_op_package": (C.c_char_p, [C.c_char_p]),
    "pdlgb300_redodims": (Error, [C.POINTER(Vtable), PP, C.POINTER(C.c_int64)]),
    "pdlgb300_run": (Error, [C.POINTER(Vtable), PP, C.POINTER(C.c_int64)]),
    "pdlgb300_run_sumover": (Error, [P, P]),
    "pdlgb300_run_dsumover": (Error, [P, P]),
    "pdlgb300_run_prodover": (Error, [P, P]),
    "pdlgb300_run_dprodover": (Error, [P, P]),
    "pdlgb300_run_cumusumover": (Error, [P, P]),
    "pdlgb300_run_dcumusumover": (Error, [P, P]),
    "pdlgb300_run_average": (Error, [P, P]),
    "pdlgb300_run_daverage": (Error, [P, P]),
    "pdlgb300_run_minimum": (Error, [P, P]),
    "pdlgb300_run_maximum": (Error, [P, P]),
    "pdlgb300_run_minimum_ind": (Error, [P, P]),
    "pdlgb300_run_minmaximum": (Error, [P, P, P, P, P]),
    "pdlgb300_run_qsort": (Error, [P, P]),
    "pdlgb300_run_qsorti": (Error, [P, P]),
    "pdlgb300_run_medover": (Error, [P, P]),
    "pdlgb300_run_oddmedover": (Error, [P, P]),
    "pdlgb300_run_pctover": (Error, [P, P, P]),
    "pdlgb300_run_oddpctover": (Error, [P, P, P]),
    "pdlgb300_run_modeover": (Error, [P, P]),
    "pdlgb300_run_qsortvec": (Error, [P, P]),
    "pdlgb300_run_qsortveci": (Error, [P, P]),
    "pdlgb300_fraw_header": (Error, [C.c_char_p, C.c_char_p, P]),
    "pdlgb300_readfraw_into": (Error, [C.c_char_p, P]),
    "pdlgb300_writefraw": (Error, [P, C.c_char_p, C.c_char_p]),
    "pdlgb300_run_expr_reduce": (Error, [C.POINTER(Vtable), C.c_int32, PP, C.c_int32, C.c_void_p, P]),
    **{f"pdlgb300_run_{op}": (Error, [P, P])
       for op in ("andover", "orover", "xorover", "zcover", "bandover", "borover",
                  "bxorover", "firstnonzeroover", "cumuprodover", "dcumuprodover")},
    "pdlgb300_run_maximum_ind": (Error, [P, P]),
    "pdlgb300_run_plus": (Error, [P, P, P, C.c_int]),
    "pdlgb300_run_mult": (Error, [P, P, P, C.c_int]),
    **{f"pdlgb300_run_{op}": (Error, [P, P, P, C.c_int])
       for op in ("minus", "divide", "gt", "lt", "le", "ge", "eq", "ne", "shiftleft",
                  "shiftright", "or2", "and2", "xor")},
    "pdlgb300_run_inner": (Error, [P, P, P]),
    "pdlgb300_run_matmult": (Error, [P, P, P]),
    "pdlgb300_run_sumover_mult_plus": (Error, [P, P, P, P]),
    "pdlgb300_convert": (Error, [P, P]),
    "pdlgb300_sumover_bwd": (Error, [P, P]),
    "pdlgb300_average_bwd": (Error, [P, P]),
    "pdlgb300_plus_bwd": (Error, [P, P, P]),
    "pdlgb300_mult_bwd": (Error, [P, P, P, P, P]),
    "pdlgb300_matmult_bwd": (Error, [P, P, P, P, P]),
    "pdlgb300_set_option": (Error, [C.c_int32, C.c_int64]),
    "pdlgb300_get_option": (C.c_int64, [C.c_int32]),
    "pdlgb300_set_stream": (Error, [C.c_void_p]),
    "pdlgb300_device_alloc": (Error, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "pdlgb300_free": (Error, [C.c_void_p]),
    "pdlgb300_to_device": (Error, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "pdlgb300_to_host": (Error, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "pdlgb300_to_device_async": (Error, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "pdlgb300_to_host_async": (Error, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "pdlgb300_sync": (Error, []),
    "pdlgb300_device_count": (Error, [C.POINTER(C.c_int32)]),
    "pdlgb300_last_launch": (Error, [C.POINTER(LaunchInfo)]),
    "pdlgb300_set_timing": (Error, [C.c_int32]),
    "pdlgb300_sumover_noalloc": (Error, [P, P]),
}

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libpdlgb300.so"
_lib = None


def lib() -> C.CDLL:
    """Load libpdlgb300.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("PDLGB300_LIB", LIB_PATH))
        if not path.exists():
            raise ImportError(
                f"{path} not found: build the GB300 kernels with "
                "`python -m pdl_gb300.build` (there is no CPU fallback)")
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class PDLError(RuntimeError):
    """An error returned by the library (PDL's barf)."""

    def __init__(self, kind: int, message: str):
        super().__init__(message)
        self.kind = kind


def check(e: Error) -> None:
    if e.error:
        msg = e.message.decode() if e.message else "unknown error"
        raise PDLError(e.error, msg)
