"""pdl_gb300 -- PDL's broadcast-loop hot path (PDL::Ufunc reductions over
dim 0, PDL::Ops plus/mult, PDL::Primitive inner/matmult) on GB300.

The compute lives in libpdlgb300.so (CUDA for sm_103a behind a C ABI,
include/pdlgb300.h).  This package is the host side: a PDL-like ndarray and
the op functions, loading the library on first use and failing loudly when
it has not been built.
"""
from ._abi import PDLError  # noqa: F401
from .ndarray import (  # noqa: F401
    TYPE_NAMES, assign, average, average_bwd, avgover, convert, cumusumover, daverage,
    dcumusumover, default_badvalue, device_count, device_empty, dprodover, dsumover,
    empty, from_numpy, inner, last_launch_info, matmult, matmult_bwd, maximum,
    maximum_ind, maxover, minimum, minimum_ind, minover, mult, mult_bwd, ndarray, null,
    ones, pdl, plus, plus_bwd, prodover, sequence, set_compensated, set_debugging,
    set_default_badvalue, set_matmult_mode, set_stream, set_timing, sumover,
    sumover_bwd, sumover_mult_plus, sync, zeroes)
from .ndarray import (  # noqa: F401
    and2, divide, eq, ge, gt, le, lt, minus, ne, or2, shiftleft, shiftright, xor, xor2,
    andover, bandover, borover, bxorover, firstnonzeroover, orover, xorover, zcover,
    cumuprodover, dcumuprodover, minmaximum, minmaxover, qsort, qsorti, medover, oddmedover,
    modeover, pctover, oddpctover, qsortvec, qsortveci)
from .whole import (  # noqa: F401
    all, and_, any, avg, band, bor, bxor, davg, dprod, dsum, max, median, min, mode, oddmedian,
    oddpct, or_, pct, prod, sum, xorall, zcheck)
from .lazy import Lazy, lazy  # noqa: F401
from .fastraw import gluefraw, mapfraw, readfraw, writefraw  # noqa: F401
from ._abi import MATMULT_BF16X3, MATMULT_BF16X6, MATMULT_SIMT_EXACT, MATMULT_SIMT_FP32  # noqa: F401

# `from pdl_gb300 import *` leaves Python's builtins alone: the whole-array
# functions named like builtins stay reachable as pdl_gb300.sum etc.
_BUILTIN_NAMES = {"sum", "min", "max", "any", "all"}
__all__ = [n for n in dir() if not n.startswith("_") and n not in _BUILTIN_NAMES]
