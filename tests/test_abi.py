"""The C ABI (CPU only): the library loads, exports every symbol that
include/pdlgb300.h declares, and its host-side planner (type selection,
broadcasting, null-output shapes, PDL's dim-check error text) agrees with
the oracle's restatement of PDL's broadcast engine.  No kernel runs here."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pdl_gb300 as P
from pdl_gb300 import _abi as A
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "pdlgb300.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pdlgb300_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_every_declared_symbol():
    L = A.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(A.LIB_PATH)],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pdlgb300_\w+)", out))
    assert set(declared_symbols()) <= exported
    assert set(A.SIGNATURES) == set(declared_symbols())


def test_abi_version_and_struct_layout():
    assert A.lib().pdlgb300_abi_version() == 1
    assert C.sizeof(A.Ndarray) == 312
    assert C.sizeof(A.Error) == 16
    assert C.sizeof(A.Anyval) == 16


def test_type_table_and_default_badvalues():
    L = A.lib()
    sizes = [1, 1, 2, 2, 4, 4, 8, 8, 8, 4, 8]
    for t, s in enumerate(sizes):
        assert L.pdlgb300_type_size(t) == s
        assert L.pdlgb300_type_name(t).decode() == P.TYPE_NAMES[t]
    assert P.default_badvalue(A.L) == -2**31
    assert P.default_badvalue(A.B) == 255
    assert P.default_badvalue(A.F) == np.float32(-3.4028234663852886e38)
    assert P.default_badvalue(A.D) == -1.7976931348623157e308


def test_vtables_mirror_pp_signatures():
    L = A.lib()
    expect = {
        "sumover": (2, 1, [1, 0]), "prodover": (2, 1, [1, 0]), "average": (2, 1, [1, 0]),
        "cumusumover": (2, 1, [1, 1]), "minimum": (2, 1, [1, 0]),
        "minimum_ind": (2, 1, [1, 0]), "plus": (3, 2, [0, 0, 0]), "mult": (3, 2, [0, 0, 0]),
        "inner": (3, 2, [1, 1, 0]), "matmult": (3, 2, [2, 2, 2]),
        "sumover_mult_plus": (4, 3, [1, 1, 1, 0]),
    }
    for name, (npdls, npar, rd) in expect.items():
        vt = L.pdlgb300_get_vtable(name.encode())
        assert vt, name
        v = vt.contents
        assert (v.npdls, v.nparents) == (npdls, npar)
        assert [v.par_realdims[i] for i in range(npdls)] == rd
    assert not L.pdlgb300_get_vtable(b"nosuchop")


def lib_redodims(op, inputs, swap=0):
    L = A.lib()
    vt = L.pdlgb300_get_vtable(op.encode())
    ds = [x._desc(False) for x in inputs]
    out = A.Ndarray()
    L.pdlgb300_ndarray_null(C.byref(out))
    arr = (A.P * (len(ds) + 1))(*[C.pointer(d) for d in ds], C.pointer(out))
    oth = (C.c_int64 * 1)(swap)
    A.check(L.pdlgb300_redodims(vt, arr, oth))
    return tuple(out.dims[i] for i in range(out.ndims)), out.datatype


def Z(t, *dims):
    return P.zeroes(t, *dims)


SHAPE_CASES = [
    ("sumover", [Z("double", 4096, 2048)]),
    ("sumover", [Z("byte", 3, 4, 5)]),
    ("sumover", [Z("float", 7)]),
    ("sumover", [Z("ulong", 0, 3)]),
    ("average", [Z("short", 2, 2)]),
    ("minimum_ind", [Z("float", 9, 2)]),
    ("cumusumover", [Z("sbyte", 4, 3)]),
    ("dsumover", [Z("long", 4)]),
    ("plus", [Z("long", 256, 1, 8192), Z("long", 256, 512, 1)]),
    ("plus", [Z("byte", 3), Z("double", 1, 2)]),
    ("mult", [Z("float", 5, 1, 3), Z("float", 1, 4)]),
    ("inner", [Z("double", 4096, 3), Z("double", 4096)]),
    ("inner", [Z("double", 1, 3), Z("double", 5)]),
    ("matmult", [Z("float", 1024, 2048, 16), Z("float", 2048, 1024)]),
    ("matmult", [Z("double", 3, 2, 1, 4), Z("double", 5, 3, 7, 1)]),
    ("sumover_mult_plus", [Z("long", 256, 1, 8192), Z("long", 256, 512, 1), Z("long", 256, 1, 8192)]),
    # the widened rows: type rules (GenericTypes, typed outputs) and shapes
    ("minus", [Z("short", 3, 1), Z("float", 1, 4)]),
    ("gt", [Z("long", 5), Z("double", 5)]),
    ("shiftleft", [Z("double", 4), Z("byte", 4)]),       # integer types only: longlong
    ("xor", [Z("float", 2, 3), Z("long", 2, 1)]),
    ("andover", [Z("float", 6, 2)]),
    ("bandover", [Z("double", 6, 2)]),                  # integer types only: longlong
    ("firstnonzeroover", [Z("ushort", 3, 3)]),
    ("cumuprodover", [Z("byte", 5, 2)]),
    ("dcumuprodover", [Z("short", 5, 2)]),
    ("qsort", [Z("float", 7, 3)]),
    ("qsorti", [Z("byte", 7, 3)]),
    ("medover", [Z("long", 9, 4, 2)]),
    ("oddmedover", [Z("double", 9)]),
    ("pctover", [Z("float", 9, 4), Z("double")]),
    ("oddpctover", [Z("long", 9, 4), Z("long", 4)]),
    ("modeover", [Z("double", 7, 2)]),                  # integer types only: longlong
]


@pytest.mark.parametrize("op,inputs", SHAPE_CASES, ids=[f"{c[0]}{i}" for i, c in enumerate(SHAPE_CASES)])
def test_null_output_shape_and_type_match_oracle(op, inputs):
    got = lib_redodims(op, inputs)
    if op == "sumover_mult_plus":  # composition of mult, plus, sumover
        assert got[0] == tuple(max(a, b, c) for a, b, c in
                               zip(*[x.dims[1:] + (1,) * (3 - x.ndims) for x in inputs]))
        return
    assert got == O.redodims(op, inputs)


ERROR_CASES = [
    # (op, inputs, outputs-spec, regex)   -- t/core.t:249-300 analogues
    ("plus", [Z("double", 3), Z("double", 4)], None, r"Mismatched implicit broadcast dimension 0: size 3 vs\. 4"),
    ("sumover", [Z("double", 3, 2)], Z("double", 1), r"implicit dim 0 size 2, but dim has size 1"),
    ("sumover", [Z("double", 3, 2)], Z("double", 3), r"Mismatched implicit broadcast dimension 0"),
    ("cumusumover", [Z("double", 3, 2)], Z("double", 2, 2), r"index 'n' size 3, but ndarray dim has size 2"),
    ("inner", [Z("double", 3), Z("double", 4)], None, r"index 'n' size 3, but ndarray dim has size 4"),
    ("sumover", [Z("double", 3, 2)], "scalar", r"implicit dim 0 size 2, can't broadcast over output ndarray with size > 1"),
    ("plus", [Z("double", 2, 2), Z("double", 2)], "dummy", r"implicit dim 1 size 2, but dim is dummy"),
    ("cumusumover", [Z("double", 2, 2)], "dummy0", r"index 'n' size 2, can't broadcast over dummy dim with size > 1"),
    ("matmult", [Z("double", 3, 2), Z("double", 2, 4)], None, r"index 't' size 3, but ndarray dim has size 4"),
    ("pctover", [Z("double", 5, 3), Z("double", 4)], None, r"Mismatched implicit broadcast dimension 0: size 3 vs\. 4"),
    ("qsort", [Z("double", 3, 2)], Z("double", 2, 2), r"index 'n' size 3, but ndarray dim has size 2"),
]


def _outspec(spec, inputs):
    if spec is None:
        return None
    if spec == "scalar":
        return P.zeroes("double")
    if spec == "dummy":
        return P.zeroes("double", 2).dummy(1, 2)
    if spec == "dummy0":
        return P.zeroes("double", 2).dummy(0, 2)
    return spec


@pytest.mark.parametrize("op,inputs,outspec,pattern", ERROR_CASES,
                         ids=[f"{c[0]}{i}" for i, c in enumerate(ERROR_CASES)])
def test_dim_errors_match_oracle_text(op, inputs, outspec, pattern):
    out = _outspec(outspec, inputs)
    L = A.lib()
    vt = L.pdlgb300_get_vtable(op.encode())
    ds = [x._desc(False) for x in inputs]
    if out is None:
        od = A.Ndarray()
        L.pdlgb300_ndarray_null(C.byref(od))
    else:
        od = out._desc(False)
    arr = (A.P * (len(ds) + 1))(*[C.pointer(d) for d in ds], C.pointer(od))
    e = L.pdlgb300_redodims(vt, arr, None)
    assert e.error == A.EUSERERROR
    msg = e.message.decode()
    assert re.search(pattern, msg), msg
    # same text as the oracle's restatement of pdl_param_error
    with pytest.raises(O.OracleError) as ei:
        O.run(op, inputs, [out])
    assert str(ei.value) == msg


def test_error_table_format():
    # pdl_param_error prints the active and broadcast dims of every pdl
    with pytest.raises(P.PDLError) as ei:
        lib_redodims("plus", [Z("double", 3), Z("double", 4)])
    msg = str(ei.value)
    assert msg.startswith("PDL::Ops::plus(a,b,c): parameter 'b': Mismatched implicit broadcast dimension 0")
    assert "There are 3 PDLs in the expression; 1 broadcast dim." in msg
    assert "   #  0 (normal):        3" in msg
    assert "   #  2 (null)" in msg


def test_matmult_wrapper_dim_mismatch_message():
    pb = P.pdl([[1.0, 1], [0, 2], [0, 2], [1, 1]])
    eq = P.pdl(np.array([[1, 1, 1, 1]], np.float32))
    with pytest.raises(P.PDLError, match=r"Dim mismatch in matmult of \[2x4\] x \[4x1\]: 2 != 1"):
        P.matmult(pb, eq)


def test_unsupported_types_rejected():
    L = A.lib()
    x = A.Ndarray()
    dims = (C.c_int64 * 1)(4)
    A.check(L.pdlgb300_ndarray_init(C.byref(x), A.LD, 1, dims, None, None))
    out = A.Ndarray()
    L.pdlgb300_ndarray_null(C.byref(out))
    e = L.pdlgb300_run_sumover(C.byref(x), C.byref(out))
    assert e.error == A.EUSERERROR and b"ldouble" in e.message


def test_options_roundtrip():
    L = A.lib()
    old = L.pdlgb300_get_option(A.OPT_MATMULT_MODE)
    for m in (0, 1, 2, 3):
        A.check(L.pdlgb300_set_option(A.OPT_MATMULT_MODE, m))
        assert L.pdlgb300_get_option(A.OPT_MATMULT_MODE) == m
    assert L.pdlgb300_set_option(A.OPT_MATMULT_MODE, 7).error
    A.check(L.pdlgb300_set_option(A.OPT_MATMULT_MODE, old))


def test_op_package_names_the_defining_package():
    """PDL names ops by their package-qualified pp_def name in its errors."""
    L = A.lib()
    assert L.pdlgb300_op_package(b"plus") == b"PDL::Ops::"
    assert L.pdlgb300_op_package(b"sumover") == b"PDL::Ufunc::"
    assert L.pdlgb300_op_package(b"matmult") == b"PDL::Primitive::"
    assert L.pdlgb300_op_package(b"sumover_mult_plus") == b""
