"""A PDL-like ndarray over libpdlgb300 (the host side of the drop-in path).

Dims are in PDL's order: dim 0 varies fastest (a numpy array of shape
(r, c) is an ndarray of dims (c, r), as `pdl([[..],[..]])` is in PDL).
Views (`xchg`, `dummy`, `slice`) share their parent's storage through
element increments and an offset, like PDL's vaffine views.  Storage lives in
host memory, in a device mirror, or both; `to_device()`/`to_host()` move it
explicitly, and an op runs on the device mirrors whenever one of its inputs
has one.  Every op is the library's; there is no CPU code path.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _abi as A
from ._abi import PDLError, check, lib

TYPE_NAMES = ["sbyte", "byte", "short", "ushort", "long", "ulong", "indx",
              "ulonglong", "longlong", "float", "double", "ldouble", "cfloat",
              "cdouble", "cldouble"]
NP_DTYPES = {A.SB: np.int8, A.B: np.uint8, A.S: np.int16, A.US: np.uint16,
             A.L: np.int32, A.UL: np.uint32, A.IND: np.int64, A.ULL: np.uint64,
             A.LL: np.int64, A.F: np.float32, A.D: np.float64}
TYPE_OF = {name: i for i, name in enumerate(TYPE_NAMES)}
_NP_TO_TYPE = {np.dtype(np.int8): A.SB, np.dtype(np.uint8): A.B, np.dtype(np.int16): A.S,
               np.dtype(np.uint16): A.US, np.dtype(np.int32): A.L, np.dtype(np.uint32): A.UL,
               np.dtype(np.int64): A.LL, np.dtype(np.uint64): A.ULL,
               np.dtype(np.float32): A.F, np.dtype(np.float64): A.D}


def type_code(t) -> int:
    if isinstance(t, str):
        return TYPE_OF[t]
    if isinstance(t, (int, np.integer)):
        return int(t)
    return _NP_TO_TYPE[np.dtype(t)]


# ------------------------------------------------------------------ storage

class Storage:
    """One data buffer with an optional device mirror."""

    def __init__(self, nbytes: int, host: Optional[np.ndarray] = None, dev: Optional[int] = None):
        self.nbytes = int(nbytes)
        self.host = host          # flat uint8 view or typed array
        self.dev = dev            # device pointer (int) or None
        self.fresh = "host" if host is not None else "dev"
        self.readonly = False     # host memory that must not be written (a read-only file map)

    def host_ptr(self) -> int:
        return self.host.ctypes.data

    def ensure_dev(self) -> int:
        if self.dev is None:
            p = C.c_void_p()
            check(lib().pdlgb300_device_alloc(max(self.nbytes, 16), C.byref(p)))
            self.dev = p.value
            if self.host is not None and self.nbytes:
                check(lib().pdlgb300_to_device(self.dev, self.host.ctypes.data, self.nbytes))
            self.fresh = "both"
        elif self.fresh == "host":
            if self.nbytes:
                check(lib().pdlgb300_to_device(self.dev, self.host.ctypes.data, self.nbytes))
            self.fresh = "both"
        return self.dev

    def ensure_host(self) -> np.ndarray:
        if self.host is None:
            self.host = np.empty(max(self.nbytes, 1), dtype=np.uint8)
        if self.fresh == "dev":
            if self.readonly:
                raise PDLError(A.EUSERERROR, "device data cannot be written back to a read-only map")
            if self.nbytes:
                check(lib().pdlgb300_to_host(self.host.ctypes.data, self.dev, self.nbytes))
            self.fresh = "both"
        return self.host

    def __del__(self):
        try:
            if self.dev is not None and lib is not None:
                lib().pdlgb300_free(self.dev)
        except Exception:
            pass


# ------------------------------------------------------------------ ndarray

def _deferred(o) -> bool:
    """o is a recorded expression: let its reflected operator record the op."""
    return getattr(o, "_deferred", False)


class ndarray:
    def __init__(self, storage: Storage, datatype: int, dims: Sequence[int],
                 incs: Optional[Sequence[int]] = None, offs: int = 0,
                 badflag: bool = False, badvalue=None):
        self.storage = storage
        self.datatype = int(datatype)
        self.dims = tuple(int(d) for d in dims)
        if incs is None:
            incs, s = [], 1
            for d in self.dims:
                incs.append(s)
                s *= d
        self.incs = tuple(int(i) for i in incs)
        self.offs = int(offs)
        self._badflag = bool(badflag)
        self._badvalue = badvalue

    # -- introspection
    @property
    def ndims(self) -> int:
        return len(self.dims)

    @property
    def nelem(self) -> int:
        return int(np.prod(self.dims, dtype=np.int64)) if self.dims else 1

    @property
    def type(self) -> str:
        return TYPE_NAMES[self.datatype]

    @property
    def np_dtype(self):
        return NP_DTYPES[self.datatype]

    def dim(self, i: int) -> int:
        return self.dims[i] if i < self.ndims else 1

    def getndims(self) -> int:
        return self.ndims

    @property
    def on_device(self) -> bool:
        return self.storage.dev is not None and self.storage.fresh in ("dev", "both")

    # -- read-only (PDL's readonly / is_readonly; a read-only file map is always)
    def readonly(self) -> "ndarray":
        self._readonly = True
        return self

    def is_readonly(self) -> bool:
        return getattr(self, "_readonly", False) or self.storage.readonly

    # -- bad values (lib/PDL/Bad.pd)
    def badflag(self, flag: Optional[bool] = None):
        if flag is None:
            return self._badflag
        self._badflag = bool(flag)
        return self._badflag

    def badvalue(self, v=None):
        if v is None:
            if self._badvalue is not None:
                return self._badvalue
            return default_badvalue(self.datatype)
        self._badvalue = v
        return v

    # -- data access
    def numpy(self) -> np.ndarray:
        """A numpy copy, shape = reversed dims."""
        host = self.storage.ensure_host()
        it = np.dtype(self.np_dtype).itemsize
        if self.nelem == 0:
            return np.zeros(self.dims[::-1], dtype=self.np_dtype)
        base = np.frombuffer(host, dtype=np.uint8)
        typed = base[: (len(base) // it) * it].view(self.np_dtype)
        v = np.lib.stride_tricks.as_strided(
            typed[self.offs:], shape=self.dims[::-1],
            strides=tuple(i * it for i in self.incs[::-1]))
        return np.array(v)

    def to_device(self) -> "ndarray":
        self.storage.ensure_dev()
        return self

    def to_host(self) -> "ndarray":
        self.storage.ensure_host()
        return self

    def at(self, *idx):
        return self.numpy()[tuple(idx[::-1])]

    def __repr__(self):
        return f"ndarray({self.type}, dims={self.dims}, badflag={int(self._badflag)})"

    # -- views (vaffine): share storage
    def _view(self, dims, incs, offs) -> "ndarray":
        return ndarray(self.storage, self.datatype, dims, incs, offs, self._badflag, self._badvalue)

    def xchg(self, i: int, j: int) -> "ndarray":
        d, s = list(self.dims), list(self.incs)
        d[i], d[j] = d[j], d[i]
        s[i], s[j] = s[j], s[i]
        return self._view(d, s, self.offs)

    def transpose(self) -> "ndarray":
        x = self
        while x.ndims < 2:
            x = x.dummy(0)
        return x.xchg(0, 1)

    def dummy(self, pos: int, size: int = 1) -> "ndarray":
        d, s = list(self.dims), list(self.incs)
        if pos < 0:
            pos = len(d) + 1 + pos
        while len(d) < pos:
            d.append(1)
            s.append(0)
        d.insert(pos, size)
        s.insert(pos, 0)
        return self._view(d, s, self.offs)

    def mv(self, n1: int, n2: int) -> "ndarray":
        """Move dim n1 to position n2, the dims between shifting over
        (lib/PDL/Slices.pd:1563-1587; negative dims count from the end)."""
        nd = self.ndims
        a, b = n1 + nd if n1 < 0 else n1, n2 + nd if n2 < 0 else n2
        if min(a, b) < 0 or max(a, b) >= nd:
            raise PDLError(A.EUSERERROR, f"One of dims {n1}, {n2} out of range: should be 0<=dim<{nd}")
        d, s = list(self.dims), list(self.incs)
        d.insert(b, d.pop(a))
        s.insert(b, s.pop(a))
        return self._view(d, s, self.offs)

    def clump(self, *args) -> "ndarray":
        """Merge dims into one (lib/PDL/Core.pm:1806-1864, Slices.pd:1373-1398).
        clump(n): n > 0 the first n dims, -1 all of them, n < -1 leaves -n-1
        dims behind; clump(d1, d2, ...): those dims, merged in the order given
        and placed at the lowest of them.  The result is a view when the
        merged dims have compatible strides, else a contiguous copy made on
        the ndarray's side (host or device), into which assignments do not
        flow back."""
        if len(args) > 1:
            nd = self.ndims
            if len(args) > nd:
                raise PDLError(A.EUSERERROR, "too many dimensions")
            seen = set()
            for k in args:
                if k > nd - 1:
                    raise PDLError(A.EUSERERROR, f"dimension index {k} larger than greatest dimension")
                if k in seen:
                    raise PDLError(A.EUSERERROR, f"duplicate dimension {k}")
                seen.add(k)
            order = list(args) + [k for k in range(nd) if k not in seen]
            v = self._view([self.dims[k] for k in order], [self.incs[k] for k in order], self.offs)
            v = v.clump(len(args))
            targd = min(min(args), nd - 1)
            return v.mv(0, targd) if targd > 0 else v
        n = int(args[0])
        nd = self.ndims
        if n > nd:
            n = nd
        if n < -1:
            n = max(nd + n + 1, 0)
        nrem = nd if n == -1 else n
        d1 = int(np.prod(self.dims[:nrem], dtype=np.int64)) if nrem else 1
        rest_d, rest_s = list(self.dims[nrem:]), list(self.incs[nrem:])
        inc, ok = None, True
        for k in range(nrem):
            if self.dims[k] == 1:
                continue
            if inc is None:
                inc = self.incs[k]
            elif self.incs[k] != expect:
                ok = False
                break
            expect = self.incs[k] * self.dims[k]
        if d1 == 0:
            ok, inc = True, 1
        if ok:
            return self._view([d1] + rest_d, [1 if inc is None else inc] + rest_s, self.offs)
        c = convert(self, self.datatype)
        c._badvalue = self._badvalue
        c._badflag = self._badflag
        return c.clump(n)

    def flat(self) -> "ndarray":
        """clump(-1) unless already 1-D (lib/PDL/Core.pm:3071-3073)."""
        return self if self.ndims == 1 else self.clump(-1)

    def sclr(self):
        """The first element as a Python number."""
        return self.numpy().reshape(-1)[0].item()

    def slice(self, *specs) -> "ndarray":
        """Per dim: slice(start, stop, step) or an int (drops the dim)."""
        d, s, o = [], [], self.offs
        for k in range(self.ndims):
            sp = specs[k] if k < len(specs) else slice(None)
            if isinstance(sp, (int, np.integer)):
                i = int(sp) % self.dims[k]
                o += i * self.incs[k]
                continue
            start, stop, step = sp.indices(self.dims[k])
            n = len(range(start, stop, step))
            o += start * self.incs[k] if n else 0
            d.append(n)
            s.append(self.incs[k] * step)
        return self._view(d, s, o)

    # -- descriptor for the C ABI
    def _desc(self, use_dev: bool) -> A.Ndarray:
        x = A.Ndarray()
        x.datatype = self.datatype
        x.ndims = self.ndims
        x.state = A.BADVAL if self._badflag else 0
        if self._badvalue is not None:
            x.has_badvalue = 1
            x.badvalue = _anyval(self.datatype, self._badvalue)
        else:
            x.badvalue.type = -1
        x.offs = self.offs
        for i, (dd, ii) in enumerate(zip(self.dims, self.incs)):
            x.dims[i] = dd
            x.incs[i] = ii
        if use_dev:
            x.ddata = self.storage.ensure_dev()
        else:
            x.data = self.storage.ensure_host().ctypes.data
        return x

    # -- operators (overloads call the functions by name, as PP.pm:1450)
    def __add__(self, o):
        return NotImplemented if _deferred(o) else plus(self, o)

    def __radd__(self, o):
        return NotImplemented if _deferred(o) else plus(self, o, swap=1)

    def __mul__(self, o):
        return NotImplemented if _deferred(o) else mult(self, o)

    def __rmul__(self, o):
        return NotImplemented if _deferred(o) else mult(self, o, swap=1)

    def __matmul__(self, o):
        return matmult(self, o)

    def __sub__(self, o): return NotImplemented if _deferred(o) else minus(self, o)
    def __rsub__(self, o): return NotImplemented if _deferred(o) else minus(self, o, swap=1)
    def __truediv__(self, o): return NotImplemented if _deferred(o) else divide(self, o)
    def __rtruediv__(self, o): return NotImplemented if _deferred(o) else divide(self, o, swap=1)
    def __gt__(self, o): return NotImplemented if _deferred(o) else gt(self, o)
    def __lt__(self, o): return NotImplemented if _deferred(o) else lt(self, o)
    def __ge__(self, o): return NotImplemented if _deferred(o) else ge(self, o)
    def __le__(self, o): return NotImplemented if _deferred(o) else le(self, o)
    def __lshift__(self, o): return NotImplemented if _deferred(o) else shiftleft(self, o)
    def __rshift__(self, o): return NotImplemented if _deferred(o) else shiftright(self, o)
    def __or__(self, o): return NotImplemented if _deferred(o) else or2(self, o)
    def __and__(self, o): return NotImplemented if _deferred(o) else and2(self, o)
    def __xor__(self, o): return NotImplemented if _deferred(o) else xor(self, o)
    def __rlshift__(self, o): return NotImplemented if _deferred(o) else shiftleft(self, o, swap=1)
    def __rrshift__(self, o): return NotImplemented if _deferred(o) else shiftright(self, o, swap=1)
    def __ror__(self, o): return NotImplemented if _deferred(o) else or2(self, o, swap=1)
    def __rand__(self, o): return NotImplemented if _deferred(o) else and2(self, o, swap=1)
    def __rxor__(self, o): return NotImplemented if _deferred(o) else xor(self, o, swap=1)

    # -- methods
    def sumover(self, out=None): return sumover(self, out)
    def dsumover(self, out=None): return dsumover(self, out)
    def prodover(self, out=None): return prodover(self, out)
    def dprodover(self, out=None): return dprodover(self, out)
    def cumusumover(self, out=None): return cumusumover(self, out)
    def dcumusumover(self, out=None): return dcumusumover(self, out)
    def average(self, out=None): return average(self, out)
    def daverage(self, out=None): return daverage(self, out)
    def minimum(self, out=None): return minimum(self, out)
    def maximum(self, out=None): return maximum(self, out)
    def minimum_ind(self, out=None): return minimum_ind(self, out)
    def maximum_ind(self, out=None): return maximum_ind(self, out)
    def inner(self, o, out=None): return inner(self, o, out)
    def minmaximum(self): return minmaximum(self)
    def qsort(self, out=None): return qsort(self, out)
    def qsorti(self, out=None): return qsorti(self, out)
    def medover(self, out=None): return medover(self, out)
    def oddmedover(self, out=None): return oddmedover(self, out)
    def modeover(self, out=None): return modeover(self, out)
    def qsortvec(self, out=None): return qsortvec(self, out)
    def qsortveci(self, out=None): return qsortveci(self, out)
    def pctover(self, p, out=None): return pctover(self, p, out)
    def oddpctover(self, p, out=None): return oddpctover(self, p, out)
    def median(self): return self.flat().medover()
    def oddmedian(self): return self.flat().oddmedover()
    def mode(self): return self.flat().modeover()
    def pct(self, p): return pctover(self.flat(), p)
    def oddpct(self, p): return oddpctover(self.flat(), p)

    # whole-array reductions (lib/PDL/Ufunc.pd:615-663): flat, then the
    # reduction over dim 0
    def sum(self): return self.flat().sumover()
    def avg(self): return self.flat().average()
    def prod(self): return self.flat().prodover()
    def dsum(self): return self.flat().dsumover()
    def davg(self): return self.flat().daverage()
    def dprod(self): return self.flat().dprodover()
    def zcheck(self): return zcover(self.flat())
    def and_(self): return andover(self.flat())
    def band(self): return bandover(self.flat())
    def or_(self): return orover(self.flat())
    def bor(self): return borover(self.flat())
    def xorall(self): return xorover(self.flat())
    def bxor(self): return bxorover(self.flat())
    def min(self): return self.flat().minimum()
    def max(self): return self.flat().maximum()
    any = or_
    all = and_
    def matmult(self, o, out=None): return matmult(self, o, out)


def _anyval(t: int, v) -> A.Anyval:
    a = A.Anyval()
    a.type = t
    if t in (A.F, A.D):
        setattr(a.value, "F" if t == A.F else "D", float(v))
    else:
        member = {A.SB: "A", A.B: "B", A.S: "S", A.US: "U", A.L: "L", A.UL: "K",
                  A.IND: "N", A.ULL: "P", A.LL: "Q"}[t]
        setattr(a.value, member, int(v))
    return a


def default_badvalue(t: int):
    a = A.Anyval()
    check(lib().pdlgb300_get_default_badvalue(int(t), C.byref(a)))
    m = {A.SB: "A", A.B: "B", A.S: "S", A.US: "U", A.L: "L", A.UL: "K", A.IND: "N",
         A.ULL: "P", A.LL: "Q", A.F: "F", A.D: "D"}[int(t)]
    return getattr(a.value, m)


def set_default_badvalue(t, v) -> None:
    t = type_code(t)
    check(lib().pdlgb300_set_default_badvalue(t, _anyval(t, v)))


# -------------------------------------------------------------- constructors

def _c_order(a: np.ndarray) -> np.ndarray:
    # (np.ascontiguousarray would turn a 0-dim array into 1-dim)
    return a if a.flags.c_contiguous else a.copy(order="C")


def pdl(x, type=None) -> ndarray:
    """From nested lists / numpy (numpy shape (r, c) -> dims (c, r))."""
    if isinstance(x, ndarray):
        return x if type is None or type_code(type) == x.datatype else convert(x, type)
    if type is not None:
        arr = _c_order(np.asarray(x, dtype=NP_DTYPES[type_code(type)]))
    else:
        arr = np.asarray(x)
        if arr.dtype == np.bool_ or arr.dtype.kind in "iu" and arr.dtype not in _NP_TO_TYPE:
            arr = arr.astype(np.int64)
        if arr.dtype.kind == "f" and arr.dtype != np.float32:
            arr = arr.astype(np.float64)
        if arr.dtype.kind in "iu" and arr.dtype == np.int64 and type is None and not isinstance(x, np.ndarray):
            arr = arr.astype(np.float64)  # PDL's pdl(...) of Perl numbers is double
        arr = _c_order(arr)
    # a named type wins over the numpy dtype (indx and longlong share int64)
    t = type_code(type) if type is not None else _NP_TO_TYPE[arr.dtype]
    flat = arr.reshape(-1).view(np.uint8) if arr.size else np.zeros(1, np.uint8)
    st = Storage(arr.nbytes, host=flat)
    return ndarray(st, t, arr.shape[::-1])


def from_numpy(arr: np.ndarray, type=None) -> ndarray:
    return pdl(np.asarray(arr) if type is None else np.asarray(arr, NP_DTYPES[type_code(type)]), type)


def zeroes(type, *dims) -> ndarray:
    t = type_code(type)
    return from_numpy(np.zeros(tuple(dims)[::-1], dtype=NP_DTYPES[t]), t)


def ones(type, *dims) -> ndarray:
    t = type_code(type)
    return from_numpy(np.ones(tuple(dims)[::-1], dtype=NP_DTYPES[t]), t)


def sequence(type, *dims) -> ndarray:
    t = type_code(type)
    n = int(np.prod(dims)) if dims else 1
    return from_numpy(np.arange(n).astype(NP_DTYPES[t]).reshape(tuple(dims)[::-1]))


def empty(type="double") -> ndarray:
    return zeroes(type, 0)


class _Null:
    """PDL->null: an output shaped by the op."""


def null():
    return _Null()


def device_empty(type, *dims) -> ndarray:
    """An uninitialised device-resident ndarray."""
    t = type_code(type)
    n = int(np.prod(dims, dtype=np.int64)) if dims else 1
    nbytes = n * np.dtype(NP_DTYPES[t]).itemsize
    p = C.c_void_p()
    check(lib().pdlgb300_device_alloc(max(nbytes, 16), C.byref(p)))
    st = Storage(nbytes, host=None, dev=p.value)
    st.fresh = "dev"
    return ndarray(st, t, dims)


# ---------------------------------------------------------------------- ops

def _scalar_to_pdl(v, like: Optional[ndarray]) -> ndarray:
    if isinstance(v, ndarray):
        return v
    if isinstance(v, (int, np.integer)) and like is not None and like.datatype < A.F:
        return pdl(np.array(v, dtype=like.np_dtype))
    if isinstance(v, (int, float, np.integer, np.floating)):
        return pdl(np.array(float(v)))
    return pdl(v)


def _run(vtname: str, inputs, outputs, other=None):
    """Shape, allocate and run one op (pdl_run_<op>: redodims, allocdata,
    readdata).  outputs: list of ndarray or None (null)."""
    L = lib()
    vt = L.pdlgb300_get_vtable(vtname.encode())
    if not vt:
        raise PDLError(A.EUSERERROR, f"unknown op {vtname}")
    for k, o in enumerate(outputs):
        # pdl__transtype_select (lib/PDL/Core/pdlapi.c:1191-1194)
        if o is not None and o.is_readonly():
            j = len(inputs) + k
            raise PDLError(A.EUSERERROR, f"{L.pdlgb300_op_package(vtname.encode()).decode()}{vtname} "
                                         f"error: output parameter {vt.contents.par_names[j].decode()} "
                                         "is read-only")
    use_dev = any(x.on_device for x in inputs) or any(
        o is not None and o.on_device for o in outputs)
    descs = [x._desc(use_dev) for x in inputs]
    odescs = []
    for o in outputs:
        if o is None:
            d = A.Ndarray()
            check(L.pdlgb300_ndarray_null(C.byref(d)))
            odescs.append(d)
        else:
            odescs.append(o._desc(use_dev))
    alld = descs + odescs
    arr = (A.P * len(alld))(*[C.pointer(d) for d in alld])
    oth = (C.c_int64 * 1)(int(other)) if other is not None else None
    # shape null outputs (host-only planning), then allocate them
    probe = [A.Ndarray.from_buffer_copy(d) for d in alld]
    parr = (A.P * len(probe))(*[C.pointer(d) for d in probe])
    check(L.pdlgb300_redodims(vt, parr, oth))
    results = []
    for k, o in enumerate(outputs):
        j = len(inputs) + k
        if o is None:
            pd = probe[j]
            dims = tuple(pd.dims[i] for i in range(pd.ndims))
            t = pd.datatype
            n = int(np.prod(dims, dtype=np.int64)) if dims else 1
            nbytes = n * np.dtype(NP_DTYPES[t]).itemsize
            if use_dev:
                p = C.c_void_p()
                check(L.pdlgb300_device_alloc(max(nbytes, 16), C.byref(p)))
                st = Storage(nbytes, host=None, dev=p.value)
                st.fresh = "dev"
            else:
                st = Storage(nbytes, host=np.zeros(max(nbytes, 1), np.uint8))
            o = ndarray(st, t, dims)
            odescs[k] = o._desc(use_dev)
            arr[j] = C.pointer(odescs[k])
        results.append(o)
    check(L.pdlgb300_run(vt, arr, oth))
    for k, o in enumerate(results):
        o._badflag = bool(odescs[k].state & A.BADVAL)
        o.storage.fresh = "dev" if use_dev else "host"
    return results


def _red(name):
    def f(a, out=None):
        a = _scalar_to_pdl(a, None)
        o = None if out is None or isinstance(out, _Null) else out
        return _run(name, [a], [o])[0]
    f.__name__ = name
    return f


sumover = _red("sumover")
dsumover = _red("dsumover")
prodover = _red("prodover")
dprodover = _red("dprodover")
cumusumover = _red("cumusumover")
dcumusumover = _red("dcumusumover")
average = _red("average")
daverage = _red("daverage")
minimum = _red("minimum")
maximum = _red("maximum")
andover = _red("andover")
orover = _red("orover")
xorover = _red("xorover")
zcover = _red("zcover")
bandover = _red("bandover")
borover = _red("borover")
bxorover = _red("bxorover")
firstnonzeroover = _red("firstnonzeroover")
cumuprodover = _red("cumuprodover")


def minmaximum(a, cmin=None, cmax=None, cmin_ind=None, cmax_ind=None):
    """(cmin, cmax, cmin_ind, cmax_ind) over dim 0 (lib/PDL/Ufunc.pd:563-613;
    alias minmaxover)."""
    a = _scalar_to_pdl(a, None)
    outs = [None if o is None or isinstance(o, _Null) else o for o in (cmin, cmax, cmin_ind, cmax_ind)]
    return tuple(_run("minmaximum", [a], outs))


minmaxover = minmaximum
qsort = _red("qsort")
qsorti = _red("qsorti")
medover = _red("medover")
oddmedover = _red("oddmedover")
modeover = _red("modeover")
qsortvec = _red("qsortvec")
qsortveci = _red("qsortveci")


def pctover(a, p, out=None) -> "ndarray":
    """The p-th percentile over dim 0, interpolated (lib/PDL/Ufunc.pd:975-989)."""
    a = _scalar_to_pdl(a, None)
    p = _scalar_to_pdl(p, a)
    o = None if out is None or isinstance(out, _Null) else out
    return _run("pctover", [a, p], [o])[0]


def oddpctover(a, p, out=None) -> "ndarray":
    """The p-th percentile over dim 0, the nearest data value (Ufunc.pd:991-1007)."""
    a = _scalar_to_pdl(a, None)
    p = _scalar_to_pdl(p, a)
    o = None if out is None or isinstance(out, _Null) else out
    return _run("oddpctover", [a, p], [o])[0]
dcumuprodover = _red("dcumuprodover")
minimum_ind = _red("minimum_ind")
maximum_ind = _red("maximum_ind")
avgover, minover, maxover = average, minimum, maximum


def _biop(name):
    def f(a, b, out=None, swap=0):
        if not isinstance(a, ndarray):
            a = _scalar_to_pdl(a, b if isinstance(b, ndarray) else None)
        b = _scalar_to_pdl(b, a)
        o = None if out is None or isinstance(out, _Null) else out
        return _run(name, [a, b], [o], other=int(swap))[0]
    f.__name__ = name
    return f


plus = _biop("plus")
mult = _biop("mult")
minus = _biop("minus")
divide = _biop("divide")
gt = _biop("gt")
lt = _biop("lt")
le = _biop("le")
ge = _biop("ge")
eq = _biop("eq")
ne = _biop("ne")
shiftleft = _biop("shiftleft")
shiftright = _biop("shiftright")
or2 = _biop("or2")
and2 = _biop("and2")
xor = _biop("xor")
xor2 = xor  # the reference's alias (lib/PDL/Ops.pd:309-313)


def inner(a, b, out=None) -> ndarray:
    a, b = _scalar_to_pdl(a, None), _scalar_to_pdl(b, None)
    o = None if out is None or isinstance(out, _Null) else out
    return _run("inner", [a, b], [o])[0]


def matmult(x, y, out=None) -> ndarray:
    """PDL::matmult's wrapper (lib/PDL/Primitive.pd:196-210) around
    _matmult_int: pad to 2-d with trailing dummy dims, a 1x1 operand is a
    scalar product, and dim(0) of x must equal dim(1) of y."""
    x = _scalar_to_pdl(x, None)
    y = _scalar_to_pdl(y, x)
    while x.ndims < 2:
        x = x.dummy(-1)
    while y.ndims < 2:
        y = y.dummy(-1)
    if (x.dim(0) == 1 and x.dim(1) == 1) or (y.dim(0) == 1 and y.dim(1) == 1):
        r = mult(x, y)
        if out is not None and not isinstance(out, _Null):
            return assign(out, r)
        return r
    if y.dim(1) != x.dim(0):
        raise PDLError(A.EUSERERROR,
                       "Dim mismatch in matmult of [%dx%d] x [%dx%d]: %d != %d"
                       % (x.dim(0), x.dim(1), y.dim(0), y.dim(1), x.dim(0), y.dim(1)))
    o = None if out is None or isinstance(out, _Null) else out
    return _run("matmult", [x, y], [o])[0]


def sumover_mult_plus(a, b, d, out=None) -> ndarray:
    """sumover(a*b + d) in one fused pass (same values as the three ops)."""
    o = None if out is None or isinstance(out, _Null) else out
    return _run("sumover_mult_plus", [a, b, d], [o])[0]


def convert(x: ndarray, type) -> ndarray:
    t = type_code(type)
    use_dev = x.on_device
    n = x.nelem
    nbytes = n * np.dtype(NP_DTYPES[t]).itemsize
    if use_dev:
        out = device_empty(t, *x.dims)
    else:
        out = ndarray(Storage(nbytes, host=np.zeros(max(nbytes, 1), np.uint8)), t, x.dims)
    sd, dd = x._desc(use_dev), out._desc(use_dev)
    check(lib().pdlgb300_convert(C.byref(sd), C.byref(dd)))
    out._badflag = bool(dd.state & A.BADVAL)
    out.storage.fresh = "dev" if use_dev else "host"
    return out


def assign(dst: ndarray, src: ndarray) -> ndarray:
    """dst .= src (through the library: plus(src, 0))."""
    z = zeroes(src.datatype, *([1] * 0))
    return plus(src, z, dst)


# -------------------------------------------------------------- backward

def _bw(fn, *args):
    L = lib()
    ds = []
    for a in args:
        ds.append(None if a is None else a[1])
    check(getattr(L, fn)(*[None if d is None else C.byref(d) for d in ds]))


def _grad_like(x: ndarray, use_dev: bool) -> ndarray:
    if use_dev:
        return device_empty(x.datatype, *x.dims)
    n = x.nelem * np.dtype(x.np_dtype).itemsize
    return ndarray(Storage(n, host=np.zeros(max(n, 1), np.uint8)), x.datatype, x.dims)


def _finish(g: ndarray, use_dev: bool):
    g.storage.fresh = "dev" if use_dev else "host"
    return g


def _grads(like, dev, out):
    """Gradient buffers shaped like `like` (new ones, or the caller's `out`,
    which must have those dims and type and be on the same side)."""
    if out is None:
        return [_grad_like(x, dev) for x in like]
    out = list(out) if isinstance(out, (tuple, list)) else [out]
    for o, x in zip(out, like):
        if o.dims != x.dims or o.datatype != x.datatype:
            raise PDLError(A.EUSERERROR, f"backward: out has dims {o.dims} type {o.type}, "
                                         f"needs {x.dims} {x.type}")
        if dev and not o.on_device:
            o.to_device()
    return out


def sumover_bwd(gb: ndarray, a: ndarray, out=None) -> ndarray:
    dev = gb.on_device or a.on_device
    (ga,) = _grads([a], dev, out)
    d1, d2 = gb._desc(dev), ga._desc(dev)
    check(lib().pdlgb300_sumover_bwd(C.byref(d1), C.byref(d2)))
    return _finish(ga, dev)


def average_bwd(gb: ndarray, a: ndarray, out=None) -> ndarray:
    dev = gb.on_device or a.on_device
    (ga,) = _grads([a], dev, out)
    d1, d2 = gb._desc(dev), ga._desc(dev)
    check(lib().pdlgb300_average_bwd(C.byref(d1), C.byref(d2)))
    return _finish(ga, dev)


def plus_bwd(gc: ndarray, a: ndarray, b: ndarray, out=None):
    dev = gc.on_device or a.on_device or b.on_device
    ga, gb = _grads([a, b], dev, out)
    d0, d1, d2 = gc._desc(dev), ga._desc(dev), gb._desc(dev)
    check(lib().pdlgb300_plus_bwd(C.byref(d0), C.byref(d1), C.byref(d2)))
    return _finish(ga, dev), _finish(gb, dev)


def mult_bwd(gc: ndarray, a: ndarray, b: ndarray, out=None):
    dev = gc.on_device or a.on_device or b.on_device
    ga, gb = _grads([a, b], dev, out)
    ds = [gc._desc(dev), a._desc(dev), b._desc(dev), ga._desc(dev), gb._desc(dev)]
    check(lib().pdlgb300_mult_bwd(*[C.byref(d) for d in ds]))
    return _finish(ga, dev), _finish(gb, dev)


def matmult_bwd(gc: ndarray, a: ndarray, b: ndarray, out=None):
    dev = gc.on_device or a.on_device or b.on_device
    ga, gb = _grads([a, b], dev, out)
    ds = [gc._desc(dev), a._desc(dev), b._desc(dev), ga._desc(dev), gb._desc(dev)]
    check(lib().pdlgb300_matmult_bwd(*[C.byref(d) for d in ds]))
    return _finish(ga, dev), _finish(gb, dev)


# ------------------------------------------------------------ runtime knobs

def set_matmult_mode(mode: int) -> None:
    check(lib().pdlgb300_set_option(A.OPT_MATMULT_MODE, int(mode)))


def set_compensated(on: bool) -> None:
    check(lib().pdlgb300_set_option(A.OPT_F32_COMPENSATED, 1 if on else 0))


def set_debugging(on: bool) -> None:
    check(lib().pdlgb300_set_option(A.OPT_DEBUG, 1 if on else 0))


def set_timing(on: bool) -> None:
    check(lib().pdlgb300_set_timing(1 if on else 0))


def set_stream(ptr: int) -> None:
    check(lib().pdlgb300_set_stream(ptr or None))


def sync() -> None:
    check(lib().pdlgb300_sync())


def last_launch_info() -> dict:
    li = A.LaunchInfo()
    check(lib().pdlgb300_last_launch(C.byref(li)))
    return li.as_dict()


def device_count() -> int:
    n = C.c_int32()
    check(lib().pdlgb300_device_count(C.byref(n)))
    return n.value
