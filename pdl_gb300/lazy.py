"""Deferred expressions: PDL::Ops binary ops recorded instead of run, so
that a reduction over the expression runs as one fused pass and the
intermediates (a*b, a*b+a, ...) are never written to memory.

    e = lazy(a) * b + a          # nothing computed yet
    s = e.sumover()              # one pass over a and b
    m = e.materialize()          # the ops one by one, as the eager API does

Each recorded op is shaped and typed at once by the library's own redodims
for that op (lib/PDL/Ops.pd:104-153, 288-307: the same broadcasting, type
selection and error messages as the eager op), so an expression that the
reference would refuse is refused when it is written.  The fused pass
(pdlgb300_run_expr_reduce) computes every element exactly as the eager ops
would, op by op in the common type with each op's bad-value rule; an
expression it does not take (mixed types, more than four distinct leaves or
eight ops, a reduction it does not fuse) runs its ops eagerly on the GPU
and then the reduction.
"""
from __future__ import annotations

import ctypes as C
import importlib
from typing import List, Optional, Union

import numpy as np

from . import _abi as A
from ._abi import check, lib
# the module (the package's own name `ndarray` is the class)
N = importlib.import_module(".ndarray", __package__)

BIOPS = ("plus", "mult", "minus", "divide", "gt", "lt", "le", "ge", "eq", "ne",
         "shiftleft", "shiftright", "or2", "and2", "xor")
FUSED_TYPES = {A.L, A.LL, A.F, A.D}
MAX_LEAVES, MAX_NODES = 4, 8


class _ExprNode(C.Structure):
    _fields_ = [("op", C.POINTER(A.Vtable)), ("a", C.c_int32), ("b", C.c_int32)]


def _shape_desc(dims, datatype: int, badflag: bool) -> A.Ndarray:
    d = A.Ndarray()
    d.datatype = datatype
    d.ndims = len(dims)
    d.state = A.BADVAL if badflag else 0
    d.badvalue.type = -1
    s = 1
    for i, x in enumerate(dims):
        d.dims[i] = x
        d.incs[i] = s
        s *= x
    return d


class Lazy:
    """One recorded binary op over ndarrays and other recorded ops."""

    __slots__ = ("op", "a", "b", "dims", "datatype", "_badflag")
    _deferred = True

    def __init__(self, op: str, a, b):
        if op not in BIOPS:
            raise A.PDLError(A.EUSERERROR, f"{op} is not a binary op of PDL::Ops")
        a, b = _unwrap(a), _unwrap(b)
        like = a if isinstance(a, (Lazy, N.ndarray)) else b if isinstance(b, (Lazy, N.ndarray)) else None
        a = a if isinstance(a, (Lazy, N.ndarray)) else N._scalar_to_pdl(a, _like(like))
        b = b if isinstance(b, (Lazy, N.ndarray)) else N._scalar_to_pdl(b, _like(like))
        self.op, self.a, self.b = op, a, b
        L = lib()
        vt = L.pdlgb300_get_vtable(op.encode())
        descs = [_shape_desc(x.dims, x.datatype, x.badflag()) for x in (a, b)]
        out = A.Ndarray()
        check(L.pdlgb300_ndarray_null(C.byref(out)))
        arr = (A.P * 3)(*[C.pointer(d) for d in descs + [out]])
        check(L.pdlgb300_redodims(vt, arr, None))
        self.dims = tuple(out.dims[i] for i in range(out.ndims))
        self.datatype = out.datatype
        self._badflag = a.badflag() or b.badflag()

    # -- the ndarray-like surface
    def badflag(self) -> bool:
        return self._badflag

    @property
    def ndims(self) -> int:
        return len(self.dims)

    @property
    def type(self) -> str:
        return N.TYPE_NAMES[self.datatype]

    def __repr__(self):
        return f"Lazy({self.op}, {self.type}, dims={self.dims})"

    # -- building
    def __add__(self, o): return Lazy("plus", self, o)
    def __radd__(self, o): return Lazy("plus", o, self)
    def __mul__(self, o): return Lazy("mult", self, o)
    def __rmul__(self, o): return Lazy("mult", o, self)
    def __sub__(self, o): return Lazy("minus", self, o)
    def __rsub__(self, o): return Lazy("minus", o, self)
    def __truediv__(self, o): return Lazy("divide", self, o)
    def __rtruediv__(self, o): return Lazy("divide", o, self)
    def __gt__(self, o): return Lazy("gt", self, o)
    def __lt__(self, o): return Lazy("lt", self, o)
    def __ge__(self, o): return Lazy("ge", self, o)
    def __le__(self, o): return Lazy("le", self, o)
    def __lshift__(self, o): return Lazy("shiftleft", self, o)
    def __rshift__(self, o): return Lazy("shiftright", self, o)
    def __or__(self, o): return Lazy("or2", self, o)
    def __and__(self, o): return Lazy("and2", self, o)
    def __xor__(self, o): return Lazy("xor", self, o)
    def __rlshift__(self, o): return Lazy("shiftleft", o, self)
    def __rrshift__(self, o): return Lazy("shiftright", o, self)
    def __ror__(self, o): return Lazy("or2", o, self)
    def __rand__(self, o): return Lazy("and2", o, self)
    def __rxor__(self, o): return Lazy("xor", o, self)

    # -- evaluation
    def materialize(self) -> N.ndarray:
        """The ops one by one through the eager API."""
        a = self.a.materialize() if isinstance(self.a, Lazy) else self.a
        b = self.b.materialize() if isinstance(self.b, Lazy) else self.b
        return getattr(N, self.op)(a, b)

    def numpy(self) -> np.ndarray:
        return self.materialize().numpy()

    def _program(self):
        """(leaves, nodes) in evaluation order, or None when not fusable."""
        leaves: List[N.ndarray] = []
        nodes = []

        seen = {}

        def ref(x) -> Optional[int]:
            if isinstance(x, Lazy):
                ia, ib = ref(x.a), ref(x.b)
                if ia is None or ib is None:
                    return None
                key = (x.op, ia, ib)  # a repeated subexpression is computed once
                if key not in seen:
                    nodes.append(key)
                    seen[key] = -len(nodes)  # node k is -(k+1) until the leaves are counted
                return seen[key]
            for i, l in enumerate(leaves):
                if l is x:
                    return i
            leaves.append(x)
            return len(leaves) - 1

        root = ref(self)
        if root is None or len(nodes) > MAX_NODES:
            return None
        T = self.datatype
        if T not in FUSED_TYPES or len(leaves) > MAX_LEAVES:
            return None
        if not _all_node_types(self, T):
            return None
        conv = []
        for l in leaves:
            if l.datatype == T:
                conv.append(l)
            elif l.ndims == 0:
                conv.append(N.convert(l, T))  # the op's own converted copy of a 0-dim
            else:
                return None
        nl = len(leaves)
        fixed = [(op, ia if ia >= 0 else nl + (-ia - 1), ib if ib >= 0 else nl + (-ib - 1))
                 for op, ia, ib in nodes]
        return conv, fixed

    def _reduce(self, name: str, out=None) -> N.ndarray:
        o = None if out is None or isinstance(out, N._Null) else out
        prog = self._program()
        if prog is not None and name == "sumover" and _is_mult_plus(prog):
            # sumover(a*b + d): the tiled kernel of sumover_mult_plus
            leaves, nodes = prog
            (_, i, j), (_, _, k) = nodes
            return N.sumover_mult_plus(leaves[i], leaves[j], leaves[k], o)
        if prog is not None and name in FUSED_REDUCTIONS:
            leaves, nodes = prog
            r = _run_fused(name, leaves, nodes, o)
            if r is not None:
                return r
        return getattr(N, name)(self.materialize(), o) if o is not None else getattr(N, name)(self.materialize())


def _is_mult_plus(prog) -> bool:
    """mult of two leaves, then plus of that and a leaf: sumover_mult_plus."""
    leaves, nodes = prog
    nl = len(leaves)
    return (len(nodes) == 2 and nodes[0][0] == "mult" and nodes[0][1] < nl and nodes[0][2] < nl
            and nodes[1][0] == "plus" and nodes[1][1] == nl and nodes[1][2] < nl)


def _like(x):
    if x is None:
        return None
    if isinstance(x, N.ndarray):
        return x

    class _T:
        pass

    t = _T()
    t.datatype = x.datatype
    t.np_dtype = N.NP_DTYPES[x.datatype]
    return t


def _all_node_types(e, T) -> bool:
    if not isinstance(e, Lazy):
        return True
    return e.datatype == T and _all_node_types(e.a, T) and _all_node_types(e.b, T)


FUSED_REDUCTIONS = {"sumover", "dsumover", "average", "daverage", "prodover", "minimum",
                    "maximum", "minimum_ind", "maximum_ind", "andover", "orover", "xorover",
                    "zcover", "bandover", "borover", "bxorover"}
_INT_ONLY = {"prodover", "bandover", "borover", "bxorover"}


def _run_fused(name, leaves, nodes, out) -> Optional[N.ndarray]:
    T = leaves[0].datatype
    if name in _INT_ONLY and T >= A.F:
        return None
    L = lib()
    rvt = L.pdlgb300_get_vtable(name.encode())
    use_dev = any(x.on_device for x in leaves) or (out is not None and out.on_device)
    descs = [x._desc(use_dev) for x in leaves]
    larr = (A.P * len(descs))(*[C.pointer(d) for d in descs])
    narr = (_ExprNode * len(nodes))()
    for k, (op, ia, ib) in enumerate(nodes):
        narr[k].op = L.pdlgb300_get_vtable(op.encode())
        narr[k].a, narr[k].b = ia, ib
    if out is None:
        # shape the output with the reduction's redodims on the expression's shape
        root = _shape_desc(_expr_dims(leaves), T, any(x.badflag() for x in leaves))
        probe = A.Ndarray()
        check(L.pdlgb300_ndarray_null(C.byref(probe)))
        parr = (A.P * 2)(C.pointer(root), C.pointer(probe))
        check(L.pdlgb300_redodims(rvt, parr, None))
        dims = tuple(probe.dims[i] for i in range(probe.ndims))
        t = probe.datatype
        n = int(np.prod(dims, dtype=np.int64)) if dims else 1
        nbytes = n * np.dtype(N.NP_DTYPES[t]).itemsize
        if use_dev:
            p = C.c_void_p()
            check(L.pdlgb300_device_alloc(max(nbytes, 16), C.byref(p)))
            st = N.Storage(nbytes, host=None, dev=p.value)
            st.fresh = "dev"
        else:
            st = N.Storage(nbytes, host=np.zeros(max(nbytes, 1), np.uint8))
        out = N.ndarray(st, t, dims)
    od = out._desc(use_dev)
    check(L.pdlgb300_run_expr_reduce(rvt, len(leaves), larr, len(nodes), narr, C.byref(od)))
    out._badflag = bool(od.state & A.BADVAL)
    out.storage.fresh = "dev" if use_dev else "host"
    return out


def _expr_dims(leaves):
    nd = max(x.ndims for x in leaves)
    dims = []
    for k in range(nd):
        d = 1
        for x in leaves:
            v = x.dims[k] if k < x.ndims else 1
            if v != 1:
                d = v
        dims.append(d)
    return tuple(dims)


def _add_reductions():
    for name in ("sumover", "dsumover", "prodover", "dprodover", "average", "daverage",
                 "minimum", "maximum", "minimum_ind", "maximum_ind", "andover", "orover",
                 "xorover", "zcover", "bandover", "borover", "bxorover", "firstnonzeroover",
                 "cumusumover", "dcumusumover", "cumuprodover", "dcumuprodover"):
        def f(self, out=None, _n=name):
            return self._reduce(_n, out)
        f.__name__ = name
        setattr(Lazy, name, f)


_add_reductions()


def lazy(x: Union[N.ndarray, Lazy]) -> "LazyLeaf":
    """Start a deferred expression at ndarray x."""
    if isinstance(x, (Lazy, LazyLeaf)):
        return x
    return LazyLeaf(N._scalar_to_pdl(x, None))


class LazyLeaf:
    """An ndarray whose binary ops are recorded (lazy(a) * b -> Lazy)."""

    __slots__ = ("x",)
    _deferred = True

    def __init__(self, x: N.ndarray):
        self.x = x

    def __getattr__(self, name):
        # anything but a binary op (a reduction, dims, numpy()) is the ndarray's
        return getattr(self.x, name)

    def __add__(self, o): return Lazy("plus", self.x, _unwrap(o))
    def __radd__(self, o): return Lazy("plus", _unwrap(o), self.x)
    def __mul__(self, o): return Lazy("mult", self.x, _unwrap(o))
    def __rmul__(self, o): return Lazy("mult", _unwrap(o), self.x)
    def __sub__(self, o): return Lazy("minus", self.x, _unwrap(o))
    def __rsub__(self, o): return Lazy("minus", _unwrap(o), self.x)
    def __truediv__(self, o): return Lazy("divide", self.x, _unwrap(o))
    def __rtruediv__(self, o): return Lazy("divide", _unwrap(o), self.x)
    def __gt__(self, o): return Lazy("gt", self.x, _unwrap(o))
    def __lt__(self, o): return Lazy("lt", self.x, _unwrap(o))
    def __ge__(self, o): return Lazy("ge", self.x, _unwrap(o))
    def __le__(self, o): return Lazy("le", self.x, _unwrap(o))
    def __lshift__(self, o): return Lazy("shiftleft", self.x, _unwrap(o))
    def __rshift__(self, o): return Lazy("shiftright", self.x, _unwrap(o))
    def __or__(self, o): return Lazy("or2", self.x, _unwrap(o))
    def __and__(self, o): return Lazy("and2", self.x, _unwrap(o))
    def __xor__(self, o): return Lazy("xor", self.x, _unwrap(o))
    def __rlshift__(self, o): return Lazy("shiftleft", _unwrap(o), self.x)
    def __rrshift__(self, o): return Lazy("shiftright", _unwrap(o), self.x)
    def __ror__(self, o): return Lazy("or2", _unwrap(o), self.x)
    def __rand__(self, o): return Lazy("and2", _unwrap(o), self.x)
    def __rxor__(self, o): return Lazy("xor", _unwrap(o), self.x)


def _unwrap(o):
    return o.x if isinstance(o, LazyLeaf) else o


def binop(op: str, a, b, swap: int = 0) -> Lazy:
    """The deferred form of PDL::Ops op(a, b, swap)."""
    a, b = _unwrap(a), _unwrap(b)
    return Lazy(op, b, a) if swap else Lazy(op, a, b)
