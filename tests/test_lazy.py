"""Deferred expressions without a GPU: each recorded op is shaped and typed
by the library's redodims (the eager op's broadcasting, type selection and
error text), and the fused program lists each distinct leaf once."""
import numpy as np
import pytest

import pdl_gb300 as P


def test_shapes_types_and_program():
    a = P.pdl(np.arange(12.0).reshape(3, 4))     # dims (4, 3)
    b = P.pdl(np.ones(4))                         # dims (4,)
    e = P.lazy(a) * b + a
    assert isinstance(e, P.Lazy) and e.dims == (4, 3) and e.type == "double"
    leaves, nodes = e._program()
    assert len(leaves) == 2 and leaves[0] is a and leaves[1] is b
    assert nodes == [("mult", 0, 1), ("plus", 2, 0)]
    # the reversed operators put the scalar first, as swap does
    r = 1.0 - P.lazy(a)
    assert r.op == "minus" and r.b is a and r.a.ndims == 0


def test_bad_flag_and_int_scalars():
    x = P.pdl(np.arange(6, dtype=np.int32))
    x.badflag(1)
    e = P.lazy(x) + 3
    assert e.type == "long" and e.badflag()
    assert e._program()[0][1].type == "long"     # the int scalar takes x's type


def test_mismatch_is_the_eager_error():
    a = P.pdl(np.zeros((3, 4)))
    with pytest.raises(P.PDLError, match="Mismatched implicit broadcast dimension 0: size 4 vs. 5"):
        P.lazy(a) + P.pdl(np.zeros(5))


def test_not_fused_programs():
    a = P.pdl(np.zeros(4, np.uint8))
    assert (P.lazy(a) + a)._program() is None                 # byte: not a fused type
    xs = [P.pdl(np.zeros(4)) for _ in range(5)]
    e = P.lazy(xs[0]) + xs[1] + xs[2] + xs[3] + xs[4]
    assert e._program() is None                               # five leaves
    f = P.lazy(P.pdl(np.zeros(4, np.float32))) + P.pdl(np.zeros(4))
    assert f.type == "double" and f._program() is None        # a float leaf converted


def test_leaf_forwards_everything_but_ops():
    a = P.pdl(np.arange(6.0).reshape(2, 3))
    leaf = P.lazy(a)
    assert leaf.dims == (3, 2) and leaf.type == "double"
    assert np.array_equal(leaf.numpy(), a.numpy())
    assert isinstance(leaf + 1, P.Lazy)
    # a leaf on the right of a recorded op is its ndarray
    e = (P.lazy(a) * a) + P.lazy(a)
    assert e.b is a and e._program()[1] == [("mult", 0, 0), ("plus", 1, 0)]


def test_random_expressions_shape_and_type_like_the_eager_chain():
    """Random trees of binary ops over broadcastable leaves of mixed types:
    each recorded node has the dims and type the oracle's planner gives the
    eager op on its operands' shapes and types."""
    from oracle import oracle as O
    rng = np.random.default_rng(21)
    types = ["byte", "short", "long", "longlong", "float", "double"]
    ops = ["plus", "mult", "minus", "divide", "gt", "le", "eq"]
    bit = ["shiftleft", "or2", "and2", "xor"]

    def leaf():
        dims = [int(rng.choice([1, 3]))] + ([int(rng.choice([1, 4]))] if rng.random() < 0.6 else [])
        return P.zeroes(str(rng.choice(types)), *dims)

    def check(e):
        if not isinstance(e, P.Lazy):
            return e
        a, b = check(e.a), check(e.b)
        dims, t = O.redodims(e.op, [a, b])
        assert (e.dims, e.datatype) == (tuple(dims), t), (e, dims, t)
        return P.zeroes(t, *dims)

    for _ in range(200):
        e = P.lazy(leaf())
        for _ in range(int(rng.integers(1, 4))):
            op = str(rng.choice(ops + bit))
            other = leaf()
            e = P.Lazy(op, e, other) if rng.random() < 0.5 else P.Lazy(op, other, e)
        check(e)


def _expr_call(red, leaves, nodes, out=None):
    import ctypes as C
    from pdl_gb300 import _abi as A
    from pdl_gb300.lazy import _ExprNode
    L = A.lib()
    descs = [x._desc(False) for x in leaves]
    larr = (A.P * len(descs))(*[C.pointer(d) for d in descs])
    narr = (_ExprNode * len(nodes))()
    for k, (op, ia, ib) in enumerate(nodes):
        narr[k].op = L.pdlgb300_get_vtable(op.encode())
        narr[k].a, narr[k].b = ia, ib
    od = A.Ndarray()
    L.pdlgb300_ndarray_null(C.byref(od))
    e = L.pdlgb300_run_expr_reduce(L.pdlgb300_get_vtable(red.encode()), len(leaves), larr,
                                   len(nodes), narr, C.byref(od))
    return e.error, (e.message.decode() if e.message else "")


def test_expression_entry_point_validates_programs():
    """pdlgb300_run_expr_reduce refuses malformed programs before any
    device work (host-only checks, no GPU needed)."""
    a = P.pdl(np.zeros((2, 3)))
    b = P.pdl(np.zeros((2, 3), np.float32))
    code, msg = _expr_call("sumover", [a, b], [("plus", 0, 1)])
    assert code and "leaves of types double and float" in msg
    code, msg = _expr_call("sumover", [a], [("plus", 0, 1)])
    assert code and "refers to 1" in msg                     # operand beyond the leaves
    code, msg = _expr_call("sumover", [a, a], [("plus", 0, 0)])
    assert code and "leaf 1 does not reach the result" in msg
    code, msg = _expr_call("sumover", [a], [("sumover", 0, 0)])
    assert code and "not a binary op" in msg
    code, msg = _expr_call("cumusumover", [a], [("plus", 0, 0)])
    assert code and "not a reduction over dim 0" in msg     # a scan: the eager path
    code, msg = _expr_call("sumover", [a], [("shiftleft", 0, 0)])
    assert code and "integer type" in msg
    code, msg = _expr_call("bandover", [a], [("plus", 0, 0)])
    assert code and "not fused" in msg


@pytest.mark.parametrize("sym,op", [("<<", "shiftleft"), (">>", "shiftright"),
                                    ("|", "or2"), ("&", "and2"), ("^", "xor")])
def test_reversed_bit_and_shift_operators_record_the_swapped_op(sym, op):
    """An ndarray or a scalar on the left of a bit or shift operator whose
    right side is deferred records op(left, right), as PDL's overload does
    with swap set; dims and type equal the eager op's (the oracle's)."""
    from oracle import oracle as O
    from pdl_gb300.lazy import LazyLeaf
    x = P.pdl(np.arange(12, dtype=np.int32).reshape(3, 4))   # dims (4, 3)
    y = P.pdl(np.arange(4, dtype=np.int64))                   # dims (4,)
    three = P.pdl(np.int32(3))
    xx = O.run("mult", [x, x])[0]                             # eager x*x
    for left, right, eager_left, eager_right in [
            (y, P.lazy(x), y, x), (3, P.lazy(x), three, x), (y, P.lazy(x) * x, y, xx),
            (3, P.lazy(x) * x, three, xx)]:
        e = eval(f"l {sym} r", {"l": left, "r": right})
        assert isinstance(e, P.Lazy) and e.op == op
        assert e.b is (right.x if isinstance(right, LazyLeaf) else right)
        ref = O.run(op, [eager_left, eager_right])[0]
        assert e.dims == ref.dims and e.type == ref.type


@pytest.mark.parametrize("sym,op", [("<<", "shiftleft"), (">>", "shiftright"),
                                    ("|", "or2"), ("&", "and2"), ("^", "xor")])
def test_reversed_bit_and_shift_operators_on_ndarrays_are_registered(sym, op):
    """A scalar on the left of an ndarray's bit or shift operator is the
    swapped op (Ops.pd's overloads pass swap); the reversed methods exist."""
    rname = {"<<": "__rlshift__", ">>": "__rrshift__", "|": "__ror__", "&": "__rand__",
             "^": "__rxor__"}[sym]
    assert callable(getattr(P.ndarray, rname))
