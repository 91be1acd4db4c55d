"""Hand-written adjoint kernels (sumover, average, plus, mult, matmult):
against gradients written out by hand (numpy, and the oracle's C versions),
against FP64 central finite differences on the config-4 chain, and through
torch.autograd.gradcheck via the verification-only autograd mirror."""
import ctypes as C

import numpy as np
import pytest

import pdl_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("t", ["float", "double"])
def test_sumover_average_bwd(gpu, t):
    rng = np.random.default_rng(1)
    dt = np.float32 if t == "float" else np.float64
    a = rng.standard_normal((7, 5, 33)).astype(dt)     # PDL dims (33, 5, 7)
    gb = rng.standard_normal((7, 5)).astype(dt)        # sumover output dims (5, 7)
    ga = P.sumover_bwd(P.pdl(gb), P.pdl(a)).numpy()
    assert np.array_equal(ga, np.broadcast_to(gb[..., None], a.shape))
    gv = P.average_bwd(P.pdl(gb), P.pdl(a)).numpy()
    np.testing.assert_allclose(gv, np.broadcast_to(gb[..., None] / 33, a.shape), rtol=1e-6)
    # the oracle's hand-derived versions agree
    if t == "double":
        out = np.empty_like(a)
        O.lib().oracle_sumover_bwd(gb.ctypes.data, out.ctypes.data, 33, 35)
        assert np.array_equal(out, ga)


@pytest.mark.parametrize("shapes", [((4, 6), (4, 6)), ((4, 6), (1, 6)), ((6,), (4, 6)),
                                    ((3, 1, 5), (1, 4, 5)), ((), (2, 3))])
def test_plus_mult_bwd_unbroadcast(gpu, shapes):
    rng = np.random.default_rng(2)
    sa, sb = shapes
    a = rng.standard_normal(sa)
    b = rng.standard_normal(sb)
    gc = rng.standard_normal(np.broadcast_shapes(sa, sb))

    def unb(g, shape):
        while g.ndim > len(shape):
            g = g.sum(0)
        for i, s in enumerate(shape):
            if s == 1 and g.shape[i] != 1:
                g = g.sum(i, keepdims=True)
        return g

    ga, gb = P.plus_bwd(P.pdl(gc), P.pdl(a), P.pdl(b))
    np.testing.assert_allclose(ga.numpy(), unb(gc, sa), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(gb.numpy(), unb(gc, sb), rtol=1e-12, atol=1e-12)
    ga, gb = P.mult_bwd(P.pdl(gc), P.pdl(a), P.pdl(b))
    np.testing.assert_allclose(ga.numpy(), unb(gc * b, sa), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(gb.numpy(), unb(gc * a, sb), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("t", ["float", "double"])
@pytest.mark.parametrize("batch", [(None, None), (3, 3), (3, None), (None, 3)])
def test_matmult_bwd(gpu, t, batch):
    rng = np.random.default_rng(3)
    dt = np.float32 if t == "float" else np.float64
    H, T, W = 37, 29, 41
    ba, bb = batch
    a = rng.standard_normal(((ba,) if ba else ()) + (H, T)).astype(dt)
    b = rng.standard_normal(((bb,) if bb else ()) + (T, W)).astype(dt)
    c = np.matmul(a.astype(np.float64), b.astype(np.float64))
    gc = rng.standard_normal(c.shape).astype(dt)
    ga, gb = P.matmult_bwd(P.pdl(gc), P.pdl(a), P.pdl(b))
    g64 = gc.astype(np.float64)
    want_a = g64 @ np.swapaxes(b.astype(np.float64), -1, -2)
    want_b = np.swapaxes(a.astype(np.float64), -1, -2) @ g64
    if ba is None and want_a.ndim == 3:
        want_a = want_a.sum(0)
    if bb is None and want_b.ndim == 3:
        want_b = want_b.sum(0)
    tol = 1e-5 if t == "float" else 1e-12
    sa = np.abs(g64) @ np.abs(np.swapaxes(b, -1, -2)).astype(np.float64)
    sb = np.abs(np.swapaxes(a, -1, -2)).astype(np.float64) @ np.abs(g64)
    if ba is None and sa.ndim == 3:
        sa = sa.sum(0)
    if bb is None and sb.ndim == 3:
        sb = sb.sum(0)
    assert np.all(np.abs(ga.numpy() - want_a) <= tol * sa + 1e-30)
    assert np.all(np.abs(gb.numpy() - want_b) <= tol * sb + 1e-30)
    if ba is None and bb is None and t == "double":
        # the oracle's hand-derived matmult gradient (C, double)
        oa, ob = np.empty_like(a), np.empty_like(b)
        O.lib().oracle_matmult_bwd(gc.ctypes.data, a.ctypes.data, b.ctypes.data,
                                   oa.ctypes.data, ob.ctypes.data, T, H, W, 1, 1, 1)
        np.testing.assert_allclose(ga.numpy(), oa, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(gb.numpy(), ob, rtol=1e-12, atol=1e-12)


def _c4_inputs():
    rng = np.random.default_rng(6)
    X = (0.1 * rng.standard_normal((8192, 512))).astype(np.float32)   # PDL X(t=512, h=8192)
    Wm = (0.1 * rng.standard_normal((512, 256))).astype(np.float32)   # PDL W(w=256, t=512)
    bias = (0.1 * rng.standard_normal(256)).astype(np.float32)        # PDL bias(w=256)
    return X, Wm, bias


def _c4_loss64(X, Wm, bias):
    Z = X.astype(np.float64) @ Wm.astype(np.float64) + bias.astype(np.float64)
    return float((Z * Z).sum() / 8192.0)


def _c4_backward_gpu(X, Wm, bias):
    """L = sumover(sumover(Z*Z))/8192, Z = matmult(X,W) + bias, through the
    library's forward ops and backward calls (nothing stored but the inputs:
    intermediates are recomputed)."""
    x, w, b = P.pdl(X).to_device(), P.pdl(Wm).to_device(), P.pdl(bias).to_device()
    Y = P.matmult(x, w)                       # (w=256, h=8192)
    Z = P.plus(Y, b)
    S = P.mult(Z, Z)
    s1 = P.sumover(S)                         # (h=8192)
    gL = P.pdl(np.array(1.0 / 8192, np.float32)).to_device()
    g_s1 = P.sumover_bwd(gL, s1)              # dL/ds1 = 1/8192
    g_S = P.sumover_bwd(g_s1, S)
    gz1, gz2 = P.mult_bwd(g_S, Z, Z)
    g_Z = P.plus(gz1, gz2)
    g_Y, g_b = P.plus_bwd(g_Z, Y, b)
    g_X, g_W = P.matmult_bwd(g_Y, x, w)
    return g_X.numpy(), g_W.numpy(), g_b.numpy()


def test_c4_chain_finite_differences(gpu):
    X, Wm, bias = _c4_inputs()
    gX, gW, gb = _c4_backward_gpu(X, Wm, bias)
    rng = np.random.default_rng(60)
    eps = 1e-3
    checks = 0
    for name, arr, g in [("X", X, gX), ("W", Wm, gW), ("bias", bias, gb)]:
        n = {"X": 24, "W": 24, "bias": 16}[name]
        idx = rng.choice(arr.size, n, replace=False)
        for i in idx:
            args = {"X": X.astype(np.float64), "W": Wm.astype(np.float64),
                    "bias": bias.astype(np.float64)}
            base = args[name].reshape(-1).copy()
            plus_ = base.copy(); plus_[i] += eps
            minus = base.copy(); minus[i] -= eps
            args[name] = plus_.reshape(arr.shape)
            lp = _c4_loss64(args["X"], args["W"], args["bias"])
            args[name] = minus.reshape(arr.shape)
            lm = _c4_loss64(args["X"], args["W"], args["bias"])
            fd = (lp - lm) / (2 * eps)
            got = float(g.reshape(-1)[i])
            assert abs(got - fd) <= 1e-3 * max(abs(fd), 1e-4) + 1e-6, (name, i, got, fd)
            checks += 1
    assert checks == 64


def test_c4_chain_matches_hand_derived_cpu_gradient(gpu):
    X, Wm, bias = _c4_inputs()
    gX, gW, gb = _c4_backward_gpu(X, Wm, bias)
    X64, W64, b64 = X.astype(np.float64), Wm.astype(np.float64), bias.astype(np.float64)
    Z = X64 @ W64 + b64
    gZ = 2.0 * Z / 8192.0
    gY = gZ
    gb_ref = gZ.sum(0)
    gX_ref, gW_ref = np.empty_like(X64), np.empty_like(W64)
    # oracle: matmult gradients written out by hand (double)
    gYc = np.ascontiguousarray(gY)
    O.lib().oracle_matmult_bwd(gYc.ctypes.data, np.ascontiguousarray(X64).ctypes.data,
                               np.ascontiguousarray(W64).ctypes.data, gX_ref.ctypes.data,
                               gW_ref.ctypes.data, 512, 8192, 256, 1, 1, 1)
    for got, ref in [(gX, gX_ref), (gW, gW_ref), (gb, gb_ref)]:
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-4 * scale


def test_autograd_mirror_gradcheck(gpu):
    torch = pytest.importorskip("torch")
    from autograd_mirror import Average, MatMult, Mult, Plus, SumOver
    g = torch.Generator().manual_seed(0)
    a = torch.randn(3, 4, 5, dtype=torch.float64, generator=g, requires_grad=True)
    b = torch.randn(1, 4, 5, dtype=torch.float64, generator=g, requires_grad=True)
    assert torch.autograd.gradcheck(SumOver.apply, (a,), eps=1e-6, atol=1e-8)
    assert torch.autograd.gradcheck(Average.apply, (a,), eps=1e-6, atol=1e-8)
    assert torch.autograd.gradcheck(Plus.apply, (a, b), eps=1e-6, atol=1e-8)
    assert torch.autograd.gradcheck(Mult.apply, (a, b), eps=1e-6, atol=1e-8)
    m1 = torch.randn(2, 6, 5, dtype=torch.float64, generator=g, requires_grad=True)
    m2 = torch.randn(5, 7, dtype=torch.float64, generator=g, requires_grad=True)
    assert torch.autograd.gradcheck(MatMult.apply, (m1, m2), eps=1e-6, atol=1e-8)
