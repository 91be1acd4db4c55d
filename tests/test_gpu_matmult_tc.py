"""float32 matmult on the tcgen05 tensor cores (split-bf16) against FP64.

Bounds, per element, with S = (|A| |B|) the product of absolute values:
  bf16x6 (3 limbs, 6 products): |C - C64| <= (K + 8) * 2^-24 * S
  bf16x3 (2 limbs, 3 products): |C - C64| <= 3 * 2^-16 * S + (K + 8) * 2^-24 * S
and the normwise error max|C - C64| / max|C64| of bf16x6 stays <= 1e-6 on
N(0,1) data (the headline's accuracy bar)."""
import numpy as np
import pytest

import pdl_gb300 as P

pytestmark = pytest.mark.gpu


def _run(mode, a, b):
    P.set_matmult_mode(mode)
    try:
        c = P.matmult(P.pdl(a), P.pdl(b))
        kern = P.last_launch_info()["kernel"]
    finally:
        P.set_matmult_mode(P.MATMULT_BF16X6)
    return c.numpy(), kern


def _check(a, b, mode):
    c, kern = _run(mode, a, b)
    ref = np.matmul(a.astype(np.float64), b.astype(np.float64))
    s = np.matmul(np.abs(a).astype(np.float64), np.abs(b).astype(np.float64))
    K = a.shape[-1]
    if mode == P.MATMULT_BF16X6:
        bound = (K + 8) * 2.0 ** -24 * s
    else:
        bound = 3 * 2.0 ** -16 * s + (K + 8) * 2.0 ** -24 * s
    err = np.abs(c - ref)
    assert np.all(err <= bound + 1e-30), f"{mode}: worst excess {np.max(err - bound)}"
    return c, ref, kern


def test_tc_single_tile_smallest(gpu):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((128, 64)).astype(np.float32)   # dims (t=64, h=128)
    b = rng.standard_normal((64, 256)).astype(np.float32)   # dims (w=256, t=64)
    c, ref, kern = _check(a, b, P.MATMULT_BF16X6)
    assert kern == "k_mm_tc_bf16x6"


@pytest.mark.parametrize("mode", [P.MATMULT_BF16X6, P.MATMULT_BF16X3])
@pytest.mark.parametrize("shape", [(130, 100, 300), (1, 1, 1), (5, 7, 3), (256, 512, 256),
                                   (300, 33, 520)])
def test_tc_shapes_and_tails(gpu, mode, shape):
    M, K, N = shape
    rng = np.random.default_rng(M * 7 + K)
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((K, N)).astype(np.float32)
    _check(a, b, mode)


def test_tc_batched_and_broadcast(gpu):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((3, 200, 64)).astype(np.float32)    # batched a
    b = rng.standard_normal((64, 300)).astype(np.float32)       # broadcast b
    _check(a, b, P.MATMULT_BF16X6)
    b3 = rng.standard_normal((3, 64, 300)).astype(np.float32)
    _check(a, b3, P.MATMULT_BF16X6)
    a1 = rng.standard_normal((200, 64)).astype(np.float32)
    _check(a1, b3, P.MATMULT_BF16X6)


def test_tc_strided_views(gpu):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((96, 130)).astype(np.float32)
    b = rng.standard_normal((260, 96)).astype(np.float32)
    x = P.pdl(a).xchg(0, 1)   # dims (h=130, ...) viewed as (t=96? no) -> transposed
    y = P.pdl(b).xchg(0, 1)
    got = P.matmult(x, y).numpy()
    ref = x.numpy().astype(np.float64) @ y.numpy().astype(np.float64)
    s = np.abs(x.numpy()).astype(np.float64) @ np.abs(y.numpy()).astype(np.float64)
    assert np.all(np.abs(got - ref) <= (96 + 8) * 2.0 ** -24 * s)


def test_tc_integer_valued_exact(gpu):
    # small integers are exact in bf16 and in the float32 accumulator
    im = np.array([[1, 2, 3, 3, 5], [2, 3, 4, 5, 6], [13, 13, 13, 13, 13],
                   [1, 3, 1, 3, 1], [10, 10, 2, 2, 2]], np.float32)
    c, _ = _run(P.MATMULT_BF16X6, im, im)
    assert np.array_equal(c, im @ im)


def test_tc_normwise_error_meets_1e6(gpu):
    rng = np.random.default_rng(4)
    a = rng.standard_normal((512, 1024)).astype(np.float32)
    b = rng.standard_normal((1024, 512)).astype(np.float32)
    c, _ = _run(P.MATMULT_BF16X6, a, b)
    ref = a.astype(np.float64) @ b.astype(np.float64)
    assert np.max(np.abs(c - ref)) / np.max(np.abs(ref)) <= 1e-6
