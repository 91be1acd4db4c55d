"""Seeded synthetic inputs of the configurations (the same numpy calls the
bench makes), shared by the real-PDL fixture script and the tests that
compare against its fixtures.  numpy's PCG64 streams give the same bytes on
every platform, and the fixtures record each input's SHA-256 to prove it."""
import functools
import hashlib

import numpy as np

F32_BAD = np.float32(-3.4028234663852886e38)


def sha(arr) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def c1():
    """float64 (4096, 2048) uniform[-1, 1), seed 1 (numpy shape (2048, 4096))."""
    return {"a": np.random.default_rng(1).uniform(-1.0, 1.0, size=(2048, 4096))}


def exp_portable(x: np.ndarray) -> np.ndarray:
    """exp(x) for float32 x with the same bits on every platform (numpy's
    vectorised exp differs between x86 and Arm in the last bits): only IEEE
    float32 multiplies, adds, floor and ldexp.  x = (e + f) ln 2 with e an
    integer and f in [0, 1); 2^f from its degree-9 Taylor series (relative
    error below 1e-6, ample for drawing lognormal magnitudes)."""
    x = np.asarray(x, dtype=np.float32)
    t = x * np.float32(1.4426950408889634)
    e = np.floor(t)
    g = (t - e) * np.float32(0.6931471805599453)
    p = np.ones_like(g)
    for k in range(9, 0, -1):
        p *= g
        p *= np.float32(1.0 / k)
        p += np.float32(1.0)
    return np.ldexp(p, e.astype(np.int32))


LN2 = 0.6931471805599453


def log_portable(x: np.ndarray) -> np.ndarray:
    """Natural log of positive normal float64 x with the same bits on every
    platform: only IEEE float64 adds, multiplies, divides and frexp.
    x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
    s = (m - 1)/(m + 1), |s| < 0.1716, from the odd series to s^23 (each
    term below 1e-18 of the sum after that)."""
    m, e = np.frexp(np.asarray(x, dtype=np.float64))
    small = m < 0.7071067811865476
    m = np.where(small, m * 2.0, m)
    e = np.where(small, e - 1, e).astype(np.float64)
    s = (m - 1.0) / (m + 1.0)
    s2 = s * s
    p = np.full_like(s, 1.0 / 23.0)
    for k in range(21, 0, -2):
        p *= s2
        p += 1.0 / k
    return e * LN2 + 2.0 * s * p


def normal_portable(rng: np.random.Generator, count: int) -> np.ndarray:
    """count standard normal float64 values by Marsaglia's polar method from
    rng.random() doubles (exact integer-derived values) and log_portable:
    the same values on every platform, unlike numpy's ziggurat, whose
    rejection step calls the platform's libm."""
    out = np.empty(count)
    got = 0
    while got < count:
        k = (count - got) // 2 + 1024
        u = 2.0 * rng.random(k) - 1.0
        v = 2.0 * rng.random(k) - 1.0
        s = u * u + v * v
        keep = (s > 0.0) & (s < 1.0)
        u, v, s = u[keep], v[keep], s[keep]
        f = np.sqrt(-2.0 * log_portable(s) / s)
        z = np.empty(2 * len(s))
        z[0::2] = u * f
        z[1::2] = v * f
        take = min(len(z), count - got)
        out[got:got + take] = z[:take]
        got += take
    return out


@functools.lru_cache(maxsize=1)
def c5(rows=4096, n=65536, long_n=1 << 27):
    """float32 (65536, 4096) and one row of 2^27: lognormal(0, 4) magnitudes
    (exp(4 z), z standard normal), random sign, 1 % float's default badvalue,
    seed 7.  The last result is cached (about 40 s to make): callers must not
    modify the arrays."""
    rng = np.random.default_rng(7)

    def gen(count):
        out = np.empty(count, dtype=np.float32)
        step = 1 << 24
        for s in range(0, count, step):                 # bounded temporaries
            m = min(step, count - s)
            z = normal_portable(rng, m).astype(np.float32)
            out[s:s + m] = exp_portable(np.float32(4.0) * z)
        out *= np.where(rng.random(count, dtype=np.float32) < 0.5, np.float32(-1), np.float32(1))
        out[rng.random(count, dtype=np.float32) < 0.01] = F32_BAD
        return out

    mat = gen(n * rows).reshape(rows, n)
    return {"mat": mat, "row": gen(long_n).reshape(1, -1) if long_n else None}


def c2_int32():
    """a int32 (256, 1, 8192), b int32 (256, 512, 1), U{-1000..1000}, seed 2."""
    rng = np.random.default_rng(2)
    a = rng.integers(-1000, 1001, size=(8192, 1, 256)).astype(np.int32)
    b = rng.integers(-1000, 1001, size=(1, 512, 256)).astype(np.int32)
    return {"a": a, "b": b}


def c2_float32_bad():
    """The same shapes, float32 N(0, 1), 2 % of a and of b BAD, seed 3."""
    rng = np.random.default_rng(3)
    a = rng.standard_normal((8192, 1, 256)).astype(np.float32)
    b = rng.standard_normal((1, 512, 256)).astype(np.float32)
    a[rng.random(a.shape) < 0.02] = F32_BAD
    b[rng.random(b.shape) < 0.02] = F32_BAD
    return {"a": a, "b": b}


def c3_inner(cols=65536):
    """float64 a, b (4096, 65536) uniform[-1, 1), seed 5."""
    rng = np.random.default_rng(5)
    a = rng.uniform(-1.0, 1.0, size=(cols, 4096))
    b = rng.uniform(-1.0, 1.0, size=(cols, 4096))
    return {"a": a, "b": b}


def c3_matmult(nb=16):
    """float32 a(t=1024, h=2048) batch 16, b(w=2048, t=1024), N(0, 1), seed 4."""
    rng = np.random.default_rng(4)
    a = rng.standard_normal((nb, 2048, 1024)).astype(np.float32)
    b = rng.standard_normal((1024, 2048)).astype(np.float32)
    return {"a": a, "b": b}


def c4():
    """The adjoint workload: X float32 PDL dims (512, 8192), W (256, 512),
    bias (256), each 0.1 N(0, 1), seed 6 (numpy shapes reversed)."""
    rng = np.random.default_rng(6)
    X = (0.1 * rng.standard_normal((8192, 512))).astype(np.float32)
    W = (0.1 * rng.standard_normal((512, 256))).astype(np.float32)
    bias = (0.1 * rng.standard_normal(256)).astype(np.float32)
    return {"X": X, "W": W, "bias": bias}
