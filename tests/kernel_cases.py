"""Seeded inputs for the per-kernel parity tests (shared by the CPU pin tests,
the golden-vector generator and the GPU tests)."""
import numpy as np

I32_MIN, I32_MAX = -(2 ** 31), 2 ** 31 - 1

SIZES = [1, 7, 8, 9, 31, 32, 33, 255, 256, 257, 1000, 4099]


def col_small(rng, n, lo=-5, hi=5):
    return rng.integers(lo, hi + 1, n, dtype=np.int64).astype(np.int32)


def col_wide(rng, n):
    """Mix of extremes and ordinary values (comparisons, wrapping arithmetic)."""
    pool = np.array([I32_MIN, I32_MIN + 1, -65536, -1, 0, 1, 2, 46341, 65536, I32_MAX - 1, I32_MAX], dtype=np.int64)
    a = rng.integers(-10 ** 9, 10 ** 9, n, dtype=np.int64)
    pick = rng.random(n) < 0.3
    a[pick] = pool[rng.integers(0, pool.size, pick.sum())]
    return a.astype(np.int32)


def flags(rng, n, p=0.5, canonical=True):
    """bool flags as bytes.  With canonical=False a few true bytes are 7: the
    CUDA kernels and the oracle read any non-zero byte as true (a C++ bool
    holding 7 is undefined behaviour, so the reference functors only get 0/1)."""
    f = (rng.random(n) < p).astype(np.uint8)
    if not canonical:
        nz = rng.random(n) < 0.05
        f[nz & (f == 1)] = 7
    return f


def divisor(rng, n):
    """Divisors with no zero, and numerators avoiding INT_MIN/-1."""
    b = col_wide(rng, n)
    b[b == 0] = 3
    return b


def numerators_for(a, b):
    a = a.copy()
    a[(a == I32_MIN) & (b == -1)] = I32_MIN + 1
    return a


def unique_keys(rng, n, lo):
    """n distinct build keys in [lo, lo + n) (SSB primary keys), shuffled."""
    return (lo + rng.permutation(n)).astype(np.int32)
