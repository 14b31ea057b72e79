"""Seeded input generators shared by the tests, the golden-vector script and the bench.

Distributions follow the reference's own test and benchmark inputs:
  * uniform random bits                         (c2h::gen in cub/test)
  * +-0.0 scattered at 1/128 density            (catch2_test_device_radix_sort_keys.cu:165-218)
  * quiet/signalling NaN of both signs, +-inf   (catch2_test_device_radix_sort_keys.cu:221-285)
  * entropy reduction by AND of k uniform words (catch2_test_device_radix_sort_keys.cu:287-340,
                                                 nvbench_helper/nvbench_helper.cu:340-400)
"""

from __future__ import annotations

import numpy as np

UINT_OF = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def uniform_bits(dtype, n: int, rng: np.random.Generator) -> np.ndarray:
    dtype = np.dtype(dtype)
    u = UINT_OF[dtype.itemsize]
    raw = rng.integers(0, np.iinfo(u).max, size=n, dtype=u, endpoint=True)
    return raw.view(dtype)


def entropy_reduced(dtype, n: int, rng: np.random.Generator, and_steps: int) -> np.ndarray:
    dtype = np.dtype(dtype)
    u = UINT_OF[dtype.itemsize]
    x = uniform_bits(u, n, rng)
    for _ in range(and_steps - 1):
        x &= uniform_bits(u, n, rng)
    return x.view(dtype)


def float_specials(dtype) -> np.ndarray:
    """Bit patterns of the special values of a float dtype."""
    dtype = np.dtype(dtype)
    u = UINT_OF[dtype.itemsize]
    bits = dtype.itemsize * 8
    mant = {2: 10, 4: 23, 8: 52}[dtype.itemsize]
    sign = u(1) << u(bits - 1)
    exp_all = ((u(1) << u(bits - 1 - mant)) - u(1)) << u(mant)
    quiet = u(1) << u(mant - 1)
    pats = [
        u(0),  # +0
        sign,  # -0
        exp_all,  # +inf
        exp_all | sign,  # -inf
        exp_all | quiet,  # +qNaN
        exp_all | quiet | sign,  # -qNaN
        exp_all | u(1),  # +sNaN
        exp_all | u(1) | sign,  # -sNaN
        exp_all | quiet | u(5),  # qNaN with payload
        u(1),  # smallest +denormal
        u(1) | sign,  # smallest -denormal
    ]
    return np.array(pats, dtype=u).view(dtype)


def with_specials(a: np.ndarray, rng: np.random.Generator, density: float = 1 / 128) -> np.ndarray:
    """Scatter +-0, +-inf, NaNs and denormals over a float array."""
    a = a.copy()
    sp = float_specials(a.dtype)
    k = max(1, int(a.size * density)) if a.size else 0
    idx = rng.choice(a.size, size=min(k, a.size), replace=False) if a.size else np.array([], dtype=np.int64)
    a.view(UINT_OF[a.dtype.itemsize])[idx] = sp.view(UINT_OF[a.dtype.itemsize])[rng.integers(0, sp.size, size=idx.size)]
    return a


def finite_floats(dtype, n: int, rng: np.random.Generator) -> np.ndarray:
    return (rng.standard_normal(n) * 1e3).astype(dtype)


def index_values(n: int, dtype=np.uint32) -> np.ndarray:
    """value = original index: makes stability visible in a pairs sort."""
    return np.arange(n, dtype=dtype)


# ---- skewed distributions of the learned-partition sort's workloads ----
def gaussian_mixture(dtype, n: int, rng: np.random.Generator, components: int = 8) -> np.ndarray:
    """Equal-weight mixture: means U(-1e3, 1e3), sigmas log-uniform in [1e-2, 1e2]."""
    means = rng.uniform(-1e3, 1e3, size=components)
    sigmas = 10.0 ** rng.uniform(-2.0, 2.0, size=components)
    c = rng.integers(0, components, size=n)
    return (means[c] + sigmas[c] * rng.standard_normal(n)).astype(dtype)


def lognormal(dtype, n: int, rng: np.random.Generator, mu: float = 0.0, sigma: float = 2.0) -> np.ndarray:
    return rng.lognormal(mu, sigma, size=n).astype(dtype)


def zipf_values(dtype, n: int, rng: np.random.Generator, s: float = 1.1, distinct: int = 1 << 20) -> np.ndarray:
    """Zipf(s) ranks over `distinct` values; rank r maps to the r-th of `distinct` seeded
    uniform values, so frequency is not monotone in the key."""
    w = np.arange(1, distinct + 1, dtype=np.float64) ** -s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ranks = np.searchsorted(cdf, rng.random(n), side="right")
    ranks = np.minimum(ranks, distinct - 1)
    table = rng.uniform(0.0, 1e6, size=distinct).astype(dtype)
    return table[ranks]


def half_uniform_mix(dtype, n: int, rng: np.random.Generator, sigma: float = 3.0) -> np.ndarray:
    """50/50 mix of lognormal(0, sigma) and U(0, 1)."""
    a = rng.lognormal(0.0, sigma, size=n)
    b = rng.random(n)
    return np.where(rng.random(n) < 0.5, a, b).astype(dtype)
