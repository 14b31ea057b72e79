"""Seeded segment layouts (the batched segmented-sort configuration and the edge cases of the
reference's segmented-sort tests, c/parallel/test/test_segmented_sort.cpp:593-724)."""

from __future__ import annotations

import numpy as np


def lognormal_segments(rng, total, mu=5.0, sigma=2.5, lo=1, hi=1 << 23, empty_frac=0.05):
    """Lengths lognormal(mu, sigma) clipped to [lo, hi], a fraction set to 0, drawn until the
    running total reaches `total` (the last one truncated)."""
    sizes = []
    acc = 0
    while acc < total:
        s = int(np.clip(rng.lognormal(mu, sigma), lo, hi))
        if rng.random() < empty_frac:
            s = 0
        s = min(s, total - acc)
        sizes.append(s)
        acc += s
    sizes = np.array(sizes, dtype=np.int64)
    ends = np.cumsum(sizes)
    return ends - sizes, ends


def edge_segments(sizes, gap=0):
    """Consecutive segments of the given sizes, optionally separated by uncovered gaps."""
    b, e, pos = [], [], 0
    for s in sizes:
        b.append(pos)
        e.append(pos + s)
        pos += s + gap
    return np.array(b, dtype=np.int64), np.array(e, dtype=np.int64), pos
