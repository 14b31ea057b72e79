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


def lognormal_segments_count(rng, count, total, mu=5.0, sigma=2.5, lo=1, hi=1 << 23, empty_frac=0.05):
    """`count` lengths lognormal(mu, sigma) clipped to [lo, hi], a fraction set to 0, then scaled
    so that they add up to `total`: every non-empty length scaled and rounded down, at least
    1, and the largest segment takes the difference. The segment count of a batch is kept and
    its keys fit `total`."""
    sizes = np.clip(rng.lognormal(mu, sigma, size=count), lo, hi)
    sizes[rng.random(count) < empty_frac] = 0
    scaled = np.floor(sizes * (total / sizes.sum())).astype(np.int64)
    scaled[(sizes > 0) & (scaled < 1)] = 1
    scaled[int(np.argmax(scaled))] += total - int(scaled.sum())
    ends = np.cumsum(scaled)
    assert ends[-1] == total
    return ends - scaled, ends


def edge_segments(sizes, gap=0):
    """Consecutive segments of the given sizes, optionally separated by uncovered gaps."""
    b, e, pos = [], [], 0
    for s in sizes:
        b.append(pos)
        e.append(pos + s)
        pos += s + gap
    return np.array(b, dtype=np.int64), np.array(e, dtype=np.int64), pos


def strided_offset_iterator(B, start: int, step: int, type_enum=None, size=8, prefix="seg", with_code=True):
    """Offsets start + i * step, as the reference's tests build them from C++ source: a state
    struct, an advance that adds the difference to an index and a dereference that scales it."""
    import struct

    type_enum = B.INT64 if type_enum is None else type_enum
    ctype = {4: "int", 8: "long long"}[size]
    state_src = f"struct {prefix}_state {{ long long index; long long step; }};\n"
    adv = (f"{prefix}_advance", state_src + f"""
extern "C" __device__ void {prefix}_advance(void* s, const void* d)
{{
  static_cast<{prefix}_state*>(s)->index += *static_cast<const unsigned long long*>(d);
}}
""")
    der = (f"{prefix}_dereference", state_src + f"""
extern "C" __device__ void {prefix}_dereference(const void* s, {ctype}* out)
{{
  const {prefix}_state* st = static_cast<const {prefix}_state*>(s);
  *out = ({ctype}) (st->index * st->step);
}}
""")
    if not with_code:  # operations named only: their code comes from the other offset iterator
        adv, der = (adv[0], ""), (der[0], "")
    return B.code_iterator(struct.pack("<qq", start // step if step else 0, step), 8, type_enum, size, adv, der)


def nvrtc_available():
    import ctypes as C

    for n in ("libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            C.CDLL(n)
            return True
        except OSError:
            pass
    return False
