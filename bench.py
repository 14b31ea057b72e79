"""Benchmark of the sort engine on one GB300 (or N replicas).

Workload (one "step"): cub::DeviceRadixSort::SortPairs of 2^28 uint64 keys (uniform over
the full 64-bit range, i.e. 64 bits of entropy) with uint32 values (value = original
index), ascending, begin_bit 0 / end_bit 64, through the library's C ABI
(cccl_device_radix_sort). Inputs (3.2 GB) exceed the 129 MB L2, so no flush is needed
between steps. Reported beside the headline line:
  * "variants": the same configuration at AND-reduced entropies, a constant key,
    descending, begin_bit 8 / end_bit 40; 2^28 uint32 keys-only (the roofline row) and
    2^24 uint32 keys-only with L2 flushed between steps;
  * "e2e": the same sort with its inputs uploaded from pinned host memory and its result
    read back every step, over back-to-back batches: three device buffer sets and three
    streams, so batch i+1 uploads and batch i-1 downloads while batch i sorts (the host
    link carries both directions at once); the one-batch-at-a-time step is reported beside it;
  * "segmented": the batched segmented sort of 2^27 f32 keys + i32 values in lognormal
    segments, plain and CUDA-graph replay, against one plain sort launch per segment;
  * "learned": the learned-partition sort against the plain sort on 2^28 f32 + u32
    (Gaussian mixture, lognormal, Zipf) and 2^30 f64 + i64 DoubleBuffer inputs (lognormal,
    lognormal/uniform mix, all-equal, sorted-then-reversed), bit-exactness checked.

Metric: sorted keys per second (higher is better); roofline on HBM with algorithmic bytes
= passes x N x 2 x (key + value bytes). Rows whose digit passes were skipped (constant
digits move no bytes) print a null roofline. "verified": the headline result checked on
the GPU after the timed steps (keys in order, equal keys in index order, values a
permutation of the indices naming their keys); the learned rows check the plain result
the same way ("plain_verified").

--impl reference times the reference library's CPU sort (thrust::sort_by_key on its
OpenMP backend, from the toolkit's CCCL headers) on a bounded sample of the workload.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def check_sorted_pairs(*args, **kw):
    """GPU-side check of a pairs sort with index values (tests/gpu_util.py)."""
    from gpu_util import check_sorted_pairs as check

    return check(*args, **kw)

N_LOG2 = 28
METRIC = "sorted keys/s (SortPairs 2^28 u64 keys + u32 values, 1 GB300)"
UNIT = "keys/s"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(torch, n, key_dtype, ands=1, constant=False, seed=1):
    g = torch.Generator(device="cuda").manual_seed(seed)
    if key_dtype == "u64":
        def draw():
            return torch.randint(-(2**63), 2**63 - 1, (n,), device="cuda", dtype=torch.int64, generator=g)
        k = draw()
        for _ in range(ands - 1):
            k &= draw()
        if constant:
            k.fill_(0x0123456789ABCDEF)
        k = k.view(torch.uint64) if hasattr(torch, "uint64") else k  # same storage, sorted as uint64
    else:  # u32
        k = torch.randint(-(2**31), 2**31 - 1, (n,), device="cuda", dtype=torch.int32, generator=g)
        k = k.view(torch.uint32) if hasattr(torch, "uint32") else k
    return k


class Sorter:
    """One configured sort through the C ABI with preallocated buffers."""

    def __init__(self, torch, keys, with_values, descending=False, begin_bit=0, end_bit=None):
        from cccl_gb300 import SortOrder, make_radix_sort

        self.torch = torch
        n = keys.numel()
        self.n = n
        self.ki = keys
        self.ko = torch.empty_like(keys)
        self.vi = torch.arange(n, device="cuda", dtype=torch.int32) if with_values else None
        self.vo = torch.empty_like(self.vi) if with_values else None
        self.begin_bit = begin_bit
        self.end_bit = end_bit if end_bit is not None else keys.element_size() * 8
        self.args = dict(d_in_keys=self.ki, d_out_keys=self.ko, d_in_values=self.vi, d_out_values=self.vo)
        self.sorter = make_radix_sort(order=SortOrder.DESCENDING if descending else SortOrder.ASCENDING, **self.args)
        nb = self.sorter(temp_storage=None, num_items=n, begin_bit=self.begin_bit, end_bit=self.end_bit, **self.args)
        self.temp = torch.empty(nb, dtype=torch.uint8, device="cuda")
        self.key_bytes = keys.element_size()
        self.value_bytes = 4 if with_values else 0
        self.passes = -(-(self.end_bit - self.begin_bit) // 8)

    def run(self, stream=None):
        self.sorter(temp_storage=self.temp, num_items=self.n, begin_bit=self.begin_bit, end_bit=self.end_bit,
                    stream=stream, **self.args)

    def algorithmic_bytes(self):
        return self.passes * self.n * 2 * (self.key_bytes + self.value_bytes)


def passes_that_run(torch, keys, begin_bit=0, end_bit=None):
    """The 8-bit digit passes of [begin_bit, end_bit) whose digit is not the same for every
    key (the others are skipped by the sort's pass plan and move no bytes). Floats fold -0.0
    into +0.0 first, as the sort's digit extraction does."""
    size = keys.element_size()
    raw = keys.view({1: torch.int8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[size]).long()
    if keys.dtype in (torch.float16, torch.float32, torch.float64):
        neg_zero = (-(1 << (8 * size - 1))) if size == 8 else (1 << (8 * size - 1))
        raw = torch.where(raw == neg_zero, torch.zeros_like(raw), raw)
    end_bit = 8 * size if end_bit is None else end_bit
    run = 0
    for bit in range(begin_bit, end_bit, 8):
        d = (raw >> bit) & ((1 << min(8, end_bit - bit)) - 1)
        run += int(bool((d != d[0]).any()))
    return run


def job_throughput(torch, ms, items_per_rank, world, device):
    """The slowest rank's time per step (max over ranks) and the whole job's throughput: the
    items all ranks sorted per step divided by that time. Ranks run independent replicas."""
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    slowest = float(t.item())
    return slowest, world * items_per_rank / (slowest / 1000.0)


def time_steps(torch, fn, steps, warmup, barrier):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        fn()
    e.record()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / steps  # ms per step


def kernel_times(torch, sorter, steps):
    """Per-role kernel durations (ms), from CUDA events recorded on the launching stream
    by the library's launch observer."""
    from cccl_gb300 import _bindings as B

    lib = B.load_library()
    stream = torch.cuda.current_stream()
    records = []

    def observer(user, role, phase, s):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        records.append((role.decode(), phase, ev))

    cb = B.LAUNCH_OBSERVER(observer)
    lib.cccl_gb300_set_launch_observer(cb, None)
    try:
        for _ in range(steps):
            sorter.run()
        torch.cuda.synchronize()
    finally:
        lib.cccl_gb300_set_launch_observer(B.LAUNCH_OBSERVER(0), None)
    out, count = {}, {}
    open_ev = {}
    for role, phase, ev in records:
        if phase == 0:
            open_ev[role] = ev
        else:
            out.setdefault(role, []).append(open_ev.pop(role).elapsed_time(ev))
            count[role] = count.get(role, 0) + 1
    launches_per_step = sum(count.values()) // steps
    return {r: statistics.mean(v) for r, v in out.items()}, launches_per_step


SEGMENTS_200K = 200_000


def segmented_workload(seed=77, total=1 << 27, segments=None):
    """The batched segmented-sort configuration: f32 N(0,1) keys, 0.1% set to +-0.0/NaN, i32 values,
    lognormal(5, 2.5) segment lengths clipped to [1, 2^23], 5% empty, int32 offsets. Lengths are
    drawn until they add up to 2^27 keys (41,398 segments), or, with `segments`, that many
    lengths are drawn and scaled to add up to 2^27 (the configuration's ~200k segments)."""
    import numpy as np

    import inputs as I
    from segments import lognormal_segments, lognormal_segments_count

    rng = np.random.default_rng(seed)
    if segments is None:
        b, e = lognormal_segments(rng, total)
    else:
        b, e = lognormal_segments_count(rng, segments, total)
    n = int(e[-1])
    k = I.with_specials(rng.standard_normal(n).astype(np.float32), rng, 1e-3)
    v = rng.integers(-(2**31), 2**31 - 1, size=n, dtype=np.int32)
    return k, v, b.astype(np.int32), e.astype(np.int32)


def run_segmented(torch, steps, per_segment_sample=None, segments=None):
    """Batched segmented sort vs one plain radix-sort launch per segment (same GPU). The
    per-segment bar sorts every non-empty segment of the batch with its own plain sort call
    (per_segment_sample limits it to a sample, for profiling runs only)."""
    import numpy as np

    from cccl_gb300 import SortOrder, make_radix_sort, make_segmented_sort

    k, v, b, e = segmented_workload(segments=segments)
    n, nseg = k.size, b.size
    kd = torch.from_numpy(k).cuda()
    vd = torch.from_numpy(v).cuda()
    ko, vo = kd.clone(), vd.clone()
    bo, eo = torch.from_numpy(b).cuda(), torch.from_numpy(e).cuda()
    args = dict(d_in_keys=kd, d_out_keys=ko, d_in_values=vd, d_out_values=vo)
    s = make_segmented_sort(order=SortOrder.ASCENDING, start_offsets_in=bo, end_offsets_in=eo, **args)
    call = dict(num_items=n, num_segments=nseg, start_offsets_in=bo, end_offsets_in=eo, **args)
    temp = torch.empty(s(temp_storage=None, **call), dtype=torch.uint8, device="cuda")

    def once():
        s(temp_storage=temp, **call)

    ms = time_steps(torch, once, steps, 3, lambda: None)
    # the same call sequence captured once in a CUDA graph and replayed
    graph_ms = None
    try:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            once()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            once()
        graph_ms = time_steps(torch, g.replay, steps, 2, lambda: None)
    except Exception as exc:  # graph capture unavailable: report the plain number only
        graph_ms = None
        print(f"graph capture failed: {exc}", file=sys.stderr)
    kt, launches = kernel_times_fn(torch, once)

    # one plain radix SortPairs launch per segment, on a sample of the segments
    sizes = e - b
    idx = np.nonzero(sizes > 0)[0]
    sample = idx if per_segment_sample is None else idx[:: max(1, idx.size // per_segment_sample)]
    rs = make_radix_sort(d_in_keys=kd, d_out_keys=ko, d_in_values=vd, d_out_values=vo, order=SortOrder.ASCENDING)
    max_seg = int(sizes.max())
    tb = max(rs(temp_storage=None, d_in_keys=kd[:max_seg], d_out_keys=ko[:max_seg], d_in_values=vd[:max_seg],
                d_out_values=vo[:max_seg], num_items=max_seg), 1)
    rtemp = torch.empty(tb, dtype=torch.uint8, device="cuda")
    views = [(kd[b[i]:e[i]], ko[b[i]:e[i]], vd[b[i]:e[i]], vo[b[i]:e[i]], int(sizes[i])) for i in sample]

    def per_segment():
        for ki, kout, vi, vout, m in views:
            rs(temp_storage=rtemp, d_in_keys=ki, d_out_keys=kout, d_in_values=vi, d_out_values=vout, num_items=m)

    ps_ms = time_steps(torch, per_segment, 1, 1, lambda: None)
    sample_items = int(sizes[sample].sum())
    # measured over every segment; a profiling sample is scaled by its share of segments
    ps_full_ms = ps_ms * max(idx.size / sample.size, 1.0)
    peak, _ = _peaks()
    alg_bytes = 4 * n * 2 * 8
    return {
        "workload": f"segmented SortPairs: 2^27 f32 keys (0.1% +-0/NaN) + i32 values, {nseg} lognormal(5,2.5) segments"
                    + (" scaled to 2^27 keys" if segments is not None else ""),
        "num_items": n,
        "num_segments": int(nseg),
        "ms": ms,
        "keys_per_s": n / (ms / 1e3),
        "graph_ms": graph_ms,
        "graph_keys_per_s": (n / (graph_ms / 1e3)) if graph_ms else None,
        "roofline_frac_radix_equivalent": alg_bytes / (ms / 1e3) / 1e9 / peak,
        "roofline_frac_one_pass_floor": (n * 16) / (ms / 1e3) / 1e9 / peak,
        "kernel_ms": kt,
        "launches_per_call": launches,
        "per_segment_launch_ms": ps_full_ms,
        "per_segment_launch_measured": {"segments": int(sample.size), "keys": sample_items,
                                        "all_segments": bool(sample.size == idx.size)},
        "speedup_vs_per_segment_launches": ps_full_ms / ms,
    }


def timed_median(torch, fn, reps, warmup=2, prep=None, flush=None):
    """Median of per-step CUDA-event times (ms); prep (untimed) restores the input of an
    in-place sort, flush (untimed) evicts L2 for inputs that fit in it."""
    times = []
    for i in range(warmup + reps):
        if prep is not None:
            prep()
        if flush is not None:
            flush()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        torch.cuda.synchronize()
        if i >= warmup:
            times.append(s.elapsed_time(e))
    return statistics.median(times)


def learned_keys(torch, dist, n, dtype, seed):
    """Seeded synthetic keys of the learned-partition workloads, drawn on the GPU:
    gmm (8 components, means U(-1e3, 1e3), sigmas log-uniform 1e-2..1e2), lognormal(0, 2)
    for 4-byte and lognormal(0, 3) for 8-byte keys, zipf (s = 1.1 over 2^20 seeded uniform
    values), mix (50/50 lognormal(0, 3) and U(0, 1)), all-equal, sorted-then-reversed."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    f64 = torch.float64
    if dist == "gmm":
        means = torch.rand(8, generator=g, device="cuda", dtype=f64) * 2e3 - 1e3
        sig = 10 ** (torch.rand(8, generator=g, device="cuda", dtype=f64) * 4 - 2)
        c = torch.randint(0, 8, (n,), generator=g, device="cuda")
        x = means[c] + sig[c] * torch.randn(n, generator=g, device="cuda", dtype=f64)
    elif dist == "lognormal":
        x = torch.exp(torch.randn(n, generator=g, device="cuda", dtype=f64) * (2.0 if dtype == torch.float32 else 3.0))
    elif dist == "zipf":
        d = 1 << 20
        w = torch.arange(1, d + 1, device="cuda", dtype=f64) ** -1.1
        cdf = torch.cumsum(w, 0)
        cdf /= cdf[-1].clone()
        u = torch.rand(n, generator=g, device="cuda", dtype=f64)
        r = torch.searchsorted(cdf, u, right=True).clamp_(max=d - 1)
        x = (torch.rand(d, generator=g, device="cuda", dtype=f64) * 1e6)[r]
    elif dist == "mix":
        a = torch.exp(torch.randn(n, generator=g, device="cuda", dtype=f64) * 3.0)
        b = torch.rand(n, generator=g, device="cuda", dtype=f64)
        x = torch.where(torch.rand(n, generator=g, device="cuda") < 0.5, a, b)
    elif dist == "all-equal":
        x = torch.full((n,), 3.25, device="cuda", dtype=f64)
    elif dist == "sorted-then-reversed":
        x, _ = torch.sort(torch.exp(torch.randn(n, generator=g, device="cuda", dtype=f64) * 3.0))
        x[n // 2 :] = torch.flip(x[n // 2 :], [0])
    else:
        raise ValueError(dist)
    return x.to(dtype)


def run_learned(torch, reps):
    """Learned-partition sort vs the plain radix sort on the same GPU and inputs: the
    Gaussian-mixture, lognormal and Zipf f32 workloads (2^28 keys + u32 values) and the
    2^30 f64 + i64 DoubleBuffer workloads, adversarial inputs included. Every result is
    checked bit for bit against the plain sort's."""
    from cccl_gb300 import DoubleBuffer, SortOrder, make_learned_sort, make_radix_sort

    peak, _ = _peaks()
    cases = [("2^28 f32 + u32", d, 28, torch.float32, torch.int32, False) for d in ("gmm", "lognormal", "zipf")]
    cases += [("2^30 f64 + i64, DoubleBuffer", d, 30, torch.float64, torch.int64, True)
              for d in ("lognormal", "mix", "all-equal", "sorted-then-reversed")]
    out = []
    for label, dist, lg, kd, vd, overwrite in cases:
        n = 1 << lg
        k0 = learned_keys(torch, dist, n, kd, seed=11)
        v0 = torch.arange(n, device="cuda", dtype=vd)
        kb, vb = k0.element_size(), v0.element_size()
        res = {"workload": f"{label}, {dist}", "num_items": n}
        results = {}
        methods = [("plain", make_radix_sort), ("learned", make_learned_sort)]
        if kb == 4:  # the cost model sends 4-byte keys to the plain sort: time the learned kernels too
            methods.append(("learned_forced", lambda **a: make_learned_sort(route="always", **a)))
        for method, maker in methods:
            k, v = (k0.clone(), v0.clone()) if overwrite else (k0, v0)
            ko, vo = torch.empty_like(k0), torch.empty_like(v0)
            if overwrite:
                dk, dv = DoubleBuffer(k, ko), DoubleBuffer(v, vo)
                args = dict(d_in_keys=dk, d_out_keys=None, d_in_values=dv, d_out_values=None)

                def prep():
                    dk.d_buffers[dk.selector].copy_(k0)
                    dv.d_buffers[dv.selector].copy_(v0)
            else:
                args = dict(d_in_keys=k, d_out_keys=ko, d_in_values=v, d_out_values=vo)
                prep = None
            s = maker(order=SortOrder.ASCENDING, **args)
            tmp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
            ms = timed_median(torch, lambda: s(temp_storage=tmp, num_items=n, **args), reps, prep=prep)
            if prep is not None:
                prep()
            kt, _ = kernel_times_fn(torch, lambda: s(temp_storage=tmp, num_items=n, **args), steps=1)
            res[method + "_ms"] = ms
            res[method + "_keys_per_s"] = n / (ms / 1e3)
            res[method + "_kernel_ms"] = {r: round(t, 4) for r, t in kt.items()}
            if method.startswith("learned"):
                res[method + "_stats"] = s.stats(temp_storage=tmp, num_items=n, **args)
            if overwrite:
                results[method] = (dk.current().clone(), dv.current().clone(), dk.selector)
            else:
                results[method] = (ko.clone(), vo.clone(), None)
            del tmp, s, k, v, ko, vo
            torch.cuda.empty_cache()
        pk, pv, psel = results["plain"]
        lk, lv, lsel = results["learned"]
        res["bitexact_vs_plain"] = bool(torch.equal(pk.view(torch.uint8), lk.view(torch.uint8))
                                        and torch.equal(pv, lv) and psel == lsel)
        if "learned_forced" in results:
            fk, fv, fsel = results["learned_forced"]
            res["learned_forced_bitexact_vs_plain"] = bool(torch.equal(pk.view(torch.uint8), fk.view(torch.uint8))
                                                           and torch.equal(pv, fv) and psel == fsel)
            res["learned_forced_speedup_vs_plain"] = res["plain_ms"] / res["learned_forced_ms"]
        # the plain result itself against an independent check (order, stability, permutation)
        res["plain_verified"] = check_sorted_pairs(k0, pk, pv, "f")
        full_passes = 8 * kb // 8
        res["plain_passes_run"] = passes_that_run(torch, k0)
        res["speedup_vs_plain"] = res["plain_ms"] / res["learned_ms"]
        plain_bytes = (8 * kb // 8) * n * 2 * (kb + vb)  # 8-bit passes x N x 2 x (K + V)
        # a fraction of bytes the sort did not move (skipped passes) would mean nothing: null
        res["roofline_frac_plain_bytes"] = {
            m: (plain_bytes / (res[m + "_ms"] / 1e3) / 1e9 / peak if res["plain_passes_run"] == full_passes else None)
            for m in ("plain", "learned")}
        # the learned route's own bytes (partition passes + the bucket sort), where it ran
        for m in [m for m, _ in methods if m.startswith("learned")]:
            st = res[m + "_stats"]
            learned_bytes = (st["partition_passes"] + 1) * n * 2 * (kb + vb)
            res["roofline_frac_learned_bytes" + m[len("learned"):]] = (
                learned_bytes / (res[m + "_ms"] / 1e3) / 1e9 / peak if st["learned"] else None)
        out.append(res)
        del k0, v0, results, pk, pv, lk, lv
        torch.cuda.empty_cache()
    return out


def kernel_times_fn(torch, fn, steps=3):
    from cccl_gb300 import _bindings as B

    lib = B.load_library()
    stream = torch.cuda.current_stream()
    records = []

    def observer(user, role, phase, s):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        records.append((role.decode(), phase, ev))

    cb = B.LAUNCH_OBSERVER(observer)
    lib.cccl_gb300_set_launch_observer(cb, None)
    try:
        for _ in range(steps):
            fn()
        torch.cuda.synchronize()
    finally:
        lib.cccl_gb300_set_launch_observer(B.LAUNCH_OBSERVER(0), None)
    out, open_ev, count = {}, {}, 0
    for role, phase, ev in records:
        if phase == 0:
            open_ev[role] = ev
        else:
            out[role] = out.get(role, 0.0) + open_ev.pop(role).elapsed_time(ev) / steps
            count += 1
    return out, count // steps


def cpu_reference_sort(n_sample, threads, key_dtype="u64", with_values=True, reps=3):
    """thrust::sort_by_key on the OpenMP backend over a bounded sample (keys/s)."""
    import numpy as np

    lib = C.CDLL(str(ROOT / "oracle" / "libthrust_omp.so"))
    lib.thrust_omp_sort.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int, C.c_int]
    lib.thrust_omp_sort.restype = C.c_int
    rng = np.random.default_rng(7)
    dt = np.uint64 if key_dtype == "u64" else np.uint32
    base = rng.integers(0, np.iinfo(dt).max, size=n_sample, dtype=dt, endpoint=True)
    code = 7 if key_dtype == "u64" else 6
    times = []
    for _ in range(reps):
        k = base.copy()
        v = np.arange(n_sample, dtype=np.uint32) if with_values else None
        t0 = time.perf_counter()
        rc = lib.thrust_omp_sort(code, k.ctypes.data, 4 if with_values else 0, v.ctypes.data if v is not None else None,
                                 n_sample, 0, threads)
        times.append(time.perf_counter() - t0)
        assert rc == 0 and bool(np.all(k[1:] >= k[:-1]))
    return n_sample / statistics.median(times), statistics.median(times)


def ensure_built():
    from cccl_gb300.build import build

    build()
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)


def run_reference(args):
    rank, world = _dist()
    if rank != 0:
        return
    ensure_built()
    threads = os.cpu_count() or 1
    n_sample = 1 << 24
    for _ in range(args.warmup):
        cpu_reference_sort(n_sample, threads, reps=1)
    vals = []
    t_total = 0.0
    for _ in range(args.steps):
        v, t = cpu_reference_sort(n_sample, threads, reps=1)
        vals.append(v)
        t_total += t
    value = statistics.median(vals)
    sample = f"2^24 of the 2^28 u64+u32 pairs per step (thrust::sort_by_key, OpenMP, {threads} threads)"
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000 * t_total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64 keys / u32 values",
        "data": "synthetic (seeded uniform 64-bit keys)",
        "config": {"workload": "SortPairs 2^28 u64 keys + u32 values, asc, bits 0..64 (CPU sample 2^24)",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_engine(args):
    import torch

    rank, world = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

        def barrier():
            dist.barrier()
    else:
        def barrier():
            pass
    if rank == 0:
        ensure_built()
    if world > 1:
        barrier()
    from cccl_gb300.build import build

    build()  # no-op when up to date

    n = 1 << N_LOG2
    keys = make_inputs(torch, n, "u64", seed=1 + rank)
    main = Sorter(torch, keys, with_values=True)

    with ClockSampler(local) as clocks:
        ms = time_steps(torch, main.run, args.steps, args.warmup, barrier)
    ms, value = job_throughput(torch, ms, n, world, "cuda")
    # the headline result itself: sorted by key, equal keys in index order, values a
    # permutation of the indices naming their keys (checked on the GPU, outside the timing)
    verified = check_sorted_pairs(main.ki, main.ko, main.vo, "u")

    # per-kernel durations (observer run, separate from the timed steps)
    ktimes, launches = kernel_times(torch, main, max(3, args.steps // 2))
    peak, peak_kind = _peaks()
    pass_bytes = n * 2 * (8 + 4)
    onesweep_ms = ktimes.get("onesweep")
    achieved = pass_bytes / (onesweep_ms / 1000.0) / 1e9 if onesweep_ms else None
    traffic = None
    tf = ROOT / "profiles" / "onesweep_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("pairs_u64_u32_bytes_per_launch_at_2p28")

    # End to end through the same C ABI: every step uploads its batch (keys and values) from
    # pinned host memory and reads its sorted result back into pinned host memory.
    #   single:    one step at a time (upload, sort, download);
    #   pipelined: back-to-back batches on SETS device buffer sets and three streams, so the
    #              upload of batch i+1 and the download of batch i-1 run beside the sort of
    #              batch i (the host link carries both directions at once). A set is busy
    #              for its batch's upload, sort and download in turn, so three sets keep
    #              every stream fed (two left the upload waiting for a download).
    hk = torch.empty(n, dtype=torch.int64, pin_memory=True)
    hv = torch.empty(n, dtype=torch.int32, pin_memory=True)
    hk.copy_(keys.view(torch.int64))
    hv.copy_(main.vi)
    SETS = 3
    outs = [(torch.empty_like(hk, pin_memory=True), torch.empty_like(hv, pin_memory=True)) for _ in range(SETS)]

    # single: keys and values cross the host link on two streams at once (separate copy engines)
    cur = torch.cuda.current_stream()
    side = [torch.cuda.Stream(), torch.cuda.Stream()]

    def e2e_step():
        ok, ov = outs[0]
        for st in side:
            st.wait_stream(cur)
        with torch.cuda.stream(side[0]):
            main.ki.view(torch.int64).copy_(hk, non_blocking=True)
        with torch.cuda.stream(side[1]):
            main.vi.copy_(hv, non_blocking=True)
        for st in side:
            cur.wait_stream(st)
        main.run()
        for st in side:
            st.wait_stream(cur)
        with torch.cuda.stream(side[0]):
            ok.copy_(main.ko.view(torch.int64), non_blocking=True)
        with torch.cuda.stream(side[1]):
            ov.copy_(main.vo, non_blocking=True)
        for st in side:
            cur.wait_stream(st)

    e2e_steps = max(3, args.steps // 2)
    e2e_single_ms = time_steps(torch, e2e_step, e2e_steps, 1, barrier)
    torch.cuda.synchronize()

    # pipelined
    sets = [main] + [Sorter(torch, torch.empty_like(keys), with_values=True) for _ in range(SETS - 1)]
    up, comp, down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    uploaded = [torch.cuda.Event() for _ in sets]
    sorted_ev = [torch.cuda.Event() for _ in sets]
    downloaded = [torch.cuda.Event() for _ in sets]
    used = [False] * SETS

    def pipelined(steps):
        for i in range(steps):
            b = i % SETS
            s = sets[b]
            if used[b]:
                up.wait_event(downloaded[b])  # the set's previous result has been read back
            with torch.cuda.stream(up):
                s.ki.view(torch.int64).copy_(hk, non_blocking=True)
                s.vi.copy_(hv, non_blocking=True)
                uploaded[b].record(up)
            comp.wait_event(uploaded[b])
            s.run(stream=comp)
            sorted_ev[b].record(comp)
            down.wait_event(sorted_ev[b])
            with torch.cuda.stream(down):
                outs[b][0].copy_(s.ko.view(torch.int64), non_blocking=True)
                outs[b][1].copy_(s.vo, non_blocking=True)
                downloaded[b].record(down)
            used[b] = True

    pipelined(max(3, args.warmup))
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(up)
    pipelined(e2e_steps)
    t1.record(down)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / e2e_steps
    last = (e2e_steps + max(3, args.warmup) - 1) % SETS
    e2e_ok = bool(torch.equal(outs[last][0], sets[last].ko.view(torch.int64).cpu())
                  and torch.equal(outs[last][1], sets[last].vo.cpu()))
    del sets
    torch.cuda.empty_cache()

    # the batched segmented configuration and the learned-partition workloads
    segmented = None
    learned = None
    if not args.no_variants:
        segmented = run_segmented(torch, max(3, args.steps // 2))
        segmented["variant_200k_segments"] = run_segmented(torch, max(3, args.steps // 2), segments=SEGMENTS_200K)
        torch.cuda.empty_cache()
        learned = run_learned(torch, max(3, args.steps // 2))

    # variants of the configuration and the keys-only roofline row
    variants = []
    if not args.no_variants:
        specs = [
            ("entropy 51.9 bit (AND of 2)", dict(ands=2)),
            ("entropy 34.8 bit (AND of 3)", dict(ands=3)),
            ("entropy 12.9 bit (AND of 5)", dict(ands=5)),
            ("constant key", dict(constant=True)),
            ("descending", dict(descending=True)),
            ("bits 8..40", dict(begin_bit=8, end_bit=40)),
            ("u32 keys-only 2^28", dict(u32=True)),
            ("u32 keys-only 2^24 (L2 flushed between steps)", dict(u32=True, log2n=24)),
        ]
        del main
        torch.cuda.empty_cache()
        flush_buf = torch.empty(1 << 28, dtype=torch.uint8, device="cuda")  # 256 MB > L2
        for name, sp in specs:
            nv = 1 << sp.get("log2n", N_LOG2)
            if sp.get("u32"):
                kk = make_inputs(torch, nv, "u32", seed=5)
                s = Sorter(torch, kk, with_values=False)
            else:
                kk = make_inputs(torch, n, "u64", ands=sp.get("ands", 1), constant=sp.get("constant", False), seed=3)
                s = Sorter(torch, kk, with_values=True, descending=sp.get("descending", False),
                           begin_bit=sp.get("begin_bit", 0), end_bit=sp.get("end_bit"))
            if nv < n:
                vms = timed_median(torch, s.run, max(3, args.steps // 2), flush=lambda: flush_buf.fill_(1))
            else:
                vms = time_steps(torch, s.run, max(3, args.steps // 2), 2, barrier)
            kt, _ = kernel_times(torch, s, 3)
            run = passes_that_run(torch, kk, s.begin_bit, s.end_bit)
            variants.append({
                "name": name,
                "num_items": nv,
                "keys_per_s": nv / (vms / 1000.0),
                "ms": vms,
                "passes": s.passes,
                "passes_run": run,
                # null where passes were skipped: those moved no bytes
                "roofline_frac": (s.algorithmic_bytes() / (vms / 1000.0) / 1e9 / peak) if run == s.passes else None,
                "verified": check_sorted_pairs(s.ki, s.ko, s.vo, "u", sp.get("descending", False))
                if s.vo is not None and s.begin_bit == 0 and s.end_bit == 8 * s.key_bytes else None,
                "onesweep_ms": kt.get("onesweep"),
                "histogram_ms": kt.get("histogram"),
            })
            del s, kk
            torch.cuda.empty_cache()
        del flush_buf

    floor = None
    if not args.no_variants:
        keys_only = next((v["onesweep_ms"] for v in variants if v["name"] == "u32 keys-only 2^28"), None)
        # the plain sort of the learned workloads' 2^28 f32 + u32 pairs: the mean of its passes
        f32_pairs = None
        if learned:
            row = learned[0]
            if row.get("plain_kernel_ms") and row.get("plain_passes_run"):
                f32_pairs = row["plain_kernel_ms"]["onesweep"] / row["plain_passes_run"]
        floor = pattern_floor(peak, {"u64 keys + u32 values": onesweep_ms, "u32 keys only": keys_only,
                                     "f32 keys + u32 values": f32_pairs})

    if rank != 0:
        return
    # CPU baseline: the reference's thrust OpenMP sort on a bounded sample (rank 0, N=1)
    cpu = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cv, _ = cpu_reference_sort(1 << 24, threads, reps=3)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "reference",
               "sample": f"2^24 u64+u32 pairs, thrust::sort_by_key on the OpenMP backend (toolkit CCCL), {threads} threads"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64 keys / u32 values (integer bit order)",
        "data": "synthetic (seeded uniform 64-bit keys, value = index)",
        "config": {"workload": "SortPairs 2^28 u64 keys + u32 values, asc, bits 0..64",
                   "num_items": n, "passes": 8, "parallelism": f"replicas x{world}",
                   "l2": "inputs (3.2 GB) larger than L2; no flush"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": "onesweep", "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": pass_bytes, "launch_ms": onesweep_ms},
        "whole_sort_roofline_frac": main_bytes(n) / (ms / 1000.0) / 1e9 / peak,
        "kernel_ms": ktimes,
        "gpu_launches": launches * args.steps,
        "clocks": clocks.summary(),
        "e2e": {"value": n / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": n * 12, "d2h_bytes_per_step": n * 12,
                "ms_per_step": e2e_ms,
                "mode": "pipelined: back-to-back batches, three device buffer sets, the upload of batch i+1 "
                        "and the download of batch i-1 beside the sort of batch i",
                "downloaded_result_matches_device": e2e_ok,
                "single_step": {"value": n / (e2e_single_ms / 1000.0), "ms_per_step": e2e_single_ms,
                                "mode": "one batch at a time: upload, sort, download"}},
        "cpu_baseline": cpu,
        "verified": verified,
        "pattern_floor": floor,
        "variants": variants,
        "segmented": segmented,
        "learned": learned,
    }
    print(json.dumps(line))


def main_bytes(n):
    return 8 * n * 2 * 12


def _floor_lib():
    import ctypes

    from cccl_gb300.build import floor_library_path

    lib = ctypes.CDLL(str(floor_library_path()))
    lib.cccl_gb300_pattern_floor.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    lib.cccl_gb300_pattern_floor.restype = ctypes.c_int
    return lib


def _floor_run(lib, kb, vb, runs, shift=0, reps=5):
    import ctypes

    out = (ctypes.c_float * 3)()
    rc = lib.cccl_gb300_pattern_floor(kb, vb, 1 << N_LOG2, runs, shift, reps, out)
    if rc != 0:
        raise RuntimeError(f"pattern floor: CUDA error {rc}")
    return out[0], int(out[1]), int(out[2])


def pattern_floor(peak, pass_ms, reps=5):
    """The digit pass's memory-pattern floor for the tile shapes of the measured passes
    (cccl_gb300/csrc/pattern_floor.cu): the pass's launch shape, tile and write-out without
    the ranking and the look-back; one run per tile writes each staged tile back contiguously,
    256 runs write its digit runs to their regions, as a pass over uniform keys does."""
    lib = _floor_lib()
    rows = []
    for name, kb, vb in (("u64 keys + u32 values", 8, 4), ("u32 keys only", 4, 0), ("f32 keys + u32 values", 4, 4)):
        c_ms, tile, moved = _floor_run(lib, kb, vb, 1, reps=reps)
        r_ms, _, _ = _floor_run(lib, kb, vb, 256, reps=reps)
        nbytes = moved * 2 * (kb + vb)
        pm = pass_ms.get(name)
        rows.append({
            "shape": name,
            "keys_per_tile": tile,
            "keys_per_digit_run": tile / 256,
            "contiguous_ms": c_ms,
            "contiguous_frac": nbytes / (c_ms / 1000.0) / 1e9 / peak,
            "digit_runs_ms": r_ms,
            "digit_runs_frac": nbytes / (r_ms / 1000.0) / 1e9 / peak,
            "pass_ms": pm,
            "pass_frac": nbytes / (pm / 1000.0) / 1e9 / peak if pm else None,
            "pass_note": "headline pass" if kb == 8 else "mean of the sort's 4 passes (first one order-free)"
                         if vb == 0 else "mean of the 4 passes of the plain sort of the learned rows' 2^28 f32 + u32 (GMM)",
        })
    return {"num_items": 1 << N_LOG2, "unit_ms": "best of 5 launches, CUDA events", "rows": rows}


def pattern_sweep():
    """Run length and alignment of the write pattern at the keys-only tile (10752 u32 keys):
    runs per tile, and runs of 32 keys (128 bytes) shifted by 0, 2 and 16 keys."""
    peak, peak_kind = _peaks()
    lib = _floor_lib()
    rows = []
    for runs, shift in ((1, 0), (64, 0), (128, 0), (224, 0), (256, 0), (336, 0), (336, 2), (336, 16), (512, 0)):
        ms, tile, moved = _floor_run(lib, 4, 0, runs, shift)
        rows.append({"runs_per_tile": runs, "keys_per_run": tile / runs, "shift_bytes": 4 * shift, "ms": ms,
                     "frac": moved * 8 / (ms / 1000.0) / 1e9 / peak})
    pairs = []
    for runs in (1, 256):
        ms, tile, moved = _floor_run(lib, 8, 4, runs)
        pairs.append({"runs_per_tile": runs, "keys_per_run": tile / runs, "ms": ms,
                      "frac": moved * 24 / (ms / 1000.0) / 1e9 / peak})
    print(json.dumps({"pattern_sweep": rows, "keys_per_tile": 10752, "u64_u32_pairs_5760_tile": pairs,
                      "num_items": 1 << N_LOG2, "peak_gbs": peak, "peak_source": peak_kind}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-case", choices=["pairs", "keys", "learned-f32", "learned-f64", "segmented", "pattern-sweep"],
                    help="run untimed sorts for ncu captures: 2^--log2n u64+u32 pairs or u32 keys (two sorts), "
                         "one learned sort of 2^--log2n lognormal f32+i32 / f64+i64 pairs, or the segmented workload; "
                         "pattern-sweep times the digit pass's write pattern by run length and alignment")
    ap.add_argument("--log2n", type=int, default=24)
    args = ap.parse_args()
    if args.profile_case == "pattern-sweep":
        ensure_built()
        pattern_sweep()
        return
    if args.profile_case:
        import torch

        ensure_built()
        n = 1 << args.log2n
        if args.profile_case.startswith("learned"):
            from cccl_gb300 import SortOrder, make_learned_sort

            kd, vd = (torch.float32, torch.int32) if args.profile_case.endswith("f32") else (torch.float64, torch.int64)
            k = learned_keys(torch, "lognormal", n, kd, seed=11)
            v = torch.arange(n, device="cuda", dtype=vd)
            la = dict(d_in_keys=k, d_out_keys=torch.empty_like(k), d_in_values=v, d_out_values=torch.empty_like(v))
            ls = make_learned_sort(order=SortOrder.ASCENDING, **la)
            tmp = torch.empty(ls(temp_storage=None, num_items=n, **la), dtype=torch.uint8, device="cuda")
            ls(temp_storage=tmp, num_items=n, **la)
        elif args.profile_case == "segmented":
            run_segmented(torch, 1, per_segment_sample=10)
        else:
            if args.profile_case == "pairs":
                s = Sorter(torch, make_inputs(torch, n, "u64"), with_values=True)
            else:
                s = Sorter(torch, make_inputs(torch, n, "u32"), with_values=False)
            s.run()
            s.run()
        torch.cuda.synchronize()
        print(f"profile case {args.profile_case} n=2^{args.log2n} done")
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
