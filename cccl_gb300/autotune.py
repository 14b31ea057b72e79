"""Autotuner of the kernel shapes on the GPU it runs on.

The shapes (threads per CTA, keys per thread, CTAs per SM the registers are sized for, the
block classes' algorithm and digit bits) are compile-time constants of the kernels, chosen per key and value
width by the table in ``cccl_gb300/csrc/sort_policy.h``. The tuner rebuilds the library once
per candidate with ``GB300_TUNE_DEFINES`` (the overrides that table honours), times the
affected kernels on synthetic inputs through the launch observer, and writes every
measurement and the best candidate per key type to a JSON table
(``cccl_gb300/tuning_gb300.json``, committed). The library is rebuilt with the shipped table
at the end.

    python -m cccl_gb300.autotune                       # every group
    python -m cccl_gb300.autotune --groups block,segpass

Groups:
  onesweep  persistent onesweep pass (plain sort): u64+u32 pairs, f32+u32 pairs, u32 keys
  sizes     the persistent pass's items per thread per size class: 2^20, 2^24, 2^28 keys
  block     segmented block classes: ~4096-key segments, f32+i32 and f64+i64
  blockbits digit bits of the block classes' passes (5 to 8), per key type and class
  segpass   segmented device-class pass: lognormal segments, f32+i32 and f64+i64
  writeout  the pass write-out with and without 32-bit positions (the onesweep group's cases)
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
TABLE = Path(__file__).resolve().parent / "tuning_gb300.json"

CANDIDATES = {
    "onesweep": [
        "",
        "-DGB300_PERSISTENT_TPB=1024 -DGB300_PERSISTENT_ITEMS=12",
        "-DGB300_PERSISTENT_TPB=1024 -DGB300_PERSISTENT_ITEMS=14",
        "-DGB300_PERSISTENT_TPB=896 -DGB300_PERSISTENT_ITEMS=16",
        "-DGB300_PERSISTENT_TPB=768 -DGB300_PERSISTENT_ITEMS=24",
        "-DGB300_PERSISTENT_TPB=1024 -DGB300_PERSISTENT_ITEMS=6",
    ],
    "block": [
        "",
        "-DGB300_SEG_BLOCK_ALGO=0 -DGB300_SEG_BLOCK_L_ITEMS=16 -DGB300_SEG_BLOCK_MINB=1",
        "-DGB300_SEG_BLOCK_ALGO=0 -DGB300_SEG_BLOCK_L_ITEMS=16 -DGB300_SEG_BLOCK_MINB=2",
        "-DGB300_SEG_BLOCK_ALGO=0 -DGB300_SEG_BLOCK_L_ITEMS=8 -DGB300_SEG_BLOCK_MINB=1",
        "-DGB300_SEG_BLOCK_ALGO=1 -DGB300_SEG_BLOCK_L_ITEMS=8 -DGB300_SEG_BLOCK_MINB=1",
    ],
    "writeout": [
        "",
        "-DGB300_WRITE_OUT_SPECIALISED=0",
    ],
    # digit bits of the block classes' in-shared-memory passes (block_s and block_l vary
    # together; each class's time depends on its own bits only)
    "blockbits": [
        "",
        "-DGB300_SEG_BLOCK_S_BITS=7 -DGB300_SEG_BLOCK_L_BITS=7",
        "-DGB300_SEG_BLOCK_S_BITS=6 -DGB300_SEG_BLOCK_L_BITS=6",
        "-DGB300_SEG_BLOCK_S_BITS=5 -DGB300_SEG_BLOCK_L_BITS=5",
    ],
    # persistent pass tile per size class: the pass time at 2^20, 2^24 and 2^28 keys
    "sizes": [
        "",
        "-DGB300_PERSISTENT_ITEMS=7",
        "-DGB300_PERSISTENT_ITEMS=4",
    ],
    "segpass": [
        "",
        "-DGB300_SEG_PASS_TPB=384 -DGB300_SEG_PASS_ITEMS=12",
        "-DGB300_SEG_PASS_TPB=512 -DGB300_SEG_PASS_ITEMS=12",
        "-DGB300_SEG_PASS_TPB=1024 -DGB300_SEG_PASS_ITEMS=8",
    ],
}


# ---------------------------------------------------------------------------------------
# measurements (run in a fresh process per build, so the rebuilt library is the one loaded)
# ---------------------------------------------------------------------------------------
def _kernel_ms(torch, fn, role, reps=3):
    import bench

    fn()
    torch.cuda.synchronize()
    kt, _ = bench.kernel_times_fn(torch, fn, steps=reps)
    return kt.get(role)


def _segmented_case(torch, kd, vd, sizes, seed=3):
    import numpy as np

    from cccl_gb300 import SortOrder, make_segmented_sort

    lengths = np.asarray(sizes, dtype=np.int64)
    b = np.concatenate([[0], np.cumsum(lengths)[:-1]])
    e = b + lengths
    n = int(e[-1])
    g = torch.Generator(device="cuda").manual_seed(seed)
    k = torch.randn(n, generator=g, device="cuda", dtype=torch.float64).to(kd)
    v = torch.arange(n, device="cuda", dtype=vd)
    bo = torch.from_numpy(b.astype(np.int32)).cuda()
    eo = torch.from_numpy(e.astype(np.int32)).cuda()
    args = dict(d_in_keys=k, d_out_keys=torch.empty_like(k), d_in_values=v, d_out_values=torch.empty_like(v))
    s = make_segmented_sort(order=SortOrder.ASCENDING, start_offsets_in=bo, end_offsets_in=eo, **args)
    call = dict(num_items=n, num_segments=len(b), start_offsets_in=bo, end_offsets_in=eo, **args)
    tmp = torch.empty(s(temp_storage=None, **call), dtype=torch.uint8, device="cuda")
    return lambda: s(temp_storage=tmp, **call)


def measure(group):
    import numpy as np
    import torch

    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import bench

    out = {}
    if group in ("onesweep", "writeout"):
        n = 1 << 26
        cases = {
            "u64+u32": (bench.make_inputs(torch, n, "u64"), True),
            "u32 keys": (bench.make_inputs(torch, n, "u32"), False),
        }
        for name, (keys, pairs) in cases.items():
            s = bench.Sorter(torch, keys, with_values=pairs)
            out[name] = _kernel_ms(torch, s.run, "onesweep")
            del s
        f = torch.randn(n, device="cuda", dtype=torch.float32)
        s = bench.Sorter(torch, f, with_values=True)
        out["f32+u32"] = _kernel_ms(torch, s.run, "onesweep")
    elif group == "sizes":
        for lg in (20, 24, 28):
            n = 1 << lg
            for name, dtype, pairs in (("u32 keys", "u32", False), ("u64+u32", "u64", True)):
                s = bench.Sorter(torch, bench.make_inputs(torch, n, dtype), with_values=pairs)
                out[f"{name} 2^{lg}"] = _kernel_ms(torch, s.run, "onesweep")
                del s
                torch.cuda.empty_cache()
    elif group in ("block", "blockbits"):
        rng = np.random.default_rng(5)
        sizes_l = rng.integers(3000, 5200, size=(1 << 25) // 4100)  # block_l
        sizes_s = rng.integers(300, 2048, size=(1 << 24) // 1200)  # block_s
        for name, kd, vd in (("f32+i32", torch.float32, torch.int32), ("f64+i64", torch.float64, torch.int64)):
            out[name + " block_l"] = _kernel_ms(torch, _segmented_case(torch, kd, vd, sizes_l), "seg_block_l")
            out[name + " block_s"] = _kernel_ms(torch, _segmented_case(torch, kd, vd, sizes_s), "seg_block_s")
    elif group == "segpass":
        import segments

        rng = np.random.default_rng(9)
        b, e = segments.lognormal_segments(rng, 1 << 26)
        sizes = (e - b).astype(np.int64)
        for name, kd, vd in (("f32+i32", torch.float32, torch.int32), ("f64+i64", torch.float64, torch.int64)):
            out[name] = _kernel_ms(torch, _segmented_case(torch, kd, vd, sizes), "seg_pass")
    else:
        raise ValueError(group)
    return out


# ---------------------------------------------------------------------------------------
# the tuning loop: rebuild per candidate, measure, record
# ---------------------------------------------------------------------------------------
def _build(defines):
    env = dict(os.environ, GB300_TUNE_DEFINES=defines)
    subprocess.run([sys.executable, "-c", "from cccl_gb300.build import build; build()"], cwd=ROOT, env=env,
                   check=True, capture_output=True, text=True)
    return env


def run(groups, out_path=TABLE):
    table = json.loads(out_path.read_text()) if out_path.exists() else {}
    for group in groups:
        rows = []
        for defines in CANDIDATES[group]:
            try:
                env = _build(defines)
            except subprocess.CalledProcessError as exc:
                rows.append({"defines": defines, "error": (exc.stderr or "").strip().splitlines()[-3:]})
                continue
            r = subprocess.run([sys.executable, "-m", "cccl_gb300.autotune", "--measure", group], cwd=ROOT, env=env,
                               capture_output=True, text=True)
            if r.returncode != 0:
                rows.append({"defines": defines, "error": r.stderr.strip().splitlines()[-1:]})
                continue
            rows.append({"defines": defines, "ms": json.loads(r.stdout.strip().splitlines()[-1])})
            print(group, repr(defines), rows[-1]["ms"], flush=True)
        best = {}
        cases = sorted({c for row in rows if "ms" in row for c in row["ms"]})
        for case in cases:
            timed = [(row["ms"][case], row["defines"]) for row in rows if "ms" in row and row["ms"].get(case)]
            if timed:
                ms, defines = min(timed)
                best[case] = {"defines": defines or "(shipped table)", "ms": ms}
        table[group] = {"candidates": rows, "best": best}
    _build("")  # back to the shipped table
    out_path.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")
    return table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--groups", default="onesweep,block,segpass")
    ap.add_argument("--measure", help=argparse.SUPPRESS)
    ap.add_argument("--out", default=str(TABLE))
    a = ap.parse_args()
    if a.measure:
        print(json.dumps(measure(a.measure)))
        return
    t = run([g for g in a.groups.split(",") if g], Path(a.out))
    for g, v in t.items():
        print(g, json.dumps(v["best"]))


if __name__ == "__main__":
    main()
