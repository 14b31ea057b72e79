"""Distributed sort (cccl_gb300.distributed_sort) on several ranks.

The cases are those of the reference's multi-GPU sort tests
(cudax/test/multi_gpu/algorithms/sort/range_basic.cu: the documentation example, random
inputs, uneven, empty and skewed rank sizes, a single item, one item per rank, all-equal and
many-equal keys, presorted and reverse-sorted inputs), in both orders, plus pairs whose
values are global indices (the order of equal keys) and floats with +-0.0 and NaN. The
expected result is the oracle's radix sort of the rank-major concatenation of the inputs,
each rank holding as many items as it passed.

* CPU: two, three and four gloo ranks, the oracle as every rank's local sort (the distributed
  steps: splitter search, exchange, merge order).
* GPU: two ranks in two processes on the one GPU, the library's radix sort as the local
  sort, the exchange through host memory (gloo); no kernel of one rank waits on the other.
"""

import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cases(world):
    """(name, dtype, per-rank key arrays, with_values, descending) for `world` ranks."""
    rng = np.random.default_rng(4242 + world)

    def rand(dtype, n):
        if np.dtype(dtype).kind == "f":
            x = rng.standard_normal(n).astype(dtype) * 1e3
            return x
        info = np.iinfo(dtype)
        return rng.integers(info.min, info.max, size=n, dtype=dtype, endpoint=True)

    out = []
    if world == 2:
        out.append(("documentation example", np.int32, [np.array([3, 1], np.int32), np.array([4, 2], np.int32)],
                    False, False))
    for dt in (np.int32, np.int64, np.float64):
        for desc in (False, True):
            out.append((f"random {np.dtype(dt).name}", dt, [rand(dt, 20_000) for _ in range(world)], False, desc))
    out.append(("uneven rank sizes", np.int64, [rand(np.int64, r * 1000 + 1) for r in range(world)], False, False))
    out.append(("some empty ranks", np.int32, [rand(np.int32, 1000 if r % 2 else 0) for r in range(world)], False, True))
    out.append(("all ranks empty", np.int32, [np.zeros(0, np.int32) for _ in range(world)], False, False))
    out.append(("a single global item", np.float64,
                [np.array([7.5]) if r == world - 1 else np.zeros(0) for r in range(world)], False, False))
    out.append(("one item per rank", np.int64, [np.array([world - r], np.int64) for r in range(world)], False, False))
    out.append(("all equal", np.int32, [np.full(1000, 5, np.int32) for _ in range(world)], True, False))
    out.append(("many equal keys", np.int64, [rng.integers(0, 4, size=1000, dtype=np.int64) for _ in range(world)],
                True, True))
    out.append(("presorted", np.int64, [np.arange(r * 1000, (r + 1) * 1000, dtype=np.int64) for r in range(world)],
                False, False))
    out.append(("reverse-sorted", np.int64,
                [np.arange(world * 1000 - r * 1000, world * 1000 - (r + 1) * 1000, -1, dtype=np.int64)
                 for r in range(world)], False, False))
    out.append(("skewed rank sizes", np.uint32, [rand(np.uint32, 1000 if r == 0 else 1) for r in range(world)],
                False, False))
    specials = np.array([0.0, -0.0, np.nan, -np.nan, np.inf, -np.inf], np.float32)
    fl = []
    for r in range(world):
        x = rand(np.float32, 3000)
        x[rng.integers(0, x.size, 300)] = rng.choice(specials, 300)
        fl.append(x)
    out.append(("float32 pairs with +-0 and NaN", np.float32, fl, True, False))
    out.append(("float32 pairs with +-0 and NaN, descending", np.float32, fl, True, True))
    out.append(("uint64 pairs", np.uint64, [rand(np.uint64, 5000) for _ in range(world)], True, False))
    return out


def _expected(oracle, parts, with_values, desc):
    counts = [p.size for p in parts]
    keys = np.concatenate(parts) if sum(counts) else parts[0]
    vals = np.arange(keys.size, dtype=np.int64) if with_values else None
    ko, vo = oracle.radix_sort(keys, vals, 0, None, desc)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return [(ko[offs[r]:offs[r + 1]], vo[offs[r]:offs[r + 1]] if with_values else None) for r in range(len(parts))]


def _rank_main(rank, world, port, device_sort):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    import torch
    import torch.distributed as dist

    from cccl_gb300 import SortOrder
    from cccl_gb300.distributed_sort import distributed_sort
    from oracle import pyoracle

    def oracle_sort(keys, values, descending):
        # the local sort of a rank on the host: the oracle's radix sort (stable, CUB's order)
        k = keys.numpy()
        v = values.numpy() if values is not None else None
        ko, vo = pyoracle.radix_sort(k, v, 0, None, descending)
        return torch.from_numpy(ko.copy()), (torch.from_numpy(vo.copy()) if v is not None else None)

    if device_sort:
        torch.cuda.set_device(0)
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        for name, dt, parts, with_values, desc in _cases(world):
            base = sum(p.size for p in parts[:rank])
            k = torch.from_numpy(parts[rank].copy())
            v = torch.arange(base, base + parts[rank].size, dtype=torch.int64) if with_values else None
            if device_sort:
                k = k.cuda()
                v = v.cuda() if v is not None else None
            distributed_sort(k, v, order=SortOrder.DESCENDING if desc else SortOrder.ASCENDING,
                             local_sort=None if device_sort else oracle_sort)
            ek, ev = _expected(pyoracle, parts, with_values, desc)[rank]
            got_k = k.cpu().numpy()
            assert got_k.size == parts[rank].size, name
            assert got_k.tobytes() == ek.tobytes(), f"{name}: keys of rank {rank} differ"
            if with_values:
                assert v.cpu().numpy().tobytes() == ev.tobytes(), f"{name}: values of rank {rank} differ"
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3, 4])
def test_distributed_sort_on_gloo_ranks(world, oracle):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, False), nprocs=world, join=True, start_method="spawn")


def test_radix_order_image_orders_like_the_oracle(oracle):
    """The integer image the splitter search bisects on sorts every key type as the radix
    sort does (floats: -0.0 equal to +0.0, NaNs by their bits), in both orders."""
    import torch

    from cccl_gb300.distributed_sort import radix_order_image

    rng = np.random.default_rng(3)
    arrays = [
        rng.integers(-(2**31), 2**31 - 1, 4000, dtype=np.int32),
        rng.integers(-(2**63), 2**63 - 1, 4000, dtype=np.int64),
        rng.integers(0, 2**32 - 1, 4000, dtype=np.uint32),
        rng.integers(0, 2**64 - 1, 4000, dtype=np.uint64, endpoint=True),
        rng.integers(-128, 127, 4000, dtype=np.int8),
        rng.integers(0, 65535, 4000, dtype=np.uint16),
    ]
    for dt in (np.float16, np.float32, np.float64):
        x = (rng.standard_normal(4000) * 100).astype(dt)
        x[:60] = np.array([0.0, -0.0, np.nan, -np.nan, np.inf, -np.inf] * 10, dt)
        bits = x.view({2: np.uint16, 4: np.uint32, 8: np.uint64}[x.itemsize])
        bits[60:70] |= np.array(1, bits.dtype)  # NaN payloads and odd mantissas
        arrays.append(x)
    for a in arrays:
        t = torch.from_numpy(a.copy())
        if a.dtype in (np.uint16, np.uint32, np.uint64) and not hasattr(torch, a.dtype.name):
            continue
        for desc in (False, True):
            img = radix_order_image(t, desc).numpy()
            perm = np.argsort(img, kind="stable")
            ko, _ = oracle.radix_sort(a, None, 0, None, desc)
            assert a[perm].tobytes() == ko.tobytes(), (a.dtype, desc)


@pytest.mark.gpu
def test_distributed_sort_two_processes_on_the_gpu(built_library, oracle):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, True), nprocs=2, join=True, start_method="spawn")
