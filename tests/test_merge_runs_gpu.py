"""Stable merge of sorted runs (cccl_gb300_merge_sorted_runs, the last step of the sort across
GPUs) against the oracle's stable radix sort of the concatenated runs: 2 to 8 runs, empty
runs, every key kind with +-0.0/NaN floats, both orders, keys only and pairs (values = global
indices, so the order of equal keys across and inside runs is checked)."""

import numpy as np
import pytest
import torch

import inputs as I
from gpu_util import from_dev, to_dev, value_tensor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    assert torch.cuda.is_available()
    return built_library


def _keys(dtype, n, rng):
    if np.dtype(dtype).kind == "f":
        k = (rng.standard_normal(n) * 100).astype(dtype)
        return I.with_specials(k, rng, 1 / 32)
    return I.entropy_reduced(dtype, n, rng, 3)  # many equal keys


@pytest.mark.parametrize("dtype", [np.uint32, np.int64, np.float32, np.float64, np.int16], ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("sizes", [[5000, 7000], [0, 3000, 1, 4096], [2049] * 5, [100, 0, 30000, 2048, 0, 7, 9000, 1]],
                         ids=["2runs", "4runs_empty", "5runs", "8runs"])
@pytest.mark.parametrize("desc", [False, True], ids=["asc", "desc"])
@pytest.mark.parametrize("vdtype", [None, np.int64], ids=["keys", "pairs"])
def test_merge_sorted_runs(oracle, dtype, sizes, desc, vdtype):
    from cccl_gb300 import SortOrder, make_radix_sort

    rng = np.random.default_rng(sum(sizes) + len(sizes) + desc)
    runs = []
    for m in sizes:
        k = _keys(dtype, m, rng)
        runs.append(oracle.radix_sort(k, None, 0, None, desc)[0])  # every run sorted
    keys = np.concatenate(runs)
    n = keys.size
    vals = np.arange(n, dtype=vdtype) if vdtype is not None else None
    ki, ko = to_dev(keys), to_dev(keys)
    vi = value_tensor(vals) if vals is not None else None
    vo = torch.empty_like(vi) if vi is not None else None
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    s = make_radix_sort(order=SortOrder.DESCENDING if desc else SortOrder.ASCENDING, **args)
    nbytes = s.merge_runs(temp_storage=None, run_offsets=offsets.tolist(), **args)
    temp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    s.merge_runs(temp_storage=temp, run_offsets=offsets.tolist(), **args)
    torch.cuda.synchronize()
    rk, rv = oracle.radix_sort(keys, vals, 0, None, desc, threads=8)
    assert from_dev(ko, keys.dtype).tobytes() == rk.tobytes()
    if vals is not None:
        assert from_dev(vo, vals.dtype).tobytes() == rv.tobytes()


def test_merge_sorted_runs_at_size(oracle):
    """Eight runs of 2^22 u64 keys with u32 values (the exchange of an eight-GPU sort)."""
    from cccl_gb300 import SortOrder, make_radix_sort

    rng = np.random.default_rng(77)
    m = 1 << 22
    runs = [oracle.radix_sort(I.entropy_reduced(np.uint64, m, rng, 1), None, threads=8)[0] for _ in range(8)]
    keys = np.concatenate(runs)
    vals = np.arange(keys.size, dtype=np.uint32)
    ki, ko, vi = to_dev(keys), to_dev(keys), to_dev(vals)
    vo = torch.empty_like(vi)
    args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    s = make_radix_sort(order=SortOrder.ASCENDING, **args)
    offsets = [i * m for i in range(9)]
    temp = torch.empty(s.merge_runs(temp_storage=None, run_offsets=offsets, **args), dtype=torch.uint8, device="cuda")
    s.merge_runs(temp_storage=temp, run_offsets=offsets, **args)
    torch.cuda.synchronize()
    rk, rv = oracle.radix_sort(keys, vals, threads=16)
    assert from_dev(ko, np.uint64).tobytes() == rk.tobytes()
    assert from_dev(vo, np.uint32).tobytes() == rv.tobytes()
