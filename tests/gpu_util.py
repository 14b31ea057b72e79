"""Helpers of the GPU tests: numpy <-> torch CUDA tensors and one sort through the C ABI."""

from __future__ import annotations

import numpy as np
import torch

from cccl_gb300 import DoubleBuffer, SortOrder, make_radix_sort

_TORCH = {
    np.dtype(np.int8): torch.int8,
    np.dtype(np.int16): torch.int16,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.float16): torch.float16,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.float64): torch.float64,
    np.dtype(np.bool_): torch.bool,
}
for _n in ("uint16", "uint32", "uint64"):
    if hasattr(torch, _n):
        _TORCH[np.dtype(_n)] = getattr(torch, _n)


def to_dev(a: np.ndarray) -> torch.Tensor:
    """Bit-exact copy of a numpy array to the GPU (torch dtypes it lacks go as raw bytes)."""
    a = np.ascontiguousarray(a)
    td = _TORCH.get(a.dtype)
    if td is None:
        raise TypeError(a.dtype)
    t = torch.empty(a.size, dtype=td, device="cuda")
    t.view(torch.uint8).copy_(torch.from_numpy(a.view(np.uint8).reshape(-1)))
    return t


def from_dev(t: torch.Tensor, dtype) -> np.ndarray:
    raw = t.view(torch.uint8).cpu().numpy()
    return raw.view(np.dtype(dtype))


def empty_like_dev(a: np.ndarray) -> torch.Tensor:
    return torch.empty(a.size, dtype=_TORCH[np.dtype(a.dtype)], device="cuda")


def value_tensor(v: np.ndarray) -> torch.Tensor:
    """Values of any width, carried as raw words of their size."""
    words = {1: torch.uint8, 2: torch.int16, 4: torch.int32, 8: torch.int64}
    if v.dtype.itemsize in words:
        t = torch.empty(v.size, dtype=words[v.dtype.itemsize], device="cuda")
        t.view(torch.uint8).copy_(torch.from_numpy(np.ascontiguousarray(v).view(np.uint8).reshape(-1)))
        return t
    # 16-byte values: complex128 has the width and alignment
    assert v.dtype.itemsize == 16
    t = torch.empty(v.size, dtype=torch.complex128, device="cuda")
    t.view(torch.uint8).copy_(torch.from_numpy(np.ascontiguousarray(v).view(np.uint8).reshape(-1)))
    return t


def gpu_sort(keys, values=None, begin_bit=0, end_bit=None, descending=False, overwrite=False, return_temp=False,
             method="plain", stats=None, route="always"):
    """Sorts through cccl_device_radix_sort (method "plain") or cccl_gb300_learned_sort
    (method "learned"; `stats`, a dict, receives the run's counters; `route` its host
    policy, "always" or "cost_model"). Returns (keys, values, selector[, temp])."""
    from cccl_gb300 import make_learned_sort

    order = SortOrder.DESCENDING if descending else SortOrder.ASCENDING
    ki = to_dev(keys)
    ko = empty_like_dev(keys)
    vi = vo = None
    if values is not None:
        vi = value_tensor(values)
        vo = torch.empty_like(vi)
    if overwrite:
        dk = DoubleBuffer(ki, ko)
        dv = DoubleBuffer(vi, vo) if vi is not None else None
        args = dict(d_in_keys=dk, d_out_keys=None, d_in_values=dv, d_out_values=None)
    else:
        args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    if method == "learned":  # route: the learned build's host policy ("always": the learned kernels)
        sorter = make_learned_sort(order=order, route=route, **args)
    else:
        sorter = make_radix_sort(order=order, **args)
    nbytes = sorter(temp_storage=None, num_items=keys.size, begin_bit=begin_bit, end_bit=end_bit, **args)
    temp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    sel0 = dk.selector if overwrite else None
    sorter(temp_storage=temp, num_items=keys.size, begin_bit=begin_bit, end_bit=end_bit, **args)
    torch.cuda.synchronize()
    if stats is not None and method == "learned":
        sel_final = dk.selector if overwrite else None
        if overwrite:  # counters are read with the buffers as they were when the run started
            dk.selector = sel0
            if dv is not None:
                dv.selector = sel0
        stats.update(sorter.stats(temp_storage=temp, num_items=keys.size, begin_bit=begin_bit, end_bit=end_bit,
                                  **args))
        if overwrite:
            dk.selector = sel_final
            if dv is not None:
                dv.selector = sel_final
    torch.cuda.synchronize()
    if overwrite:
        sel = dk.selector
        kout = dk.current()
        vout = dv.current() if dv is not None else None
    else:
        sel = None
        kout, vout = ko, vo
    kres = from_dev(kout, keys.dtype)
    vres = from_dev(vout, values.dtype) if values is not None else None
    if return_temp:
        return kres, vres, sel, temp
    return kres, vres, sel


def gpu_seg_sort(keys, values, begin, end, descending=False, overwrite=False, offsets_dtype=np.int32, radix_bits=None):
    """Sorts segments through cccl_device_segmented_sort, or with radix_bits=(begin_bit, end_bit)
    through cccl_gb300_segmented_radix_sort. Output buffers start as copies of the input so
    positions outside every segment compare equal. Returns (keys, values, selector)."""
    import torch

    from cccl_gb300 import DoubleBuffer, SortOrder, make_segmented_radix_sort, make_segmented_sort

    order = SortOrder.DESCENDING if descending else SortOrder.ASCENDING
    ki = to_dev(keys)
    ko = to_dev(keys)
    vi = vo = None
    if values is not None:
        vi = value_tensor(values)
        vo = value_tensor(values)
    bo = torch.from_numpy(np.ascontiguousarray(begin, dtype=offsets_dtype)).cuda()
    eo = torch.from_numpy(np.ascontiguousarray(end, dtype=offsets_dtype)).cuda()
    if overwrite:
        dk = DoubleBuffer(ki, ko)
        dv = DoubleBuffer(vi, vo) if vi is not None else None
        args = dict(d_in_keys=dk, d_out_keys=None, d_in_values=dv, d_out_values=None)
    else:
        args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    maker = make_segmented_sort if radix_bits is None else make_segmented_radix_sort
    s = maker(order=order, start_offsets_in=bo, end_offsets_in=eo, **args)
    call = dict(num_items=keys.size, num_segments=len(begin), start_offsets_in=bo, end_offsets_in=eo, **args)
    if radix_bits is not None:
        call.update(begin_bit=radix_bits[0], end_bit=radix_bits[1])
    nbytes = s(temp_storage=None, **call)
    temp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    s(temp_storage=temp, **call)
    torch.cuda.synchronize()
    if overwrite:
        sel = dk.selector
        kout, vout = dk.current(), (dv.current() if dv is not None else None)
    else:
        sel = None
        kout, vout = ko, vo
    return from_dev(kout, keys.dtype), (from_dev(vout, values.dtype) if values is not None else None), sel


def radix_order(t: torch.Tensor, kind: str, descending: bool = False) -> torch.Tensor:
    """int64 ranks of a key tensor in CUB's radix order, computed with plain torch integer
    operations (an independent check of the engine): unsigned / signed integer order, floats
    by their bit order with -0.0 equal to +0.0 (cub/cub/util_type.cuh:893-963,
    cub/cub/block/radix_rank_sort_operations.cuh:43-80), NaNs placed by their bits.
    Descending order reverses the ranks. kind is "u", "i" or "f"."""
    size = t.element_size()
    raw = t.view({1: torch.int8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[size])
    min64 = torch.iinfo(torch.int64).min
    if kind == "i":
        o = raw.long()
    elif size < 8:
        bits = 8 * size
        u = raw.long() & ((1 << bits) - 1)  # the unsigned bit pattern
        if kind == "f":
            sign = 1 << (bits - 1)
            u = torch.where(u == sign, torch.zeros_like(u), u)  # -0.0 ranks with +0.0
            u = torch.where(u >= sign, u ^ ((1 << bits) - 1), u | sign)
        o = u
    else:
        o = raw.clone()
        if kind == "f":
            o = torch.where(o == min64, torch.zeros_like(o), o)
            o = o ^ ((o >> 63) | min64)  # sortable unsigned bits
        o = o ^ min64  # unsigned order as signed int64
    return ~o if descending else o


def check_sorted_pairs(keys_in: torch.Tensor, keys_out: torch.Tensor, values_out: torch.Tensor, kind: str,
                       descending: bool = False) -> bool:
    """True when keys_out/values_out are the stable radix sort of keys_in with values equal to
    the input index: keys in order, equal keys in index order, values a permutation of the
    indices, and every output key the input key its value names (bit for bit). Together these
    fix the output uniquely. Runs on the GPU."""
    n = keys_in.numel()
    if n == 0:
        return True
    o = radix_order(keys_out, kind, descending)
    if not bool((o[1:] >= o[:-1]).all()):
        return False
    idx = values_out.long()
    if n > 1:
        eq = o[1:] == o[:-1]
        if not bool((idx[1:][eq] > idx[:-1][eq]).all()):
            return False
    del o
    if bool(((idx < 0) | (idx >= n)).any()):
        return False
    seen = torch.zeros(n, dtype=torch.bool, device=keys_in.device)
    seen[idx] = True
    if not bool(seen.all()):
        return False
    size = keys_in.element_size()
    w = {1: torch.int8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[size]
    return bool((keys_in.view(w)[idx] == keys_out.view(w)).all())
