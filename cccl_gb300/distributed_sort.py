"""Distributed sort over several GPUs, one process per GPU (the role of the reference's
``cudax::sort(cudax::distributed, comms, envs, inputs, sizes)``,
cudax/include/cuda/experimental/__multi_gpu/algorithm/sort/sort.h:53-118 and
hss/execute.h:39-108).

Every rank passes its own keys (and optionally values) on its own GPU. The sort runs in
place: afterwards rank r holds, in the same number of items it passed, its slice of the
global sequence sorted in radix order, the slices following each other in rank order (the
reference's ``distributed`` result policy; each rank keeps its count, as after its
rebalancing step, hss/rebalance.h). Equal keys keep the order of (rank, index in the rank's
input), so the concatenated result is bit-identical to one ``radix_sort`` of the rank-major
concatenation of the inputs.

The steps, each GB300-side work on the rank's own GPU:
  1. local sort: the radix sort of this library (``radix_sort``, the C ABI);
  2. splitters: for every rank boundary g (a global position), the smallest key v (in the
     sort's order) such that more than g keys are <= v; found by bisection on the keys'
     radix-order integer images, one all-reduce of per-rank counts per round (at most 64
     rounds, every boundary at once). Keys equal to v are then split in rank order, so every
     boundary is exact: the histogramming phase of the reference (hss/histogramming.h) with
     exact counts in place of sampled candidates;
  3. exchange: one all-to-all of the locally sorted keys (and values), each rank sending
     every other rank the run that falls into its slice (hss/data_exchange.h);
  4. merge: the runs a rank receives arrive in rank order, each sorted; ceil(log2(ranks))
     rounds of stable two-way merges on the GPU put them in order, equal keys in rank order
     (cccl_gb300_merge_sorted_runs; the reference merges them k ways, hss/merge_k_way.h).

Transport: ``torch.distributed`` collectives. With the NCCL backend the CUDA tensors are
exchanged directly; with gloo (no GPU collectives) they are staged through host memory.
Keys of every type of the radix sort are taken, in ascending or descending order; custom
comparators and custom key types of the reference (``cmp`` other than less/greater) are
not: the order is the radix sort's (floats: -0.0 equal to +0.0, NaNs by their bits).
"""

from __future__ import annotations

from typing import Callable, Optional

import torch
import torch.distributed as dist

from .radix_sort import SortOrder

_INT64_MIN = -(1 << 63)


def radix_order_image(keys: torch.Tensor, descending: bool = False) -> torch.Tensor:
    """int64 image of every key whose signed order is the radix sort's order of the keys:
    unsigned keys by value, signed keys by value, floats by their bits (negative floats
    inverted, positive ones with the sign bit set, -0.0 folded into +0.0), then the image
    complemented for a descending sort. Equal images are equal keys for the sort."""
    dt = keys.dtype
    if dt in (torch.bool, torch.uint8, torch.int8, torch.int16, torch.int32, torch.int64):
        img = keys.to(torch.int64)
    elif dt in _UNSIGNED_NARROW:
        img = keys.view(_SIGNED_OF[dt]).to(torch.int64) & ((1 << (8 * keys.element_size())) - 1)
    elif dt == getattr(torch, "uint64", None):
        img = keys.view(torch.int64) ^ _INT64_MIN
    elif dt in (torch.float16, torch.float32):
        width = 8 * keys.element_size()
        mask = (1 << width) - 1
        sign = 1 << (width - 1)
        bits = keys.view(_SIGNED_OF[dt]).to(torch.int64) & mask
        bits = torch.where(bits == sign, torch.zeros_like(bits), bits)  # -0.0 -> +0.0
        img = torch.where((bits & sign) != 0, bits ^ mask, bits | sign)  # unsigned order, < 2^width
    elif dt == torch.float64:
        bits = keys.view(torch.int64)
        bits = torch.where(bits == _INT64_MIN, torch.zeros_like(bits), bits)  # -0.0 -> +0.0
        # unsigned image: negative -> ~bits, positive -> bits | sign; signed image = unsigned ^ sign
        img = torch.where(bits < 0, ~bits ^ _INT64_MIN, bits)
    else:
        raise TypeError(f"distributed_sort: keys of dtype {dt} are not supported")
    return ~img if descending else img


_SIGNED_OF = {torch.float16: torch.int16, torch.float32: torch.int32}
_UNSIGNED_NARROW = set()
for _name, _signed in (("uint16", torch.int16), ("uint32", torch.int32)):
    if hasattr(torch, _name):
        _UNSIGNED_NARROW.add(getattr(torch, _name))
        _SIGNED_OF[getattr(torch, _name)] = _signed


def _device_merge(keys: torch.Tensor, values: Optional[torch.Tensor], run_counts: list, descending: bool):
    """Step 4: the stable pairwise merge of the received runs (cccl_gb300_merge_sorted_runs).
    Values of a width the merge kernels do not carry (not 1, 2, 4, 8 or 16 bytes) take the
    radix sort of the concatenation instead, which gives the same order."""
    from .radix_sort import make_radix_sort

    if values is not None and values.element_size() not in (1, 2, 4, 8, 16):
        return _device_radix_sort(keys, values, descending)

    ko = torch.empty_like(keys)
    vo = torch.empty_like(values) if values is not None else None
    offsets = [0]
    for c in run_counts:
        offsets.append(offsets[-1] + int(c))
    args = dict(d_in_keys=keys, d_out_keys=ko, d_in_values=values, d_out_values=vo)
    s = make_radix_sort(order=SortOrder.DESCENDING if descending else SortOrder.ASCENDING, **args)
    nbytes = s.merge_runs(temp_storage=None, run_offsets=offsets, **args)
    temp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=keys.device)
    s.merge_runs(temp_storage=temp, run_offsets=offsets, **args)
    return ko, vo


def _device_radix_sort(keys: torch.Tensor, values: Optional[torch.Tensor], descending: bool):
    """The local sort of step 1 and step 4: this library's radix sort, out of place."""
    from .radix_sort import radix_sort

    n = keys.numel()
    ko = torch.empty_like(keys)
    vo = torch.empty_like(values) if values is not None else None
    if n > 0:
        radix_sort(d_in_keys=keys, d_out_keys=ko, d_in_values=values, d_out_values=vo, num_items=n,
                   order=SortOrder.DESCENDING if descending else SortOrder.ASCENDING)
    return ko, vo


class _Transport:
    """The collectives of one process group: tensors go through host memory on gloo and
    through the rank's GPU on NCCL."""

    def __init__(self, group, device: torch.device):
        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.host_staged = dist.get_backend(group) == "gloo"
        self.device = device

    def _to_wire(self, t: torch.Tensor) -> torch.Tensor:
        if self.host_staged:
            return t.cpu() if t.is_cuda else t
        return t if t.is_cuda else t.to(self.device)

    def all_reduce_sum(self, t: torch.Tensor) -> torch.Tensor:
        w = self._to_wire(t).clone()
        dist.all_reduce(w, op=dist.ReduceOp.SUM, group=self.group)
        return w.to(t.device)

    def all_reduce_minmax(self, lo: int, hi: int) -> tuple[int, int]:
        a = self._to_wire(torch.tensor([lo], dtype=torch.int64))
        b = self._to_wire(torch.tensor([hi], dtype=torch.int64))
        dist.all_reduce(a, op=dist.ReduceOp.MIN, group=self.group)
        dist.all_reduce(b, op=dist.ReduceOp.MAX, group=self.group)
        return int(a.cpu()[0]), int(b.cpu()[0])

    def all_gather(self, t: torch.Tensor) -> torch.Tensor:
        w = self._to_wire(t).contiguous()
        out = [torch.empty_like(w) for _ in range(self.world)]
        dist.all_gather(out, w, group=self.group)
        return torch.stack(out).to(t.device)

    def all_to_all(self, t: torch.Tensor, send: list[int], recv: list[int]) -> torch.Tensor:
        w = self._to_wire(t)
        # a dense copy with unit stride (tensors of one element may carry any stride)
        w = torch.empty(w.numel(), dtype=w.dtype, device=w.device).copy_(w.reshape(-1))
        out = torch.empty(sum(recv), dtype=w.dtype, device=w.device)
        # reinterpret wide or unsigned types as bytes rows: gloo and NCCL move raw elements
        dist.all_to_all_single(out.view(torch.uint8).view(-1, w.element_size()),
                               w.view(torch.uint8).view(-1, w.element_size()),
                               output_split_sizes=recv, input_split_sizes=send, group=self.group)
        return out.to(t.device)


def _count_le(img_sorted: torch.Tensor, probes: torch.Tensor) -> torch.Tensor:
    return torch.searchsorted(img_sorted, probes, right=True)


def _count_lt(img_sorted: torch.Tensor, probes: torch.Tensor) -> torch.Tensor:
    return torch.searchsorted(img_sorted, probes, right=False)


def _cuts(tr: _Transport, img: torch.Tensor, bounds: list[int]) -> list[int]:
    """Rank-local cut of every global boundary g in `bounds` (0 < g < N): how many of this
    rank's sorted keys precede global position g in the (key, rank, index) order."""
    m = len(bounds)
    if m == 0:
        return []
    dev = img.device
    n_local = img.numel()
    big = (1 << 63) - 1
    lo_local = int(img[0]) if n_local else big
    hi_local = int(img[-1]) if n_local else -big - 1
    gmin, gmax = tr.all_reduce_minmax(lo_local, hi_local)
    g = torch.tensor(bounds, dtype=torch.int64, device=dev)
    # smallest v in [gmin, gmax] with count_le(v) > g: pred(gmax) holds (count_le = N > g)
    lo = [gmin - 1] * m  # pred false (nothing is <= gmin - 1)
    hi = [gmax] * m
    while any(h - l > 1 for l, h in zip(lo, hi)):
        mids = [l + (h - l) // 2 if h - l > 1 else h for l, h in zip(lo, hi)]
        probes = torch.tensor(mids, dtype=torch.int64, device=dev)
        cnt = tr.all_reduce_sum(_count_le(img, probes))
        pred = (cnt > g).tolist()
        for j in range(m):
            if hi[j] - lo[j] > 1:
                if pred[j]:
                    hi[j] = mids[j]
                else:
                    lo[j] = mids[j]
    v = torch.tensor(hi, dtype=torch.int64, device=dev)
    lt = _count_lt(img, v)
    eq = _count_le(img, v) - lt
    lt_total = tr.all_reduce_sum(lt)
    eq_all = tr.all_gather(eq)  # [world, m]
    eq_before = eq_all[: tr.rank].sum(dim=0) if tr.rank > 0 else torch.zeros_like(eq)
    take = torch.clamp(g - lt_total - eq_before, min=0)
    take = torch.minimum(take, eq)
    return (lt + take).tolist()


def distributed_sort(
    keys: torch.Tensor,
    values: Optional[torch.Tensor] = None,
    *,
    order: SortOrder = SortOrder.ASCENDING,
    group=None,
    local_sort: Optional[Callable] = None,
) -> None:
    """Sorts the keys (and values) of all ranks of `group` in place; see the module
    docstring. Every rank calls it with its own 1-D tensors (CUDA tensors on its own GPU;
    with gloo, host tensors are accepted too when `local_sort` sorts them). `local_sort`
    (keys, values, descending) -> (sorted keys, values) replaces the library's radix sort,
    for tests of the distributed steps on hosts without a GPU."""
    if keys.dim() != 1 or not keys.is_contiguous():
        raise ValueError("distributed_sort: keys must be a contiguous 1-D tensor")
    if values is not None and (values.shape != keys.shape or not values.is_contiguous()):
        raise ValueError("distributed_sort: values must be a contiguous tensor of the keys' shape")
    descending = order == SortOrder.DESCENDING
    sort = local_sort or _device_radix_sort
    tr = _Transport(group, keys.device)

    # 1. local sort
    ks, vs = sort(keys, values, descending)
    if tr.world == 1:
        keys.copy_(ks)
        if values is not None:
            values.copy_(vs)
        return

    # every rank's count: rank r's slice of the result is [offset_r, offset_r + n_r)
    counts = tr.all_gather(torch.tensor([keys.numel()], dtype=torch.int64)).view(-1).tolist()
    total = sum(counts)
    if total == 0:
        return
    offsets = [0]
    for c in counts:
        offsets.append(offsets[-1] + c)
    bounds = [b for b in offsets[1:-1] if 0 < b < total]

    # 2. exact splitters in the keys' radix-order images
    img = radix_order_image(ks, descending)
    cut_of = dict(zip(bounds, _cuts(tr, img, bounds)))
    n_local = keys.numel()

    def cut(b):
        return 0 if b <= 0 else n_local if b >= total else cut_of[b]

    my_cuts = [cut(b) for b in offsets]
    send = [my_cuts[r + 1] - my_cuts[r] for r in range(tr.world)]
    all_send = tr.all_gather(torch.tensor(send, dtype=torch.int64)).tolist()  # [src][dst]
    recv = [all_send[src][tr.rank] for src in range(tr.world)]
    assert sum(recv) == n_local, (recv, n_local)

    # 3. exchange
    rk = tr.all_to_all(ks, send, recv)
    rv = tr.all_to_all(vs, send, recv) if values is not None else None

    # 4. merge of the rank-ordered runs: pairwise stable merges on the GPU (with a host-side
    # local sort, a stable sort of their concatenation, which gives the same order)
    if local_sort is None:
        fk, fv = _device_merge(rk, rv, recv, descending)
    else:
        fk, fv = sort(rk, rv, descending)
    keys.copy_(fk)
    if values is not None:
        values.copy_(fv)
