"""Python host API of the learned-partition sort: the same calls as ``make_radix_sort`` /
``radix_sort`` (and the same results, bit for bit, and the same ``DoubleBuffer`` selector),
through the C ABI ``cccl_gb300_learned_sort*`` of the in-tree library. ``stats`` reports
what the last run did: bucket count, partition passes and how many buckets (and keys) went
to the plain radix passes."""

from __future__ import annotations

import ctypes as C

import torch

from . import _bindings as B
from .radix_sort import (
    DoubleBuffer,
    SortOrder,
    _arrays,
    _cc,
    _check_device_array,
    _itemsize,
    _key_iterator,
    _stream_handle,
    _value_iterator,
    check,
)


ROUTES = {"cost_model": 0, "always": 1}  # CCCL_GB300_LEARNED_ROUTE_*


class _LearnedSort:
    def __init__(self, d_in_keys, d_out_keys, d_in_values, d_out_values, order: SortOrder, route="cost_model"):
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        _check_device_array(ki, "d_in_keys")
        self.lib = B.load_library()
        self.order = order
        self.build_result = B.LearnedSortBuildResult()
        major, minor = _cc()
        rc = self.lib.cccl_gb300_learned_sort_build(
            C.byref(self.build_result),
            B.ASCENDING if order is SortOrder.ASCENDING else B.DESCENDING,
            _key_iterator(ki),
            _value_iterator(vi),
            major,
            minor,
        )
        check(rc, "cccl_gb300_learned_sort_build")
        check(self.lib.cccl_gb300_learned_sort_set_route(C.byref(self.build_result), ROUTES[route]),
              "cccl_gb300_learned_sort_set_route")

    def __del__(self):
        try:
            if getattr(self, "build_result", None) is not None and self.build_result.setup:
                self.lib.cccl_gb300_learned_sort_cleanup(C.byref(self.build_result))
        except Exception:
            pass

    def _args(self, d_in_keys, d_out_keys, d_in_values, d_out_values, begin_bit, end_bit):
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        for t, n in ((ki, "keys in"), (ko, "keys out"), (vi, "values in"), (vo, "values out")):
            _check_device_array(t, n)
        begin_bit = 0 if begin_bit is None else begin_bit
        end_bit = _itemsize(ki) * 8 if end_bit is None else end_bit
        return ki, ko, vi, vo, int(begin_bit), int(end_bit), isinstance(d_in_keys, DoubleBuffer)

    def __call__(
        self,
        *,
        temp_storage,
        d_in_keys,
        d_out_keys,
        d_in_values,
        d_out_values,
        num_items: int,
        begin_bit: int | None = None,
        end_bit: int | None = None,
        stream=None,
    ) -> int:
        ki, ko, vi, vo, b, e, overwrite = self._args(d_in_keys, d_out_keys, d_in_values, d_out_values, begin_bit, end_bit)
        if temp_storage is None:
            temp_ptr, temp_bytes = None, C.c_size_t(0)
        else:
            temp_ptr, temp_bytes = temp_storage.data_ptr(), C.c_size_t(temp_storage.numel() * temp_storage.element_size())
        selector = C.c_int(-1)
        rc = self.lib.cccl_gb300_learned_sort(
            self.build_result,
            temp_ptr,
            C.byref(temp_bytes),
            _key_iterator(ki),
            _key_iterator(ko),
            _value_iterator(vi),
            _value_iterator(vo),
            B.no_op(),
            int(num_items),
            b,
            e,
            bool(overwrite),
            C.byref(selector),
            _stream_handle(stream),
        )
        check(rc, "cccl_gb300_learned_sort")
        if overwrite and temp_storage is not None:
            new_sel = d_in_keys.selector ^ selector.value
            d_in_keys.selector = new_sel
            if isinstance(d_in_values, DoubleBuffer):
                d_in_values.selector = new_sel
        return temp_bytes.value

    def stats(
        self,
        *,
        temp_storage,
        d_in_keys,
        d_out_keys,
        d_in_values,
        d_out_values,
        num_items: int,
        begin_bit: int | None = None,
        end_bit: int | None = None,
    ) -> dict:
        """Counters of the last run that used ``temp_storage`` with these arguments (a
        ``DoubleBuffer`` is read at the selector it had when that run started). Synchronizes
        the device."""
        torch.cuda.synchronize()
        ki, ko, vi, vo, b, e, overwrite = self._args(d_in_keys, d_out_keys, d_in_values, d_out_values, begin_bit, end_bit)
        st = B.LearnedSortStats()
        rc = self.lib.cccl_gb300_learned_sort_stats(
            self.build_result,
            temp_storage.data_ptr(),
            _key_iterator(ki),
            _key_iterator(ko),
            _value_iterator(vi),
            _value_iterator(vo),
            int(num_items),
            b,
            e,
            bool(overwrite),
            C.byref(st),
        )
        check(rc, "cccl_gb300_learned_sort_stats")
        return {name: getattr(st, name) for name, _ in B.LearnedSortStats._fields_}


def make_learned_sort(*, d_in_keys, d_out_keys, d_in_values, d_out_values, order: SortOrder,
                      route: str = "cost_model") -> _LearnedSort:
    """Builds a reusable learned-partition sort for the given arrays' dtypes and ``order``.
    ``route="always"`` switches the host cost model off (every qualifying input takes the
    learned kernels); by default 4-byte keys take the plain sort."""
    return _LearnedSort(d_in_keys, d_out_keys, d_in_values, d_out_values, order, route)


def learned_sort(
    *,
    d_in_keys,
    d_out_keys,
    d_in_values=None,
    d_out_values=None,
    num_items: int,
    order: SortOrder,
    begin_bit: int | None = None,
    end_bit: int | None = None,
    stream=None,
):
    """Device-wide learned-partition sort; allocates the temporary storage itself."""
    sorter = make_learned_sort(
        d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values, d_out_values=d_out_values, order=order
    )
    args = dict(
        d_in_keys=d_in_keys,
        d_out_keys=d_out_keys,
        d_in_values=d_in_values,
        d_out_values=d_out_values,
        num_items=num_items,
        begin_bit=begin_bit,
        end_bit=end_bit,
        stream=stream,
    )
    nbytes = sorter(temp_storage=None, **args)
    ref = d_in_keys.current() if isinstance(d_in_keys, DoubleBuffer) else d_in_keys
    tmp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=ref.device)
    if isinstance(stream, torch.cuda.Stream):
        tmp.record_stream(stream)
    sorter(temp_storage=tmp, **args)
