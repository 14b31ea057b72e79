"""Python host API of the batched segmented sort, mirroring the reference's
``cuda.compute`` (python/cuda_cccl/cuda/compute/algorithms/_sort/_segmented_sort.py:24-260):
``make_segmented_sort`` and ``segmented_sort`` with the same argument names. Every call goes
through the C ABI (``cccl_device_segmented_sort*``) of the in-tree library.

``make_segmented_radix_sort`` / ``segmented_radix_sort`` add ``begin_bit`` / ``end_bit`` and
give cub::DeviceSegmentedRadixSort's results (radix order in every segment, its selector),
through ``cccl_gb300_segmented_radix_sort``.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _bindings as B
from .radix_sort import (
    DoubleBuffer,
    SortOrder,
    _arrays,
    _check_device_array,
    _key_iterator,
    _stream_handle,
    _value_iterator,
    check,
    type_code,
)


def _offset_iterator(t) -> B.Iterator:
    """A device array of int32/int64 offsets, or an iterator given as code
    (``_bindings.code_iterator``), which the build compiles into an evaluation kernel."""
    if isinstance(t, B.Iterator):
        if t.type != B.ITERATOR or t.value_type.size not in (4, 8):
            raise TypeError("segment offset iterators must yield int32 or int64")
        return t
    _check_device_array(t, "segment offsets")
    if t.dtype not in (torch.int32, torch.int64):
        raise TypeError("segment offsets must be int32 or int64")
    return B.pointer_iterator(t.data_ptr(), type_code(t.dtype), t.element_size())


class _SegmentedSort:
    """A built segmented sort for one key/value dtype pair and order. Calling it with
    ``temp_storage=None`` returns the temp-storage size."""

    def __init__(self, d_in_keys, d_out_keys, d_in_values, d_out_values, start_offsets_in, end_offsets_in,
                 order: SortOrder):
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        _check_device_array(ki, "d_in_keys")
        self.lib = B.load_library()
        self.build_result = B.SegmentedSortBuildResult()
        major, minor = torch.cuda.get_device_capability()
        rc = self.lib.cccl_device_segmented_sort_build(
            C.byref(self.build_result),
            B.ASCENDING if order is SortOrder.ASCENDING else B.DESCENDING,
            _key_iterator(ki),
            _value_iterator(vi),
            _offset_iterator(start_offsets_in),
            _offset_iterator(end_offsets_in),
            major,
            minor,
            None,
            None,
            None,
            None,
        )
        check(rc, "cccl_device_segmented_sort_build")

    def __del__(self):
        try:
            if getattr(self, "build_result", None) is not None and self.build_result.payload:
                self.lib.cccl_device_segmented_sort_cleanup(C.byref(self.build_result))
        except Exception:
            pass

    radix_only = False

    def __call__(self, *, temp_storage, d_in_keys, d_out_keys, d_in_values, d_out_values, num_items, num_segments,
                 start_offsets_in, end_offsets_in, stream=None, begin_bit=None, end_bit=None) -> int:
        if num_segments > 2**31 - 1:
            raise RuntimeError("Segmented sort does not currently support more than 2^31-1 segments.")
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        for t, n in ((ki, "keys in"), (ko, "keys out"), (vi, "values in"), (vo, "values out")):
            _check_device_array(t, n)
        is_overwrite_okay = isinstance(d_in_keys, DoubleBuffer)
        if temp_storage is None:
            temp_ptr, temp_bytes = None, C.c_size_t(0)
        else:
            temp_ptr = temp_storage.data_ptr()
            temp_bytes = C.c_size_t(temp_storage.numel() * temp_storage.element_size())
        selector = C.c_int(-1)
        common = (
            self.build_result,
            temp_ptr,
            C.byref(temp_bytes),
            _key_iterator(ki),
            _key_iterator(ko),
            _value_iterator(vi),
            _value_iterator(vo),
            int(num_items),
            int(num_segments),
            _offset_iterator(start_offsets_in),
            _offset_iterator(end_offsets_in),
        )
        tail = (bool(is_overwrite_okay), C.byref(selector), _stream_handle(stream))
        if self.radix_only:
            b = 0 if begin_bit is None else int(begin_bit)
            e = ki.element_size() * 8 if end_bit is None else int(end_bit)
            rc = self.lib.cccl_gb300_segmented_radix_sort(*common, b, e, *tail)
            check(rc, "cccl_gb300_segmented_radix_sort")
        else:
            if begin_bit is not None or end_bit is not None:
                raise TypeError("bit windows belong to the segmented radix sort")
            rc = self.lib.cccl_device_segmented_sort(*common, *tail)
            check(rc, "cccl_device_segmented_sort")
        if is_overwrite_okay and temp_storage is not None:
            new_sel = d_in_keys.selector ^ selector.value
            d_in_keys.selector = new_sel
            if isinstance(d_in_values, DoubleBuffer):
                d_in_values.selector = new_sel
        return temp_bytes.value


def make_segmented_sort(*, d_in_keys, d_out_keys=None, d_in_values=None, d_out_values=None, start_offsets_in,
                        end_offsets_in, order: SortOrder) -> _SegmentedSort:
    """Builds a reusable segmented sort for the given arrays' dtypes and ``order``."""
    return _SegmentedSort(d_in_keys, d_out_keys, d_in_values, d_out_values, start_offsets_in, end_offsets_in, order)


def segmented_sort(*, d_in_keys, d_out_keys=None, d_in_values=None, d_out_values=None, num_items: int,
                   num_segments: int, start_offsets_in, end_offsets_in, order: SortOrder, stream=None):
    """Device-wide segmented sort; allocates the temporary storage itself."""
    s = make_segmented_sort(d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values,
                            d_out_values=d_out_values, start_offsets_in=start_offsets_in,
                            end_offsets_in=end_offsets_in, order=order)
    args = dict(d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values, d_out_values=d_out_values,
                num_items=num_items, num_segments=num_segments, start_offsets_in=start_offsets_in,
                end_offsets_in=end_offsets_in, stream=stream)
    nbytes = s(temp_storage=None, **args)
    ref = d_in_keys.current() if isinstance(d_in_keys, DoubleBuffer) else d_in_keys
    tmp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=ref.device)
    if isinstance(stream, torch.cuda.Stream):
        tmp.record_stream(stream)
    s(temp_storage=tmp, **args)


class _SegmentedRadixSort(_SegmentedSort):
    """cub::DeviceSegmentedRadixSort semantics over the same build."""

    radix_only = True


def make_segmented_radix_sort(*, d_in_keys, d_out_keys=None, d_in_values=None, d_out_values=None, start_offsets_in,
                              end_offsets_in, order: SortOrder) -> _SegmentedRadixSort:
    """Builds a reusable segmented radix sort (call it with ``begin_bit`` / ``end_bit``)."""
    return _SegmentedRadixSort(d_in_keys, d_out_keys, d_in_values, d_out_values, start_offsets_in, end_offsets_in,
                               order)


def segmented_radix_sort(*, d_in_keys, d_out_keys=None, d_in_values=None, d_out_values=None, num_items: int,
                         num_segments: int, start_offsets_in, end_offsets_in, order: SortOrder, begin_bit=None,
                         end_bit=None, stream=None):
    """Device-wide segmented radix sort; allocates the temporary storage itself."""
    s = make_segmented_radix_sort(d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values,
                                  d_out_values=d_out_values, start_offsets_in=start_offsets_in,
                                  end_offsets_in=end_offsets_in, order=order)
    args = dict(d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values, d_out_values=d_out_values,
                num_items=num_items, num_segments=num_segments, start_offsets_in=start_offsets_in,
                end_offsets_in=end_offsets_in, stream=stream, begin_bit=begin_bit, end_bit=end_bit)
    nbytes = s(temp_storage=None, **args)
    ref = d_in_keys.current() if isinstance(d_in_keys, DoubleBuffer) else d_in_keys
    tmp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=ref.device)
    if isinstance(stream, torch.cuda.Stream):
        tmp.record_stream(stream)
    s(temp_storage=tmp, **args)
