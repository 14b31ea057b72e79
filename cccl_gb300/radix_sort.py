"""Python host API of the radix sort, mirroring the reference's ``cuda.compute``
sort algorithms (python/cuda_cccl/cuda/compute/algorithms/_sort/_radix_sort.py:23-260,
_sort_common.py:16-56): ``SortOrder``, ``DoubleBuffer``, ``make_radix_sort`` and
``radix_sort`` with the same argument names and meaning. Device arrays are torch CUDA
tensors; every call goes through the C ABI (``cccl_device_radix_sort*``) of the in-tree
library.
"""

from __future__ import annotations

import ctypes as C
from enum import Enum

import torch

from . import _bindings as B


class SortOrder(Enum):
    ASCENDING = 0
    DESCENDING = 1


class DoubleBuffer:
    """A pair of device buffers; ``selector`` names the one holding the current data."""

    def __init__(self, d_current, d_alternate):
        self.d_buffers = [d_current, d_alternate]
        self.selector = 0

    def current(self):
        return self.d_buffers[self.selector]

    def alternate(self):
        return self.d_buffers[1 - self.selector]


_KEY_TYPES = {
    torch.int8: B.INT8,
    torch.int16: B.INT16,
    torch.int32: B.INT32,
    torch.int64: B.INT64,
    torch.uint8: B.UINT8,
    torch.float16: B.FLOAT16,
    torch.float32: B.FLOAT32,
    torch.float64: B.FLOAT64,
    torch.bool: B.BOOLEAN,
}
for _name, _code in (("uint16", B.UINT16), ("uint32", B.UINT32), ("uint64", B.UINT64)):
    if hasattr(torch, _name):
        _KEY_TYPES[getattr(torch, _name)] = _code


def type_code(dtype: torch.dtype) -> int:
    """cccl_type_enum of a torch dtype (CCCL_STORAGE for types without one)."""
    return _KEY_TYPES.get(dtype, B.STORAGE)


def _itemsize(t: torch.Tensor) -> int:
    return t.element_size()


def _check_device_array(t, what):
    if t is None:
        return
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{what} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{what} must be contiguous")


def _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values):
    if isinstance(d_in_keys, DoubleBuffer):
        ki, ko = d_in_keys.current(), d_in_keys.alternate()
        if d_in_values is not None:
            if not isinstance(d_in_values, DoubleBuffer):
                raise TypeError("values must be a DoubleBuffer when keys are")
            vi, vo = d_in_values.current(), d_in_values.alternate()
        else:
            vi = vo = None
        return ki, ko, vi, vo
    return d_in_keys, d_out_keys, d_in_values, d_out_values


def _stream_handle(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    if hasattr(stream, "__cuda_stream__"):
        return int(stream.__cuda_stream__()[1])
    return int(stream)


def _key_iterator(t: torch.Tensor) -> B.Iterator:
    return B.pointer_iterator(t.data_ptr(), type_code(t.dtype), _itemsize(t))


def _value_iterator(t) -> B.Iterator:
    if t is None:
        # keys-only: a pointer iterator with a null state (radix_sort.cu:240)
        return B.pointer_iterator(0, B.STORAGE, 4)
    return B.pointer_iterator(t.data_ptr(), type_code(t.dtype), _itemsize(t))


def _cc() -> tuple[int, int]:
    return torch.cuda.get_device_capability()


def check(rc: int, what: str):
    if rc != B.CUDA_SUCCESS:
        raise RuntimeError(f"{what} failed with CUresult {rc}")


class _RadixSort:
    """A built radix sort for one key/value dtype pair and order (the reference's
    ``_RadixSort``). Calling it with ``temp_storage=None`` returns the temp-storage size."""

    def __init__(self, d_in_keys, d_out_keys, d_in_values, d_out_values, order: SortOrder):
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        _check_device_array(ki, "d_in_keys")
        self.lib = B.load_library()
        self.order = order
        self.build_result = B.RadixSortBuildResult()
        major, minor = _cc()
        rc = self.lib.cccl_device_radix_sort_build(
            C.byref(self.build_result),
            B.ASCENDING if order is SortOrder.ASCENDING else B.DESCENDING,
            _key_iterator(ki),
            _value_iterator(vi),
            B.no_op(),
            b"",
            major,
            minor,
            None,
            None,
            None,
            None,
        )
        check(rc, "cccl_device_radix_sort_build")

    def __del__(self):
        try:
            if getattr(self, "build_result", None) is not None and self.build_result.payload:
                self.lib.cccl_device_radix_sort_cleanup(C.byref(self.build_result))
        except Exception:
            pass

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
        ki, ko, vi, vo = _arrays(d_in_keys, d_out_keys, d_in_values, d_out_values)
        for t, n in ((ki, "keys in"), (ko, "keys out"), (vi, "values in"), (vo, "values out")):
            _check_device_array(t, n)
        is_overwrite_okay = isinstance(d_in_keys, DoubleBuffer)
        if begin_bit is None:
            begin_bit = 0
        if end_bit is None:
            end_bit = _itemsize(ki) * 8
        if temp_storage is None:
            temp_ptr, temp_bytes = None, C.c_size_t(0)
        else:
            temp_ptr, temp_bytes = temp_storage.data_ptr(), C.c_size_t(temp_storage.numel() * temp_storage.element_size())
        selector = C.c_int(-1)
        rc = self.lib.cccl_device_radix_sort(
            self.build_result,
            temp_ptr,
            C.byref(temp_bytes),
            _key_iterator(ki),
            _key_iterator(ko),
            _value_iterator(vi),
            _value_iterator(vo),
            B.no_op(),
            int(num_items),
            int(begin_bit),
            int(end_bit),
            bool(is_overwrite_okay),
            C.byref(selector),
            _stream_handle(stream),
        )
        check(rc, "cccl_device_radix_sort")
        if is_overwrite_okay and temp_storage is not None:
            # the returned selector is relative to (current, alternate) of this call
            new_sel = d_in_keys.selector ^ selector.value
            d_in_keys.selector = new_sel
            if isinstance(d_in_values, DoubleBuffer):
                d_in_values.selector = new_sel
        return temp_bytes.value


def _merge_runs(self, *, temp_storage, d_in_keys, d_out_keys, d_in_values, d_out_values, run_offsets, stream=None) -> int:
    """Stable merge of the sorted runs [run_offsets[r], run_offsets[r + 1]) of the inputs into the
    outputs (cccl_gb300_merge_sorted_runs), in this build's order: equal keys keep run order.
    ``temp_storage=None`` returns the temp-storage size."""
    for t, n in ((d_in_keys, "keys in"), (d_out_keys, "keys out"), (d_in_values, "values in"),
                 (d_out_values, "values out")):
        _check_device_array(t, n)
    offs = (C.c_uint64 * len(run_offsets))(*[int(x) for x in run_offsets])
    if temp_storage is None:
        temp_ptr, temp_bytes = None, C.c_size_t(0)
    else:
        temp_ptr, temp_bytes = temp_storage.data_ptr(), C.c_size_t(temp_storage.numel() * temp_storage.element_size())
    rc = self.lib.cccl_gb300_merge_sorted_runs(
        self.build_result,
        temp_ptr,
        C.byref(temp_bytes),
        _key_iterator(d_in_keys),
        _key_iterator(d_out_keys),
        _value_iterator(d_in_values),
        _value_iterator(d_out_values),
        offs,
        len(run_offsets) - 1,
        _stream_handle(stream),
    )
    check(rc, "cccl_gb300_merge_sorted_runs")
    return temp_bytes.value


_RadixSort.merge_runs = _merge_runs


def make_radix_sort(*, d_in_keys, d_out_keys, d_in_values, d_out_values, order: SortOrder) -> _RadixSort:
    """Builds a reusable radix sort for the given arrays' dtypes and ``order``."""
    return _RadixSort(d_in_keys, d_out_keys, d_in_values, d_out_values, order)


def radix_sort(
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
    """Device-wide radix sort; allocates the temporary storage itself."""
    sorter = make_radix_sort(
        d_in_keys=d_in_keys, d_out_keys=d_out_keys, d_in_values=d_in_values, d_out_values=d_out_values, order=order
    )
    nbytes = sorter(
        temp_storage=None,
        d_in_keys=d_in_keys,
        d_out_keys=d_out_keys,
        d_in_values=d_in_values,
        d_out_values=d_out_values,
        num_items=num_items,
        begin_bit=begin_bit,
        end_bit=end_bit,
        stream=stream,
    )
    ref = d_in_keys.current() if isinstance(d_in_keys, DoubleBuffer) else d_in_keys
    tmp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=ref.device)
    if isinstance(stream, torch.cuda.Stream):
        tmp.record_stream(stream)  # the kernels may still read it after we return
    sorter(
        temp_storage=tmp,
        d_in_keys=d_in_keys,
        d_out_keys=d_out_keys,
        d_in_values=d_in_values,
        d_out_values=d_out_values,
        num_items=num_items,
        begin_bit=begin_bit,
        end_bit=end_bit,
        stream=stream,
    )


def sort_status(temp_storage=None, stream=None) -> tuple[int, int]:
    """Waits for ``stream`` and returns ``(CUresult, status bits)`` of the sort that last ran
    with ``temp_storage`` (cccl_gb300_sort_status): CUDA_SUCCESS, or CUDA_ERROR_LAUNCH_TIMEOUT
    when a bounded wait on the GPU ran out (the result is then incomplete), or
    CUDA_ERROR_INVALID_VALUE for segments the segmented sort could not take. The word is
    cleared. ``temp_storage=None`` reads the allocation-free entry point's status."""
    lib = B.load_library()
    bits = C.c_uint32(0)
    if temp_storage is None:
        ptr, nbytes = None, 0
    else:
        ptr, nbytes = temp_storage.data_ptr(), temp_storage.numel() * temp_storage.element_size()
    rc = lib.cccl_gb300_sort_status(ptr, nbytes, _stream_handle(stream), C.byref(bits))
    return rc, bits.value

