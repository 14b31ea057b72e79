"""numpy front end of the CPU oracle (liboracle.so). TEST INFRASTRUCTURE ONLY: used by
tests/, the smoke check and the CPU-baseline leg of bench.py, never by the library."""

from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

# cccl_type_enum codes of numpy dtypes (c/parallel/include/cccl/c/types.h:31-47)
TYPE_CODES = {
    np.dtype(np.int8): 0,
    np.dtype(np.int16): 1,
    np.dtype(np.int32): 2,
    np.dtype(np.int64): 3,
    np.dtype(np.uint8): 4,
    np.dtype(np.uint16): 5,
    np.dtype(np.uint32): 6,
    np.dtype(np.uint64): 7,
    np.dtype(np.float16): 8,
    np.dtype(np.float32): 9,
    np.dtype(np.float64): 10,
    np.dtype(np.bool_): 12,
}

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        l = C.CDLL(str(LIB))
        vp, u64, i = C.c_void_p, C.c_uint64, C.c_int
        l.oracle_radix_sort.argtypes = [i, vp, vp, u64, vp, vp, u64, i, i, i, i]
        l.oracle_radix_sort.restype = i
        l.oracle_radix_permutation.argtypes = [i, vp, u64, i, i, i, i, vp]
        l.oracle_radix_permutation.restype = i
        if hasattr(l, "oracle_segmented_sort"):
            l.oracle_segmented_sort.argtypes = [i, vp, vp, u64, vp, vp, u64, u64, vp, vp, i, i]
            l.oracle_segmented_sort.restype = i
        _lib = l
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def radix_sort(keys, values=None, begin_bit=0, end_bit=None, descending=False, threads=1, onesweep_zeros=False):
    """cub::DeviceRadixSort result for numpy ``keys`` (and ``values``). With
    ``onesweep_zeros`` a descending sort folds +0.0 into -0.0, as CUB's onesweep passes do
    (inputs larger than the single tile); it differs only under a bit window."""
    keys = np.ascontiguousarray(keys)
    if end_bit is None:
        end_bit = keys.dtype.itemsize * 8
    ko = np.empty_like(keys)
    vo = None
    vb = 0
    if values is not None:
        values = np.ascontiguousarray(values)
        vo = np.empty_like(values)
        vb = values.dtype.itemsize
    rc = lib().oracle_radix_sort(
        TYPE_CODES[keys.dtype], _ptr(keys), _ptr(ko), vb, _ptr(values), _ptr(vo), keys.size,
        begin_bit, end_bit, (2 if onesweep_zeros else 1) if descending else 0, threads,
    )
    if rc:
        raise ValueError(f"oracle_radix_sort rejected its arguments ({rc})")
    return ko, vo


def radix_permutation(keys, begin_bit=0, end_bit=None, descending=False, threads=1):
    keys = np.ascontiguousarray(keys)
    if end_bit is None:
        end_bit = keys.dtype.itemsize * 8
    perm = np.empty(keys.size, dtype=np.uint64)
    rc = lib().oracle_radix_permutation(
        TYPE_CODES[keys.dtype], _ptr(keys), keys.size, begin_bit, end_bit, int(bool(descending)), threads, _ptr(perm)
    )
    if rc:
        raise ValueError(f"oracle_radix_permutation rejected its arguments ({rc})")
    return perm


def segmented_sort(keys, values, begin_offsets, end_offsets, descending=False, threads=1):
    """cub::DeviceSegmentedSort result (size classes and merge network included)."""
    keys = np.ascontiguousarray(keys)
    ko = keys.copy()  # positions outside every segment keep the input (the sort does not write them)
    vo = None
    vb = 0
    if values is not None:
        values = np.ascontiguousarray(values)
        vo = values.copy()
        vb = values.dtype.itemsize
    b = np.ascontiguousarray(begin_offsets, dtype=np.int64)
    e = np.ascontiguousarray(end_offsets, dtype=np.int64)
    rc = lib().oracle_segmented_sort(
        TYPE_CODES[keys.dtype], _ptr(keys), _ptr(ko), vb, _ptr(values), _ptr(vo), keys.size, b.size,
        _ptr(b), _ptr(e), int(bool(descending)), threads,
    )
    if rc:
        raise ValueError(f"oracle_segmented_sort rejected its arguments ({rc})")
    return ko, vo
