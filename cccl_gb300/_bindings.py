"""ctypes declarations of the sort C ABI (include/cccl/c/*.h) and the library loader.

The struct layouts mirror c/parallel/include/cccl/c/types.h, radix_sort.h and
segmented_sort.h of the reference, so these classes bind either library.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libccclsort.so"

# cccl_type_enum (types.h:31-47)
INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64 = range(8)
FLOAT16, FLOAT32, FLOAT64, STORAGE, BOOLEAN = 8, 9, 10, 11, 12
POINTER, ITERATOR = 0, 1  # cccl_iterator_kind_t
OP_LTOIR, OP_CPP_SOURCE = 0, 1  # cccl_op_code_type
ASCENDING, DESCENDING = 0, 1  # cccl_sort_order_t
PAYLOAD_LTOIR, PAYLOAD_CUBIN = 0, 1

CUDA_SUCCESS = 0
CUDA_ERROR_INVALID_VALUE = 1
CUDA_ERROR_NOT_INITIALIZED = 3
CUDA_ERROR_NOT_SUPPORTED = 801
CUDA_ERROR_INVALID_SOURCE = 300
CUDA_ERROR_UNKNOWN = 999


class TypeInfo(C.Structure):
    _fields_ = [("size", C.c_size_t), ("alignment", C.c_size_t), ("type", C.c_int)]


class Op(C.Structure):
    _fields_ = [
        ("type", C.c_int),
        ("name", C.c_char_p),
        ("code", C.c_char_p),
        ("code_size", C.c_size_t),
        ("code_type", C.c_int),
        ("size", C.c_size_t),
        ("alignment", C.c_size_t),
        ("state", C.c_void_p),
        ("extra_ltoirs", C.c_void_p),
        ("extra_ltoir_sizes", C.c_void_p),
        ("num_extra_ltoirs", C.c_size_t),
        ("extra_code_types", C.c_void_p),
    ]


class BuildConfig(C.Structure):
    _fields_ = [
        ("extra_compile_flags", C.c_void_p),
        ("num_extra_compile_flags", C.c_size_t),
        ("extra_include_dirs", C.c_void_p),
        ("num_extra_include_dirs", C.c_size_t),
    ]


HOST_ADVANCE = C.CFUNCTYPE(None, C.c_void_p, C.c_uint64)


class Iterator(C.Structure):
    _fields_ = [
        ("size", C.c_size_t),
        ("alignment", C.c_size_t),
        ("type", C.c_int),
        ("advance", Op),
        ("dereference", Op),
        ("value_type", TypeInfo),
        ("state", C.c_void_p),
        ("host_advance", C.c_void_p),
    ]


_RADIX_KERNELS = [
    "single_tile",
    "upsweep",
    "alt_upsweep",
    "scan_bins",
    "downsweep",
    "alt_downsweep",
    "histogram",
    "exclusive_sum",
    "init_bins_and_counters",
    "init_lookback",
    "onesweep",
]


class RadixSortBuildResult(C.Structure):
    _fields_ = (
        [
            ("cc", C.c_int),
            ("payload", C.c_void_p),
            ("payload_size", C.c_size_t),
            ("payload_kind", C.c_int),
            ("library", C.c_void_p),
            ("key_type", TypeInfo),
            ("value_type", TypeInfo),
        ]
        + [(k + "_kernel", C.c_void_p) for k in _RADIX_KERNELS]
        + [("order", C.c_int), ("runtime_policy", C.c_void_p), ("runtime_policy_size", C.c_size_t)]
        + [(k + "_kernel_lowered_name", C.c_char_p) for k in _RADIX_KERNELS]
    )


_SEG_KERNELS = [
    "segmented_sort_fallback",
    "segmented_sort_kernel_small",
    "segmented_sort_kernel_large",
    "three_way_partition_init",
    "three_way_partition",
]


class SegmentedSortBuildResult(C.Structure):
    _fields_ = [
        ("cc", C.c_int),
        ("payload", C.c_void_p),
        ("payload_size", C.c_size_t),
        ("payload_kind", C.c_int),
        ("library", C.c_void_p),
        ("key_type", TypeInfo),
        ("offset_type", TypeInfo),
        ("large_segments_selector_op", Op),
        ("small_segments_selector_op", Op),
        ("segmented_sort_fallback_kernel", C.c_void_p),
        ("segmented_sort_kernel_small", C.c_void_p),
        ("segmented_sort_kernel_large", C.c_void_p),
        ("three_way_partition_init_kernel", C.c_void_p),
        ("three_way_partition_kernel", C.c_void_p),
        ("runtime_policy", C.c_void_p),
        ("runtime_policy_size", C.c_size_t),
        ("partition_runtime_policy", C.c_void_p),
        ("partition_runtime_policy_size", C.c_size_t),
        ("order", C.c_int),
        ("segmented_sort_fallback_kernel_lowered_name", C.c_char_p),
        ("segmented_sort_kernel_small_lowered_name", C.c_char_p),
        ("segmented_sort_kernel_large_lowered_name", C.c_char_p),
        ("three_way_partition_init_kernel_lowered_name", C.c_char_p),
        ("three_way_partition_kernel_lowered_name", C.c_char_p),
    ]


class LearnedSortBuildResult(C.Structure):
    _fields_ = [
        ("cc", C.c_int),
        ("key_type", TypeInfo),
        ("value_type", TypeInfo),
        ("order", C.c_int),
        ("radix_library", C.c_void_p),
        ("segmented_library", C.c_void_p),
        ("learned_library", C.c_void_p),
        ("setup", C.c_void_p),
        ("setup_size", C.c_size_t),
    ]


class LearnedSortStats(C.Structure):
    _fields_ = [
        ("learned", C.c_int),
        ("bucket_log2", C.c_int),
        ("partition_passes", C.c_int),
        ("block_buckets", C.c_uint32),
        ("device_buckets", C.c_uint32),
        ("device_items", C.c_uint64),
    ]


# Every symbol the headers under include/ declare.
EXPORTED_SYMBOLS = [
    "cccl_serialization_buffer_free",
    "cccl_device_radix_sort_build",
    "cccl_device_radix_sort_build_ex",
    "cccl_device_radix_sort_compile",
    "cccl_device_radix_sort_load",
    "cccl_device_radix_sort",
    "cccl_device_radix_sort_link_ltoir",
    "cccl_device_radix_sort_serialize",
    "cccl_device_radix_sort_deserialize",
    "cccl_device_radix_sort_cleanup",
    "cccl_device_segmented_sort_build",
    "cccl_device_segmented_sort_build_ex",
    "cccl_device_segmented_sort_compile",
    "cccl_device_segmented_sort_load",
    "cccl_device_segmented_sort",
    "cccl_device_segmented_sort_link_ltoir",
    "cccl_device_segmented_sort_serialize",
    "cccl_device_segmented_sort_deserialize",
    "cccl_device_segmented_sort_cleanup",
    "cccl_gb300_set_launch_observer",
    "cccl_gb300_radix_sort_u32_noalloc",
    "cccl_gb300_learned_sort_build",
    "cccl_gb300_learned_sort",
    "cccl_gb300_learned_sort_stats",
    "cccl_gb300_learned_sort_cleanup",
    "cccl_gb300_learned_sort_set_route",
    "cccl_gb300_segmented_radix_sort",
    "cccl_gb300_merge_sorted_runs",
    "cccl_gb300_sort_status",
    "cccl_gb300_testing_set_wait_fault",
]

# CCCL_GB300_STATUS_* bits (include/cccl_gb300/sort_status.h)
STATUS_WAIT_TIMEOUT, STATUS_BAD_SEGMENT, STATUS_SEG_CAPACITY = 1, 2, 4
CUDA_ERROR_LAUNCH_TIMEOUT = 702

NOALLOC_MAX_ITEMS = 1 << 20  # CCCL_GB300_NOALLOC_MAX_ITEMS

LAUNCH_OBSERVER = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p, C.c_int, C.c_void_p)

_lib = None


def _declare(lib):
    P = C.POINTER
    R = P(RadixSortBuildResult)
    S = P(SegmentedSortBuildResult)
    paths = [C.c_char_p] * 4
    lib.cccl_device_radix_sort_build.argtypes = [R, C.c_int, Iterator, Iterator, Op, C.c_char_p, C.c_int, C.c_int] + paths
    lib.cccl_device_radix_sort_build_ex.argtypes = lib.cccl_device_radix_sort_build.argtypes + [P(BuildConfig)]
    lib.cccl_device_radix_sort_compile.argtypes = lib.cccl_device_radix_sort_build_ex.argtypes
    lib.cccl_device_radix_sort_load.argtypes = [R]
    lib.cccl_device_radix_sort.argtypes = [
        RadixSortBuildResult,
        C.c_void_p,
        P(C.c_size_t),
        Iterator,
        Iterator,
        Iterator,
        Iterator,
        Op,
        C.c_uint64,
        C.c_int,
        C.c_int,
        C.c_bool,
        P(C.c_int),
        C.c_void_p,
    ]
    lib.cccl_gb300_merge_sorted_runs.argtypes = [RadixSortBuildResult, C.c_void_p, P(C.c_size_t), Iterator, Iterator,
                                                 Iterator, Iterator, P(C.c_uint64), C.c_int, C.c_void_p]
    lib.cccl_device_radix_sort_link_ltoir.argtypes = [R, C.c_void_p, C.c_void_p, C.c_size_t]
    lib.cccl_device_radix_sort_serialize.argtypes = [R, P(C.c_void_p), P(C.c_size_t)]
    lib.cccl_device_radix_sort_deserialize.argtypes = [R, C.c_void_p, C.c_size_t]
    lib.cccl_device_radix_sort_cleanup.argtypes = [R]

    lib.cccl_device_segmented_sort_build.argtypes = [S, C.c_int, Iterator, Iterator, Iterator, Iterator, C.c_int, C.c_int] + paths
    lib.cccl_device_segmented_sort_build_ex.argtypes = lib.cccl_device_segmented_sort_build.argtypes + [P(BuildConfig)]
    lib.cccl_device_segmented_sort_compile.argtypes = lib.cccl_device_segmented_sort_build_ex.argtypes
    lib.cccl_device_segmented_sort_load.argtypes = [S]
    lib.cccl_device_segmented_sort.argtypes = [
        SegmentedSortBuildResult,
        C.c_void_p,
        P(C.c_size_t),
        Iterator,
        Iterator,
        Iterator,
        Iterator,
        C.c_uint64,
        C.c_uint64,
        Iterator,
        Iterator,
        C.c_bool,
        P(C.c_int),
        C.c_void_p,
    ]
    lib.cccl_device_segmented_sort_link_ltoir.argtypes = [S, C.c_void_p, C.c_void_p, C.c_size_t]
    lib.cccl_device_segmented_sort_serialize.argtypes = [S, P(C.c_void_p), P(C.c_size_t)]
    lib.cccl_device_segmented_sort_deserialize.argtypes = [S, C.c_void_p, C.c_size_t]
    lib.cccl_device_segmented_sort_cleanup.argtypes = [S]
    lib.cccl_serialization_buffer_free.argtypes = [C.c_void_p]
    lib.cccl_serialization_buffer_free.restype = None
    lib.cccl_gb300_set_launch_observer.argtypes = [LAUNCH_OBSERVER, C.c_void_p]
    lib.cccl_gb300_set_launch_observer.restype = None
    lib.cccl_gb300_radix_sort_u32_noalloc.argtypes = [
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_bool, C.c_void_p]
    lib.cccl_gb300_segmented_radix_sort.argtypes = list(lib.cccl_device_segmented_sort.argtypes[:11]) + [
        C.c_int, C.c_int] + list(lib.cccl_device_segmented_sort.argtypes[11:])
    L = P(LearnedSortBuildResult)
    lib.cccl_gb300_learned_sort_build.argtypes = [L, C.c_int, Iterator, Iterator, C.c_int, C.c_int]
    lib.cccl_gb300_learned_sort.argtypes = [LearnedSortBuildResult] + list(lib.cccl_device_radix_sort.argtypes[1:])
    lib.cccl_gb300_learned_sort_stats.argtypes = [
        LearnedSortBuildResult,
        C.c_void_p,
        Iterator,
        Iterator,
        Iterator,
        Iterator,
        C.c_uint64,
        C.c_int,
        C.c_int,
        C.c_bool,
        P(LearnedSortStats),
    ]
    lib.cccl_gb300_learned_sort_cleanup.argtypes = [L]
    lib.cccl_gb300_learned_sort_set_route.argtypes = [L, C.c_int]
    lib.cccl_gb300_sort_status.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, P(C.c_uint32)]
    lib.cccl_gb300_testing_set_wait_fault.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64]
    for name in EXPORTED_SYMBOLS:
        if name not in ("cccl_serialization_buffer_free", "cccl_gb300_set_launch_observer"):
            getattr(lib, name).restype = C.c_int


CUDA_STUB = Path("/usr/local/cuda/lib64/stubs/libcuda.so")


def load_library(allow_driver_stub: bool = False):
    """Loads the in-tree sort library. Raises when it has not been built: there is no
    fallback implementation.

    ``allow_driver_stub`` lets a machine without an NVIDIA driver load the library for
    host-only calls (compile/serialize/argument checks) by pre-loading the toolkit's
    libcuda stub; any GPU call then fails with CUDA_ERROR_STUB_LIBRARY."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it first (python -m cccl_gb300.build or __graft_entry__.build())"
            )
        try:
            lib = C.CDLL(str(LIB_PATH))
        except OSError as e:
            if not (allow_driver_stub and "libcuda" in str(e) and CUDA_STUB.exists()):
                raise
            C.CDLL(str(CUDA_STUB), mode=C.RTLD_GLOBAL)
            lib = C.CDLL(str(LIB_PATH))
        _declare(lib)
        _lib = lib
    return _lib


def pointer_iterator(ptr: int, type_enum: int, size: int, alignment: int | None = None) -> Iterator:
    """A CCCL_POINTER iterator over device memory at ``ptr`` (0 = absent)."""
    it = Iterator()
    it.size = 8
    it.alignment = 8
    it.type = POINTER
    it.value_type = TypeInfo(size, alignment or size, type_enum)
    it.state = ptr or None
    return it


def code_iterator(state: bytes, alignment: int, type_enum: int, size: int, advance: tuple, dereference: tuple,
                  code_type: int = OP_CPP_SOURCE) -> Iterator:
    """A CCCL_ITERATOR whose operations are given as code (the reference's calling convention:
    ``extern "C" __device__ void advance(void* state, const void* diff)`` with a 64-bit
    unsigned ``diff``, ``extern "C" __device__ void dereference(const void* state, T* out)``).
    ``advance`` and ``dereference`` are ``(name, code)`` pairs, ``code`` C++ source or LTO-IR
    bytes. ``state`` holds the iterator's state bytes; the returned object keeps every buffer
    it points to alive."""
    it = Iterator()
    it.size = len(state)
    it.alignment = alignment
    it.type = ITERATOR
    it.value_type = TypeInfo(size, size, type_enum)
    keep = [C.create_string_buffer(bytes(state), len(state))]
    it.state = C.cast(keep[0], C.c_void_p)
    for field, (name, code) in (("advance", advance), ("dereference", dereference)):
        op = Op()
        op.type = 0  # CCCL_STATELESS
        keep += [name.encode() if isinstance(name, str) else name, code.encode() if isinstance(code, str) else code]
        op.name = keep[-2]
        op.code = keep[-1]
        op.code_size = len(keep[-1])
        op.code_type = code_type
        setattr(it, field, op)
    it._keep = keep
    return it


def no_op() -> Op:
    return Op()
