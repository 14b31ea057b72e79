"""Host-side checks of the C ABI that need no GPU: the library loads, exports every symbol
the headers declare, and its compile / serialize / deserialize / cleanup / argument
checks behave like the reference's (c/parallel/test/test_radix_sort.cpp:332-471)."""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib(built_library):
    from cccl_gb300 import _bindings as B

    return B.load_library(allow_driver_stub=True)


def header_symbols():
    names = set()
    for h in (ROOT / "include").glob("**/*.h"):
        text = h.read_text()
        names |= set(re.findall(r"CCCL_(?:C|GB300)_API\s+(?:\w+\s+)*?(cccl_\w+)\s*\(", text))
        names |= set(re.findall(r"CCCL_C_API\s+CUresult\s*\n\s*(cccl_\w+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(lib):
    from cccl_gb300 import _bindings as B

    declared = header_symbols()
    assert declared == set(B.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(lib, name), name


def _compile(lib, key_type=None, value_type=None, order=0, cc=(10, 3), decomposer_name=None):
    from cccl_gb300 import _bindings as B

    key_type = key_type if key_type is not None else (B.UINT32, 4)
    build = B.RadixSortBuildResult()
    keys = B.pointer_iterator(0x1000, key_type[0], key_type[1])
    vals = B.pointer_iterator(0x2000 if value_type else 0, *(value_type or (B.STORAGE, 4)))
    op = B.Op()
    if decomposer_name:
        op.name = decomposer_name
    rc = lib.cccl_device_radix_sort_compile(
        C.byref(build), order, keys, vals, op, b"", cc[0], cc[1], None, None, None, None, None
    )
    return rc, build


def test_compile_fills_build_result(lib):
    from cccl_gb300 import _bindings as B

    rc, b = _compile(lib, (B.FLOAT32, 4), (B.UINT32, 4), order=B.DESCENDING)
    assert rc == B.CUDA_SUCCESS
    assert b.cc == 103 and b.payload and b.payload_size > 0 and b.payload_kind == B.PAYLOAD_CUBIN
    assert b.runtime_policy and b.runtime_policy_size > 0 and b.order == B.DESCENDING
    assert b.onesweep_kernel_lowered_name == b"gb300_onesweep_k4_v4_f"
    assert b.histogram_kernel_lowered_name == b"gb300_histogram_k4_f"
    for f, _ in B.RadixSortBuildResult._fields_:
        if f.endswith("_lowered_name"):
            assert getattr(b, f), f
    assert not b.library and not b.onesweep_kernel  # nothing loaded before _load
    assert lib.cccl_device_radix_sort_cleanup(C.byref(b)) == B.CUDA_SUCCESS


def test_serialize_round_trip(lib):
    from cccl_gb300 import _bindings as B

    rc, b = _compile(lib, (B.INT64, 8), (B.FLOAT64, 8))
    assert rc == 0
    buf, size = C.c_void_p(), C.c_size_t()
    assert lib.cccl_device_radix_sort_serialize(C.byref(b), C.byref(buf), C.byref(size)) == 0
    assert size.value > b.payload_size
    b2 = B.RadixSortBuildResult()
    assert lib.cccl_device_radix_sort_deserialize(C.byref(b2), buf, size) == 0
    assert b2.payload_size == b.payload_size and b2.cc == b.cc and b2.order == b.order
    assert C.string_at(b2.payload, b2.payload_size) == C.string_at(b.payload, b.payload_size)
    assert b2.onesweep_kernel_lowered_name == b.onesweep_kernel_lowered_name
    assert b2.key_type.type == B.INT64 and b2.value_type.size == 8
    assert not b2.library
    # a truncated or foreign blob is rejected and leaves the target untouched
    b3 = B.RadixSortBuildResult()
    assert lib.cccl_device_radix_sort_deserialize(C.byref(b3), buf, 10) != 0
    assert not b3.payload
    raw = bytearray(C.string_at(buf, size.value))
    raw[8] = 8  # algorithm tag: segmented sort
    assert lib.cccl_device_radix_sort_deserialize(C.byref(b3), bytes(raw), len(raw)) != 0
    lib.cccl_serialization_buffer_free(buf)
    for x in (b, b2):
        assert lib.cccl_device_radix_sort_cleanup(C.byref(x)) == 0


def test_compile_rejections(lib):
    from cccl_gb300 import _bindings as B

    assert _compile(lib, cc=(9, 0))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _compile(lib, decomposer_name=b"my_decomposer")[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _compile(lib, key_type=(B.STORAGE, 12))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _compile(lib, value_type=(B.STORAGE, 16))[0] == B.CUDA_SUCCESS
    # values of other widths (custom structs) are accepted: the kernels carry 32-bit indices
    # (the build's kernels are the 4-byte-value ones) and the run gathers the values
    rc, b = _compile(lib, value_type=(B.STORAGE, 12))
    assert rc == B.CUDA_SUCCESS and b.onesweep_kernel_lowered_name.endswith(b"_v4_i")
    assert lib.cccl_device_radix_sort_cleanup(C.byref(b)) == B.CUDA_SUCCESS
    assert _compile(lib, value_type=(B.STORAGE, 0))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert lib.cccl_device_radix_sort_cleanup(None) == B.CUDA_ERROR_INVALID_VALUE
    assert lib.cccl_device_radix_sort_load(None) == B.CUDA_ERROR_INVALID_VALUE


def test_run_rejects_non_pointer_iterators(lib):
    from cccl_gb300 import _bindings as B

    rc, b = _compile(lib)
    it = B.pointer_iterator(0x1000, B.UINT32, 4)
    bad = B.pointer_iterator(0x1000, B.UINT32, 4)
    bad.type = B.ITERATOR
    nbytes, sel = C.c_size_t(0), C.c_int(-1)
    r = lib.cccl_device_radix_sort(b, None, C.byref(nbytes), bad, it, it, it, B.Op(), 16, 0, 32, False, C.byref(sel), None)
    assert r == B.CUDA_ERROR_UNKNOWN
    lib.cccl_device_radix_sort_cleanup(C.byref(b))


def test_link_ltoir_has_nothing_to_link(lib):
    from cccl_gb300 import _bindings as B

    rc, b = _compile(lib)
    assert lib.cccl_device_radix_sort_link_ltoir(C.byref(b), None, None, 0) == B.CUDA_ERROR_INVALID_VALUE
    lib.cccl_device_radix_sort_cleanup(C.byref(b))


def _learned_build(lib, key_type, value_type=None, order=0, cc=(10, 3)):
    from cccl_gb300 import _bindings as B

    build = B.LearnedSortBuildResult()
    keys = B.pointer_iterator(0x1000, key_type[0], key_type[1])
    vals = B.pointer_iterator(0x2000 if value_type else 0, *(value_type or (B.STORAGE, 4)))
    return lib.cccl_gb300_learned_sort_build(C.byref(build), order, keys, vals, cc[0], cc[1]), build


def test_learned_build_rejections(lib):
    """Argument checks that run before any device work."""
    from cccl_gb300 import _bindings as B

    assert _learned_build(lib, (B.FLOAT32, 4), cc=(10, 0))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _learned_build(lib, (B.UINT16, 2))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _learned_build(lib, (B.FLOAT16, 2))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _learned_build(lib, (B.STORAGE, 12))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _learned_build(lib, (B.FLOAT64, 8), (B.STORAGE, 16))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _learned_build(lib, (B.FLOAT64, 8), order=7)[0] == B.CUDA_ERROR_INVALID_VALUE
    assert lib.cccl_gb300_learned_sort_cleanup(None) == B.CUDA_ERROR_INVALID_VALUE


def test_learned_run_rejects_what_the_plain_run_rejects(lib):
    from cccl_gb300 import _bindings as B

    b = B.LearnedSortBuildResult()  # never built: every check below comes first
    it = B.pointer_iterator(0x1000, B.FLOAT32, 4)
    bad = B.pointer_iterator(0x1000, B.FLOAT32, 4)
    bad.type = B.ITERATOR
    nbytes, sel = C.c_size_t(0), C.c_int(-1)
    r = lib.cccl_gb300_learned_sort(b, None, C.byref(nbytes), bad, it, it, it, B.Op(), 16, 0, 32, False, C.byref(sel), None)
    assert r == B.CUDA_ERROR_UNKNOWN
    r = lib.cccl_gb300_learned_sort(b, None, None, it, it, it, it, B.Op(), 16, 0, 32, False, C.byref(sel), None)
    assert r == B.CUDA_ERROR_INVALID_VALUE
    op = B.Op()
    op.name = b"decomposer"
    r = lib.cccl_gb300_learned_sort(b, None, C.byref(nbytes), it, it, it, it, op, 16, 0, 32, False, C.byref(sel), None)
    assert r == B.CUDA_ERROR_NOT_SUPPORTED


# ---- segmented sort C ABI (c/parallel/include/cccl/c/segmented_sort.h), host side ----
def _seg_compile(lib, key_type, value_type=None, order=0, cc=(10, 3), offset_type=None):
    from cccl_gb300 import _bindings as B

    offset_type = offset_type or (B.INT32, 4)
    build = B.SegmentedSortBuildResult()
    keys = B.pointer_iterator(0x1000, key_type[0], key_type[1])
    vals = B.pointer_iterator(0x2000 if value_type else 0, *(value_type or (B.STORAGE, 4)))
    offs = B.pointer_iterator(0x3000, offset_type[0], offset_type[1])
    rc = lib.cccl_device_segmented_sort_compile(C.byref(build), order, keys, vals, offs, offs, cc[0], cc[1], None, None,
                                                None, None, None)
    return rc, build


def test_segmented_compile_serialize_round_trip(lib):
    from cccl_gb300 import _bindings as B

    rc, b = _seg_compile(lib, (B.FLOAT32, 4), (B.INT32, 4), order=B.DESCENDING)
    assert rc == B.CUDA_SUCCESS and b.cc == 103 and b.payload and b.payload_size > 0
    assert b.runtime_policy and b.partition_runtime_policy and b.order == B.DESCENDING
    assert not b.library
    buf, size = C.c_void_p(), C.c_size_t()
    assert lib.cccl_device_segmented_sort_serialize(C.byref(b), C.byref(buf), C.byref(size)) == 0
    b2 = B.SegmentedSortBuildResult()
    assert lib.cccl_device_segmented_sort_deserialize(C.byref(b2), buf, size) == 0
    assert b2.payload_size == b.payload_size and b2.order == b.order and b2.key_type.type == B.FLOAT32
    assert C.string_at(b2.payload, b2.payload_size) == C.string_at(b.payload, b.payload_size)
    assert C.string_at(b2.partition_runtime_policy, b2.partition_runtime_policy_size) == C.string_at(
        b.partition_runtime_policy, b.partition_runtime_policy_size)
    b3 = B.SegmentedSortBuildResult()
    assert lib.cccl_device_segmented_sort_deserialize(C.byref(b3), buf, 12) != 0
    lib.cccl_serialization_buffer_free(buf)
    for x in (b, b2):
        assert lib.cccl_device_segmented_sort_cleanup(C.byref(x)) == 0


def test_segmented_compile_rejections(lib):
    from cccl_gb300 import _bindings as B

    assert _seg_compile(lib, (B.FLOAT32, 4), cc=(9, 0))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    assert _seg_compile(lib, (B.STORAGE, 12))[0] == B.CUDA_ERROR_NOT_SUPPORTED
    # 16-byte values (the reference's custom_pair) are carried as 32-bit indices and gathered
    rc, b = _seg_compile(lib, (B.FLOAT32, 4), (B.STORAGE, 16))
    assert rc == B.CUDA_SUCCESS
    assert lib.cccl_device_segmented_sort_cleanup(C.byref(b)) == B.CUDA_SUCCESS
    assert _seg_compile(lib, (B.FLOAT32, 4), order=5)[0] == B.CUDA_ERROR_INVALID_VALUE
    assert lib.cccl_device_segmented_sort_cleanup(None) == B.CUDA_ERROR_INVALID_VALUE


@pytest.mark.parametrize("entry", ["cccl_device_segmented_sort", "cccl_gb300_segmented_radix_sort"])
def test_segmented_run_rejections(lib, entry):
    """Checks made before any device work (segmented_sort.cu:875-917 for the reference entry)."""
    from cccl_gb300 import _bindings as B

    rc, b = _seg_compile(lib, (B.FLOAT32, 4), (B.INT32, 4))
    assert rc == 0
    fn = getattr(lib, entry)
    it = B.pointer_iterator(0x1000, B.FLOAT32, 4)
    off = B.pointer_iterator(0x3000, B.INT32, 4)
    bad = B.pointer_iterator(0x1000, B.FLOAT32, 4)
    bad.type = B.ITERATOR
    narrow = B.pointer_iterator(0x3000, B.INT16, 2)
    bits = (0, 32) if entry.endswith("radix_sort") else ()
    nbytes, sel = C.c_size_t(0), C.c_int(-1)

    def call(k=it, o=off, e=off, selector=C.byref(sel)):
        return fn(b, None, C.byref(nbytes), k, it, it, it, 16, 2, o, e, *bits, False, selector, None)

    assert call(selector=None) == B.CUDA_ERROR_UNKNOWN  # null selector
    assert call(k=bad) == B.CUDA_ERROR_UNKNOWN  # keys must be pointers
    assert call(o=bad) == B.CUDA_ERROR_NOT_SUPPORTED  # offsets through iterators
    assert call(o=narrow, e=narrow) == B.CUDA_ERROR_INVALID_VALUE  # 16-bit offsets
    lib.cccl_device_segmented_sort_cleanup(C.byref(b))


# ---- segment offsets given as iterators (compiled at build time with NVRTC + nvJitLink) ----
from segments import nvrtc_available as _nvrtc_available, strided_offset_iterator  # noqa: E402

@pytest.mark.skipif(not _nvrtc_available(), reason="NVRTC is not installed")
@pytest.mark.parametrize("osize", [4, 8])
def test_segmented_compile_with_offset_iterators(lib, osize):
    from cccl_gb300 import _bindings as B

    otype = B.INT32 if osize == 4 else B.INT64
    begin = strided_offset_iterator(B, 0, 100, otype, osize, "b")
    end = strided_offset_iterator(B, 100, 100, otype, osize, "e")
    keys = B.pointer_iterator(0x1000, B.UINT32, 4)
    vals = B.pointer_iterator(0, B.STORAGE, 4)
    b = B.SegmentedSortBuildResult()
    rc = lib.cccl_device_segmented_sort_compile(C.byref(b), 0, keys, vals, begin, end, 10, 3, None, None, None, None,
                                                None)
    assert rc == B.CUDA_SUCCESS
    # the evaluation images travel with a serialized build
    buf, size = C.c_void_p(), C.c_size_t()
    assert lib.cccl_device_segmented_sort_serialize(C.byref(b), C.byref(buf), C.byref(size)) == 0
    plain_rc, plain = _seg_compile(lib, (B.UINT32, 4), offset_type=(otype, osize))
    pbuf, psize = C.c_void_p(), C.c_size_t()
    assert lib.cccl_device_segmented_sort_serialize(C.byref(plain), C.byref(pbuf), C.byref(psize)) == 0
    assert size.value > psize.value + 2 * 1000  # two linked cubins
    b2 = B.SegmentedSortBuildResult()
    assert lib.cccl_device_segmented_sort_deserialize(C.byref(b2), buf, size) == 0
    # a truncated blob is rejected without leaking the images read so far
    b3 = B.SegmentedSortBuildResult()
    assert lib.cccl_device_segmented_sort_deserialize(C.byref(b3), buf, size.value - 8) == B.CUDA_ERROR_INVALID_VALUE
    for x in (buf, pbuf):
        lib.cccl_serialization_buffer_free(x)
    for x in (b, b2, plain):
        assert lib.cccl_device_segmented_sort_cleanup(C.byref(x)) == 0


@pytest.mark.skipif(not _nvrtc_available(), reason="NVRTC is not installed")
def test_segmented_offset_iterator_rejections(lib):
    from cccl_gb300 import _bindings as B

    keys = B.pointer_iterator(0x1000, B.UINT32, 4)
    vals = B.pointer_iterator(0, B.STORAGE, 4)
    off = B.pointer_iterator(0x3000, B.INT64, 8)

    def compile_with(begin, end=off):
        b = B.SegmentedSortBuildResult()
        rc = lib.cccl_device_segmented_sort_compile(C.byref(b), 0, keys, vals, begin, end, 10, 3, None, None, None,
                                                    None, None)
        if rc == 0:
            lib.cccl_device_segmented_sort_cleanup(C.byref(b))
        return rc

    good = strided_offset_iterator(B, 0, 8)
    assert compile_with(good) == B.CUDA_SUCCESS  # an iterator beside a pointer
    broken = strided_offset_iterator(B, 0, 8)
    broken.dereference.code = b"this is not C++"
    broken.dereference.code_size = len(broken.dereference.code)
    broken._keep.append(broken.dereference.code)
    assert compile_with(broken) == B.CUDA_ERROR_INVALID_SOURCE
    assert compile_with(strided_offset_iterator(B, 0, 8, B.INT16, 2) if False else
                        B.code_iterator(b"\0" * 8, 8, B.FLOAT64, 8, ("a", "x"), ("d", "y"))) == B.CUDA_ERROR_NOT_SUPPORTED
    unnamed = strided_offset_iterator(B, 0, 8)
    unnamed.advance.name = b"bad name"
    unnamed._keep.append(unnamed.advance.name)
    assert compile_with(unnamed) == B.CUDA_ERROR_INVALID_VALUE


def test_merge_sorted_runs_argument_checks(lib):
    """cccl_gb300_merge_sorted_runs rejects, before touching the GPU: iterators that are not
    pointers, a missing size pointer, and run offsets that are missing, empty, not starting
    at 0 or decreasing."""
    from cccl_gb300 import _bindings as B

    rc, build = _compile(lib, (B.UINT64, 8), (B.UINT32, 4))
    assert rc == B.CUDA_SUCCESS
    keys = B.pointer_iterator(0x1000, B.UINT64, 8)
    vals = B.pointer_iterator(0x2000, B.UINT32, 4)
    temp = C.c_size_t(0)

    def call(offsets, num_runs, k=keys, tb=C.byref(temp)):
        arr = (C.c_uint64 * len(offsets))(*offsets) if offsets is not None else None
        return lib.cccl_gb300_merge_sorted_runs(build, None, tb, k, k, vals, vals, arr, num_runs, None)

    it = B.Iterator()
    it.type = 1  # an iterator kind other than a pointer
    assert call([0, 4, 8], 2, k=it) == B.CUDA_ERROR_UNKNOWN
    assert call([0, 4, 8], 2, tb=None) == B.CUDA_ERROR_INVALID_VALUE
    assert call(None, 2) == B.CUDA_ERROR_INVALID_VALUE
    assert call([0], 0) == B.CUDA_ERROR_INVALID_VALUE
    assert call([1, 4, 8], 2) == B.CUDA_ERROR_INVALID_VALUE
    assert call([0, 8, 4], 2) == B.CUDA_ERROR_INVALID_VALUE
    lib.cccl_device_radix_sort_cleanup(C.byref(build))
