"""Parity of the batched segmented sort (through cccl_device_segmented_sort) with the
oracle's restatement of cub::DeviceSegmentedSort, bit for bit: size classes, the sub-warp
merge network's NaN placement, +-0, empty and uncovered segments, both orders, DoubleBuffer
selectors, int32/int64 offsets."""

import numpy as np
import pytest

import inputs as I
from segments import edge_segments, lognormal_segments

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    import torch

    assert torch.cuda.is_available()
    return built_library


def _check(oracle, keys, values, b, e, desc=False, overwrite=False, offsets_dtype=np.int32):
    from gpu_util import gpu_seg_sort

    ko, vo, sel = gpu_seg_sort(keys, values, b, e, desc, overwrite, offsets_dtype)
    rk, rv = oracle.segmented_sort(keys, values, b, e, descending=desc, threads=8)
    bad = np.nonzero(ko.view(np.uint8).reshape(keys.size, -1).any(1) != rk.view(np.uint8).reshape(keys.size, -1).any(1))
    assert ko.tobytes() == rk.tobytes(), "keys differ from the oracle"
    if values is not None:
        assert vo.tobytes() == rv.tobytes(), "values differ from the oracle"
    return sel


def _nan_keys(dtype, n, rng, density=1 / 8):
    return I.with_specials(I.finite_floats(dtype, n, rng), rng, density)


EDGE_SIZES = [1, 2, 3, 4, 17, 18, 19, 20, 111, 112, 113, 200, 511, 512, 513, 2047, 2048, 2049, 8191, 8192, 8193, 20000,
              100_000]


@pytest.mark.parametrize("many", [False, True], ids=["fallback", "partitioned"])
@pytest.mark.parametrize("desc", [False, True])
def test_size_class_edges_with_nans(oracle, many, desc):
    rng = np.random.default_rng(7 + many + 2 * desc)
    sizes = EDGE_SIZES * (30 if many else 1)  # > 500 segments switches on partitioning
    b, e, n = edge_segments(sizes, gap=0)
    k = _nan_keys(np.float32, n, rng)
    v = I.index_values(n)
    _check(oracle, k, v, b, e, desc)


@pytest.mark.parametrize("desc", [False, True])
@pytest.mark.parametrize("npairs", [False, True])
def test_lognormal_batch_f32(oracle, desc, npairs):
    """The batched configuration at 2^22 keys: lognormal(5, 2.5) lengths, 5% empty,
    N(0,1) keys with 0.1% +-0 and NaN."""
    rng = np.random.default_rng(2025 + desc)
    b, e = lognormal_segments(rng, 1 << 22)
    n = int(e[-1])
    k = I.with_specials(rng.standard_normal(n).astype(np.float32), rng, 1e-3)
    v = rng.integers(-(2**31), 2**31 - 1, size=n, dtype=np.int32) if npairs else None
    _check(oracle, k, v, b, e, desc)


@pytest.mark.parametrize(
    "dtype,vdtype", [(np.int32, np.uint32), (np.uint64, np.uint64), (np.float64, np.int64), (np.float16, np.uint32),
                     (np.uint8, None), (np.int16, np.uint32), (np.int64, None), (np.float32, None)]
)
def test_key_types(oracle, dtype, vdtype):
    rng = np.random.default_rng(np.dtype(dtype).itemsize * 11 + (vdtype is None))
    b, e = lognormal_segments(rng, 600_000, mu=4.0, sigma=2.0)
    n = int(e[-1])
    k = _nan_keys(dtype, n, rng, 1 / 64) if np.dtype(dtype).kind == "f" else I.entropy_reduced(dtype, n, rng, 2)
    v = None if vdtype is None else I.uniform_bits(vdtype, n, rng)
    for desc in (False, True):
        _check(oracle, k, v, b, e, desc)


@pytest.mark.parametrize("dtype", [np.float32, np.uint64, np.uint8, np.float16])
def test_overwrite_selector_matches_cub(oracle, dtype):
    """With a DoubleBuffer the result lands where CUB's 6-bit (4-bit for 1-byte keys) radix
    pass count puts it: selector = passes & 1 (dispatch_segmented_sort.cuh:730-739)."""
    rng = np.random.default_rng(3)
    b, e, n = edge_segments([5, 100, 3000, 9000, 70000, 1], gap=3)
    k = _nan_keys(dtype, n, rng) if np.dtype(dtype).kind == "f" else I.uniform_bits(dtype, n, rng)
    v = I.index_values(n)
    kb = np.dtype(dtype).itemsize
    expect = (-(-8 * kb // (6 if kb > 1 else 4))) & 1
    sel = _check(oracle, k, v, b, e, overwrite=True)
    assert sel == expect


def test_empty_reversed_and_uncovered_segments(oracle):
    rng = np.random.default_rng(9)
    n = 50_000
    k = _nan_keys(np.float32, n, rng)
    v = I.index_values(n)
    b = np.array([0, 10, 10, 500, 400, 20000, 45000], dtype=np.int64)
    e = np.array([5, 10, 300, 499, 300, 44000, 50000], dtype=np.int64)  # empty, reversed (empty), gaps
    _check(oracle, k, v, b, e, offsets_dtype=np.int64)
    _check(oracle, k, v, b, e, desc=True, offsets_dtype=np.int32)


def test_few_huge_segments(oracle):
    """Device class: segments of millions of keys share the batched onesweep passes."""
    rng = np.random.default_rng(11)
    b, e, n = edge_segments([3_000_000, 1_500_001, 40_000, 2_000_000], gap=7)
    k = I.with_specials(rng.standard_normal(n).astype(np.float32), rng, 1e-3)
    v = I.index_values(n)
    _check(oracle, k, v, b, e)
    _check(oracle, k, v, b, e, desc=True, overwrite=True)


def test_no_segments_and_no_items():
    from gpu_util import gpu_seg_sort

    k = np.arange(10, dtype=np.float32)
    ko, _, _ = gpu_seg_sort(k, None, np.array([], dtype=np.int64), np.array([], dtype=np.int64))
    assert ko.tobytes() == k.tobytes()


# ---- DeviceSegmentedRadixSort semantics (cccl_gb300_segmented_radix_sort) ----
def _radix_reference(oracle, keys, values, b, e, bits, desc):
    """Per segment, the plain radix oracle over the bit window; positions outside every
    segment keep the input."""
    rk, rv = keys.copy(), (values.copy() if values is not None else None)
    for lo, hi in zip(b, e):
        if hi > lo:
            sk, sv = oracle.radix_sort(keys[lo:hi], None if values is None else values[lo:hi], bits[0], bits[1], desc,
                                       threads=1)
            rk[lo:hi] = sk
            if values is not None:
                rv[lo:hi] = sv
    return rk, rv


@pytest.mark.parametrize("bits", [(0, None), (3, 29), (8, 8)], ids=["full", "window", "empty"])
@pytest.mark.parametrize("desc", [False, True])
@pytest.mark.parametrize("overwrite", [False, True], ids=["out", "doublebuffer"])
def test_segmented_radix_sort(oracle, bits, desc, overwrite):
    from gpu_util import gpu_seg_sort

    rng = np.random.default_rng(31 + desc + 2 * overwrite)
    b, e = edge_segments([1, 17, 112, 113, 256, 257, 512, 513, 2048, 2049, 8193, 30000, 5, 0, 700], gap=3)[:2]
    n = int(e[-1]) + 5
    k = I.with_specials(I.finite_floats(np.float32, n, rng), rng, 1 / 16)
    v = I.index_values(n)
    window = (bits[0], 32 if bits[1] is None else bits[1])
    ko, vo, sel = gpu_seg_sort(k, v, b, e, desc, overwrite, radix_bits=window)
    rk, rv = _radix_reference(oracle, k, v, b, e, window, desc)
    assert ko.tobytes() == rk.tobytes() and vo.tobytes() == rv.tobytes()
    if overwrite:
        # DeviceSegmentedRadixSort: selector = max(ceil(bits / 6), 1) & 1; no bits and a
        # DoubleBuffer: nothing runs (dispatch_segmented_radix_sort.cuh:541)
        expect = 0 if window[0] == window[1] else max(-(-(window[1] - window[0]) // 6), 1) % 2
        assert sel == expect


@pytest.mark.parametrize("osize", [4, 8])
@pytest.mark.parametrize("seg_size", [1000, 70_000])
def test_offsets_through_iterators(oracle, osize, seg_size):
    """Segment offsets given as iterators compiled from C++ source, the form the reference's
    test sketches with its step-counting iterator (c/parallel/test/test_segmented_sort.cpp:
    230-268): begin = i * size, end = (i + 1) * size, the end iterator naming the begin
    iterator's operations without code. Results equal the pointer-offset sort's."""
    import torch
    from segments import nvrtc_available, strided_offset_iterator

    import cccl_gb300 as cg
    from cccl_gb300 import _bindings as B

    if not nvrtc_available():
        pytest.skip("NVRTC is not installed")
    rng = np.random.default_rng(seg_size + osize)
    nseg = max(4, 4_000_000 // seg_size)
    n = nseg * seg_size
    k = _nan_keys(np.float32, n, rng)
    v = I.index_values(n)
    otype = B.INT32 if osize == 4 else B.INT64
    begin = strided_offset_iterator(B, 0, seg_size, otype, osize, "off")
    end = strided_offset_iterator(B, seg_size, seg_size, otype, osize, "off", with_code=False)
    dk = torch.from_numpy(k).cuda()
    dv = torch.from_numpy(v).cuda()
    ok = torch.empty_like(dk)
    ov = torch.empty_like(dv)
    cg.segmented_sort(d_in_keys=dk, d_out_keys=ok, d_in_values=dv, d_out_values=ov, num_items=n,
                      num_segments=nseg, start_offsets_in=begin, end_offsets_in=end,
                      order=cg.SortOrder.ASCENDING)
    torch.cuda.synchronize()
    b = np.arange(nseg, dtype=np.int64) * seg_size
    rk, rv = oracle.segmented_sort(k, v, b, b + seg_size, descending=False, threads=8)
    assert ok.cpu().numpy().tobytes() == rk.tobytes(), "keys differ from the oracle"
    assert ov.cpu().numpy().tobytes() == rv.tobytes(), "values differ from the oracle"


def test_iterator_beside_pointer_offsets(oracle):
    """Begin offsets as a device array, end offsets as an iterator (and the build reused with
    both as arrays)."""
    import torch
    from segments import nvrtc_available, strided_offset_iterator

    import cccl_gb300 as cg
    from cccl_gb300 import _bindings as B

    if not nvrtc_available():
        pytest.skip("NVRTC is not installed")
    rng = np.random.default_rng(99)
    seg, nseg = 333, 3000
    n = seg * nseg
    k = rng.integers(0, 2**32, n, dtype=np.uint32)
    b = np.arange(nseg, dtype=np.int64) * seg
    db = torch.from_numpy(b).cuda()
    de = torch.from_numpy(b + seg).cuda()
    end = strided_offset_iterator(B, seg, seg, B.INT64, 8, "endit")
    dk = torch.from_numpy(k.view(np.int32)).cuda()
    ok = torch.empty_like(dk)
    sorter = cg.make_segmented_sort(d_in_keys=dk, d_out_keys=ok, start_offsets_in=db, end_offsets_in=end,
                                    order=cg.SortOrder.DESCENDING)
    rk, _ = oracle.segmented_sort(k.view(np.int32), None, b, b + seg, descending=True, threads=8)
    for e_arg in (end, de):
        ok.zero_()
        nbytes = sorter(temp_storage=None, d_in_keys=dk, d_out_keys=ok, d_in_values=None, d_out_values=None,
                        num_items=n, num_segments=nseg, start_offsets_in=db, end_offsets_in=e_arg)
        tmp = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
        sorter(temp_storage=tmp, d_in_keys=dk, d_out_keys=ok, d_in_values=None, d_out_values=None, num_items=n,
               num_segments=nseg, start_offsets_in=db, end_offsets_in=e_arg)
        torch.cuda.synchronize()
        assert ok.cpu().numpy().tobytes() == rk.tobytes()
