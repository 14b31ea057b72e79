"""Parity of the GPU radix sort (through the C ABI) with the oracle and the reference's
golden vectors, plus the reference's edge cases (cub/test/catch2_test_device_radix_sort_keys.cu,
..._pairs.cu, c/parallel/test/test_radix_sort.cpp). Bit-exact everywhere."""

import glob
from pathlib import Path

import numpy as np
import pytest

import inputs as I

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(str(Path(__file__).parent / "golden" / "radix_*.npz")))
SINGLE_TILE_4B = 4864  # CUB's single-tile cut for 4-byte keys


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    import torch

    assert torch.cuda.is_available()
    return built_library


def _check(oracle, keys, values=None, b=0, e=None, desc=False, overwrite=False):
    from gpu_util import gpu_sort

    ko, vo, sel = gpu_sort(keys, values, b, e, desc, overwrite)
    rk, rv = oracle.radix_sort(keys, values, b, e, desc, threads=4)
    assert ko.tobytes() == rk.tobytes(), "keys differ from the oracle"
    if values is not None:
        assert vo.tobytes() == rv.tobytes(), "values differ from the oracle"
    return sel


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: Path(p).stem)
def test_golden_vectors(path):
    from gpu_util import gpu_sort

    g = np.load(path)
    vals = g["values_in"] if "values_in" in g else None
    ko, vo, _ = gpu_sort(g["keys_in"], vals, int(g["begin_bit"]), int(g["end_bit"]), bool(g["descending"]))
    assert ko.tobytes() == g["keys_out"].tobytes()
    if vals is not None:
        assert vo.tobytes() == g["values_out"].tobytes()


KEY_TYPES = [np.uint8, np.int8, np.uint16, np.int16, np.float16, np.uint32, np.int32, np.float32, np.uint64,
             np.int64, np.float64]


@pytest.mark.parametrize("n", [1, 17, SINGLE_TILE_4B, SINGLE_TILE_4B + 1, 300_001])
@pytest.mark.parametrize("dtype", KEY_TYPES, ids=lambda d: np.dtype(d).name)
def test_keys_and_pairs_vs_oracle(oracle, dtype, n):
    rng = np.random.default_rng(n * 31 + np.dtype(dtype).itemsize)
    if np.dtype(dtype).kind == "f":
        k = I.with_specials(I.finite_floats(dtype, n, rng), rng, 1 / 16)
    else:
        k = I.uniform_bits(dtype, n, rng)
    for desc in (False, True):
        _check(oracle, k, None, desc=desc)
        _check(oracle, k, I.index_values(n), desc=desc)


@pytest.mark.parametrize("vbytes", [1, 2, 4, 8, 16])
def test_value_widths(oracle, vbytes):
    rng = np.random.default_rng(vbytes)
    n = 200_003
    k = I.entropy_reduced(np.uint32, n, rng, 3)
    v = rng.integers(0, 255, size=n * vbytes, dtype=np.uint8).view(f"V{vbytes}") if vbytes == 16 else \
        I.uniform_bits({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[vbytes], n, rng)
    if vbytes == 16:
        from gpu_util import gpu_sort

        ko, vo, _ = gpu_sort(k, v.view(np.uint8).reshape(n, 16).view(np.complex128).reshape(n))
        perm = oracle.radix_permutation(k)
        assert ko.tobytes() == k[perm].tobytes()
        assert vo.tobytes() == v[perm].tobytes()
    else:
        _check(oracle, k, v)


@pytest.mark.parametrize(
    "dtype,b,e", [(np.uint32, 0, 5), (np.uint32, 3, 27), (np.int32, 16, 32), (np.float32, 0, 31), (np.uint64, 8, 40),
                  (np.float64, 1, 63), (np.uint16, 4, 13), (np.uint64, 60, 64)]
)
def test_bit_windows(oracle, dtype, b, e):
    rng = np.random.default_rng(b * 100 + e)
    n = 123_457
    k = I.uniform_bits(dtype, n, rng)
    for desc in (False, True):
        _check(oracle, k, I.index_values(n), b, e, desc)


@pytest.mark.parametrize("ands", [1, 3, 9, 15])
def test_entropy_reduction(oracle, ands):
    rng = np.random.default_rng(ands)
    k = I.entropy_reduced(np.uint64, 500_000, rng, ands)
    _check(oracle, k, I.index_values(k.size))
    _check(oracle, k, I.index_values(k.size), desc=True)


def test_negative_zero_bitwise(oracle):
    rng = np.random.default_rng(11)
    for dtype in (np.float32, np.float64, np.float16):
        k = I.finite_floats(dtype, 100_000, rng)
        k[rng.choice(k.size, k.size // 128, replace=False)] = dtype(-0.0)
        k[rng.choice(k.size, k.size // 128, replace=False)] = dtype(0.0)
        for desc in (False, True):
            _check(oracle, k, I.index_values(k.size), desc=desc)


def test_uniform_values(oracle):
    for dtype in (np.uint32, np.float64, np.int8):
        k = np.full(100_000, 5, dtype=dtype)
        _check(oracle, k, I.index_values(k.size))
        _check(oracle, k, I.index_values(k.size), desc=True)


@pytest.mark.parametrize("n", [100, SINGLE_TILE_4B + 1, 1_000_000])
@pytest.mark.parametrize("bits", [(0, 32), (0, 8), (0, 16), (4, 28)])
def test_double_buffer_selector(oracle, n, bits):
    """With is_overwrite_okay the result is wherever the selector points; the selector
    equals CUB's: 1 for the single-tile path, passes & 1 otherwise."""
    rng = np.random.default_rng(n)
    k = I.uniform_bits(np.uint32, n, rng)
    sel = _check(oracle, k, I.index_values(n), bits[0], bits[1], overwrite=True)
    passes = -(-(bits[1] - bits[0]) // 8)
    expect = 1 if n <= SINGLE_TILE_4B else passes & 1
    assert sel == expect


def test_begin_equals_end(oracle):
    from gpu_util import gpu_sort

    k = I.uniform_bits(np.uint32, 10_000, np.random.default_rng(0))
    ko, _, _ = gpu_sort(k, None, 7, 7)  # copy
    assert ko.tobytes() == k.tobytes()
    ko, _, sel = gpu_sort(k, None, 7, 7, overwrite=True)  # nothing to do, data stays put
    assert sel == 0 and ko.tobytes() == k.tobytes()


def test_empty_input():
    import torch

    from cccl_gb300 import SortOrder, make_radix_sort

    k = torch.empty(0, dtype=torch.int32, device="cuda")
    s = make_radix_sort(d_in_keys=k, d_out_keys=k, d_in_values=None, d_out_values=None, order=SortOrder.ASCENDING)
    assert s(temp_storage=None, d_in_keys=k, d_out_keys=k, d_in_values=None, d_out_values=None, num_items=0) == 1


def test_c_abi_reference_cases(oracle):
    """c/parallel/test/test_radix_sort.cpp:180-330: uint8/int16/uint32/half/double keys,
    float items, descending and overwrite variants, 500 / 1e6 / 2e6 / random sizes."""
    rng = np.random.default_rng(2024)
    params = [(np.uint8, False, False), (np.int16, True, False), (np.uint32, False, True), (np.float16, True, True),
              (np.float64, False, False)]
    for dtype, desc, ow in params:
        for n in (500, 1_000_000, 2_000_000, int(rng.integers(1, 1_000_000))):
            if np.dtype(dtype).kind == "f":
                k = rng.permutation(n).astype(dtype)
            else:
                k = (rng.permutation(n) % (np.iinfo(dtype).max + 1)).astype(dtype)
            items = k.astype(np.float32)
            _check(oracle, k, items, desc=desc, overwrite=ow)


def test_status_word_clean_after_sort():
    """The exported status query reads word 0 of the call's temp storage: no error after a
    normal sort (onesweep path), and none after a single-tile sort that reuses the buffer."""
    import torch

    from cccl_gb300 import _bindings as B, sort_status
    from gpu_util import gpu_sort

    k = I.uniform_bits(np.uint32, 3_000_000, np.random.default_rng(5))
    _, _, _, temp = gpu_sort(k, None, return_temp=True)
    rc, bits = sort_status(temp)
    assert (rc, bits) == (B.CUDA_SUCCESS, 0)
    temp.view(torch.int32)[0] = B.STATUS_WAIT_TIMEOUT  # a stale word from an earlier call ...
    from cccl_gb300 import SortOrder, make_radix_sort
    from gpu_util import to_dev

    small = to_dev(k[:1000])
    out = torch.empty_like(small)
    s = make_radix_sort(d_in_keys=small, d_out_keys=out, d_in_values=None, d_out_values=None,
                        order=SortOrder.ASCENDING)
    s(temp_storage=temp, d_in_keys=small, d_out_keys=out, d_in_values=None, d_out_values=None, num_items=1000)
    assert sort_status(temp) == (B.CUDA_SUCCESS, 0)  # ... is cleared by the next call


def test_wait_timeout_is_reported_and_the_gpu_stays_usable(oracle):
    """The failure path of the bounded look-back wait, without a GPU fault: one tile of every
    digit pass withholds its counts (a test hook of the loaded kernels), the wait limit is
    1 ms, so its successors' waits run out. The sort returns, the status query reports
    CUDA_ERROR_LAUNCH_TIMEOUT, and the next sort on the same GPU and build is bit-exact."""
    import ctypes as C

    import torch

    from cccl_gb300 import _bindings as B, SortOrder, make_radix_sort, sort_status
    from gpu_util import from_dev, to_dev

    lib = B.load_library()
    rng = np.random.default_rng(99)
    n = 1 << 22
    k = I.uniform_bits(np.uint32, n, rng)
    v = I.index_values(n)
    kd, vd = to_dev(k), to_dev(v)
    ko, vo = torch.empty_like(kd), torch.empty_like(vd)
    args = dict(d_in_keys=kd, d_out_keys=ko, d_in_values=vd, d_out_values=vo)
    s = make_radix_sort(order=SortOrder.ASCENDING, **args)
    temp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
    library = C.c_void_p(s.build_result.library)
    assert lib.cccl_gb300_testing_set_wait_fault(library, 5, 1_000_000) == B.CUDA_SUCCESS
    try:
        s(temp_storage=temp, num_items=n, **args)
        rc, bits = sort_status(temp)
        assert rc == B.CUDA_ERROR_LAUNCH_TIMEOUT and bits & B.STATUS_WAIT_TIMEOUT
        assert sort_status(temp) == (B.CUDA_SUCCESS, 0)  # read and cleared
    finally:
        assert lib.cccl_gb300_testing_set_wait_fault(library, 0xFFFFFFFF, 1_000_000_000) == B.CUDA_SUCCESS
    s(temp_storage=temp, num_items=n, **args)
    assert sort_status(temp) == (B.CUDA_SUCCESS, 0)
    rk, rv = oracle.radix_sort(k, v, threads=4)
    assert from_dev(ko, np.uint32).tobytes() == rk.tobytes()
    assert from_dev(vo, np.uint32).tobytes() == rv.tobytes()


def test_large_full_size_properties():
    """2^28 keys (the benchmark size): sorted, stable and a permutation, checked on the
    GPU with independent torch operations."""
    import torch

    from cccl_gb300 import SortOrder, make_radix_sort

    n = 1 << 28
    g = torch.Generator(device="cuda").manual_seed(3)
    k = torch.randint(0, 1 << 20, (n,), device="cuda", dtype=torch.int32, generator=g)
    v = torch.arange(n, device="cuda", dtype=torch.int32)
    ko, vo = torch.empty_like(k), torch.empty_like(v)
    s = make_radix_sort(d_in_keys=k, d_out_keys=ko, d_in_values=v, d_out_values=vo, order=SortOrder.ASCENDING)
    nb = s(temp_storage=None, d_in_keys=k, d_out_keys=ko, d_in_values=v, d_out_values=vo, num_items=n)
    t = torch.empty(nb, dtype=torch.uint8, device="cuda")
    s(temp_storage=t, d_in_keys=k, d_out_keys=ko, d_in_values=v, d_out_values=vo, num_items=n)
    torch.cuda.synchronize()
    assert bool((ko[1:] >= ko[:-1]).all())
    eq = ko[1:] == ko[:-1]
    assert bool((vo[1:][eq] > vo[:-1][eq]).all())  # stable: equal keys keep index order
    assert bool((k[vo.long()] == ko).all())  # values are the source positions of the keys
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt.index_add_(0, vo.long(), torch.ones_like(vo))
    assert bool((cnt == 1).all())


@pytest.mark.parametrize("offset", [1, 3])
def test_unaligned_buffers_use_the_fallback_pass(oracle, offset):
    """Buffers that are not 16-byte aligned take the CTA-per-tile pass kernel; the temp size
    queried for an aligned buffer of the same length must still be enough."""
    import torch

    from cccl_gb300 import SortOrder, make_radix_sort
    from gpu_util import from_dev, to_dev

    rng = np.random.default_rng(offset)
    n = 700_001
    k = I.uniform_bits(np.uint32, n + offset, rng)
    v = I.index_values(n + offset)
    kd, vd = to_dev(k), to_dev(v)
    ki, vi = kd[offset:], vd[offset:]
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    s = make_radix_sort(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo, order=SortOrder.ASCENDING)
    aligned = torch.empty(n, dtype=ki.dtype, device="cuda")
    nbytes = s(temp_storage=None, d_in_keys=aligned, d_out_keys=aligned, d_in_values=vi, d_out_values=vo, num_items=n)
    temp = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s(temp_storage=temp, d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo, num_items=n)
    torch.cuda.synchronize()
    rk, rv = oracle.radix_sort(k[offset:], v[offset:])
    assert from_dev(ko, np.uint32).tobytes() == rk.tobytes()
    assert from_dev(vo, np.uint32).tobytes() == rv.tobytes()


@pytest.mark.parametrize("case", ["top_digit_only", "low_digits_all_ones", "constant_then_random"])
@pytest.mark.parametrize("dtype", [np.uint32, np.uint64, np.float32], ids=lambda d: np.dtype(d).name)
def test_single_digit_tiles(oracle, dtype, case):
    """Tiles whose keys all share the pass's digit take the direct-copy path; the digit may
    equal the padding keys' digit of a partial tile (all ones)."""
    n = 3_000_017
    rng = np.random.default_rng(17)
    u = I.UINT_OF[np.dtype(dtype).itemsize]
    bits = np.dtype(dtype).itemsize * 8
    if case == "top_digit_only":
        k = (rng.integers(0, 256, n).astype(u) << u(bits - 8)) | u(0x5A)
    elif case == "low_digits_all_ones":
        low = (u(1) << u(bits - 8)) - u(1)
        k = (rng.integers(0, 4, n).astype(u) << u(bits - 8)) | low
    else:
        k = I.uniform_bits(u, n, rng)
        k[: n // 2] = u(0x1234)
    k = k.view(dtype)
    for desc in (False, True):
        _check(oracle, k, I.index_values(n), desc=desc)


@pytest.mark.parametrize("n", [2000, 300_001], ids=["single_tile", "onesweep"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.float16], ids=lambda d: np.dtype(d).name)
def test_descending_bit_window_zeros(oracle, dtype, n):
    """Descending float sorts under a bit window: CUB's single tile folds -0.0 into +0.0,
    its onesweep passes fold +0.0 into -0.0 (cub/cub/block/radix_rank_sort_operations.cuh:43-56),
    and the two orders differ only here."""
    from gpu_util import gpu_sort

    rng = np.random.default_rng(n + np.dtype(dtype).itemsize)
    k = I.with_specials(I.finite_floats(dtype, n, rng), rng, 1 / 8)
    bits = np.dtype(dtype).itemsize * 8
    for b, e in ((0, bits - 3), (3, bits - 5)):
        ko, vo, _ = gpu_sort(k, I.index_values(n), b, e, True)
        # 2000 pairs fit CUB's single tile for every key width here (>= 2304 with u32 values)
        rk, rv = oracle.radix_sort(k, I.index_values(n), b, e, True, threads=4, onesweep_zeros=n > 2304)
        assert ko.tobytes() == rk.tobytes() and vo.tobytes() == rv.tobytes()


def _trivial_pass_keys(case, n, rng):
    """Keys whose digit is the same for every key in some 8-bit passes, and the passes that
    are not: (keys, begin_bit, end_bit)."""
    if case == "u64_low_half":  # the top four bytes are zero: passes 4-7 skip
        return I.uniform_bits(np.uint64, n, rng) >> np.uint64(32), 0, 64
    if case == "u32_byte1_only":  # one pass runs; the parity asks for one more
        return (rng.integers(0, 256, n).astype(np.uint32) << np.uint32(8)) | np.uint32(0x3C0000A5), 0, 32
    if case == "u16_high_only":
        return rng.integers(0, 256, n).astype(np.uint16) << np.uint16(8), 0, 16
    if case == "u8_all_equal":
        return np.full(n, 0x5A, np.uint8), 0, 8
    if case == "u32_all_equal":
        return np.full(n, 0xDEADBEEF, np.uint32), 0, 32
    if case == "f64_all_equal":
        return np.full(n, -2.5, np.float64), 0, 64
    if case == "f32_signed_zeros":  # +0.0 and -0.0 fold to one digit in every pass
        return np.where(rng.random(n) < 0.5, np.float32(0.0), np.float32(-0.0)).astype(np.float32), 0, 32
    if case == "f32_small_integers":  # the low mantissa bytes are zero
        return rng.integers(-1000, 1000, n).astype(np.float32), 0, 32
    if case == "u64_window_constant_low":  # bits 8..15 constant inside the window 8..40
        k = I.uniform_bits(np.uint64, n, rng) & ~np.uint64(0xFF00)
        return k | np.uint64(0x7700), 8, 40
    raise ValueError(case)


@pytest.mark.parametrize("overwrite", [False, True], ids=["pointers", "double_buffer"])
@pytest.mark.parametrize(
    "case",
    ["u64_low_half", "u32_byte1_only", "u16_high_only", "u8_all_equal", "u32_all_equal", "f64_all_equal",
     "f32_signed_zeros", "f32_small_integers", "u64_window_constant_low"],
)
def test_trivial_passes_skipped(oracle, case, overwrite):
    """Digit passes whose digit is the same for every key are skipped (the histogram's pass
    plan); the result, the stable order of equal keys and the DoubleBuffer selector stay
    CUB's, including when no pass runs and when the parity makes one skippable pass run."""
    from gpu_util import gpu_sort

    rng = np.random.default_rng(len(case) * 101 + overwrite)
    for n in (300_001, 1_500_007):  # several tiles per CTA in the larger
        k, b, e = _trivial_pass_keys(case, n, rng)
        passes = -(-(e - b) // 8)
        for desc in (False, True):
            for vals in (None, I.index_values(n)):
                ko, vo, sel = gpu_sort(k, vals, b, e, desc, overwrite)
                rk, rv = oracle.radix_sort(k, vals, b, e, desc, threads=4)
                assert ko.tobytes() == rk.tobytes(), (case, n, desc, vals is None)
                if vals is not None:
                    assert vo.tobytes() == rv.tobytes(), (case, n, desc)
                if overwrite:
                    assert sel == passes & 1
