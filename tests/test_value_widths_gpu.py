"""Values of any width through the C ABI (the reference's custom value types: a struct is a
CCCL_STORAGE value of its size, c/parallel/test/test_segmented_sort.cpp:455-591 uses
`struct custom_pair { int key; size_t value; }`). Widths the kernels do not carry (the radix
sort carries 1, 2, 4, 8 and 16 bytes, the segmented sort 4 and 8) are sorted as 32-bit
indices and gathered. Checked against the oracle's stable permutation, with both buffer
modes and both orders; positions outside every segment stay untouched."""

import ctypes as C

import numpy as np
import pytest

import inputs as I

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built_library):
    import torch

    from cccl_gb300 import _bindings as B

    assert torch.cuda.is_available()
    return B.load_library()


def _raw(nbytes, fill=None, seed=0):
    """Device buffer of nbytes (uint8), random or filled."""
    import torch

    if fill is not None:
        return torch.full((nbytes,), fill, dtype=torch.uint8, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randint(0, 256, (nbytes,), dtype=torch.uint8, device="cuda", generator=g)


def _key_code(dtype):
    from oracle import pyoracle

    return pyoracle.TYPE_CODES[np.dtype(dtype)]


def _run_radix(lib, keys, width, align, desc, overwrite):
    import torch

    from cccl_gb300 import _bindings as B
    from gpu_util import from_dev, to_dev

    n = keys.size
    kb = keys.dtype.itemsize
    kin, kout = to_dev(keys), to_dev(keys)
    vin = _raw(n * width, seed=n + width)
    vout = _raw(n * width, fill=0x5A)
    vals0 = vin.cpu().numpy().reshape(n, width).copy()
    kit = lambda t: B.pointer_iterator(t.data_ptr(), _key_code(keys.dtype), kb)
    vit = lambda t: B.pointer_iterator(t.data_ptr(), B.STORAGE, width, align)
    build = B.RadixSortBuildResult()
    major, minor = torch.cuda.get_device_capability()
    rc = lib.cccl_device_radix_sort_build(C.byref(build), int(desc), kit(kin), vit(vin), B.no_op(), b"", major, minor,
                                          None, None, None, None)
    assert rc == 0
    try:
        nbytes, sel = C.c_size_t(0), C.c_int(-1)
        stream = torch.cuda.current_stream().cuda_stream
        args = (kit(kin), kit(kout), vit(vin), vit(vout), B.no_op(), n, 0, 8 * kb, overwrite, C.byref(sel), stream)
        assert lib.cccl_device_radix_sort(build, None, C.byref(nbytes), *args) == 0
        temp = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device="cuda")
        assert lib.cccl_device_radix_sort(build, temp.data_ptr(), C.byref(nbytes), *args) == 0
        torch.cuda.synchronize()
    finally:
        lib.cccl_device_radix_sort_cleanup(C.byref(build))
    s = sel.value if overwrite else 1
    ko = from_dev([kin, kout][s], keys.dtype)
    vo = [vin, vout][s].cpu().numpy().reshape(n, width)
    return ko, vo, vals0


@pytest.mark.parametrize("width,align", [(3, 1), (12, 4), (24, 8), (32, 16), (6, 2)])
@pytest.mark.parametrize("n", [1000, 300_001])
def test_radix_custom_value_widths(lib, oracle, width, align, n):
    rng = np.random.default_rng(width * 1000 + n)
    for dtype in (np.uint32, np.float64):
        keys = I.entropy_reduced(dtype, n, rng, 3) if dtype == np.uint32 else I.with_specials(
            I.finite_floats(dtype, n, rng), rng, 1 / 64)
        for desc in (False, True):
            for overwrite in (False, True):
                ko, vo, v0 = _run_radix(lib, keys, width, align, desc, overwrite)
                perm = oracle.radix_permutation(keys, descending=desc)
                assert ko.tobytes() == keys[perm].tobytes(), (dtype, desc, overwrite)
                assert vo.tobytes() == v0[perm].tobytes(), (dtype, desc, overwrite)


def _run_segmented(lib, keys, b, e, width, align, desc, overwrite):
    import torch

    from cccl_gb300 import _bindings as B
    from gpu_util import from_dev, to_dev

    n = keys.size
    kb = keys.dtype.itemsize
    kin, kout = to_dev(keys), to_dev(keys)
    vin = _raw(n * width, seed=n + width + 1)
    vout = vin.clone()  # positions outside every segment compare equal
    vals0 = vin.cpu().numpy().reshape(n, width).copy()
    bo = torch.from_numpy(np.ascontiguousarray(b, dtype=np.int64)).cuda()
    eo = torch.from_numpy(np.ascontiguousarray(e, dtype=np.int64)).cuda()
    kit = lambda t: B.pointer_iterator(t.data_ptr(), _key_code(keys.dtype), kb)
    vit = lambda t: B.pointer_iterator(t.data_ptr(), B.STORAGE, width, align)
    oit = lambda t: B.pointer_iterator(t.data_ptr(), B.INT64, 8)
    build = B.SegmentedSortBuildResult()
    major, minor = torch.cuda.get_device_capability()
    rc = lib.cccl_device_segmented_sort_build(C.byref(build), int(desc), kit(kin), vit(vin), oit(bo), oit(eo), major,
                                              minor, None, None, None, None)
    assert rc == 0
    try:
        nbytes, sel = C.c_size_t(0), C.c_int(-1)
        stream = torch.cuda.current_stream().cuda_stream
        args = (kit(kin), kit(kout), vit(vin), vit(vout), n, len(b), oit(bo), oit(eo), overwrite, C.byref(sel), stream)
        assert lib.cccl_device_segmented_sort(build, None, C.byref(nbytes), *args) == 0
        temp = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device="cuda")
        assert lib.cccl_device_segmented_sort(build, temp.data_ptr(), C.byref(nbytes), *args) == 0
        torch.cuda.synchronize()
    finally:
        lib.cccl_device_segmented_sort_cleanup(C.byref(build))
    s = sel.value if overwrite else 1
    ko = from_dev([kin, kout][s], keys.dtype)
    vo = [vin, vout][s].cpu().numpy().reshape(n, width)
    return ko, vo, vals0


@pytest.mark.parametrize("width,align", [(16, 8), (12, 4), (2, 2), (1, 1), (40, 8)])
def test_segmented_custom_value_widths(lib, oracle, width, align):
    """width 16 / align 8 is the reference's custom_pair {int, size_t}; segments of every
    size class, with gaps between some segments (positions outside every segment)."""
    rng = np.random.default_rng(width)
    sizes = np.concatenate([rng.integers(0, 20, 300), rng.integers(20, 3000, 40), [20000, 70000]])
    rng.shuffle(sizes)
    gaps = rng.integers(0, 3, sizes.size) * (rng.random(sizes.size) < 0.2)
    b = np.cumsum(np.concatenate([[0], (sizes + gaps)[:-1]]))
    e = b + sizes
    n = int(e[-1] + 5)
    for dtype in (np.int32, np.float32):
        keys = I.entropy_reduced(np.uint32, n, rng, 2).view(dtype) if dtype == np.int32 else I.with_specials(
            I.finite_floats(dtype, n, rng), rng, 1 / 64)
        idx = I.index_values(n)
        for desc in (False, True):
            for overwrite in (False, True):
                ko, vo, v0 = _run_segmented(lib, keys, b, e, width, align, desc, overwrite)
                rk, rv = oracle.segmented_sort(keys, idx, b, e, descending=desc, threads=8)
                assert ko.tobytes() == rk.tobytes(), (dtype, desc, overwrite)
                assert vo.tobytes() == v0[rv.astype(np.int64)].tobytes(), (dtype, desc, overwrite)
