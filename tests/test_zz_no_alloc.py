"""The allocation-free entry point cccl_gb300_radix_sort_u32_noalloc.

It exists for callers that must not allocate device memory on their sort path (cudaMalloc
and cudaFree synchronize the whole device, and some host frameworks give a component a
fixed device-memory budget it may not grow). It keeps its scratch space in a fixed array
inside the library, so it is limited to CCCL_GB300_NOALLOC_MAX_ITEMS keys, and calls that
overlap on the GPU share that array.

These tests call it through the C ABI and check that its output is bit-identical to the
regular entry point cccl_device_radix_sort (which takes caller-provided temporary storage)
on the same inputs, on two calls in a row (the second call must not be disturbed by what
the first left in the shared scratch array). This file is collected last on purpose.
"""

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


def _noalloc(lib, keys, values=None, b=0, e=32, desc=False):
    import torch

    from gpu_util import from_dev, to_dev

    ki = to_dev(keys)
    ko = torch.empty_like(ki)
    vi = to_dev(values) if values is not None else None
    vo = torch.empty_like(vi) if vi is not None else None
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.cccl_gb300_radix_sort_u32_noalloc(
        ki.data_ptr(), ko.data_ptr(), vi.data_ptr() if vi is not None else None,
        vo.data_ptr() if vo is not None else None, keys.size, b, e, desc, stream)
    assert rc == 0, f"noalloc sort failed with CUresult {rc}"
    torch.cuda.synchronize()
    return from_dev(ko, keys.dtype), (from_dev(vo, values.dtype) if values is not None else None)


CASES = [
    (1000, True, 0, 32, False),      # single-tile path
    (4865, False, 0, 32, False),     # one past the single-tile cut: the smallest multi-pass sort
    (4865, True, 0, 32, True),
    (300_001, False, 0, 32, False),  # 4 passes, keys only
    (300_001, True, 0, 32, True),    # pairs, descending
    (300_001, True, 7, 7, False),    # begin_bit == end_bit: a copy
    (1 << 20, True, 4, 27, False),   # the maximum size, a bit window (3 passes)
]


def _status_clean():
    from cccl_gb300 import _bindings as B, sort_status

    assert sort_status(None) == (B.CUDA_SUCCESS, 0)  # the built-in array's status word


@pytest.mark.parametrize("n,with_values,b,e,desc", CASES)
def test_noalloc_matches_regular_entry_point(lib, n, with_values, b, e, desc):
    from gpu_util import gpu_sort

    for call in range(2):  # two calls in a row, different data
        rng = np.random.default_rng(1000 * call + n)
        keys = I.entropy_reduced(np.uint32, n, rng, 1 + call)
        values = rng.integers(0, 2**32, size=n, dtype=np.uint32) if with_values else None
        ko, vo = _noalloc(lib, keys, values, b, e, desc)
        _status_clean()
        rk, rv, _ = gpu_sort(keys, values, b, e, desc)
        assert ko.tobytes() == rk.tobytes()
        if with_values:
            assert vo.tobytes() == rv.tobytes()


def test_noalloc_keys_then_pairs(lib):
    """A keys-only call and then a pairs call of another size: the two use different tile
    sizes (so different numbers of look-back rows in the shared array) and must not see
    each other's leftovers."""
    from gpu_util import gpu_sort

    rng = np.random.default_rng(4242)
    for n, with_values in ((700_001, False), (250_003, True), (900_000, False)):
        keys = I.uniform_bits(np.uint32, n, rng)
        values = I.index_values(n) if with_values else None
        ko, vo = _noalloc(lib, keys, values)
        _status_clean()
        rk, rv, _ = gpu_sort(keys, values)
        assert ko.tobytes() == rk.tobytes()
        if with_values:
            assert vo.tobytes() == rv.tobytes()


def test_noalloc_empty_input(lib):
    import torch

    rc = lib.cccl_gb300_radix_sort_u32_noalloc(None, None, None, None, 0, 0, 32, False,
                                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    _status_clean()


def test_noalloc_rejects_too_many_items(lib):
    import torch

    from cccl_gb300 import _bindings as B

    k = torch.zeros(B.NOALLOC_MAX_ITEMS + 1, dtype=torch.int32, device="cuda")
    o = torch.empty_like(k)
    rc = lib.cccl_gb300_radix_sort_u32_noalloc(
        k.data_ptr(), o.data_ptr(), None, None, k.numel(), 0, 32, False, torch.cuda.current_stream().cuda_stream)
    assert rc == B.CUDA_ERROR_INVALID_VALUE
