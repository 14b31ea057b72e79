"""Parity at the sizes of the benchmark configurations, and the reference's large-offset
cases.

* SortPairs of u64 keys + u32 values (value = index) at 2^24 pairs against the oracle: the
  entropy levels of the AND rule (1, 3 and 5 words), a constant key, descending, and the
  bit window 8..40 in both orders (the 2^28 headline itself is checked by bench.py on every
  run, with the GPU-side checker below).
* The full batched segmented configuration (2^27 f32 + i32 pairs in lognormal segments:
  41,398 segments drawn until they hold 2^27 keys, and 200,000 segments scaled to 2^27 keys)
  against the segmented oracle.
* cub/test/catch2_test_device_radix_sort_keys.cu:488-519: num_items = 2^32 - 5 and 2^32 - 1
  (the 32-bit offset limit) and one size in (2^32, 2^33], u8 keys, both orders, checked as a
  sorted permutation of the input; and a pairs sort of 2^30 + 12345 keys, which runs as two
  portions, checked for order, stability and permutation on the GPU.
"""

import numpy as np
import pytest

import inputs as I

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    import torch

    assert torch.cuda.is_available()
    return built_library


C2_CASES = [
    ("and1", 1, False, 0, 64, False),
    ("and3", 3, False, 0, 64, False),
    ("and5", 5, False, 0, 64, False),
    ("constant", 1, True, 0, 64, False),
    ("descending", 1, False, 0, 64, True),
    ("bits_8_40", 1, False, 8, 40, False),
    ("bits_8_40_desc", 3, False, 8, 40, True),
]


@pytest.mark.parametrize("name,ands,constant,b,e,desc", C2_CASES, ids=[c[0] for c in C2_CASES])
def test_sortpairs_u64_u32_at_2p24_vs_oracle(oracle, name, ands, constant, b, e, desc):
    from gpu_util import gpu_sort

    n = 1 << 24
    rng = np.random.default_rng(2024 + ands)
    k = I.entropy_reduced(np.uint64, n, rng, ands)
    if constant:
        k[:] = np.uint64(0x0123456789ABCDEF)
    v = I.index_values(n)
    ko, vo, _ = gpu_sort(k, v, b, e, desc)
    rk, rv = oracle.radix_sort(k, v, b, e, desc, threads=16)
    assert ko.tobytes() == rk.tobytes()
    assert vo.tobytes() == rv.tobytes()


@pytest.mark.parametrize("segments", [None, 200_000], ids=["41398_segments", "200k_segments"])
def test_full_batched_segmented_configuration_vs_oracle(oracle, segments):
    from bench import segmented_workload
    from gpu_util import gpu_seg_sort

    k, v, b, e = segmented_workload(segments=segments)
    assert k.size == 1 << 27
    assert b.size == (41398 if segments is None else segments)
    ko, vo, _ = gpu_seg_sort(k, v, b, e)
    rk, rv = oracle.segmented_sort(k, v, b, e, threads=16)
    assert ko.tobytes() == rk.tobytes()
    assert vo.tobytes() == rv.tobytes()


def _sorted_u8_permutation(keys_in, keys_out, descending):
    """keys_out is keys_in sorted: the same count of every byte value, in order."""
    import torch

    chunk = 1 << 28
    n = keys_in.numel()
    cin = torch.zeros(256, dtype=torch.int64, device="cuda")
    cout = torch.zeros(256, dtype=torch.int64, device="cuda")
    for s in range(0, n, chunk):
        cin += torch.bincount(keys_in[s : s + chunk].int(), minlength=256)
        cout += torch.bincount(keys_out[s : s + chunk].int(), minlength=256)
        a = keys_out[s : min(n, s + chunk + 1)].int()  # one past the chunk: its boundary pair
        ok = (a[1:] <= a[:-1]) if descending else (a[1:] >= a[:-1])
        if not bool(ok.all()):
            return False
    return bool(torch.equal(cin, cout))


@pytest.mark.parametrize("n", [(1 << 32) - 5, (1 << 32) - 1, (1 << 32) + 1_987_654_321],
                         ids=["2^32-5", "2^32-1", "2^32+1987654321"])
def test_large_offsets_u8_keys(n):
    import torch

    from cccl_gb300 import DoubleBuffer, SortOrder, make_radix_sort

    g = torch.Generator(device="cuda").manual_seed(n & 0xFFFF)
    ki = torch.randint(0, 256, (n,), dtype=torch.uint8, device="cuda", generator=g)
    for desc in (False, True):
        k0 = ki.clone()
        ko = torch.empty_like(ki)
        dk = DoubleBuffer(k0, ko)  # the reference's test sorts through a DoubleBuffer
        args = dict(d_in_keys=dk, d_out_keys=None, d_in_values=None, d_out_values=None)
        s = make_radix_sort(order=SortOrder.DESCENDING if desc else SortOrder.ASCENDING, **args)
        temp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
        s(temp_storage=temp, num_items=n, **args)
        torch.cuda.synchronize()
        assert _sorted_u8_permutation(ki, dk.current(), desc), (n, desc)
        del k0, ko, dk, temp
        torch.cuda.empty_cache()


def test_two_portions_pairs():
    """2^30 + 12345 i32 keys + u32 index values: more than one portion (a portion holds
    < 2^30 keys), so the digit bases of the second portion come from the first's last tile."""
    import torch

    from cccl_gb300 import SortOrder, make_radix_sort
    from gpu_util import check_sorted_pairs

    n = (1 << 30) + 12345
    g = torch.Generator(device="cuda").manual_seed(5)
    ki = torch.randint(-(2**31), 2**31 - 1, (n,), dtype=torch.int32, device="cuda", generator=g)
    ki &= torch.randint(-(2**31), 2**31 - 1, (n,), dtype=torch.int32, device="cuda", generator=g)  # duplicates
    vi = torch.arange(n, dtype=torch.int32, device="cuda")
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    for desc in (False, True):
        args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
        s = make_radix_sort(order=SortOrder.DESCENDING if desc else SortOrder.ASCENDING, **args)
        temp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
        s(temp_storage=temp, num_items=n, **args)
        torch.cuda.synchronize()
        assert check_sorted_pairs(ki, ko, vo, "i", desc), desc  # int32 tensors sort as signed keys
        del temp
