"""The sorts captured in a CUDA graph and replayed: the plain radix sort (SortPairs through the
C ABI), the batched segmented sort (its whole on-device launch sequence) and the learned-
partition sort (sample, fit, route and both routes' gated kernels). Each call is captured once
with preallocated temporary storage, then replayed on two different inputs copied into the
captured buffers; every replay is checked byte for byte against the oracle. Nothing in the
captured calls synchronizes with the host or allocates."""

import numpy as np
import pytest
import torch

import inputs as I
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    assert torch.cuda.is_available()
    return built_library


def _capture(call):
    """Warms `call` up on a side stream, captures it once and returns the graph."""
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        call()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        call()
    return g


def test_radix_sort_pairs_replayed(oracle):
    from cccl_gb300 import SortOrder, make_radix_sort

    n = 1 << 22
    rng = np.random.default_rng(31)
    k0 = I.entropy_reduced(np.uint64, n, rng, 1)
    ki, ko = to_dev(k0), to_dev(k0)
    vi = torch.arange(n, dtype=torch.int32, device="cuda")
    vo = torch.empty_like(vi)
    args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    s = make_radix_sort(order=SortOrder.ASCENDING, **args)
    temp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
    g = _capture(lambda: s(temp_storage=temp, num_items=n, **args))
    for ands in (1, 3):
        k = I.entropy_reduced(np.uint64, n, rng, ands)
        ki.copy_(to_dev(k))
        vi.copy_(torch.arange(n, dtype=torch.int32, device="cuda"))
        g.replay()
        torch.cuda.synchronize()
        rk, rv = oracle.radix_sort(k, np.arange(n, dtype=np.int32), threads=8)
        assert from_dev(ko, np.uint64).tobytes() == rk.tobytes()
        assert from_dev(vo, np.int32).tobytes() == rv.tobytes()


def test_segmented_sort_replayed(oracle):
    from cccl_gb300 import SortOrder, make_segmented_sort
    from segments import lognormal_segments

    rng = np.random.default_rng(32)
    b, e = lognormal_segments(rng, 1 << 21)
    n, nseg = int(e[-1]), b.size
    ki = torch.empty(n, dtype=torch.float32, device="cuda")
    ko = torch.empty_like(ki)
    vi = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty_like(vi)
    bo = torch.from_numpy(b.astype(np.int32)).cuda()
    eo = torch.from_numpy(e.astype(np.int32)).cuda()
    args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    s = make_segmented_sort(order=SortOrder.ASCENDING, start_offsets_in=bo, end_offsets_in=eo, **args)
    call = dict(num_items=n, num_segments=nseg, start_offsets_in=bo, end_offsets_in=eo, **args)
    temp = torch.empty(s(temp_storage=None, **call), dtype=torch.uint8, device="cuda")
    g = _capture(lambda: s(temp_storage=temp, **call))
    for _ in range(2):
        k = I.with_specials(rng.standard_normal(n).astype(np.float32), rng, 1e-3)
        v = rng.integers(-(2**31), 2**31 - 1, size=n, dtype=np.int32)
        ki.copy_(to_dev(k))
        vi.copy_(to_dev(v))
        g.replay()
        torch.cuda.synchronize()
        rk, rv = oracle.segmented_sort(k, v, b, e, threads=8)
        assert from_dev(ko, np.float32).tobytes() == rk.tobytes()
        assert from_dev(vo, np.int32).tobytes() == rv.tobytes()


def test_learned_sort_replayed(oracle):
    from cccl_gb300 import SortOrder, make_learned_sort

    n = 1 << 21
    rng = np.random.default_rng(33)
    ki = torch.empty(n, dtype=torch.float64, device="cuda")
    ko = torch.empty_like(ki)
    vi = torch.empty(n, dtype=torch.int64, device="cuda")
    vo = torch.empty_like(vi)
    args = dict(d_in_keys=ki, d_out_keys=ko, d_in_values=vi, d_out_values=vo)
    s = make_learned_sort(order=SortOrder.ASCENDING, **args)
    temp = torch.empty(s(temp_storage=None, num_items=n, **args), dtype=torch.uint8, device="cuda")
    g = _capture(lambda: s(temp_storage=temp, num_items=n, **args))
    # a skewed input (learned route) and an all-equal one (the plain route chosen on the device)
    for k in (I.lognormal(np.float64, n, rng, 0.0, 3.0), np.full(n, 2.5)):
        v = np.arange(n, dtype=np.int64)
        ki.copy_(to_dev(k))
        vi.copy_(to_dev(v))
        g.replay()
        torch.cuda.synchronize()
        rk, rv = oracle.radix_sort(k, v, threads=8)
        assert from_dev(ko, np.float64).tobytes() == rk.tobytes()
        assert from_dev(vo, np.int64).tobytes() == rv.tobytes()
