"""Parity of the learned-partition sort (through its C ABI) with the oracle and with the
plain radix sort: bit-exact keys and values and the same DoubleBuffer selector, on the
skewed distributions it is built for (Gaussian mixture, lognormal, Zipf, lognormal/uniform
mix), on every 4- and 8-byte key type, and on the adversarial inputs whose buckets overflow
(all keys equal, few distinct keys, sorted and reversed runs)."""

import numpy as np
import pytest

import inputs as I

pytestmark = pytest.mark.gpu

N = (1 << 21) + 12345  # above the learned path's minimum (2^20), ragged tail tile


@pytest.fixture(scope="module", autouse=True)
def _lib(built_library):
    import torch

    assert torch.cuda.is_available()
    return built_library


def _expected_buckets(n, key_bytes):
    """2048 keys per bucket where that takes no more partition passes than 4096, else 4096;
    2^8 to 2^24 buckets, whatever the key width."""
    log2n = int(np.ceil(np.log2(n)))
    b11, b12 = (min(max(log2n - i, 8), 24) for i in (11, 12))
    b = b11 if (b11 + 7) // 8 == (b12 + 7) // 8 else b12
    return b, (b + 7) // 8


DIST_SEED = {"gmm": 1, "lognormal": 2, "zipf": 3, "mix": 4}


def _check(oracle, keys, values=None, desc=False, overwrite=False, expect_learned=True):
    from gpu_util import gpu_sort

    st = {}
    ko, vo, sel = gpu_sort(keys, values, 0, None, desc, overwrite, method="learned", stats=st)
    rk, rv = oracle.radix_sort(keys, values, 0, None, desc, threads=8)
    assert ko.tobytes() == rk.tobytes(), "keys differ from the oracle"
    if values is not None:
        assert vo.tobytes() == rv.tobytes(), "values differ from the oracle"
    assert st["learned"] == int(expect_learned), st
    if overwrite:
        _, _, plain_sel = gpu_sort(keys, values, 0, None, desc, overwrite)
        assert sel == plain_sel
    return st


def _skewed(name, dtype, n, rng):
    if name == "gmm":
        return I.gaussian_mixture(dtype, n, rng)
    if name == "lognormal":
        return I.lognormal(dtype, n, rng, 0.0, 2.0 if np.dtype(dtype).itemsize == 4 else 3.0)
    if name == "zipf":
        return I.zipf_values(dtype, n, rng)
    if name == "mix":
        return I.half_uniform_mix(dtype, n, rng)
    raise ValueError(name)


@pytest.mark.parametrize("dist", ["gmm", "lognormal", "zipf", "mix"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=lambda d: np.dtype(d).name)
def test_skewed_floats_pairs(oracle, dtype, dist):
    rng = np.random.default_rng(DIST_SEED[dist] * 16 + np.dtype(dtype).itemsize)
    k = I.with_specials(_skewed(dist, dtype, N, rng), rng, 1e-3)
    vtype = np.uint32 if np.dtype(dtype).itemsize == 4 else np.int64
    st = _check(oracle, k, I.index_values(N, vtype))
    assert (st["bucket_log2"], st["partition_passes"]) == _expected_buckets(N, np.dtype(dtype).itemsize)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64],
                         ids=lambda d: np.dtype(d).name)
@pytest.mark.parametrize("desc", [False, True], ids=["asc", "desc"])
def test_key_types_keys_only(oracle, dtype, desc):
    rng = np.random.default_rng(np.dtype(dtype).itemsize * 7 + desc)
    if np.dtype(dtype).kind == "f":
        k = I.with_specials(I.gaussian_mixture(dtype, N, rng), rng, 1 / 64)
    else:
        k = I.entropy_reduced(dtype, N, rng, 2)
    _check(oracle, k, None, desc=desc)


@pytest.mark.parametrize("vdtype", [np.uint32, np.uint64], ids=["v4", "v8"])
@pytest.mark.parametrize("overwrite", [False, True], ids=["out", "doublebuffer"])
def test_values_and_doublebuffer(oracle, vdtype, overwrite):
    rng = np.random.default_rng(5 + overwrite)
    k = I.with_specials(I.lognormal(np.float32, N, rng), rng, 1e-3)
    _check(oracle, k, I.index_values(N, vdtype), desc=True, overwrite=overwrite)


def test_negative_and_positive_zero_keep_input_order(oracle):
    n = 1 << 21
    rng = np.random.default_rng(9)
    # 30 % zeros of either sign among normal keys: one large bucket of equal ordering keys,
    # while the input stays on the learned route
    k = rng.standard_normal(n).astype(np.float32)
    zeros = rng.random(n) < 0.3
    k[zeros] = np.where(rng.random(int(zeros.sum())) < 0.5, np.float32(0.0), np.float32(-0.0))
    _check(oracle, k, I.index_values(n))


@pytest.mark.parametrize(
    "case", ["all_equal", "two_values", "one_heavy_value", "sorted", "reversed", "sorted_then_reversed"]
)
@pytest.mark.parametrize("overwrite", [False, True], ids=["pointers", "double_buffer"])
def test_adversarial_inputs(oracle, case, overwrite):
    """Near-constant inputs (most neighbouring sample keys share a bucket) take the plain
    route chosen on the device; a heavy value that leaves most buckets small stays on the
    learned route and its bucket goes to the segmented sort."""
    rng = np.random.default_rng(11)
    n = N
    if case == "all_equal":
        k = np.full(n, 3.25, dtype=np.float64)
    elif case == "two_values":
        k = np.where(rng.random(n) < 0.9, 1.0, -7.5).astype(np.float64)
    elif case == "one_heavy_value":
        k = I.lognormal(np.float64, n, rng, 0.0, 3.0)
        k[rng.random(n) < 0.25] = 2.0
    else:
        k = np.sort(I.lognormal(np.float64, n, rng, 0.0, 3.0))
        if case == "reversed":
            k = k[::-1].copy()
        elif case == "sorted_then_reversed":
            k = np.concatenate([k[: n // 2], k[n // 2 :][::-1]])
    plain_route = case in ("all_equal", "two_values")
    st = _check(oracle, k, I.index_values(n, np.int64), overwrite=overwrite, expect_learned=not plain_route)
    if case == "one_heavy_value":
        assert st["device_buckets"] >= 1 and st["device_items"] >= n // 5, st


@pytest.mark.parametrize("n", [1, 4864, (1 << 20) - 1])
def test_small_inputs_take_the_plain_path(oracle, n):
    rng = np.random.default_rng(n)
    k = I.gaussian_mixture(np.float32, n, rng)
    _check(oracle, k, I.index_values(n), expect_learned=False)


def test_bit_window_takes_the_plain_path(oracle):
    from gpu_util import gpu_sort

    rng = np.random.default_rng(3)
    k = I.uniform_bits(np.uint32, N, rng)
    st = {}
    ko, _, _ = gpu_sort(k, None, 8, 24, method="learned", stats=st)
    rk, _ = oracle.radix_sort(k, None, 8, 24, False, threads=8)
    assert ko.tobytes() == rk.tobytes() and st["learned"] == 0


def test_larger_bucket_count(oracle):
    # 2^25 keys: 2^14 buckets of 2048 keys, two passes; the bucket id's top digit has 6 bits
    n = 1 << 25
    rng = np.random.default_rng(21)
    k = I.lognormal(np.float32, n, rng, 0.0, 2.0)
    st = _check(oracle, k, I.index_values(n))
    assert (st["bucket_log2"], st["partition_passes"]) == _expected_buckets(n, 4) == (14, 2)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=lambda d: np.dtype(d).name)
def test_sparse_buckets_with_specials(oracle, dtype):
    """A dense cluster and a sparse tail: the tail's buckets hold a handful of keys, NaNs of
    both signs and payloads, infinities and zeros among them; they must come out in radix
    order (bit patterns), as the plain sort gives them."""
    rng = np.random.default_rng(41)
    n = N
    k = rng.random(n).astype(dtype)
    tail = rng.choice(n, size=n // 500, replace=False)
    k[tail] = (10.0 ** rng.uniform(-30, 30, size=tail.size) * rng.choice([-1, 1], size=tail.size)).astype(dtype)
    k = I.with_specials(k, rng, 1e-4)
    for desc in (False, True):
        _check(oracle, k, I.index_values(n), desc=desc)


@pytest.mark.parametrize("dtype,expect", [(np.float32, False), (np.uint32, False), (np.float64, True),
                                          (np.int64, True)], ids=lambda x: str(x))
def test_cost_model_route(oracle, dtype, expect):
    """The host cost model: 4-byte keys go to the plain sort (two partition passes and the
    bucket sort cannot beat four plain passes), 8-byte keys take the learned kernels. The
    result is the plain sort's either way."""
    from gpu_util import gpu_sort

    rng = np.random.default_rng(77)
    k = (I.lognormal(dtype, N, rng) if np.dtype(dtype).kind == "f" else I.uniform_bits(dtype, N, rng))
    v = I.index_values(N)
    st = {}
    ko, vo, _ = gpu_sort(k, v, method="learned", stats=st, route="cost_model")
    rk, rv = oracle.radix_sort(k, v, threads=8)
    assert ko.tobytes() == rk.tobytes() and vo.tobytes() == rv.tobytes()
    assert st["learned"] == int(expect), st

