"""The oracle against the reference's own CPU sort reference (golden vectors made by
tests/golden/make_golden.py from cub/test/catch2_radix_sort_helper.cuh) and against
independent numpy sorts."""

import glob
from pathlib import Path

import numpy as np
import pytest

import inputs as I

GOLDEN = sorted(glob.glob(str(Path(__file__).parent / "golden" / "radix_*.npz")))


def test_golden_vectors_exist():
    assert len(GOLDEN) >= 15


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: Path(p).stem)
def test_oracle_matches_reference_golden(oracle, path):
    g = np.load(path)
    vals = g["values_in"] if "values_in" in g else None
    ko, vo = oracle.radix_sort(
        g["keys_in"], vals, int(g["begin_bit"]), int(g["end_bit"]), bool(g["descending"]), threads=1
    )
    assert ko.tobytes() == g["keys_out"].tobytes()
    if vals is not None:
        assert vo.tobytes() == g["values_out"].tobytes()


@pytest.mark.parametrize("threads", [1, 4])
@pytest.mark.parametrize("dtype", [np.uint32, np.int64, np.int8, np.uint16])
def test_oracle_integers_match_numpy_stable_sort(oracle, dtype, threads):
    rng = np.random.default_rng(42)
    k = I.entropy_reduced(dtype, 100_000, rng, 2)
    v = I.index_values(k.size)
    ko, vo = oracle.radix_sort(k, v, threads=threads)
    perm = np.argsort(k, kind="stable")
    assert np.array_equal(ko, k[perm]) and np.array_equal(vo, v[perm])
    ko, vo = oracle.radix_sort(k, v, descending=True, threads=threads)
    # stable descending: larger first, equal keys keep input order
    perm = (k.size - 1 - np.argsort(k[::-1], kind="stable"))[::-1]
    assert np.array_equal(ko, k[perm]) and np.array_equal(vo, v[perm])


def test_oracle_floats_order_and_zero_rule(oracle):
    rng = np.random.default_rng(7)
    k = I.finite_floats(np.float32, 50_000, rng)
    k[::97] = 0.0
    k[::89] = -0.0
    v = I.index_values(k.size)
    ko, vo = oracle.radix_sort(k, v)
    # numeric order with +-0 equal and stable == numpy stable argsort (numpy treats -0 == +0)
    perm = np.argsort(k, kind="stable")
    assert np.array_equal(vo, v[perm])
    assert ko.tobytes() == k[perm].tobytes()  # -0.0 keeps its bit pattern


def test_oracle_nan_placement(oracle):
    k = np.array([np.nan, 1.0, -np.inf, np.inf, -1.0], dtype=np.float32)
    neg_nan = np.array([0xFFC00000], dtype=np.uint32).view(np.float32)
    k = np.concatenate([k, neg_nan])
    ko, _ = oracle.radix_sort(k)
    bits = ko.view(np.uint32)
    # -NaN before -inf, +NaN after +inf (raw twiddled bit order)
    assert bits[0] == 0xFFC00000 and np.isneginf(ko[1]) and np.isposinf(ko[-2]) and np.isnan(ko[-1])


def test_oracle_bit_window(oracle):
    rng = np.random.default_rng(3)
    k = I.uniform_bits(np.uint64, 20_000, rng)
    v = I.index_values(k.size)
    ko, vo = oracle.radix_sort(k, v, begin_bit=8, end_bit=40)
    sub = (k >> np.uint64(8)) & np.uint64((1 << 32) - 1)
    perm = np.argsort(sub, kind="stable")
    assert np.array_equal(vo, v[perm])


def test_oracle_rejects_bad_bits(oracle):
    with pytest.raises(ValueError):
        oracle.radix_sort(np.zeros(4, np.uint32), begin_bit=0, end_bit=40)
