"""The GPU-side result checker (gpu_util.check_sorted_pairs), run on CPU tensors against the
oracle: it accepts the oracle's output and rejects outputs with a planted mistake (an order
error, a stability error, a value that does not belong to its key). The checker judges the
full-size GPU results, so it is pinned here first."""

import numpy as np
import pytest
import torch

import inputs as I
from gpu_util import check_sorted_pairs

SIGNED = {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}
KINDS = [(np.uint8, "u"), (np.int16, "i"), (np.uint32, "u"), (np.int32, "i"), (np.float32, "f"), (np.uint64, "u"),
         (np.int64, "i"), (np.float64, "f"), (np.float16, "f")]


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(SIGNED[a.dtype.itemsize]).copy())


@pytest.mark.parametrize("dtype,kind", KINDS, ids=lambda x: np.dtype(x).name if not isinstance(x, str) else x)
@pytest.mark.parametrize("desc", [False, True])
def test_checker_accepts_oracle_and_rejects_planted_mistakes(oracle, dtype, kind, desc):
    rng = np.random.default_rng(np.dtype(dtype).itemsize * 7 + desc)
    n = 20_000
    if kind == "f":
        k = I.with_specials(I.finite_floats(dtype, n, rng), rng, 1 / 16)
        k[rng.choice(n, 300, replace=False)] = dtype(-0.0)
        k[rng.choice(n, 300, replace=False)] = dtype(0.0)
    else:
        k = I.entropy_reduced(dtype, n, rng, 3)
    v = I.index_values(n)
    rk, rv = oracle.radix_sort(k, v, descending=desc)
    ki, ko, vo = _t(k), _t(rk), torch.from_numpy(rv.view(np.int32).copy())
    assert check_sorted_pairs(ki, ko, vo, kind, desc)
    # order: swap two neighbours with different keys (and their values)
    order_bits = ko.numpy()
    i = int(np.nonzero(order_bits[1:] != order_bits[:-1])[0][len(order_bits) // 3 % 50])
    bad_k, bad_v = ko.clone(), vo.clone()
    bad_k[[i, i + 1]] = bad_k[[i + 1, i]]
    bad_v[[i, i + 1]] = bad_v[[i + 1, i]]
    assert not check_sorted_pairs(ki, bad_k, bad_v, kind, desc)
    # stability: swap the values of two neighbouring equal keys
    j = int(np.nonzero(order_bits[1:] == order_bits[:-1])[0][0])
    bad_v = vo.clone()
    bad_v[[j, j + 1]] = bad_v[[j + 1, j]]
    assert not check_sorted_pairs(ki, ko, bad_v, kind, desc)
    # a value that names another key's position
    bad_v = vo.clone()
    bad_v[n // 2] = bad_v[n // 2 + 1] if order_bits[n // 2] != order_bits[n // 2 + 1] else bad_v[0]
    assert not check_sorted_pairs(ki, ko, bad_v, kind, desc)
