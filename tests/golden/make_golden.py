"""Generates the golden vectors that pin the oracle to the reference.

Each case's inputs are drawn from tests/inputs.py with a fixed seed; the expected output
comes from the reference's own CPU sort reference (radix_sort_reference in
cub/test/catch2_radix_sort_helper.cuh), compiled from the reference tree by
``make -C oracle ref`` into oracle/_ref/ref_pin. Run in a container that has the
reference tree:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT))

import inputs as I  # noqa: E402
from oracle.pyoracle import TYPE_CODES  # noqa: E402

REF_PIN = ROOT / "oracle" / "_ref" / "ref_pin"


def cases():
    """(name, keys, values, begin_bit, end_bit, descending)"""
    out = []

    def rng(seed):
        return np.random.default_rng(seed)

    n = 5000
    out.append(("u32_keys_asc", I.uniform_bits(np.uint32, n, rng(1)), None, 0, 32, False))
    out.append(("u32_keys_desc", I.uniform_bits(np.uint32, n, rng(2)), None, 0, 32, True))
    k = I.uniform_bits(np.int16, 3000, rng(3))
    out.append(("i16_pairs_desc", k, I.index_values(k.size), 0, 16, True))
    for d, seed in ((False, 4), (True, 5)):
        k = I.with_specials(I.finite_floats(np.float32, 20000, rng(seed)), rng(seed + 100), 1 / 16)
        out.append((f"f32_specials_pairs_{'desc' if d else 'asc'}", k, I.index_values(k.size), 0, 32, d))
    k = I.with_specials(I.finite_floats(np.float64, 7000, rng(6)), rng(106), 1 / 16)
    out.append(("f64_specials_pairs_asc", k, I.index_values(k.size, np.uint64), 0, 64, False))
    k = I.uniform_bits(np.uint64, 10000, rng(7))
    out.append(("u64_bits_8_40_pairs", k, I.index_values(k.size), 8, 40, False))
    out.append(("u64_bits_8_40_pairs_desc", k, I.index_values(k.size), 8, 40, True))
    k = I.uniform_bits(np.int64, 1000, rng(8))
    out.append(("i64_single_tile_desc", k, I.index_values(k.size, np.uint64), 0, 64, True))
    k = I.uniform_bits(np.uint8, 50000, rng(9))
    out.append(("u8_pairs_asc", k, I.index_values(k.size), 0, 8, False))
    k = I.with_specials(I.finite_floats(np.float16, 4000, rng(10)), rng(110), 1 / 8)
    out.append(("f16_specials_pairs_desc", k, I.index_values(k.size), 0, 16, True))
    k = I.entropy_reduced(np.int32, 30000, rng(11), 3)
    out.append(("i32_entropy3_pairs_asc", k, I.index_values(k.size), 0, 32, False))
    k = I.with_specials(I.finite_floats(np.float32, 9000, rng(12)), rng(112), 1 / 32)
    out.append(("f32_bits_3_27_pairs_asc", k, I.index_values(k.size), 3, 27, False))
    out.append(("f32_one_key", np.array([-0.0], dtype=np.float32), None, 0, 32, False))
    k = np.zeros(7000, dtype=np.uint32)
    out.append(("u32_all_equal_pairs", k, I.index_values(k.size), 0, 32, False))
    return out


def run_ref(keys, values, b, e, desc):
    vb = 0 if values is None else values.dtype.itemsize
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        blob = keys.tobytes() + (b"" if values is None else values.tobytes())
        fin.write_bytes(blob)
        subprocess.run(
            [str(REF_PIN), str(TYPE_CODES[keys.dtype]), str(vb), str(keys.size), str(b), str(e), str(int(desc)),
             str(fin), str(fout)],
            check=True,
        )
        raw = fout.read_bytes()
    ko = np.frombuffer(raw[: keys.nbytes], dtype=keys.dtype).copy()
    vo = None if values is None else np.frombuffer(raw[keys.nbytes :], dtype=values.dtype).copy()
    return ko, vo


def main():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    for name, keys, values, b, e, desc in cases():
        ko, vo = run_ref(keys, values, b, e, desc)
        arrays = dict(keys_in=keys, keys_out=ko, begin_bit=b, end_bit=e, descending=int(desc))
        if values is not None:
            arrays.update(values_in=values, values_out=vo)
        np.savez_compressed(HERE / f"radix_{name}.npz", **arrays)
        print("wrote", name, keys.dtype, keys.size)


if __name__ == "__main__":
    main()
