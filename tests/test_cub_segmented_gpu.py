"""Pins the segmented-sort oracle (and the engine) against CUB's own DeviceSegmentedSort,
compiled on the GPU machine from the CUDA toolkit's CCCL headers: NaN-heavy float keys in
segments of every size class, with and without partitioning (> 500 segments), both orders.

The toolkit's CCCL is an earlier release of the reference library; where it is missing this
test is skipped and parity rests on the oracle's restatement of the reference source."""

import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

import inputs as I
from segments import edge_segments, lognormal_segments

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent
SRC = HERE / "cub_check" / "cub_segmented.cu"
OUT = HERE / "cub_check" / "_build" / "cub_segmented"
CCCL_INC = Path("/usr/local/cuda/include/cccl")


@pytest.fixture(scope="module")
def cub_binary():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not CCCL_INC.exists():
        pytest.skip("no CCCL headers in the CUDA toolkit")
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if not OUT.exists() or OUT.stat().st_mtime < SRC.stat().st_mtime:
        subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(CCCL_INC),
                        str(SRC), "-o", str(OUT)], check=True)
    return OUT


def run_cub(binary, keys, vals, b, e, desc):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        fin.write_bytes(keys.tobytes() + vals.tobytes() + b.astype(np.int32).tobytes() + e.astype(np.int32).tobytes())
        subprocess.run([str(binary), str(keys.size), str(b.size), str(int(desc)), str(fin), str(fout)], check=True)
        raw = fout.read_bytes()
    return np.frombuffer(raw[: keys.nbytes], dtype=np.float32), np.frombuffer(raw[keys.nbytes:], dtype=np.int32)


CASES = {
    "edges_fallback": lambda rng: edge_segments([1, 2, 3, 5, 17, 18, 19, 64, 111, 112, 113, 500, 3000, 9000], gap=0)[:2],
    "edges_partitioned": lambda rng: edge_segments([1, 2, 3, 5, 17, 18, 19, 64, 111, 112, 113, 500, 3000] * 45, gap=0)[:2],
    "lognormal": lambda rng: lognormal_segments(rng, 1 << 20, mu=4.0, sigma=2.0),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("desc", [False, True])
def test_engine_and_oracle_match_cub(cub_binary, oracle, case, desc):
    from gpu_util import gpu_seg_sort

    rng = np.random.default_rng(len(case) * 7 + desc)
    b, e = CASES[case](rng)
    n = int(e[-1])
    k = I.with_specials(I.finite_floats(np.float32, n, rng), rng, 1 / 6)
    v = I.index_values(n).astype(np.int32)
    ck, cv = run_cub(cub_binary, k, v, b, e, desc)
    ok_, ov = oracle.segmented_sort(k, v, b, e, descending=desc, threads=8)
    gk, gv, _ = gpu_seg_sort(k, v, b, e, desc)
    assert ok_.tobytes() == ck.tobytes() and ov.tobytes() == cv.tobytes(), "oracle differs from CUB"
    assert gk.tobytes() == ck.tobytes() and gv.tobytes() == cv.tobytes(), "engine differs from CUB"
