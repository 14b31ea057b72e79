"""The cub-compatible C++ shim (include/cccl_gb300/cub_shim.h) against CUB itself: the same
DeviceRadixSort and DeviceSegmentedSort calls (pointer and DoubleBuffer overloads, both
orders, bit windows, 1- to 8-byte keys and values, +-0/NaN/inf floats, 32- and 64-bit
segment offsets) compiled into one program from the CUDA toolkit's CCCL headers, every output
byte and selector compared (tests/cub_check/shim_vs_cub.cu)."""

import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cub_check" / "shim_vs_cub.cu"
OUT = ROOT / "tests" / "cub_check" / "_build" / "shim_vs_cub"
CCCL_INC = Path("/usr/local/cuda/include/cccl")


def test_shim_matches_cub(built_library):
    if not CCCL_INC.exists():
        pytest.skip("no CCCL headers in the CUDA toolkit")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    lib_dir = Path(built_library).parent
    OUT.parent.mkdir(parents=True, exist_ok=True)
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(CCCL_INC),
                    "-I", str(ROOT / "include"), str(SRC), "-o", str(OUT), "-L", str(lib_dir), "-lccclsort", "-lcuda",
                    "-Xlinker", f"-rpath={lib_dir}"], check=True)
    r = subprocess.run([str(OUT)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failure(s)" in r.stdout
