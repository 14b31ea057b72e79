"""Build recipe of the sort library: sm_103a cubins (nvcc) embedded into a host shared
library (g++), all in-tree under ``cccl_gb300/_build``.

The recipe needs only nvcc, g++ and the CUDA driver library; it runs the same on x86_64
and aarch64 hosts. Outputs are reused when the sources have not changed.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
ROOT = PKG.parent
INCLUDE = ROOT / "include"
LIB_NAME = "libccclsort.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17"]  # no fast-math: comparisons must not flush denormals
# Tile-shape overrides for tuning builds, e.g. "-DGB300_PERSISTENT_TPB=1024 -DGB300_PERSISTENT_ITEMS=6";
# applied to the kernels and to the host dispatcher alike.
TUNE_DEFINES = os.environ.get("GB300_TUNE_DEFINES", "").split()

IMAGES = {
    "radix_k1": "radix_k1.cu",
    "radix_k2": "radix_k2.cu",
    "radix_k4": "radix_k4.cu",
    "radix_k8": "radix_k8.cu",
    "seg_k1": "seg_k1.cu",
    "seg_k2": "seg_k2.cu",
    "seg_k4": "seg_k4.cu",
    "seg_k8": "seg_k8.cu",
    "learned_k4": "learned_k4.cu",
    "learned_k8": "learned_k8.cu",
}
HOST_SOURCES = [
    "images.cpp",
    "radix_plan.cpp",
    "radix_sort_abi.cpp",
    "segmented_plan.cpp",
    "segmented_sort_abi.cpp",
    "learned_plan.cpp",
    "learned_sort_abi.cpp",
    "status_abi.cpp",
    "value_gather.cpp",
    "offset_iterators.cpp",
]
# Runtime-API translation units (host + device code in one object, linked with static cudart)
RUNTIME_SOURCES = ["noalloc_sort.cu"]
# Measurement library of bench.py (the digit pass's memory-pattern floor), kept out of the
# sort library
FLOOR_SOURCE = "pattern_floor.cu"
FLOOR_LIB_NAME = "libpatternfloor.so"


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in sorted(str(x) for x in paths):
        h.update(p.encode())
        h.update(Path(p).read_bytes())
    return h.hexdigest()


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def library_path() -> Path:
    return BUILD / LIB_NAME


def floor_library_path() -> Path:
    return BUILD / FLOOR_LIB_NAME


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every kernel image for sm_103a and link the host library."""
    BUILD.mkdir(exist_ok=True)
    sources = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(
        CSRC.glob("*.cpp")
    ) + list(INCLUDE.glob("*/*.h")) + list(INCLUDE.glob("*/*/*.h")) + [Path(__file__)]
    stamp = BUILD / "stamp.txt"
    digest = _digest(sources) + " ".join(TUNE_DEFINES)
    lib = library_path()
    if not force and lib.exists() and floor_library_path().exists() and stamp.exists() and stamp.read_text() == digest:
        return lib

    def cubin(name_src):
        name, src = name_src
        out = BUILD / f"{name}.cubin"
        _run([NVCC, "-cubin", *ARCH, *NVCC_FLAGS, *TUNE_DEFINES, "-I", str(CSRC), str(CSRC / src), "-o", str(out)],
             verbose)
        return out

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(cubin, IMAGES.items()))

    embed = BUILD / "embed.c"
    lines = ["/* generated by cccl_gb300/build.py: links the sm_103a cubins into the library */", "__asm__("]
    lines.append('".section .rodata\\n"')
    for name in IMAGES:
        path = (BUILD / f"{name}.cubin").as_posix()
        lines += [
            '".balign 64\\n"',
            f'".global gb300_img_{name}\\n"',
            f'"gb300_img_{name}:\\n"',
            f'".incbin \\"{path}\\"\\n"',
            f'".global gb300_img_{name}_end\\n"',
            f'"gb300_img_{name}_end:\\n"',
            '".byte 0\\n"',
        ]
    lines.append('".previous\\n"')
    lines.append(");")
    embed.write_text("\n".join(lines) + "\n")

    cxx = os.environ.get("CXX", "g++")
    objs = []

    def host_obj(src):
        out = BUILD / (Path(src).stem + ".o")
        _run(
            [cxx, "-O2", "-fPIC", "-std=c++17", "-DCCCL_C_EXPERIMENTAL", *TUNE_DEFINES, "-fvisibility=hidden", "-Wall", "-I", str(INCLUDE), "-I",
             str(CSRC), "-I", str(CUDA_HOME / "include"), "-c", str(src), "-o", str(out)],
            verbose,
        )
        return out

    def runtime_obj(src):
        out = BUILD / (Path(src).stem + ".o")
        _run(
            [NVCC, "-c", *ARCH, *NVCC_FLAGS, *TUNE_DEFINES, "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
             "-I", str(INCLUDE), "-I", str(CSRC), str(CSRC / src), "-o", str(out)],
            verbose,
        )
        return out

    def floor_lib():
        out = floor_library_path()
        _run([NVCC, "-shared", *ARCH, *NVCC_FLAGS, *TUNE_DEFINES, "-Xcompiler", "-fPIC", "-Xcompiler",
              "-fvisibility=hidden", "-I", str(CSRC), str(CSRC / FLOOR_SOURCE), "-o", str(out) + ".tmp"], verbose)
        shutil.move(str(out) + ".tmp", str(out))

    host = [CSRC / s for s in HOST_SOURCES] + [embed]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        floor_job = ex.submit(floor_lib)
        objs = list(ex.map(host_obj, host)) + list(ex.map(runtime_obj, RUNTIME_SOURCES))
        floor_job.result()

    libdirs = []
    for d in (CUDA_HOME / "lib64", CUDA_HOME / "lib64" / "stubs", CUDA_HOME / "targets" / "sbsa-linux" / "lib" / "stubs"):
        if d.exists():
            libdirs += ["-L", str(d)]
    tmp = BUILD / (LIB_NAME + ".tmp")
    _run([cxx, "-shared", "-o", str(tmp), *map(str, objs), *libdirs, "-lcudart_static", "-lcuda", "-lrt", "-ldl",
          "-lpthread", "-Wl,--no-undefined"], verbose)
    shutil.move(str(tmp), str(lib))
    stamp.write_text(digest)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force=True))
