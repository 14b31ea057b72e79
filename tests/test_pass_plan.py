"""The plain sort's pass plan on the CPU: plan_pass_words (cccl_gb300/csrc/sort_policy.h, the
code the histogram kernel runs) compiled with g++ and checked for every pass count, buffer
mode and set of skippable passes (tests/host/pass_plan_check.cpp): the result lands where
running every pass puts it, the passes that run hand their buffers on in turn, the first
encodes and the last decodes, a skippable pass runs only when the buffer parity needs it,
and every pass that runs finds its look-back rows cleared although a skipped pass clears
its successor's rows only after a pass that ran."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_pass_plan_every_mask(tmp_path):
    exe = tmp_path / "pass_plan_check"
    subprocess.run(
        ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "cccl_gb300" / "csrc"),
         str(ROOT / "tests" / "host" / "pass_plan_check.cpp"), "-o", str(exe)],
        check=True,
    )
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "1020 cases, 0 failures" in r.stdout, r.stdout
