"""GPU: the hardware property the chain kernel is designed around -- FP64 FMA
throughput is a small fraction of FP32's on GB300 (tests/cuda/fp64_pipe_probe.cu)."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def test_fp64_pipe_is_much_slower_than_fp32(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "pipe_probe"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", str(HERE / "cuda" / "fp64_pipe_probe.cu"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rates = {m.group(1): float(m.group(2)) for m in re.finditer(r"^(\w+): [0-9.]+ ms -> ([0-9.]+) T", out, re.M)}
    assert rates["FFMA"] > 16 * rates["DFMA"], out
