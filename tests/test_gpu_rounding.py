"""The contact laws' 1 / sqrt(d) is computed with the engine's own correctly
rounded reciprocal and square root (a Newton-Raphson step with a fused
residual on the hardware estimates).  Bit-exact parity with the reference's float32
arithmetic needs them equal to IEEE division and sqrtf: checked here on every
float, on the GPU."""

import subprocess
from pathlib import Path

import numpy as np
import pytest

from jaxdem_gb300 import build as B

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.gpu
def test_reciprocal_and_square_root_are_correctly_rounded(tmp_path):
    exe = tmp_path / "rounding_check"
    src = ROOT / "tests" / "csrc" / "rounding_check.cu"
    subprocess.run([B.nvcc(), *B.ARCH, "-O3", "-std=c++17", "-I", str(B.CSRC), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout.split()
    counts = dict(zip(out[0::2], map(int, out[1::2])))
    # the reciprocal and 1 / sqrt(max(d, 1e-16)) match on every float
    assert counts["rcp"] == 0 and counts["inv_norm"] == 0, counts
    # the square root on every float of [1e-16, FLT_MAX] (far below, its residual underflows)
    assert counts["sqrt"] == 0 or counts["sqrt_hi"] < np.float32(1e-16).view(np.uint32), counts
