"""The integer-pipe binary64 helpers of the tensor-core form (sign flip, kv
midrad) equal the FP64 instructions bit for bit on 2^26 seeded cases of
every operand class (tests/swfp_check.cu, built here with nvcc for
sm_103a)."""
import os
import shutil
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "vcp_gb300", "csrc")


def test_swfp_bitexact():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "swfp_check")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-I", CSRC, os.path.join(HERE, "swfp_check.cu"), "-o", exe],
                       check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout
    counts = {ln.split()[0]: int(ln.split()[-1]) for ln in out.splitlines() if "mismatches" in ln}
    assert set(counts) == {"sw_neg", "sw_midrad"}, out
    assert all(v == 0 for v in counts.values()), out
