"""The reciprocal-based division of the convective adjustment equals the IEEE division
bit for bit (tests/div_check.cu, 2^28 quotients)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_div_rn_recip_matches_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "div_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "cgenie_gb300", "csrc"),
                    os.path.join(HERE, "div_check.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
