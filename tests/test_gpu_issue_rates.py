"""Issue rates of the arithmetic the step is built from, on the GPU at hand
(tests/issue_rates.cu): the FP64 rates must be far below the FP32 rate on GB300, which
is what the split-precision form is designed around.  Prints the table."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_issue_rates(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "issue_rates")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", os.path.join(HERE, "issue_rates.cu"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    rate = {m.group(1): float(m.group(2)) for m in re.finditer(r"^(\w+)\s.*?([\d.]+) op/clk/SM$", r.stdout, re.M)}
    assert rate["FFMA"] > 10 * rate["DFMA"]
