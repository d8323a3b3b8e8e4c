"""Double-float arithmetic (epic_gb300/csrc/df.cuh), which the mixed form uses for its pressure
gradient and vertical integration: products, quotients, differences, exp and log against
binary64 over 4M seeded arguments each, every error below 2e-13 (relative; absolute for log)
(tests/cuda/df_check.cu, compiled here with nvcc)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "epic_gb300", "csrc")


def test_double_float_accuracy(gpu, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "df_check")
    subprocess.run([nvcc, "-O3", "-std=c++17", "-fmad=false", "-prec-div=false", "-prec-sqrt=false",
                    "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "cuda", "df_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
