"""The integer-pipe binary64 <-> binary32 conversions that the mixed form uses on its state
(d2f, f2d in epic_gb300/csrc/device_common.cuh) give the hardware conversions' bits: every
binary32 value, 2^32 hashed binary64 values and every rounding boundary of each binary32
exponent (tests/cuda/conversions_check.cu, compiled here with nvcc); and the host's TF32 rounding
of the tensor-core filter's operator tiles gives cvt.rna.tf32.f32's bits for every finite normal
binary32 value."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "epic_gb300", "csrc")


def test_conversions_bit_exact(gpu, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "conversions_check")
    subprocess.run([nvcc, "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "cuda", "conversions_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches d2f=0 f2d=0 tf32=0" in r.stdout
