"""div_by() against IEEE division on the GPU: the engine divides by fixed
masses and bond windows with a rounded reciprocal and one correction step,
which must give the correctly rounded quotient for every numerator."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300", "csrc")


def test_div_by_matches_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "div_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I" + CSRC, "-I" + os.path.join(REPO, "include"), os.path.join(HERE, "gpu_src", "div_check.cu"),
                    "-o", exe], check=True, capture_output=True, timeout=300)
    out = subprocess.run([exe, "16384", "65536"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout
