"""f32_no_event() against d_predict_c() on the GPU: the single-precision
screen may settle a pair prediction as "no event" only when the
double-precision prediction is no event, including pairs placed within a
hair of the separation, grazing and well-boundary edges."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300", "csrc")


def test_screen_never_drops_an_event(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "screen_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "-I" + CSRC, "-I" + os.path.join(REPO, "include"), os.path.join(HERE, "gpu_src", "screen_check.cu"),
                    "-o", exe], check=True, capture_output=True, timeout=300)
    out = subprocess.run([exe, str(1 << 20), "8"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    m = re.search(r"pairs (\d+) no-event (\d+) screened (\d+) failures (\d+)", out.stdout)
    assert m, out.stdout
    pairs, none, screened, fail = map(int, m.groups())
    assert fail == 0
    assert screened > 0.5 * none, out.stdout     # the screen settles most no-event pairs
