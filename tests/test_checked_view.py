"""The bounds-checked build's matrix views, on the host (CPU): a small
program (tests/c/view_check.cu) compiled with CBK_CUDA_CHECKED against the
device header makes in-range and out-of-range accesses through views and
checks that exactly the out-of-range ones are refused, counted and recorded,
and that none of them touches memory. The GPU side of the checked build is
tests/test_gpu_checked.py."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_checked_views_refuse_out_of_range_accesses(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    exe = str(tmp_path / "view_check")
    subprocess.run([nvcc, "-std=c++17", "-DCBK_CUDA_CHECKED", "-gencode",
                    "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "cbk_gb300", "csrc"),
                    os.path.join(HERE, "c", "view_check.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "view check ok" in r.stdout
