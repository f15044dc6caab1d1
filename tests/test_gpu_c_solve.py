"""A C program solving on the GPU through the C ABI: tests/c/solve_check.c
builds a compact batch on the host, copies it to the device with the CUDA
runtime, calls cbk_cuda_dposv_compact and cbk_cuda_dposv_refined_compact and
checks every solution's backward error on the host."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_program_solves_on_the_gpu(tmp_path, cuda):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(cuda.lib_path())
    cudalib = os.path.join(cuda_home, "lib64")
    exe = str(tmp_path / "solve_check")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda_home, "include"),
                    os.path.join(HERE, "c", "solve_check.c"),
                    "-L", libdir, "-lcbk_cuda", "-L", cudalib, "-lcudart", "-lm",
                    f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudalib}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "c solve ok" in r.stdout
