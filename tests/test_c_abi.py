"""The C ABI from a C program (CPU): tests/c/abi_check.c is compiled with the
system C compiler against include/cbk_cuda.h and linked with libcbk_cuda.so,
as a C caller of the reference's include/cbk.h would be, then run. Its calls
return before any device work."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_c_program_against_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    import cbk_gb300
    libdir = os.path.dirname(cbk_gb300.lib_path())
    exe = str(tmp_path / "abi_check")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c", "abi_check.c"),
                    "-L", libdir, "-lcbk_cuda", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "c abi ok" in r.stdout
