"""The allocation-free refined solve, cbk_cuda_dposv_refined_compact_noalloc_async
(GPU; collected last on purpose).

This entry point is for callers that cannot allocate device memory when they
call -- code inside a host that owns every device allocation, or a loop that
must not call cudaMalloc -- so its scratch is the library's own fixed array
instead of a caller workspace. It runs the same kernels on the same data as
the workspace entry point, so through the C ABI its solutions, iteration
counts and backward errors must equal that entry point's bit for bit, twice
in a row (the array keeps the previous call's contents, and nothing in it may
leak into the next result); a warmed-up call must not change the device's
free memory; and a C program checks the refusal of a first address lookup
under stream capture and, where the device allows a second CUDA context, the
results in it (tests/c/noalloc_check.c). Its argument codes are checked on the CPU in
tests/test_abi.py.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _noalloc():
    import cbk_gb300
    f = cbk_gb300.lib().cbk_cuda_dposv_refined_compact_noalloc_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _batch(seed, n, nm, V):
    rng = np.random.default_rng(seed)
    A, _ = C.gen_spd_cond(rng, nm, n)
    B = rng.standard_normal((nm, n, 1))
    return A, B, O.pack(A, V), O.pack(B, V, pad_diag=0.0)


def _bits(t):
    return t.cpu().numpy().view(np.uint8)


def _solve_both(n, nm, V, seed):
    """The same batch through the workspace entry point and the no-alloc one;
    returns (A, B, X of the no-alloc call, whether x, iters and berr are
    bit-identical)."""
    import torch

    import cbk_gb300
    A, B, ap, bp = _batch(seed, n, nm, V)
    ref_a, ref_b = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    ref_it = torch.empty(nm, dtype=torch.int32, device="cuda")
    ref_be = torch.empty(nm, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dposv_refined_compact("C", "L", n, 1, ref_a, n, ref_b, n, V, nm, 10,
                                           ref_it, ref_be) == 0
    na_a, na_b = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    na_it = torch.full((nm,), 99, dtype=torch.int32, device="cuda")
    na_be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    info = _noalloc()(b"C", b"L", n, 1, na_a.data_ptr(), n, na_b.data_ptr(), n, V, nm, 10,
                      na_it.data_ptr(), na_be.data_ptr(), stream)
    torch.cuda.synchronize()
    assert info == 0, info
    same = (np.array_equal(_bits(ref_b), _bits(na_b)) and np.array_equal(_bits(ref_a), _bits(na_a))
            and np.array_equal(_bits(ref_it), _bits(na_it))
            and np.array_equal(_bits(ref_be), _bits(na_be)))
    return A, B, O.unpack(na_b.cpu().numpy(), nm, n, 1, V), same


@pytest.mark.parametrize("n,nm", [(80, 2000), (70, 2900), (48, 4000), (12, 5000)])
def test_noalloc_bit_identical_to_workspace_entry_point_twice(n, nm, cuda):
    V = 32
    for call, seed in enumerate((11 * n, 11 * n + 1)):  # two calls in a row, new data each
        A, B, X, same = _solve_both(n, nm, V, seed)
        assert same, f"call {call}: results differ from the workspace entry point's"
        assert (C.backward_error(A, X, B) <= 8 * n * EPS).all()


def test_noalloc_call_allocates_nothing(cuda):
    """A warmed-up call (the module and its array already loaded) leaves the
    device's free memory exactly as it was."""
    import torch
    n, nm, V = 80, 1000, 32
    _, _, ap, bp = _batch(5, n, nm, V)
    a, b = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    it = torch.empty(nm, dtype=torch.int32, device="cuda")
    f = _noalloc()
    stream = torch.cuda.current_stream().cuda_stream
    assert f(b"C", b"L", n, 1, a.data_ptr(), n, b.data_ptr(), n, V, nm, 10, it.data_ptr(),
             None, stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert f(b"C", b"L", n, 1, a.data_ptr(), n, b.data_ptr(), n, V, nm, 10, it.data_ptr(),
                 None, stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_refuses_lookup_under_capture_and_serves_contexts(tmp_path, cuda):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(cuda.lib_path())
    cudalib = os.path.join(cuda_home, "lib64")
    exe = str(tmp_path / "noalloc_check")
    subprocess.run([cc, "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda_home, "include"),
                    os.path.join(HERE, "c", "noalloc_check.c"),
                    "-L", libdir, "-lcbk_cuda", "-L", cudalib, "-lcudart",
                    f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudalib}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "noalloc ok" in r.stdout
