"""The allocation-free refined solve, cbk_cuda_dposv_refined_compact_noalloc_async
(GPU; collected last on purpose).

This entry point is for callers that cannot allocate device memory when they
call -- code inside a host that owns every device allocation, or a loop that
must not call cudaMalloc -- so its scratch is the library's own fixed array
instead of a caller workspace. Called through the C ABI, its results must
match the workspace entry point's within the tests' bound, twice in a row
(the array keeps the previous call's contents, and nothing in it may leak
into the next result), and a batch too large for the array is refused.
"""
import ctypes

import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
SCRATCH = 64 << 20  # CBK_CUDA_NOALLOC_SCRATCH_BYTES


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


def _solve_both(n, nm, V, seed):
    """The same batch through the workspace entry point and the no-alloc one."""
    import torch

    import cbk_gb300
    A, B, ap, bp = _batch(seed, n, nm, V)
    ref_a, ref_b = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    ref_it = torch.empty(nm, dtype=torch.int32, device="cuda")
    assert cbk_gb300.dposv_refined_compact("C", "L", n, 1, ref_a, n, ref_b, n, V, nm, 10,
                                           ref_it) == 0
    na_a, na_b = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    na_it = torch.empty(nm, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    info = _noalloc()(b"C", b"L", n, 1, na_a.data_ptr(), n, na_b.data_ptr(), n, V, nm, 10,
                      na_it.data_ptr(), None, stream)
    torch.cuda.synchronize()
    assert info == 0
    X_ref = O.unpack(ref_b.cpu().numpy(), nm, n, 1, V)
    X_na = O.unpack(na_b.cpu().numpy(), nm, n, 1, V)
    return A, B, X_ref, X_na, ref_it.cpu().numpy(), na_it.cpu().numpy()


@pytest.mark.parametrize("n,nm", [(80, 2000), (70, 2900), (48, 4000), (12, 5000)])
def test_noalloc_matches_workspace_entry_point_twice(n, nm, cuda):
    V = 32
    for call, seed in enumerate((11 * n, 11 * n + 1)):  # two calls in a row, new data each
        A, B, X_ref, X_na, it_ref, it_na = _solve_both(n, nm, V, seed)
        scale = np.abs(X_ref).reshape(nm, -1).max(axis=1)
        diff = np.abs(X_na - X_ref).reshape(nm, -1).max(axis=1)
        assert (diff <= 8 * n * EPS * scale).all(), (call, float((diff / scale).max() / EPS))
        assert np.array_equal(it_ref, it_na)
        assert (C.backward_error(A, X_na, B) <= 8 * n * EPS).all()


def test_noalloc_rejects_a_batch_beyond_its_scratch(cuda):
    import cbk_gb300
    n, V = 80, 32
    f = _noalloc()
    lw = cbk_gb300.dposv_refined_lwork
    fits = max(nm for nm in range(32, 20000, 32) if lw(n, 1, V, nm) <= SCRATCH)
    assert lw(n, 1, V, fits + 32) > SCRATCH
    # refused before any device work: null pointers are never touched
    assert f(b"C", b"L", n, 1, None, n, None, n, V, fits + 32, 10, None, None, None) == -10
    assert f(b"C", b"L", n, 1, None, n, None, n, V, 0, 10, None, None, None) == 0
    assert f(b"C", b"L", n, 1, None, n, None, n, V, 64, -1, None, None, None) == -11
