"""Runs a broad set of the library's kernels on the bounds-checked build and
prints its status (test infrastructure: tests/test_gpu_checked.py starts this
in a process of its own with CBK_CUDA_LIB naming libcbk_cuda_checked.so).

Covers every routine of the sweep at width 32 and the benchmark orders, the
mixed-precision solves on all three kernels (registers, one warp per matrix,
workspace) and both least-squares kernels, the bucketed launch and the
pack / unpack kernels. Prints "checked: <count> <i> <j> <failures>" where
count is the number of view accesses refused, and <failures> the cases whose
results were not the oracle's.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import cases as C  # noqa: E402
import gpu_util as G  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    import torch

    import cbk_gb300
    assert cbk_gb300.lib_path().endswith("libcbk_cuda_checked.so"), cbk_gb300.lib_path()
    lib = cbk_gb300.lib()
    ora = O.oracle()
    bad = []
    for c in C.sweep(V_list=(32,), quick=True) + C.benchmark_shapes(32, 37):
        gi, g = G.run_gpu(c)
        oi, o = C.run(ora, c)
        r = G.lane_ratios_scaled(g, o, c)
        if gi != oi or not all(v <= 8 * G.order_of(c) for v in r.values()):
            bad.append(c.label)
    rng = np.random.default_rng(11)
    for n in (5, 8, 16, 24, 48, 70):
        nm, V = 40, 32
        A, _ = C.gen_spd_cond(rng, nm, n)
        B = rng.standard_normal((nm, n, 2))
        ap = torch.from_numpy(O.pack(A, V)).cuda()
        bp = torch.from_numpy(O.pack(B, V, pad_diag=0.0)).cuda()
        work = torch.empty(max(1, cbk_gb300.dposv_refined_lwork(n, 2, V, nm)), dtype=torch.uint8,
                           device="cuda")
        if cbk_gb300.dposv_refined_compact("C", "L", n, 2, ap, n, bp, n, V, nm, 10, None, None,
                                           work) != 0:
            bad.append(f"refined posv n={n}")
    for m, n in ((16, 8), (64, 16), (40, 12)):
        nm, V, nrhs = 40, 32, 2
        A, Bm, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
        ap = torch.from_numpy(O.pack(A, V)).cuda()
        bp = torch.from_numpy(O.pack(Bm, V, pad_diag=0.0)).cuda()
        tau = torch.zeros(((nm + V - 1) // V) * V * n, dtype=torch.float64, device="cuda")
        work = torch.empty(max(1, cbk_gb300.dgels_refined_lwork(m, n, nrhs, V, nm)),
                           dtype=torch.uint8, device="cuda")
        if cbk_gb300.dgels_refined_compact("C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm, 10,
                                           None, None, work) != 0:
            bad.append(f"refined gels {m}x{n}")
    bks, keep = [], []
    for n in (4, 17, 33):
        nm, V = 50, 32
        A = C.gen_sym_ldlt(rng, nm, n, np.float64)
        a = torch.from_numpy(O.pack(A, V)).cuda()
        b = torch.from_numpy(O.pack(rng.standard_normal((nm, n, 2)), V, pad_diag=0.0)).cuda()
        keep += [a, b]
        bks.append((n, nm, V, a, n, b, n))
    work = torch.empty(cbk_gb300.BUCKETED_LWORK, dtype=torch.uint8, device="cuda")
    if cbk_gb300.bucketed_compact("sysvnp", "d", "C", "L", 2, bks, work) != 0:
        bad.append("bucketed sysvnp")
    torch.cuda.synchronize()
    f = lib.cbk_cuda_check_status
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    count, i, j = ctypes.c_ulonglong(0), ctypes.c_int(0), ctypes.c_int(0)
    rc = f(ctypes.byref(count), ctypes.byref(i), ctypes.byref(j), 1)
    print(f"checked: {count.value} {i.value} {j.value} rc={rc} failures={bad}")
    return 0 if rc == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
