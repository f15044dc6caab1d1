"""Mixed-precision least squares (FP32 QR + FP64 refinement) on the GPU.

The least-squares configuration: A = U diag(s) V^T with kappa in 1e1 .. 1e4,
B = A X + 1e-3 noise, m = 64, n = 16, nrhs = 8 (and smaller shapes). Gates per
matrix: the normal-equations residual ||A^T (b - A x)|| / (||A|| (||A|| ||x||
+ ||b||)) <= 8 n eps64 in float64 here, and agreement with the plain FP64
dgels_compact on the GPU within the least-squares condition number
(kappa + kappa^2 ||r|| / (||A|| ||x||), Wedin) times 8 n eps64.
"""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _normal_residual(A, X, B):
    R = B - A @ X
    G = A.transpose(0, 2, 1) @ R
    an = np.abs(A).sum(axis=2).max(axis=1)
    xn = np.abs(X).max(axis=1)
    bn = np.abs(B).max(axis=1)
    return (np.abs(G).max(axis=1) / (an[:, None] * (an[:, None] * xn + bn))).max(axis=1)


@pytest.mark.parametrize("m,n,nrhs", [(64, 16, 8), (20, 6, 1), (33, 17, 3), (16, 16, 2)])
def test_refined_gels_meets_fp64_accuracy(m, n, nrhs, cuda):
    import torch

    import cbk_gb300
    rng = np.random.default_rng(m * 100 + n)
    nm, V = 150, 32
    A, B, X, kappa = C.gen_ls_cond(rng, nm, m, n, nrhs)
    ap, bp = O.pack(A, V), O.pack(B, V, pad_diag=0.0)
    ng = (nm + V - 1) // V
    # refined
    a1, b1 = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    t1 = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
    it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dgels_refined_compact("C", "N", m, n, nrhs, a1, m, b1, m, t1, V, nm,
                                           iters=it, berr=be) == 0
    # plain FP64 on the GPU
    a2, b2 = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    t2 = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dgels_compact("C", "N", m, n, nrhs, a2, m, b2, m, t2, V, nm) == 0
    torch.cuda.synchronize()
    X1 = O.unpack(b1.cpu().numpy(), nm, m, nrhs, V)[:, :n]
    X2 = O.unpack(b2.cpu().numpy(), nm, m, nrhs, V)[:, :n]
    it, be = it.cpu().numpy(), be.cpu().numpy()
    ne1 = _normal_residual(A, X1, B)
    ne2 = _normal_residual(A, X2, B)
    assert (ne1 <= 8 * n * EPS).all(), (ne1.max() / (n * EPS), kappa[ne1.argmax()])
    assert (ne2 <= 8 * n * EPS).all()
    # the two FP64-accurate solutions agree within the LS condition number
    R = B - A @ X2
    an = np.linalg.norm(A, 2, axis=(1, 2))
    theta = np.linalg.norm(R, axis=1).max(axis=1) / (an * np.linalg.norm(X2, axis=1).max(axis=1))
    kls = kappa + kappa ** 2 * theta
    rel = np.abs(X1 - X2).reshape(nm, -1).max(axis=1) / np.abs(X2).reshape(nm, -1).max(axis=1)
    assert (rel <= 8 * n * EPS * kls).all(), float((rel / (EPS * kls)).max())
    conv = it >= 0
    # converged lanes leave A untouched; the reported error is the bounded one
    A1 = O.unpack(a1.cpu().numpy(), nm, m, n, V)
    assert np.array_equal(A1[conv], O.unpack(ap, nm, m, n, V)[conv])
    assert (be[conv] <= 8 * n * EPS).all()
    assert np.isnan(be[~conv]).all()
    print(f"m={m} n={n} nrhs={nrhs}: converged {conv.mean():.3f}, mean steps "
          f"{it[conv].mean():.2f}, worst normal residual {ne1.max() / EPS:.2f} eps")


def test_refined_gels_argument_checks(cuda):
    import cbk_gb300
    f = cbk_gb300.dgels_refined_compact
    assert f("C", "T", 8, 4, 1, None, 8, None, 8, None, 32, 64) == -2
    assert f("C", "N", 4, 8, 1, None, 4, None, 8, None, 32, 64) == -4
    assert f("C", "N", 80, 70, 1, None, 80, None, 80, None, 32, 64) == -4
    assert f("C", "N", 8, 4, 1, None, 8, None, 8, None, 32, 64, max_iter=-1) == -13
    assert f("C", "N", 8, 4, 0, None, 8, None, 8, None, 32, 64) == 0
