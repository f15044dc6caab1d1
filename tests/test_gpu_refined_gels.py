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


# (64, 16, 8), (16, 16, 2), (40, 8, 4) and (12, 8, 3) run the warp-per-matrix
# kernel (variant 0); lane=True forces the lane-per-matrix one
@pytest.mark.parametrize("m,n,nrhs,lane", [(64, 16, 8, False), (20, 6, 1, False),
                                           (33, 17, 3, False), (16, 16, 2, False),
                                           (40, 8, 4, False), (12, 8, 3, False),
                                           (64, 16, 8, True), (40, 8, 4, True)])
def test_refined_gels_meets_fp64_accuracy(m, n, nrhs, lane, cuda):
    import cbk_gb300
    if lane:
        assert cbk_gb300.tune_set("gels_refined", "d", n, variant=1) == 0
    try:
        _check_refined_gels(m, n, nrhs)
    finally:
        cbk_gb300.tune_reset()


def _check_refined_gels(m, n, nrhs):
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


@pytest.mark.parametrize("m,n,nrhs,lane", [(64, 16, 3, False), (40, 8, 2, False),
                                           (64, 16, 3, True), (20, 6, 2, False)])
def test_refined_gels_fallback_is_the_plain_solve(m, n, nrhs, lane, cuda):
    """Matrices beyond the FP32 range (iters -2) and with a NaN (-3) are solved
    by the plain FP64 path: A, tau and B bit-identical to dgels_compact's; the
    other matrices converge and leave A and tau untouched."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(7 * m + n)
    nm, V = 96, 32
    A, B, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
    big, nan = [3, 40, 95], [10, 64]
    A[big] *= 1e42
    A[nan, 1, 0] = np.nan
    ap, bp = O.pack(A, V), O.pack(B, V, pad_diag=0.0)
    ng = (nm + V - 1) // V
    if lane:
        assert cbk_gb300.tune_set("gels_refined", "d", n, variant=1) == 0
    try:
        a1, b1 = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
        t1 = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
        it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
        be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
        assert cbk_gb300.dgels_refined_compact("C", "N", m, n, nrhs, a1, m, b1, m, t1, V, nm,
                                               iters=it, berr=be) == 0
        a2, b2 = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
        t2 = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
        assert cbk_gb300.dgels_compact("C", "N", m, n, nrhs, a2, m, b2, m, t2, V, nm) == 0
        torch.cuda.synchronize()
    finally:
        cbk_gb300.tune_reset()
    it, be = it.cpu().numpy(), be.cpu().numpy()
    assert (it[big] == -2).all() and (it[nan] == -3).all()
    ok = np.setdiff1d(np.arange(nm), big + nan)
    assert (it[ok] >= 0).all()
    assert np.isnan(be[big + nan]).all() and (be[ok] <= 8 * n * EPS).all()
    A1, A2 = O.unpack(a1.cpu().numpy(), nm, m, n, V), O.unpack(a2.cpu().numpy(), nm, m, n, V)
    B1, B2 = (O.unpack(x.cpu().numpy(), nm, m, nrhs, V) for x in (b1, b2))
    T1 = t1.cpu().numpy().reshape(ng, n, V).transpose(0, 2, 1).reshape(-1, n)[:nm]
    T2 = t2.cpu().numpy().reshape(ng, n, V).transpose(0, 2, 1).reshape(-1, n)[:nm]
    fb = big + nan
    assert np.array_equal(A1[fb], A2[fb], equal_nan=True)
    assert np.array_equal(B1[fb], B2[fb], equal_nan=True)
    assert np.array_equal(T1[fb], T2[fb], equal_nan=True)
    assert np.array_equal(A1[ok], O.unpack(ap, nm, m, n, V)[ok])
    assert (T1[ok] == 0).all()


@pytest.mark.parametrize("m,n,nrhs", [(40, 8, 3), (64, 16, 2), (12, 8, 2), (20, 6, 2)])
def test_refined_gels_layouts_agree_bitwise(m, n, nrhs, cuda):
    """The same batch in column-major (tight and padded leading dimensions) and
    row-major layouts: x, the residual coordinates, iters and berr are
    bit-identical (both kernels read A and B through the layout's view)."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(5 * m + n)
    nm, V = 70, 32
    A, B, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
    ng = (nm + V - 1) // V
    out = []
    for layout, lda, ldb in (("C", m, m), ("C", m + 3, m + 1), ("R", n + 2, nrhs + 1)):
        row = layout == "R"
        a = torch.from_numpy(O.pack(A, V, ld=lda, rowmajor=row)).cuda()
        b = torch.from_numpy(O.pack(B, V, ld=ldb, rowmajor=row, pad_diag=0.0)).cuda()
        t = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
        it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
        be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
        assert cbk_gb300.dgels_refined_compact(layout, "N", m, n, nrhs, a, lda, b, ldb, t, V, nm,
                                               iters=it, berr=be) == 0
        torch.cuda.synchronize()
        out.append((O.unpack(b.cpu().numpy(), nm, m, nrhs, V, ldb, row), it.cpu().numpy(),
                    be.cpu().numpy()))
    for X, it, be in out[1:]:
        assert np.array_equal(X, out[0][0])
        assert np.array_equal(it, out[0][1]) and np.array_equal(be, out[0][2])
    assert (out[0][1] >= 0).all()


@pytest.mark.parametrize("m,n,nrhs", [(64, 16, 2), (40, 8, 3), (20, 6, 2)])
def test_refined_gels_independent_of_width(m, n, nrhs, cuda):
    """x, iters and berr at V = 16 and 64 equal V = 32's bit for bit."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(9 * m + n)
    nm = 90
    A, B, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
    out = []
    for V in (32, 16, 64):
        ng = (nm + V - 1) // V
        a = torch.from_numpy(O.pack(A, V)).cuda()
        b = torch.from_numpy(O.pack(B, V, pad_diag=0.0)).cuda()
        t = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
        it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
        be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
        assert cbk_gb300.dgels_refined_compact("C", "N", m, n, nrhs, a, m, b, m, t, V, nm,
                                               iters=it, berr=be) == 0
        torch.cuda.synchronize()
        out.append((O.unpack(b.cpu().numpy(), nm, m, nrhs, V), it.cpu().numpy(),
                    be.cpu().numpy()))
    for X, it, be in out[1:]:
        assert np.array_equal(X, out[0][0])
        assert np.array_equal(it, out[0][1]) and np.array_equal(be, out[0][2])


def _dense(M, ld, stride, fill):
    nm, rows, cols = M.shape
    out = np.full(nm * stride, fill)
    for k in range(nm):
        out[k * stride:k * stride + cols * ld].reshape(cols, ld)[:, :rows] = M[k].T
    return out


def _undense(buf, nm, rows, cols, ld, stride):
    return np.stack([buf[k * stride:k * stride + cols * ld].reshape(cols, ld)[:, :rows].T
                     for k in range(nm)])


@pytest.mark.parametrize("m,n,nrhs", [(64, 16, 3), (40, 8, 2), (20, 6, 2)])
def test_refined_gels_batched_equals_compact(m, n, nrhs, cuda):
    """A strided dense batch (padded lda, ldb, strides) through
    dgels_refined_batched: B (x and the residual coordinates), iters, berr,
    and for a matrix that falls back its FP64 QR and tau, bit-identical to
    the compact entry point's; padding untouched; n = 0 sets B to zero."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(31 * m + n)
    nm, V = 70, 32
    A, B, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
    A[4] *= 1e42                                   # falls back (iters -2)
    ng = (nm + V - 1) // V
    a1 = torch.from_numpy(O.pack(A, V)).cuda()
    b1 = torch.from_numpy(O.pack(B, V, pad_diag=0.0)).cuda()
    t1 = torch.zeros(ng * V * n, dtype=torch.float64, device="cuda")
    it1 = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    be1 = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dgels_refined_compact("C", "N", m, n, nrhs, a1, m, b1, m, t1, V, nm,
                                           iters=it1, berr=be1) == 0
    lda, ldb = m + 2, m + 3
    sa, sb = lda * n + 7, ldb * nrhs + 1
    a2 = torch.from_numpy(_dense(A, lda, sa, 5.0)).cuda()
    b2 = torch.from_numpy(_dense(B, ldb, sb, 6.0)).cuda()
    t2 = torch.zeros(nm * n, dtype=torch.float64, device="cuda")
    it2 = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    be2 = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dgels_refined_batched("N", m, n, nrhs, a2, lda, sa, b2, ldb, sb, t2, nm,
                                           iters=it2, berr=be2) == 0
    torch.cuda.synchronize()
    it = it1.cpu().numpy()
    assert it[4] == -2 and np.array_equal(it2.cpu().numpy(), it)
    assert np.array_equal(be2.cpu().numpy(), be1.cpu().numpy(), equal_nan=True)
    bh, ah = b2.cpu().numpy(), a2.cpu().numpy()
    assert np.array_equal(_undense(bh, nm, m, nrhs, ldb, sb),
                          O.unpack(b1.cpu().numpy(), nm, m, nrhs, V))
    Ad, Ac = _undense(ah, nm, m, n, lda, sa), O.unpack(a1.cpu().numpy(), nm, m, n, V)
    assert np.array_equal(Ad, Ac)
    T1 = t1.cpu().numpy().reshape(ng, n, V).transpose(0, 2, 1).reshape(-1, n)[:nm]
    assert np.array_equal(t2.cpu().numpy().reshape(nm, n), T1)
    assert (bh[_dense(np.zeros_like(B), ldb, sb, 1.0) == 1.0] == 6.0).all()
    assert (ah[_dense(np.zeros_like(A), lda, sa, 1.0) == 1.0] == 5.0).all()
    # n = 0: B := 0 inside each matrix, the padding kept
    b3 = torch.from_numpy(_dense(B, ldb, sb, 6.0)).cuda()
    assert cbk_gb300.dgels_refined_batched("N", m, 0, nrhs, a2, lda, sa, b3, ldb, sb, t2,
                                           nm) == 0
    torch.cuda.synchronize()
    b3h = b3.cpu().numpy()
    inside = _dense(np.zeros_like(B), ldb, sb, 1.0) == 0.0
    assert (b3h[inside] == 0.0).all() and (b3h[~inside] == 6.0).all()
