"""The mixed-precision SPD solve (FP32 factor + FP64 refinement) on the GPU.

Workload as the mixed-precision configuration: A = U diag(s) U^T with U
Haar-random and s log-uniform for condition numbers 1e1 .. 1e6, n in
{8, 16, 32, 48} (plus orders around the register / workspace boundary).
Gates, per matrix:
  * normwise backward error ||b - A x|| / (||A|| ||x|| + ||b||) <= 8 n eps64,
    computed here in float64 from the original A and B -- the plain FP64
    path's bound, so both paths meet equal FP64 error;
  * a converged matrix leaves A bit-for-bit unchanged; a matrix that fell
    back holds exactly the plain path's FP64 factor;
  * the reported iters / berr agree with what happened.
"""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _run(A, B, V=32, layout="C", uplo="L", max_iter=10, nrhs=None):
    import torch

    import cbk_gb300
    nm, n, _ = A.shape
    nrhs = B.shape[2]
    row = layout == "R"
    ap = torch.from_numpy(O.pack(A, V, n, row)).cuda()
    bp = torch.from_numpy(O.pack(B, V, (nrhs if row else n), row, pad_diag=0.0)).cuda()
    a0 = ap.clone()
    it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    info = cbk_gb300.dposv_refined_compact(layout, uplo, n, nrhs, ap, n, bp,
                                           (nrhs if row else n), V, nm, max_iter=max_iter,
                                           iters=it, berr=be)
    torch.cuda.synchronize()
    X = O.unpack(bp.cpu().numpy(), nm, n, nrhs, V, (nrhs if row else n), row)
    return info, X, ap.cpu().numpy(), a0.cpu().numpy(), it.cpu().numpy(), be.cpu().numpy()


def _plain_factor(A, V, layout="C", uplo="L"):
    import torch

    import cbk_gb300
    nm, n, _ = A.shape
    ap = torch.from_numpy(O.pack(A, V, n, layout == "R")).cuda()
    assert cbk_gb300.dpotrf_compact(layout, uplo, n, ap, n, V, nm) == 0
    torch.cuda.synchronize()
    return ap.cpu().numpy()


@pytest.mark.parametrize("n", [8, 16, 32, 48, 5, 12, 17, 24, 33, 40, 56, 64, 65, 70])
@pytest.mark.parametrize("layout,uplo", [("C", "L"), ("R", "U")])
def test_refined_meets_fp64_backward_error(n, layout, uplo, cuda):
    rng = np.random.default_rng(1000 + n)
    nm, nrhs, V = (200 if n <= 64 else 70), 1 if n % 2 == 0 else 2, 32
    A, kappa = C.gen_spd_cond(rng, nm, n)
    B = rng.standard_normal((nm, n, nrhs))
    info, X, a1, a0, it, be = _run(A, B, V, layout, uplo)
    assert info == 0
    berr = C.backward_error(A, X, B)
    assert (berr <= 8 * n * EPS).all(), (berr.max() / (n * EPS), kappa[berr.argmax()])
    conv = it >= 0
    fell = ~conv
    assert set(np.unique(it[fell])) <= {-1, -3}
    # converged lanes: A untouched, bit for bit
    row = layout == "R"
    A0 = O.unpack(a0, nm, n, n, V, n, row)
    A1 = O.unpack(a1, nm, n, n, V, n, row)
    assert np.array_equal(A0[conv].view(np.uint64), A1[conv].view(np.uint64))
    # fallen-back lanes: exactly the plain path's FP64 factor
    if fell.any():
        F = O.unpack(_plain_factor(A, V, layout, uplo), nm, n, n, V, n, row)
        assert np.array_equal(F[fell].view(np.uint64), A1[fell].view(np.uint64))
    # the kernel's own berr is the FP64 residual's: within rounding of ours
    assert np.isnan(be[fell]).all()
    assert (be[conv] <= 8 * n * EPS).all()
    # well-conditioned matrices converge in few corrections
    good = kappa < 1e3
    assert (it[good] >= 0).all() and (it[good] <= 3).all()
    print(f"n={n}: {conv.mean():.3f} converged, mean corrections {it[conv].mean():.2f}, "
          f"worst berr {berr.max() / EPS:.2f} eps, fallbacks {np.unique(it[fell])}")


@pytest.mark.parametrize("n", [5, 8, 16, 24, 33, 40, 48, 70])
def test_refined_exact_fp32_solution_takes_no_correction(n, cuda):
    """A diagonal of powers of two with a right-hand side exact in FP32: the
    FP32 solve is already exact, so r0 = 0 and every kernel (register, warp
    with and without the double-FP32 first residual, workspace) must accept
    x0 with zero corrections -- through the FP64 residual, since a
    double-FP32 one that is not clearly above the threshold hands the step to
    FP64 -- and return x = b / d bit for bit."""
    rng = np.random.default_rng(77 + n)
    nm, V = 96, 32
    k = 2 * rng.integers(-20, 21, size=(nm, n))          # even exponents: sqrt exact
    d = np.ldexp(1.0, k)
    A = np.zeros((nm, n, n))
    A[:, np.arange(n), np.arange(n)] = d
    B = rng.standard_normal((nm, n, 1)).astype(np.float32).astype(np.float64)
    info, X, a1, a0, it, be = _run(A, B, V)
    assert info == 0
    assert (it == 0).all(), np.unique(it)
    assert np.array_equal(X, B / d[:, :, None])
    assert (be == 0).all()


def test_refined_fallback_codes(cuda):
    """-2: an entry overflows FP32; -1: the FP32 factor breaks down
    (indefinite in FP32, SPD in FP64); -3: max_iter = 0 with an inexact FP32
    solve. Every such lane still meets the FP64 bound through the fallback."""
    rng = np.random.default_rng(7)
    n, nm, V = 8, 64, 32
    A, _ = C.gen_spd_cond(rng, nm, n, (1.0, 2.0))
    A[3] *= 1e39                       # overflows FP32
    A[4] = np.eye(n)
    A[4, 0, 0] = 1.0 + 1e-12           # exact in FP64; fine in FP32 too
    Q = C.haar(rng, 1, n)[0]
    s = np.ones(n)
    s[-1] = 1e-9                       # SPD in FP64, not positive definite in FP32
    A[5] = (Q * s) @ Q.T
    A[5] = np.tril(A[5]) + np.tril(A[5], -1).T
    B = rng.standard_normal((nm, n, 1))
    info, X, a1, a0, it, be = _run(A, B, V)
    assert info == 0
    assert it[3] == -2
    assert it[5] in (-1, -3)
    berr = C.backward_error(A, X, B)
    assert (berr <= 8 * n * EPS).all()
    # max_iter = 0: any lane whose FP32 solution is not already FP64-accurate falls back
    info, X, a1, a0, it, be = _run(A, B, V, max_iter=0)
    assert info == 0 and (it[it < 0] == -3).sum() + (it == -2).sum() + (it == -1).sum() == (it < 0).sum()
    assert (C.backward_error(A, X, B) <= 8 * n * EPS).all()


def test_refined_argument_checks(cuda):
    import cbk_gb300
    f = cbk_gb300.dposv_refined_compact
    assert f("X", "L", 8, 1, None, 8, None, 8, 32, 64) == -1
    assert f("C", "L", 8, 1, None, 8, None, 8, 32, 64, max_iter=-1) == -11
    assert f("C", "L", 70, 1, None, 70, None, 70, 32, 64, work=0, lwork=0) == -15
    assert f("C", "L", 0, 1, None, 1, None, 1, 32, 64) == 0
    assert cbk_gb300.dposv_refined_lwork(8, 1, 32, 64) == 0
    assert cbk_gb300.dposv_refined_lwork(48, 1, 32, 64) == 0  # one warp per matrix, on chip
    assert cbk_gb300.dposv_refined_lwork(70, 1, 32, 64) > 70 * 70 * 4 * 64


@pytest.mark.parametrize("n", [8, 16, 24, 48, 70])
def test_refined_results_independent_of_width(n, cuda):
    """Each matrix's arithmetic is the same whatever the interleave width: at
    V = 8, 16 and 64 (blocks of the warp kernel then straddle groups, or hold
    a group's quarter) x, iters and berr equal V = 32's bit for bit."""
    rng = np.random.default_rng(400 + n)
    nm = 150
    A, _ = C.gen_spd_cond(rng, nm, n)
    B = rng.standard_normal((nm, n, 1))
    ref = _run(A, B, 32)
    assert ref[0] == 0
    for V in (8, 16, 64):
        got = _run(A, B, V)
        assert got[0] == 0
        assert np.array_equal(got[1], ref[1]), V
        assert np.array_equal(got[4], ref[4]) and np.array_equal(got[5], ref[5]), V


def _dense(M, ld, stride, fill):
    """(nm, rows, cols) -> a flat strided column-major batch, padding = fill."""
    nm, rows, cols = M.shape
    out = np.full(nm * stride, fill)
    for k in range(nm):
        out[k * stride:k * stride + cols * ld].reshape(cols, ld)[:, :rows] = M[k].T
    return out


@pytest.mark.parametrize("n,nrhs", [(8, 1), (16, 2), (24, 1), (48, 1), (70, 1)])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_refined_batched_equals_compact(n, nrhs, uplo, cuda):
    """A strided dense batch (padded lda, ldb and strides) through
    dposv_refined_batched gives each matrix's x, iters, berr -- and, for a
    matrix that falls back, the FP64 factor -- bit-identical to the compact
    entry point's; the padding is untouched."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(70 * n + nrhs)
    nm = 75
    A, _ = C.gen_spd_cond(rng, nm, n)
    A[5] *= 1e42                                    # falls back (iters -2)
    B = rng.standard_normal((nm, n, nrhs))
    info, X, a1, a0, it, be = _run(A, B, 32, "C", uplo)
    assert info == 0 and it[5] == -2
    lda, ldb = n + 3, n + 1
    sa, sb = lda * n + 5, ldb * nrhs + 2
    ad = torch.from_numpy(_dense(A, lda, sa, 7.0)).cuda()
    bd = torch.from_numpy(_dense(B, ldb, sb, 9.0)).cuda()
    itd = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    bed = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dposv_refined_batched(uplo, n, nrhs, ad, lda, sa, bd, ldb, sb, nm,
                                           iters=itd, berr=bed) == 0
    torch.cuda.synchronize()
    bh, ah = bd.cpu().numpy(), ad.cpu().numpy()
    Xd = np.stack([bh[k * sb:k * sb + nrhs * ldb].reshape(nrhs, ldb)[:, :n].T for k in range(nm)])
    assert np.array_equal(Xd, X)
    assert np.array_equal(itd.cpu().numpy(), it)
    assert np.array_equal(bed.cpu().numpy(), be, equal_nan=True)
    # padding untouched: B's and A's gaps and the rows past n
    mb = _dense(np.zeros_like(B), ldb, sb, 1.0) == 1.0
    assert (bh[mb] == 9.0).all()
    ma = _dense(np.zeros_like(A), lda, sa, 1.0) == 1.0
    assert (ah[ma] == 7.0).all()
    # the fallen matrix holds the FP64 factor, as in the compact layout; the
    # others their input
    Ad = np.stack([ah[k * sa:k * sa + n * lda].reshape(n, lda)[:, :n].T for k in range(nm)])
    Ac = O.unpack(a1, nm, n, n, 32)
    assert np.array_equal(Ad[5], Ac[5])
    ok = it >= 0
    assert np.array_equal(Ad[ok], A[ok])


@pytest.mark.parametrize("n,nrhs,nm", [(1, 1, 5), (3, 3, 1), (64, 2, 9), (65, 1, 7), (17, 3, 33)])
def test_refined_batched_edges(n, nrhs, nm, cuda):
    """Dense batches at the edges: order 1, a single matrix, the last order of
    the warp kernel (64) and the first of the workspace kernel (65), several
    right-hand sides -- each matrix's x bit-identical to the compact path's."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(13 * n + nm)
    A, _ = C.gen_spd_cond(rng, nm, n)
    B = rng.standard_normal((nm, n, nrhs))
    info, X, a1, a0, it, be = _run(A, B, 32, "C", "L")
    assert info == 0
    lda, ldb = n + 1, n + 2
    sa, sb = lda * n + 3, ldb * nrhs
    ad = torch.from_numpy(_dense(A, lda, sa, 0.0)).cuda()
    bd = torch.from_numpy(_dense(B, ldb, sb, 0.0)).cuda()
    itd = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    assert cbk_gb300.dposv_refined_batched("L", n, nrhs, ad, lda, sa, bd, ldb, sb, nm,
                                           iters=itd) == 0
    torch.cuda.synchronize()
    bh = bd.cpu().numpy()
    Xd = np.stack([bh[k * sb:k * sb + nrhs * ldb].reshape(nrhs, ldb)[:, :n].T for k in range(nm)])
    assert np.array_equal(Xd, X) and np.array_equal(itd.cpu().numpy(), it)


@pytest.mark.parametrize("n", [16, 24, 40, 48, 64, 70])
def test_forced_fallback_is_the_plain_factor(n, cuda):
    """Matrices scaled past the FP32 range fall back (iters -2) in every
    kernel -- the lane kernel (16), the warp kernel (24 .. 64, whose inlined
    fallback sweeps its panels in memory) and the workspace kernel (70) --
    and hold exactly dpotrf_compact's factor (whose panel sweep keeps each
    row in registers) and the plain solve's x."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(400 + n)
    nm, V = 96, 32
    A, _ = C.gen_spd_cond(rng, nm, n)
    big = np.arange(0, nm, 7)
    A[big] *= 1e42
    B = rng.standard_normal((nm, n, 1))
    info, X, a1, a0, it, be = _run(A, B, V)
    assert info == 0 and (it[big] == -2).all()
    F = O.unpack(_plain_factor(A, V), nm, n, n, V, n)
    A1 = O.unpack(a1, nm, n, n, V, n)
    assert np.array_equal(F[big].view(np.uint64), A1[big].view(np.uint64))
    ap = torch.from_numpy(O.pack(A, V, n)).cuda()
    bp = torch.from_numpy(O.pack(B, V, n, pad_diag=0.0)).cuda()
    assert cbk_gb300.dposv_compact("C", "L", n, 1, ap, n, bp, n, V, nm) == 0
    torch.cuda.synchronize()
    Xp = O.unpack(bp.cpu().numpy(), nm, n, 1, V, n)
    assert np.array_equal(Xp[big].view(np.uint64), X[big].view(np.uint64))
