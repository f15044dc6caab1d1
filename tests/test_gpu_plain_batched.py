"""The plain drivers on strided dense batches (?posv_batched,
?sysvnp_batched, ?gels_batched): each matrix's outputs bit-identical to the
compact entry points' on the same matrices, the gaps between and inside the
matrices never written."""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

V = 32


def _dense(M, ld, stride, fill):
    """(nm, rows, cols) -> a flat strided column-major batch, gaps = fill."""
    nm, rows, cols = M.shape
    out = np.full(nm * stride, fill, dtype=M.dtype)
    for k in range(nm):
        out[k * stride:k * stride + cols * ld].reshape(cols, ld)[:, :rows] = M[k].T
    return out


def _undense(buf, nm, rows, cols, ld, stride):
    return np.stack([buf[k * stride:k * stride + cols * ld].reshape(cols, ld)[:, :rows].T
                     for k in range(nm)])


def _gaps(nm, rows, cols, ld, stride, dtype):
    """Mask of the elements of a strided batch outside every matrix."""
    return _dense(np.zeros((nm, rows, cols), dtype), ld, stride, 1) == 1


def _compact(p, routine, *args):
    import torch

    import cbk_gb300
    dev = [torch.from_numpy(a).cuda() if isinstance(a, np.ndarray) else a for a in args]
    info = getattr(cbk_gb300, f"{p}{routine}_compact")(*dev)
    torch.cuda.synchronize()
    return info, [d.cpu().numpy() for a, d in zip(args, dev) if isinstance(a, np.ndarray)]


def _batched(p, routine, *args):
    import torch

    import cbk_gb300
    dev = [torch.from_numpy(a).cuda() if isinstance(a, np.ndarray) else a for a in args]
    info = getattr(cbk_gb300, f"{p}{routine}_batched")(*dev)
    torch.cuda.synchronize()
    return info, [d.cpu().numpy() for a, d in zip(args, dev) if isinstance(a, np.ndarray)]


def _strides(rows, cols, pad):
    ld = max(1, rows) + (3 if pad else 0)
    return ld, ld * cols + (5 if pad else 0)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("routine", ["posv", "sysvnp"])
@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 2), (8, 1), (9, 3), (16, 1), (33, 2), (12, 0)])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("pad", [False, True])
def test_sym_batched_equals_compact(dtype, routine, n, nrhs, uplo, pad, cuda):
    """Cholesky (the register kernel up to n = 8, the generic one beyond) and
    LDL^T without pivoting: x and the factor bit-identical; nrhs = 0 factors."""
    rng = np.random.default_rng(1000 * n + 10 * nrhs + (routine == "sysvnp"))
    nm = 37
    gen = C.gen_spd if routine == "posv" else C.gen_sym_ldlt
    A = gen(rng, nm, n, dtype)
    B = rng.standard_normal((nm, n, nrhs)).astype(dtype)
    p = "d" if dtype == np.float64 else "s"
    info, (ac, bc) = _compact(p, routine, "C", uplo, n, nrhs, O.pack(A, V), n,
                              O.pack(B, V, ld=n), n, V, nm)
    assert info == 0
    lda, sa = _strides(n, n, pad)
    ldb, sb = _strides(n, nrhs, pad)
    fa, fb = dtype(7), dtype(9)
    info, (ad, bd) = _batched(p, routine, uplo, n, nrhs, _dense(A, lda, sa, fa), lda, sa,
                              _dense(B, ldb, sb, fb), ldb, sb, nm)
    assert info == 0
    assert np.array_equal(_undense(ad, nm, n, n, lda, sa), O.unpack(ac, nm, n, n, V))
    assert (ad[_gaps(nm, n, n, lda, sa, dtype)] == fa).all()
    if nrhs:
        assert np.array_equal(_undense(bd, nm, n, nrhs, ldb, sb), O.unpack(bc, nm, n, nrhs, V, n))
        assert (bd[_gaps(nm, n, nrhs, ldb, sb, dtype)] == fb).all()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,trans", [(12, 5, "N"), (12, 5, "T"), (5, 12, "N"), (5, 12, "T"),
                                       (64, 16, "N"), (40, 40, "T"), (33, 70, "N")])
@pytest.mark.parametrize("pad", [False, True])
def test_gels_batched_equals_compact(dtype, m, n, trans, pad, cuda):
    """QR / LQ least squares and minimum norm, with the blocked (compact-WY)
    QR from 32 rows on: the factors, tau and the solution bit-identical."""
    rng = np.random.default_rng(100 * m + n + (trans == "T"))
    nm, nrhs, mx, k = 35, 2, max(m, n), min(m, n)
    A = C.gen_boosted(rng, nm, m, n, dtype)
    B = rng.standard_normal((nm, mx, nrhs)).astype(dtype)
    p = "d" if dtype == np.float64 else "s"
    tauc = np.zeros(((nm + V - 1) // V) * V * k, dtype)
    info, (ac, bc, tc) = _compact(p, "gels", "C", trans, m, n, nrhs, O.pack(A, V), m,
                                  O.pack(B, V, ld=mx), mx, tauc, V, nm)
    assert info == 0
    lda, sa = _strides(m, n, pad)
    ldb, sb = _strides(mx, nrhs, pad)
    fa, fb = dtype(7), dtype(9)
    info, (ad, bd, td) = _batched(p, "gels", trans, m, n, nrhs, _dense(A, lda, sa, fa), lda, sa,
                                  _dense(B, ldb, sb, fb), ldb, sb, np.zeros(nm * k, dtype), nm)
    assert info == 0
    assert np.array_equal(_undense(ad, nm, m, n, lda, sa), O.unpack(ac, nm, m, n, V))
    assert np.array_equal(_undense(bd, nm, mx, nrhs, ldb, sb), O.unpack(bc, nm, mx, nrhs, V, mx))
    assert np.array_equal(td.reshape(nm, k), O.unpack_tau(tc, nm, k, V))
    assert (ad[_gaps(nm, m, n, lda, sa, dtype)] == fa).all()
    assert (bd[_gaps(nm, mx, nrhs, ldb, sb, dtype)] == fb).all()


@pytest.mark.parametrize("p", ["d", "s"])
def test_gels_batched_empty_factor_zeroes_b(p, cuda):
    """min(m, n) = 0 with nrhs > 0: B's max(m, n) x nrhs block is set to zero
    (the LAPACK quick return), its gaps untouched."""
    dtype = np.float64 if p == "d" else np.float32
    nm, m, n, nrhs = 9, 6, 0, 2
    ldb, sb = 8, 8 * nrhs + 3
    b = np.full(nm * sb, dtype(5))
    info, (bd,) = _batched(p, "gels", "N", m, n, nrhs, None, m, 0, b, ldb, sb, None, nm)
    assert info == 0
    mask = _gaps(nm, m, nrhs, ldb, sb, dtype)
    assert (bd[~mask] == 0).all() and (bd[mask] == 5).all()


def test_batched_on_nondefault_stream(cuda):
    """The entry points run on the stream they are given."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(3)
    nm, n = 50, 16
    A = C.gen_spd(rng, nm, n, np.float64)
    B = rng.standard_normal((nm, n, 1))
    info, (ac, bc) = _compact("d", "posv", "C", "L", n, 1, O.pack(A, V), n, O.pack(B, V, ld=n), n,
                              V, nm)
    s = torch.cuda.Stream()
    ad = torch.from_numpy(_dense(A, n, n * n, 0.0)).cuda()
    bd = torch.from_numpy(_dense(B, n, n, 0.0)).cuda()
    torch.cuda.synchronize()
    assert cbk_gb300.dposv_batched("L", n, 1, ad, n, n * n, bd, n, n, nm, stream=s) == 0
    s.synchronize()
    assert np.array_equal(_undense(bd.cpu().numpy(), nm, n, 1, n, n), O.unpack(bc, nm, n, 1, V))
