"""The benchmark configurations at their full batch sizes (GPU), checked by
properties that hold at any size: backward errors and the normal equations
within their bounds, orthogonality, every refined matrix converged, and the
bit-identities the library promises -- fused == separate, dense batches ==
the compact layout, bucketed == one call per order. At these sizes byte
offsets into the batch pass 2^31 (A at n = 48: 4.8 GB), which the small
parity cases never reach. Inputs are made on the device from seeds (orthogonal factors by this
library's own dgeqrf/dorgqr); every check runs on the device in FP64.
"""
import pytest

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -52
V = 32


def _gen(seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return g


def _randn(g, *shape):
    import torch
    return torch.randn(*shape, dtype=torch.float64, device="cuda", generator=g)


def _pack(M):
    """(nm, rows, cols), nm a multiple of V -> compact, column-major, ld = rows."""
    nm, r, c = M.shape
    return M.reshape(nm // V, V, r, c).permute(0, 3, 2, 1).contiguous().reshape(-1)


def _unpack(buf, nm, r, c):
    return buf.view(nm // V, c, r, V).permute(0, 3, 2, 1).reshape(nm, r, c)


def _dense(M):
    """(nm, rows, cols) -> the strided dense batch (column-major, ld = rows),
    always a copy (for one column, the transposed view already counts as
    contiguous and .contiguous() would hand back M itself)."""
    import torch
    return M.transpose(1, 2).clone(memory_format=torch.contiguous_format)


def _berr(A, X, B):
    """Per matrix ||B - A X|| / (||A|| ||X|| + ||B||), infinity norms."""
    R = B - A @ X
    an = A.abs().sum(dim=2).amax(dim=1)
    return R.abs().amax(dim=(1, 2)) / (an * X.abs().amax(dim=(1, 2)) + B.abs().amax(dim=(1, 2)))


def _normal(A, X, B):
    """Per matrix ||A^T (B - A X)|| / (||A|| (||A|| ||X|| + ||B||)), infinity norms."""
    G = A.transpose(1, 2) @ (B - A @ X)
    an = A.abs().sum(dim=2).amax(dim=1)
    return G.abs().amax(dim=(1, 2)) / (an * (an * X.abs().amax(dim=(1, 2)) +
                                             B.abs().amax(dim=(1, 2))))


def _orth(g, m, n, nm):
    """Orthonormal columns (nm, m, n): the Q of a Gaussian's QR."""
    import torch

    import cbk_gb300
    gp = _pack(_randn(g, nm, m, n))
    tau = torch.empty(nm * n, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dgeqrf_compact("C", m, n, gp, m, tau, V, nm) == 0
    assert cbk_gb300.dorgqr_compact("C", m, n, n, gp, m, tau, V, nm) == 0
    return _unpack(gp, nm, m, n)


def _spread(g, nm, k, lo, hi):
    """Per matrix k values from 1 down to 1/kappa, log10 kappa uniform in
    [lo, hi], the exponents sorted uniform with both ends taken."""
    import torch
    lk = torch.empty(nm, dtype=torch.float64, device="cuda").uniform_(lo, hi, generator=g)
    u = torch.sort(torch.rand(nm, k, dtype=torch.float64, device="cuda", generator=g),
                   dim=1).values
    u[:, 0], u[:, -1] = 0, 1
    return torch.pow(10.0, -lk[:, None] * u)


def test_c1_dposv_n8_65536(cuda):
    """dposv n = 8, 65,536 matrices: backward error <= 8 n eps; posv ==
    potrf + potrs and the dense batch == the compact one, bit for bit."""
    import torch

    import cbk_gb300 as cbk
    n, nm = 8, 65536
    g = _gen(1)
    G = _randn(g, nm, n, n)
    A = G @ G.transpose(1, 2) + n * torch.eye(n, dtype=torch.float64, device="cuda")
    B = _randn(g, nm, n, 1)
    ap, bp = _pack(A), _pack(B)
    assert cbk.dposv_compact("C", "L", n, 1, ap, n, bp, n, V, nm) == 0
    ap2, bp2 = _pack(A), _pack(B)
    assert cbk.dpotrf_compact("C", "L", n, ap2, n, V, nm) == 0
    assert cbk.dpotrs_compact("C", "L", n, 1, ap2, n, bp2, n, V, nm) == 0
    ad, bd = _dense(A), _dense(B)
    assert cbk.dposv_batched("L", n, 1, ad, n, n * n, bd, n, n, nm) == 0
    torch.cuda.synchronize()
    X = _unpack(bp, nm, n, 1)
    assert float(_berr(A, X, B).max()) <= 8 * n * EPS
    assert torch.equal(ap, ap2) and torch.equal(bp, bp2)
    assert torch.equal(ad.transpose(1, 2), _unpack(ap, nm, n, n))
    assert torch.equal(bd.transpose(1, 2), X)


def test_c2_dgels_16x8_1m(cuda):
    """dgels 16 x 8, 4 right-hand sides, 1,048,576 matrices: the normal
    equations within 8 n eps; dorgqr's Q orthonormal to 8 m eps and Q R = A
    to 8 m eps ||A||_F."""
    import torch

    import cbk_gb300 as cbk
    m, n, nrhs, nm = 16, 8, 4, 1 << 20
    g = _gen(2)
    A, B = _randn(g, nm, m, n), _randn(g, nm, m, nrhs)
    ap, bp = _pack(A), _pack(B)
    tau = torch.empty(nm * n, dtype=torch.float64, device="cuda")
    assert cbk.dgels_compact("C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm) == 0
    X = _unpack(bp, nm, m, nrhs)[:, :n]
    assert float(_normal(A, X, B).max()) <= 8 * n * EPS
    R = torch.triu(_unpack(ap, nm, m, n)[:, :n, :])
    assert cbk.dorgqr_compact("C", m, n, n, ap, m, tau, V, nm) == 0
    Q = _unpack(ap, nm, m, n)
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    assert float((Q.transpose(1, 2) @ Q - eye).abs().amax()) <= 8 * m * EPS
    rel = (Q @ R - A).abs().amax(dim=(1, 2)) / torch.linalg.matrix_norm(A)
    assert float(rel.max()) <= 8 * m * EPS


@pytest.mark.parametrize("n", [8, 16, 32, 48])
def test_c3_refined_dposv_262144(n, cuda):
    """The headline workload, one order at a time: A = U diag(s) U^T with
    kappa 1e1 .. 1e6, 262,144 matrices. Every matrix converges (no FP64
    fallback), the reported and the recomputed backward errors are within
    8 n eps64, and the dense-batch entry point gives the same bits."""
    import torch

    import cbk_gb300 as cbk
    nm = 262144
    g = _gen(30 + n)
    U = _orth(g, n, n, nm)
    A = (U * _spread(g, nm, n, 1.0, 6.0)[:, None, :]) @ U.transpose(1, 2)
    del U
    A = torch.tril(A) + torch.tril(A, -1).transpose(1, 2)
    B = _randn(g, nm, n, 1)
    ap, bp = _pack(A), _pack(B)
    it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    be = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk.dposv_refined_compact("C", "L", n, 1, ap, n, bp, n, V, nm, iters=it, berr=be) == 0
    ad, bd = _dense(A), _dense(B)
    it2 = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    assert cbk.dposv_refined_batched("L", n, 1, ad, n, n * n, bd, n, n, nm, iters=it2) == 0
    torch.cuda.synchronize()
    X = _unpack(bp, nm, n, 1)
    assert int(it.min()) >= 0 and int(it.max()) <= 10
    assert float(be.max()) <= 8 * n * EPS
    assert float(_berr(A, X, B).max()) <= 8 * n * EPS
    assert torch.equal(bd.transpose(1, 2), X) and torch.equal(it2, it)


def test_c4_uneven_sysvnp_1m(cuda):
    """dsysvnp on 45 orders 4 .. 48, 23,296 matrices each (1,048,320), two
    right-hand sides, in one bucketed launch: each order bit-identical to its
    own dsysvnp_compact call, backward error within 8 n eps."""
    import torch

    import cbk_gb300 as cbk
    per, nrhs = 23296, 2
    g = _gen(4)
    orders = list(range(4, 49))
    mats, together, alone = [], [], []
    for n in orders:
        G = _randn(g, per, n, n)
        A = (G + G.transpose(1, 2)) / 2 + 2 * n * torch.eye(n, dtype=torch.float64,
                                                            device="cuda")
        B = _randn(g, per, n, nrhs)
        mats.append((A, B))
        together.append((n, per, V, _pack(A), n, _pack(B), n))
        alone.append((_pack(A), _pack(B)))
    assert cbk.bucketed_compact("sysvnp", "d", "C", "L", nrhs, together) == 0
    for n, (ap, bp) in zip(orders, alone):
        assert cbk.dsysvnp_compact("C", "L", n, nrhs, ap, n, bp, n, V, per) == 0
    torch.cuda.synchronize()
    for n, (A, B), t, (ap, bp) in zip(orders, mats, together, alone):
        assert torch.equal(t[3], ap) and torch.equal(t[5], bp), n
        assert float(_berr(A, _unpack(bp, per, n, nrhs), B).max()) <= 8 * n * EPS, n


def test_c5_refined_dgels_64x16_131072(cuda):
    """The least-squares workload: A = U diag(s) V^T with kappa 1e1 .. 1e4,
    B = A X + 1e-3 N(0,1), 64 x 16, 8 right-hand sides, 131,072 matrices.
    Every matrix converges and meets the normal equations within 8 n eps64."""
    import torch

    import cbk_gb300 as cbk
    m, n, nrhs, nm = 64, 16, 8, 131072
    g = _gen(5)
    U, W = _orth(g, m, n, nm), _orth(g, n, n, nm)
    A = (U * _spread(g, nm, n, 1.0, 4.0)[:, None, :]) @ W.transpose(1, 2)
    del U, W
    B = A @ _randn(g, nm, n, nrhs) + 1e-3 * _randn(g, nm, m, nrhs)
    ap, bp = _pack(A), _pack(B)
    tau = torch.empty(nm * n, dtype=torch.float64, device="cuda")
    it = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    assert cbk.dgels_refined_compact("C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm,
                                     iters=it) == 0
    torch.cuda.synchronize()
    X = _unpack(bp, nm, m, nrhs)[:, :n]
    assert int(it.min()) >= 0
    assert float(_normal(A, X, B).max()) <= 8 * n * EPS
