"""The mixed-precision SPD solve on batches in host memory,
cbk_cuda_dposv_refined_compact_host (GPU).

The host entry point cuts the batch into chunks that pass through three
device slots with the copies pipelined; each lane is solved by the same
kernel as the device entry point's, so every output -- X in bp, A in ap
(untouched, or the FP64 factor of a lane that fell back), iters and berr --
must be bit-identical to the device entry point on the same batch, for both
layouts and triangles, leading dimensions beyond the order, several chunks and
a ragged last group.
"""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _batch(rng, nm, n, nrhs, fallbacks):
    A, _ = C.gen_spd_cond(rng, nm, n)
    if fallbacks:
        A[1] *= 1e42                    # overflows FP32: iters -2
        Q = C.haar(rng, 1, n)[0]
        s = np.ones(n)
        s[-1] = 1e-10                   # SPD in FP64, not in FP32: -1 or -3
        A[2] = (Q * s) @ Q.T
        A[2] = np.tril(A[2]) + np.tril(A[2], -1).T
        A[3, 0, 0] = np.nan             # NaN residual: -3, never "converged"
    B = rng.standard_normal((nm, n, nrhs))
    return A, B


def _both(A, B, layout, uplo, V, ldap, ldbp, pinned):
    import torch

    import cbk_gb300
    nm, n, _ = A.shape
    nrhs = B.shape[2]
    row = layout == "R"
    ap = O.pack(A, V, ldap, row)
    bp = O.pack(B, V, ldbp, row, pad_diag=0.0)
    # device entry point
    dap, dbp = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    dit = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    dbe = torch.full((nm,), -1.0, dtype=torch.float64, device="cuda")
    assert cbk_gb300.dposv_refined_compact(layout, uplo, n, nrhs, dap, ldap, dbp, ldbp, V, nm,
                                           iters=dit, berr=dbe) == 0
    torch.cuda.synchronize()
    # host entry point
    if pinned:
        hap = torch.from_numpy(ap.copy()).pin_memory()
        hbp = torch.from_numpy(bp.copy()).pin_memory()
        hit = torch.full((nm,), -99, dtype=torch.int32).pin_memory()
        hbe = torch.full((nm,), -1.0, dtype=torch.float64).pin_memory()
    else:
        hap, hbp = ap.copy(), bp.copy()
        hit = np.full(nm, -99, dtype=np.int32)
        hbe = np.full(nm, -1.0)
    assert cbk_gb300.dposv_refined_compact_host(layout, uplo, n, nrhs, hap, ldap, hbp, ldbp, V,
                                                nm, iters=hit, berr=hbe) == 0
    as_np = (lambda t: t.numpy()) if pinned else (lambda t: t)
    return ((dap.cpu().numpy(), dbp.cpu().numpy(), dit.cpu().numpy(), dbe.cpu().numpy()),
            (as_np(hap), as_np(hbp), as_np(hit), as_np(hbe)))


def _same(x, y):
    return np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("n,nm,nrhs", [(8, 20000, 1), (24, 9000, 2), (48, 9000, 1), (70, 600, 1)])
@pytest.mark.parametrize("layout,uplo", [("C", "L"), ("C", "U"), ("R", "L"), ("R", "U")])
def test_host_entry_matches_device_entry(n, nm, nrhs, layout, uplo, cuda):
    rng = np.random.default_rng(31 * n + nm)
    V = 32
    A, B = _batch(rng, nm, n, nrhs, fallbacks=True)
    row = layout == "R"
    ldap = n + 3
    ldbp = (nrhs if row else n) + 2
    dev, host = _both(A, B, layout, uplo, V, ldap, ldbp, pinned=(n != 24))
    for name, d, h in zip(("ap", "bp", "iters", "berr"), dev, host):
        assert _same(d, h), name
    it = host[2]
    assert it[1] == -2 and it[2] in (-1, -3) and it[3] < 0
    X = O.unpack(host[1], nm, n, nrhs, V, ldbp, row)
    ok = np.ones(nm, bool)
    ok[3] = False                       # the NaN matrix has no finite solution
    assert (C.backward_error(A[ok], X[ok], B[ok]) <= 8 * n * EPS).all()


def test_host_entry_argument_checks_and_workspace(cuda):
    import cbk_gb300
    f = cbk_gb300.dposv_refined_compact_host
    need = cbk_gb300.dposv_refined_host_lwork("C", 48, 1, 48, 48, 32, 9000)
    assert need > 0
    assert f("C", "L", 48, 1, None, 48, None, 48, 32, 9000, dwork=0, lwork=need - 1) == -15
    assert f("C", "L", 0, 1, None, 1, None, 1, 32, 64, dwork=0, lwork=0) == 0


def _pinned(a, offset):
    """A pinned copy of a, starting `offset` doubles into its allocation."""
    import torch
    big = torch.empty(a.size + offset, dtype=torch.float64).pin_memory()
    view = big[offset:]
    view.copy_(torch.from_numpy(a))
    return view


@pytest.mark.parametrize("a_kind,b_kind", [("pinned", "pageable"), ("pinned+8", "pinned"),
                                           ("pinned", "pinned+8"), ("pinned", "pinned")])
def test_host_entry_mixed_memory_kinds(a_kind, b_kind, cuda):
    """Every combination of pinned, pageable and pinned-but-only-8-byte-aligned
    A and B gives the device entry point's bits. The device reads a pinned,
    16-byte aligned A's triangle with 16-byte moves; a pinned A that is only
    8-byte aligned goes by the copy engine, as a pageable one does."""
    import torch

    import cbk_gb300
    rng = np.random.default_rng(77)
    n, nm, nrhs, V = 16, 12000, 1, 32
    A, B = _batch(rng, nm, n, nrhs, fallbacks=True)
    ap = O.pack(A, V, n)
    bp = O.pack(B, V, n, pad_diag=0.0)
    dap, dbp = torch.from_numpy(ap).cuda(), torch.from_numpy(bp).cuda()
    dit = torch.full((nm,), -99, dtype=torch.int32, device="cuda")
    assert cbk_gb300.dposv_refined_compact("C", "L", n, nrhs, dap, n, dbp, n, V, nm,
                                           iters=dit) == 0
    torch.cuda.synchronize()

    def host(a, kind):
        if kind == "pageable":
            return a.copy()
        return _pinned(a, 1 if kind.endswith("+8") else 0)
    hap, hbp = host(ap, a_kind), host(bp, b_kind)
    hit = np.full(nm, -99, dtype=np.int32)
    assert cbk_gb300.dposv_refined_compact_host("C", "L", n, nrhs, hap, n, hbp, n, V, nm,
                                                iters=hit) == 0
    as_np = (lambda t: t) if isinstance(hap, np.ndarray) else (lambda t: t.numpy())
    as_npb = (lambda t: t) if isinstance(hbp, np.ndarray) else (lambda t: t.numpy())
    assert _same(as_np(hap), dap.cpu().numpy())
    assert _same(as_npb(hbp), dbp.cpu().numpy())
    assert _same(hit, dit.cpu().numpy())
    assert hit[1] == -2


@pytest.mark.parametrize("pinned", [True, False])
def test_host_entry_many_chunks(pinned, cuda, monkeypatch):
    """A batch cut into many small chunks (CBK_CUDA_HOST_CHUNK_GROUPS): every
    device slot is reused several times, and chunks past the first hold lanes
    that fall back (their A comes back as the FP64 factor) -- still the device
    entry point's bits."""
    monkeypatch.setenv("CBK_CUDA_HOST_CHUNK_GROUPS", "5")
    rng = np.random.default_rng(5)
    n, nm, nrhs, V = 16, 32 * 37 + 7, 2, 32      # 38 groups: chunks of 1, 5, .., 5, 1
    A, B = _batch(rng, nm, n, nrhs, fallbacks=True)
    A[700] *= 1e42                      # group 21: iters -2
    A[1100, 3, 3] = np.nan              # group 34: iters -3
    dev, host = _both(A, B, "C", "L", V, n + 1, n, pinned=pinned)
    for name, d, h in zip(("ap", "bp", "iters", "berr"), dev, host):
        assert _same(d, h), name
    it = host[2]
    assert it[1] == -2 and it[700] == -2 and it[1100] < 0
