"""The autotuner on the GPU: it measures, keeps a valid winner in the table,
and no launch shape it can pick changes a result (bit-identical outputs for
every threads-per-block choice and every block shape of the warp-per-matrix
refined solve)."""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture
def tune():
    import cbk_gb300
    cbk_gb300.tune_reset()
    yield cbk_gb300
    cbk_gb300.tune_reset()


@pytest.mark.parametrize("routine,prec,m,n,nrhs", [
    ("posv", "d", 16, 16, 1), ("sysvnp", "s", 12, 12, 2), ("geqrf", "d", 16, 8, 0),
    ("gels", "d", 16, 8, 4), ("orgqr", "s", 16, 8, 0), ("posv_refined", "d", 48, 48, 1),
    ("posv_refined", "d", 8, 8, 1)])
def test_autotune_picks_a_measured_shape(tune, routine, prec, m, n, nrhs, cuda):
    info, r = tune.autotune(routine, prec, m, n, nrhs, 4096)
    assert info == 0
    assert r["vlen"] in (32, 64, 128) and r["ms"] > 0
    warp = routine == "posv_refined" and 16 < n <= 64
    if warp:
        assert r["variant"] in (0, 1, 2, 3) and r["threads"] == 0
    elif routine == "posv_refined":
        assert r["threads"] in (32, 64, 128)
    else:
        assert r["threads"] in (64, 128, 256)
    key = m if routine in ("geqrf", "ormqr", "orgqr", "gels") else n
    assert tune.tune_get(routine, prec, key)[1] == {k: r[k] for k in ("threads", "variant", "vlen")}


def _solve(tune, A, B, V, refined):
    import torch
    nm, n, _ = A.shape
    ap = torch.from_numpy(O.pack(A, V)).cuda()
    bp = torch.from_numpy(O.pack(B, V, pad_diag=0.0)).cuda()
    if refined:
        it = torch.empty(nm, dtype=torch.int32, device="cuda")
        assert tune.dposv_refined_compact("C", "L", n, 1, ap, n, bp, n, V, nm, iters=it) == 0
    else:
        assert tune.dposv_compact("C", "L", n, 1, ap, n, bp, n, V, nm) == 0
    torch.cuda.synchronize()
    return ap.cpu().numpy(), bp.cpu().numpy()


@pytest.mark.parametrize("n", [8, 24, 48, 61])
def test_launch_shape_never_changes_results(tune, n, cuda):
    rng = np.random.default_rng(n)
    A, _ = C.gen_spd_cond(rng, 3000, n)
    B = rng.standard_normal((3000, n, 1))
    outs = []
    for t in (64, 128, 256):
        assert tune.tune_set("posv", "d", n, threads=t) == 0
        outs.append(_solve(tune, A, B, 32, refined=False))
    for o in outs[1:]:
        assert all(np.array_equal(x, y) for x, y in zip(outs[0], o))
    outs = []
    for shape in ((64, 0), (256, 0), (0, 0), (0, 1), (0, 2), (0, 3)):
        assert tune.tune_set("posv_refined", "d", n, threads=shape[0], variant=shape[1]) == 0
        outs.append(_solve(tune, A, B, 32, refined=True))
    for o in outs[1:]:
        assert all(np.array_equal(x, y) for x, y in zip(outs[0], o))


@pytest.mark.parametrize("routine", ["sysvnp_bucketed", "posv_bucketed"])
def test_bucketed_grid_is_tuned_and_never_changes_results(tune, routine, cuda):
    """The bucketed launch's persistent grid (variant v: one wave of warps
    halved v times) is measured and stored at the largest order; every
    variant gives the same bits."""
    import torch
    info, r = tune.autotune(routine, "d", 24, 24, 2, 4096)
    assert info == 0 and r["variant"] in (0, 1, 2, 3) and r["threads"] == 0 and r["ms"] > 0
    assert tune.tune_get(routine, "d", 24)[1]["variant"] == r["variant"]
    rng = np.random.default_rng(5)
    V, bks, host = 32, [], []
    for n, nm in ((24, 300), (13, 500), (4, 900)):
        A = C.gen_sym_ldlt(rng, nm, n, np.float64) if routine.startswith("sysvnp") else \
            C.gen_spd(rng, nm, n, np.float64)
        host.append((n, nm, O.pack(A, V), O.pack(rng.standard_normal((nm, n, 2)), V,
                                                  pad_diag=0.0)))
    outs = []
    for v in (0, 1, 2, 3):
        assert tune.tune_set(routine, "d", 24, variant=v) == 0
        dev = [(n, nm, torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
               for n, nm, a, b in host]
        bks = [(n, nm, V, a, n, b, n) for n, nm, a, b in dev]
        assert tune.bucketed_compact(routine.split("_")[0], "d", "C", "L", 2, bks) == 0
        torch.cuda.synchronize()
        outs.append([(a.cpu().numpy(), b.cpu().numpy()) for _, _, a, b in dev])
    for o in outs[1:]:
        assert all(np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
                   for x, y in zip(outs[0], o))


def test_warp_block_shape_is_searched_and_applied(tune, cuda):
    """The warp-per-matrix refined solve's block shape (variant 0: four
    matrices per block, 1: the same at a lower register cap, 2: two matrices,
    3: one) is a tuning dimension: the autotuner times all four at the order
    and stores one; a shape set in the table is the one the next launch uses
    -- its kernel runs (the grid follows the shape) and the solution is the
    bits of every other shape, with every matrix converged."""
    import torch
    info, r = tune.autotune_at("posv_refined", "d", 32, 32, 1, 16384, 32)
    assert info == 0 and r["variant"] in (0, 1, 2, 3) and r["vlen"] == 32
    assert tune.tune_get("posv_refined", "d", 32)[1]["variant"] == r["variant"]
    rng = np.random.default_rng(32)
    A, _ = C.gen_spd_cond(rng, 777, 32)
    B = rng.standard_normal((777, 32, 1))
    ref = None
    for v in (3, 2, 1, 0):
        assert tune.tune_set("posv_refined", "d", 32, variant=v) == 0
        assert tune.tune_get("posv_refined", "d", 32)[1]["variant"] == v
        ap = torch.from_numpy(O.pack(A, 32)).cuda()
        bp = torch.from_numpy(O.pack(B, 32, pad_diag=0.0)).cuda()
        it = torch.empty(777, dtype=torch.int32, device="cuda")
        assert tune.dposv_refined_compact("C", "L", 32, 1, ap, 32, bp, 32, 32, 777, iters=it) == 0
        torch.cuda.synchronize()
        assert int(it.min()) >= 0
        got = bp.cpu().numpy()
        if ref is None:
            ref = got
        assert np.array_equal(got, ref), v
