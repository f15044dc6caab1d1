"""Uneven orders in one persistent launch (GPU).

Buckets of different orders (4 .. 48, partial last groups, several widths)
go through the bucketed entry points in one launch; every bucket must come
out bit-identical to the single-order ?sysvnp_compact / ?posv_compact call on
that bucket alone (same per-lane arithmetic), and a captured CUDA graph of the
launch must reproduce the direct call bit for bit, replay after replay.
"""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _make(rng, routine, dtype, sizes, layout, nrhs):
    row = layout == "R"
    out = []
    for k, n in enumerate(sizes):
        V = (32, 64, 8)[k % 3]
        nm = int(rng.integers(1, 150))
        if routine == "posv":
            A = C.gen_spd(rng, nm, n, dtype)
        else:
            G = rng.standard_normal((nm, n, n))
            A = ((G + G.transpose(0, 2, 1)) / 2 + 2 * n * np.eye(n)).astype(dtype)
        B = rng.standard_normal((nm, n, nrhs)).astype(dtype)
        ldb = max(1, nrhs if row else n)
        out.append(dict(n=n, nm=nm, V=V, ap=O.pack(A, V, n, row), ldap=n,
                        bp=O.pack(B, V, ldb, row, pad_diag=0.0), ldbp=ldb))
    return out


def _dev(bks):
    import torch
    return [dict(b, ap=torch.from_numpy(b["ap"]).cuda(), bp=torch.from_numpy(b["bp"]).cuda())
            for b in bks]


def _tuples(dbks):
    return [(b["n"], b["nm"], b["V"], b["ap"], b["ldap"], b["bp"], b["ldbp"]) for b in dbks]


@pytest.mark.parametrize("routine", ["sysvnp", "posv"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("layout,uplo", [("C", "L"), ("R", "U")])
def test_bucketed_equals_one_call_per_order(routine, dtype, layout, uplo, cuda):
    import torch

    import cbk_gb300
    rng = np.random.default_rng(5)
    sizes = sorted(rng.choice(np.arange(4, 49), size=12, replace=False).tolist())
    nrhs = 2
    bks = _make(rng, routine, dtype, sizes, layout, nrhs)
    p = "d" if dtype == np.float64 else "s"
    together = _dev(bks)
    assert cbk_gb300.bucketed_compact(routine, p, layout, uplo, nrhs, _tuples(together)) == 0
    alone = _dev(bks)
    for b in alone:
        assert cbk_gb300.call(p, routine, layout, uplo, b["n"], nrhs, b["ap"], b["ldap"], b["bp"],
                              b["ldbp"], b["V"], b["nm"]) == 0
    torch.cuda.synchronize()
    for x, y in zip(together, alone):
        assert torch.equal(x["ap"], y["ap"]) and torch.equal(x["bp"], y["bp"]), x["n"]


def test_bucketed_graph_replays_bit_exactly(cuda):
    import torch

    import cbk_gb300
    rng = np.random.default_rng(8)
    sizes = list(range(4, 49, 3))
    bks = _make(rng, "sysvnp", np.float64, sizes, "C", 2)
    direct = _dev(bks)
    assert cbk_gb300.bucketed_compact("sysvnp", "d", "C", "L", 2, _tuples(direct)) == 0
    staged = _dev(bks)
    work = torch.empty(cbk_gb300.BUCKETED_LWORK, dtype=torch.uint8, device="cuda")
    g = cbk_gb300.BucketedGraph("C", "L", 2, _tuples(staged), work)
    for rep in range(2):
        for b, src in zip(staged, bks):
            b["ap"].copy_(torch.from_numpy(src["ap"]))
            b["bp"].copy_(torch.from_numpy(src["bp"]))
        assert g.launch() == 0
        torch.cuda.synchronize()
        for x, y in zip(staged, direct):
            assert torch.equal(x["ap"], y["ap"]) and torch.equal(x["bp"], y["bp"]), (rep, x["n"])
    g.close()


def test_bucketed_matches_oracle(cuda, oracle_lib):
    """Each bucket against the oracle's single-order call (8 n eps relative)."""
    import torch

    import cbk_gb300
    import gpu_util as G
    rng = np.random.default_rng(9)
    bks = _make(rng, "sysvnp", np.float64, [4, 9, 17, 33, 48], "C", 2)
    dev = _dev(bks)
    assert cbk_gb300.bucketed_compact("sysvnp", "d", "C", "L", 2, _tuples(dev)) == 0
    torch.cuda.synchronize()
    for b, d in zip(bks, dev):
        case = C.Case("sysvnp", np.float64, dict(layout="C", uplo="L", n=b["n"], nrhs=2,
                                                 A=b["ap"], lda=b["ldap"], B=b["bp"],
                                                 ldb=b["ldbp"], V=b["V"], nm=b["nm"]))
        _, want = C.run(oracle_lib, case)
        got = case.copy()
        got.kw["A"] = d["ap"].cpu().numpy()
        got.kw["B"] = d["bp"].cpu().numpy()
        r = G.lane_ratios_scaled(got, want, case)
        assert all(v <= 8 * b["n"] for v in r.values()), (b["n"], r)
