"""GPU parity: every routine of the CUDA library against the oracle (GPU).

Each case of the sweep (tests/cases.py: every routine, both precisions,
both layouts, both triangles / sides / transposes, diagonal kinds, alpha
values, orders 0..33 across the 8-column panel recursion, padded partial
groups and padded leading dimensions) runs through the C ABI on the GPU and
on the oracle with identical inputs. Gates:

  * the return code is the oracle's;
  * every output array, lane by lane (padded lanes included), agrees with the
    oracle to within the relative bound 8 * n * eps of the precision (the
    factors, tau, Q); a solution, whose difference between two backward-stable
    solves scales with the system's condition number, to within
    8 * n * eps * kappa -- the GPU rounds differently only through fused
    multiply-adds and reciprocal multiplies;
  * NaN/Inf positions agree exactly, and nothing outside the matrices (the
    leading-dimension padding, the dummy element of an empty operand) is
    written.

The golden fixtures repeat the comparison against the reference's own
outputs.
"""
import numpy as np
import pytest

import cases as C
import gpu_util as G
import make_golden

pytestmark = pytest.mark.gpu

BOUND = 8.0  # * order * eps, the relative factor-difference bound


def _check(case, got_info, got, want_info, want):
    assert got_info == want_info, (case.label, got_info, want_info)
    ratios = G.lane_ratios_scaled(got, want, case)
    bound = BOUND * G.order_of(case)
    bad = {k: r for k, r in ratios.items() if not r <= bound}
    assert not bad, f"{case.label}: ratios {bad} > {bound}"
    assert G.ld_padding_equal(got, case), f"{case.label}: wrote outside the matrices"
    return max(ratios.values(), default=0.0) / max(1, G.order_of(case))


@pytest.mark.parametrize("V,quick", [(8, True), (32, False), (64, True), (96, True)])
def test_parity_sweep(V, quick, cuda, oracle_lib):
    worst = 0.0
    cases = C.sweep(V_list=(V,), quick=quick)
    for c in cases:
        gi, g = G.run_gpu(c)
        oi, o = C.run(oracle_lib, c)
        worst = max(worst, _check(c, gi, g, oi, o))
    print(f"V={V}: {len(cases)} cases, worst ratio / order = {worst:.2f} eps")


@pytest.mark.parametrize("V,nm", [(32, 37), (8, 11)])
def test_parity_benchmark_shapes(V, nm, cuda, oracle_lib):
    """The benchmark configurations' orders and shapes (plain FP64 and FP32
    posv at n = 32 / 48, sysvnp and both factorizations at n = 48, gels at
    64 x 16 with 8 right-hand sides and 16 x 8 with 4, orgqr 16 x 8) against
    the oracle."""
    worst = 0.0
    cases = C.benchmark_shapes(V, nm)
    for c in cases:
        gi, g = G.run_gpu(c)
        oi, o = C.run(oracle_lib, c)
        worst = max(worst, _check(c, gi, g, oi, o))
    print(f"benchmark shapes V={V}: {len(cases)} cases, worst ratio / order = {worst:.2f} eps")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["C", "R"])
def test_parity_blocked_qr(dtype, layout, cuda, oracle_lib):
    """From 32 rows on the QR family applies its reflectors in compact-WY
    blocks of four: geqrf (whole blocks and a ragged last one), ormqr from
    both sides in both directions (forward and backward block order), gels
    over- and under-determined, and orgqr on the blocked QR's reflectors --
    against the oracle, which applies them one at a time."""
    worst = 0.0
    cases = []
    seed = 8100
    for mm, nn in ((40, 12), (64, 16), (33, 7), (48, 48)):
        seed += 1
        cases.append(C.make_case("geqrf", dtype, seed, 32, 37, layout, m=mm, n=nn,
                                 ldpad=seed % 2))
    for side in "LR":
        for tr in "NT":
            for (mm, nn, kk) in ((40, 5, 12), (36, 40, 9), (64, 8, 16)):
                seed += 1
                if kk > (mm if side == "L" else nn):
                    continue
                cases.append(C.make_case("ormqr", dtype, seed, 32, 37, layout, m=mm, n=nn, k=kk,
                                         side=side, trans=tr, ldpad=seed % 2))
    for tr in "NT":
        for (mm, nn, nr) in ((64, 16, 8), (40, 13, 3), (16, 48, 2)):
            seed += 1
            cases.append(C.make_case("gels", dtype, seed, 32, 37, layout, m=mm, n=nn, nrhs=nr,
                                     trans=tr, ldpad=seed % 2))
    seed += 1
    cases.append(C.make_case("orgqr", dtype, seed, 32, 37, layout, m=48, n=16, k=16))
    for c in cases:
        gi, g = G.run_gpu(c)
        oi, o = C.run(oracle_lib, c)
        worst = max(worst, _check(c, gi, g, oi, o))
    print(f"blocked QR {layout}: {len(cases)} cases, worst ratio / order = {worst:.2f} eps")


def test_parity_golden(cuda):
    worst = 0.0
    for cin, cout, info in make_golden.load():
        gi, g = G.run_gpu(cin)
        worst = max(worst, _check(cin, gi, g, info, cout))
    print(f"golden: worst ratio / order = {worst:.2f} eps")


@pytest.mark.parametrize("routine", ["potrf", "sytrfnp", "posv", "sysvnp"])
@pytest.mark.parametrize("layout,uplo", [("C", "L"), ("C", "U"), ("R", "L"), ("R", "U")])
def test_opposite_triangle_untouched(routine, layout, uplo, cuda):
    """The strictly-opposite triangle is neither read nor written, bit for bit
    (tests/test_potrf_compact.cpp:74-85)."""
    for n in (1, 5, 8, 13, 24):
        c = C.make_case(routine, np.float64, 40 + n, 32, 45, layout, uplo, n, 2)
        _, g = G.run_gpu(c)
        V, nm = 32, 45
        A0 = C.O.unpack(c.kw["A"], 64, n, n, V, c.kw["lda"], layout == "R")
        A1 = C.O.unpack(g.kw["A"], 64, n, n, V, c.kw["lda"], layout == "R")
        mask = np.triu(np.ones((n, n), bool), 1) if uplo == "L" else np.tril(np.ones((n, n), bool), -1)
        assert np.array_equal(A0[:, mask].view(np.uint64), A1[:, mask].view(np.uint64)), (routine, n)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("layout,uplo", [("C", "L"), ("R", "U"), ("C", "U"), ("R", "L")])
def test_fused_equals_separate(dtype, layout, uplo, cuda):
    """?posv == ?potrf then ?potrs and ?sysvnp == ?sytrfnp then ?sytrsnp, bit
    for bit on the whole buffers (include/cbk.h:196-212, 263-279)."""
    for n, nrhs in ((8, 1), (16, 3), (33, 5)):
        for fused, fac, sol in (("posv", "potrf", "potrs"), ("sysvnp", "sytrfnp", "sytrsnp")):
            c = C.make_case(fused, dtype, 7 * n + nrhs, 32, 70, layout, uplo, n, nrhs)
            _, f = G.run_gpu(c)
            cf = c.copy()
            cf.routine = fac
            for k in ("nrhs", "B", "ldb"):
                cf.kw.pop(k)
            _, a = G.run_gpu(cf)
            cs = c.copy()
            cs.routine = sol
            cs.kw["A"] = a.kw["A"]
            _, s = G.run_gpu(cs)
            assert C.outputs_equal(f, s), (fused, n, nrhs)


@pytest.mark.parametrize("routine", ["potrf", "posv", "sytrfnp"])
def test_bad_lane_is_confined(routine, cuda):
    """A non-SPD (or zero-pivot) lane poisons only itself with NaN/Inf; every
    sibling lane is bit-identical to a run where that lane is healthy
    (tests/test_potrf_compact.cpp:254-316), and the return code stays 0."""
    n, V, nm, bad = 12, 32, 64, 5
    c = C.make_case(routine, np.float64, 99, V, nm, "C", "L", n, 2)
    A = C.O.unpack(c.kw["A"], nm, n, n, V)
    Ab = A.copy()
    Ab[bad] = np.eye(n)
    Ab[bad, 0, 0] = -1.0 if routine != "sytrfnp" else 0.0
    cb = c.copy()
    cb.kw["A"] = C.O.pack(Ab, V)
    ig, good = G.run_gpu(c)
    ib, poisoned = G.run_gpu(cb)
    assert ig == 0 and ib == 0
    F0 = C.O.unpack(good.kw["A"], nm, n, n, V)
    F1 = C.O.unpack(poisoned.kw["A"], nm, n, n, V)
    others = [i for i in range(nm) if i != bad]
    assert np.array_equal(F0[others].view(np.uint64), F1[others].view(np.uint64))
    assert not np.isfinite(np.tril(F1[bad])).all()


def test_trsm_alpha_zero_never_reads_a(cuda):
    """alpha = 0 sets B := 0 without reading A (src/cbk_trsm_compact.hpp:284-289):
    a null A pointer is never dereferenced."""
    import torch

    import cbk_gb300
    B = torch.randn(2 * 5 * 3 * 32, dtype=torch.float64, device="cuda")
    info = cbk_gb300.dtrsm_compact("C", "L", "U", "N", "N", 5, 3, 0.0, None, 5, B, 5, 32, 40)
    torch.cuda.synchronize()
    assert info == 0 and bool((B == 0).all())


def test_gels_empty_cases(cuda):
    """nrhs = 0 leaves everything untouched; min(m,n) = 0 sets all max(m,n)
    rows of B to 0 without reading A or tau (include/cbk.h:335-340)."""
    import torch

    import cbk_gb300
    B = torch.randn(2 * 6 * 2 * 32, dtype=torch.float64, device="cuda")
    B0 = B.clone()
    assert cbk_gb300.dgels_compact("C", "N", 6, 4, 0, None, 6, B, 6, None, 32, 40) == 0
    torch.cuda.synchronize()
    assert torch.equal(B, B0)
    assert cbk_gb300.dgels_compact("C", "N", 0, 6, 2, None, 1, B, 6, None, 32, 40) == 0
    torch.cuda.synchronize()
    assert bool((B == 0).all())


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["C", "R"])
def test_pack_unpack(dtype, layout, cuda):
    """Device pack == the host pack of the reference tests (padded lanes
    carry pad_diag on the diagonal), and unpack inverts it."""
    import torch

    import cbk_gb300
    p = "d" if dtype == np.float64 else "s"
    rng = np.random.default_rng(3)
    for (m, n, V, nm, lda_pad, ldap_pad) in ((8, 8, 32, 70, 0, 0), (16, 4, 64, 33, 2, 1),
                                             (5, 7, 8, 19, 1, 3), (1, 1, 32, 1, 0, 0)):
        row = layout == "R"
        lda = (n if row else m) + lda_pad
        ldap = (n if row else m) + ldap_pad
        mats = rng.standard_normal((nm, m, n)).astype(dtype)
        dense = np.zeros((nm, (m if row else n), lda), dtype=dtype)
        if row:
            dense[:, :, :n] = mats
        else:
            dense[:, :, :m] = mats.transpose(0, 2, 1)
        stride = dense[0].size
        a = torch.from_numpy(dense.reshape(-1).copy()).cuda()
        want = C.O.pack(mats, V, ldap, row, pad_diag=0.5)
        ap = torch.full((want.size,), 0.0, dtype=a.dtype, device="cuda")
        assert cbk_gb300.call(p, "pack", layout, m, n, a, lda, stride, ap, ldap, V, nm, 0.5) == 0
        torch.cuda.synchronize()
        assert np.array_equal(ap.cpu().numpy(), want)
        back = torch.zeros_like(a)
        assert cbk_gb300.call(p, "unpack", layout, m, n, ap, ldap, back, lda, stride, V, nm) == 0
        torch.cuda.synchronize()
        got = back.cpu().numpy().reshape(dense.shape)
        got = got[:, :, :n] if row else got[:, :, :m].transpose(0, 2, 1)
        assert np.array_equal(got, mats)


def test_nondefault_stream(cuda):
    """The _async entry points run on the given stream."""
    import torch
    s = torch.cuda.Stream()
    c = C.make_case("posv", np.float64, 5, 32, 100, "C", "L", 8, 1)
    with torch.cuda.stream(s):
        gi, g = G.run_gpu(c, stream=s)
    oi, o = C.run(C.O.oracle(), c)
    _check(c, gi, g, oi, o)
