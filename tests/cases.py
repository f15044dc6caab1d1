"""Seeded input cases for the compact batch routines (test infrastructure).

A case is one call of one include/cbk.h routine: its argument list, with the
array arguments as flat compact numpy buffers. The same cases drive the
oracle-vs-reference pin, the golden fixtures and the GPU parity tests, so
every implementation sees identical inputs.

Generators follow the reference's test suites (tests/test_compact_util.hpp):
gen_spd (A = M^T M + n I, :338-366), gen_sym_ldlt-style symmetric matrices
with a known-good unpivoted LDL^T (:376-399), gen_tri (:423-434), gen_boosted
(:317-324) and known_solution (X(:,j) = j+1, :252-260), with numpy's PCG64 in
place of mt19937_64 (the draws need only be fixed, not the same).
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np

from oracle import oracle as O

# argument names per routine, in include/cbk.h order
ARGS = {
    "geqrf": ["layout", "m", "n", "A", "lda", "tau", "V", "nm"],
    "ormqr": ["layout", "side", "trans", "m", "n", "k", "A", "lda", "tau", "C", "ldc", "V", "nm"],
    "orgqr": ["layout", "m", "n", "k", "A", "lda", "tau", "V", "nm"],
    "potrf": ["layout", "uplo", "n", "A", "lda", "V", "nm"],
    "sytrfnp": ["layout", "uplo", "n", "A", "lda", "V", "nm"],
    "potrs": ["layout", "uplo", "n", "nrhs", "A", "lda", "B", "ldb", "V", "nm"],
    "posv": ["layout", "uplo", "n", "nrhs", "A", "lda", "B", "ldb", "V", "nm"],
    "sytrsnp": ["layout", "uplo", "n", "nrhs", "A", "lda", "B", "ldb", "V", "nm"],
    "sysvnp": ["layout", "uplo", "n", "nrhs", "A", "lda", "B", "ldb", "V", "nm"],
    "trsm": ["layout", "side", "uplo", "transa", "diag", "m", "n", "alpha", "A", "lda", "B",
             "ldb", "V", "nm"],
    "gels": ["layout", "trans", "m", "n", "nrhs", "A", "lda", "B", "ldb", "tau", "V", "nm"],
}
ARRAYS = {"A", "B", "C", "tau"}


@dataclass
class Case:
    routine: str
    dtype: type
    kw: dict
    dense: dict = field(default_factory=dict)  # the dense inputs, for checks

    def args(self):
        return [self.kw[a] for a in ARGS[self.routine]]

    def copy(self):
        return Case(self.routine, self.dtype, copy.deepcopy(self.kw), self.dense)

    @property
    def label(self):
        skip = ARRAYS | {"nm"}
        parts = [f"{k}={v}" for k, v in self.kw.items() if k not in skip]
        return f"{self.routine}[{np.dtype(self.dtype).name} {' '.join(parts)} nm={self.kw['nm']}]"


def run(lib, case: Case) -> tuple[int, Case]:
    """Run a copy of the case on a CbkLib; returns (info, the case after)."""
    c = case.copy()
    info = lib.call(c.routine, c.dtype, *c.args())
    return info, c


def outputs_equal(a: Case, b: Case) -> bool:
    """Bit-for-bit equality of every array argument (NaNs compare by bits)."""
    for k in ARRAYS:
        if k in a.kw:
            x, y = a.kw[k], b.kw[k]
            ui = np.uint64 if x.dtype == np.float64 else np.uint32
            if x.shape != y.shape or not np.array_equal(x.view(ui), y.view(ui)):
                return False
    return True


# ---------------------------------------------------------------------------
# generators
# ---------------------------------------------------------------------------

def _rng(seed):
    return np.random.default_rng(seed)


def gen_spd(rng, nm, n, dtype, cond=0.0):
    """A = M^T M + n I with M uniform(-1,1); cond > 0 squeezes the spectrum by
    the congruence D A D, D = diag(10^(-cond i/(n-1))); mirrored to be exactly
    symmetric."""
    M = rng.uniform(-1, 1, (nm, n, n))
    A = M.transpose(0, 2, 1) @ M + n * np.eye(n)
    if cond > 0 and n > 1:
        d = 10.0 ** (-cond * np.arange(n) / (n - 1))
        A = A * d[None, :, None] * d[None, None, :]
    A = np.tril(A) + np.tril(A, -1).transpose(0, 2, 1)
    return A.astype(dtype)


def gen_sym_ldlt(rng, nm, n, dtype):
    """Symmetric indefinite A = L D L^T with unit-lower L (entries in
    (-0.5, 0.5)) and |D| in [0.5, 2.5) of mixed sign (D(1) < 0)."""
    L = np.tril(rng.uniform(-0.5, 0.5, (nm, n, n)), -1) + np.eye(n)
    mag = 0.5 + 2.0 * np.abs(rng.uniform(-1, 1, (nm, n)))
    sgn = np.where(rng.uniform(-1, 1, (nm, n)) < 0, -1.0, 1.0)
    if n > 1:
        sgn[:, 1] = -1.0
    D = mag * sgn
    A = (L * D[:, None, :]) @ L.transpose(0, 2, 1)
    A = np.tril(A) + np.tril(A, -1).transpose(0, 2, 1)
    return A.astype(dtype)


def gen_tri(rng, nm, s, upper, dtype):
    """Random triangular factor in the referenced triangle, diagonal pushed to
    2 + |u| with its sign kept, the other triangle zero."""
    A = rng.uniform(-1, 1, (nm, s, s))
    A = np.triu(A) if upper else np.tril(A)
    d = np.einsum("kii->ki", A)
    sign = np.where(d >= 0, 1.0, -1.0)
    idx = np.arange(s)
    A[:, idx, idx] = sign * (2.0 + np.abs(rng.uniform(-1, 1, (nm, s))))
    return A.astype(dtype)


def gen_boosted(rng, nm, m, n, dtype, boost=2.0):
    A = rng.uniform(-1, 1, (nm, m, n))
    k = min(m, n)
    A[:, np.arange(k), np.arange(k)] += boost
    return A.astype(dtype)


def known_solution(n, nrhs, dtype):
    return np.tile(np.arange(1, nrhs + 1, dtype=dtype), (n, 1))


def _ld(rowmajor, rows, cols, pad):
    return max(1, (cols if rowmajor else rows)) + pad


def make_case(routine, dtype=np.float64, seed=0, V=8, nm=11, layout="C", uplo="L", n=8,
              nrhs=3, m=None, k=None, side="L", trans="N", transa="N", diag="N", alpha=1.0,
              ldpad=0, cond=0.0, known_x=False):
    """Build one case. ldpad > 0 gives leading dimensions beyond the minimum."""
    rng = _rng(seed)
    row = layout in "Rr"
    kw = {"layout": layout, "V": V, "nm": nm}
    dense = {}
    if routine in ("potrf", "sytrfnp", "potrs", "posv", "sytrsnp", "sysvnp"):
        chol = routine in ("potrf", "potrs", "posv")
        A = gen_spd(rng, nm, n, dtype, cond) if chol else gen_sym_ldlt(rng, nm, n, dtype)
        lda = max(1, n) + ldpad
        Ap = O.pack(A, V, lda, row)
        if routine in ("potrs", "sytrsnp"):
            # the solve takes a real factor: the oracle's, of a well-conditioned matrix
            O.oracle().call("potrf" if chol else "sytrfnp", dtype, layout, uplo, n, Ap, lda, V,
                            nm)
        kw.update(uplo=uplo, n=n, A=Ap, lda=lda)
        dense["A"] = A
        if routine not in ("potrf", "sytrfnp"):
            if known_x:
                X = np.broadcast_to(known_solution(n, nrhs, dtype), (nm, n, nrhs))
                B = (A.astype(np.float64) @ X).astype(dtype)
                dense["X"] = np.ascontiguousarray(X)
            else:
                B = rng.standard_normal((nm, n, nrhs)).astype(dtype)
            ldb = _ld(row, n, nrhs, ldpad)
            kw.update(nrhs=nrhs, B=O.pack(B, V, ldb, row, pad_diag=0.0), ldb=ldb)
            dense["B"] = B
    elif routine == "trsm":
        m = n if m is None else m
        left = side in "Ll"
        s = m if left else n
        A = gen_tri(rng, nm, s, uplo in "Uu", dtype)
        B = rng.uniform(-1, 1, (nm, m, n)).astype(dtype)
        lda = max(1, s) + ldpad
        ldb = _ld(row, m, n, ldpad)
        kw.update(side=side, uplo=uplo, transa=transa, diag=diag, m=m, n=n, alpha=alpha,
                  A=O.pack(A, V, lda, row), lda=lda, B=O.pack(B, V, ldb, row, pad_diag=0.0),
                  ldb=ldb)
        dense.update(A=A, B=B)
    elif routine == "geqrf":
        m = n if m is None else m
        A = rng.uniform(-1, 1, (nm, m, n)).astype(dtype)
        lda = _ld(row, m, n, ldpad)
        kq = min(m, n)
        kw.update(m=m, n=n, A=O.pack(A, V, lda, row), lda=lda,
                  tau=np.full(O.compact_size(nm, kq, 1, max(1, kq), V), np.nan, dtype=dtype))
        dense["A"] = A
    elif routine == "ormqr":
        m = n if m is None else m
        left = side in "Ll"
        nq = m if left else n
        k = nq if k is None else k
        # reflectors from a real QR so that Q is orthogonal
        H = rng.uniform(-1, 1, (nm, nq, k)).astype(dtype)
        lda = _ld(row, nq, k, ldpad)
        tau = np.zeros((nm, k), dtype=dtype)
        Hp = O.pack(H, V, lda, row)
        tp = O.pack_tau(tau, V)
        O.oracle().call("geqrf", dtype, layout, nq, k, Hp, lda, tp, V, nm)
        C = rng.uniform(-1, 1, (nm, m, n)).astype(dtype)
        ldc = _ld(row, m, n, ldpad)
        kw.update(side=side, trans=trans, m=m, n=n, k=k, A=Hp, lda=lda, tau=tp,
                  C=O.pack(C, V, ldc, row, pad_diag=0.0), ldc=ldc)
        dense.update(C=C)
    elif routine == "orgqr":
        m = n if m is None else m
        k = n if k is None else k
        H = rng.uniform(-1, 1, (nm, m, n)).astype(dtype)
        lda = _ld(row, m, n, ldpad)
        Hp = O.pack(H, V, lda, row)
        tp = O.pack_tau(np.zeros((nm, max(k, 0)), dtype=dtype), V)
        if k > 0:
            O.oracle().call("geqrf", dtype, layout, m, k, Hp, lda, tp, V, nm)
        kw.update(m=m, n=n, k=k, A=Hp, lda=lda, tau=tp)
    elif routine == "gels":
        m = n if m is None else m
        A = gen_boosted(rng, nm, m, n, dtype)
        mx = max(m, n)
        rows_in = n if trans in "TtCc" else m
        B = np.zeros((nm, mx, nrhs), dtype=dtype)
        B[:, :rows_in, :] = rng.uniform(-1, 1, (nm, rows_in, nrhs))
        lda = _ld(row, m, n, ldpad)
        ldb = _ld(row, mx, nrhs, ldpad)
        kq = min(m, n)
        kw.update(trans=trans, m=m, n=n, nrhs=nrhs, A=O.pack(A, V, lda, row), lda=lda,
                  B=O.pack(B, V, ldb, row, pad_diag=0.0), ldb=ldb,
                  tau=np.full(O.compact_size(nm, kq, 1, max(1, kq), V), np.nan, dtype=dtype))
        dense.update(A=A, B=B)
    else:
        raise ValueError(routine)
    return Case(routine, dtype, kw, dense)


def sweep(V_list=(2, 4, 8, 16), dtypes=(np.float64, np.float32), quick=False):
    """The pin/golden sweep: every routine over layouts, triangles, sides,
    transposes, the small-dimension list {0,1,2,3,5} and orders that cross the
    8-column panel recursion, padded partial groups and padded leading
    dimensions."""
    cases = []
    seed = 1000
    orders = [0, 1, 2, 3, 5, 8, 9, 17] if quick else [0, 1, 2, 3, 5, 8, 9, 12, 16, 17, 24, 33]
    for dt in dtypes:
        for V in V_list:
            nm = 2 * V + 3 if V <= 16 else V + 5
            for lay in "CR":
                for up in "LU":
                    for n in orders:
                        for r in ("potrf", "sytrfnp"):
                            seed += 1
                            cases.append(make_case(r, dt, seed, V, nm, lay, up, n))
                        for nrhs in (0, 1, 2, 3, 5):
                            for r in ("potrs", "posv", "sytrsnp", "sysvnp"):
                                seed += 1
                                cases.append(make_case(r, dt, seed, V, nm, lay, up, n, nrhs,
                                                       ldpad=(seed % 2)))
                for side in "LR":
                    for up in "LU":
                        for ta in "NT":
                            for dg in "NU":
                                for (mm, nn) in ((5, 3), (8, 1), (8, 4), (1, 7), (9, 5), (0, 2)):
                                    seed += 1
                                    al = (1.0, 0.5, -2.0, 0.0)[seed % 4]
                                    cases.append(make_case("trsm", dt, seed, V, nm, lay, up, nn,
                                                           m=mm, side=side, transa=ta, diag=dg,
                                                           alpha=al, ldpad=seed % 2))
                for (mm, nn) in ((16, 8), (8, 8), (5, 9), (1, 1), (0, 3), (3, 0), (12, 5)):
                    seed += 1
                    cases.append(make_case("geqrf", dt, seed, V, nm, lay, m=mm, n=nn,
                                           ldpad=seed % 2))
                for side in "LR":
                    for tr in "NT":
                        for (mm, nn, kk) in ((16, 4, 8), (6, 9, 3), (5, 5, 5), (7, 1, 0), (4, 6, 4)):
                            seed += 1
                            if kk > (mm if side == "L" else nn):
                                continue
                            cases.append(make_case("ormqr", dt, seed, V, nm, lay, m=mm, n=nn,
                                                   k=kk, side=side, trans=tr, ldpad=seed % 2))
                for (mm, nn, kk) in ((16, 8, 8), (9, 5, 3), (4, 4, 0), (7, 7, 7), (6, 1, 1)):
                    seed += 1
                    cases.append(make_case("orgqr", dt, seed, V, nm, lay, m=mm, n=nn, k=kk,
                                           ldpad=seed % 2))
                for tr in "NT":
                    for (mm, nn, nr) in ((16, 8, 4), (8, 16, 3), (9, 9, 1), (5, 2, 2), (0, 3, 2),
                                         (4, 0, 1), (6, 4, 0), (3, 7, 5)):
                        seed += 1
                        cases.append(make_case("gels", dt, seed, V, nm, lay, m=mm, n=nn,
                                               nrhs=nr, trans=tr, ldpad=seed % 2))
    return cases


def benchmark_shapes(V=32, nm=37, dtypes=(np.float64, np.float32)):
    """The orders and shapes the benchmark configurations run at, beyond the
    sweep's orders (which stop at 33): the Cholesky solve at n = 32 and 48
    with one right-hand side (the mixed-precision solve's FP64 comparator),
    the LDL^T solve and both factorizations at n = 48, least squares at
    64 x 16 with 8 right-hand sides and 16 x 8 with 4, and the thin Q at
    16 x 8 -- both layouts and triangles, padded partial groups."""
    out = []
    seed = 9000
    for dt in dtypes:
        for lay, up in (("C", "L"), ("R", "U")):
            for n in (32, 48):
                seed += 1
                out.append(make_case("posv", dt, seed, V, nm, lay, up, n, 1))
            seed += 1
            out.append(make_case("sysvnp", dt, seed, V, nm, lay, up, 48, 2))
            seed += 1
            out.append(make_case("potrf", dt, seed, V, nm, lay, up, 48))
            seed += 1
            out.append(make_case("sytrfnp", dt, seed, V, nm, lay, up, 48))
        for lay in "CR":
            seed += 1
            out.append(make_case("gels", dt, seed, V, nm, lay, m=64, n=16, nrhs=8))
            seed += 1
            out.append(make_case("gels", dt, seed, V, nm, lay, m=16, n=8, nrhs=4))
            seed += 1
            out.append(make_case("orgqr", dt, seed, V, nm, lay, m=16, n=8, k=8))
    return out


# ---------------------------------------------------------------------------
# shapes of the array arguments, and re-interleaving a case at another width
# ---------------------------------------------------------------------------

def array_shapes(case: Case) -> dict:
    """name -> (rows, cols, ld, rowmajor) of each array argument's matrices."""
    kw, r = case.kw, case.routine
    row = kw["layout"] in "Rr"
    out = {}
    if r in ("potrf", "sytrfnp", "potrs", "posv", "sytrsnp", "sysvnp"):
        out["A"] = (kw["n"], kw["n"], kw["lda"], row)
        if "B" in kw:
            out["B"] = (kw["n"], kw["nrhs"], kw["ldb"], row)
    elif r == "trsm":
        s = kw["m"] if kw["side"] in "Ll" else kw["n"]
        out["A"] = (s, s, kw["lda"], row)
        out["B"] = (kw["m"], kw["n"], kw["ldb"], row)
    elif r == "geqrf":
        k = min(kw["m"], kw["n"])
        out["A"] = (kw["m"], kw["n"], kw["lda"], row)
        out["tau"] = (k, 1, max(1, k), False)
    elif r == "ormqr":
        nq = kw["m"] if kw["side"] in "Ll" else kw["n"]
        out["A"] = (nq, kw["k"], kw["lda"], row)
        out["tau"] = (kw["k"], 1, max(1, kw["k"]), False)
        out["C"] = (kw["m"], kw["n"], kw["ldc"], row)
    elif r == "orgqr":
        out["A"] = (kw["m"], kw["n"], kw["lda"], row)
        out["tau"] = (kw["k"], 1, max(1, kw["k"]), False)
    elif r == "gels":
        k = min(kw["m"], kw["n"])
        out["A"] = (kw["m"], kw["n"], kw["lda"], row)
        out["B"] = (max(kw["m"], kw["n"]), kw["nrhs"], kw["ldb"], row)
        out["tau"] = (k, 1, max(1, k), False)
    return out


def _repack(buf, shape, nlanes, V_from, V_to):
    rows, cols, ld, row = shape
    if rows == 0 or cols == 0:
        ng = (nlanes + V_to - 1) // V_to
        return np.zeros(max(1, ng * O.group_stride(row, ld, rows, cols, V_to)), dtype=buf.dtype)
    dense = O.unpack(buf, nlanes, rows, cols, V_from, ld, row)
    return O.pack(dense, V_to, ld, row)


def reinterleave(case: Case, V_to: int) -> Case:
    """The same batch at interleave width V_to, every lane of the original's
    groups (padded lanes included) carried over as a real matrix, so that the
    routine computes exactly the same lanes. Needs the lane count to be a
    multiple of V_to."""
    V = case.kw["V"]
    nlanes = ((case.kw["nm"] + V - 1) // V) * V
    assert nlanes % V_to == 0 or nlanes == 0
    c = case.copy()
    for name, shp in array_shapes(case).items():
        c.kw[name] = _repack(case.kw[name], shp, nlanes, V, V_to)
    c.kw["V"] = V_to
    c.kw["nm"] = nlanes
    return c


def back_to(case_out: Case, like: Case) -> Case:
    """Outputs of a reinterleave()d case, laid out as the original case."""
    V_from, V_to = case_out.kw["V"], like.kw["V"]
    nlanes = case_out.kw["nm"]
    c = like.copy()
    for name, shp in array_shapes(like).items():
        if shp[0] == 0 or shp[1] == 0:
            continue  # an empty operand is never touched: keep the original buffer
        c.kw[name] = _repack(case_out.kw[name], shp, nlanes, V_from, V_to)
        # keep the original buffer's length (a dummy element for empty operands)
        if c.kw[name].shape != like.kw[name].shape:
            fixed = like.kw[name].copy()
            fixed[: min(fixed.size, c.kw[name].size)] = c.kw[name][: fixed.size]
            c.kw[name] = fixed
    return c


def run_any_width(lib, case: Case, lib_widths=(2, 4, 8, 16)) -> tuple[int, Case]:
    """Run a case on a library that only accepts lib_widths (the reference),
    re-interleaving a wider case at 16 lanes and back."""
    V = case.kw["V"]
    if V in lib_widths:
        return run(lib, case)
    inner = reinterleave(case, 16)
    info, out = run(lib, inner)
    return info, back_to(out, case)


# ---------------------------------------------------------------------------
# conditioned SPD batches (the mixed-precision workloads)
# ---------------------------------------------------------------------------

def haar(rng, nm, n, k=None):
    """Haar-distributed orthogonal (n x n) or thin (n x k) factors: the Q of a
    Gaussian's QR with the signs of R's diagonal folded in (Mezzadri 2007)."""
    k = n if k is None else k
    G = rng.standard_normal((nm, n, k))
    Q, R = np.linalg.qr(G)
    d = np.sign(np.einsum("kii->ki", R))
    d[d == 0] = 1.0
    return Q * d[:, None, :]


def gen_spd_cond(rng, nm, n, log10_kappa=(1.0, 6.0)):
    """A = U diag(s) U^T, U Haar, s log-uniform between 1 and 1/kappa with
    log10(kappa) uniform in log10_kappa; returns (A, kappa)."""
    kappa = 10.0 ** rng.uniform(*log10_kappa, nm)
    u = np.sort(rng.uniform(0, 1, (nm, n)), axis=1)
    if n > 1:
        u[:, 0], u[:, -1] = 0.0, 1.0
    s = kappa[:, None] ** (-u)
    U = haar(rng, nm, n)
    A = (U * s[:, None, :]) @ U.transpose(0, 2, 1)
    A = np.tril(A) + np.tril(A, -1).transpose(0, 2, 1)
    return A, kappa


def backward_error(A, X, B):
    """Per matrix, the largest normwise backward error over the right-hand
    sides: ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), in float64."""
    A = A.astype(np.float64)
    X = X.astype(np.float64)
    B = B.astype(np.float64)
    R = B - A @ X
    an = np.abs(A).sum(axis=2).max(axis=1)
    rn = np.abs(R).max(axis=1)
    xn = np.abs(X).max(axis=1)
    bn = np.abs(B).max(axis=1)
    den = an[:, None] * xn + bn
    return np.where(den > 0, rn / np.where(den > 0, den, 1), 0).max(axis=1)


def gen_ls_cond(rng, nm, m, n, nrhs, log10_kappa=(1.0, 4.0), noise=1e-3):
    """A = U diag(s) V^T (U Haar m x n thin, V Haar n x n), s log-uniform with
    log10 kappa uniform in log10_kappa; B = A X + noise * N(0,1), X ~ N(0,1).
    Returns (A, B, X, kappa)."""
    kappa = 10.0 ** rng.uniform(*log10_kappa, nm)
    u = np.sort(rng.uniform(0, 1, (nm, n)), axis=1)
    if n > 1:
        u[:, 0], u[:, -1] = 0.0, 1.0
    s = kappa[:, None] ** (-u)
    U = haar(rng, nm, m, n)
    Vh = haar(rng, nm, n)
    A = (U * s[:, None, :]) @ Vh.transpose(0, 2, 1)
    X = rng.standard_normal((nm, n, nrhs))
    B = A @ X + noise * rng.standard_normal((nm, m, nrhs))
    return A, B, X, kappa
