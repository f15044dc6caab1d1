"""Running cases on the GPU through the C ABI, and comparing (test infrastructure)."""
import numpy as np

import cases as C
from oracle import oracle as O


def run_gpu(case, stream=None):
    """Copy the case's arrays to the device, call the cbk_cuda_* entry point,
    copy back; returns (info, the case after)."""
    import torch

    import cbk_gb300
    c = case.copy()
    dev = {k: torch.from_numpy(c.kw[k]).cuda() for k in C.ARRAYS if k in c.kw}
    args = [dev[a] if a in dev else c.kw[a] for a in C.ARGS[c.routine]]
    p = "d" if c.dtype == np.float64 else "s"
    info = cbk_gb300.call(p, c.routine, *args, stream=stream)
    torch.cuda.synchronize()
    for k, t in dev.items():
        c.kw[k] = t.cpu().numpy()
    return info, c


def eps_of(dtype):
    return float(np.finfo(dtype).eps)


def order_of(case):
    kw = case.kw
    return max([1] + [kw[k] for k in ("m", "n", "k", "nrhs") if k in kw])


def lane_ratios(got, want, case):
    """Per array argument: the worst over lanes of
    max|got - want| / (max|want| * eps) over the lane's elements, padded lanes
    included. NaN positions must agree exactly and are left out of the norm."""
    V = case.kw["V"]
    nlanes = ((case.kw["nm"] + V - 1) // V) * V
    eps = eps_of(case.dtype)
    out = {}
    for name, (rows, cols, ld, row) in C.array_shapes(case).items():
        if rows == 0 or cols == 0 or nlanes == 0:
            continue
        g = O.unpack(got.kw[name], nlanes, rows, cols, V, ld, row).astype(np.float64)
        w = O.unpack(want.kw[name], nlanes, rows, cols, V, ld, row).astype(np.float64)
        gn, wn = np.isnan(g), np.isnan(w)
        if not np.array_equal(gn, wn):
            out[name] = np.inf
            continue
        g = np.where(wn, 0, g)
        w = np.where(wn, 0, w)
        d = np.abs(g - w).reshape(nlanes, -1).max(axis=1)
        s = np.abs(w).reshape(nlanes, -1).max(axis=1)
        s = np.where(s > 0, s, 1.0)
        out[name] = float((d / s).max() / eps)
    return out


def ld_padding_equal(got, orig):
    """Elements inside the leading dimension but outside the matrix -- and the
    dummy element of an empty operand -- are never written."""
    V = orig.kw["V"]
    ng = (orig.kw["nm"] + V - 1) // V
    for name, (rows, cols, ld, row) in C.array_shapes(orig).items():
        a, b = got.kw[name], orig.kw[name]
        if rows == 0 or cols == 0 or ng == 0:
            if not np.array_equal(a.view(np.uint8), b.view(np.uint8)):
                return False
            continue
        inner, outer = (cols, rows) if row else (rows, cols)
        ga = a[: ng * outer * ld * V].reshape(ng, outer, ld, V)[:, :, inner:, :]
        gb = b[: ng * outer * ld * V].reshape(ng, outer, ld, V)[:, :, inner:, :]
        if not np.array_equal(ga.view(np.uint8), gb.view(np.uint8)):
            return False
    return True


# ---------------------------------------------------------------------------
# solutions: gate by condition-scaled difference from the oracle
# ---------------------------------------------------------------------------

def _cond2(M):
    """2-norm condition number per matrix (inf for a singular one)."""
    if M.shape[-1] == 0 or M.shape[-2] == 0:
        return np.ones(M.shape[0])
    s = np.linalg.svd(M, compute_uv=False)
    with np.errstate(divide="ignore"):
        return np.where(s[:, -1] > 0, s[:, 0] / s[:, -1], np.inf)


def solution_condition(case):
    """Per lane, the condition number that bounds how far two backward-stable
    solutions of the case's system may differ: kappa(op(A)) for square and
    minimum-norm systems, kappa + kappa^2 for least squares (Wedin), of the
    triangular factor(s) for the solves. None for routines with no solution
    output. Padded lanes included (identity systems: kappa = 1)."""
    kw, r = case.kw, case.routine
    V = kw["V"]
    nl = ((kw["nm"] + V - 1) // V) * V
    row = kw["layout"] in "Rr"
    if r in ("posv", "sysvnp", "potrs", "sytrsnp"):
        n = kw["n"]
        A = O.unpack(kw["A"], nl, n, n, V, kw["lda"], row).astype(np.float64)
        if r in ("potrs", "sytrsnp"):
            L = np.tril(A, -1) if kw["uplo"] in "Ll" else np.triu(A, 1).transpose(0, 2, 1)
            d = np.einsum("kii->ki", A)
            L = L + (np.eye(n) if r == "sytrsnp" else np.einsum("ki,ij->kij", d, np.eye(n)))
            return _cond2(L) ** 2 if r == "potrs" else _cond2(L) ** 2 * _cond2(
                np.einsum("ki,ij->kij", d, np.eye(n)))
        S = np.tril(A) + np.tril(A, -1).transpose(0, 2, 1) if kw["uplo"] in "Ll" else \
            np.triu(A) + np.triu(A, 1).transpose(0, 2, 1)
        return _cond2(S)
    if r == "trsm":
        s = kw["m"] if kw["side"] in "Ll" else kw["n"]
        A = O.unpack(kw["A"], nl, s, s, V, kw["lda"], row).astype(np.float64)
        T = np.triu(A) if kw["uplo"] in "Uu" else np.tril(A)
        if kw["diag"] in "Uu":
            T = T - np.einsum("kii->ki", T)[:, :, None] * np.eye(s) + np.eye(s)
        return _cond2(T)
    if r == "gels":
        m, n = kw["m"], kw["n"]
        A = O.unpack(kw["A"], nl, m, n, V, kw["lda"], row).astype(np.float64)
        k = _cond2(A)
        overdet = (m >= n) != (kw["trans"] in "TtCc")
        return k + k * k if overdet and m != n else k
    return None


SOLUTION = {"posv": "B", "sysvnp": "B", "potrs": "B", "sytrsnp": "B", "trsm": "B", "gels": "B"}


def lane_ratios_scaled(got, want, case):
    """lane_ratios with the solution array's per-lane ratio divided by the
    lane's condition number (so the gate reads as a backward-error bound)."""
    base = {}
    V = case.kw["V"]
    nlanes = ((case.kw["nm"] + V - 1) // V) * V
    eps = eps_of(case.dtype)
    kappa = solution_condition(case)
    sol = SOLUTION.get(case.routine)
    for name, (rows, cols, ld, row) in C.array_shapes(case).items():
        if rows == 0 or cols == 0 or nlanes == 0:
            continue
        g = O.unpack(got.kw[name], nlanes, rows, cols, V, ld, row).astype(np.float64)
        w = O.unpack(want.kw[name], nlanes, rows, cols, V, ld, row).astype(np.float64)
        gn, wn = np.isnan(g), np.isnan(w)
        if not np.array_equal(gn, wn):
            base[name] = np.inf
            continue
        g = np.where(wn, 0, g)
        w = np.where(wn, 0, w)
        d = np.abs(g - w).reshape(nlanes, -1).max(axis=1)
        s = np.abs(w).reshape(nlanes, -1).max(axis=1)
        s = np.where(s > 0, s, 1.0)
        r = d / s / eps
        if name == sol and kappa is not None:
            r = r / np.maximum(kappa, 1.0)
        base[name] = float(r.max())
    return base
