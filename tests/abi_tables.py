"""Argument-check tables for the C APIs (test infrastructure).

Rows of illegal arguments and of empty problems for every routine, in the
spirit of the reference's validation tables (tests/test_compact_util.hpp:
580-675, tests/test_gels_compact.cpp:181-212). Every row returns before any
array is touched -- an illegal argument (-j) or a quick return (0) -- so the
array arguments are null pointers and the rows can run anywhere, a host
without a GPU included.
"""
import numpy as np

N = None  # a null array pointer: never dereferenced by these rows


def _factor(V):
    b = dict(layout="C", uplo="L", n=8, A=N, lda=8, V=V, nm=4)
    order = ["layout", "uplo", "n", "A", "lda", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, uplo="X"), -2), (dict(b, n=-1), -3),
        (dict(b, lda=7), -5), (dict(b, V=3), -6), (dict(b, V=0), -6), (dict(b, nm=-1), -7),
        (dict(b, layout="X", n=-1), -1), (dict(b, layout="c", n=-1), -3),
        (dict(b, uplo="u", lda=0), -5), (dict(b, layout="r", V=5), -6),
        (dict(b, n=0, lda=1), 0), (dict(b, nm=0), 0), (dict(b, n=0, lda=0), -5),
    ]
    return order, rows


def _solve(V, fused):
    b = dict(layout="C", uplo="L", n=8, nrhs=3, A=N, lda=8, B=N, ldb=8, V=V, nm=4)
    order = ["layout", "uplo", "n", "nrhs", "A", "lda", "B", "ldb", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, uplo="X"), -2), (dict(b, n=-1), -3),
        (dict(b, nrhs=-1), -4), (dict(b, lda=7), -6), (dict(b, ldb=7), -8),
        (dict(b, layout="R", ldb=2), -8), (dict(b, layout="R", ldb=3, V=3), -9),
        (dict(b, V=12), -9), (dict(b, nm=-1), -10), (dict(b, n=0, lda=1, ldb=1), 0),
        (dict(b, nm=0), 0), (dict(b, uplo="U", nrhs=-2, lda=1), -4),
    ]
    if not fused:
        rows.append((dict(b, nrhs=0), 0))
    return order, rows


def _trsm(V):
    b = dict(layout="C", side="L", uplo="U", transa="N", diag="N", m=5, n=3, alpha=1.0, A=N,
             lda=5, B=N, ldb=5, V=V, nm=4)
    order = ["layout", "side", "uplo", "transa", "diag", "m", "n", "alpha", "A", "lda", "B",
             "ldb", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, side="X"), -2), (dict(b, uplo="X"), -3),
        (dict(b, transa="X"), -4), (dict(b, diag="X"), -5), (dict(b, m=-1), -6),
        (dict(b, n=-1), -7), (dict(b, lda=4), -10), (dict(b, side="R", lda=2), -10),
        (dict(b, ldb=4), -12), (dict(b, layout="R", ldb=2), -12), (dict(b, V=1), -13),
        (dict(b, nm=-1), -14), (dict(b, m=0, lda=1, ldb=1), 0), (dict(b, n=0), 0),
        (dict(b, nm=0), 0), (dict(b, transa="c", diag="u", m=-3), -6),
    ]
    return order, rows


def _geqrf(V):
    b = dict(layout="C", m=6, n=4, A=N, lda=6, tau=N, V=V, nm=4)
    order = ["layout", "m", "n", "A", "lda", "tau", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, m=-1), -2), (dict(b, n=-1), -3),
        (dict(b, lda=5), -5), (dict(b, layout="R", lda=3), -5), (dict(b, V=6), -7),
        (dict(b, nm=-1), -8), (dict(b, m=0, lda=1), 0), (dict(b, n=0), 0), (dict(b, nm=0), 0),
    ]
    return order, rows


def _ormqr(V):
    b = dict(layout="C", side="L", trans="T", m=6, n=3, k=4, A=N, lda=6, tau=N, C=N, ldc=6, V=V,
             nm=4)
    order = ["layout", "side", "trans", "m", "n", "k", "A", "lda", "tau", "C", "ldc", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, side="X"), -2), (dict(b, trans="C"), -3),
        (dict(b, trans="X"), -3), (dict(b, m=-1), -4), (dict(b, n=-1), -5), (dict(b, k=-1), -6),
        (dict(b, k=7), -6), (dict(b, side="R", k=4), -6), (dict(b, lda=5), -8),
        (dict(b, layout="R", lda=3, ldc=3), -8), (dict(b, ldc=5), -11), (dict(b, V=48), -12),
        (dict(b, nm=-1), -13), (dict(b, m=0, k=0, lda=1, ldc=1), 0), (dict(b, n=0), 0),
        (dict(b, k=0), 0), (dict(b, nm=0), 0),
    ]
    return order, rows


def _orgqr(V):
    b = dict(layout="C", m=6, n=4, k=3, A=N, lda=6, tau=N, V=V, nm=4)
    order = ["layout", "m", "n", "k", "A", "lda", "tau", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, m=-1), -2), (dict(b, n=-1), -3), (dict(b, n=7), -3),
        (dict(b, k=-1), -4), (dict(b, k=5), -4), (dict(b, lda=5), -6),
        (dict(b, layout="R", lda=3), -6), (dict(b, V=24), -8), (dict(b, nm=-1), -9),
        (dict(b, m=0, n=0, k=0, lda=1), 0), (dict(b, n=0, k=0), 0), (dict(b, nm=0), 0),
    ]
    return order, rows


def _gels(V):
    b = dict(layout="C", trans="N", m=6, n=4, nrhs=2, A=N, lda=6, B=N, ldb=6, tau=N, V=V, nm=4)
    order = ["layout", "trans", "m", "n", "nrhs", "A", "lda", "B", "ldb", "tau", "V", "nm"]
    rows = [
        (dict(b, layout="X"), -1), (dict(b, trans="X"), -2), (dict(b, m=-1), -3),
        (dict(b, n=-1), -4), (dict(b, nrhs=-1), -5), (dict(b, lda=5), -7),
        (dict(b, layout="R", lda=3, ldb=2), -7), (dict(b, ldb=5), -9),
        (dict(b, m=3, n=7, lda=3, ldb=6), -9), (dict(b, layout="R", ldb=1), -9),
        (dict(b, V=17), -11), (dict(b, nm=-1), -12), (dict(b, nrhs=0), 0), (dict(b, nm=0), 0),
        (dict(b, m=0, n=0, lda=1, ldb=1), 0), (dict(b, trans="c", nrhs=0), 0),
    ]
    return order, rows


def rows(reference_widths=False):
    """(routine, dtype, args, expected code) over every routine, both types."""
    widths = (4,) if reference_widths else (4, 32)
    out = []
    for V in widths:
        tables = {
            "potrf": _factor(V), "sytrfnp": _factor(V),
            "potrs": _solve(V, False), "sytrsnp": _solve(V, False),
            "posv": _solve(V, True), "sysvnp": _solve(V, True),
            "trsm": _trsm(V), "geqrf": _geqrf(V), "ormqr": _ormqr(V), "orgqr": _orgqr(V),
            "gels": _gels(V),
        }
        for routine, (order, rs) in tables.items():
            for dt in (np.float64, np.float32):
                for kw, code in rs:
                    out.append((routine, dt, [kw[k] for k in order], code))
    return [(r, dt, args) for r, dt, args, _ in out] if reference_widths else out


def rows_with_codes():
    return rows(reference_widths=False)
