/* cbk_oracle_body.h -- TEST INFRASTRUCTURE (the oracle), not the product.
 *
 * The per-group algorithms of the compact batch kernels, restated in plain C
 * so that the CUDA path can be checked against them. Included by
 * cbk_oracle.c once per (scalar type T, lane-chunk width W); the macros
 *   T      the scalar type (double or float)
 *   W      the number of lanes advanced together (a compile-time constant,
 *          so every "for v < W" loop vectorises)
 *   VIEWT  the view type for T
 *   SQRT   the correctly rounded square root for T
 *   FN(x)  the name of x for this instantiation
 * must be defined. A "pack" is W consecutive scalars: element (i,j) of W
 * matrices of one compact group.
 *
 * Every function follows the reference's arithmetic element by element --
 * the same operations on each element, in the same order, with the same
 * intermediate roundings -- so that, compiled without floating-point
 * contraction, the results are bit-identical to the reference compiled the
 * same way. The reference's register tiles and column blockings change no
 * element's sequence of operations; the factorizations keep them anyway (so
 * that the CPU baseline built from this file runs as fast as the reference),
 * the solves keep only the blocking that does change an order (the single
 * trailing right-hand side of the tuned triangular solve).
 *
 * Reference files (ivan-pi/cbk v0.2.0):
 *   src/cbk_sytrfnp_compact.hpp  panel, rank-1 and rank-K updates, recursion
 *   src/cbk_potrf_compact.hpp    Cholesky panel (reordered pivot), recursion
 *   src/cbk_trsm_compact.hpp     tuned row-dot / column-axpy / strided solves
 *   src/cbk_potrs_compact.hpp, src/cbk_sytrsnp_compact.hpp  solve sweeps
 *   src/cbk_geqrf_compact.hpp    geqr2 with the branch-free larfg
 *   src/cbk_ormqr_compact.hpp    larf and the reflector sweeps
 *   src/cbk_orgqr_compact.hpp    org2r backward accumulation
 *   src/cbk_gels_compact.hpp     the four least-squares cases
 */

#define LANES for (int v = 0; v < W; ++v)

/* A(i,j) of the view: W consecutive scalars (strides si, sj are in packs of V
 * scalars; the view's p already points at this chunk's first lane). */
static inline T *FN(at)(VIEWT A, int i, int j)
{
    return A.p + ((ptrdiff_t)i * A.si + (ptrdiff_t)j * A.sj) * A.V;
}
#define AT(A, i, j) FN(at)((A), (i), (j))

static inline VIEWT FN(transposed)(VIEWT A)
{
    VIEWT t = {A.p, A.sj, A.si, A.V};
    return t;
}

/* ------------------------------------------------------------------ */
/* Cholesky and LDL^T (src/cbk_sytrfnp_compact.hpp:96-265,             */
/* src/cbk_potrf_compact.hpp:79-135)                                  */
/* ------------------------------------------------------------------ */

/* The in-panel rank-1 update of columns j+1 .. j1-1, rows c .. n-1, by the
 * unscaled pivot column j with the weight parked at A(j,j):
 * A(i,c) -= A(i,j) * (A(c,j) * A(j,j)), in blocks of four columns then one,
 * each row's A(i,j) loaded once per block (sytrfnp_update_block:96-112). */
static void FN(rank1_block)(int j, int n, VIEWT A, int jj, int jb)
{
    const T *d = AT(A, j, j);
    T w[4][W];
    for (int c = 0; c < jb; ++c) {
        const T *acj = AT(A, jj + c, j);
        LANES w[c][v] = acj[v] * d[v];
    }
    for (int c = 0; c < jb; ++c)
        for (int r = c; r < jb; ++r) {
            T *a = AT(A, jj + r, jj + c);
            const T *aj = AT(A, jj + r, j);
            LANES a[v] -= aj[v] * w[c][v];
        }
    for (int i = jj + jb; i < n; ++i) {
        const T *av = AT(A, i, j);
        for (int c = 0; c < jb; ++c) {
            T *a = AT(A, i, jj + c);
            LANES a[v] -= av[v] * w[c][v];
        }
    }
}

static void FN(rank1_panel)(int j, int j1, int n, VIEWT A)
{
    int jj = j + 1;
    for (; jj + 4 <= j1; jj += 4)
        FN(rank1_block)(j, n, A, jj, 4);
    for (; jj < j1; ++jj)
        FN(rank1_block)(j, n, A, jj, 1);
}

/* Cholesky panel with the reordered pivot (potrf_compact_panel:79-105):
 * 1/a parked on the diagonal for the rank-1 step, then d = sqrt(a) and the
 * column scaled by d * (1/a). */
static void FN(potrf_panel)(int j0, int j1, int n, VIEWT A)
{
    for (int j = j0; j < j1; ++j) {
        T *ajj = AT(A, j, j);
        T a[W], inva[W], invd[W];
        LANES a[v] = ajj[v];
        LANES inva[v] = (T)1 / a[v];
        LANES ajj[v] = inva[v];
        FN(rank1_panel)(j, j1, n, A);
        LANES {
            const T d = SQRT(a[v]);
            ajj[v] = d;
            invd[v] = d * inva[v];
        }
        for (int i = j + 1; i < n; ++i) {
            T *aij = AT(A, i, j);
            LANES aij[v] = aij[v] * invd[v];
        }
    }
}

/* LDL^T panel (sytrfnp_compact_panel:216-235): 1/d parked for the rank-1
 * step, d restored, the column scaled by 1/d. */
static void FN(ldlt_panel)(int j0, int j1, int n, VIEWT A)
{
    for (int j = j0; j < j1; ++j) {
        T *ajj = AT(A, j, j);
        T d[W], invd[W];
        LANES d[v] = ajj[v];
        LANES invd[v] = (T)1 / d[v];
        LANES ajj[v] = invd[v];
        FN(rank1_panel)(j, j1, n, A);
        LANES ajj[v] = d[v];
        for (int i = j + 1; i < n; ++i) {
            T *aij = AT(A, i, j);
            LANES aij[v] = aij[v] * invd[v];
        }
    }
}

/* One IB x JB tile of the rank-(k1-k0) update, rows i .. i+IB-1, columns
 * jj .. jj+JB-1 (diag: the tile sits on the diagonal, only r >= c exists),
 * accumulated in registers in pivot order (sytrfnp_syrk_tile:132-173):
 *   acc -= A(i,k) * (A(c,k) * D(k))   with D, or   acc -= A(i,k) * A(c,k) */
static void FN(rankk_tile)(int withd, int diag, int ib, int jb, VIEWT A, int i, int jj, int k0,
                           int k1)
{
    T acc[4][4][W];
    for (int r = 0; r < ib; ++r)
        for (int c = 0; c < jb; ++c)
            if (!diag || r >= c) {
                const T *a = AT(A, i + r, jj + c);
                LANES acc[r][c][v] = a[v];
            }
    for (int k = k0; k < k1; ++k) {
        T w[4][W];
        for (int c = 0; c < jb; ++c) {
            const T *u = AT(A, jj + c, k);
            if (withd) {
                const T *d = AT(A, k, k);
                LANES w[c][v] = u[v] * d[v];
            }
            else {
                LANES w[c][v] = u[v];
            }
        }
        for (int r = 0; r < ib; ++r) {
            const T *av = AT(A, i + r, k);
            for (int c = 0; c < jb; ++c)
                if (!diag || r >= c) LANES acc[r][c][v] -= av[v] * w[c][v];
        }
    }
    for (int r = 0; r < ib; ++r)
        for (int c = 0; c < jb; ++c)
            if (!diag || r >= c) {
                T *a = AT(A, i + r, jj + c);
                LANES a[v] = acc[r][c][v];
            }
}

/* Rank-(k1-k0) update of the lower trapezoid of columns k1 .. jend-1 by the
 * finished columns k0 .. k1-1 (sytrfnp_syrk_cols:182-191,
 * sytrfnp_trailing_update:196-209): four-column blocks, each a diagonal tile
 * then 4-row tiles then single rows; the leftover columns as one block. */
static void FN(rankk_update)(int withd, int n, int jend, VIEWT A, int k0, int k1)
{
    for (int jj = k1; jj < jend; jj += 4) {
        const int jb = (jend - jj) < 4 ? (jend - jj) : 4;
        FN(rankk_tile)(withd, 1, jb, jb, A, jj, jj, k0, k1);
        int i = jj + jb;
        for (; i + 4 <= n; i += 4)
            FN(rankk_tile)(withd, 0, 4, jb, A, i, jj, k0, k1);
        for (; i < n; ++i)
            FN(rankk_tile)(withd, 0, 1, jb, A, i, jj, k0, k1);
    }
}

/* The recursive halving at 8-column panel boundaries shared by both
 * factorizations (potrf_compact_block:112-124, sytrfnp_compact_block:242-254). */
static void FN(factor_block)(int ldlt, int j0, int j1, int n, VIEWT A)
{
    if (j1 - j0 <= 8) {
        if (ldlt)
            FN(ldlt_panel)(j0, j1, n, A);
        else
            FN(potrf_panel)(j0, j1, n, A);
        return;
    }
    const int npanels = (j1 - j0 + 7) / 8;
    const int mid = j0 + (npanels / 2) * 8;
    FN(factor_block)(ldlt, j0, mid, n, A);
    FN(rankk_update)(ldlt, n, j1, A, j0, mid);
    FN(factor_block)(ldlt, mid, j1, n, A);
}

/* ------------------------------------------------------------------ */
/* Triangular solve (src/cbk_trsm_compact.hpp:49-266)                  */
/* ------------------------------------------------------------------ */

/* Row-dot substitution of one right-hand-side column, side L, with A and B
 * both read with unit row stride: A(r,c) at a + (c*lda + r)*V, B column at b
 * (trsm_dot_block:73-104). The sum runs over l in ascending order. */
static void FN(trsm_dot_col)(int upper, int tran, int unit, int m, const T *a,
                             ptrdiff_t lda, T *b, T alpha, int V)
{
    const int back = (upper != tran);
    for (int t = 0; t < m; ++t) {
        const int i = back ? m - 1 - t : t;
        T w[W];
        T *bi = b + (ptrdiff_t)i * V;
        LANES w[v] = bi[v] * alpha;
        const int lo = back ? i + 1 : 0, hi = back ? m : i;
        for (int l = lo; l < hi; ++l) {
            const T *av = tran ? a + ((ptrdiff_t)i * lda + l) * V
                               : a + ((ptrdiff_t)l * lda + i) * V;
            const T *bl = b + (ptrdiff_t)l * V;
            LANES w[v] -= av[v] * bl[v];
        }
        if (!unit) {
            const T *d = a + ((ptrdiff_t)i * lda + i) * V;
            LANES w[v] = w[v] / d[v];
        }
        LANES bi[v] = w[v];
    }
}

/* Column-axpy substitution of the single trailing column, side L, op(A) = A
 * (trsm_axpy_col:49-67): scale by alpha, then each solved x_k is subtracted
 * from the remaining rows in sweep order. */
static void FN(trsm_axpy_col)(int upper, int unit, int m, const T *a, ptrdiff_t lda,
                              T *b, T alpha, int V)
{
    for (int i = 0; i < m; ++i) {
        T *bi = b + (ptrdiff_t)i * V;
        LANES bi[v] = bi[v] * alpha;
    }
    for (int t = 0; t < m; ++t) {
        const int kk = upper ? m - 1 - t : t;
        const T *ak = a + (ptrdiff_t)kk * lda * V;
        T *bk = b + (ptrdiff_t)kk * V;
        T xk[W];
        if (unit) {
            LANES xk[v] = bk[v];
        }
        else {
            const T *d = ak + (ptrdiff_t)kk * V;
            LANES xk[v] = bk[v] / d[v];
            LANES bk[v] = xk[v];
        }
        const int lo = upper ? 0 : kk + 1, hi = upper ? kk : m;
        for (int i = lo; i < hi; ++i) {
            T *bi = b + (ptrdiff_t)i * V;
            const T *ai = ak + (ptrdiff_t)i * V;
            LANES bi[v] -= ai[v] * xk[v];
        }
    }
}

/* The tuned side-L path (trsm_left_dot_tb:110-145): every column by the row
 * dot, except that a single column left after the 4- and 2-column blocks
 * (n % 4 odd) takes the column axpy when op(A) = A. */
static void FN(trsm_left_tuned)(int upper, int tran, int unit, int m, int n, T alpha,
                                const T *a, ptrdiff_t lda, T *b, ptrdiff_t ldb, int V)
{
    const int single = (n % 4 == 1 || n % 4 == 3);
    for (int c = 0; c < n; ++c) {
        T *bc = b + (ptrdiff_t)c * ldb * V;
        if (!tran && single && c == n - 1)
            FN(trsm_axpy_col)(upper, unit, m, a, lda, bc, alpha, V);
        else
            FN(trsm_dot_col)(upper, tran, unit, m, a, lda, bc, alpha, V);
    }
}

/* Any side and layout through the views (trsm_compact_group_strided:179-228). */
static void FN(trsm_strided)(int left, int upper, int tran, int unit, int m, int n,
                             T alpha, VIEWT A, VIEWT B)
{
    if (left) {
        const int back = (upper != tran);
        for (int j = 0; j < n; ++j)
            for (int t = 0; t < m; ++t) {
                const int i = back ? m - 1 - t : t;
                T *bij = AT(B, i, j);
                T w[W];
                LANES w[v] = bij[v] * alpha;
                const int lo = back ? i + 1 : 0, hi = back ? m : i;
                for (int l = lo; l < hi; ++l) {
                    const T *av = tran ? AT(A, l, i) : AT(A, i, l);
                    const T *blj = AT(B, l, j);
                    LANES w[v] -= av[v] * blj[v];
                }
                if (unit) {
                    LANES bij[v] = w[v];
                }
                else {
                    const T *d = AT(A, i, i);
                    LANES bij[v] = w[v] / d[v];
                }
            }
    }
    else {
        const int fwd = (upper != tran);
        for (int t = 0; t < n; ++t) {
            const int j = fwd ? t : n - 1 - t;
            for (int i = 0; i < m; ++i) {
                T *bij = AT(B, i, j);
                LANES bij[v] = bij[v] * alpha;
            }
            const int lo = fwd ? 0 : j + 1, hi = fwd ? j : n;
            for (int l = lo; l < hi; ++l) {
                const T *c = tran ? AT(A, j, l) : AT(A, l, j);
                for (int i = 0; i < m; ++i) {
                    T *bij = AT(B, i, j);
                    const T *bil = AT(B, i, l);
                    LANES bij[v] -= c[v] * bil[v];
                }
            }
            if (!unit) {
                const T *d = AT(A, j, j);
                for (int i = 0; i < m; ++i) {
                    T *bij = AT(B, i, j);
                    LANES bij[v] = bij[v] / d[v];
                }
            }
        }
    }
}

/* Route one group to the tuned or the strided solve exactly as
 * trsm_compact_group:239-254 does: side L with B's rows contiguous goes to
 * the tuned path, directly when A's rows are contiguous too, or with uplo and
 * trans flipped when A's columns are (A read as its transpose). */
static void FN(trsm_view)(int left, int upper, int tran, int unit, int m, int n, T alpha,
                          VIEWT A, VIEWT B)
{
    if (left && B.si == 1 && A.si == 1)
        FN(trsm_left_tuned)(upper, tran, unit, m, n, alpha, A.p, A.sj, B.p, B.sj, B.V);
    else if (left && B.si == 1 && A.sj == 1)
        FN(trsm_left_tuned)(!upper, !tran, unit, m, n, alpha, A.p, A.si, B.p, B.sj, B.V);
    else
        FN(trsm_strided)(left, upper, tran, unit, m, n, alpha, A, B);
}

static VIEWT FN(make_view)(T *p, int rowmajor, int ld, int V)
{
    VIEWT A;
    A.p = p;
    A.si = rowmajor ? ld : 1;
    A.sj = rowmajor ? 1 : ld;
    A.V = V;
    return A;
}

/* B(i0:i1, 0:ncols) := 0 (zero_block, src/cbk_common.hpp:301-307). */
static void FN(zero_block)(VIEWT B, int i0, int i1, int ncols)
{
    for (int j = 0; j < ncols; ++j)
        for (int i = i0; i < i1; ++i) {
            T *bij = AT(B, i, j);
            LANES bij[v] = (T)0;
        }
}

/* ------------------------------------------------------------------ */
/* Cholesky / LDL^T solves (src/cbk_potrs_compact.hpp:46-58,           */
/* src/cbk_sytrsnp_compact.hpp:51-78)                                  */
/* ------------------------------------------------------------------ */

static void FN(potrs_group)(int rowmajor, int upper, int n, int nrhs, T *a, int ldap, T *b,
                            int ldbp, int V)
{
    const VIEWT A = FN(make_view)(a, rowmajor, ldap, V);
    const VIEWT B = FN(make_view)(b, rowmajor, ldbp, V);
    FN(trsm_view)(1, upper, upper, 0, n, nrhs, (T)1, A, B);
    FN(trsm_view)(1, upper, !upper, 0, n, nrhs, (T)1, A, B);
}

static void FN(sytrsnp_group)(int rowmajor, int upper, int n, int nrhs, T *a, int ldap,
                              T *b, int ldbp, int V)
{
    const VIEWT A = FN(make_view)(a, rowmajor, ldap, V);
    const VIEWT B = FN(make_view)(b, rowmajor, ldbp, V);
    FN(trsm_view)(1, upper, upper, 1, n, nrhs, (T)1, A, B);
    for (int i = 0; i < n; ++i) {
        const T *d = AT(A, i, i);
        T invd[W];
        LANES invd[v] = (T)1 / d[v];
        for (int j = 0; j < nrhs; ++j) {
            T *bij = AT(B, i, j);
            LANES bij[v] = bij[v] * invd[v];
        }
    }
    FN(trsm_view)(1, upper, !upper, 1, n, nrhs, (T)1, A, B);
}

/* ------------------------------------------------------------------ */
/* QR family (src/cbk_geqrf_compact.hpp:74-131,                        */
/* src/cbk_ormqr_compact.hpp:68-124, src/cbk_orgqr_compact.hpp:50-87)  */
/* ------------------------------------------------------------------ */

/* Apply H(kk) = I - t v v^T (v: implicit 1 at kk, A(kk+1:len, kk) below) to
 * the slices p0 .. p1-1 of C (larf_block:68-91): w = C(kk,c) + sum A(i,kk)
 * C(i,c) in ascending i, w *= t, C(kk,c) -= w, C(i,c) -= A(i,kk) w. */
static void FN(larf)(int kk, int len, VIEWT A, const T *t, VIEWT C, int p0, int p1)
{
    for (int c = p0; c < p1; ++c) {
        T w[W];
        T *ckk = AT(C, kk, c);
        LANES w[v] = ckk[v];
        for (int i = kk + 1; i < len; ++i) {
            const T *av = AT(A, i, kk);
            const T *cic = AT(C, i, c);
            LANES w[v] += av[v] * cic[v];
        }
        LANES w[v] *= t[v];
        LANES ckk[v] -= w[v];
        for (int i = kk + 1; i < len; ++i) {
            const T *av = AT(A, i, kk);
            T *cic = AT(C, i, c);
            LANES cic[v] -= av[v] * w[v];
        }
    }
}

/* geqr2 (geqrf_reflector:95-110 with larfg_pack:74-90, group:113-131).
 * tau has a pack stride of V scalars. */
static void FN(geqrf_group)(int m, int n, VIEWT A, T *tau)
{
    const int k = m < n ? m : n;
    for (int kk = 0; kk < k; ++kk) {
        T tail[W], t[W], inv[W], rdiag[W];
        LANES tail[v] = (T)0;
        for (int i = kk + 1; i < m; ++i) {
            const T *a = AT(A, i, kk);
            LANES tail[v] += a[v] * a[v];
        }
        T *akk = AT(A, kk, kk);
        LANES {
            const T x0 = akk[v];
            const T norm = SQRT(x0 * x0 + tail[v]);
            const T beta = (x0 >= (T)0) ? -norm : norm;
            const int has = tail[v] > (T)0;
            t[v] = has ? (beta - x0) / beta : (T)0;
            inv[v] = has ? (T)1 / (x0 - beta) : (T)0;
            rdiag[v] = has ? beta : x0;
        }
        T *tk = tau + (ptrdiff_t)kk * A.V;
        LANES tk[v] = t[v];
        for (int i = kk + 1; i < m; ++i) {
            T *a = AT(A, i, kk);
            LANES a[v] = a[v] * inv[v];
        }
        LANES akk[v] = rdiag[v];
        FN(larf)(kk, m, A, t, A, kk + 1, n);
    }
}

/* One reflector sweep over all npanel slices of C (ormqr_compact_group:109-124). */
static void FN(ormqr_group)(int forward, int len, int npanel, int k, VIEWT A, const T *tau,
                            VIEWT C)
{
    for (int s = 0; s < k; ++s) {
        const int kk = forward ? s : k - 1 - s;
        FN(larf)(kk, len, A, tau + (ptrdiff_t)kk * A.V, C, 0, npanel);
    }
}

/* org2r (orgqr_compact_group:50-87). */
static void FN(orgqr_group)(int m, int n, int k, VIEWT A, const T *tau)
{
    for (int j = k; j < n; ++j) {
        for (int i = 0; i < m; ++i) {
            T *a = AT(A, i, j);
            LANES a[v] = (T)0;
        }
        T *ajj = AT(A, j, j);
        LANES ajj[v] = (T)1;
    }
    for (int kk = k - 1; kk >= 0; --kk) {
        const T *t = tau + (ptrdiff_t)kk * A.V;
        FN(larf)(kk, m, A, t, A, kk + 1, n);
        T mt[W];
        LANES mt[v] = -t[v];
        for (int i = kk + 1; i < m; ++i) {
            T *a = AT(A, i, kk);
            LANES a[v] = a[v] * mt[v];
        }
        T *akk = AT(A, kk, kk);
        LANES akk[v] = (T)1 - t[v];
        for (int i = 0; i < kk; ++i) {
            T *a = AT(A, i, kk);
            LANES a[v] = (T)0;
        }
    }
}

/* One group of the least-squares solve (gels_compact_group:84-106). */
static void FN(gels_group)(int overdet, int p, int q, int nrhs, VIEWT F, T *tau, VIEWT B)
{
    FN(geqrf_group)(p, q, F, tau);
    if (overdet) {
        FN(ormqr_group)(1, p, nrhs, q, F, tau, B);
        FN(trsm_view)(1, 1, 0, 0, q, nrhs, (T)1, F, B);
    }
    else {
        FN(trsm_view)(1, 1, 1, 0, q, nrhs, (T)1, F, B);
        FN(zero_block)(B, q, p, nrhs);
        FN(ormqr_group)(0, p, nrhs, q, F, tau, B);
    }
}

#undef LANES
#undef AT
