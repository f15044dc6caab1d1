/* cbk_oracle.c -- TEST INFRASTRUCTURE (the oracle), not the product.
 *
 * A CPU restatement, in plain C, of ivan-pi/cbk v0.2.0's compact batch
 * kernels behind include/cbk.h: the same 22 entry points (prefixed oracle_),
 * the same LAPACK-style argument checks and quick returns (src/cbk.cpp:46-320),
 * the same per-group drivers and strides (the *_compact drivers in
 * src/cbk_*_compact.hpp), and an OpenMP loop over groups gated like
 * for_each_group (src/cbk_common.hpp:277-297).
 *
 * It exists to check the CUDA library: only the tests, the smoke check and
 * the CPU-baseline leg of the benchmark load it. Compiled with
 * -ffp-contract=off it is bit-identical to the reference compiled the same
 * way (the pin, tests/test_oracle_pin.py); the -ffp-contract=fast build is
 * the CPU baseline.
 *
 * Interleave widths: besides the reference's 2/4/8/16 it accepts any multiple
 * of 32 up to 1024 (the GPU library's widths), processing such a group in
 * chunks of 16 lanes -- lanes never interact, so the chunking changes no
 * result.
 */

#include "cbk_oracle.h"

#include <math.h>
#include <stddef.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double *p;
    ptrdiff_t si, sj;
    int V;
} dview;
typedef struct {
    float *p;
    ptrdiff_t si, sj;
    int V;
} sview;

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)

/* ---- instantiate the bodies: (double | float) x W in {2, 4, 8, 16} ---- */
#define T double
#define VIEWT dview
#define SQRT sqrt
#define W 2
#define FN(x) CAT(x, d2)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 4
#define FN(x) CAT(x, d4)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 8
#define FN(x) CAT(x, d8)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 16
#define FN(x) CAT(x, d16)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#undef T
#undef VIEWT
#undef SQRT

#define T float
#define VIEWT sview
#define SQRT sqrtf
#define W 2
#define FN(x) CAT(x, s2)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 4
#define FN(x) CAT(x, s4)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 8
#define FN(x) CAT(x, s8)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#define W 16
#define FN(x) CAT(x, s16)
#include "cbk_oracle_body.h"
#undef W
#undef FN
#undef T
#undef VIEWT
#undef SQRT

/* ------------------------------------------------------------------ */
/* argument checks (src/cbk.cpp:46-58)                                 */
/* ------------------------------------------------------------------ */

static int opt(char c, char upper)
{
    return c == upper || c == upper + ('a' - 'A');
}

static int max1(int x)
{
    return x < 1 ? 1 : x;
}

int oracle_vlen_ok(int V)
{
    if (V == 2 || V == 4 || V == 8 || V == 16) return 1;
    return V >= 32 && V <= 1024 && V % 32 == 0;
}

/* the lane-chunk width a group of V lanes is processed in */
static int chunk_width(int V)
{
    return V <= 16 ? V : 16;
}

/* scalars per group (group_stride, src/cbk_common.hpp:210-214) */
static size_t gstride(int rowmajor, int ld, int rows, int cols, int V)
{
    return (size_t)ld * (size_t)(rowmajor ? rows : cols) * (size_t)V;
}

/* The threading gate of for_each_group: a team only for two or more groups
 * and at least 5e4 flops in total. */
static int use_team(long ngroups, double flops_per_group)
{
    return ngroups > 1 && flops_per_group * (double)ngroups >= 5e4;
}

/* Run BODY(g, v0) for every group g and every lane chunk v0 of it. */
#define FOR_GROUPS_AND_CHUNKS(nm, V, flops, BODY)                                         \
    do {                                                                                 \
        const long ngroups_ = ((long)(nm) + (V) - 1) / (V);                              \
        const int W_ = chunk_width(V);                                                   \
        const int team_ = use_team(ngroups_, (flops));                                   \
        _Pragma("omp parallel for schedule(static) if (team_)")                         \
        for (long g = 0; g < ngroups_; ++g)                                              \
            for (int v0 = 0; v0 < (V); v0 += W_) {                                       \
                BODY;                                                                    \
            }                                                                            \
    } while (0)

/* dispatch a body call on the chunk width: NAME_<p><W>(args) */
#define DISPATCH_W(PFX, W_, NAME, ARGS)                                                    \
    do {                                                                                 \
        switch (W_) {                                                                    \
        case 2: NAME##_##PFX##2 ARGS; break;                                               \
        case 4: NAME##_##PFX##4 ARGS; break;                                               \
        case 8: NAME##_##PFX##8 ARGS; break;                                               \
        default: NAME##_##PFX##16 ARGS; break;                                             \
        }                                                                                \
    } while (0)

/* The entry points, generated for (double, d) and (float, s). */
#define ORACLE_ENTRY_POINTS(T, PFX, VIEWT)                                                  \
                                                                                         \
    static VIEWT PFX##mkview(T *ptr, int rowmajor, int ld, int V)                            \
    {                                                                                    \
        VIEWT A;                                                                         \
        A.p = ptr;                                                                       \
        A.si = rowmajor ? ld : 1;                                                        \
        A.sj = rowmajor ? 1 : ld;                                                        \
        A.V = V;                                                                         \
        return A;                                                                        \
    }                                                                                    \
    static VIEWT PFX##mktview(VIEWT A)                                                       \
    {                                                                                    \
        VIEWT t = {A.p, A.sj, A.si, A.V};                                                \
        return t;                                                                        \
    }                                                                                    \
                                                                                         \
    /* every group of a rows x cols batch := 0 (zero_compact) */                        \
    static void PFX##zero_all(int rowmajor, int rows, int cols, T *bp, int ldbp, int V,    \
                            int nm)                                                      \
    {                                                                                    \
        const size_t str = gstride(rowmajor, ldbp, rows, cols, V);                       \
        FOR_GROUPS_AND_CHUNKS(nm, V, (double)rows * cols * V, {                          \
            VIEWT B = PFX##mkview(bp + g * str + v0, rowmajor, ldbp, V);                     \
            DISPATCH_W(PFX, W_, zero_block, (B, 0, rows, cols));                           \
        });                                                                              \
    }                                                                                    \
                                                                                         \
    static void PFX##factor_all(int ldlt, int rowmajor, int upper, int n, T *ap, int ldap, \
                              int V, int nm)                                             \
    {                                                                                    \
        const size_t str = gstride(rowmajor, ldap, n, n, V);                             \
        FOR_GROUPS_AND_CHUNKS(nm, V, (double)n * n * n / 3.0 * V, {                      \
            VIEWT A = PFX##mkview(ap + g * str + v0, rowmajor, ldap, V);                     \
            if (upper) A = PFX##mktview(A);                                                  \
            DISPATCH_W(PFX, W_, factor_block, (ldlt, 0, n, n, A));                         \
        });                                                                              \
    }                                                                                    \
                                                                                         \
    int oracle_##PFX##geqrf_compact(char layout, int m, int n, T *ap, int ldap, T *taup,   \
                                  int V, int nm)                                         \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        if (!col && !row) return -1;                                                     \
        if (m < 0) return -2;                                                            \
        if (n < 0) return -3;                                                            \
        if (ldap < max1(row ? n : m)) return -5;                                         \
        if (!oracle_vlen_ok(V)) return -7;                                               \
        if (nm < 0) return -8;                                                           \
        if (m == 0 || n == 0 || nm == 0) return 0;                                       \
        const int k = m < n ? m : n;                                                     \
        const size_t str_a = gstride(row, ldap, m, n, V), str_t = (size_t)k * V;         \
        FOR_GROUPS_AND_CHUNKS(nm, V, 2.0 * m * n * k * V, {                              \
            VIEWT A = PFX##mkview(ap + g * str_a + v0, row, ldap, V);                        \
            DISPATCH_W(PFX, W_, geqrf_group, (m, n, A, taup + g * str_t + v0));            \
        });                                                                              \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    int oracle_##PFX##ormqr_compact(char layout, char side, char trans, int m, int n,      \
                                  int k, const T *ap, int ldap, const T *taup, T *cp,    \
                                  int ldcp, int V, int nm)                               \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        const int left = opt(side, 'L'), right = opt(side, 'R');                         \
        const int nq = left ? m : n;                                                     \
        if (!col && !row) return -1;                                                     \
        if (!left && !right) return -2;                                                  \
        if (!opt(trans, 'T') && !opt(trans, 'N')) return -3;                             \
        if (m < 0) return -4;                                                            \
        if (n < 0) return -5;                                                            \
        if (k < 0 || k > nq) return -6;                                                  \
        if (ldap < max1(row ? k : nq)) return -8;                                        \
        if (ldcp < max1(row ? n : m)) return -11;                                        \
        if (!oracle_vlen_ok(V)) return -12;                                              \
        if (nm < 0) return -13;                                                          \
        if (m == 0 || n == 0 || k == 0 || nm == 0) return 0;                             \
        const int tran = opt(trans, 'T') || opt(trans, 'C');                             \
        const int forward = (left == tran);                                              \
        const int len = left ? m : n, npanel = left ? n : m;                             \
        const size_t str_a = gstride(row, ldap, len, k, V), str_t = (size_t)k * V;       \
        const size_t str_c = gstride(row, ldcp, m, n, V);                                \
        FOR_GROUPS_AND_CHUNKS(nm, V, 4.0 * len * npanel * k * V, {                       \
            VIEWT A = PFX##mkview((T *)ap + g * str_a + v0, row, ldap, V);                   \
            VIEWT C = PFX##mkview(cp + g * str_c + v0, row, ldcp, V);                        \
            if (!left) C = PFX##mktview(C);                                                  \
            DISPATCH_W(PFX, W_, ormqr_group,                                               \
                       (forward, len, npanel, k, A, taup + g * str_t + v0, C));          \
        });                                                                              \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    int oracle_##PFX##orgqr_compact(char layout, int m, int n, int k, T *ap, int ldap,     \
                                  const T *taup, int V, int nm)                          \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        if (!col && !row) return -1;                                                     \
        if (m < 0) return -2;                                                            \
        if (n < 0 || n > m) return -3;                                                   \
        if (k < 0 || k > n) return -4;                                                   \
        if (ldap < max1(row ? n : m)) return -6;                                         \
        if (!oracle_vlen_ok(V)) return -8;                                               \
        if (nm < 0) return -9;                                                           \
        if (m == 0 || n == 0 || nm == 0) return 0;                                       \
        const size_t str_a = gstride(row, ldap, m, n, V), str_t = (size_t)k * V;         \
        FOR_GROUPS_AND_CHUNKS(nm, V, 4.0 * m * n * (k + 1) * V, {                        \
            VIEWT A = PFX##mkview(ap + g * str_a + v0, row, ldap, V);                        \
            DISPATCH_W(PFX, W_, orgqr_group, (m, n, k, A, taup + g * str_t + v0));         \
        });                                                                              \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    static int PFX##factor_api(int ldlt, char layout, char uplo, int n, T *ap, int ldap,   \
                             int V, int nm)                                              \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        const int lo = opt(uplo, 'L'), up = opt(uplo, 'U');                              \
        if (!col && !row) return -1;                                                     \
        if (!lo && !up) return -2;                                                       \
        if (n < 0) return -3;                                                            \
        if (ldap < max1(n)) return -5;                                                   \
        if (!oracle_vlen_ok(V)) return -6;                                               \
        if (nm < 0) return -7;                                                           \
        if (n == 0 || nm == 0) return 0;                                                 \
        PFX##factor_all(ldlt, row, up, n, ap, ldap, V, nm);                                \
        return 0;                                                                        \
    }                                                                                    \
    int oracle_##PFX##potrf_compact(char layout, char uplo, int n, T *ap, int ldap, int V, \
                                  int nm)                                                \
    {                                                                                    \
        return PFX##factor_api(0, layout, uplo, n, ap, ldap, V, nm);                       \
    }                                                                                    \
    int oracle_##PFX##sytrfnp_compact(char layout, char uplo, int n, T *ap, int ldap,      \
                                    int V, int nm)                                       \
    {                                                                                    \
        return PFX##factor_api(1, layout, uplo, n, ap, ldap, V, nm);                       \
    }                                                                                    \
                                                                                         \
    /* kind: 0 potrs, 1 posv, 2 sytrsnp, 3 sysvnp (sym_solve_args, cbk.cpp:173-260) */  \
    static int PFX##sym_solve(int kind, char layout, char uplo, int n, int nrhs, T *ap,    \
                            int ldap, T *bp, int ldbp, int V, int nm)                    \
    {                                                                                    \
        const int col = opt(layout, 'C'), lo = opt(uplo, 'L');                           \
        const int row = opt(layout, 'R'), up = opt(uplo, 'U');                           \
        if (!col && !row) return -1;                                                     \
        if (!lo && !up) return -2;                                                       \
        if (n < 0) return -3;                                                            \
        if (nrhs < 0) return -4;                                                         \
        if (ldap < max1(n)) return -6;                                                   \
        if (ldbp < max1(row ? nrhs : n)) return -8;                                      \
        if (!oracle_vlen_ok(V)) return -9;                                               \
        if (nm < 0) return -10;                                                          \
        const int fused = (kind == 1 || kind == 3), ldlt = (kind >= 2);                  \
        if (n == 0 || nm == 0) return 0;                                                 \
        if (!fused && nrhs == 0) return 0;                                               \
        if (fused && nrhs == 0) {                                                        \
            PFX##factor_all(ldlt, row, up, n, ap, ldap, V, nm);                            \
            return 0;                                                                    \
        }                                                                                \
        const size_t str_a = gstride(row, ldap, n, n, V);                                \
        const size_t str_b = gstride(row, ldbp, n, nrhs, V);                             \
        const double fl = ((fused ? (double)n * n * n / 3.0 : 0.0) +                     \
                           2.0 * n * n * nrhs) * V;                                      \
        FOR_GROUPS_AND_CHUNKS(nm, V, fl, {                                               \
            T *a = ap + g * str_a + v0;                                                  \
            T *b = bp + g * str_b + v0;                                                  \
            if (fused) {                                                                 \
                VIEWT A = PFX##mkview(a, row, ldap, V);                                      \
                if (up) A = PFX##mktview(A);                                                 \
                DISPATCH_W(PFX, W_, factor_block, (ldlt, 0, n, n, A));                     \
            }                                                                            \
            if (ldlt)                                                                    \
                DISPATCH_W(PFX, W_, sytrsnp_group, (row, up, n, nrhs, a, ldap, b, ldbp, V)); \
            else                                                                         \
                DISPATCH_W(PFX, W_, potrs_group, (row, up, n, nrhs, a, ldap, b, ldbp, V)); \
        });                                                                              \
        return 0;                                                                        \
    }                                                                                    \
    int oracle_##PFX##potrs_compact(char layout, char uplo, int n, int nrhs, const T *ap,  \
                                  int ldap, T *bp, int ldbp, int V, int nm)              \
    {                                                                                    \
        return PFX##sym_solve(0, layout, uplo, n, nrhs, (T *)ap, ldap, bp, ldbp, V, nm);   \
    }                                                                                    \
    int oracle_##PFX##posv_compact(char layout, char uplo, int n, int nrhs, T *ap,         \
                                 int ldap, T *bp, int ldbp, int V, int nm)               \
    {                                                                                    \
        return PFX##sym_solve(1, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm);        \
    }                                                                                    \
    int oracle_##PFX##sytrsnp_compact(char layout, char uplo, int n, int nrhs,             \
                                    const T *ap, int ldap, T *bp, int ldbp, int V,       \
                                    int nm)                                              \
    {                                                                                    \
        return PFX##sym_solve(2, layout, uplo, n, nrhs, (T *)ap, ldap, bp, ldbp, V, nm);   \
    }                                                                                    \
    int oracle_##PFX##sysvnp_compact(char layout, char uplo, int n, int nrhs, T *ap,       \
                                   int ldap, T *bp, int ldbp, int V, int nm)             \
    {                                                                                    \
        return PFX##sym_solve(3, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm);        \
    }                                                                                    \
                                                                                         \
    int oracle_##PFX##trsm_compact(char layout, char side, char uplo, char transa,         \
                                 char diag, int m, int n, T alpha, const T *ap,          \
                                 int ldap, T *bp, int ldbp, int V, int nm)               \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        const int left = opt(side, 'L'), right = opt(side, 'R');                         \
        const int up = opt(uplo, 'U'), lo = opt(uplo, 'L');                             \
        const int tran = opt(transa, 'T') || opt(transa, 'C');                           \
        const int unit = opt(diag, 'U');                                                 \
        const int s = left ? m : n;                                                      \
        if (!col && !row) return -1;                                                     \
        if (!left && !right) return -2;                                                  \
        if (!up && !lo) return -3;                                                       \
        if (!tran && !opt(transa, 'N')) return -4;                                       \
        if (!unit && !opt(diag, 'N')) return -5;                                         \
        if (m < 0) return -6;                                                            \
        if (n < 0) return -7;                                                            \
        if (ldap < max1(s)) return -10;                                                  \
        if (ldbp < max1(row ? n : m)) return -12;                                        \
        if (!oracle_vlen_ok(V)) return -13;                                              \
        if (nm < 0) return -14;                                                          \
        if (m == 0 || n == 0 || nm == 0) return 0;                                       \
        if (alpha == (T)0) {                                                             \
            PFX##zero_all(row, m, n, bp, ldbp, V, nm);                                     \
            return 0;                                                                    \
        }                                                                                \
        const size_t str_a = gstride(row, ldap, s, s, V);                                \
        const size_t str_b = gstride(row, ldbp, m, n, V);                                \
        FOR_GROUPS_AND_CHUNKS(nm, V, (double)s * s * (left ? n : m) * V, {               \
            VIEWT A = PFX##mkview((T *)ap + g * str_a + v0, row, ldap, V);                   \
            VIEWT B = PFX##mkview(bp + g * str_b + v0, row, ldbp, V);                        \
            DISPATCH_W(PFX, W_, trsm_view, (left, up, tran, unit, m, n, alpha, A, B));     \
        });                                                                              \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    int oracle_##PFX##gels_compact(char layout, char trans, int m, int n, int nrhs, T *ap, \
                                 int ldap, T *bp, int ldbp, T *taup, int V, int nm)      \
    {                                                                                    \
        const int col = opt(layout, 'C'), row = opt(layout, 'R');                        \
        const int mx = m > n ? m : n;                                                    \
        if (!col && !row) return -1;                                                     \
        if (!opt(trans, 'N') && !opt(trans, 'T') && !opt(trans, 'C')) return -2;         \
        if (m < 0) return -3;                                                            \
        if (n < 0) return -4;                                                            \
        if (nrhs < 0) return -5;                                                         \
        if (ldap < max1(row ? n : m)) return -7;                                         \
        if (ldbp < max1(row ? nrhs : mx)) return -9;                                     \
        if (!oracle_vlen_ok(V)) return -11;                                              \
        if (nm < 0) return -12;                                                          \
        if (nrhs == 0 || nm == 0 || mx == 0) return 0;                                   \
        const int tran = opt(trans, 'T') || opt(trans, 'C');                             \
        const int tall = (m >= n);                                                       \
        const int pp = tall ? m : n, q = tall ? n : m;                                   \
        const int overdet = (tall != tran);                                              \
        const size_t str_a = gstride(row, ldap, m, n, V);                                \
        const size_t str_b = gstride(row, ldbp, pp, nrhs, V);                            \
        const size_t str_t = (size_t)q * V;                                              \
        if (q == 0) {                                                                    \
            PFX##zero_all(row, pp, nrhs, bp, ldbp, V, nm);                                 \
            return 0;                                                                    \
        }                                                                                \
        FOR_GROUPS_AND_CHUNKS(                                                           \
            nm, V, (2.0 * pp * q * q + 4.0 * pp * q * nrhs + 1.0 * q * q * nrhs) * V, {  \
                VIEWT A = PFX##mkview(ap + g * str_a + v0, row, ldap, V);                    \
                VIEWT F = tall ? A : PFX##mktview(A);                                        \
                VIEWT B = PFX##mkview(bp + g * str_b + v0, row, ldbp, V);                    \
                DISPATCH_W(PFX, W_, gels_group,                                            \
                           (overdet, pp, q, nrhs, F, taup + g * str_t + v0, B));         \
            });                                                                          \
        return 0;                                                                        \
    }

ORACLE_ENTRY_POINTS(double, d, dview)
ORACLE_ENTRY_POINTS(float, s, sview)

int oracle_get_version(void)
{
    return 200; /* the reference version this restates: 0.2.0 */
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
