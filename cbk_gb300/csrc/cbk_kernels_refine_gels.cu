// cbk_kernels_refine_gels.cu -- mixed-precision least squares: FP32 QR, FP64
// iterative refinement of the augmented system, per-matrix FP64 fallback.
//
// No counterpart in the reference (src/cbk_gels_compact.hpp is FP64 or FP32
// throughout). Per lane of the compact batch, for the overdetermined
// min ||b - A x|| (trans 'N', m >= n):
//   * A is rounded to FP32 and factored A = Q [R; 0] in FP32 (geqr2, the
//     plain path's code in single precision);
//   * per right-hand side, x0 = R^-1 (Q^T b)(0:n) and r0 = b - A x0 (FP64);
//     then refinement of the augmented system [I A; A^T 0][r; x] = [b; 0]
//     (Bjorck): the FP64 residuals f = b - r - A x and g = -A^T r, and the
//     correction from the FP32 QR -- h = R^-T g, [f1; f2] = Q^T f,
//     dx = R^-1 (f1 - h), dr = Q [h; f2] -- until both residuals are at the
//     FP64 rounding level of their terms: ||g|| <= sqrt(n) eps64 ||A||
//     (||A|| ||x|| + ||b|| + ||r||) and ||f|| <= sqrt(n) eps64 (||A|| ||x|| +
//     ||b|| + ||r||). Its rate is kappa(A) eps32 per step whatever the size of
//     the least-squares residual (semi-normal equations would square kappa).
//   * a lane whose FP32 rounding overflows (iters -2) or whose refinement
//     stalls or exceeds max_iter (-3) is solved by the plain FP64 path on its
//     own A and on the right-hand sides not yet solved; A and tau then hold
//     the FP64 QR. A converged lane leaves A and tau untouched.
// On exit B(0:n, c) holds x; B(n:m, c) holds (Q^T r)(n:m) for the final FP64
// residual r rounded through the FP32 Q, whose squared norm is the residual
// sum of squares to FP32 accuracy. berr[idx] is the largest normal-equations
// residual ||A^T (b - A x)||_inf / (||A||_inf (||A||_inf ||x||_inf + ||b||_inf))
// over the lane's right-hand sides (NaN for a lane that fell back).
//
// The FP64 work per right-hand side and step is 2 m n fused multiply-adds
// (f and g read A once, together), against 2 m n^2 - 2 n^3 / 3 flops for the
// FP64 QR that all right-hand sides share: refinement saves FP64 work only
// while nrhs * steps stays below about n / 2.
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <float.h>
#include <math.h>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr double EPS64 = 2.220446049250313e-16;
constexpr int GELS_NMAX = 64;

struct GelsWork {
    float *a;   // m x n FP32 QR per lane, compact, ld = m
    float *tau; // n per lane
    float *w;   // m per lane: the FP32 right-hand side of a correction
    double *r;  // m per lane: the FP64 residual estimate
};

__global__ void __launch_bounds__(128, 4)
    k_gels_refined(bool row, int m, int n, int nrhs, double *ap, int ldap, double *bp, int ldbp,
                   double *taup, int V, long ngroups, size_t sa, size_t sb, GelsWork w,
                   int max_iter, int *iters, double *berr, int nm)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    const long idx = ln.g * V + ln.v;
    const LV<double> A = lv_make<double>(ap + ln.g * sa + ln.v, row, ldap, V, m, n);
    const LV<double> B = lv_make<double>(bp + ln.g * sb + ln.v, row, ldbp, V, m, nrhs);
    double *tau64 = taup + ln.g * ((size_t)n * V) + ln.v;
    const LV<float> Q =
        lv_make<float>(w.a + ln.g * ((size_t)m * n * V) + ln.v, false, m, V, m, n);
    float *t32 = w.tau + ln.g * ((size_t)n * V) + ln.v;
    float *W = w.w + ln.g * ((size_t)m * V) + ln.v;
    double *R = w.r + ln.g * ((size_t)m * V) + ln.v;
    const LV<float> Wv = lv_make<float>(W, false, m, V, m, 1); // the work vector, m x 1

    int status = 0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) {
            const double a = A(i, j);
            if (fabs(a) > (double)FLT_MAX) status = -2;
            Q(i, j) = (float)a;
        }
    float anorm = 0.f; // ||A||_inf from the FP32 copy: a scale for the reported error
    for (int i = 0; i < m; ++i) {
        float rs = 0.f;
        for (int j = 0; j < n; ++j)
            rs += fabsf(Q(i, j));
        anorm = fmaxf(anorm, rs);
    }
    if (status == 0) geqrf_lane<float>(m, n, Q, t32, V);
    const double cte = EPS64 * sqrt((double)n);
    int it_max = 0, col = 0;
    float worst = 0.f;
    double x[GELS_NMAX];
    for (; col < nrhs && status == 0; ++col) {
        // x0 = R^-1 (Q^T b)(0:n) in FP32
        float bn = 0.f;
        for (int i = 0; i < m; ++i) {
            W[(long)i * V] = (float)B(i, col);
            bn = fmaxf(bn, fabsf(W[(long)i * V]));
        }
        ormqr_lane<float>(true, m, 1, n, Q, t32, V, Wv);
        trsm_lane<float>(true, true, false, false, n, 1, 1.0f, Q, Wv);
        for (int j = 0; j < n; ++j)
            x[j] = (double)W[(long)j * V];
        // r0 = b - A x0 (FP64)
        for (int i = 0; i < m; ++i) {
            double acc = B(i, col);
            for (int j = 0; j < n; ++j)
                acc = fma(-A(i, j), x[j], acc);
            R[(long)i * V] = acc;
        }
        // residual-based stopping, as LAPACK's mixed-precision solvers stop:
        // x is accepted once both residuals of the augmented system are at the
        // FP64 rounding level of their terms -- g = -A^T r (the normal
        // equations) and f = b - r - A x (r consistent with x). The size of
        // the correction is no test: it floors at kappa eps64 ||x||.
        float gprev = INFINITY, fprev = INFINITY;
        for (int it = 0;; ++it) {
            // f = b - r - A x and g = -A^T r, reading A once
            double g[GELS_NMAX];
            for (int j = 0; j < n; ++j)
                g[j] = 0.0;
            float fn = 0.f, rn = 0.f, xn = 0.f;
            for (int i = 0; i < m; ++i) {
                const double ri = R[(long)i * V];
                double acc = B(i, col) - ri;
                for (int j = 0; j < n; ++j) {
                    const double a = A(i, j);
                    acc = fma(-a, x[j], acc);
                    g[j] = fma(-a, ri, g[j]);
                }
                const float fi = (float)acc;
                W[(long)i * V] = fi;
                fn = fmax_nan(fn, fabsf(fi));
                rn = fmaxf(rn, fabsf((float)ri));
            }
            float h[GELS_NMAX];
            float gn = 0.f;
            for (int j = 0; j < n; ++j) {
                h[j] = (float)g[j];
                gn = fmax_nan(gn, fabsf(h[j]));
                xn = fmaxf(xn, fabsf((float)x[j]));
            }
            const double scale = (double)anorm * xn + bn;
            if ((double)gn <= cte * (double)anorm * (scale + rn) &&
                (double)fn <= cte * (scale + rn)) {
                const float den = anorm * (anorm * xn + bn);
                worst = fmaxf(worst, den > 0.f ? gn / den : 0.f);
                it_max = max(it_max, it);
                break;
            }
            if (it >= max_iter || (gn > 0.5f * gprev && fn > 0.5f * fprev)) {
                status = -3;
                break;
            }
            gprev = gn;
            fprev = fn;
            // the correction from the FP32 QR: h := R^-T g (forward
            // substitution with the upper R), W := Q^T f = [f1; f2],
            // dx = R^-1 (f1 - h), dr = Q [h; f2]
            for (int i = 0; i < n; ++i) {
                float s = h[i];
                for (int l = 0; l < i; ++l)
                    s = fmaf(-Q(l, i), h[l], s);
                h[i] = s / Q(i, i);
            }
            ormqr_lane<float>(true, m, 1, n, Q, t32, V, Wv);
            float dx[GELS_NMAX];
            for (int i = n - 1; i >= 0; --i) {
                float s = W[(long)i * V] - h[i];
                for (int l = i + 1; l < n; ++l)
                    s = fmaf(-Q(i, l), dx[l], s);
                dx[i] = s / Q(i, i);
            }
            for (int j = 0; j < n; ++j)
                x[j] += (double)dx[j];
            for (int j = 0; j < n; ++j)
                W[(long)j * V] = h[j];
            ormqr_lane<float>(false, m, 1, n, Q, t32, V, Wv);
            for (int i = 0; i < m; ++i)
                R[(long)i * V] += (double)W[(long)i * V];
        }
        if (status == 0) {
            // B(0:n) := x; B(n:m) := (Q^T r)(n:m), the residual's coordinates
            for (int i = 0; i < m; ++i)
                W[(long)i * V] = (float)R[(long)i * V];
            ormqr_lane<float>(true, m, 1, n, Q, t32, V, Wv);
            for (int j = 0; j < n; ++j)
                B(j, col) = x[j];
            for (int i = n; i < m; ++i)
                B(i, col) = (double)W[(long)i * V];
        }
    }
    if (status != 0)
        gels_fallback_lane(m, n, nrhs, status == -3 ? col - 1 : 0, A, tau64, V, B);
    if (idx < nm) {
        if (iters) iters[idx] = status != 0 ? status : it_max;
        if (berr) berr[idx] = status != 0 ? (double)NAN : (double)worst;
    }
}

inline size_t align256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

} // namespace

size_t gels_refined_lwork(int m, int n, int nrhs, int V, int nm)
{
    (void)nrhs;
    if (nm <= 0 || m <= 0 || n <= 0) return 0;
    const size_t lanes = (size_t)((nm + V - 1) / V) * V;
    return align256(lanes * (size_t)m * n * sizeof(float)) +
           align256(lanes * (size_t)n * sizeof(float)) + align256(lanes * (size_t)m * sizeof(float)) +
           align256(lanes * (size_t)m * sizeof(double));
}

int gels_refined_nmax()
{
    return GELS_NMAX;
}

cudaError_t launch_gels_refined(bool row, int m, int n, int nrhs, double *ap, int ldap, double *bp,
                                int ldbp, double *taup, int V, int nm, int max_iter, int *iters,
                                double *berr, void *work, cudaStream_t s, size_t sa_, size_t sb_)
{
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, m, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, m, nrhs, V);
    // variant 0: one warp per matrix where it is compiled; 1: one lane per matrix
    if (gels_refined_warp_ok(m, n) && variant_for(R_GELS_REFINED, n, 8) == 0)
        return launch_gels_refined_warp(row, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                        max_iter, iters, berr, s, sa, sb);
    const long ng = ((long)nm + V - 1) / V;
    const size_t lanes = (size_t)ng * V;
    char *base = static_cast<char *>(work);
    GelsWork w;
    w.a = reinterpret_cast<float *>(base);
    base += align256(lanes * (size_t)m * n * sizeof(float));
    w.tau = reinterpret_cast<float *>(base);
    base += align256(lanes * (size_t)n * sizeof(float));
    w.w = reinterpret_cast<float *>(base);
    base += align256(lanes * (size_t)m * sizeof(float));
    w.r = reinterpret_cast<double *>(base);
    const int th = 128;
    k_gels_refined<<<(unsigned)((lanes + th - 1) / th), th, 0, s>>>(
        row, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, ng, sa, sb, w, max_iter, iters, berr, nm);
    return cudaGetLastError();
}

} // namespace cbkcuda
