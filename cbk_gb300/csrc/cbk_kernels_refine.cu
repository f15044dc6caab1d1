// cbk_kernels_refine.cu -- mixed-precision SPD solve: FP32 Cholesky, FP64
// iterative refinement, per-matrix FP64 fallback.
//
// No counterpart in the reference (whose solves are FP64 or FP32 throughout,
// src/cbk_posv_compact.hpp); the method is LAPACK dsposv's, per lane of the
// compact batch:
//   1. A (FP64, the lower triangle of the view) is rounded to FP32 -- a lane
//      whose entries overflow FP32 falls back (iters = -2) -- and factored in
//      FP32 -- a lane with a non-positive FP32 pivot falls back (iters = -1);
//   2. per right-hand side: x = solve32(b); then repeat r = b - A x in FP64,
//      stop when ||r||_inf <= sqrt(n) eps64 ||A||_inf ||x||_inf (dsposv's
//      test), else x += solve32(fl32(r)); a lane falls back (iters = -3) when
//      max_iter corrections did not converge or a correction failed to halve
//      the residual (refinement stalled);
//   3. a lane that falls back runs the plain FP64 path's factor and solve on
//      its own A and on the right-hand sides not yet solved: A then holds the
//      FP64 factor (as dsposv leaves it); a converged lane leaves A untouched.
// iters[idx] = corrections used (max over the right-hand sides), or the
// negative fallback code; berr[idx] = the largest normwise backward error
// ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) of the lane's solutions,
// from the FP64 residual of the accepted x (NaN for a lane that fell back).
//
// On a GB300 the FP64 pipe runs at ~1/58 of the FP32 rate, so the FP64 work
// per right-hand side falls from n^3/6 + n^2 fused multiply-adds and 2n long
// operations to n^2 per refinement step.
//
// Three variants: orders up to 16 keep the FP32 factor and x in registers
// (compile-time order, one thread per matrix, below); orders 17 .. 64 run one
// warp per matrix with the matrix staged in shared memory
// (cbk_kernels_refine_warp.cu); larger orders keep the FP32 factor, x and the
// correction in the caller's workspace, in the compact layout (coalesced),
// sized by cbk_cuda_dposv_refined_compact_lwork.
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <algorithm>

#include "../../include/cbk_cuda.h"

#include <mutex>
#include <float.h>
#include <math.h>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr double EPS64 = 2.220446049250313e-16;
constexpr int REG_NMAX = 16;
// orders whose first residual is taken in double-FP32 arithmetic (above it
// the register kernel has no registers to spare for it: measured slower)
constexpr int FF_NMAX = 8;

// packed lower-triangle index (column-major), i >= j
__host__ __device__ constexpr int tix(int i, int j, int N)
{
    return j * (2 * N - j + 1) / 2 + (i - j);
}


// The exact FP32-range test of the lower triangle (the rare path after a
// quick screen; not inlined, so that it takes no registers from the caller).
__device__ __noinline__ bool any_beyond_fp32(int n, LV<double> A)
{
    bool any = false;
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i)
            any |= beyond_fp32(A(i, j));
    return any;
}

struct RefineOut {
    int *iters;
    double *berr;
    int nm;
    int max_iter;
};

// The FP64 fallback of one lane: factor A in place (the plain path's
// arithmetic) and solve columns first .. nrhs-1 of B. Not inlined: the rare
// path keeps its registers out of the refinement loop's budget.
__device__ __noinline__ void fallback_lane(int n, int nrhs, int first, LV<double> A, LV<double> B)
{
    factor_lane<double, false>(n, A);
    if (first < nrhs) {
        const LV<double> Bs = lv_from_col(B, first);
        sym_solve_lane<double, false>(n, nrhs - first, A, Bs);
    }
}

__device__ __forceinline__ void write_status(const RefineOut &o, long idx, int status, int it,
                                             double berr)
{
    if (idx >= o.nm) return; // padded lanes compute but report nothing
    if (o.iters) o.iters[idx] = status != 0 ? status : it;
    if (o.berr) o.berr[idx] = status != 0 ? (double)NAN : berr;
}

// ---------------------------------------------------------------------
// registers: compile-time order N <= 16
// ---------------------------------------------------------------------

// z := (L L^T)^-1 z in FP32, L packed lower with reciprocal pivots rinv
template <int N>
__device__ __forceinline__ void solve32(const float (&L)[N * (N + 1) / 2], const float (&rinv)[N],
                                        float (&z)[N])
{
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float w = z[i];
#pragma unroll
        for (int l = 0; l < i; ++l)
            w = fmaf(-L[tix(i, l, N)], z[l], w);
        z[i] = w * rinv[i];
    }
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
        float w = z[i];
#pragma unroll
        for (int l = i + 1; l < N; ++l)
            w = fmaf(-L[tix(l, i, N)], z[l], w);
        z[i] = w * rinv[i];
    }
}

// The first step's residual r = b - A x0 in double-FP32 arithmetic on the
// FP32 pipe (dot2_sub): x0, the FP32 solve, is exact in FP32, and A's entries
// are split into two FP32 parts (47 bits). Its error stays below
// 2^-38 ||A|| ||x0|| at these orders, far under the first residual itself
// (~eps32 ||A|| ||x0||), so the correction it gives is as good as an FP64
// residual's; the stopping test is only ever taken on an FP64 residual.
// z: x0 in, the residual rounded to nearest FP32 out; returns
// its largest magnitude (NaN if any entry is NaN).
template <int N>
__device__ __forceinline__ float ff_residual(LV<double> A, LV<double> B, int col, float (&z)[N])
{
    float rr[N];
#pragma unroll
    for (int k = 0; k < N; ++k)
        rr[k] = 0.f;
    float rnorm = 0.f;
    // rows one after another (unrolled rows take more registers and, above
    // order 8, overflow the instruction cache); each row's result enters at
    // the end of rr
#pragma unroll 1
    for (int i = 0; i < N; ++i) {
        float s, c;
        split2_rz_any(B(i, col), s, c);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float ah, al;
            split2_rz(j <= i ? A(i, j) : A(j, i), ah, al);
            dot2_sub(s, c, ah, al, z[j]);
        }
        const float r = s + c;
        rnorm = fmax_nan(rnorm, fabsf(r));
#pragma unroll
        for (int k = 0; k + 1 < N; ++k)
            rr[k] = rr[k + 1];
        rr[N - 1] = r;
    }
#pragma unroll
    for (int k = 0; k < N; ++k)
        z[k] = rr[k];
    return rnorm;
}

// Up to order 8 the registers are capped at 128 (four blocks of 128 threads
// per SM): measured at n = 8, 16 warps per SM with a few spills beat 12
// without (0.179 against 0.196 ms for 262,144 matrices); at n = 16 every cap
// was slower.
template <int N>
__global__ void __launch_bounds__(128, N <= FF_NMAX ? 4 : 1)
    k_posv_refined_reg(bool row, bool up, int nrhs, double *ap, int ldap, double *bp, int ldbp,
                       int V, long ngroups, size_t sa, size_t sb, RefineOut out)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    const long idx = ln.g * V + ln.v;
    LV<double> A = lv_make<double>(ap + ln.g * sa + ln.v, row, ldap, V, N, N);
    if (up) A = A.t();
    const LV<double> B = lv_make<double>(bp + ln.g * sb + ln.v, row, ldbp, V, N, nrhs);

    // FP64 <-> FP32 conversions and range tests are integer operations here:
    // a hardware conversion or FP64 compare takes an FP64-pipe slot
    float L[N * (N + 1) / 2];
    float rs[N];
    int status = 0;
    unsigned hmax = 0; // largest high word of |a|: a quick screen for the FP32 range
#pragma unroll
    for (int i = 0; i < N; ++i)
        rs[i] = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
        for (int i = j; i < N; ++i) {
            const double a = A(i, j);
            hmax = max(hmax, (unsigned)__double2hiint(a) & 0x7fffffffu);
            const float f = d2f_rz_inrange(a);
            L[tix(i, j, N)] = f;
            rs[i] += fabsf(f);
            if (i != j) rs[j] += fabsf(f);
        }
    if (hmax >= 0x47efffffu && any_beyond_fp32(N, A)) status = -2;
    float anorm = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i)
        anorm = fmaxf(anorm, rs[i]);
    float rinv[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float a = L[tix(j, j, N)];
        if (!(a > 0.f) && status == 0) status = -1;
        const float d = sqrtf(a);
        const float r = 1.0f / d;
        rinv[j] = r;
        L[tix(j, j, N)] = d;
#pragma unroll
        for (int i = j + 1; i < N; ++i)
            L[tix(i, j, N)] *= r;
#pragma unroll
        for (int c = j + 1; c < N; ++c)
#pragma unroll
            for (int i = c; i < N; ++i)
                L[tix(i, c, N)] = fmaf(-L[tix(i, j, N)], L[tix(c, j, N)], L[tix(i, c, N)]);
    }
    // every quantity that only steers the iteration (norms, the stopping test,
    // the reported backward error) is kept in FP32: the FP64 pipe is left to
    // the residual itself and the FP64 update of x
    // LAPACK dsposv's test ||r|| <= sqrt(n) eps64 ||A|| ||x||, in FP32 while
    // the right side is a normal FP32 number, in FP64 below that
    const double cte = (double)anorm * EPS64 * sqrt((double)N);
    const float cte32 = (float)cte;
    int it_max = 0, col = 0;
    float worst = 0.f;
    for (; col < nrhs && status == 0; ++col) {
        double x[N];
        float z[N];
        float bnorm = 0.f;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            z[i] = d2f_rz(B(i, col));
            bnorm = fmaxf(bnorm, fabsf(z[i]));
        }
        solve32<N>(L, rinv, z);
#pragma unroll
        for (int i = 0; i < N; ++i)
            x[i] = f2d_int(z[i]);
        float rprev = INFINITY;
        for (int it = 0;; ++it) {
            float rnorm = 0.f, xnorm = 0.f;
            bool fp64 = true;
            if (N <= FF_NMAX && it == 0) {
                // x0 is z: the double-FP32 residual, unless x0 may already
                // meet the test (then the FP64 residual below decides)
#pragma unroll
                for (int i = 0; i < N; ++i)
                    xnorm = fmaxf(xnorm, fabsf(z[i]));
                rnorm = ff_residual<N>(A, B, col, z);
                // FP64 unless clearly unconverged and finite (an FP32
                // overflow in the products is no reason to fall back)
                fp64 = !(rnorm > cte32 * xnorm + 0x1p-38f * anorm * xnorm && rnorm <= FLT_MAX);
            }
            if (fp64) {
                // opaque strides: the n^2 addresses of A are recomputed each
                // step (cheap integer work) instead of being hoisted into
                // registers
                LV<double> Ar = A;
                asm volatile("" : "+l"(Ar.si), "+l"(Ar.sj));
                rnorm = 0.f;
                xnorm = 0.f;
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    double acc = B(i, col);
#pragma unroll
                    for (int j = 0; j < N; ++j)
                        acc = fma(-(j <= i ? Ar(i, j) : Ar(j, i)), x[j], acc);
                    z[i] = d2f_rz(acc);
                    rnorm = fmax_nan(rnorm, fabsf(z[i]));
                    xnorm = fmaxf(xnorm, fabsf(d2f_rz_inrange(x[i])));
                }
                const float thr = cte32 * xnorm;
                if (thr >= 0x1p-100f ? rnorm <= thr : (double)rnorm <= cte * (double)xnorm) {
                    const float den = anorm * xnorm + bnorm;
                    worst = fmaxf(worst, den > 0.f ? rnorm / den : 0.f);
                    it_max = max(it_max, it);
                    break;
                }
            }
            if (it >= out.max_iter || !(rnorm <= 0.5f * rprev)) {
                status = -3;
                break;
            }
            rprev = rnorm;
            solve32<N>(L, rinv, z);
#pragma unroll
            for (int i = 0; i < N; ++i)
                x[i] += f2d_int(z[i]);
        }
        if (status == 0) {
#pragma unroll
            for (int i = 0; i < N; ++i)
                B(i, col) = x[i];
        }
    }
    if (status != 0) fallback_lane(N, nrhs, status == -3 ? col - 1 : 0, A, B);
    write_status(out, idx, status, it_max, (double)worst);
}

// ---------------------------------------------------------------------
// workspace: any order
// ---------------------------------------------------------------------

struct RefineWork {
    float *L;   // n x n FP32 factor per lane, compact, ld = n
    double *x;  // n per lane
    float *z;   // n per lane
};

// Rows i0 .. i0+NR-1 of r = b - A x in FP64, four independent accumulators
// (A symmetric, lower triangle of the view: A(i,j) for j <= i, A(j,i) above),
// each x_j loaded once for the NR rows. The rounded residual goes to Z; its
// largest magnitude (FP32) is folded into rnorm.
template <int NR>
__device__ __forceinline__ void resid_rows(int n, int i0, int col, LV<double> A, LV<double> B,
                                           const double *X, float *Z, int V, float &rnorm)
{
    double acc[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r)
        acc[r] = B(i0 + r, col);
    for (int j = 0; j < i0; ++j) {
        const double xj = X[(long)j * V];
#pragma unroll
        for (int r = 0; r < NR; ++r)
            acc[r] = fma(-A(i0 + r, j), xj, acc[r]);
    }
#pragma unroll
    for (int c = 0; c < NR; ++c) {
        const double xj = X[(long)(i0 + c) * V];
#pragma unroll
        for (int r = 0; r < NR; ++r)
            acc[r] = fma(-(c <= r ? A(i0 + r, i0 + c) : A(i0 + c, i0 + r)), xj, acc[r]);
    }
    for (int j = i0 + NR; j < n; ++j) {
        const double xj = X[(long)j * V];
#pragma unroll
        for (int r = 0; r < NR; ++r)
            acc[r] = fma(-A(j, i0 + r), xj, acc[r]);
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const float z = d2f_rz(acc[r]);
        Z[(long)(i0 + r) * V] = z;
        rnorm = fmax_nan(rnorm, fabsf(z));
    }
}

__global__ void __launch_bounds__(128, 4)
    k_posv_refined_ws(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                      int ldbp, int V, long ngroups, size_t sa, size_t sb, RefineWork w,
                      RefineOut out)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    const long idx = ln.g * V + ln.v;
    LV<double> A = lv_make<double>(ap + ln.g * sa + ln.v, row, ldap, V, n, n);
    if (up) A = A.t();
    const LV<double> B = lv_make<double>(bp + ln.g * sb + ln.v, row, ldbp, V, n, nrhs);
    const LV<float> W =
        lv_make<float>(w.L + ln.g * ((size_t)n * n * V) + ln.v, false, n, V, n, n);
    double *X = w.x + ln.g * ((size_t)n * V) + ln.v;
    float *Z = w.z + ln.g * ((size_t)n * V) + ln.v;
    const LV<float> Zv = lv_make<float>(Z, false, n, V, n, 1);

    int status = 0;
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i) {
            const double a = A(i, j);
            if (beyond_fp32(a)) status = -2;
            W(i, j) = d2f_rz_inrange(a);
        }
    float anorm = 0.f;
    for (int i = 0; i < n; ++i) {
        float s = 0.f;
        for (int j = 0; j <= i; ++j)
            s += fabsf(W(i, j));
        for (int j = i + 1; j < n; ++j)
            s += fabsf(W(j, i));
        anorm = fmaxf(anorm, s);
    }
    float rinv[RINV]; // 1/L(i,i) of the FP32 factor, for every solve below
    if (status == 0) {
        factor_lane<float, false>(n, W);
        for (int i = 0; i < n; ++i)
            if (!(W(i, i) > 0.f)) status = -1;
        for (int i = 0; i < RINV && i < n; ++i)
            rinv[i] = rcp(W(i, i));
    }
    // the norms, the stopping test and the reported backward error are FP32
    // (they only steer the iteration); the FP64 pipe does the residual and x
    const double cte = (double)anorm * EPS64 * sqrt((double)n);
    int it_max = 0, col = 0;
    float worst = 0.f;
    for (; col < nrhs && status == 0; ++col) {
        float bnorm = 0.f;
        for (int i = 0; i < n; ++i) {
            const float b = d2f_rz(B(i, col));
            bnorm = fmaxf(bnorm, fabsf(b));
            Z[(long)i * V] = b;
        }
        sym_solve_block<float, false, 1>(n, W, Zv, 0, rinv);
        float xnorm = 0.f;
        for (int i = 0; i < n; ++i) {
            const float z = Z[(long)i * V];
            X[(long)i * V] = f2d_int(z);
            xnorm = fmaxf(xnorm, fabsf(z));
        }
        float rprev = INFINITY;
        for (int it = 0;; ++it) {
            float rnorm = 0.f;
            int i0 = 0;
            for (; i0 + 4 <= n; i0 += 4)
                resid_rows<4>(n, i0, col, A, B, X, Z, V, rnorm);
            switch (n - i0) {
            case 3: resid_rows<3>(n, i0, col, A, B, X, Z, V, rnorm); break;
            case 2: resid_rows<2>(n, i0, col, A, B, X, Z, V, rnorm); break;
            case 1: resid_rows<1>(n, i0, col, A, B, X, Z, V, rnorm); break;
            default: break;
            }
            const float thr = (float)cte * xnorm;
            if (thr >= 0x1p-100f ? rnorm <= thr : (double)rnorm <= cte * (double)xnorm) {
                const float den = anorm * xnorm + bnorm;
                worst = fmaxf(worst, den > 0.f ? rnorm / den : 0.f);
                it_max = max(it_max, it);
                break;
            }
            if (it >= out.max_iter || !(rnorm <= 0.5f * rprev)) {
                status = -3;
                break;
            }
            rprev = rnorm;
            sym_solve_block<float, false, 1>(n, W, Zv, 0, rinv);
            xnorm = 0.f;
            for (int i = 0; i < n; ++i) {
                const double xi = X[(long)i * V] + f2d_int(Z[(long)i * V]);
                X[(long)i * V] = xi;
                xnorm = fmaxf(xnorm, fabsf(d2f_rz(xi)));
            }
        }
        if (status == 0)
            for (int i = 0; i < n; ++i)
                B(i, col) = X[(long)i * V];
    }
    if (status != 0) fallback_lane(n, nrhs, status == -3 ? col - 1 : 0, A, B);
    write_status(out, idx, status, it_max, (double)worst);
}

inline size_t align256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

} // namespace

// bytes of workspace the refined solve needs (0 when it runs from registers)
size_t posv_refined_lwork(int n, int nrhs, int V, int nm)
{
    (void)nrhs;
    if (n <= REG_NMAX || posv_refined_warp_ok(n) || nm <= 0) return 0;
    const size_t lanes = (size_t)((nm + V - 1) / V) * V;
    return align256(lanes * (size_t)n * n * sizeof(float)) +
           align256(lanes * (size_t)n * sizeof(double)) + align256(lanes * (size_t)n * sizeof(float));
}

cudaError_t launch_posv_refined(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                double *bp, int ldbp, int V, int nm, int max_iter, int *iters,
                                double *berr, void *work, cudaStream_t s, size_t sa_, size_t sb_)
{
    const long ng = ((long)nm + V - 1) / V;
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, n, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, n, nrhs, V);
    const RefineOut out{iters, berr, nm, max_iter};
    // the lane-per-matrix variants are compiled for at most 128 threads
    // built-in: 64 threads per block up to order 8 (measured fastest there
    // with the register cap), 128 above
    const int th =
        std::min(threads_or(R_POSV_REFINED, n, sizeof(double), n <= FF_NMAX ? 64 : 128), 128);
    const unsigned bl = (unsigned)((ng * V + th - 1) / th);
    if (n <= REG_NMAX) {
        switch (n) {
#define CBK_REG_CASE(N)                                                                            \
    case N:                                                                                        \
        k_posv_refined_reg<N><<<bl, th, 0, s>>>(row, up, nrhs, ap, ldap, bp, ldbp, V, ng, sa, sb,  \
                                                out);                                              \
        break;
            CBK_REG_CASE(1) CBK_REG_CASE(2) CBK_REG_CASE(3) CBK_REG_CASE(4) CBK_REG_CASE(5)
            CBK_REG_CASE(6) CBK_REG_CASE(7) CBK_REG_CASE(8) CBK_REG_CASE(9) CBK_REG_CASE(10)
            CBK_REG_CASE(11) CBK_REG_CASE(12) CBK_REG_CASE(13) CBK_REG_CASE(14) CBK_REG_CASE(15)
            CBK_REG_CASE(16)
#undef CBK_REG_CASE
        default: break;
        }
        return cudaGetLastError();
    }
    if (posv_refined_warp_ok(n))
        return launch_posv_refined_warp(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter,
                                        iters, berr, s, sa, sb);
    const size_t lanes = (size_t)ng * V;
    char *base = static_cast<char *>(work);
    RefineWork w;
    w.L = reinterpret_cast<float *>(base);
    base += align256(lanes * (size_t)n * n * sizeof(float));
    w.x = reinterpret_cast<double *>(base);
    base += align256(lanes * (size_t)n * sizeof(double));
    w.z = reinterpret_cast<float *>(base);
    k_posv_refined_ws<<<bl, th, 0, s>>>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, ng, sa, sb, w,
                                        out);
    return cudaGetLastError();
}

namespace {

__global__ void k_count_negative(const int *iters, int n, int *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool neg = i < n && iters[i] < 0;
    const unsigned b = __ballot_sync(0xffffffffu, neg);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, __popc(b));
}

} // namespace

cudaError_t launch_count_negative(const int *iters, int n, int *count, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_count_negative<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(iters, n, count);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------
// Scratch for callers that cannot allocate device memory
// ---------------------------------------------------------------------
// cbk_cuda_dposv_refined_compact_noalloc_async takes no workspace: for
// n > 64 the FP32 factor, x and the correction live in this one array,
// reserved on every GPU that loads the library for as long as the process
// runs. Host code cannot use the array's name as a device address: the
// address belongs to the CUDA context the module is loaded in, so it is
// looked up (cudaGetSymbolAddress, which allocates nothing) with that context
// current and cached under the context's unique ID -- a context made later
// on the same device (a driver-API host's own, or the primary context again
// after cudaDeviceReset) has a new ID and gets its own lookup. A lookup is
// refused on a capturing stream (it may load the module, which a capture
// does not allow): the first call in each context must come before any
// capture. Every call shares the array and nothing in it needs to start at
// zero: the kernel writes each element it reads (the FP32 copy of A before
// the factorization, x and the correction before each use).

namespace {

static_assert(CBK_CUDA_NOALLOC_SCRATCH_BYTES % 256 == 0, "scratch size");
__device__ __align__(256) unsigned char g_noalloc_scratch[CBK_CUDA_NOALLOC_SCRATCH_BYTES];

// the driver's cuCtxGetCurrent and cuCtxGetId, resolved through the runtime
// (no link-time dependence on libcuda)
typedef int (*CtxGetCurrentFn)(void **ctx);
typedef int (*CtxGetIdFn)(void *ctx, unsigned long long *id);

struct CtxFns {
    CtxGetCurrentFn current = nullptr;
    CtxGetIdFn id = nullptr;
};

const CtxFns &ctx_fns()
{
    static const CtxFns f = [] {
        CtxFns r;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            r.current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            r.id = reinterpret_cast<CtxGetIdFn>(p);
        return r;
    }();
    return f;
}

// the unique ID of the current context; false when none is current
bool current_ctx_id(unsigned long long &id)
{
    const CtxFns &f = ctx_fns();
    void *ctx = nullptr;
    return f.current && f.id && f.current(&ctx) == 0 && ctx != nullptr && f.id(ctx, &id) == 0;
}

constexpr int CACHE = 64;
struct Slot {
    unsigned long long ctx;
    void *addr;
};
std::mutex g_cache_mu;
Slot g_cache[CACHE];
int g_cache_n = 0, g_cache_next = 0;

// The scratch array's address in the current context. On a capturing stream
// only a cached address is used: *capturing is set, and nothing looked up,
// when there is none.
cudaError_t noalloc_scratch(cudaStream_t s, void **out, bool *capturing)
{
    *capturing = false;
    unsigned long long id = 0;
    bool have = current_ctx_id(id);
    if (have) {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        for (int k = 0; k < g_cache_n; ++k)
            if (g_cache[k].ctx == id) {
                *out = g_cache[k].addr;
                return cudaSuccess;
            }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusNone) {
        *capturing = true;
        return cudaSuccess;
    }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (!have) have = current_ctx_id(id); // the lookup made the primary context current
    if (have) {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        g_cache[g_cache_next] = Slot{id, p};
        g_cache_next = (g_cache_next + 1) % CACHE;
        g_cache_n = g_cache_n < CACHE ? g_cache_n + 1 : CACHE;
    }
    *out = p;
    return cudaSuccess;
}

} // namespace

int launch_posv_refined_noalloc(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                double *bp, int ldbp, int V, int nm, int max_iter, int *iters,
                                double *berr, cudaStream_t s)
{
    void *work = nullptr;
    if (posv_refined_lwork(n, nrhs, V, nm) > 0) {
        bool capturing = false;
        const cudaError_t e = noalloc_scratch(s, &work, &capturing);
        if (e != cudaSuccess) return CBK_CUDA_ERROR_BASE + (int)e;
        if (capturing) return CBK_CUDA_NOALLOC_IN_CAPTURE;
    }
    const cudaError_t e = launch_posv_refined(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm,
                                              max_iter, iters, berr, work, s);
    return e == cudaSuccess ? 0 : CBK_CUDA_ERROR_BASE + (int)e;
}

} // namespace cbkcuda
