// cbk_kernels_chol_reg.cu -- Cholesky factor (+ solve) of small orders with
// each lane's matrix held in registers.
//
// One thread per lane of the compact batch, as the generic kernels, but the
// lower triangle of an order N <= 8 is loaded once into registers, factored
// and solved there, and stored once: the generic kernel keeps the factor in
// global memory and waits on a load at every step of its dependency chain.
// The arithmetic is the generic kernels', operation for operation, in the
// same order (cbk_device.cuh: panel_sweep_nc for a single 8-column
// panel, then sym_solve_lane), so potrf and posv here give exactly the bits
// of the generic potrf and potrs -- fused == separate holds whichever kernel
// runs. (The reference: src/cbk_potrf_compact.hpp:79-105 for the panel,
// src/cbk_potrs_compact.hpp:46-58 for the solve.)
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <algorithm>

namespace cbkcuda {
using namespace cbkdev;

namespace {

template <typename T, int N, bool SOLVE>
__global__ void __launch_bounds__(128)
    k_chol_small(bool row, bool up, int nrhs, T *ap, int ldap, T *bp, int ldbp, int V,
                 long ngroups, size_t sa, size_t sb)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    LV<T> A = lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, N, N);
    if (up) A = A.t();
    T a[N][N]; // the lower triangle, a[i][j] for j <= i
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
        for (int i = j; i < N; ++i)
            a[i][j] = A(i, j);
    // pivot j: the weight 1/a, the rank-1 step on the unscaled column, then the
    // diagonal and the column scale (panel_sweep_nc's diagonal block)
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const T ajj = a[j][j];
        const bool pos = ajj > T(0) && ajj <= FLT_OR_DBL_MAX<T>();
        T inva;
        if (pos) {
            const T r = rsqrt(ajj);
            inva = r * r;
        }
        else {
            inva = rcp(ajj);
        }
        T w[N];
#pragma unroll
        for (int q = 0; q + j + 1 < N; ++q)
            w[q] = a[j + 1 + q][j] * inva;
#pragma unroll
        for (int r = 0; r + j + 1 < N; ++r) {
            const int i = j + 1 + r;
            const T aij = a[i][j];
#pragma unroll
            for (int q = 0; q <= r; ++q)
                a[i][j + 1 + q] = fma(-aij, w[q], a[i][j + 1 + q]);
        }
        T scale;
        if (pos) {
            const T r = rsqrt(ajj);
            a[j][j] = ajj * r;
            scale = r;
        }
        else {
            const T d = sqrt(ajj);
            a[j][j] = d;
            scale = d * inva;
        }
#pragma unroll
        for (int i = j + 1; i < N; ++i)
            a[i][j] = a[i][j] * scale;
    }
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
        for (int i = j; i < N; ++i)
            A(i, j) = a[i][j];
    if (!SOLVE) return;
    // L z = b, L^T x = z per right-hand side, one reciprocal per row
    // (sym_solve_lane / sym_solve_block)
    T rinv[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
        rinv[i] = rcp(a[i][i]);
    const LV<T> B = lv_make<T>(bp + ln.g * sb + ln.v, row, ldbp, V, N, nrhs);
    for (int c = 0; c < nrhs; ++c) {
        T x[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            T w = B(i, c);
#pragma unroll
            for (int l = 0; l < i; ++l)
                w = fma(-a[i][l], x[l], w);
            x[i] = w * rinv[i];
        }
#pragma unroll
        for (int i = N - 1; i >= 0; --i) {
            T w = x[i];
#pragma unroll
            for (int l = i + 1; l < N; ++l)
                w = fma(-a[l][i], x[l], w);
            x[i] = w * rinv[i];
        }
#pragma unroll
        for (int i = 0; i < N; ++i)
            B(i, c) = x[i];
    }
}

inline unsigned blocks_for(long ngroups, int V, int threads)
{
    return (unsigned)((ngroups * (long)V + threads - 1) / threads);
}

} // namespace

bool chol_small_ok(int n)
{
    return n >= 1 && n <= CHOL_SMALL_NMAX;
}

template <typename T>
cudaError_t launch_chol_small(bool solve, bool row, bool up, int n, int nrhs, T *ap, int ldap,
                              T *bp, int ldbp, int V, int nm, cudaStream_t s, size_t sa_,
                              size_t sb_)
{
    const long ng = ((long)nm + V - 1) / V;
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, n, n, V);
    const size_t sb = solve ? (sb_ ? sb_ : gstride(row, ldbp, n, nrhs, V)) : 0;
    const int th = std::min(threads_for(solve ? R_POSV : R_POTRF, n, sizeof(T)), 128);
    const unsigned bl = blocks_for(ng, V, th);
#define CBK_CHOL_CASE(N)                                                                           \
    case N:                                                                                        \
        if (solve)                                                                                 \
            k_chol_small<T, N, true><<<bl, th, 0, s>>>(row, up, nrhs, ap, ldap, bp, ldbp, V, ng,   \
                                                       sa, sb);                                    \
        else                                                                                       \
            k_chol_small<T, N, false><<<bl, th, 0, s>>>(row, up, 0, ap, ldap, bp, ldbp, V, ng, sa, \
                                                        sb);                                       \
        break;
    switch (n) {
        CBK_CHOL_CASE(1) CBK_CHOL_CASE(2) CBK_CHOL_CASE(3) CBK_CHOL_CASE(4)
        CBK_CHOL_CASE(5) CBK_CHOL_CASE(6) CBK_CHOL_CASE(7) CBK_CHOL_CASE(8)
    default: return cudaErrorInvalidValue;
    }
#undef CBK_CHOL_CASE
    return cudaGetLastError();
}

template cudaError_t launch_chol_small<float>(bool, bool, bool, int, int, float *, int, float *,
                                              int, int, int, cudaStream_t, size_t, size_t);
template cudaError_t launch_chol_small<double>(bool, bool, bool, int, int, double *, int, double *,
                                               int, int, int, cudaStream_t, size_t, size_t);

} // namespace cbkcuda
