// cbk_kernels_refine_warp.cu -- the mixed-precision SPD solve for orders
// 17 .. 64, one warp per matrix.
//
// The method is cbk_kernels_refine.cu's (FP32 factorization, FP64 refinement,
// LAPACK dsposv's stopping test, per-matrix FP64 fallback); the mapping and
// the form of the FP32 solve differ. One thread per matrix cannot hold an FP32
// factor of order 48 on chip; here the 32 lanes of a warp share one matrix:
//   * the block's matrices (consecutive lanes of the compact batch) are staged
//     once into shared memory as full symmetric FP64 matrices, by all threads
//     of the block with coalesced loads (odd leading dimension: row and
//     column sweeps free of bank conflicts);
//   * lane l holds rows l and l + 32 of the FP32 matrix in registers (the
//     order's upper bound NMAX is a template parameter, so every register
//     index is static) and the warp inverts it in place with the symmetric
//     sweep operator -- Gauss-Jordan elimination without pivoting, stable for
//     positive-definite matrices (Beaton 1964; Goodnight 1979): pivot k
//     broadcasts column k through shared memory and every lane updates its
//     rows, the matrix staying symmetric throughout;
//   * each FP32 solve is then one matrix-vector product with the inverse --
//     a lane per row, no serial chain -- where triangular sweeps would be n
//     dependent shuffle steps each; refinement converges at the same rate
//     (||I - M A|| ~ kappa eps32);
//   * the FP64 residual r = b - A x is row-parallel: lane l sweeps its rows of
//     the staged A with x broadcast from shared memory -- n FMAs per row, the
//     FP64 pipe's only large load.
// FP64 -> FP32 rounding of A (once per matrix) is done with integer bit
// operations (round toward zero, subnormals flushed): a hardware conversion
// takes an FP64-pipe slot on a GB300, and the FP32 inverse only steers the
// refinement. A non-positive FP32 pivot (not positive definite in FP32) sends
// the matrix to the FP64 fallback (iters = -1).
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <float.h>
#include <math.h>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr double EPS64 = 2.220446049250313e-16;
constexpr unsigned FULL = 0xffffffffu;

// FP64 -> FP32 toward zero on the integer pipe; sets *overflow for a finite
// value beyond the FP32 range (it becomes an infinity).
__device__ __forceinline__ float d2f_rz(double a, bool &overflow)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const int fe = e - 1023 + 127;
    unsigned bits;
    if (e == 0x7ff)
        bits = sign | 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u | mant : 0u);
    else if (fe >= 255) {
        bits = sign | 0x7f800000u;
        overflow = true;
    }
    else if (fe <= 0)
        bits = sign;
    else
        bits = sign | ((unsigned)fe << 23) | mant;
    return __uint_as_float(bits);
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

struct WarpOut {
    int *iters;
    double *berr;
    int nm;
    int max_iter;
};

// The FP64 fallback of one matrix, run by lane 0 (the rare path): the plain
// path's factor and solve on the global A and the unsolved columns of B.
// Inlined: a call here makes the compiler keep the register rows of the FP32
// factor in local memory for the whole kernel.
__device__ __forceinline__ void warp_fallback(int n, int nrhs, int first, LV<double> A, LV<double> B)
{
    factor_lane<double, false>(n, A);
    if (first < nrhs) {
        LV<double> Bs = B;
        Bs.p += (long)first * B.sj;
        sym_solve_lane<double, false>(n, nrhs - first, A, Bs);
    }
}

// d (this lane's rows) := -M z, M = -A32^-1 held as register rows: z is
// broadcast from shared memory (SR, this warp's n floats).
template <int NMAX>
__device__ __forceinline__ void apply_inverse(int n, int lane, const float (&Mr)[(NMAX + 31) / 32][NMAX],
                                              float *SR, float (&z)[(NMAX + 31) / 32])
{
    constexpr int NR = (NMAX + 31) / 32;
    __syncwarp();
#pragma unroll
    for (int r = 0; r < NR; ++r)
        if (lane + 32 * r < n) SR[lane + 32 * r] = z[r];
    __syncwarp();
    float acc[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r)
        acc[r] = 0.f;
#pragma unroll
    for (int j = 0; j < NMAX; ++j) {
        if (j >= n) break;
        const float zj = SR[j];
#pragma unroll
        for (int r = 0; r < NR; ++r)
            acc[r] = fmaf(Mr[r][j], zj, acc[r]);
    }
#pragma unroll
    for (int r = 0; r < NR; ++r)
        z[r] = -acc[r];
}

template <int NMAX, int WPB>
__global__ void __launch_bounds__(WPB * 32)
    k_posv_refined_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                        int ldbp, int V, long nlanes, size_t sa, size_t sb, WarpOut out)
{
    constexpr int NR = (NMAX + 31) / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long m0 = (long)blockIdx.x * WPB;
    const long m = m0 + warp;
    const int lds = n | 1; // odd: row and column sweeps free of bank conflicts
    const int nx = (n + 1) & ~1, nc = (n + 3) & ~3; // vector lengths padded for 16-byte loads
    double *SAall = reinterpret_cast<double *>(smem);
    double *SA = SAall + (size_t)warp * n * lds;
    double *SX = SAall + (((size_t)WPB * n * lds + 1) & ~(size_t)1) + (size_t)warp * nx;
    float *SC = reinterpret_cast<float *>(SAall + (((size_t)WPB * n * lds + 1) & ~(size_t)1) +
                                          (size_t)WPB * nx) +
                (size_t)warp * 2 * nc;
    float *SR = SC + nc;

    // ---- stage A (the lower triangle of each matrix's view, mirrored) ----
    {
        long gw[WPB];
        int vw[WPB];
#pragma unroll
        for (int w = 0; w < WPB; ++w) {
            gw[w] = (m0 + w) / V;
            vw[w] = (int)(m0 + w - gw[w] * V);
        }
        for (int j = 0; j < n; ++j) {
            const int cnt = (n - j) * WPB;
            for (int p = threadIdx.x; p < cnt; p += WPB * 32) {
                const int w = p % WPB, i = j + p / WPB;
                if (m0 + w >= nlanes) continue;
                long g = 0;
                int v = 0;
#pragma unroll
                for (int q = 0; q < WPB; ++q)
                    if (q == w) {
                        g = gw[q];
                        v = vw[q];
                    }
                LV<double> A = lv_make<double>(ap + g * sa + v, row, ldap, V);
                if (up) A = A.t();
                const double a = A(i, j);
                double *S = SAall + (size_t)w * n * lds;
                S[(size_t)j * lds + i] = a;
                S[(size_t)i * lds + j] = a;
            }
        }
    }
    __syncthreads();
    if (m >= nlanes) return;
    const long g = m / V;
    const int v = (int)(m - g * V);
    LV<double> Ag = lv_make<double>(ap + g * sa + v, row, ldap, V);
    if (up) Ag = Ag.t();
    const LV<double> B = lv_make<double>(bp + g * sb + v, row, ldbp, V);

    // ---- FP32 rows (both triangles) in registers, ||A||_inf ----
    float Mr[NR][NMAX];
    bool ovf = false;
    float rs = 0.f;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const int i = lane + 32 * r;
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < NMAX; ++j) {
            float f = 0.f;
            if (i < n && j < n) {
                f = d2f_rz(SA[(size_t)j * lds + i], ovf);
                s += fabsf(f);
            }
            Mr[r][j] = f;
        }
        rs = fmaxf(rs, s);
    }
    const float anorm = warp_max(rs);
    int status = __any_sync(FULL, ovf) ? -2 : 0;

    // ---- FP32 inverse by the symmetric sweep: after all n pivots Mr = -A^-1 ----
    // pivot k, with c = column k (= row k) and p = c_k:
    //   rows i != k:  M(i,j) -= (c_i / p) c_j  (j != k),  M(i,k) = c_i / p
    //   row k:        M(k,j)  = c_j / p        (j != k),  M(k,k) = -1 / p
    // the row-k case is the same FMA with the coefficient 1/p - 1 (its row
    // equals c before the pivot), so every lane runs one instruction stream
#pragma unroll
    for (int k = 0; k < NMAX; ++k) {
        if (k >= n) break;
        __syncwarp();
#pragma unroll
        for (int r = 0; r < NR; ++r)
            if (lane + 32 * r < n) SC[lane + 32 * r] = Mr[r][k];
        __syncwarp();
        const float p = SC[k];
        if (!(p > 0.f) && status == 0) status = -1;
        const float rp = 1.0f / p;
        float beta[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const bool own = (lane + 32 * r == k);
            const float wi = Mr[r][k] * rp;
            beta[r] = own ? rp - 1.0f : -wi;
            Mr[r][k] = own ? -rp : wi;
        }
#pragma unroll
        for (int j = 0; j < NMAX; ++j) {
            if (j >= n) break;
            if (j == k) continue;
            const float cj = SC[j];
#pragma unroll
            for (int r = 0; r < NR; ++r)
                Mr[r][j] = fmaf(beta[r], cj, Mr[r][j]);
        }
    }

    const double cte = (double)anorm * EPS64 * sqrt((double)n);
    int it_max = 0, col = 0;
    float worst = 0.f;
    for (; col < nrhs && status == 0; ++col) {
        float w[NR];
        double b64[NR], x[NR];
        float bn = 0.f;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const int i = lane + 32 * r;
            b64[r] = (i < n) ? B(i, col) : 0.0;
            w[r] = (float)b64[r];
            bn = fmaxf(bn, fabsf(w[r]));
        }
        bn = warp_max(bn);
        apply_inverse<NMAX>(n, lane, Mr, SR, w);
        float xn = 0.f;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            x[r] = (lane + 32 * r < n) ? (double)w[r] : 0.0;
            xn = fmaxf(xn, fabsf(w[r]));
        }
        xn = warp_max(xn);
        float rprev = INFINITY;
        for (int it = 0;; ++it) {
            __syncwarp();
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (lane + 32 * r < n) SX[lane + 32 * r] = x[r];
            __syncwarp();
            // r = b - A x, lane-parallel over rows, x broadcast from shared
            double acc[NR];
#pragma unroll
            for (int r = 0; r < NR; ++r)
                acc[r] = b64[r];
            for (int j = 0; j < n; ++j) {
                const double xj = SX[j];
                const double *Sj = SA + (size_t)j * lds + lane;
#pragma unroll
                for (int r = 0; r < NR; ++r)
                    if (lane + 32 * r < n) acc[r] = fma(-Sj[32 * r], xj, acc[r]);
            }
            float rn = 0.f;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                w[r] = (lane + 32 * r < n) ? (float)acc[r] : 0.f;
                rn = fmaxf(rn, fabsf(w[r]));
            }
            rn = warp_max(rn);
            if ((double)rn <= cte * (double)xn) {
                const float den = anorm * xn + bn;
                worst = fmaxf(worst, den > 0.f ? rn / den : 0.f);
                it_max = max(it_max, it);
                break;
            }
            if (it >= out.max_iter || !(rn <= 0.5f * rprev)) {
                status = -3;
                break;
            }
            rprev = rn;
            apply_inverse<NMAX>(n, lane, Mr, SR, w);
            float xm = 0.f;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                if (lane + 32 * r < n) x[r] += (double)w[r];
                xm = fmaxf(xm, fabsf((float)x[r]));
            }
            xn = warp_max(xm);
        }
        if (status == 0) {
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (lane + 32 * r < n) B(lane + 32 * r, col) = x[r];
        }
    }
    if (status != 0 && lane == 0) warp_fallback(n, nrhs, status == -3 ? col - 1 : 0, Ag, B);
    if (lane == 0 && m < out.nm) {
        if (out.iters) out.iters[m] = status != 0 ? status : it_max;
        if (out.berr) out.berr[m] = status != 0 ? (double)NAN : (double)worst;
    }
}

template <int NMAX, int WPB>
cudaError_t launch_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                        int ldbp, int V, int nm, const WarpOut &out, cudaStream_t s)
{
    const long ng = ((long)nm + V - 1) / V;
    const long nlanes = ng * V;
    const size_t nx = (n + 1) & ~1, nc = (n + 3) & ~3;
    const size_t smem = (((size_t)WPB * n * (n | 1) + 1) & ~(size_t)1) * sizeof(double) +
                        (size_t)WPB * nx * sizeof(double) + (size_t)WPB * 2 * nc * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_posv_refined_warp<NMAX, WPB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((nlanes + WPB - 1) / WPB);
    k_posv_refined_warp<NMAX, WPB><<<blocks, WPB * 32, smem, s>>>(
        row, up, n, nrhs, ap, ldap, bp, ldbp, V, nlanes, gstride(row, ldap, n, n, V),
        gstride(row, ldbp, n, nrhs, V), out);
    return cudaGetLastError();
}

} // namespace

// orders the warp-per-matrix variant takes
bool posv_refined_warp_ok(int n)
{
    return n > 16 && n <= 64;
}

cudaError_t launch_posv_refined_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                     double *bp, int ldbp, int V, int nm, int max_iter,
                                     int *iters, double *berr, cudaStream_t s)
{
    const WarpOut out{iters, berr, nm, max_iter};
    // four matrices per block: the staging loads then use whole 32-byte
    // sectors of the compact layout (four FP64 lanes)
    if (n <= 32) return launch_warp<32, 4>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s);
    if (n <= 48) return launch_warp<48, 4>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s);
    return launch_warp<64, 4>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s);
}

} // namespace cbkcuda
