// cbk_refine_warp.cuh -- the mixed-precision SPD solve for orders
// 17 .. 64, one warp per matrix.
//
// The method is cbk_kernels_refine.cu's (FP32 factorization, FP64 refinement,
// LAPACK dsposv's stopping test, per-matrix FP64 fallback); the mapping and
// the form of the FP32 solve differ. One thread per matrix cannot hold an FP32
// factor of order 48 on chip; here the 32 lanes of a warp share one matrix.
// The kernel is compiled for a padded order N (24, 32, .., 64) and a matrix
// of order n <= N is extended by the identity, so every loop bound and
// register index is static:
//   * the block's matrices (consecutive lanes of the compact batch) are staged
//     once into shared memory, each as the packed lower triangle of its FP64
//     matrix (column-major, N (N + 1) / 2 values -- half of a full square, so
//     twice as many matrices fit on an SM), by all threads of the block with
//     coalesced loads;
//   * lane l holds rows l and l + 32 of the FP32 matrix in registers and the
//     warp inverts it in place with the symmetric sweep operator --
//     Gauss-Jordan elimination without pivoting, stable for positive-definite
//     matrices (Beaton 1964; Goodnight 1979): pivot k broadcasts column k
//     through shared memory and every lane updates its rows. The pivot loop
//     is not unrolled (its body is one pass over the row); instead every
//     step rotates the register row by one place as it updates it, so the
//     pivot column is always register 0;
//   * the FP32 matrix is the symmetrically scaled D A D, D = diag(2^-h_i) with
//     h_i = floor(log2(a_ii) / 2): an exact scaling that puts the diagonal in
//     [1, 4), so every pivot lies in (0, 4) whatever the scale of A, and the
//     pivot row's update can share the other rows' FMA (coefficient 1/p - 1,
//     exact or accurate to eps32 for such pivots);
//   * each FP32 solve is then one matrix-vector product with the inverse --
//     a lane per row, no serial chain -- where triangular sweeps would be n
//     dependent shuffle steps each; refinement converges at the same rate
//     (||I - M A|| ~ kappa eps32);
//   * the FP64 residual r = b - A x is row-parallel over the packed FP64
//     triangle with x broadcast from shared memory: N FMAs per row, the FP64
//     pipe's only large load. For N <= 48 the rows past 32 are split by
//     columns over the two half-warps (summed with one shuffle), so no lane
//     idles in the FP64 pipe.
// FP64 -> FP32 rounding of A (once per matrix) is done with integer bit
// operations (round toward zero, subnormals flushed): a hardware conversion
// takes an FP64-pipe slot on a GB300, and the FP32 inverse only steers the
// refinement. An entry beyond the FP32 range sends the matrix to the FP64
// fallback with iters = -2 (as LAPACK dsposv); a non-positive FP32 pivot
// (not positive definite in FP32) with iters = -1.
#pragma once

#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <float.h>
#include <math.h>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr double EPS64 = 2.220446049250313e-16;
constexpr unsigned FULL = 0xffffffffu;

// 1/p from the SFU's approximate reciprocal (relative error below 2^-22):
// the FP32 inverse only steers the refinement
__device__ __forceinline__ float rcp_approx(float p)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(p));
    return r;
}

// floor(e / 2) for a = m 2^e > 0 (m in [1, 2)), clamped to [-63, 63); 0 for a
// diagonal that is not a positive normal number (the pivot test catches it)
__device__ __forceinline__ int half_exp(double a)
{
    const int hi = __double2hiint(a);
    const int eb = (hi >> 20) & 0x7ff;
    if (hi < 0 || eb == 0 || eb == 0x7ff) return 0;
    return min(max((eb - 1023) >> 1, -63), 63);
}

// 2^k as a float, |k| <= 126
__device__ __forceinline__ float exp2i(int k)
{
    return __int_as_float((127 + k) << 23);
}

// Two FP32 values in one 64-bit register pair, for sm_100's packed FP32 FMA
// (fma.rn.f32x2: two IEEE fmaf in one instruction, bit-identical to them).
// The FP32 rows live in such pairs, so the sweep and the matrix-vector
// products issue half the FMA instructions.
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2(float lo, float hi)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ float f2lo(f2_t p)
{
    float a;
    asm("{\n\t.reg .f32 t;\n\tmov.b64 {%0, t}, %1;\n\t}" : "=f"(a) : "l"(p));
    return a;
}

__device__ __forceinline__ float f2hi(f2_t p)
{
    float b;
    asm("{\n\t.reg .f32 t;\n\tmov.b64 {t, %0}, %1;\n\t}" : "=f"(b) : "l"(p));
    return b;
}

// d = a * b + c, element-wise
__device__ __forceinline__ f2_t ffma2(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// element q (static) of a row held in pairs
template <int P> __device__ __forceinline__ float el(const f2_t (&R)[P], int q)
{
    return (q & 1) ? f2hi(R[q >> 1]) : f2lo(R[q >> 1]);
}

template <int P> __device__ __forceinline__ void set_el(f2_t (&R)[P], int q, float v)
{
    R[q >> 1] = (q & 1) ? f2(f2lo(R[q >> 1]), v) : f2(v, f2hi(R[q >> 1]));
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// the packed lower triangle of an order-N matrix, column-major: column j
// starts at pk_col(N, j) and element (i, j), i >= j, is at pk_col(N, j) + i - j
__host__ __device__ constexpr int pk_col(int N, int j)
{
    return j * (2 * N - j + 1) / 2;
}

// doubles per staged matrix: the triangle, padded to 8 (mod 16) doubles so
// that the block's matrices start in alternate halves of the 32 banks
__host__ __device__ constexpr int pk_stride(int N)
{
    return N * (N + 1) / 2 + ((8 - (N * (N + 1) / 2) % 16) + 16) % 16;
}

template <int N, int WPB> constexpr size_t warp_smem_bytes()
{
    return (size_t)WPB * ((size_t)pk_stride(N) * sizeof(double) + (size_t)2 * N * sizeof(double) +
                          (size_t)5 * N * sizeof(float));
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
    factor_lane<double, false, true>(n, A); // the in-memory sweep: the kernel's registers are spoken for
    if (first < nrhs) {
        const LV<double> Bs = lv_from_col(B, first);
        sym_solve_lane<double, false>(n, nrhs - first, A, Bs);
    }
}

// Where the FP32 matrix lives. R0 is row `lane` (all N columns, zero for a
// lane past N). R1 is the second row part: none for N <= 32 (one unused
// register), row lane + 32 for N > 48, and for 32 < N <= 48 half of row
// 32 + lane % 16 -- columns [0, N/2) in lanes 0..15, [N/2, N) in lanes
// 16..31 -- so that no lane carries an empty row through the sweep.
template <int N> struct Rows {
    static constexpr bool TWO = N > 32;
    static constexpr bool SPLIT = TWO && N <= 48;
    static constexpr int H = N / 2;
    static constexpr int W1 = !TWO ? 1 : (SPLIT ? H : N);
    static constexpr int P0 = N / 2;          // pairs of R0
    static constexpr int P1 = (W1 + 1) / 2;   // pairs of R1
};

// z := -M z for this lane's rows, with M = -(D A D)^-1 in R0 / R1 and z
// broadcast through shared memory (SR, this warp's N floats): given z = D v,
// D z is then A32^-1 v. Row lane + 32 r is z[r] (lanes 0..15 for r = 1 when
// the second rows are split). Two partial sums per row break the FMA chain.
template <int N>
__device__ __forceinline__ void apply_inverse(int lane, const f2_t (&R0)[Rows<N>::P0],
                                              const f2_t (&R1)[Rows<N>::P1], float *SR,
                                              float (&z)[(N + 31) / 32])
{
    using L = Rows<N>;
    constexpr int NR = (N + 31) / 32;
    __syncwarp();
#pragma unroll
    for (int r = 0; r < NR; ++r)
        if (lane + 32 * r < N) SR[lane + 32 * r] = z[r];
    __syncwarp();
    // the even and odd columns' partial sums are the two halves of a pair
    const f2_t *SP = reinterpret_cast<const f2_t *>(SR);
    f2_t a0 = 0ull, a1 = 0ull;
    if constexpr (L::SPLIT) {
        const bool lower = lane < 16;
#pragma unroll
        for (int t = 0; t < L::H / 2; ++t) {
            const f2_t za = SP[t], zb = SP[t + L::H / 2];
            a0 = ffma2(R0[t], za, a0);
            a0 = ffma2(R0[t + L::H / 2], zb, a0);
            a1 = ffma2(R1[t], lower ? za : zb, a1);
        }
        float b = f2lo(a1) + f2hi(a1);
        b += __shfl_xor_sync(FULL, b, 16);
        z[0] = -(f2lo(a0) + f2hi(a0));
        z[1] = -b;
    }
    else {
#pragma unroll
        for (int j = 0; j < N / 2; ++j) {
            const f2_t zj = SP[j];
            a0 = ffma2(R0[j], zj, a0);
            if constexpr (L::TWO) a1 = ffma2(R1[j], zj, a1);
        }
        z[0] = -(f2lo(a0) + f2hi(a0));
        if constexpr (L::TWO) z[NR - 1] = -(f2lo(a1) + f2hi(a1));
    }
}

// A(i, j) of the packed triangle for a static column j: row i's own part
// (j <= i) at lo[pk_col(N, j) - j] with lo = SA + i, or column i's part
// (j > i) at hi[j] with hi = SA + pk_col(N, i) - i. Two predicated loads from
// per-lane bases with constant offsets: no index arithmetic per element.
template <int N>
__device__ __forceinline__ double tri_at(const double *lo, const double *hi, int i, int j)
{
    double a;
    if (j <= i)
        a = lo[pk_col(N, j) - j];
    else
        a = hi[j];
    return a;
}

// acc[r] := b[r] - (A x)(row lane + 32 r) from the packed FP64 triangle SA and
// x in SX. Rows 32 .. N-1 of an order N <= 48 go to both half-warps, lane l
// summing columns [0, N/2) (l < 16) or [N/2, N) (l >= 16) of row 32 + l % 16.
// Each row sums in two halves (columns below and above N/2) interleaved with
// the other row's chain: a single warp then keeps the FP64 pipe busy, where
// one chain of dependent FMAs waits out the pipe's latency at every step.
template <int N>
__device__ __forceinline__ void residual(int lane, const double *SA, const double *SX,
                                         const double (&b)[(N + 31) / 32],
                                         double (&acc)[(N + 31) / 32])
{
    constexpr int NR = (N + 31) / 32;
    constexpr int H = N / 2;
    static_assert(N % 2 == 0, "an even order");
    const int i0 = min(lane, N - 1); // lanes past N (N < 32) compute a row they discard
    const double *lo0 = SA + i0, *hi0 = SA + pk_col(N, i0) - i0;
    double s0 = b[0], s0h = 0.0;
    if constexpr (NR == 1) {
#pragma unroll
        for (int t = 0; t < H; ++t) {
            s0 = fma(-tri_at<N>(lo0, hi0, i0, t), SX[t], s0);
            s0h = fma(-tri_at<N>(lo0, hi0, i0, H + t), SX[H + t], s0h);
        }
        acc[0] = s0 + s0h;
    }
    else if constexpr (N <= 48) {
        const bool lower = lane < 16;
        const int i1 = min(32 + (lane & 15), N - 1);
        // lower half: columns t < H <= 32 <= i1, all in row i1's own part;
        // upper half: columns H + t
        const double *lo1 = SA + i1, *hi1 = SA + pk_col(N, i1) - i1;
        const double *X1 = SX + (lower ? 0 : H);
        double s1 = lower ? b[1] : 0.0;
#pragma unroll
        for (int t = 0; t < H; ++t) {
            s0 = fma(-tri_at<N>(lo0, hi0, i0, t), SX[t], s0);
            s0h = fma(-tri_at<N>(lo0, hi0, i0, H + t), SX[H + t], s0h);
            double a;
            if (lower)
                a = lo1[pk_col(N, t) - t];
            else
                a = tri_at<N>(lo1, hi1, i1, H + t);
            s1 = fma(-a, X1[t], s1);
        }
        acc[0] = s0 + s0h;
        acc[1] = s1 + __shfl_xor_sync(FULL, s1, 16);
    }
    else {
        const int i1 = min(lane + 32, N - 1);
        const double *lo1 = SA + i1, *hi1 = SA + pk_col(N, i1) - i1;
        double s1 = b[1], s1h = 0.0;
#pragma unroll
        for (int t = 0; t < H; ++t) {
            s0 = fma(-tri_at<N>(lo0, hi0, i0, t), SX[t], s0);
            s1 = fma(-tri_at<N>(lo1, hi1, i1, t), SX[t], s1);
            s0h = fma(-tri_at<N>(lo0, hi0, i0, H + t), SX[H + t], s0h);
            s1h = fma(-tri_at<N>(lo1, hi1, i1, H + t), SX[H + t], s1h);
        }
        acc[0] = s0 + s0h;
        acc[1] = s1 + s1h;
    }
}

// (s, c) of this lane's rows := (s, c) - (D A D) v in double-FP32 arithmetic
// (dot2_sub), with v = SV[0 .. N) broadcast from shared memory and the scaled
// entries d_i a_ij d_j of the packed FP64 triangle split on the integer pipe
// (D = diag(2^-SH[i]): the scaling is an exponent shift). The rows are
// residual<N>'s: row lane over all columns and, for N <= 48, row 32 + lane % 16
// by column halves, the lower half carrying the row's starting value and the
// two halves' sums joined with one exchange (both then hold the row's total);
// for N > 48 row lane + 32 over all columns (the kernel takes this path up to
// N = 40 only; the routine holds for any N).
template <int N>
__device__ __forceinline__ void ff_update(int lane, const double *SA, const int *SH,
                                          const float *SV, float (&s)[(N + 31) / 32],
                                          float (&c)[(N + 31) / 32])
{
    constexpr int NR = (N + 31) / 32;
    constexpr int H = N / 2;
    const int i0 = min(lane, N - 1); // lanes past N (N < 32) compute a row they discard
    const int c0 = pk_col(N, i0) - i0;
    const int h0 = SH[i0];
    // columns in groups of 8, to keep the kernel's code small
#pragma unroll 8
    for (int t = 0; t < N; ++t) {
        float ah, al;
        split2_rz(SA[t <= i0 ? i0 + (pk_col(N, t) - t) : c0 + t], ah, al, -(h0 + SH[t]));
        dot2_sub(s[0], c[0], ah, al, SV[t]);
    }
    if constexpr (NR == 2) {
        if constexpr (N <= 48) {
            const bool lower = lane < 16;
            const int i1 = min(32 + (lane & 15), N - 1);
            const int c1 = pk_col(N, i1) - i1;
            const int h1 = SH[i1];
            float s1 = lower ? s[1] : 0.f, k1 = lower ? c[1] : 0.f;
#pragma unroll 8
            for (int t = 0; t < H; ++t) {
                const int j = (lower ? 0 : H) + t;
                float ah, al;
                split2_rz(SA[j <= i1 ? i1 + (pk_col(N, j) - j) : c1 + j], ah, al, -(h1 + SH[j]));
                dot2_sub(s1, k1, ah, al, SV[j]);
            }
            dd_add(s1, k1, __shfl_xor_sync(FULL, s1, 16), __shfl_xor_sync(FULL, k1, 16));
            s[1] = s1;
            c[1] = k1;
        }
        else {
            const int i1 = min(lane + 32, N - 1);
            const int c1 = pk_col(N, i1) - i1;
            const int h1 = SH[i1];
#pragma unroll 8
            for (int t = 0; t < N; ++t) {
                float ah, al;
                split2_rz(SA[t <= i1 ? i1 + (pk_col(N, t) - t) : c1 + t], ah, al, -(h1 + SH[t]));
                dot2_sub(s[1], c[1], ah, al, SV[t]);
            }
        }
    }
}

template <int N, int WPB, int MINB>
__global__ void __launch_bounds__(WPB * 32, MINB)
    k_posv_refined_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                        int ldbp, int V, long nlanes, size_t sa, size_t sb, WarpOut out)
{
    constexpr int NR = (N + 31) / 32;
    constexpr int PKS = pk_stride(N);
    static_assert(N % 8 == 0 && N >= 24 && N <= 64, "padded order");
    extern __shared__ __align__(16) unsigned char smem[];
    double *const SAall = reinterpret_cast<double *>(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long m0 = (long)blockIdx.x * WPB;
    const long m = m0 + warp;
    double *const SA = SAall + warp * PKS;
    double *const SX = SAall + WPB * PKS + warp * N;       // x
    double *const SB = SAall + WPB * (PKS + N) + warp * N; // b, the right-hand side being solved
    // the pivot column twice over (SC, 16-byte aligned: N is a multiple of 8)
    // and the vector of a matrix-vector product (SR)
    float *const SC = reinterpret_cast<float *>(SAall + WPB * (PKS + 2 * N)) + warp * 5 * N;
    float *const SR = SC + 4 * N;

    // ---- stage the block's matrices: packed lower triangles, identity past n ----
    // Thread t copies matrix t % WPB, rows t / WPB + 32 s of each column, with
    // asynchronous 8-byte copies (all of a thread's copies in flight at once):
    // a warp's copies cover WPB neighbouring lanes of eight rows (whole 32-byte
    // sectors), and its shared-memory writes two wavefronts.
    {
        LV<double> A0 = lv_make<double>(ap, row, ldap, V, n, n);
        if (up) A0 = A0.t();
        const int w = threadIdx.x % WPB, rr = threadIdx.x / WPB;
        const bool have = m0 + w < nlanes;
        const long mw = have ? m0 + w : nlanes - 1;
        const long gw = mw / V;
        const double *bw = ap + gw * sa + (mw - gw * V);
        // element (j + rr + 32 s, j): its source steps by si + sj and its
        // packed index by N - j from one column to the next
        constexpr int NS = (N + 31) / 32;
        const double *src[NS];
        int dst[NS];
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            src[q] = bw + (long)(rr + 32 * q) * A0.si;
            dst[q] = w * PKS + rr + 32 * q;
        }
        const long step = A0.si + A0.sj;
#pragma unroll 1
        for (int j = 0; j < N; ++j) {
            const bool jn = have && j < n;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                const int i = j + rr + 32 * q;
                if (i < N) {
                    if (jn && i < n)
                        cp_async8(SAall + dst[q], src[q]);
                    else
                        SAall[dst[q]] = (i == j) ? 1.0 : 0.0;
                }
                src[q] += step;
                dst[q] += N - j;
            }
        }
        cp_async_wait_all();
    }
    __syncthreads();
    if (m >= nlanes) return;
    const long g = m / V;
    const int v = (int)(m - g * V);
    LV<double> Ag = lv_make<double>(ap + g * sa + v, row, ldap, V, n, n);
    if (up) Ag = Ag.t();
    const LV<double> B = lv_make<double>(bp + g * sb + v, row, ldbp, V, n, nrhs);

    // ---- the scaling D and the FP32 rows of D A D; ||A||_inf of the n rows ----
    int h[NR]; // D(i, i) = 2^-h
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const int i = lane + 32 * r;
        h[r] = 0;
        if (i < N) {
            h[r] = half_exp(SA[pk_col(N, i)]);
            SR[i] = exp2i(-h[r]);
        }
    }
    __syncwarp();
    using L = Rows<N>;
    constexpr int H = L::H;
    f2_t R0[L::P0], R1[L::P1]; // the FP32 rows, in pairs of columns
    unsigned hmax = 0; // largest high word of |a| read: a quick screen for the FP32 range
    float rs = 0.f;
    {
        const int i = min(lane, N - 1);
        const int ci = pk_col(N, i) - i;
        const bool real = N >= 32 || lane < N;
        const float di = exp2i(-h[0]);
        float sum = 0.f, prev = 0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const double a = SA[j <= i ? pk_col(N, j) - j + i : ci + j];
            hmax = max(hmax, (unsigned)__double2hiint(a) & 0x7fffffffu);
            const float f = d2f_rz_inrange(a);
            sum += fabsf(f);
            const float e = real ? f * (di * SR[j]) : 0.f;
            if (j & 1)
                R0[j >> 1] = f2(prev, e);
            else
                prev = e;
        }
        if (lane < n) rs = sum;
    }
    if constexpr (!L::TWO) {
        R1[0] = 0ull;
    }
    else if constexpr (L::SPLIT) {
        const bool lower = lane < 16;
        const int ib = 32 + (lane & 15);
        const int i = min(ib, N - 1);
        const int ci = pk_col(N, i) - i;
        const bool real = N >= 48 || ib < N;
        const float di = SR[i];
        float sum = 0.f, prev = 0.f;
#pragma unroll
        for (int t = 0; t < H; ++t) {
            const int j = (lower ? 0 : H) + t;
            const int off = lower ? pk_col(N, t) - t + i
                                  : (H + t <= i ? pk_col(N, H + t) - (H + t) + i : ci + j);
            const double a = SA[off];
            hmax = max(hmax, (unsigned)__double2hiint(a) & 0x7fffffffu);
            const float f = d2f_rz_inrange(a);
            sum += fabsf(f);
            const float e = real ? f * (di * SR[j]) : 0.f;
            if (t & 1)
                R1[t >> 1] = f2(prev, e);
            else
                prev = e;
        }
        sum += __shfl_xor_sync(FULL, sum, 16);
        if (ib < n) rs = fmaxf(rs, sum);
    }
    else {
        const int i = min(lane + 32, N - 1);
        const int ci = pk_col(N, i) - i;
        const bool real = lane + 32 < N;
        const float di = exp2i(-h[1]);
        float sum = 0.f, prev = 0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const double a = SA[j <= i ? pk_col(N, j) - j + i : ci + j];
            hmax = max(hmax, (unsigned)__double2hiint(a) & 0x7fffffffu);
            const float f = d2f_rz_inrange(a);
            sum += fabsf(f);
            const float e = real ? f * (di * SR[j]) : 0.f;
            if (j & 1)
                R1[j >> 1] = f2(prev, e);
            else
                prev = e;
        }
        if (lane + 32 < n) rs = fmaxf(rs, sum);
    }
    const float anorm = warp_max(rs);
    int status = 0;
    if (__any_sync(FULL, hmax >= 0x47efffffu)) {
        // an entry at or near the FP32 limit: the exact test, on the rare path
        bool ovf = false;
        for (int e = lane; e < pk_col(N, N); e += 32)
            ovf |= beyond_fp32(SA[e]);
        if (__any_sync(FULL, ovf)) status = -2;
    }

    // ---- FP32 inverse by the symmetric sweep: after all N pivots M = -(D A D)^-1 ----
    // pivot k, with c = column k (= row k) and p = c_k:
    //   rows i != k:  M(i,j) -= (c_i / p) c_j  (j != k),  M(i,k) = c_i / p
    //   row k:        M(k,j)  = c_j / p        (j != k),  M(k,k) = -1 / p
    // the row-k case is the same FMA with the coefficient 1/p - 1 (its row
    // equals c before the pivot), so every lane runs one instruction stream.
    // The pivots go in groups of U = 8: at the start of the group of pivots
    // k0 .. k0+7, register q of a row holds column (k0 + q) mod N, so within
    // the group every register index is static; the group ends by rotating
    // the registers by 8 (a split row passes 8 values across with shuffles).
    constexpr int U = 8;
    static_assert(N % U == 0 && U % 2 == 0 && H % 4 == 0, "pivot groups, buffers, float4 columns");
    bool nonpos = false;
    // The pivot column alternates between two buffers: a step writes the one
    // the step before last read, which every lane finished before the last
    // step's barrier -- so one barrier per step, and the next step's column
    // can be written while this step's updates are still being issued.
#pragma unroll 1
    for (int k0 = 0; k0 < N; k0 += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u;
            float *const S = (u & 1) ? SC + 2 * N : SC;
            // c = column (k0 + q) mod N from the doubled column, read in
            // pairs; the upper half of a split row reads from c[H] on
            const ulonglong2 *C4 = reinterpret_cast<const ulonglong2 *>(S + k0);
            const ulonglong2 *CB4 =
                reinterpret_cast<const ulonglong2 *>(S + k0 + ((L::SPLIT && lane >= 16) ? H : 0));
            const float r0u = el(R0, u);
            if (N >= 32 || lane < N) {
                S[lane] = r0u;
                S[lane + N] = r0u;
            }
            float r1u = 0.f;
            if constexpr (L::TWO) {
                r1u = el(R1, u);
                if ((!L::SPLIT || lane < 16) && 32 + lane < N) {
                    S[32 + lane] = r1u;
                    S[32 + lane + N] = r1u;
                }
            }
            __syncwarp();
            const float p = S[k];
            nonpos |= !(p > 0.f);
            const float rp = rcp_approx(p);
            const bool own0 = lane == k;
            const float w0 = r0u * rp;
            const float beta0 = own0 ? rp - 1.0f : -w0;
            const float last0 = own0 ? -rp : w0;
            float betab = 0.f, lastb = 0.f;
            if constexpr (L::TWO) {
                float vb = r1u;
                if constexpr (L::SPLIT) {
                    const float o = __shfl_xor_sync(FULL, r1u, 16);
                    vb = lane < 16 ? r1u : o; // column k of row 32 + lane % 16
                }
                const bool ownb = (L::SPLIT ? 32 + (lane & 15) : 32 + lane) == k;
                const float wb = vb * rp;
                betab = ownb ? rp - 1.0f : -wb;
                lastb = ownb ? -rp : wb;
            }
            const f2_t bb0 = f2(beta0, beta0), bb1 = f2(betab, betab);
            const int PU = u >> 1, UO = u ^ 1; // u's pair, the other column in it
#pragma unroll
            for (int q4 = 0; q4 < N / 4; ++q4) {
                const ulonglong2 c = C4[q4];
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int P = 2 * q4 + hh;
                    const f2_t cp = hh ? c.y : c.x;
                    if (P != PU) {
                        R0[P] = ffma2(bb0, cp, R0[P]);
                        if constexpr (L::TWO && !L::SPLIT) R1[P] = ffma2(bb1, cp, R1[P]);
                    }
                    else {
                        // column u takes its final value; the other is updated
                        const float co = (UO & 1) ? f2hi(cp) : f2lo(cp);
                        const float n0 = fmaf(beta0, co, el(R0, UO));
                        R0[P] = (u & 1) ? f2(n0, last0) : f2(last0, n0);
                        if constexpr (L::TWO && !L::SPLIT) {
                            const float n1 = fmaf(betab, co, el(R1, UO));
                            R1[P] = (u & 1) ? f2(n1, lastb) : f2(lastb, n1);
                        }
                    }
                }
            }
            if constexpr (L::SPLIT) {
#pragma unroll
                for (int t4 = 0; t4 < H / 4; ++t4) {
                    const ulonglong2 c = CB4[t4];
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh) {
                        const int P = 2 * t4 + hh;
                        const f2_t nv = ffma2(bb1, hh ? c.y : c.x, R1[P]);
                        if (P == PU) {
                            // the pivot column sits in the lower half (u < 8 <= H)
                            const float eu = lane < 16 ? lastb : ((u & 1) ? f2hi(nv) : f2lo(nv));
                            R1[P] = (u & 1) ? f2(f2lo(nv), eu) : f2(eu, f2hi(nv));
                        }
                        else {
                            R1[P] = nv;
                        }
                    }
                }
            }
        }
        // rotate by U: register pair q takes columns k0 + U + 2q, +1
        constexpr int UP = U / 2;
        {
            f2_t t0[UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                t0[e] = R0[e];
#pragma unroll
            for (int q = 0; q < L::P0 - UP; ++q)
                R0[q] = R0[q + UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                R0[L::P0 - UP + e] = t0[e];
        }
        if constexpr (L::TWO && !L::SPLIT) {
            f2_t t1[UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                t1[e] = R1[e];
#pragma unroll
            for (int q = 0; q < L::P1 - UP; ++q)
                R1[q] = R1[q + UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                R1[L::P1 - UP + e] = t1[e];
        }
        if constexpr (L::SPLIT) {
            // lower half: V[t] = V[t + 8], the last 8 from the upper half's
            // first 8; upper half: the same, the last 8 from the lower half's
            f2_t t1[UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                t1[e] = __shfl_xor_sync(FULL, R1[e], 16);
#pragma unroll
            for (int q = 0; q < L::P1 - UP; ++q)
                R1[q] = R1[q + UP];
#pragma unroll
            for (int e = 0; e < UP; ++e)
                R1[L::P1 - UP + e] = t1[e];
        }
    }
    if (nonpos && status == 0) status = -1;
    // up to order 40 the first residual is taken in double-FP32 (below); it
    // needs the row scales h of every row, kept in the sweep's column buffers
    // (free now)
    constexpr bool FF_FIRST = N <= 40;
    int *const SH = reinterpret_cast<int *>(SC);
    if constexpr (FF_FIRST) {
        __syncwarp();
#pragma unroll
        for (int r = 0; r < NR; ++r)
            if (lane + 32 * r < N) SH[lane + 32 * r] = h[r];
    }
    // this lane's residual rows: lane, and lane + 32 or (N <= 48) 32 + lane % 16
    const int i0 = min(lane, N - 1);
    const int i1 = min(L::SPLIT ? 32 + (lane & 15) : lane + 32, N - 1);
    const bool real0 = lane < n;
    const bool real1 = NR == 2 && (L::SPLIT ? lane < 16 : true) && lane + 32 < n;

    // LAPACK dsposv's test ||r|| <= sqrt(n) eps64 ||A|| ||x||, in FP32 while
    // the right side is a normal FP32 number, in FP64 below that
    const double cte = (double)anorm * EPS64 * sqrt((double)n);
    const float cte32 = (float)cte;
    int it_max = 0, col = 0;
    float worst = 0.f;
    for (; col < nrhs && status == 0; ++col) {
        // all FP64 <-> FP32 conversions here are integer operations; w holds
        // D b and then D r (the scaling folded into the exponent). x and b
        // live in shared memory: registers are kept for the FP32 rows.
        float w[NR];
        float bn = 0.f;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const int i = lane + 32 * r;
            const double b = (i < n) ? B(i, col) : 0.0;
            if (i < N) SB[i] = b;
            bn = fmaxf(bn, fabsf(d2f_rz(b)));
            w[r] = d2f_rz(b, -h[r]);
        }
        bn = warp_max(bn);
        apply_inverse<N>(lane, R0, R1, SR, w);
        float xn = 0.f;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const int i = lane + 32 * r;
            const double x = (i < n) ? f2d_int(w[r], -h[r]) : 0.0;
            xn = fmaxf(xn, fabsf(d2f_rz(x)));
            if (i < N) SX[i] = x;
        }
        xn = warp_max(xn);
        // Up to order 40 the first residual is taken in double-FP32 on the
        // FP32 pipe: rs + rc = D b - (D A D) w0, w0 = D^-1 x0 exact in FP32
        // (Dot2 over the two-float split of A, ff_update). Its error, near
        // n 2^-48 ||A|| ||x||, is far below the first residual (about eps32
        // ||A|| ||x||), so the first correction is as good as from an FP64
        // residual; every later residual, and every stopping test, is FP64
        // (a correction from a double-FP32 residual would leave its error in
        // x). Measured at 262,144 matrices: n = 24 1.40 against 1.65 ms,
        // n = 32 1.78 against 2.01, n = 40 4.17 against 4.31; from n = 48 on
        // the extra code in a kernel at its register cap cost more than the
        // FP64 residual it saves (5.64 against 5.41 ms), so it is left out.
        float rprev = INFINITY;
        for (int it = 0;; ++it) {
            bool fp64 = true;
            float rn = 0.f;
            if (FF_FIRST && it == 0) {
                float rs_[NR], rc_[NR];
                __syncwarp();
#pragma unroll
                for (int r = 0; r < NR; ++r)
                    if (lane + 32 * r < N) SR[lane + 32 * r] = (lane + 32 * r < n) ? w[r] : 0.f;
                __syncwarp();
                split2_rz_any(SB[i0], rs_[0], rc_[0], -SH[i0]);
                if constexpr (NR == 2) split2_rz_any(SB[i1], rs_[1], rc_[1], -SH[i1]);
                ff_update<N>(lane, SA, SH, SR, rs_, rc_);
                bool nan = false;
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const bool real = r == 0 ? real0 : real1;
                    const float v = real ? fabsf(rs_[r] + rc_[r]) * exp2i(SH[r == 0 ? i0 : i1]) : 0.f;
                    nan |= v != v;
                    rn = fmaxf(rn, v);
                }
                rn = warp_max(rn);
                // FP64 unless clearly above the stopping threshold and finite
                const float clear = cte32 * xn + 0x1p-40f * anorm * xn;
                fp64 = __any_sync(FULL, nan) || !(rn > clear && rn <= FLT_MAX);
                if (!fp64) {
#pragma unroll
                    for (int r = 0; r < NR; ++r)
                        w[r] = (lane + 32 * r < n) ? rs_[r] + rc_[r] : 0.f;
                }
            }
            if (fp64) {
                __syncwarp();
                double acc[NR];
#pragma unroll
                for (int r = 0; r < NR; ++r)
                    acc[r] = (lane + 32 * r < N) ? SB[lane + 32 * r] : 0.0;
                residual<N>(lane, SA, SX, acc, acc);
                rn = 0.f;
                bool nan = false; // fmaxf drops a NaN: a NaN residual must stop the refinement
#pragma unroll
                for (int r = 0; r < NR; ++r) {
                    const bool real = lane + 32 * r < n;
                    const float v = real ? fabsf(d2f_rz(acc[r])) : 0.f;
                    nan |= v != v;
                    rn = fmaxf(rn, v);
                    w[r] = real ? d2f_rz(acc[r], -h[r]) : 0.f;
                }
                rn = __any_sync(FULL, nan) ? NAN : warp_max(rn);
                const float thr = cte32 * xn;
                const bool done = thr >= 0x1p-100f ? rn <= thr : (double)rn <= cte * (double)xn;
                if (done) {
                    const float den = anorm * xn + bn;
                    worst = fmaxf(worst, den > 0.f ? rn / den : 0.f);
                    it_max = max(it_max, it);
                    break;
                }
            }
            if (it >= out.max_iter || !(rn <= 0.5f * rprev)) {
                status = -3;
                break;
            }
            rprev = rn;
            apply_inverse<N>(lane, R0, R1, SR, w); // syncs the warp: SX reads are done
            float xm = 0.f;
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const int i = lane + 32 * r;
                if (i < n) {
                    const double x = SX[i] + f2d_int(w[r], -h[r]);
                    SX[i] = x;
                    xm = fmaxf(xm, fabsf(d2f_rz(x)));
                }
            }
            xn = warp_max(xm);
        }
        if (status == 0) {
            __syncwarp();
#pragma unroll
            for (int r = 0; r < NR; ++r)
                if (lane + 32 * r < n) B(lane + 32 * r, col) = SX[lane + 32 * r];
        }
    }
    if (status != 0 && lane == 0) warp_fallback(n, nrhs, status == -3 ? col - 1 : 0, Ag, B);
    if (lane == 0 && m < out.nm) {
        if (out.iters) out.iters[m] = status != 0 ? status : it_max;
        if (out.berr) out.berr[m] = status != 0 ? (double)NAN : (double)worst;
    }
}

template <int N, int WPB, int MINB>
cudaError_t launch_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                        int ldbp, int V, int nm, const WarpOut &out, cudaStream_t s, size_t sa,
                        size_t sb)
{
    const long ng = ((long)nm + V - 1) / V;
    const long nlanes = ng * V;
    constexpr size_t smem = warp_smem_bytes<N, WPB>();
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k_posv_refined_warp<N, WPB, MINB>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
        if (e != cudaSuccess) return e;
    }
    const unsigned blocks = (unsigned)((nlanes + WPB - 1) / WPB);
    k_posv_refined_warp<N, WPB, MINB><<<blocks, WPB * 32, smem, s>>>(
        row, up, n, nrhs, ap, ldap, bp, ldbp, V, nlanes, sa, sb, out);
    return cudaGetLastError();
}

} // namespace

} // namespace cbkcuda
