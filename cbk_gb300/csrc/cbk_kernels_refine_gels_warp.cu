// cbk_kernels_refine_gels_warp.cu -- the mixed-precision least-squares solve
// for m <= 64 and n in {8, 16}, one warp per matrix.
//
// The method is cbk_kernels_refine_gels.cu's (FP32 QR, FP64 refinement of the
// augmented system [I A; A^T 0][r; x] = [b; 0] (Bjorck), residual-based
// stopping, per-matrix FP64 fallback, the same outputs); the mapping differs.
// One thread per matrix keeps the FP32 QR in a global workspace and waits on
// memory at every step, and a warp of 32 matrices runs until its slowest
// lane converges. Here the 32 lanes share one matrix:
//   * the block's four matrices are staged into shared memory in FP64 with
//     asynchronous copies (coalesced across the block), column-major with
//     rows past m zero (which changes no result); the FP64 residuals read A
//     from there at every step;
//   * lane l takes rows l and l + 32 of the FP32 copy into registers, and
//     the FP32 Householder QR works on these rows: each column's norm and
//     each reflector application is a warp sum (the trailing columns' sums
//     interleaved); the factored columns (R and the reflectors) are stored
//     to shared memory;
//   * the thin Q1 (m x n, in registers) and R^-1 (shared memory) are formed
//     explicitly once per matrix. A correction is then t = Q1^T f - R^-T g,
//     dx = R^-1 t and dr = f - Q1 t: two column sums and three broadcast
//     products instead of 2n dependent reflector applications. The
//     reflectors themselves are applied once per right-hand side, for the
//     residual coordinates returned in B(n:m);
//   * per step f = b - r - A x is row-parallel (x broadcast from shared
//     memory), and g = -A^T r takes 32/n lanes per column, each over
//     interleaved rows, then log2(32/n) shuffle-adds: the FP64 work is the
//     FMAs alone, with no reduction tree per column.
// The FP64 work is the lane kernel's (2 m n fused multiply-adds per
// right-hand side and step, less the first step's f, see below), with every
// lane of the warp busy until its one matrix converges.
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <float.h>
#include <math.h>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr double EPS64 = 2.220446049250313e-16;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float wsum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(FULL, v, o);
    return v;
}

__device__ __forceinline__ float wmax(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmax_nan(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// The N column sums of p[N] over the warp by recursive halving: each exchange
// sends half of the values still held, so the sums cost N - 1 + log2(32 / N)
// additions and shuffles per lane. After it lane l holds the sum of column
// l >> (5 - log2 N).
template <typename T, int N> __device__ __forceinline__ T column_sums(int lane, T (&p)[N])
{
    static_assert(N == 8 || N == 16, "N is 8 or 16");
    constexpr int LOGN = N == 8 ? 3 : 4;
#pragma unroll
    for (int s = 0; s < LOGN; ++s) {
        const int o = 16 >> s;
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int t = 0; t < (N >> (s + 1)); ++t) {
            const int h = N >> (s + 1);
            const T send = upper ? p[t] : p[t + h];
            const T keep = upper ? p[t + h] : p[t];
            p[t] = keep + __shfl_xor_sync(FULL, send, o);
        }
    }
    T v = p[0];
#pragma unroll
    for (int o = 16 >> LOGN; o > 0; o >>= 1)
        v += __shfl_xor_sync(FULL, v, o);
    return v;
}

struct GelsOut {
    int *iters;
    double *berr;
    int nm;
    int max_iter;
};

// The per-warp shared memory of k_gels_refined_warp<MR, N>: m <= 32 MR rows
// (MP, zero past m), N columns.
template <int MR, int N> struct GW {
    static constexpr int MP = 32 * MR;
    static constexpr int HB = 32 / N;          // lanes per column in the sums A^T r
    static constexpr int S = N == 8 ? 2 : 1;   // log2 HB
    static constexpr int RB = MP / HB;         // rows per lane in A^T r
    // column stride of the FP64 copy of A, in doubles: == HB (mod 16), so the
    // A^T r reads (lane: column lane >> S, rows lane & (HB-1) + HB t) meet 32
    // distinct banks per 16 lanes, and the row-parallel reads are contiguous
    static constexpr int CS = MP + HB;
    static constexpr int RS = N + 1;           // row stride of R^-1, in floats
    static constexpr int OFF_R = N * CS * 8;              // r, FP64, MP
    static constexpr int OFF_X = OFF_R + MP * 8;          // x, FP64, N
    static constexpr int OFF_V = OFF_X + N * 8;           // the FP32 QR, column-major, N x MP
    static constexpr int OFF_TAU = OFF_V + N * MP * 4;    // tau, FP32, N
    static constexpr int OFF_RI = OFF_TAU + N * 4;        // R^-1, FP32, row-major N x RS
    static constexpr int OFF_G = OFF_RI + N * RS * 4;     // a broadcast vector, FP32, N
    static constexpr int OFF_T = OFF_G + N * 4;           // another, FP32, N
    static constexpr int BYTES = (OFF_T + N * 4 + 15) / 16 * 16;
    static_assert(OFF_G % 16 == 0 && OFF_T % 16 == 0, "broadcast vectors are read as float4");
};

// sum_i w[i] s[i], s a 16-byte aligned shared vector read by the whole warp
template <int N> __device__ __forceinline__ float dot_bcast(const float (&w)[N], const float *s)
{
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < N; q += 4) {
        const float4 v = *reinterpret_cast<const float4 *>(s + q);
        acc = fmaf(w[q + 0], v.x, acc);
        acc = fmaf(w[q + 1], v.y, acc);
        acc = fmaf(w[q + 2], v.z, acc);
        acc = fmaf(w[q + 3], v.w, acc);
    }
    return acc;
}

// The FP32 Householder QR of the warp's register rows q (row lane + 32 r),
// geqr2 as geqrf_lane: per column the tail sum of squares, the branch-free
// larfg (no reflector when the tail is exactly zero), then H applied to the
// trailing columns with one warp sum per column (independent, interleaved).
template <int MR, int N>
__device__ __forceinline__ void qr_rows(int lane, float (&q)[MR][N], float *stau)
{
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float tl = 0.f;
#pragma unroll
        for (int r = 0; r < MR; ++r)
            if (r > 0 || lane > k) tl = fmaf(q[r][k], q[r][k], tl);
        const float tail = wsum(tl);
        const float x0 = __shfl_sync(FULL, q[0][k], k);
        const float norm = sqrtf(fmaf(x0, x0, tail));
        const float beta = x0 >= 0.f ? -norm : norm;
        const bool has = tail > 0.f;
        const float tau = has ? (beta - x0) / beta : 0.f;
        const float inv = has ? 1.f / (x0 - beta) : 0.f;
        float v[MR];
#pragma unroll
        for (int r = 0; r < MR; ++r) {
            if (r > 0 || lane > k) q[r][k] *= inv;
            v[r] = (r > 0 || lane > k) ? q[r][k] : (lane == k ? 1.f : 0.f);
        }
        if (lane == k) q[0][k] = has ? beta : x0;
        if (lane == 0) stau[k] = tau;
        float s[N];
#pragma unroll
        for (int j = k + 1; j < N; ++j) {
            float a = 0.f;
#pragma unroll
            for (int r = 0; r < MR; ++r)
                a = fmaf(v[r], q[r][j], a);
            s[j] = a;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int j = k + 1; j < N; ++j)
                s[j] += __shfl_xor_sync(FULL, s[j], o);
#pragma unroll
        for (int j = k + 1; j < N; ++j) {
            const float w = s[j] * tau;
#pragma unroll
            for (int r = 0; r < MR; ++r)
                q[r][j] = fmaf(-v[r], w, q[r][j]);
        }
    }
}

// The thin Q1 = H_0 .. H_{N-1} [I; 0] in the register rows e (orgqr's backward
// accumulation; the reflectors are read from the stored QR sv)
template <int MR, int N>
__device__ __forceinline__ void form_q1(int lane, const float *sv, const float *stau,
                                        float (&e)[MR][N])
{
    constexpr int MP = 32 * MR;
#pragma unroll
    for (int r = 0; r < MR; ++r)
#pragma unroll
        for (int j = 0; j < N; ++j)
            e[r][j] = (r == 0 && lane == j) ? 1.f : 0.f;
#pragma unroll
    for (int k = N - 1; k >= 0; --k) {
        const float tau = stau[k];
        float v[MR];
#pragma unroll
        for (int r = 0; r < MR; ++r)
            v[r] = (r > 0 || lane > k) ? sv[k * MP + lane + 32 * r] : (lane == k ? 1.f : 0.f);
        float s[N];
#pragma unroll
        for (int j = k; j < N; ++j) {
            float a = 0.f;
#pragma unroll
            for (int r = 0; r < MR; ++r)
                a = fmaf(v[r], e[r][j], a);
            s[j] = a;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int j = k; j < N; ++j)
                s[j] += __shfl_xor_sync(FULL, s[j], o);
#pragma unroll
        for (int j = k; j < N; ++j) {
            const float w = s[j] * tau;
#pragma unroll
            for (int r = 0; r < MR; ++r)
                e[r][j] = fmaf(-v[r], w, e[r][j]);
        }
    }
}

// Q^T w for the register rows w, the reflectors applied one by one
template <int MR, int N>
__device__ __forceinline__ void apply_qt(int lane, const float *sv, const float *stau,
                                         float (&w)[MR])
{
    constexpr int MP = 32 * MR;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        float v[MR], a = 0.f;
#pragma unroll
        for (int r = 0; r < MR; ++r) {
            v[r] = (r > 0 || lane > k) ? sv[k * MP + lane + 32 * r] : (lane == k ? 1.f : 0.f);
            a = fmaf(v[r], w[r], a);
        }
        const float s = wsum(a) * stau[k];
#pragma unroll
        for (int r = 0; r < MR; ++r)
            w[r] = fmaf(-v[r], s, w[r]);
    }
}

template <int MR, int N, int WPB, int MINB>
__global__ void __launch_bounds__(32 * WPB, MINB)
    k_gels_refined_warp(bool row, int m, int nrhs, double *ap, int ldap, double *bp, int ldbp,
                        double *taup, int V, long total, size_t sa, size_t sb, GelsOut out)
{
    using G = GW<MR, N>;
    constexpr int MP = G::MP, CS = G::CS, HB = G::HB, S = G::S, RB = G::RB, RS = G::RS;
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long first = (long)blockIdx.x * WPB;

    // the block's matrices, FP64, into shared memory (rows past m zero)
    for (int e = threadIdx.x; e < WPB * MP * N; e += 32 * WPB) {
        const int w = e % WPB, rest = e / WPB, i = rest % MP, j = rest / MP;
        const long idx = first + w;
        if (idx >= total) continue;
        double *dst = reinterpret_cast<double *>(smem + w * G::BYTES) + j * CS + i;
        if (i < m) {
            const long g = idx / V;
            const int v = (int)(idx - g * V);
            const LV<double> A = lv_make<double>(ap + g * sa + v, row, ldap, V, m, N);
            cp_async8(dst, &A(i, j));
        }
        else {
            *dst = 0.0;
        }
    }
    cp_async_wait_all();
    __syncthreads();
    const long idx = first + warp;
    if (idx >= total) return;

    unsigned char *ws = smem + warp * G::BYTES;
    const double *sA = reinterpret_cast<const double *>(ws);
    double *sR = reinterpret_cast<double *>(ws + G::OFF_R);
    double *sX = reinterpret_cast<double *>(ws + G::OFF_X);
    float *sV = reinterpret_cast<float *>(ws + G::OFF_V);
    float *sTau = reinterpret_cast<float *>(ws + G::OFF_TAU);
    float *sRi = reinterpret_cast<float *>(ws + G::OFF_RI);
    float *sG = reinterpret_cast<float *>(ws + G::OFF_G);
    float *sT = reinterpret_cast<float *>(ws + G::OFF_T);
    const long g = idx / V;
    const int v = (int)(idx - g * V);
    const LV<double> B = lv_make<double>(bp + g * sb + v, row, ldbp, V, m, nrhs);
    const int jg = lane >> S;        // this lane's column in the column-wise phases
    const int hb = lane & (HB - 1);  // its row phase in A^T r
    int status = 0;

    // the FP32 copy: range check (LAPACK dlag2s), ||A||_inf, QR
    float q[MR][N];
    bool big = false;
    float rs[MR];
#pragma unroll
    for (int r = 0; r < MR; ++r) {
        rs[r] = 0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const double a = sA[j * CS + lane + 32 * r];
            big |= beyond_fp32(a);
            q[r][j] = d2f_rz_inrange(a);
            rs[r] += fabsf(q[r][j]);
        }
    }
    float anorm = rs[0];
#pragma unroll
    for (int r = 1; r < MR; ++r)
        anorm = fmaxf(anorm, rs[r]);
    anorm = wmax(anorm);
    if (__any_sync(FULL, big)) status = -2;

    float e[MR][N]; // Q1, the thin FP32 Q
    float rc[N];    // column jg of R^-1
    if (status == 0) {
        qr_rows<MR, N>(lane, q, sTau);
#pragma unroll
        for (int r = 0; r < MR; ++r)
#pragma unroll
            for (int j = 0; j < N; ++j)
                sV[j * MP + lane + 32 * r] = q[r][j];
        __syncwarp();
        form_q1<MR, N>(lane, sV, sTau, e);
        // R^-1 column by column (column jg per lane), by back substitution
        // on the stored R: R(i, l) = sV[l MP + i]
#pragma unroll
        for (int i = N - 1; i >= 0; --i) {
            float s = (i == jg) ? 1.f : 0.f;
#pragma unroll
            for (int l = i + 1; l < N; ++l)
                s = fmaf(-sV[l * MP + i], rc[l], s);
            rc[i] = s / sV[i * MP + i];
        }
        if (hb == 0)
#pragma unroll
            for (int i = 0; i < N; ++i)
                sRi[i * RS + jg] = rc[i];
        __syncwarp();
    }

    const double cte = EPS64 * sqrt((double)N);
    const float cte32 = (float)cte;
    int it_max = 0, col = 0;
    float worst = 0.f;
    for (; col < nrhs && status == 0; ++col) {
        double b[MR], rr[MR];
        float bf[MR], bn = 0.f;
#pragma unroll
        for (int r = 0; r < MR; ++r) {
            const int i = lane + 32 * r;
            b[r] = i < m ? B(i, col) : 0.0;
            bf[r] = d2f_rz(b[r]);
            bn = fmaxf(bn, fabsf(bf[r]));
        }
        bn = wmax(bn);
        // x0 = R^-1 (Q1^T b) in FP32
        float p[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float a = 0.f;
#pragma unroll
            for (int r = 0; r < MR; ++r)
                a = fmaf(e[r][j], bf[r], a);
            p[j] = a;
        }
        const float c = column_sums<float, N>(lane, p);
        if (hb == 0) sT[jg] = c;
        __syncwarp();
        float ri[N]; // row jg of R^-1
#pragma unroll
        for (int i = 0; i < N; ++i)
            ri[i] = sRi[jg * RS + i];
        double x = f2d_int(dot_bcast<N>(ri, sT));
        if (hb == 0) sX[jg] = x;
        __syncwarp();
        // r0 = b - A x0 (FP64)
#pragma unroll
        for (int r = 0; r < MR; ++r) {
            const int i = lane + 32 * r;
            double acc = b[r];
#pragma unroll
            for (int j = 0; j < N; ++j)
                acc = fma(-sA[j * CS + i], sX[j], acc);
            rr[r] = acc;
            sR[i] = acc;
        }
        __syncwarp();
        // refinement of the augmented system until both residuals reach the
        // FP64 rounding level of their terms (the lane kernel's test)
        float gprev = INFINITY, fprev = INFINITY;
        for (int it = 0;; ++it) {
            // f = b - r - A x (rows) and g = -A^T r (columns, HB lanes each).
            // At the first step r is the FP64 residual of x just computed, and
            // f only its rounding error (far below the correction g brings):
            // it is taken as zero, which saves a third of that step's FP64 work.
            float ff[MR], fn = 0.f, rn = 0.f;
            if (it == 0) {
#pragma unroll
                for (int r = 0; r < MR; ++r) {
                    ff[r] = 0.f;
                    rn = fmaxf(rn, fabsf(d2f_rz(rr[r])));
                }
            }
            else {
#pragma unroll
                for (int r = 0; r < MR; ++r) {
                    const int i = lane + 32 * r;
                    double acc = b[r] - rr[r];
#pragma unroll
                    for (int j = 0; j < N; ++j)
                        acc = fma(-sA[j * CS + i], sX[j], acc);
                    ff[r] = d2f_rz(acc);
                    fn = fmax_nan(fn, fabsf(ff[r]));
                    rn = fmaxf(rn, fabsf(d2f_rz(rr[r])));
                }
            }
            double gp = 0.0;
#pragma unroll
            for (int t = 0; t < RB; ++t) {
                const int i = hb + HB * t;
                gp = fma(-sA[jg * CS + i], sR[i], gp);
            }
#pragma unroll
            for (int o = 1; o < HB; o <<= 1)
                gp += __shfl_xor_sync(FULL, gp, o);
            const float h0 = d2f_rz(gp);
            float gn = fabsf(h0), xn = fabsf(d2f_rz(x));
            fn = wmax(fn);
            rn = wmax(rn);
#pragma unroll
            for (int o = HB; o < 32; o <<= 1) {
                gn = fmax_nan(gn, __shfl_xor_sync(FULL, gn, o));
                xn = fmaxf(xn, __shfl_xor_sync(FULL, xn, o));
            }
            if (fn != fn || gn != gn) { // a NaN residual never converges
                status = -3;
                break;
            }
            const float scale = anorm * xn + bn;
            const float thf = cte32 * (scale + rn), thg = anorm * thf;
            bool done;
            if (thg >= 0x1p-100f && thf >= 0x1p-100f && thg <= 0x1p100f && thf <= 0x1p100f) {
                done = gn <= thg && fn <= thf;
            }
            else {
                const double sc = (double)anorm * xn + bn;
                done = (double)gn <= cte * (double)anorm * (sc + rn) &&
                       (double)fn <= cte * (sc + rn);
            }
            if (done) {
                const float den = anorm * (anorm * xn + bn);
                worst = fmaxf(worst, den > 0.f ? gn / den : 0.f);
                it_max = max(it_max, it);
                break;
            }
            if (it >= out.max_iter || (gn > 0.5f * gprev && fn > 0.5f * fprev)) {
                status = -3;
                break;
            }
            gprev = gn;
            fprev = fn;
            // h = R^-T g, w1 = Q1^T f, t = w1 - h, dx = R^-1 t, dr = f - Q1 t
            if (hb == 0) sG[jg] = h0;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                float a = 0.f;
#pragma unroll
                for (int r = 0; r < MR; ++r)
                    a = fmaf(e[r][j], ff[r], a);
                p[j] = a;
            }
            const float w1 = column_sums<float, N>(lane, p);
            __syncwarp();
            const float hj = dot_bcast<N>(rc, sG);
            if (hb == 0) sT[jg] = w1 - hj;
            __syncwarp();
            x += f2d_int(dot_bcast<N>(ri, sT));
#pragma unroll
            for (int r = 0; r < MR; ++r) {
                const int i = lane + 32 * r;
                rr[r] += f2d_int(ff[r] - dot_bcast<N>(e[r], sT));
                sR[i] = rr[r];
            }
            __syncwarp();
            if (hb == 0) sX[jg] = x;
            __syncwarp();
        }
        if (status == 0) {
            // B(0:n) := x; B(n:m) := (Q^T r)(n:m), the residual's coordinates
            float w[MR];
#pragma unroll
            for (int r = 0; r < MR; ++r)
                w[r] = d2f_rz(rr[r]);
            apply_qt<MR, N>(lane, sV, sTau, w);
            if (hb == 0) B(jg, col) = x;
#pragma unroll
            for (int r = 0; r < MR; ++r) {
                const int i = lane + 32 * r;
                if (i >= N && i < m) B(i, col) = (double)w[r];
            }
        }
        __syncwarp();
    }
    if (status != 0 && lane == 0) {
        const LV<double> A = lv_make<double>(ap + g * sa + v, row, ldap, V, m, N);
        gels_fallback_lane(m, N, nrhs, status == -3 ? col - 1 : 0, A,
                           taup + g * ((size_t)N * V) + v, V, B);
    }
    if (lane == 0 && idx < out.nm) {
        if (out.iters) out.iters[idx] = status != 0 ? status : it_max;
        if (out.berr) out.berr[idx] = status != 0 ? (double)NAN : (double)worst;
    }
}

} // namespace

namespace {

template <int MR, int N, int MINB>
cudaError_t launch_warp_gels(bool row, int m, int nrhs, double *ap, int ldap, double *bp, int ldbp,
                             double *taup, int V, int nm, GelsOut out, cudaStream_t s, size_t sa,
                             size_t sb)
{
    constexpr int WPB = 4;
    const size_t smem = (size_t)WPB * GW<MR, N>::BYTES;
    // per device, so on every launch (the current device may change)
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k_gels_refined_warp<MR, N, WPB, MINB>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
        if (e != cudaSuccess) return e;
    }
    const long ng = ((long)nm + V - 1) / V;
    const long total = ng * V;
    const unsigned blocks = (unsigned)((total + WPB - 1) / WPB);
    k_gels_refined_warp<MR, N, WPB, MINB><<<blocks, 32 * WPB, smem, s>>>(
        row, m, nrhs, ap, ldap, bp, ldbp, taup, V, total, sa, sb, out);
    return cudaGetLastError();
}

} // namespace

bool gels_refined_warp_ok(int m, int n)
{
    return (n == 8 || n == 16) && m >= n && m <= 64;
}

cudaError_t launch_gels_refined_warp(bool row, int m, int n, int nrhs, double *ap, int ldap,
                                     double *bp, int ldbp, double *taup, int V, int nm,
                                     int max_iter, int *iters, double *berr, cudaStream_t s,
                                     size_t sa_, size_t sb_)
{
    const GelsOut out{iters, berr, nm, max_iter};
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, m, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, m, nrhs, V);
    if (n == 16)
        return m <= 32 ? launch_warp_gels<1, 16, 4>(row, m, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                                    out, s, sa, sb)
                       : launch_warp_gels<2, 16, 3>(row, m, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                                    out, s, sa, sb);
    if (n == 8)
        return m <= 32 ? launch_warp_gels<1, 8, 4>(row, m, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                                   out, s, sa, sb)
                       : launch_warp_gels<2, 8, 4>(row, m, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                                   out, s, sa, sb);
    return cudaErrorInvalidValue;
}

} // namespace cbkcuda
