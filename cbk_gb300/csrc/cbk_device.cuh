// cbk_device.cuh -- per-lane device algorithms of the compact batch kernels.
//
// Thread model: one CUDA thread advances one matrix of the compact batch (one
// "lane" v of group g). Element (i,j) of V consecutive matrices is stored in V
// adjacent scalars (include/cbk.h:22-29 of the reference), so the 32 threads
// of a warp reading element (i,j) of 32 consecutive lanes issue one coalesced
// 256-byte (FP64) or 128-byte (FP32) access. Every lane of the grid runs,
// including the padded lanes of a partial last group, exactly as the
// reference's SIMD lanes do (src/cbk_common.hpp:277-297): a padded identity
// lane factors and solves harmlessly, and the whole buffer comes out as the
// reference leaves it.
//
// The algorithms below are the reference's (right-looking, recursive-panel
// Cholesky / LDL^T with the reordered pivot, row-dot substitution, geqr2 with
// the branch-free larfg, dlarf sweeps, org2r), restated for one lane:
//  * factorizations are blocked left-looking by 8-column panels: a panel's
//    columns first take the whole rank-j0 update from the finished columns in
//    pivot order (4 x 8 register tiles), then the in-panel rank-1 sweep
//    (each row below the panel's diagonal block in registers) --
//    the same per-element operation sequence as the reference's recursion
//    (src/cbk_potrf_compact.hpp:79-124, src/cbk_sytrfnp_compact.hpp:96-254);
//  * the FP64 pipe of a GB300 SM retires about two FMAs per clock, so each
//    element update is one fused multiply-add and repeated divides by the
//    same pivot become one reciprocal (results then differ from the
//    reference by rounding only, within the tests' n*eps bounds);
//  * integer address arithmetic is free next to FP64 work and is left plain.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cbkdev {

// ---------------------------------------------------------------------
// The checked build (CBK_CUDA_CHECKED defined: libcbk_cuda_checked.so)
// ---------------------------------------------------------------------
// Every element access through a matrix view (LV below) is tested against
// the matrix's logical extent -- 0 <= i < rows, 0 <= j < cols of the view --
// before it is made. An access outside is not made: it reads or writes a
// scratch element instead, counts itself in this translation unit's status
// word and records its (i, j) if it was the first; the host reads the words
// through cbk_cuda_check_status. No trap, no fault: the kernel runs on. The
// normal build compiles none of this (the view carries no extent).
#ifdef CBK_CUDA_CHECKED
struct CheckWord {
    unsigned long long count; // accesses outside their view
    unsigned long long first; // (i << 32) | j of the first, as unsigned 32-bit halves
};
static __device__ CheckWord g_check;
static __device__ double g_check_scratch;
// the host side keeps its own scratch and word (host-side uses of a view)
inline CheckWord &host_check_word()
{
    static CheckWord w{0, 0};
    return w;
}
inline double &host_check_scratch()
{
    static double d = 0.0;
    return d;
}

template <typename T> __host__ __device__ inline T &check_fail(int i, int j)
{
    const unsigned long long code = ((unsigned long long)(unsigned)i << 32) | (unsigned)j;
#ifdef __CUDA_ARCH__
    if (atomicAdd(&g_check.count, 1ull) == 0ull) g_check.first = code;
    return *reinterpret_cast<T *>(&g_check_scratch);
#else
    if (host_check_word().count++ == 0) host_check_word().first = code;
    return *reinterpret_cast<T *>(&host_check_scratch());
#endif
}
#endif

#ifdef CBK_CUDA_CHECKED
} // namespace cbkdev

namespace cbkcuda {
// one reader per translation unit's status word; cbk_cuda_check_status sums
// them (count; first (i, j) of the first unit that has one; reset to zero)
typedef int (*CheckReader)(unsigned long long *count, unsigned long long *first, int reset);
void register_check_reader(CheckReader r);
} // namespace cbkcuda

namespace {
int cbk_check_read_unit(unsigned long long *count, unsigned long long *first, int reset)
{
    cbkdev::CheckWord w{0, 0};
    cudaError_t e = cudaMemcpyFromSymbol(&w, cbkdev::g_check, sizeof w);
    if (e == cudaSuccess && reset) {
        const cbkdev::CheckWord z{0, 0};
        e = cudaMemcpyToSymbol(cbkdev::g_check, &z, sizeof z);
    }
    *count = w.count;
    *first = w.first;
    return (int)e;
}
const bool cbk_check_registered = (cbkcuda::register_check_reader(&cbk_check_read_unit), true);
} // namespace

namespace cbkdev {
#endif

// A strided view of one lane's matrix: element (i,j) at p[i*si + j*sj], the
// strides in scalars (the compact pack stride times V); in the checked build
// also the logical extent rows x cols.
template <typename T> struct LV {
    T *p;
    long si, sj;
#ifdef CBK_CUDA_CHECKED
    int rows, cols;
#endif
    __host__ __device__ __forceinline__ T &operator()(int i, int j) const
    {
#ifdef CBK_CUDA_CHECKED
        if ((unsigned)i >= (unsigned)rows || (unsigned)j >= (unsigned)cols)
            return check_fail<T>(i, j);
#endif
        return p[(long)i * si + (long)j * sj];
    }
    __host__ __device__ __forceinline__ LV t() const
    {
#ifdef CBK_CUDA_CHECKED
        return {p, sj, si, cols, rows};
#else
        return {p, sj, si};
#endif
    }
};

// The same view from column `first` on (columns first .. cols-1 become 0 ..)
template <typename T> __host__ __device__ __forceinline__ LV<T> lv_from_col(LV<T> v, int first)
{
    v.p += (long)first * v.sj;
#ifdef CBK_CUDA_CHECKED
    v.cols -= first;
#endif
    return v;
}

// The view of a lane's rows x cols matrix stored with leading dimension ld
// (column-major, or row-major when row), V lanes interleaved.
template <typename T>
__host__ __device__ __forceinline__ LV<T> lv_make(T *p, bool row, int ld, int V, int rows, int cols)
{
#ifdef CBK_CUDA_CHECKED
    return row ? LV<T>{p, (long)ld * V, (long)V, rows, cols}
               : LV<T>{p, (long)V, (long)ld * V, rows, cols};
#else
    (void)rows;
    (void)cols;
    return row ? LV<T>{p, (long)ld * V, (long)V} : LV<T>{p, (long)V, (long)ld * V};
#endif
}

// Scalars per group of V interleaved rows x cols matrices.
__host__ __device__ __forceinline__ size_t gstride(bool row, int ld, int rows, int cols, int V)
{
    return (size_t)ld * (size_t)(row ? rows : cols) * (size_t)V;
}

// The lane this thread runs: returns false past the last padded lane.
struct Lane {
    long g;
    int v;
};
__device__ __forceinline__ bool lane_of(long ngroups, int V, Lane &ln)
{
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ngroups * (long)V) return false;
    ln.g = idx / V;
    ln.v = (int)(idx - ln.g * V);
    return true;
}

template <typename T> __device__ __forceinline__ T rcp(T x) { return T(1) / x; }

template <typename T> __host__ __device__ constexpr T FLT_OR_DBL_MAX()
{
    return sizeof(T) == 8 ? T(1.7976931348623157e308) : T(3.40282347e38f);
}

// ---------------------------------------------------------------------
// FP64 <-> FP32 on the integer pipe. On a GB300 a hardware conversion (and an
// FP64 compare) takes a slot of the FP64 pipe -- the pipe the mixed-precision
// solves are bound by -- so the refined kernels convert with bit operations.
// ---------------------------------------------------------------------

// FP64 -> FP32 toward zero on the integer pipe, times 2^shift (subnormal
// results flushed, values beyond the FP32 range become infinities).
__device__ __forceinline__ float d2f_rz(double a, int shift = 0)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const int fe = e - 1023 + 127 + shift;
    unsigned bits;
    if (e == 0x7ff)
        bits = sign | 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u | mant : 0u);
    else if (e == 0 || fe <= 0)
        bits = sign;
    else if (fe >= 255)
        bits = sign | 0x7f800000u;
    else
        bits = sign | ((unsigned)fe << 23) | mant;
    return __uint_as_float(bits);
}

// The same for |a| < 2^128 (callers check the range apart): no branches.
// Zeros, FP64 subnormals and results below the FP32 normal range give a
// signed zero; a NaN gives some float (its residual stays NaN).
__device__ __forceinline__ float d2f_rz_inrange(double a)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const int fe = (int)((hi >> 20) & 0x7ffu) - 896;
    const unsigned bits =
        (hi & 0x80000000u) | ((unsigned)fe << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    return __uint_as_float(fe > 0 ? bits : hi & 0x80000000u);
}

// FP32 -> FP64 times 2^shift on the integer pipe (exact; FP32 subnormals
// flushed to zero)
__device__ __forceinline__ double f2d_int(float f, int shift = 0)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u;
    const int e = (int)((u >> 23) & 0xffu);
    const unsigned mant = u & 0x7fffffu;
    unsigned hi;
    if (e == 0)
        return __hiloint2double((int)sign, 0);
    if (e == 0xff)
        hi = sign | 0x7ff00000u | (mant >> 3) | (mant ? 0x80000u : 0u);
    else
        hi = sign | ((unsigned)(e - 127 + 1023 + shift) << 20) | (mant >> 3);
    return __hiloint2double((int)hi, (int)(mant << 29));
}

// a 2^sh = hi + lo + d on the integer pipe: hi = a 2^sh toward zero to 24
// significant bits, lo = the next 23 bits toward zero (exact: a 23-bit integer
// times a power of two), |d| < 2^-47 |a 2^sh|; the power of two only moves the
// exponent. For |a 2^sh| < 2^128 (callers screen the range); hi = lo = 0 below
// the FP32 normal range.
__device__ __forceinline__ void split2_rz(double a, float &hi, float &lo, int sh = 0)
{
    const unsigned h = (unsigned)__double2hiint(a), l = (unsigned)__double2loint(a);
    const unsigned sign = h & 0x80000000u;
    const int e = (int)((h >> 20) & 0x7ffu);
    const int fe = e - 896 + sh;
    const unsigned hb = sign | ((unsigned)fe << 23) | ((h & 0xfffffu) << 3) | (l >> 29);
    hi = __uint_as_float(fe > 0 ? hb : sign);
    // bits 28..6 of l as an integer: exact in FP32 through the 2^23 offset
    const float m = __uint_as_float(0x4b000000u | ((l >> 6) & 0x7fffffu)) - 8388608.0f;
    // their weight 2^(e - 1069 + sh): FP32 exponent field e - 942 + sh (zero
    // below range)
    const int se = e - 942 + sh;
    lo = m * __uint_as_float(sign | ((unsigned)(se > 0 ? se : 0) << 23));
}

// The same for any a: beyond the FP32 range hi is an infinity (a NaN stays a
// NaN) and lo is 0.
__device__ __forceinline__ void split2_rz_any(double a, float &hi, float &lo, int sh = 0)
{
    const int e = (int)(((unsigned)__double2hiint(a) >> 20) & 0x7ffu);
    if (e + sh >= 1151) {
        hi = d2f_rz(a, sh);
        lo = 0.f;
        return;
    }
    split2_rz(a, hi, lo, sh);
}

// (s, c) := (s, c) + (s2, c2), both double-FP32 values (TwoSum on the leading
// parts, the rest into c)
__device__ __forceinline__ void dd_add(float &s, float &c, float s2, float c2)
{
    const float t = s + s2;
    const float bb = t - s;
    const float err = (s - (t - bb)) + (s2 - bb);
    s = t;
    c = (c + c2) + err;
}

// (s, c) := (s, c) - a x in double-FP32 arithmetic, a = ah + al, x exact:
// TwoProduct by the FMA and TwoSum (Knuth), the errors gathered in c --
// Ogita, Rump & Oishi, "Accurate sum and dot product" (2005), Dot2. Needs
// floating-point contraction off (each rounding is the algorithm's).
__device__ __forceinline__ void dot2_sub(float &s, float &c, float ah, float al, float x)
{
    const float p = ah * x;
    const float e = fmaf(al, x, fmaf(ah, x, -p)); // ah x - p exactly, plus al x
    const float t = s - p;
    const float bb = t - s;
    const float err = (s - (t - bb)) + (-p - bb); // s - p - t exactly
    s = t;
    c = c + (err - e);
}

// |a| > FLT_MAX, infinities included and NaN not (LAPACK dlag2s's test), on
// the 32-bit halves of a
__device__ __forceinline__ bool beyond_fp32(double a)
{
    const unsigned ah = (unsigned)__double2hiint(a) & 0x7fffffffu, lo = (unsigned)__double2loint(a);
    const bool big = ah > 0x47efffffu || (ah == 0x47efffffu && lo > 0xe0000000u);
    const bool nan = ah > 0x7ff00000u || (ah == 0x7ff00000u && lo != 0u);
    return big && !nan;
}

// 8-byte asynchronous copy global -> shared (cp.async, cached in L1 and L2)
__device__ __forceinline__ void cp_async8(double *dst, const double *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

// wait for every cp.async this thread issued
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// max(a, b) that keeps a NaN (fmaxf drops it): a NaN residual norm must stop
// a refinement rather than pass its convergence test
__device__ __forceinline__ float fmax_nan(float a, float b)
{
    return (a > b || a != a) ? a : b;
}

// ---------------------------------------------------------------------
// Cholesky / LDL^T of the lower triangle of a lane view
// ---------------------------------------------------------------------
// Every loop that issues FP64 arithmetic has compile-time bounds or exact
// runtime bounds: a predicated-off FMA still occupies the (slow) FP64 pipe,
// so no tile is padded.

// The update of the NC panel columns j0 .. j0+NC-1 by the finished columns
// k < j0, accumulated in pivot order (the reference's syrk tile,
// src/cbk_sytrfnp_compact.hpp:132-173): acc -= L(i,k) * L(c,k) (Cholesky) or
// acc -= (L(i,k) D(k)) * L(c,k) (LDL^T). The diagonal block is one
// lower-triangular register tile; the rows below go four at a time.
template <typename T, bool LDLT, int NC>
__device__ void cross_panel_update_nc(int n, LV<T> A, int j0)
{
    {   // diagonal block: rows and columns j0 .. j0+NC-1, c <= r
        T acc[NC][NC];
#pragma unroll
        for (int r = 0; r < NC; ++r)
#pragma unroll
            for (int c = 0; c <= r; ++c)
                acc[r][c] = A(j0 + r, j0 + c);
        for (int k = 0; k < j0; ++k) {
            T l[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c)
                l[c] = A(j0 + c, k);
            const T dk = LDLT ? A(k, k) : T(1);
#pragma unroll
            for (int r = 0; r < NC; ++r) {
                const T li = LDLT ? l[r] * dk : l[r];
#pragma unroll
                for (int c = 0; c <= r; ++c)
                    acc[r][c] = fma(-li, l[c], acc[r][c]);
            }
        }
#pragma unroll
        for (int r = 0; r < NC; ++r)
#pragma unroll
            for (int c = 0; c <= r; ++c)
                A(j0 + r, j0 + c) = acc[r][c];
    }
    int i0 = j0 + NC;
    for (; i0 + 4 <= n; i0 += 4) {
        T acc[4][NC];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < NC; ++c)
                acc[r][c] = A(i0 + r, j0 + c);
        for (int k = 0; k < j0; ++k) {
            T lc[NC], li[4];
#pragma unroll
            for (int c = 0; c < NC; ++c)
                lc[c] = A(j0 + c, k);
            const T dk = LDLT ? A(k, k) : T(1);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const T l = A(i0 + r, k);
                li[r] = LDLT ? l * dk : l;
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    acc[r][c] = fma(-li[r], lc[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < NC; ++c)
                A(i0 + r, j0 + c) = acc[r][c];
    }
    for (; i0 < n; ++i0) {
        T acc[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c)
            acc[c] = A(i0, j0 + c);
        for (int k = 0; k < j0; ++k) {
            const T l = A(i0, k);
            const T li = LDLT ? l * A(k, k) : l;
#pragma unroll
            for (int c = 0; c < NC; ++c)
                acc[c] = fma(-li, A(j0 + c, k), acc[c]);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c)
            A(i0, j0 + c) = acc[c];
    }
}

template <typename T, bool LDLT>
__device__ void cross_panel_update(int n, LV<T> A, int j0, int j1)
{
    switch (j1 - j0) {
    case 8: cross_panel_update_nc<T, LDLT, 8>(n, A, j0); break;
    case 7: cross_panel_update_nc<T, LDLT, 7>(n, A, j0); break;
    case 6: cross_panel_update_nc<T, LDLT, 6>(n, A, j0); break;
    case 5: cross_panel_update_nc<T, LDLT, 5>(n, A, j0); break;
    case 4: cross_panel_update_nc<T, LDLT, 4>(n, A, j0); break;
    case 3: cross_panel_update_nc<T, LDLT, 3>(n, A, j0); break;
    case 2: cross_panel_update_nc<T, LDLT, 2>(n, A, j0); break;
    default: cross_panel_update_nc<T, LDLT, 1>(n, A, j0); break;
    }
}

// The unblocked sweep of the NC panel columns j0 .. j0+NC-1 (already updated
// by the columns left of them), per pivot j: the weight 1/a, the rank-1 step
// on the unscaled column A(i,q) -= A(i,j) * (A(q,j) / a) for the panel columns
// q > j, then the sqrt and the column scaling off the pivot-to-pivot chain
// (src/cbk_potrf_compact.hpp:79-105; src/cbk_sytrfnp_compact.hpp:96-112,
// 216-235). The NC x NC diagonal block is swept in place first, leaving the
// weights w(j, q) = A(q,j) / a_j and the column scales in registers; every
// row below it is then carried through all NC pivots in registers, with the
// same operations in the same order, so each of its elements is read and
// written once instead of once per pivot (a lane's matrix does not fit in L1
// from order 32 on: those passes went to L2 or DRAM, and took a quarter of
// the time of posv at n = 16 .. 48).
template <typename T, bool LDLT, int NC>
__device__ void panel_sweep_nc(int n, LV<T> A, int j0)
{
    constexpr int NW = NC * (NC - 1) / 2 > 0 ? NC * (NC - 1) / 2 : 1;
    T w[NW];   // w(j, q) at j (2 NC - j - 1) / 2 + (q - j - 1), q > j
    T scl[NC]; // the column scales
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const T a = A(j0 + j, j0 + j);
        const bool pos = !LDLT && a > T(0) && a <= FLT_OR_DBL_MAX<T>();
        T inva, rs = T(0);
        if (pos) {
            rs = rsqrt(a);
            inva = rs * rs;
        }
        else {
            inva = rcp(a);
        }
#pragma unroll
        for (int q = j + 1; q < NC; ++q)
            w[j * (2 * NC - j - 1) / 2 + (q - j - 1)] = A(j0 + q, j0 + j) * inva;
#pragma unroll
        for (int r = j + 1; r < NC; ++r) {
            const T aij = A(j0 + r, j0 + j);
#pragma unroll
            for (int q = j + 1; q <= r; ++q)
                A(j0 + r, j0 + q) =
                    fma(-aij, w[j * (2 * NC - j - 1) / 2 + (q - j - 1)], A(j0 + r, j0 + q));
        }
        T scale;
        if (LDLT) {
            scale = inva;
        }
        else if (pos) {
            A(j0 + j, j0 + j) = a * rs;
            scale = rs;
        }
        else {
            const T s = sqrt(a);
            A(j0 + j, j0 + j) = s;
            scale = s * inva;
        }
        scl[j] = scale;
#pragma unroll
        for (int r = j + 1; r < NC; ++r)
            A(j0 + r, j0 + j) = A(j0 + r, j0 + j) * scale;
    }
    // the rows below the block, one at a time
    for (int i = j0 + NC; i < n; ++i) {
        T x[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c)
            x[c] = A(i, j0 + c);
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const T aij = x[j];
#pragma unroll
            for (int q = j + 1; q < NC; ++q)
                x[q] = fma(-aij, w[j * (2 * NC - j - 1) / 2 + (q - j - 1)], x[q]);
            x[j] = x[j] * scl[j];
        }
#pragma unroll
        for (int c = 0; c < NC; ++c)
            A(i, j0 + c) = x[c];
    }
}

template <typename T, bool LDLT> __device__ void panel_sweep(int n, LV<T> A, int j0, int j1)
{
    switch (j1 - j0) {
    case 8: panel_sweep_nc<T, LDLT, 8>(n, A, j0); break;
    case 7: panel_sweep_nc<T, LDLT, 7>(n, A, j0); break;
    case 6: panel_sweep_nc<T, LDLT, 6>(n, A, j0); break;
    case 5: panel_sweep_nc<T, LDLT, 5>(n, A, j0); break;
    case 4: panel_sweep_nc<T, LDLT, 4>(n, A, j0); break;
    case 3: panel_sweep_nc<T, LDLT, 3>(n, A, j0); break;
    case 2: panel_sweep_nc<T, LDLT, 2>(n, A, j0); break;
    default: panel_sweep_nc<T, LDLT, 1>(n, A, j0); break;
    }
}

// The in-panel rank-1 step of pivot j on the NQ panel columns to its right,
// on the unscaled column with the weight 1/a (sytrfnp_update_block,
// src/cbk_sytrfnp_compact.hpp:96-112): A(i,c) -= A(i,j) * (A(c,j) / a),
// the triangular corner first, then every row below the panel.
template <typename T, int NQ> __device__ void rank1_panel(int n, LV<T> A, int j, T inva)
{
    T w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
        w[q] = A(j + 1 + q, j) * inva;
#pragma unroll
    for (int r = 0; r < NQ; ++r) {
        const int i = j + 1 + r;
        const T aij = A(i, j);
#pragma unroll
        for (int q = 0; q <= r; ++q)
            A(i, j + 1 + q) = fma(-aij, w[q], A(i, j + 1 + q));
    }
    for (int i = j + 1 + NQ; i < n; ++i) {
        const T aij = A(i, j);
#pragma unroll
        for (int q = 0; q < NQ; ++q)
            A(i, j + 1 + q) = fma(-aij, w[q], A(i, j + 1 + q));
    }
}

// panel_sweep's operations in the same order, each pivot's step applied to
// the panel in memory: slower from order 16 on, but it keeps no weights in
// registers, for a caller whose registers are spoken for (the FP64 fallback
// inlined in the refined warp kernel).
template <typename T, bool LDLT> __device__ void panel_sweep_mem(int n, LV<T> A, int j0, int j1)
{
    for (int j = j0; j < j1; ++j) {
        const T a = A(j, j);
        T inva;
        if (!LDLT && a > T(0) && a <= FLT_OR_DBL_MAX<T>()) {
            const T r = rsqrt(a);
            inva = r * r;
        }
        else {
            inva = rcp(a);
        }
        switch (j1 - j - 1) {
        case 7: rank1_panel<T, 7>(n, A, j, inva); break;
        case 6: rank1_panel<T, 6>(n, A, j, inva); break;
        case 5: rank1_panel<T, 5>(n, A, j, inva); break;
        case 4: rank1_panel<T, 4>(n, A, j, inva); break;
        case 3: rank1_panel<T, 3>(n, A, j, inva); break;
        case 2: rank1_panel<T, 2>(n, A, j, inva); break;
        case 1: rank1_panel<T, 1>(n, A, j, inva); break;
        default: break;
        }
        T scale;
        if (LDLT) {
            scale = inva; // D(j) = a stays on the diagonal
        }
        else if (a > T(0) && a <= FLT_OR_DBL_MAX<T>()) {
            // r = 1/sqrt(a): then 1/a = r^2, sqrt(a) = a r and the column
            // scale sqrt(a)/a = r -- one reciprocal square root where the
            // reciprocal and the square root each take several FP64-pipe
            // passes (a few ulps apart from the separate operations)
            const T r = rsqrt(a);
            A(j, j) = a * r;
            scale = r;
        }
        else { // zero, negative, infinite or NaN pivot: the plain operations
            const T d = sqrt(a);
            A(j, j) = d;
            scale = d * inva;
        }
        for (int i = j + 1; i < n; ++i)
            A(i, j) = A(i, j) * scale;
    }
}

// MEM: the panel sweep in memory (panel_sweep_mem; the same bits)
template <typename T, bool LDLT, bool MEM = false> __device__ void factor_lane(int n, LV<T> A)
{
    for (int j0 = 0; j0 < n; j0 += 8) {
        const int j1 = min(j0 + 8, n);
        if (j0 > 0) cross_panel_update<T, LDLT>(n, A, j0, j1);
        if (MEM)
            panel_sweep_mem<T, LDLT>(n, A, j0, j1);
        else
            panel_sweep<T, LDLT>(n, A, j0, j1);
    }
}

// ---------------------------------------------------------------------
// Solves from a factor held in the lower triangle of the view L
// ---------------------------------------------------------------------

// L z = B (forward) then L^T X = z (backward) on NB right-hand sides at once,
// so every factor load feeds NB FMAs. UNIT: the diagonal holds D (LDL^T): the
// sweeps use a unit diagonal and the D^-1 row scaling between them is folded
// into the backward sweep's first touch of each row
// (src/cbk_sytrsnp_compact.hpp:51-78); otherwise each row is scaled by
// 1/L(i,i) (src/cbk_potrs_compact.hpp:46-58).
// 1/L(i,i) of the first RINV rows is computed once per lane (sym_solve_lane)
// and shared by both sweeps and every block of right-hand sides; rows past it
// recompute it.
constexpr int RINV = 64;

template <typename T, bool UNIT, int NB>
__device__ void sym_solve_block(int n, LV<T> L, LV<T> B, int c0, const T *rinv)
{
    for (int i = 0; i < n; ++i) {
        T w[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c)
            w[c] = B(i, c0 + c);
        for (int l = 0; l < i; ++l) {
            const T a = L(i, l);
#pragma unroll
            for (int c = 0; c < NB; ++c)
                w[c] = fma(-a, B(l, c0 + c), w[c]);
        }
        if (UNIT) {
#pragma unroll
            for (int c = 0; c < NB; ++c)
                B(i, c0 + c) = w[c];
        }
        else {
            const T r = i < RINV ? rinv[i] : rcp(L(i, i));
#pragma unroll
            for (int c = 0; c < NB; ++c)
                B(i, c0 + c) = w[c] * r;
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        T w[NB];
        const T r = i < RINV ? rinv[i] : rcp(L(i, i));
#pragma unroll
        for (int c = 0; c < NB; ++c)
            w[c] = UNIT ? B(i, c0 + c) * r : B(i, c0 + c);
        for (int l = i + 1; l < n; ++l) {
            const T a = L(l, i);
#pragma unroll
            for (int c = 0; c < NB; ++c)
                w[c] = fma(-a, B(l, c0 + c), w[c]);
        }
#pragma unroll
        for (int c = 0; c < NB; ++c)
            B(i, c0 + c) = UNIT ? w[c] : w[c] * r;
    }
}

template <typename T, bool UNIT> __device__ void sym_solve_lane(int n, int nrhs, LV<T> L, LV<T> B)
{
    T rinv[RINV];
    const int nr = n < RINV ? n : RINV;
    for (int i = 0; i < nr; ++i)
        rinv[i] = rcp(L(i, i));
    int c0 = 0;
    for (; c0 + 4 <= nrhs; c0 += 4)
        sym_solve_block<T, UNIT, 4>(n, L, B, c0, rinv);
    if (nrhs - c0 >= 2) {
        sym_solve_block<T, UNIT, 2>(n, L, B, c0, rinv);
        c0 += 2;
    }
    if (nrhs - c0 >= 1) sym_solve_block<T, UNIT, 1>(n, L, B, c0, rinv);
}

// ---------------------------------------------------------------------
// Triangular solve, any side / uplo / trans / diag, through views
// (src/cbk_trsm_compact.hpp:73-228)
// ---------------------------------------------------------------------

// op(A) X = alpha B for the NB columns c0 .. c0+NB-1 of B, row by row
// (the reference's row-dot form, src/cbk_trsm_compact.hpp:73-104).
template <typename T, int NB>
__device__ void trsm_left_block(bool back, bool tran, bool unit, int m, T alpha, LV<T> A, LV<T> B,
                                int c0)
{
    for (int t = 0; t < m; ++t) {
        const int i = back ? m - 1 - t : t;
        T w[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c)
            w[c] = B(i, c0 + c) * alpha;
        const int lo = back ? i + 1 : 0, hi = back ? m : i;
        for (int l = lo; l < hi; ++l) {
            const T a = tran ? A(l, i) : A(i, l);
#pragma unroll
            for (int c = 0; c < NB; ++c)
                w[c] = fma(-a, B(l, c0 + c), w[c]);
        }
        if (unit) {
#pragma unroll
            for (int c = 0; c < NB; ++c)
                B(i, c0 + c) = w[c];
        }
        else {
            const T r = rcp(A(i, i));
#pragma unroll
            for (int c = 0; c < NB; ++c)
                B(i, c0 + c) = w[c] * r;
        }
    }
}

template <typename T>
__device__ void trsm_left(bool upper, bool tran, bool unit, int m, int n, T alpha, LV<T> A, LV<T> B)
{
    const bool back = (upper != tran);
    int c0 = 0;
    for (; c0 + 4 <= n; c0 += 4)
        trsm_left_block<T, 4>(back, tran, unit, m, alpha, A, B, c0);
    if (n - c0 >= 2) {
        trsm_left_block<T, 2>(back, tran, unit, m, alpha, A, B, c0);
        c0 += 2;
    }
    if (n - c0 >= 1) trsm_left_block<T, 1>(back, tran, unit, m, alpha, A, B, c0);
}

template <typename T>
__device__ void trsm_lane(bool left, bool upper, bool tran, bool unit, int m, int n, T alpha,
                          LV<T> A, LV<T> B)
{
    if (left) {
        trsm_left<T>(upper, tran, unit, m, n, alpha, A, B);
    }
    else {
        // X op(A) = alpha B is op(A)^T X^T = alpha B^T: the left solve on B's
        // transposed view (the view only swaps its strides) with the
        // transpose flag flipped. Its row-dot blocks keep four right-hand
        // sides in registers, where the reference's side-R form
        // (src/cbk_trsm_compact.hpp:206-227) sweeps one column of B through
        // memory per step: measured 1.5x faster at 16 x 16.
        trsm_left<T>(upper, !tran, unit, n, m, alpha, A, B.t());
    }
}

template <typename T> __device__ void zero_lane(LV<T> B, int i0, int i1, int ncols)
{
    for (int j = 0; j < ncols; ++j)
        for (int i = i0; i < i1; ++i)
            B(i, j) = T(0);
}

// ---------------------------------------------------------------------
// Householder QR family (src/cbk_geqrf_compact.hpp:74-131,
// src/cbk_ormqr_compact.hpp:68-124, src/cbk_orgqr_compact.hpp:50-87)
// ---------------------------------------------------------------------

// H(kk) = I - t v v^T applied to the NB slices c0 .. c0+NB-1 of C,
// v = (1, A(kk+1:len, kk)): w = v^T c, w *= t, c -= v w
// (larf_block, src/cbk_ormqr_compact.hpp:68-91).
template <typename T, int NB>
__device__ void larf_block(int kk, int len, LV<T> A, T t, LV<T> C, int c0)
{
    T w[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c)
        w[c] = C(kk, c0 + c);
    for (int i = kk + 1; i < len; ++i) {
        const T a = A(i, kk);
#pragma unroll
        for (int c = 0; c < NB; ++c)
            w[c] = fma(a, C(i, c0 + c), w[c]);
    }
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        w[c] *= t;
        C(kk, c0 + c) -= w[c];
    }
    for (int i = kk + 1; i < len; ++i) {
        const T a = A(i, kk);
#pragma unroll
        for (int c = 0; c < NB; ++c)
            C(i, c0 + c) = fma(-a, w[c], C(i, c0 + c));
    }
}

template <typename T>
__device__ void larf_lane(int kk, int len, LV<T> A, T t, LV<T> C, int p0, int p1)
{
    int c0 = p0;
    for (; c0 + 4 <= p1; c0 += 4)
        larf_block<T, 4>(kk, len, A, t, C, c0);
    if (p1 - c0 >= 2) {
        larf_block<T, 2>(kk, len, A, t, C, c0);
        c0 += 2;
    }
    if (p1 - c0 >= 1) larf_block<T, 1>(kk, len, A, t, C, c0);
}

// ---------------------------------------------------------------------
// Compact WY: JB consecutive reflectors j0 .. j0+JB-1 applied in one pass
// ---------------------------------------------------------------------
// H(j0) ... H(j0+JB-1) = I - Y Tm Y^T with Y the reflectors' unit lower
// trapezoid (rows j0 .. len-1; Y(j0+q, q) = 1, above it 0, below it the
// stored A(i, j0+q)) and Tm upper triangular (LAPACK's larft, forward,
// column-wise; Schreiber & Van Loan 1989). Applying the block reads each
// trailing column and each reflector row once for JB reflectors, where one
// reflector at a time reads them JB times: a lane-per-matrix QR streams its
// matrix through the cache, and this cuts its loads per multiply-add from
// about 1.25 to 0.5 (4 reflectors, 4 columns at a time). The products are
// the same; only the rounding order differs from the one-at-a-time sweep.

// Y(i, q) of the block at j0 (0 above its diagonal, 1 on it)
template <typename T> __device__ __forceinline__ T wy_y(LV<T> A, int j0, int i, int q)
{
    return i > j0 + q ? A(i, j0 + q) : (i == j0 + q ? T(1) : T(0));
}

template <typename T, int JB>
__device__ void wy_form_t(int j0, int len, LV<T> A, const T *tau, int V, T (&Tm)[JB][JB])
{
#pragma unroll
    for (int j = 0; j < JB; ++j) {
        const T tj = tau[(long)(j0 + j) * V];
        // z = Y(:, 0:j)^T y_j over rows j0+j .. len-1
        T z[JB];
#pragma unroll
        for (int q = 0; q < JB; ++q)
            z[q] = T(0);
#pragma unroll
        for (int q = 0; q < j; ++q)
            z[q] = A(j0 + j, j0 + q); // y_j's unit entry at row j0 + j
        for (int i = j0 + j + 1; i < len; ++i) {
            const T yij = A(i, j0 + j);
#pragma unroll
            for (int q = 0; q < j; ++q)
                z[q] = fma(A(i, j0 + q), yij, z[q]);
        }
        // Tm(0:j, j) = -tj Tm(0:j, 0:j) z, Tm(j, j) = tj
#pragma unroll
        for (int r = 0; r < JB; ++r) {
            if (r < j) {
                T acc = T(0);
#pragma unroll
                for (int q = r; q < j; ++q)
                    acc = fma(Tm[r][q], z[q], acc);
                Tm[r][j] = -tj * acc;
            }
            else if (r == j) {
                Tm[r][j] = tj;
            }
            else {
                Tm[r][j] = T(0);
            }
        }
    }
}

// C(:, c0 .. c0+NC-1) := (I - Y op(Tm) Y^T) C over rows j0 .. len-1, with
// op(Tm) = Tm^T when trans (the block of H(j0+JB-1) ... H(j0), Q^T's order)
template <typename T, int JB, int NC>
__device__ void wy_apply_cols(int j0, int len, LV<T> A, const T (&Tm)[JB][JB], bool trans,
                              LV<T> C, int c0)
{
    T w[JB][NC];
#pragma unroll
    for (int q = 0; q < JB; ++q)
#pragma unroll
        for (int c = 0; c < NC; ++c)
            w[q][c] = T(0);
    // W = Y^T C
#pragma unroll
    for (int r = 0; r < JB; ++r) { // the unit-triangular top rows
        const int i = j0 + r;
        T ci[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c)
            ci[c] = C(i, c0 + c);
#pragma unroll
        for (int q = 0; q <= r; ++q) {
            const T y = q == r ? T(1) : A(i, j0 + q);
#pragma unroll
            for (int c = 0; c < NC; ++c)
                w[q][c] = fma(y, ci[c], w[q][c]);
        }
    }
    for (int i = j0 + JB; i < len; ++i) {
        T y[JB], ci[NC];
#pragma unroll
        for (int q = 0; q < JB; ++q)
            y[q] = A(i, j0 + q);
#pragma unroll
        for (int c = 0; c < NC; ++c)
            ci[c] = C(i, c0 + c);
#pragma unroll
        for (int q = 0; q < JB; ++q)
#pragma unroll
            for (int c = 0; c < NC; ++c)
                w[q][c] = fma(y[q], ci[c], w[q][c]);
    }
    // W := op(Tm) W (upper triangular Tm; Tm^T lower)
    T u[JB][NC];
#pragma unroll
    for (int r = 0; r < JB; ++r)
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T acc = T(0);
#pragma unroll
            for (int q = 0; q < JB; ++q) {
                const T t = trans ? Tm[q][r] : Tm[r][q];
                if (trans ? q <= r : q >= r) acc = fma(t, w[q][c], acc);
            }
            u[r][c] = acc;
        }
    // C -= Y W
#pragma unroll
    for (int r = 0; r < JB; ++r) {
        const int i = j0 + r;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T acc = C(i, c0 + c);
#pragma unroll
            for (int q = 0; q <= r; ++q) {
                const T y = q == r ? T(1) : A(i, j0 + q);
                acc = fma(-y, u[q][c], acc);
            }
            C(i, c0 + c) = acc;
        }
    }
    for (int i = j0 + JB; i < len; ++i) {
        T y[JB];
#pragma unroll
        for (int q = 0; q < JB; ++q)
            y[q] = A(i, j0 + q);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T acc = C(i, c0 + c);
#pragma unroll
            for (int q = 0; q < JB; ++q)
                acc = fma(-y[q], u[q][c], acc);
            C(i, c0 + c) = acc;
        }
    }
}

template <typename T, int JB>
__device__ void wy_apply(int j0, int len, LV<T> A, const T (&Tm)[JB][JB], bool trans, LV<T> C,
                         int p0, int p1)
{
    int c0 = p0;
    for (; c0 + 4 <= p1; c0 += 4)
        wy_apply_cols<T, JB, 4>(j0, len, A, Tm, trans, C, c0);
    if (p1 - c0 >= 2) {
        wy_apply_cols<T, JB, 2>(j0, len, A, Tm, trans, C, c0);
        c0 += 2;
    }
    if (p1 - c0 >= 1) wy_apply_cols<T, JB, 1>(j0, len, A, Tm, trans, C, c0);
}

constexpr int WY_NB = 4;   // reflectors per block
constexpr int WY_MMIN = 32; // blocked from this many rows on: below it the block's
                            // T and extra passes cost more than the loads they save
                            // (16 x 8 least squares 12 % slower blocked, 64 x 16 26 % faster)

// geqr2 on the lane view: per column the tail sum of squares, the branch-free
// larfg (no reflector when the tail is exactly zero), the body scaled by
// 1/(x0 - beta), then H applied to the trailing columns. From WY_MMIN rows on,
// within a panel of WY_NB columns one reflector at a time and to the columns
// right of the panel as one compact-WY block; below, one at a time
// throughout. tau has stride V.
template <typename T, bool WY = true>
__device__ void geqrf_lane(int m, int n, LV<T> A, T *tau, int V)
{
    const int k = min(m, n);
    const bool blocked = WY && m >= WY_MMIN;
    const int nb = blocked ? WY_NB : k; // one panel: the one-at-a-time sweep
    for (int j0 = 0; j0 < k; j0 += nb) {
        const int j1 = min(j0 + nb, k);
        for (int kk = j0; kk < j1; ++kk) {
            T tail = T(0);
            for (int i = kk + 1; i < m; ++i) {
                const T a = A(i, kk);
                tail = fma(a, a, tail);
            }
            const T x0 = A(kk, kk);
            const T norm = sqrt(fma(x0, x0, tail));
            const T beta = (x0 >= T(0)) ? -norm : norm;
            const bool has = tail > T(0);
            const T t = has ? (beta - x0) / beta : T(0);
            const T inv = has ? rcp(x0 - beta) : T(0);
            tau[(long)kk * V] = t;
            for (int i = kk + 1; i < m; ++i)
                A(i, kk) = A(i, kk) * inv;
            A(kk, kk) = has ? beta : x0;
            larf_lane<T>(kk, m, A, t, A, kk + 1, blocked && j1 == j0 + WY_NB ? j1 : n);
        }
        if (WY && blocked && j1 == j0 + WY_NB && j1 < n) {
            T Tm[WY_NB][WY_NB];
            wy_form_t<T, WY_NB>(j0, m, A, tau, V, Tm);
            wy_apply<T, WY_NB>(j0, m, A, Tm, true, A, j1, n);
        }
    }
}

// Q^T C (forward) or Q C (backward) with Q = H(0) ... H(k-1) of the QR in A:
// from WY_MMIN rows on whole blocks of WY_NB reflectors in compact WY, the
// rest one at a time
template <typename T, bool WY = true>
__device__ void ormqr_lane(bool forward, int len, int npanel, int k, LV<T> A, const T *tau, int V,
                           LV<T> C)
{
    const int kb = WY && len >= WY_MMIN ? k / WY_NB * WY_NB : 0; // reflectors in whole blocks
    if (forward) {
        for (int j0 = 0; j0 < kb; j0 += WY_NB) {
            T Tm[WY_NB][WY_NB];
            wy_form_t<T, WY_NB>(j0, len, A, tau, V, Tm);
            wy_apply<T, WY_NB>(j0, len, A, Tm, true, C, 0, npanel);
        }
        for (int kk = kb; kk < k; ++kk)
            larf_lane<T>(kk, len, A, tau[(long)kk * V], C, 0, npanel);
    }
    else {
        for (int kk = k - 1; kk >= kb; --kk)
            larf_lane<T>(kk, len, A, tau[(long)kk * V], C, 0, npanel);
        for (int j0 = kb - WY_NB; j0 >= 0; j0 -= WY_NB) {
            T Tm[WY_NB][WY_NB];
            wy_form_t<T, WY_NB>(j0, len, A, tau, V, Tm);
            wy_apply<T, WY_NB>(j0, len, A, Tm, false, C, 0, npanel);
        }
    }
}

template <typename T> __device__ void orgqr_lane(int m, int n, int k, LV<T> A, const T *tau, int V)
{
    for (int j = k; j < n; ++j) {
        for (int i = 0; i < m; ++i)
            A(i, j) = T(0);
        A(j, j) = T(1);
    }
    for (int kk = k - 1; kk >= 0; --kk) {
        const T t = tau[(long)kk * V];
        larf_lane<T>(kk, m, A, t, A, kk + 1, n);
        const T mt = -t;
        for (int i = kk + 1; i < m; ++i)
            A(i, kk) = A(i, kk) * mt;
        A(kk, kk) = T(1) - t;
        for (int i = 0; i < kk; ++i)
            A(i, kk) = T(0);
    }
}

// One lane of the least-squares solve (src/cbk_gels_compact.hpp:84-106): F is
// the tall (p x q) view of A, B its p x nrhs right-hand sides.
template <typename T, bool WY = true>
__device__ void gels_lane(bool overdet, int p, int q, int nrhs, LV<T> F, T *tau, int V, LV<T> B)
{
    geqrf_lane<T, WY>(p, q, F, tau, V);
    if (overdet) {
        ormqr_lane<T, WY>(true, p, nrhs, q, F, tau, V, B);
        trsm_lane<T>(true, true, false, false, q, nrhs, T(1), F, B);
    }
    else {
        trsm_lane<T>(true, true, true, false, q, nrhs, T(1), F, B);
        zero_lane<T>(B, q, p, nrhs);
        ormqr_lane<T, WY>(false, p, nrhs, q, F, tau, V, B);
    }
}

// The plain FP64 least squares of one lane, the fallback of the
// mixed-precision solves: QR of A in place (tau), then the right-hand sides
// first .. nrhs-1 of B solved through Q^T and R -- blocked exactly where the
// plain routine is (from WY_MMIN rows on), so a fallen-back lane holds the
// plain routine's results bit for bit.
__device__ __forceinline__ void gels_fallback_lane(int m, int n, int nrhs, int first, LV<double> A,
                                                   double *taup, int V, LV<double> B)
{
    geqrf_lane<double>(m, n, A, taup, V);
    if (first < nrhs) {
        const LV<double> Bs = lv_from_col(B, first);
        ormqr_lane<double>(true, m, nrhs - first, n, A, taup, V, Bs);
        trsm_lane<double>(true, true, false, false, n, nrhs - first, 1.0, A, Bs);
    }
}

} // namespace cbkdev
