// cbk_autotune.cu -- the autotuner: measured launch shapes and interleave
// widths per (routine, precision, order).
//
// No counterpart in the reference (one code path per V, chosen by the
// caller). cbk_cuda_autotune times a routine on a synthetic batch of nm
// matrices generated on the device -- uniform entries in [-1, 1), with the
// diagonal raised by n + 1 where the routine needs a positive-definite or
// well-conditioned triangular matrix (for the mixed-precision solve, SPD
// matrices of condition 1e1 .. 1e6: its time depends on the refinement
// steps), and the factors computed first where
// the routine consumes them (potrs, sytrsnp: the factor; ormqr, orgqr: the
// QR) -- for every candidate shape: threads per block 64 / 128 / 256 for the
// lane-per-matrix kernels (32 / 64 / 128 for the lane-per-matrix refined
// solves, which are compiled for at most 128), the two register caps of the warp-per-matrix
// refined solve (orders 17 .. 64), each at interleave widths 32, 64 and 128.
// Each candidate is timed with CUDA events, best of three runs, inputs
// restored from a pristine copy before each run. The winner goes into the
// tuning table that every later launch reads (threads / variant for the
// routine's order, and the width as advice for the caller's layout).
// Launch shapes never change results, so tuning is safe at any time.
#include "../../include/cbk_cuda.h"
#include "cbk_launch.h"

#include <algorithm>
#include <cfloat>
#include <cuda_runtime.h>

namespace cbkcuda {

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    // splitmix64's finaliser (Steele, Lea, Flood 2014)
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// a[i] = uniform [-1, 1) from (seed, i)
template <typename T> __global__ void k_fill_uniform(T *a, long count, unsigned long long seed)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count;
         i += (long)gridDim.x * blockDim.x)
        a[i] = (T)((double)(mix64(seed ^ (unsigned long long)i) >> 11) * 0x1p-52 - 1.0);
}

// A(i, i) += shift for every lane of a column-major compact batch (ld = n)
template <typename T> __global__ void k_shift_diag(T *a, int n, int V, long lanes, T shift)
{
    const long l = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (l >= lanes) return;
    const long g = l / V;
    const int v = (int)(l - g * V);
    T *p = a + g * (long)n * n * V + v;
    for (int i = 0; i < n; ++i)
        p[((long)i * n + i) * V] += shift;
}

// An SPD batch shaped like the mixed-precision solve's work: per lane
// A = H D H with H = I - 2 v v^T / v^T v (v uniform in [-1, 1)^n: a dense
// orthogonal H) and D = diag(kappa^-u_i), u_0 = 0 < u_i < u_{n-1} = 1,
// kappa = 10^(1..6) log-uniform per lane -- condition numbers that a diagonal
// scaling does not remove, so the refinement takes its usual 2 to 3 steps
// (a diagonally dominant batch converges in one and times the wrong kernel
// mix). Written column-major compact, ld = n.
template <typename T> __global__ void k_fill_spd_reflector(T *a, int n, int V, long lanes,
                                                           unsigned long long seed)
{
    const long l = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (l >= lanes) return;
    const long g = l / V;
    const int v0 = (int)(l - g * V);
    T *p = a + g * (long)n * n * V + v0;
    auto unif = [&](unsigned long long k) {
        return (double)(mix64(seed ^ ((unsigned long long)l << 20) ^ k) >> 11) * 0x1p-53;
    };
    const double lk = 1.0 + 5.0 * unif(0xFFFFF);
    double s = 0.0, w = 0.0;
    for (int i = 0; i < n; ++i) {
        const double vi = 2.0 * unif(2 * i) - 1.0;
        const double ui = n == 1 ? 0.0 : (i == 0 ? 0.0 : (i == n - 1 ? 1.0 : unif(2 * i + 1)));
        const double di = exp10(-lk * ui);
        s += vi * vi;
        w += di * vi * vi;
    }
    for (int j = 0; j < n; ++j) {
        const double vj = 2.0 * unif(2 * j) - 1.0;
        const double uj = n == 1 ? 0.0 : (j == 0 ? 0.0 : (j == n - 1 ? 1.0 : unif(2 * j + 1)));
        const double dj = exp10(-lk * uj);
        for (int i = 0; i < n; ++i) {
            const double vi = 2.0 * unif(2 * i) - 1.0;
            const double ui = n == 1 ? 0.0 : (i == 0 ? 0.0 : (i == n - 1 ? 1.0 : unif(2 * i + 1)));
            const double di = exp10(-lk * ui);
            const double aij = (i == j ? di : 0.0) - 2.0 * (di + dj) * vi * vj / s +
                               4.0 * vi * vj * w / (s * s);
            p[((long)j * n + i) * V] = (T)aij;
        }
    }
}

template <typename T> struct Batch {
    int m, n, nrhs, V, nm;
    long lanes;
    T *a = nullptr, *a0 = nullptr, *b = nullptr, *b0 = nullptr, *tau = nullptr;
    void *ws = nullptr;
    size_t sa = 0, sb = 0, ws_bytes = 0;
};

template <typename T> void release(Batch<T> &B)
{
    cudaFree(B.a);
    cudaFree(B.a0);
    cudaFree(B.b);
    cudaFree(B.b0);
    cudaFree(B.tau);
    cudaFree(B.ws);
    B = Batch<T>{};
}

enum Kind { FACTOR, SOLVE, FUSED, TRSM, GEQRF, ORMQR, ORGQR, GELS, REFINED };

struct Spec {
    int routine;
    Kind kind;
    bool ldlt;
    bool spd;  // diagonal raised
    int key;   // the order the launcher keys the table on
};

template <typename T>
cudaError_t run(const Spec &sp, Batch<T> &B, cudaStream_t s)
{
    const int m = B.m, n = B.n, nrhs = B.nrhs, V = B.V, nm = B.nm;
    switch (sp.kind) {
    case FACTOR: return launch_factor<T>(sp.ldlt, false, false, n, B.a, n, V, nm, s);
    case SOLVE:
        return launch_sym_solve<T>(sp.ldlt, false, false, false, n, nrhs, B.a, n, B.b, n, V, nm, s);
    case FUSED:
        return launch_sym_solve<T>(sp.ldlt, true, false, false, n, nrhs, B.a, n, B.b, n, V, nm, s);
    case TRSM:
        return launch_trsm<T>(true, false, false, false, false, n, nrhs, T(1), B.a, n, B.b, n, V,
                              nm, s);
    case GEQRF: return launch_geqrf<T>(false, m, n, B.a, m, B.tau, V, nm, s);
    case ORMQR:
        return launch_ormqr<T>(true, false, true, m, nrhs, n, B.a, m, B.tau, B.b, m, V, nm, s);
    case ORGQR: return launch_orgqr<T>(false, m, n, n, B.a, m, B.tau, V, nm, s);
    case GELS: return launch_gels<T>(false, false, m, n, nrhs, B.a, m, B.b, m, B.tau, V, nm, s);
    case REFINED:
        if constexpr (sizeof(T) == 8)
            return launch_posv_refined(false, false, n, nrhs, B.a, n, B.b, n, V, nm, 10, nullptr,
                                       nullptr, B.ws, s);
        return cudaErrorInvalidValue;
    }
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t make_batch(const Spec &sp, int m, int n, int nrhs, int V, int nm, Batch<T> &B,
                       cudaStream_t s)
{
    B.m = m;
    B.n = n;
    B.nrhs = nrhs;
    B.V = V;
    B.nm = nm;
    B.lanes = ((long)nm + V - 1) / V * V;
    const int rows = (sp.kind == GEQRF || sp.kind == ORMQR || sp.kind == ORGQR ||
                      sp.kind == GELS) ? m : n;
    B.sa = (size_t)B.lanes * rows * n;
    B.sb = (size_t)B.lanes * std::max(rows, 1) * std::max(nrhs, 1);
    cudaError_t e;
    if ((e = cudaMalloc(&B.a, B.sa * sizeof(T))) || (e = cudaMalloc(&B.a0, B.sa * sizeof(T))) ||
        (e = cudaMalloc(&B.b, B.sb * sizeof(T))) || (e = cudaMalloc(&B.b0, B.sb * sizeof(T))) ||
        (e = cudaMalloc(&B.tau, (size_t)B.lanes * std::max(std::min(m, n), 1) * sizeof(T))))
        return e;
    if (sp.kind == REFINED) {
        B.ws_bytes = posv_refined_lwork(n, nrhs, V, nm);
        if (B.ws_bytes && (e = cudaMalloc(&B.ws, B.ws_bytes))) return e;
    }
    const unsigned grid = 1024;
    k_fill_uniform<T><<<grid, 256, 0, s>>>(B.a0, (long)B.sa, 0x5EEDull);
    k_fill_uniform<T><<<grid, 256, 0, s>>>(B.b0, (long)B.sb, 0xB0Bull);
    if (sp.kind == REFINED)
        k_fill_spd_reflector<T><<<(unsigned)((B.lanes + 127) / 128), 128, 0, s>>>(
            B.a0, n, V, B.lanes, 0x5EEDull);
    else if (sp.spd)
        k_shift_diag<T><<<(unsigned)((B.lanes + 255) / 256), 256, 0, s>>>(B.a0, n, V, B.lanes,
                                                                          T(n + 1));
    if ((e = cudaGetLastError())) return e;
    // routines that consume a factorization get it once, untimed
    if (sp.kind == SOLVE) e = launch_factor<T>(sp.ldlt, false, false, n, B.a0, n, V, nm, s);
    if (sp.kind == ORMQR || sp.kind == ORGQR) e = launch_geqrf<T>(false, m, n, B.a0, m, B.tau, V, nm, s);
    return e;
}

template <typename T>
cudaError_t time_one(const Spec &sp, Batch<T> &B, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1,
                     float &best)
{
    best = FLT_MAX;
    for (int rep = 0; rep < 4; ++rep) {
        cudaError_t e;
        if ((e = cudaMemcpyAsync(B.a, B.a0, B.sa * sizeof(T), cudaMemcpyDeviceToDevice, s)) ||
            (e = cudaMemcpyAsync(B.b, B.b0, B.sb * sizeof(T), cudaMemcpyDeviceToDevice, s)) ||
            (e = cudaEventRecord(e0, s)) || (e = run<T>(sp, B, s)) || (e = cudaEventRecord(e1, s)) ||
            (e = cudaEventSynchronize(e1)))
            return e;
        float ms = 0.f;
        if ((e = cudaEventElapsedTime(&ms, e0, e1))) return e;
        if (rep > 0) best = std::min(best, ms); // the first run warms up
    }
    return cudaSuccess;
}

template <typename T>
int autotune(const Spec &sp, int m, int n, int nrhs, int nm, int only_V,
             const cbk_cuda_tune_result &old, cbk_cuda_tune_result *out)
{
    constexpr int ds = sizeof(T);
    const bool warp = sp.kind == REFINED && posv_refined_warp_ok(n);
    const int all_widths[] = {32, 64, 128};
    const int one_width[] = {only_V};
    const int nwidths = only_V ? 1 : 3;
    const int *widths = only_V ? one_width : all_widths;
    // the lane-per-matrix refined kernels are compiled for at most 128 threads
    const int lane_threads[] = {64, 128, 256}, refined_threads[] = {32, 64, 128};
    const int *threads = sp.kind == REFINED ? refined_threads : lane_threads;
    const int nshape = warp ? MAX_VARIANTS : 3;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (!err) err = cudaEventCreate(&e0);
    if (!err) err = cudaEventCreate(&e1);
    float best = FLT_MAX;
    int best_shape = 0, best_V = 32;
    for (int wi = 0; wi < nwidths; ++wi) {
        const int V = widths[wi];
        if (err) break;
        Batch<T> B;
        err = make_batch<T>(sp, m, n, nrhs, V, nm, B, s);
        for (int k = 0; k < nshape && !err; ++k) {
            if (warp) set_variant(sp.routine, sp.key, ds, k);
            else set_threads(sp.routine, sp.key, ds, threads[k]);
            float ms = 0.f;
            err = time_one<T>(sp, B, s, e0, e1, ms);
            if (!err && ms < best) {
                best = ms;
                best_shape = k;
                best_V = V;
            }
        }
        cudaStreamSynchronize(s);
        release(B);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (err) { // the entry keeps what it held before the search
        set_variant(sp.routine, sp.key, ds, old.variant);
        set_threads(sp.routine, sp.key, ds, old.threads);
        return CBK_CUDA_ERROR_BASE + (int)err;
    }
    if (warp) set_variant(sp.routine, sp.key, ds, best_shape);
    else set_threads(sp.routine, sp.key, ds, threads[best_shape]);
    set_vlen(sp.routine, sp.key, ds, best_V);
    if (out) {
        out->threads = warp ? 0 : threads[best_shape];
        out->variant = warp ? best_shape : 0;
        out->vlen = best_V;
        out->ms = best;
    }
    return 0;
}

// The bucketed launch: a synthetic uneven batch -- orders from 4 (or 1) up
// to n, nm matrices split evenly, each bucket uniform in [-1, 1) with the
// diagonal raised by 2 k (diagonally dominant: both LDL^T without pivoting
// and Cholesky apply) -- timed at every grid variant (the persistent warps
// per SM halved 0 .. 3 times); the winner is stored at the largest order,
// the key the launch reads.
template <typename T>
int autotune_bucketed(int routine, bool ldlt, int n, int nrhs, int nm, int only_V,
                      const cbk_cuda_tune_result &old, cbk_cuda_tune_result *out)
{
    constexpr int ds = sizeof(T);
    const int V = only_V ? only_V : 32;
    const int lo = std::max(1, std::min(4, n));
    int nb = n - lo + 1;
    if (nb > CBK_CUDA_MAX_BUCKETS) nb = CBK_CUDA_MAX_BUCKETS;
    const int per = std::max(32, nm / nb);
    int ns[CBK_CUDA_MAX_BUCKETS], nms[CBK_CUDA_MAX_BUCKETS], Vs[CBK_CUDA_MAX_BUCKETS];
    int lda[CBK_CUDA_MAX_BUCKETS], ldb[CBK_CUDA_MAX_BUCKETS];
    T *a[CBK_CUDA_MAX_BUCKETS] = {}, *a0[CBK_CUDA_MAX_BUCKETS] = {};
    T *b[CBK_CUDA_MAX_BUCKETS] = {}, *b0[CBK_CUDA_MAX_BUCKETS] = {};
    size_t sa[CBK_CUDA_MAX_BUCKETS], sb[CBK_CUDA_MAX_BUCKETS];
    void *work = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (!err) err = cudaEventCreate(&e0);
    if (!err) err = cudaEventCreate(&e1);
    if (!err) err = cudaMalloc(&work, CBK_CUDA_BUCKETED_LWORK);
    for (int k = 0; k < nb && !err; ++k) {
        // orders spread over lo .. n when there are more than the bucket limit
        const int ord = nb == n - lo + 1 ? lo + k : lo + (int)((long)k * (n - lo) / (nb - 1));
        ns[k] = ord;
        nms[k] = per;
        Vs[k] = V;
        lda[k] = ord;
        ldb[k] = ord;
        const long lanes = ((long)per + V - 1) / V * V;
        sa[k] = (size_t)lanes * ord * ord;
        sb[k] = (size_t)lanes * ord * std::max(nrhs, 1);
        if ((err = cudaMalloc(&a[k], sa[k] * ds)) || (err = cudaMalloc(&a0[k], sa[k] * ds)) ||
            (err = cudaMalloc(&b[k], sb[k] * ds)) || (err = cudaMalloc(&b0[k], sb[k] * ds)))
            break;
        k_fill_uniform<T><<<256, 256, 0, s>>>(a0[k], (long)sa[k], 0x5EEDull + k);
        k_fill_uniform<T><<<256, 256, 0, s>>>(b0[k], (long)sb[k], 0xB0Bull + k);
        k_shift_diag<T><<<(unsigned)((lanes + 255) / 256), 256, 0, s>>>(a0[k], ord, V, lanes,
                                                                        T(2 * ord));
        err = cudaGetLastError();
    }
    float best = FLT_MAX;
    int best_v = 0;
    for (int v = 0; v < MAX_VARIANTS && !err; ++v) {
        set_variant(routine, n, ds, v);
        float vbest = FLT_MAX;
        for (int rep = 0; rep < 4 && !err; ++rep) {
            for (int k = 0; k < nb && !err; ++k)
                if ((err = cudaMemcpyAsync(a[k], a0[k], sa[k] * ds, cudaMemcpyDeviceToDevice, s)) ||
                    (err = cudaMemcpyAsync(b[k], b0[k], sb[k] * ds, cudaMemcpyDeviceToDevice, s)))
                    break;
            if (err || (err = cudaEventRecord(e0, s)) ||
                (err = launch_bucketed<T>(ldlt, false, false, nrhs, nb, ns, nms, Vs, a, lda, b, ldb,
                                          work, s)) ||
                (err = cudaEventRecord(e1, s)) || (err = cudaEventSynchronize(e1)))
                break;
            float ms = 0.f;
            if ((err = cudaEventElapsedTime(&ms, e0, e1))) break;
            if (rep > 0) vbest = std::min(vbest, ms); // the first run warms up
        }
        if (!err && vbest < best) {
            best = vbest;
            best_v = v;
        }
    }
    if (s) cudaStreamSynchronize(s);
    for (int k = 0; k < nb; ++k) {
        cudaFree(a[k]);
        cudaFree(a0[k]);
        cudaFree(b[k]);
        cudaFree(b0[k]);
    }
    cudaFree(work);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (err) {
        set_variant(routine, n, ds, old.variant);
        return CBK_CUDA_ERROR_BASE + (int)err;
    }
    set_variant(routine, n, ds, best_v);
    set_vlen(routine, n, ds, V);
    if (out) {
        out->threads = 0;
        out->variant = best_v;
        out->vlen = V;
        out->ms = best;
    }
    return 0;
}

} // namespace

} // namespace cbkcuda

using namespace cbkcuda;

namespace {

int autotune_entry(const char *routine, char prec, int m, int n, int nrhs, int nm, int only_V,
                   cbk_cuda_tune_result *out)
{
    const int r = routine_of(routine);
    if (r < 0) return -1;
    if (prec != 'd' && prec != 's') return -2;
    const bool qr = r == R_GEQRF || r == R_ORMQR || r == R_ORGQR || r == R_GELS;
    if (m < 0 || (qr && m < n)) return -3;
    if (n < 1) return -4;
    const bool rhs = r == R_POTRS || r == R_POSV || r == R_SYTRSNP || r == R_SYSVNP ||
                     r == R_TRSM || r == R_ORMQR || r == R_GELS || r == R_POSV_REFINED;
    if (nrhs < (rhs ? 1 : 0)) return -5;
    if (nm < 1) return -6;
    if (r == R_POSV_REFINED && prec != 'd') return -2;
    if (r == R_SYSVNP_BUCKETED || r == R_POSV_BUCKETED) {
        cbk_cuda_tune_result old{};
        cbk_cuda_tune_get(routine, prec, n, &old);
        const bool ldlt = r == R_SYSVNP_BUCKETED;
        return prec == 'd' ? autotune_bucketed<double>(r, ldlt, n, nrhs, nm, only_V, old, out)
                           : autotune_bucketed<float>(r, ldlt, n, nrhs, nm, only_V, old, out);
    }
    Spec sp{r, FACTOR, false, false, n};
    switch (r) {
    case R_POTRF: sp = {r, FACTOR, false, true, n}; break;
    case R_SYTRFNP: sp = {r, FACTOR, true, true, n}; break;
    case R_POTRS: sp = {r, SOLVE, false, true, n}; break;
    case R_SYTRSNP: sp = {r, SOLVE, true, true, n}; break;
    case R_POSV: sp = {r, FUSED, false, true, n}; break;
    case R_SYSVNP: sp = {r, FUSED, true, true, n}; break;
    case R_TRSM: sp = {r, TRSM, false, true, n}; break;
    case R_GEQRF: sp = {r, GEQRF, false, false, m}; break;
    case R_ORMQR: sp = {r, ORMQR, false, false, m}; break;
    case R_ORGQR: sp = {r, ORGQR, false, false, m}; break;
    case R_GELS: sp = {r, GELS, false, false, m}; break;
    case R_POSV_REFINED: sp = {r, REFINED, false, true, n}; break;
    default: return -1;
    }
    cbk_cuda_tune_result old{};
    cbk_cuda_tune_get(routine, prec, sp.key, &old);
    return prec == 'd' ? autotune<double>(sp, m, n, nrhs, nm, only_V, old, out)
                       : autotune<float>(sp, m, n, nrhs, nm, only_V, old, out);
}

} // namespace

extern "C" int cbk_cuda_autotune(const char *routine, char prec, int m, int n, int nrhs, int nm,
                                 cbk_cuda_tune_result *out)
{
    return autotune_entry(routine, prec, m, n, nrhs, nm, 0, out);
}

extern "C" int cbk_cuda_autotune_at(const char *routine, char prec, int m, int n, int nrhs, int nm,
                                    int V, cbk_cuda_tune_result *out)
{
    if (routine_of(routine) < 0) return -1;
    if (V < 32 || V > 1024 || V % 32 != 0) return -7;
    return autotune_entry(routine, prec, m, n, nrhs, nm, V, out);
}
