// cbk_api.cpp -- the extern "C" entry points of include/cbk_cuda.h.
//
// Each routine checks its arguments in argument order and returns -j for the
// first illegal one, takes the reference's quick returns, then enqueues the
// CUDA kernel(s) on the caller's stream. The checks and quick returns restate
// the reference's C adapter, src/cbk.cpp:46-320 (per-routine templates geqrf
// :61-78, ormqr :80-105, orgqr :107-127, potrf :129-147, sytrfnp :149-167,
// sym_solve_args :173-188, potrs :190-205, posv :207-224, sytrsnp :226-241,
// sysvnp :243-260, trsm :262-293, gels :295-320), with the accepted interleave
// widths widened to multiples of 32. Pointers are never inspected.
#include "../../include/cbk_cuda.h"
#include "cbk_launch.h"

#include <cuda_runtime.h>

#ifdef CBK_CUDA_CHECKED
// The checked build's status words: every translation unit that includes the
// device header registers a reader of its own word at load time.
namespace cbkcuda {
typedef int (*CheckReader)(unsigned long long *count, unsigned long long *first, int reset);
namespace {
constexpr int MAX_READERS = 64;
struct Readers {
    CheckReader r[MAX_READERS];
    int n = 0;
};
Readers &readers()
{
    static Readers g;
    return g;
}
} // namespace
void register_check_reader(CheckReader r)
{
    Readers &g = readers();
    if (g.n < MAX_READERS) g.r[g.n++] = r;
}
inline const CheckReader *check_readers() { return readers().r; }
inline int check_readers_n() { return readers().n; }
} // namespace cbkcuda
#endif

namespace {

using namespace cbkcuda;

inline bool opt(char c, char upper)
{
    return c == upper || c == upper + ('a' - 'A');
}

inline int max1(int x)
{
    return x < 1 ? 1 : x;
}

inline bool vlen_ok(int V)
{
    if (V == 2 || V == 4 || V == 8 || V == 16) return true;
    return V >= 32 && V <= 1024 && V % 32 == 0;
}

inline int cuda_status(cudaError_t e)
{
    return e == cudaSuccess ? 0 : CBK_CUDA_ERROR_BASE + (int)e;
}

// The host-pointer layer runs a routine's checks and quick returns first
// without its launch (a dry run): every routine below returns 0 at the point
// where it would launch, and records that it would have.
thread_local bool tl_dry = false;
thread_local bool tl_would_launch = false;

inline bool dry_stop()
{
    if (!tl_dry) return false;
    tl_would_launch = true;
    return true;
}

template <typename T>
int geqrf(char layout, int m, int n, T *ap, int ldap, T *taup, int V, int nm, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    if (!col && !row) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (ldap < max1(row ? n : m)) return -5;
    if (!vlen_ok(V)) return -7;
    if (nm < 0) return -8;
    if (m == 0 || n == 0 || nm == 0) return 0;
    if (dry_stop()) return 0;
    return cuda_status(launch_geqrf<T>(row, m, n, ap, ldap, taup, V, nm, s));
}

template <typename T>
int ormqr(char layout, char side, char trans, int m, int n, int k, const T *ap, int ldap,
          const T *taup, T *cp, int ldcp, int V, int nm, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const bool left = opt(side, 'L'), right = opt(side, 'R');
    const int nq = left ? m : n;
    if (!col && !row) return -1;
    if (!left && !right) return -2;
    if (!opt(trans, 'T') && !opt(trans, 'N')) return -3;
    if (m < 0) return -4;
    if (n < 0) return -5;
    if (k < 0 || k > nq) return -6;
    if (ldap < max1(row ? k : nq)) return -8;
    if (ldcp < max1(row ? n : m)) return -11;
    if (!vlen_ok(V)) return -12;
    if (nm < 0) return -13;
    if (m == 0 || n == 0 || k == 0 || nm == 0) return 0;
    if (dry_stop()) return 0;
    return cuda_status(launch_ormqr<T>(left, row, opt(trans, 'T'), m, n, k, ap, ldap, taup, cp,
                                       ldcp, V, nm, s));
}

template <typename T>
int orgqr(char layout, int m, int n, int k, T *ap, int ldap, const T *taup, int V, int nm,
          cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    if (!col && !row) return -1;
    if (m < 0) return -2;
    if (n < 0 || n > m) return -3;
    if (k < 0 || k > n) return -4;
    if (ldap < max1(row ? n : m)) return -6;
    if (!vlen_ok(V)) return -8;
    if (nm < 0) return -9;
    // k == 0 is not empty: Q = I(:, 0:n-1) is still written
    if (m == 0 || n == 0 || nm == 0) return 0;
    if (dry_stop()) return 0;
    return cuda_status(launch_orgqr<T>(row, m, n, k, ap, ldap, taup, V, nm, s));
}

template <typename T>
int factor(bool ldlt, char layout, char uplo, int n, T *ap, int ldap, int V, int nm,
           cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const bool lo = opt(uplo, 'L'), up = opt(uplo, 'U');
    if (!col && !row) return -1;
    if (!lo && !up) return -2;
    if (n < 0) return -3;
    if (ldap < max1(n)) return -5;
    if (!vlen_ok(V)) return -6;
    if (nm < 0) return -7;
    if (n == 0 || nm == 0) return 0;
    if (dry_stop()) return 0;
    return cuda_status(launch_factor<T>(ldlt, row, up, n, ap, ldap, V, nm, s));
}

// ?potrs / ?posv / ?sytrsnp / ?sysvnp share one signature and one check
// (sym_solve_args): -1 layout -2 uplo -3 n -4 nrhs -6 ldap -8 ldbp -9 V -10 nm.
int sym_solve_args(char layout, char uplo, int n, int nrhs, int ldap, int ldbp, int V, int nm,
                   bool &row, bool &up)
{
    const bool col = opt(layout, 'C'), lo = opt(uplo, 'L');
    row = opt(layout, 'R');
    up = opt(uplo, 'U');
    if (!col && !row) return -1;
    if (!lo && !up) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (ldap < max1(n)) return -6;
    if (ldbp < max1(row ? nrhs : n)) return -8;
    if (!vlen_ok(V)) return -9;
    if (nm < 0) return -10;
    return 0;
}

template <typename T>
int sym_solve(bool ldlt, bool fused, char layout, char uplo, int n, int nrhs, T *ap, int ldap,
              T *bp, int ldbp, int V, int nm, cudaStream_t s)
{
    bool row, up;
    if (int e = sym_solve_args(layout, uplo, n, nrhs, ldap, ldbp, V, nm, row, up)) return e;
    if (n == 0 || nm == 0) return 0;
    if (nrhs == 0) {
        // the solve alone has nothing to do; the fused driver still factors
        // (LAPACK ?posv / ?sysv), never referencing bp
        if (!fused) return 0;
        if (dry_stop()) return 0;
        return cuda_status(launch_factor<T>(ldlt, row, up, n, ap, ldap, V, nm, s));
    }
    if (dry_stop()) return 0;
    return cuda_status(
        launch_sym_solve<T>(ldlt, fused, row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, s));
}

template <typename T>
int trsm(char layout, char side, char uplo, char transa, char diag, int m, int n, T alpha,
         const T *ap, int ldap, T *bp, int ldbp, int V, int nm, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const bool left = opt(side, 'L'), right = opt(side, 'R');
    const bool up = opt(uplo, 'U'), lo = opt(uplo, 'L');
    const bool tran = opt(transa, 'T') || opt(transa, 'C');
    const bool unit = opt(diag, 'U');
    const int sdim = left ? m : n;
    if (!col && !row) return -1;
    if (!left && !right) return -2;
    if (!up && !lo) return -3;
    if (!tran && !opt(transa, 'N')) return -4;
    if (!unit && !opt(diag, 'N')) return -5;
    if (m < 0) return -6;
    if (n < 0) return -7;
    // -8 alpha: every value is legal (0 means B := 0)
    if (ldap < max1(sdim)) return -10;
    if (ldbp < max1(row ? n : m)) return -12;
    if (!vlen_ok(V)) return -13;
    if (nm < 0) return -14;
    if (m == 0 || n == 0 || nm == 0) return 0;
    if (dry_stop()) return 0;
    if (alpha == T(0)) return cuda_status(launch_zero<T>(row, m, n, bp, ldbp, V, nm, s));
    return cuda_status(
        launch_trsm<T>(left, up, row, tran, unit, m, n, alpha, ap, ldap, bp, ldbp, V, nm, s));
}

template <typename T>
int gels(char layout, char trans, int m, int n, int nrhs, T *ap, int ldap, T *bp, int ldbp,
         T *taup, int V, int nm, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const int mx = m > n ? m : n;
    if (!col && !row) return -1;
    if (!opt(trans, 'N') && !opt(trans, 'T') && !opt(trans, 'C')) return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (nrhs < 0) return -5;
    if (ldap < max1(row ? n : m)) return -7;
    if (ldbp < max1(row ? nrhs : mx)) return -9;
    if (!vlen_ok(V)) return -11;
    if (nm < 0) return -12;
    if (nrhs == 0 || nm == 0 || mx == 0) return 0;
    const bool tran = opt(trans, 'T') || opt(trans, 'C');
    if (dry_stop()) return 0;
    return cuda_status(
        launch_gels<T>(row, tran, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, s));
}

template <typename T>
int pack(char layout, int m, int n, const T *a, int lda, long long stride, T *ap, int ldap,
         int V, int nm, T pad_diag, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    if (!col && !row) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (lda < max1(row ? n : m)) return -5;
    if (stride < (long long)lda * (row ? m : n)) return -6;
    if (ldap < max1(row ? n : m)) return -8;
    if (!vlen_ok(V)) return -9;
    if (nm < 0) return -10;
    if (m == 0 || n == 0 || nm == 0) return 0;
    return cuda_status(launch_pack<T>(row, m, n, a, lda, stride, ap, ldap, V, nm, pad_diag, s));
}

template <typename T>
int unpack(char layout, int m, int n, const T *ap, int ldap, T *a, int lda, long long stride,
           int V, int nm, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    if (!col && !row) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (ldap < max1(row ? n : m)) return -5;
    if (lda < max1(row ? n : m)) return -7;
    if (stride < (long long)lda * (row ? m : n)) return -8;
    if (!vlen_ok(V)) return -9;
    if (nm < 0) return -10;
    if (m == 0 || n == 0 || nm == 0) return 0;
    return cuda_status(launch_unpack<T>(row, m, n, ap, ldap, a, lda, stride, V, nm, s));
}

int posv_refined(char layout, char uplo, int n, int nrhs, double *ap, int ldap, double *bp,
                 int ldbp, int V, int nm, int max_iter, int *iters, double *berr, void *work,
                 long long lwork, cudaStream_t s)
{
    bool row, up;
    if (int e = sym_solve_args(layout, uplo, n, nrhs, ldap, ldbp, V, nm, row, up)) return e;
    if (max_iter < 0) return -11;
    if (n == 0 || nm == 0 || nrhs == 0) return 0;
    const size_t need = posv_refined_lwork(n, nrhs, V, nm);
    if (need > 0 && (work == nullptr || lwork < (long long)need)) return -15;
    return cuda_status(launch_posv_refined(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter,
                                           iters, berr, work, s));
}

// The refined solve on a strided dense batch: matrix k's A at a + k stride_a
// (column-major, leading dimension lda), its B at b + k stride_b. That is
// the compact layout at V = 1 with the caller's group strides, so the kernels
// read and write the dense arrays directly (no pack or unpack pass).
int posv_refined_batched(char uplo, int n, int nrhs, double *a, int lda, long long stride_a,
                         double *b, int ldb, long long stride_b, int nm, int max_iter, int *iters,
                         double *berr, void *work, long long lwork, cudaStream_t s)
{
    const bool lo = opt(uplo, 'L'), up = opt(uplo, 'U');
    if (!lo && !up) return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (lda < max1(n)) return -5;
    if (stride_a < (long long)lda * n) return -6;
    if (ldb < max1(n)) return -8;
    if (stride_b < (long long)ldb * nrhs) return -9;
    if (nm < 0) return -10;
    if (max_iter < 0) return -11;
    if (n == 0 || nm == 0 || nrhs == 0) return 0;
    const size_t need = posv_refined_lwork(n, nrhs, 1, nm);
    if (need > 0 && (work == nullptr || lwork < (long long)need)) return -15;
    return cuda_status(launch_posv_refined(false, up, n, nrhs, a, lda, b, ldb, 1, nm, max_iter,
                                           iters, berr, work, s, (size_t)stride_a,
                                           (size_t)stride_b));
}

// The plain FP64 / FP32 drivers on a strided dense batch: the compact layout
// at V = 1 with the caller's group strides, so the lane kernels read and
// write the dense arrays directly (no pack or unpack pass), matrix by matrix
// with the compact entry point's operations (identical bits). ?posv_batched /
// ?sysvnp_batched: -1 uplo -2 n -3 nrhs -5 lda -6 stride_a -8 ldb -9 stride_b
// -10 nm; nrhs = 0 still factors (as the compact drivers).
template <typename T>
int sym_solve_batched(bool ldlt, char uplo, int n, int nrhs, T *a, int lda, long long stride_a,
                      T *b, int ldb, long long stride_b, int nm, cudaStream_t s)
{
    const bool lo = opt(uplo, 'L'), up = opt(uplo, 'U');
    if (!lo && !up) return -1;
    if (n < 0) return -2;
    if (nrhs < 0) return -3;
    if (lda < max1(n)) return -5;
    if (stride_a < (long long)lda * n) return -6;
    if (ldb < max1(n)) return -8;
    if (stride_b < (long long)ldb * nrhs) return -9;
    if (nm < 0) return -10;
    if (n == 0 || nm == 0) return 0;
    if (nrhs == 0)
        return cuda_status(launch_factor<T>(ldlt, false, up, n, a, lda, 1, nm, s, (size_t)stride_a));
    return cuda_status(launch_sym_solve<T>(ldlt, true, false, up, n, nrhs, a, lda, b, ldb, 1, nm, s,
                                           (size_t)stride_a, (size_t)stride_b));
}

// ?gels_batched: A m x n at a + k stride_a, B max(m, n) x nrhs at
// b + k stride_b, the min(m, n) tau values at tau + k min(m, n).
// -1 trans -2 m -3 n -4 nrhs -6 lda -7 stride_a -9 ldb -10 stride_b -12 nm.
template <typename T>
int gels_batched(char trans, int m, int n, int nrhs, T *a, int lda, long long stride_a, T *b,
                 int ldb, long long stride_b, T *tau, int nm, cudaStream_t s)
{
    const int mx = m > n ? m : n;
    if (!opt(trans, 'N') && !opt(trans, 'T') && !opt(trans, 'C')) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (lda < max1(m)) return -6;
    if (stride_a < (long long)lda * n) return -7;
    if (ldb < max1(mx)) return -9;
    if (stride_b < (long long)ldb * nrhs) return -10;
    if (nm < 0) return -12;
    if (nrhs == 0 || nm == 0 || mx == 0) return 0;
    const bool tran = opt(trans, 'T') || opt(trans, 'C');
    return cuda_status(launch_gels<T>(false, tran, m, n, nrhs, a, lda, b, ldb, tau, 1, nm, s,
                                      (size_t)stride_a, (size_t)stride_b));
}

// The refined least squares on a strided dense batch (A m x n at
// a + k stride_a, B m x nrhs at b + k stride_b, column-major; tau n per
// matrix at tau + k n): the compact layout at V = 1 with these strides.
int gels_refined_batched(char trans, int m, int n, int nrhs, double *a, int lda,
                         long long stride_a, double *b, int ldb, long long stride_b, double *tau,
                         int nm, int max_iter, int *iters, double *berr, void *work,
                         long long lwork, cudaStream_t s)
{
    if (!opt(trans, 'N')) return -1; // the refined path solves A X = B
    if (m < 0) return -2;
    if (n < 0 || n > m || n > gels_refined_nmax()) return -3;
    if (nrhs < 0) return -4;
    if (lda < max1(m)) return -6;
    if (stride_a < (long long)lda * n) return -7;
    if (ldb < max1(m)) return -9;
    if (stride_b < (long long)ldb * nrhs) return -10;
    if (nm < 0) return -12;
    if (max_iter < 0) return -13;
    if (nrhs == 0 || nm == 0 || m == 0) return 0;
    if (n == 0)
        return cuda_status(
            launch_zero<double>(false, m, nrhs, b, ldb, 1, nm, s, (size_t)stride_b));
    const size_t need = gels_refined_lwork(m, n, nrhs, 1, nm);
    if (work == nullptr || lwork < (long long)need) return -17;
    return cuda_status(launch_gels_refined(false, m, n, nrhs, a, lda, b, ldb, tau, 1, nm,
                                           max_iter, iters, berr, work, s, (size_t)stride_a,
                                           (size_t)stride_b));
}

int gels_refined(char layout, char trans, int m, int n, int nrhs, double *ap, int ldap, double *bp,
                 int ldbp, double *taup, int V, int nm, int max_iter, int *iters, double *berr,
                 void *work, long long lwork, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const int mx = m > n ? m : n;
    if (!col && !row) return -1;
    if (!opt(trans, 'N')) return -2; // the refined path solves A X = B
    if (m < 0) return -3;
    if (n < 0 || n > m || n > gels_refined_nmax()) return -4;
    if (nrhs < 0) return -5;
    if (ldap < max1(row ? n : m)) return -7;
    if (ldbp < max1(row ? nrhs : mx)) return -9;
    if (!vlen_ok(V)) return -11;
    if (nm < 0) return -12;
    if (max_iter < 0) return -13;
    if (nrhs == 0 || nm == 0 || m == 0) return 0;
    if (n == 0) return cuda_status(launch_zero<double>(row, m, nrhs, bp, ldbp, V, nm, s));
    const size_t need = gels_refined_lwork(m, n, nrhs, V, nm);
    if (work == nullptr || lwork < (long long)need) return -17;
    return cuda_status(launch_gels_refined(row, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                                           max_iter, iters, berr, work, s));
}

template <typename T, typename Bucket>
int bucketed(bool ldlt, char layout, char uplo, int nrhs, int nbuckets, const Bucket *bk,
             void *work, long long lwork, cudaStream_t s)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    const bool lo = opt(uplo, 'L'), up = opt(uplo, 'U');
    if (!col && !row) return -1;
    if (!lo && !up) return -2;
    if (nrhs < 0) return -3;
    if (nbuckets < 0 || nbuckets > CBK_CUDA_MAX_BUCKETS) return -4;
    if (nbuckets > 0 && bk == nullptr) return -5;
    int n[CBK_CUDA_MAX_BUCKETS], nm[CBK_CUDA_MAX_BUCKETS], V[CBK_CUDA_MAX_BUCKETS];
    int lda[CBK_CUDA_MAX_BUCKETS], ldb[CBK_CUDA_MAX_BUCKETS];
    T *ap[CBK_CUDA_MAX_BUCKETS], *bp[CBK_CUDA_MAX_BUCKETS];
    bool any = false;
    for (int b = 0; b < nbuckets; ++b) {
        const Bucket &e = bk[b];
        if (e.n < 0 || e.nm < 0 || !vlen_ok(e.V) || e.ldap < max1(e.n) ||
            e.ldbp < max1(row ? nrhs : e.n))
            return -5;
        n[b] = e.n;
        nm[b] = e.nm;
        V[b] = e.V;
        lda[b] = e.ldap;
        ldb[b] = e.ldbp;
        ap[b] = e.ap;
        bp[b] = e.bp;
        any = any || (e.n > 0 && e.nm > 0);
    }
    if (work == nullptr) return -6;
    if (lwork < CBK_CUDA_BUCKETED_LWORK) return -7;
    if (!any) return 0;
    return cuda_status(
        launch_bucketed<T>(ldlt, row, up, nrhs, nbuckets, n, nm, V, ap, lda, bp, ldb, work, s));
}

inline cudaStream_t S(cbk_stream_t s)
{
    return reinterpret_cast<cudaStream_t>(s);
}

// ---------------------------------------------------------------------
// The host-pointer layer: the reference's calling convention (every array
// on the host) over the device routines above, through a caller-provided
// device workspace
// ---------------------------------------------------------------------

struct HostArray {
    void *host;
    size_t bytes;
    bool in, out;
};

inline size_t align256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

// bytes of a compact batch of nm rows x cols matrices, leading dimension ld
inline size_t compact_bytes(bool row, int ld, int rows, int cols, int V, int nm, size_t es)
{
    if (rows <= 0 || cols <= 0 || nm <= 0) return 0;
    const size_t ng = ((size_t)nm + V - 1) / V;
    return ng * (size_t)ld * (size_t)(row ? rows : cols) * (size_t)V * es;
}

// a routine's checks and quick returns, without its launch: its code, and in
// `launch` whether it has device work
template <typename F> int dry_run(F &&call, bool &launch)
{
    tl_dry = true;
    tl_would_launch = false;
    const int info = call();
    tl_dry = false;
    launch = tl_would_launch;
    return info;
}

// nothing to copy (an illegal argument or a quick return): a size query
// answers 0
inline int host_quick(int info, long long *lwork)
{
    if (info == 0 && lwork && *lwork < 0) *lwork = 0;
    return info;
}

// The arrays into the workspace (256-byte aligned, in order), the routine on
// them, the outputs back, the stream synchronised. wpos: the position of
// the dwork argument (-wpos: dwork null or *lwork too small; -(wpos + 1):
// lwork null). *lwork < 0 asks for the size instead.
template <typename F>
int host_run(int wpos, const HostArray *arr, int na, void *dwork, long long *lwork, cudaStream_t s,
             F &&run)
{
    size_t off[4], need = 0;
    for (int i = 0; i < na; ++i) {
        off[i] = need;
        need += align256(arr[i].bytes);
    }
    if (!lwork) return -(wpos + 1);
    if (*lwork < 0) {
        *lwork = (long long)need;
        return 0;
    }
    if ((size_t)*lwork < need || (need > 0 && !dwork)) return -wpos;
    char *d = static_cast<char *>(dwork);
    void *dev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < na && e == cudaSuccess; ++i) {
        dev[i] = arr[i].bytes ? d + off[i] : nullptr;
        if (arr[i].in && arr[i].bytes)
            e = cudaMemcpyAsync(dev[i], arr[i].host, arr[i].bytes, cudaMemcpyHostToDevice, s);
    }
    int info = e == cudaSuccess ? run(dev) : cuda_status(e);
    if (info == 0)
        for (int i = 0; i < na && e == cudaSuccess; ++i)
            if (arr[i].out && arr[i].bytes)
                e = cudaMemcpyAsync(arr[i].host, dev[i], arr[i].bytes, cudaMemcpyDeviceToHost, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (info != 0) return info;
    if (e != cudaSuccess) return cuda_status(e);
    return cuda_status(e2);
}

template <typename T>
int host_geqrf(char layout, int m, int n, T *ap, int ldap, T *taup, int V, int nm, void *dw,
               long long *lw, cudaStream_t s)
{
    bool go;
    const int info = dry_run([&] { return geqrf<T>(layout, m, n, ap, ldap, taup, V, nm, s); }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const int k = m < n ? m : n;
    const HostArray a[2] = {{ap, compact_bytes(row, ldap, m, n, V, nm, sizeof(T)), true, true},
                            {taup, compact_bytes(false, k, k, 1, V, nm, sizeof(T)), false, true}};
    return host_run(9, a, 2, dw, lw, s, [&](void **d) {
        return geqrf<T>(layout, m, n, (T *)d[0], ldap, (T *)d[1], V, nm, s);
    });
}

template <typename T>
int host_ormqr(char layout, char side, char trans, int m, int n, int k, const T *ap, int ldap,
               const T *taup, T *cp, int ldcp, int V, int nm, void *dw, long long *lw,
               cudaStream_t s)
{
    bool go;
    const int info = dry_run(
        [&] { return ormqr<T>(layout, side, trans, m, n, k, ap, ldap, taup, cp, ldcp, V, nm, s); },
        go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const int nq = opt(side, 'L') ? m : n;
    const HostArray a[3] = {
        {const_cast<T *>(ap), compact_bytes(row, ldap, nq, k, V, nm, sizeof(T)), true, false},
        {const_cast<T *>(taup), compact_bytes(false, k, k, 1, V, nm, sizeof(T)), true, false},
        {cp, compact_bytes(row, ldcp, m, n, V, nm, sizeof(T)), true, true}};
    return host_run(14, a, 3, dw, lw, s, [&](void **d) {
        return ormqr<T>(layout, side, trans, m, n, k, (const T *)d[0], ldap, (const T *)d[1],
                        (T *)d[2], ldcp, V, nm, s);
    });
}

template <typename T>
int host_orgqr(char layout, int m, int n, int k, T *ap, int ldap, const T *taup, int V, int nm,
               void *dw, long long *lw, cudaStream_t s)
{
    bool go;
    const int info =
        dry_run([&] { return orgqr<T>(layout, m, n, k, ap, ldap, taup, V, nm, s); }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const HostArray a[2] = {
        {ap, compact_bytes(row, ldap, m, n, V, nm, sizeof(T)), true, true},
        {const_cast<T *>(taup), compact_bytes(false, k, k, 1, V, nm, sizeof(T)), true, false}};
    return host_run(10, a, 2, dw, lw, s, [&](void **d) {
        return orgqr<T>(layout, m, n, k, (T *)d[0], ldap, (const T *)d[1], V, nm, s);
    });
}

template <typename T>
int host_factor(bool ldlt, char layout, char uplo, int n, T *ap, int ldap, int V, int nm,
                void *dw, long long *lw, cudaStream_t s)
{
    bool go;
    const int info =
        dry_run([&] { return factor<T>(ldlt, layout, uplo, n, ap, ldap, V, nm, s); }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const HostArray a[1] = {
        {ap, compact_bytes(opt(layout, 'R'), ldap, n, n, V, nm, sizeof(T)), true, true}};
    return host_run(8, a, 1, dw, lw, s, [&](void **d) {
        return factor<T>(ldlt, layout, uplo, n, (T *)d[0], ldap, V, nm, s);
    });
}

// ?potrs / ?sytrsnp (fused = false: A read only) and ?posv / ?sysvnp
template <typename T>
int host_sym_solve(bool ldlt, bool fused, char layout, char uplo, int n, int nrhs, T *ap,
                   int ldap, T *bp, int ldbp, int V, int nm, void *dw, long long *lw,
                   cudaStream_t s)
{
    bool go;
    const int info = dry_run([&] {
        return sym_solve<T>(ldlt, fused, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, s);
    }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const HostArray a[2] = {{ap, compact_bytes(row, ldap, n, n, V, nm, sizeof(T)), true, fused},
                            {bp, compact_bytes(row, ldbp, n, nrhs, V, nm, sizeof(T)), true, true}};
    return host_run(11, a, 2, dw, lw, s, [&](void **d) {
        return sym_solve<T>(ldlt, fused, layout, uplo, n, nrhs, (T *)d[0], ldap, (T *)d[1], ldbp,
                            V, nm, s);
    });
}

template <typename T>
int host_trsm(char layout, char side, char uplo, char transa, char diag, int m, int n, T alpha,
              const T *ap, int ldap, T *bp, int ldbp, int V, int nm, void *dw, long long *lw,
              cudaStream_t s)
{
    bool go;
    const int info = dry_run([&] {
        return trsm<T>(layout, side, uplo, transa, diag, m, n, alpha, ap, ldap, bp, ldbp, V, nm,
                       s);
    }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const int sdim = opt(side, 'L') ? m : n;
    const size_t abytes = alpha == T(0) ? 0 : compact_bytes(row, ldap, sdim, sdim, V, nm, sizeof(T));
    const HostArray a[2] = {{const_cast<T *>(ap), abytes, true, false},
                            {bp, compact_bytes(row, ldbp, m, n, V, nm, sizeof(T)), true, true}};
    return host_run(15, a, 2, dw, lw, s, [&](void **d) {
        return trsm<T>(layout, side, uplo, transa, diag, m, n, alpha, (const T *)d[0], ldap,
                       (T *)d[1], ldbp, V, nm, s);
    });
}

template <typename T>
int host_gels(char layout, char trans, int m, int n, int nrhs, T *ap, int ldap, T *bp, int ldbp,
              T *taup, int V, int nm, void *dw, long long *lw, cudaStream_t s)
{
    bool go;
    const int info = dry_run(
        [&] { return gels<T>(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, s); }, go);
    if (info != 0 || !go) return host_quick(info, lw);
    const bool row = opt(layout, 'R');
    const int k = m < n ? m : n, mx = m > n ? m : n;
    const HostArray a[3] = {{ap, compact_bytes(row, ldap, m, n, V, nm, sizeof(T)), true, true},
                            {bp, compact_bytes(row, ldbp, mx, nrhs, V, nm, sizeof(T)), true, true},
                            {taup, compact_bytes(false, k, k, 1, V, nm, sizeof(T)), false, true}};
    return host_run(13, a, 3, dw, lw, s, [&](void **d) {
        return gels<T>(layout, trans, m, n, nrhs, (T *)d[0], ldap, (T *)d[1], ldbp, (T *)d[2], V,
                       nm, s);
    });
}

} // namespace

extern "C" {

int cbk_cuda_get_version(void)
{
    return CBK_CUDA_VERSION;
}

int cbk_cuda_vlen_ok(int V)
{
    return vlen_ok(V) ? 1 : 0;
}

int cbk_cuda_check_status(unsigned long long *count, int *first_i, int *first_j, int reset)
{
    unsigned long long total = 0, first = 0;
    int rc = 0;
#ifdef CBK_CUDA_CHECKED
    for (int k = 0; k < cbkcuda::check_readers_n(); ++k) {
        unsigned long long c = 0, f = 0;
        const int e = cbkcuda::check_readers()[k](&c, &f, reset);
        if (e != 0 && rc == 0) rc = CBK_CUDA_ERROR_BASE + e;
        if (c != 0 && total == 0) first = f;
        total += c;
    }
#else
    (void)reset;
    rc = -1;
#endif
    if (count) *count = total;
    if (first_i) *first_i = (int)(unsigned)(first >> 32);
    if (first_j) *first_j = (int)(unsigned)(first & 0xffffffffull);
    return rc;
}

const char *cbk_cuda_status_string(int info)
{
    if (info == 0) return "success";
    if (info < 0) return "illegal argument (the -info-th)";
    if (info >= CBK_CUDA_ERROR_BASE)
        return cudaGetErrorString((cudaError_t)(info - CBK_CUDA_ERROR_BASE));
    if (info == CBK_CUDA_NOALLOC_TOO_LARGE) return "batch too large for the no-allocation scratch";
    if (info == CBK_CUDA_NOALLOC_IN_CAPTURE)
        return "first no-allocation call in this CUDA context made on a capturing stream";
    return "unknown status";
}

// One definition per routine and scalar type: NAME_async with the stream and
// NAME on the legacy default stream.
#define CBK_CUDA_ENTRY_POINTS(T, p)                                                               \
    int cbk_cuda_##p##geqrf_compact_async(char layout, int m, int n, T *ap, int ldap, T *taup,    \
                                          int V, int nm, cbk_stream_t st)                         \
    {                                                                                             \
        return geqrf<T>(layout, m, n, ap, ldap, taup, V, nm, S(st));                              \
    }                                                                                             \
    int cbk_cuda_##p##geqrf_compact(char layout, int m, int n, T *ap, int ldap, T *taup, int V,   \
                                    int nm)                                                       \
    {                                                                                             \
        return geqrf<T>(layout, m, n, ap, ldap, taup, V, nm, 0);                                  \
    }                                                                                             \
    int cbk_cuda_##p##ormqr_compact_async(char layout, char side, char trans, int m, int n,       \
                                          int k, const T *ap, int ldap, const T *taup, T *cp,     \
                                          int ldcp, int V, int nm, cbk_stream_t st)               \
    {                                                                                             \
        return ormqr<T>(layout, side, trans, m, n, k, ap, ldap, taup, cp, ldcp, V, nm, S(st));    \
    }                                                                                             \
    int cbk_cuda_##p##ormqr_compact(char layout, char side, char trans, int m, int n, int k,      \
                                    const T *ap, int ldap, const T *taup, T *cp, int ldcp, int V, \
                                    int nm)                                                       \
    {                                                                                             \
        return ormqr<T>(layout, side, trans, m, n, k, ap, ldap, taup, cp, ldcp, V, nm, 0);        \
    }                                                                                             \
    int cbk_cuda_##p##orgqr_compact_async(char layout, int m, int n, int k, T *ap, int ldap,      \
                                          const T *taup, int V, int nm, cbk_stream_t st)          \
    {                                                                                             \
        return orgqr<T>(layout, m, n, k, ap, ldap, taup, V, nm, S(st));                           \
    }                                                                                             \
    int cbk_cuda_##p##orgqr_compact(char layout, int m, int n, int k, T *ap, int ldap,            \
                                    const T *taup, int V, int nm)                                 \
    {                                                                                             \
        return orgqr<T>(layout, m, n, k, ap, ldap, taup, V, nm, 0);                               \
    }                                                                                             \
    int cbk_cuda_##p##potrf_compact_async(char layout, char uplo, int n, T *ap, int ldap, int V,  \
                                          int nm, cbk_stream_t st)                                \
    {                                                                                             \
        return factor<T>(false, layout, uplo, n, ap, ldap, V, nm, S(st));                         \
    }                                                                                             \
    int cbk_cuda_##p##potrf_compact(char layout, char uplo, int n, T *ap, int ldap, int V,        \
                                    int nm)                                                       \
    {                                                                                             \
        return factor<T>(false, layout, uplo, n, ap, ldap, V, nm, 0);                             \
    }                                                                                             \
    int cbk_cuda_##p##sytrfnp_compact_async(char layout, char uplo, int n, T *ap, int ldap,       \
                                            int V, int nm, cbk_stream_t st)                       \
    {                                                                                             \
        return factor<T>(true, layout, uplo, n, ap, ldap, V, nm, S(st));                          \
    }                                                                                             \
    int cbk_cuda_##p##sytrfnp_compact(char layout, char uplo, int n, T *ap, int ldap, int V,      \
                                      int nm)                                                     \
    {                                                                                             \
        return factor<T>(true, layout, uplo, n, ap, ldap, V, nm, 0);                              \
    }                                                                                             \
    int cbk_cuda_##p##potrs_compact_async(char layout, char uplo, int n, int nrhs, const T *ap,   \
                                          int ldap, T *bp, int ldbp, int V, int nm,               \
                                          cbk_stream_t st)                                        \
    {                                                                                             \
        return sym_solve<T>(false, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap, bp,   \
                            ldbp, V, nm, S(st));                                                  \
    }                                                                                             \
    int cbk_cuda_##p##potrs_compact(char layout, char uplo, int n, int nrhs, const T *ap,         \
                                    int ldap, T *bp, int ldbp, int V, int nm)                     \
    {                                                                                             \
        return sym_solve<T>(false, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap, bp,   \
                            ldbp, V, nm, 0);                                                      \
    }                                                                                             \
    int cbk_cuda_##p##posv_compact_async(char layout, char uplo, int n, int nrhs, T *ap,          \
                                         int ldap, T *bp, int ldbp, int V, int nm,                \
                                         cbk_stream_t st)                                         \
    {                                                                                             \
        return sym_solve<T>(false, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm,        \
                            S(st));                                                               \
    }                                                                                             \
    int cbk_cuda_##p##posv_compact(char layout, char uplo, int n, int nrhs, T *ap, int ldap,      \
                                   T *bp, int ldbp, int V, int nm)                                \
    {                                                                                             \
        return sym_solve<T>(false, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, 0);    \
    }                                                                                             \
    int cbk_cuda_##p##sytrsnp_compact_async(char layout, char uplo, int n, int nrhs,              \
                                            const T *ap, int ldap, T *bp, int ldbp, int V,        \
                                            int nm, cbk_stream_t st)                              \
    {                                                                                             \
        return sym_solve<T>(true, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap, bp,    \
                            ldbp, V, nm, S(st));                                                  \
    }                                                                                             \
    int cbk_cuda_##p##sytrsnp_compact(char layout, char uplo, int n, int nrhs, const T *ap,       \
                                      int ldap, T *bp, int ldbp, int V, int nm)                   \
    {                                                                                             \
        return sym_solve<T>(true, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap, bp,    \
                            ldbp, V, nm, 0);                                                      \
    }                                                                                             \
    int cbk_cuda_##p##sysvnp_compact_async(char layout, char uplo, int n, int nrhs, T *ap,        \
                                           int ldap, T *bp, int ldbp, int V, int nm,              \
                                           cbk_stream_t st)                                       \
    {                                                                                             \
        return sym_solve<T>(true, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, S(st)); \
    }                                                                                             \
    int cbk_cuda_##p##sysvnp_compact(char layout, char uplo, int n, int nrhs, T *ap, int ldap,    \
                                     T *bp, int ldbp, int V, int nm)                              \
    {                                                                                             \
        return sym_solve<T>(true, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, 0);     \
    }                                                                                             \
    int cbk_cuda_##p##trsm_compact_async(char layout, char side, char uplo, char transa,          \
                                         char diag, int m, int n, T alpha, const T *ap, int ldap, \
                                         T *bp, int ldbp, int V, int nm, cbk_stream_t st)         \
    {                                                                                             \
        return trsm<T>(layout, side, uplo, transa, diag, m, n, alpha, ap, ldap, bp, ldbp, V, nm,  \
                       S(st));                                                                    \
    }                                                                                             \
    int cbk_cuda_##p##trsm_compact(char layout, char side, char uplo, char transa, char diag,     \
                                   int m, int n, T alpha, const T *ap, int ldap, T *bp, int ldbp, \
                                   int V, int nm)                                                 \
    {                                                                                             \
        return trsm<T>(layout, side, uplo, transa, diag, m, n, alpha, ap, ldap, bp, ldbp, V, nm,  \
                       0);                                                                        \
    }                                                                                             \
    int cbk_cuda_##p##gels_compact_async(char layout, char trans, int m, int n, int nrhs, T *ap,  \
                                         int ldap, T *bp, int ldbp, T *taup, int V, int nm,       \
                                         cbk_stream_t st)                                         \
    {                                                                                             \
        return gels<T>(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, S(st));        \
    }                                                                                             \
    int cbk_cuda_##p##gels_compact(char layout, char trans, int m, int n, int nrhs, T *ap,        \
                                   int ldap, T *bp, int ldbp, T *taup, int V, int nm)             \
    {                                                                                             \
        return gels<T>(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, 0);            \
    }                                                                                             \
    int cbk_cuda_##p##pack_compact_async(char layout, int m, int n, const T *a, int lda,          \
                                         long long stridea, T *ap, int ldap, int V, int nm,       \
                                         T pad_diag, cbk_stream_t st)                             \
    {                                                                                             \
        return pack<T>(layout, m, n, a, lda, stridea, ap, ldap, V, nm, pad_diag, S(st));          \
    }                                                                                             \
    int cbk_cuda_##p##unpack_compact_async(char layout, int m, int n, const T *ap, int ldap,      \
                                           T *a, int lda, long long stridea, int V, int nm,       \
                                           cbk_stream_t st)                                       \
    {                                                                                             \
        return unpack<T>(layout, m, n, ap, ldap, a, lda, stridea, V, nm, S(st));                  \
    }

long long cbk_cuda_dposv_refined_compact_lwork(int n, int nrhs, int V, int nm)
{
    if (n < 0 || nrhs < 0 || !vlen_ok(V) || nm < 0) return -1;
    return (long long)posv_refined_lwork(n, nrhs, V, nm);
}

int cbk_cuda_dposv_refined_compact_async(char layout, char uplo, int n, int nrhs, double *ap,
                                         int ldap, double *bp, int ldbp, int V, int nm,
                                         int max_iter, int *iters, double *berr, void *work,
                                         long long lwork, cbk_stream_t st)
{
    return posv_refined(layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter, iters, berr,
                        work, lwork, S(st));
}

long long cbk_cuda_dposv_refined_batched_lwork(int n, int nrhs, int nm)
{
    if (n < 0 || nrhs < 0 || nm < 0) return -1;
    return (long long)posv_refined_lwork(n, nrhs, 1, nm);
}

int cbk_cuda_dposv_refined_batched_async(char uplo, int n, int nrhs, double *a, int lda,
                                         long long stride_a, double *b, int ldb,
                                         long long stride_b, int nm, int max_iter, int *iters,
                                         double *berr, void *work, long long lwork,
                                         cbk_stream_t st)
{
    return posv_refined_batched(uplo, n, nrhs, a, lda, stride_a, b, ldb, stride_b, nm, max_iter,
                                iters, berr, work, lwork, S(st));
}

#define CBK_PLAIN_BATCHED(P, T)                                                                    \
    int cbk_cuda_##P##posv_batched_async(char uplo, int n, int nrhs, T *a, int lda,                \
                                         long long stride_a, T *b, int ldb, long long stride_b,    \
                                         int nm, cbk_stream_t st)                                  \
    {                                                                                              \
        return sym_solve_batched<T>(false, uplo, n, nrhs, a, lda, stride_a, b, ldb, stride_b, nm,  \
                                    S(st));                                                        \
    }                                                                                              \
    int cbk_cuda_##P##sysvnp_batched_async(char uplo, int n, int nrhs, T *a, int lda,              \
                                           long long stride_a, T *b, int ldb, long long stride_b,  \
                                           int nm, cbk_stream_t st)                                \
    {                                                                                              \
        return sym_solve_batched<T>(true, uplo, n, nrhs, a, lda, stride_a, b, ldb, stride_b, nm,   \
                                    S(st));                                                        \
    }                                                                                              \
    int cbk_cuda_##P##gels_batched_async(char trans, int m, int n, int nrhs, T *a, int lda,        \
                                         long long stride_a, T *b, int ldb, long long stride_b,    \
                                         T *tau, int nm, cbk_stream_t st)                          \
    {                                                                                              \
        return gels_batched<T>(trans, m, n, nrhs, a, lda, stride_a, b, ldb, stride_b, tau, nm,     \
                               S(st));                                                             \
    }
CBK_PLAIN_BATCHED(d, double)
CBK_PLAIN_BATCHED(s, float)
#undef CBK_PLAIN_BATCHED

long long cbk_cuda_dposv_refined_compact_host_lwork(char layout, int n, int nrhs, int ldap,
                                                    int ldbp, int V, int nm)
{
    const bool col = opt(layout, 'C'), row = opt(layout, 'R');
    if ((!col && !row) || n < 0 || nrhs < 0 || ldap < max1(n) ||
        ldbp < max1(row ? nrhs : n) || !vlen_ok(V) || nm < 0)
        return -1;
    return (long long)posv_refined_host_lwork(row, n, nrhs, ldap, ldbp, V, nm);
}

int cbk_cuda_dposv_refined_compact_host(char layout, char uplo, int n, int nrhs, double *ap,
                                        int ldap, double *bp, int ldbp, int V, int nm,
                                        int max_iter, int *iters, double *berr, void *dwork,
                                        long long lwork, cbk_stream_t stream)
{
    bool row, up;
    if (int e = sym_solve_args(layout, uplo, n, nrhs, ldap, ldbp, V, nm, row, up)) return e;
    if (max_iter < 0) return -11;
    if (n == 0 || nm == 0 || nrhs == 0) return 0;
    const size_t need = posv_refined_host_lwork(row, n, nrhs, ldap, ldbp, V, nm);
    if (dwork == nullptr || lwork < (long long)need) return -15;
    return cuda_status(posv_refined_host(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter,
                                         iters, berr, dwork, S(stream)));
}

// The refined solve for callers that cannot allocate: scratch from the
// library's fixed array; a batch whose scratch would not fit is rejected as an
// illegal nm (-10).
int cbk_cuda_dposv_refined_compact_noalloc_async(char layout, char uplo, int n, int nrhs,
                                                 double *ap, int ldap, double *bp, int ldbp, int V,
                                                 int nm, int max_iter, int *iters, double *berr,
                                                 cbk_stream_t st)
{
    bool row, up;
    if (int e = sym_solve_args(layout, uplo, n, nrhs, ldap, ldbp, V, nm, row, up)) return e;
    if (max_iter < 0) return -11;
    if (n == 0 || nm == 0 || nrhs == 0) return 0;
    if (posv_refined_lwork(n, nrhs, V, nm) > (size_t)CBK_CUDA_NOALLOC_SCRATCH_BYTES)
        return CBK_CUDA_NOALLOC_TOO_LARGE;
    return launch_posv_refined_noalloc(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter,
                                       iters, berr, S(st));
}

long long cbk_cuda_dgels_refined_compact_lwork(int m, int n, int nrhs, int V, int nm)
{
    if (m < 0 || n < 0 || nrhs < 0 || !vlen_ok(V) || nm < 0) return -1;
    return (long long)gels_refined_lwork(m, n, nrhs, V, nm);
}

int cbk_cuda_dgels_refined_compact_async(char layout, char trans, int m, int n, int nrhs,
                                         double *ap, int ldap, double *bp, int ldbp,
                                         double *taup, int V, int nm, int max_iter, int *iters,
                                         double *berr, void *work, long long lwork,
                                         cbk_stream_t st)
{
    return gels_refined(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, max_iter,
                        iters, berr, work, lwork, S(st));
}

long long cbk_cuda_dgels_refined_batched_lwork(int m, int n, int nrhs, int nm)
{
    if (m < 0 || n < 0 || nrhs < 0 || nm < 0) return -1;
    return (long long)gels_refined_lwork(m, n, nrhs, 1, nm);
}

int cbk_cuda_dgels_refined_batched_async(char trans, int m, int n, int nrhs, double *a, int lda,
                                         long long stride_a, double *b, int ldb,
                                         long long stride_b, double *tau, int nm, int max_iter,
                                         int *iters, double *berr, void *work, long long lwork,
                                         cbk_stream_t st)
{
    return gels_refined_batched(trans, m, n, nrhs, a, lda, stride_a, b, ldb, stride_b, tau, nm,
                                max_iter, iters, berr, work, lwork, S(st));
}

int cbk_cuda_dsysvnp_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_dbucket *buckets, void *work,
                                            long long lwork, cbk_stream_t st)
{
    return bucketed<double>(true, layout, uplo, nrhs, nbuckets, buckets, work, lwork, S(st));
}
int cbk_cuda_ssysvnp_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_sbucket *buckets, void *work,
                                            long long lwork, cbk_stream_t st)
{
    return bucketed<float>(true, layout, uplo, nrhs, nbuckets, buckets, work, lwork, S(st));
}
int cbk_cuda_dposv_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                          const cbk_cuda_dbucket *buckets, void *work,
                                          long long lwork, cbk_stream_t st)
{
    return bucketed<double>(false, layout, uplo, nrhs, nbuckets, buckets, work, lwork, S(st));
}
int cbk_cuda_sposv_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                          const cbk_cuda_sbucket *buckets, void *work,
                                          long long lwork, cbk_stream_t st)
{
    return bucketed<float>(false, layout, uplo, nrhs, nbuckets, buckets, work, lwork, S(st));
}

struct cbk_cuda_graph_st {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

int cbk_cuda_dsysvnp_compact_bucketed_graph(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_dbucket *buckets, void *work,
                                            long long lwork, cbk_cuda_graph *graph)
{
    if (graph == nullptr) return -8;
    *graph = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return cuda_status(e);
    }
    const int info = bucketed<double>(true, layout, uplo, nrhs, nbuckets, buckets, work, lwork, s);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    cudaStreamDestroy(s);
    if (info != 0) {
        if (g) cudaGraphDestroy(g);
        return info;
    }
    if (e != cudaSuccess) return cuda_status(e);
    cudaGraphExec_t x = nullptr;
    e = cudaGraphInstantiate(&x, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_status(e);
    }
    *graph = new cbk_cuda_graph_st{g, x};
    return 0;
}

int cbk_cuda_graph_launch(cbk_cuda_graph graph, cbk_stream_t st)
{
    if (graph == nullptr) return -1;
    return cuda_status(cudaGraphLaunch(graph->exec, S(st)));
}

int cbk_cuda_graph_destroy(cbk_cuda_graph graph)
{
    if (graph == nullptr) return 0;
    cudaError_t e1 = cudaGraphExecDestroy(graph->exec);
    cudaError_t e2 = cudaGraphDestroy(graph->graph);
    delete graph;
    return cuda_status(e1 != cudaSuccess ? e1 : e2);
}

CBK_CUDA_ENTRY_POINTS(double, d)
CBK_CUDA_ENTRY_POINTS(float, s)

#undef CBK_CUDA_ENTRY_POINTS


// The host-pointer forms, one per routine and scalar type.
#define CBK_CUDA_HOST_ENTRY_POINTS(T, p)                                                          \
    int cbk_cuda_host_##p##geqrf_compact(char layout, int m, int n, T *ap, int ldap, T *taup,    \
                                         int V, int nm, void *dwork, long long *lwork,            \
                                         cbk_stream_t st)                                         \
    {                                                                                             \
        return host_geqrf<T>(layout, m, n, ap, ldap, taup, V, nm, dwork, lwork, S(st));           \
    }                                                                                             \
    int cbk_cuda_host_##p##ormqr_compact(char layout, char side, char trans, int m, int n, int k, \
                                         const T *ap, int ldap, const T *taup, T *cp, int ldcp,   \
                                         int V, int nm, void *dwork, long long *lwork,            \
                                         cbk_stream_t st)                                         \
    {                                                                                             \
        return host_ormqr<T>(layout, side, trans, m, n, k, ap, ldap, taup, cp, ldcp, V, nm,       \
                             dwork, lwork, S(st));                                                \
    }                                                                                             \
    int cbk_cuda_host_##p##orgqr_compact(char layout, int m, int n, int k, T *ap, int ldap,       \
                                         const T *taup, int V, int nm, void *dwork,               \
                                         long long *lwork, cbk_stream_t st)                       \
    {                                                                                             \
        return host_orgqr<T>(layout, m, n, k, ap, ldap, taup, V, nm, dwork, lwork, S(st));        \
    }                                                                                             \
    int cbk_cuda_host_##p##potrf_compact(char layout, char uplo, int n, T *ap, int ldap, int V,   \
                                         int nm, void *dwork, long long *lwork, cbk_stream_t st)  \
    {                                                                                             \
        return host_factor<T>(false, layout, uplo, n, ap, ldap, V, nm, dwork, lwork, S(st));      \
    }                                                                                             \
    int cbk_cuda_host_##p##sytrfnp_compact(char layout, char uplo, int n, T *ap, int ldap, int V, \
                                           int nm, void *dwork, long long *lwork,                 \
                                           cbk_stream_t st)                                       \
    {                                                                                             \
        return host_factor<T>(true, layout, uplo, n, ap, ldap, V, nm, dwork, lwork, S(st));       \
    }                                                                                             \
    int cbk_cuda_host_##p##potrs_compact(char layout, char uplo, int n, int nrhs, const T *ap,    \
                                         int ldap, T *bp, int ldbp, int V, int nm, void *dwork,   \
                                         long long *lwork, cbk_stream_t st)                       \
    {                                                                                             \
        return host_sym_solve<T>(false, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap,  \
                                 bp, ldbp, V, nm, dwork, lwork, S(st));                           \
    }                                                                                             \
    int cbk_cuda_host_##p##posv_compact(char layout, char uplo, int n, int nrhs, T *ap, int ldap, \
                                        T *bp, int ldbp, int V, int nm, void *dwork,              \
                                        long long *lwork, cbk_stream_t st)                        \
    {                                                                                             \
        return host_sym_solve<T>(false, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm,   \
                                 dwork, lwork, S(st));                                            \
    }                                                                                             \
    int cbk_cuda_host_##p##sytrsnp_compact(char layout, char uplo, int n, int nrhs, const T *ap,  \
                                           int ldap, T *bp, int ldbp, int V, int nm, void *dwork, \
                                           long long *lwork, cbk_stream_t st)                     \
    {                                                                                             \
        return host_sym_solve<T>(true, false, layout, uplo, n, nrhs, const_cast<T *>(ap), ldap,   \
                                 bp, ldbp, V, nm, dwork, lwork, S(st));                           \
    }                                                                                             \
    int cbk_cuda_host_##p##sysvnp_compact(char layout, char uplo, int n, int nrhs, T *ap,         \
                                          int ldap, T *bp, int ldbp, int V, int nm, void *dwork,  \
                                          long long *lwork, cbk_stream_t st)                      \
    {                                                                                             \
        return host_sym_solve<T>(true, true, layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm,    \
                                 dwork, lwork, S(st));                                            \
    }                                                                                             \
    int cbk_cuda_host_##p##trsm_compact(char layout, char side, char uplo, char transa,          \
                                        char diag, int m, int n, T alpha, const T *ap, int ldap,  \
                                        T *bp, int ldbp, int V, int nm, void *dwork,              \
                                        long long *lwork, cbk_stream_t st)                        \
    {                                                                                             \
        return host_trsm<T>(layout, side, uplo, transa, diag, m, n, alpha, ap, ldap, bp, ldbp, V, \
                            nm, dwork, lwork, S(st));                                             \
    }                                                                                             \
    int cbk_cuda_host_##p##gels_compact(char layout, char trans, int m, int n, int nrhs, T *ap,   \
                                        int ldap, T *bp, int ldbp, T *taup, int V, int nm,        \
                                        void *dwork, long long *lwork, cbk_stream_t st)           \
    {                                                                                             \
        return host_gels<T>(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm, dwork,    \
                            lwork, S(st));                                                        \
    }

CBK_CUDA_HOST_ENTRY_POINTS(double, d)
CBK_CUDA_HOST_ENTRY_POINTS(float, s)
#undef CBK_CUDA_HOST_ENTRY_POINTS

} // extern "C"
