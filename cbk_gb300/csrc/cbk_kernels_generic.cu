// cbk_kernels_generic.cu -- the lane-per-matrix kernels for every routine,
// any order, layout, triangle, side and transpose (the complete drop-in
// surface). The small-order Cholesky kernels with the matrix held in
// registers live in cbk_kernels_chol_reg.cu and take over where they apply.
#include "cbk_device.cuh"
#include "cbk_launch.h"

namespace cbkcuda {
using namespace cbkdev;

namespace {

inline unsigned blocks_for(long ngroups, int V, int threads)
{
    const long lanes = ngroups * (long)V;
    return (unsigned)((lanes + threads - 1) / threads);
}
inline long groups_of(int nm, int V)
{
    return ((long)nm + V - 1) / V;
}

template <typename T>
__global__ void k_zero(bool row, int rows, int cols, T *bp, int ldbp, int V, long ngroups,
                       size_t sb)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    zero_lane<T>(lv_make<T>(bp + ln.g * sb + ln.v, row, ldbp, V, rows, cols), 0, rows, cols);
}

template <typename T, bool LDLT>
__global__ void k_factor(bool row, bool up, int n, T *ap, int ldap, int V, long ngroups, size_t sa)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    LV<T> A = lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, n, n);
    if (up) A = A.t();
    factor_lane<T, LDLT>(n, A);
}

template <typename T, bool LDLT, bool FUSED>
__global__ void k_sym_solve(bool row, bool up, int n, int nrhs, T *ap, int ldap, T *bp, int ldbp,
                            int V, long ngroups, size_t sa, size_t sb)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    LV<T> A = lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, n, n);
    if (up) A = A.t();
    if (FUSED) factor_lane<T, LDLT>(n, A);
    sym_solve_lane<T, LDLT>(n, nrhs, A, lv_make<T>(bp + ln.g * sb + ln.v, row, ldbp, V, n, nrhs));
}

template <typename T>
__global__ void k_trsm(bool left, bool up, bool row, bool tran, bool unit, int m, int n, T alpha,
                       const T *ap, int ldap, T *bp, int ldbp, int V, long ngroups, size_t sa,
                       size_t sb)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    const int s = left ? m : n;
    const LV<T> A = lv_make<T>(const_cast<T *>(ap) + ln.g * sa + ln.v, row, ldap, V, s, s);
    trsm_lane<T>(left, up, tran, unit, m, n, alpha, A,
                 lv_make<T>(bp + ln.g * sb + ln.v, row, ldbp, V, m, n));
}

template <typename T, bool WY>
__global__ void k_geqrf(bool row, int m, int n, T *ap, int ldap, T *taup, int V, long ngroups,
                        size_t sa, size_t st)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    geqrf_lane<T, WY>(m, n, lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, m, n),
                  taup + ln.g * st + ln.v, V);
}

template <typename T, bool WY>
__global__ void k_ormqr(bool left, bool row, bool forward, int m, int n, int k, const T *ap,
                        int ldap, const T *taup, T *cp, int ldcp, int V, long ngroups, size_t sa,
                        size_t st, size_t sc)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    const LV<T> A =
        lv_make<T>(const_cast<T *>(ap) + ln.g * sa + ln.v, row, ldap, V, left ? m : n, k);
    LV<T> C = lv_make<T>(cp + ln.g * sc + ln.v, row, ldcp, V, m, n);
    if (!left) C = C.t();
    ormqr_lane<T, WY>(forward, left ? m : n, left ? n : m, k, A, taup + ln.g * st + ln.v, V, C);
}

template <typename T>
__global__ void k_orgqr(bool row, int m, int n, int k, T *ap, int ldap, const T *taup, int V,
                        long ngroups, size_t sa, size_t st)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    orgqr_lane<T>(m, n, k, lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, m, n),
                  taup + ln.g * st + ln.v, V);
}

template <typename T, bool WY>
__global__ void k_gels(bool row, bool tall, bool overdet, int p, int q, int nrhs, T *ap, int ldap,
                       T *bp, int ldbp, T *taup, int V, long ngroups, size_t sa, size_t sb,
                       size_t st)
{
    Lane ln;
    if (!lane_of(ngroups, V, ln)) return;
    LV<T> A = lv_make<T>(ap + ln.g * sa + ln.v, row, ldap, V, tall ? p : q, tall ? q : p);
    if (!tall) A = A.t();
    gels_lane<T, WY>(overdet, p, q, nrhs, A, taup + ln.g * st + ln.v, V,
                 lv_make<T>(bp + ln.g * sb + ln.v, row, ldbp, V, p, nrhs));
}

} // namespace

template <typename T>
cudaError_t launch_zero(bool row, int rows, int cols, T *bp, int ldbp, int V, int nm,
                        cudaStream_t s, size_t sb_)
{
    const long ng = groups_of(nm, V);
    const int th = threads_for(R_ZERO, rows, sizeof(T));
    k_zero<T><<<blocks_for(ng, V, th), th, 0, s>>>(row, rows, cols, bp, ldbp, V, ng,
                                                   sb_ ? sb_ : gstride(row, ldbp, rows, cols, V));
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_factor(bool ldlt, bool row, bool up, int n, T *ap, int ldap, int V, int nm,
                          cudaStream_t s, size_t sa_)
{
    const long ng = groups_of(nm, V);
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, n, n, V);
    if (!ldlt && chol_small_ok(n))
        return launch_chol_small<T>(false, row, up, n, 0, ap, ldap, nullptr, 1, V, nm, s, sa);
    const int th = threads_for(ldlt ? R_SYTRFNP : R_POTRF, n, sizeof(T));
    if (ldlt)
        k_factor<T, true><<<blocks_for(ng, V, th), th, 0, s>>>(row, up, n, ap, ldap, V, ng, sa);
    else
        k_factor<T, false><<<blocks_for(ng, V, th), th, 0, s>>>(row, up, n, ap, ldap, V, ng, sa);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sym_solve_generic(bool ldlt, bool fused, bool row, bool up, int n, int nrhs,
                                     T *ap, int ldap, T *bp, int ldbp, int V, int nm,
                                     cudaStream_t s, size_t sa_ = 0, size_t sb_ = 0)
{
    const long ng = groups_of(nm, V);
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, n, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, n, nrhs, V);
    const int r = ldlt ? (fused ? R_SYSVNP : R_SYTRSNP) : (fused ? R_POSV : R_POTRS);
    const int th = threads_for(r, n, sizeof(T));
    const unsigned bl = blocks_for(ng, V, th);
#define CBK_SOLVE_LAUNCH(L, F)                                                                    \
    k_sym_solve<T, L, F><<<bl, th, 0, s>>>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, ng, sa, sb)
    if (ldlt) {
        if (fused) CBK_SOLVE_LAUNCH(true, true);
        else CBK_SOLVE_LAUNCH(true, false);
    }
    else {
        if (fused) CBK_SOLVE_LAUNCH(false, true);
        else CBK_SOLVE_LAUNCH(false, false);
    }
#undef CBK_SOLVE_LAUNCH
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trsm(bool left, bool up, bool row, bool tran, bool unit, int m, int n, T alpha,
                        const T *ap, int ldap, T *bp, int ldbp, int V, int nm, cudaStream_t s)
{
    const long ng = groups_of(nm, V);
    const int sdim = left ? m : n;
    const int th = threads_for(R_TRSM, sdim, sizeof(T));
    k_trsm<T><<<blocks_for(ng, V, th), th, 0, s>>>(left, up, row, tran, unit, m, n, alpha, ap, ldap,
                                                   bp, ldbp, V, ng,
                                                   gstride(row, ldap, sdim, sdim, V),
                                                   gstride(row, ldbp, m, n, V));
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_geqrf(bool row, int m, int n, T *ap, int ldap, T *taup, int V, int nm,
                         cudaStream_t s)
{
    const long ng = groups_of(nm, V);
    const int k = m < n ? m : n;
    const int th = threads_for(R_GEQRF, m, sizeof(T));
    // the compact-WY kernel from WY_MMIN rows on (its extra registers would
    // cost the one-at-a-time kernel occupancy)
    auto kern = m >= WY_MMIN ? k_geqrf<T, true> : k_geqrf<T, false>;
    kern<<<blocks_for(ng, V, th), th, 0, s>>>(row, m, n, ap, ldap, taup, V, ng,
                                              gstride(row, ldap, m, n, V), (size_t)k * V);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ormqr(bool left, bool row, bool tran, int m, int n, int k, const T *ap,
                         int ldap, const T *taup, T *cp, int ldcp, int V, int nm, cudaStream_t s)
{
    const long ng = groups_of(nm, V);
    const int len = left ? m : n;
    const bool forward = (left == tran);
    const int th = threads_for(R_ORMQR, len, sizeof(T));
    auto kern = len >= WY_MMIN ? k_ormqr<T, true> : k_ormqr<T, false>;
    kern<<<blocks_for(ng, V, th), th, 0, s>>>(left, row, forward, m, n, k, ap, ldap, taup, cp, ldcp,
                                              V, ng, gstride(row, ldap, len, k, V), (size_t)k * V,
                                              gstride(row, ldcp, m, n, V));
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_orgqr(bool row, int m, int n, int k, T *ap, int ldap, const T *taup, int V,
                         int nm, cudaStream_t s)
{
    const long ng = groups_of(nm, V);
    const int th = threads_for(R_ORGQR, m, sizeof(T));
    k_orgqr<T><<<blocks_for(ng, V, th), th, 0, s>>>(row, m, n, k, ap, ldap, taup, V, ng,
                                                    gstride(row, ldap, m, n, V), (size_t)k * V);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gels(bool row, bool tran, int m, int n, int nrhs, T *ap, int ldap, T *bp,
                        int ldbp, T *taup, int V, int nm, cudaStream_t s, size_t sa_, size_t sb_)
{
    const long ng = groups_of(nm, V);
    const bool tall = m >= n;
    const int p = tall ? m : n, q = tall ? n : m;
    const bool overdet = (tall != tran);
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, m, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, p, nrhs, V);
    if (q == 0) return launch_zero<T>(row, p, nrhs, bp, ldbp, V, nm, s, sb);
    const int th = threads_for(R_GELS, p, sizeof(T));
    auto kern = p >= WY_MMIN ? k_gels<T, true> : k_gels<T, false>;
    kern<<<blocks_for(ng, V, th), th, 0, s>>>(row, tall, overdet, p, q, nrhs, ap, ldap, bp, ldbp,
                                              taup, V, ng, sa, sb, (size_t)q * V);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sym_solve(bool ldlt, bool fused, bool row, bool up, int n, int nrhs, T *ap,
                             int ldap, T *bp, int ldbp, int V, int nm, cudaStream_t s,
                             size_t sa_, size_t sb_)
{
    if (!ldlt && fused && chol_small_ok(n))
        return launch_chol_small<T>(true, row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, s, sa_,
                                    sb_);
    return launch_sym_solve_generic<T>(ldlt, fused, row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm,
                                       s, sa_, sb_);
}

#define CBK_INSTANTIATE(T)                                                                        \
    template cudaError_t launch_zero<T>(bool, int, int, T *, int, int, int, cudaStream_t, size_t); \
    template cudaError_t launch_factor<T>(bool, bool, bool, int, T *, int, int, int,               \
                                          cudaStream_t, size_t);                                  \
    template cudaError_t launch_sym_solve_generic<T>(bool, bool, bool, bool, int, int, T *, int,   \
                                                     T *, int, int, int, cudaStream_t, size_t,    \
                                                     size_t);                                     \
    template cudaError_t launch_sym_solve<T>(bool, bool, bool, bool, int, int, T *, int, T *, int, \
                                             int, int, cudaStream_t, size_t, size_t);             \
    template cudaError_t launch_trsm<T>(bool, bool, bool, bool, bool, int, int, T, const T *, int, \
                                        T *, int, int, int, cudaStream_t);                        \
    template cudaError_t launch_geqrf<T>(bool, int, int, T *, int, T *, int, int, cudaStream_t);   \
    template cudaError_t launch_ormqr<T>(bool, bool, bool, int, int, int, const T *, int,          \
                                         const T *, T *, int, int, int, cudaStream_t);            \
    template cudaError_t launch_orgqr<T>(bool, int, int, int, T *, int, const T *, int, int,       \
                                         cudaStream_t);                                           \
    template cudaError_t launch_gels<T>(bool, bool, int, int, int, T *, int, T *, int, T *, int,   \
                                        int, cudaStream_t, size_t, size_t);
CBK_INSTANTIATE(float)
CBK_INSTANTIATE(double)
#undef CBK_INSTANTIATE

} // namespace cbkcuda
