// cbk_launch.h -- internal interface between the C-ABI layer (cbk_api.cpp)
// and the CUDA kernels. Not installed; include/cbk_cuda.h is the public ABI.
//
// Every launcher enqueues its kernel(s) on `stream` and returns the CUDA
// error of the launch (cudaSuccess when it was queued). Arguments are already
// validated by the caller; nm >= 1 and every extent the kernel reads is >= 1.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace cbkcuda {

// Threads per block of the lane-per-matrix kernels (the autotuner may change
// it per routine and order; 0 selects the built-in default).
int threads_for(int routine, int n, int dsize);
// the same with the built-in choice dflt
int threads_or(int routine, int n, int dsize, int dflt);
void set_threads(int routine, int n, int dsize, int threads);

// Compiled shape of a kernel that has several (0 = the built-in default):
// 0 .. 3 for the warp-per-matrix refined solve (four matrices per block at
// two register caps, two matrices, one matrix), the least squares' kernel
// choice; 0 .. 3 for the bucketed launch (the persistent grid's warps per SM
// halved `variant` times).
constexpr int MAX_VARIANTS = 4;
int variant_for(int routine, int n, int dsize);
void set_variant(int routine, int n, int dsize, int variant);
// the interleave width measured fastest (0: untuned)
int vlen_for(int routine, int n, int dsize);
void set_vlen(int routine, int n, int dsize, int V);
// routine names of the tuning API ("posv", "posv_refined", ...) <-> Routine
int routine_of(const char *name);
const char *routine_name(int routine);
int tune_slots();

enum Routine {
    R_POTRF = 0, R_SYTRFNP, R_POTRS, R_POSV, R_SYTRSNP, R_SYSVNP, R_TRSM, R_GEQRF, R_ORMQR,
    R_ORGQR, R_GELS, R_ZERO, R_PACK, R_UNPACK, R_POSV_REFINED, R_GELS_REFINED, R_SYSVNP_BUCKETED,
    R_POSV_BUCKETED, R_COUNT
};

// every group of a rows x cols batch := 0
template <typename T>
cudaError_t launch_zero(bool row, int rows, int cols, T *bp, int ldbp, int V, int nm,
                        cudaStream_t s, size_t sb_ = 0);

// potrf (ldlt = false) / sytrfnp (ldlt = true) of the named triangle
template <typename T>
cudaError_t launch_factor(bool ldlt, bool row, bool up, int n, T *ap, int ldap, int V, int nm,
                          cudaStream_t s, size_t sa_ = 0);

// Cholesky factor (+ solve when `solve`) of orders 1 .. CHOL_SMALL_NMAX with the
// matrix in registers (cbk_kernels_chol_reg.cu): the generic kernels' bits
constexpr int CHOL_SMALL_NMAX = 8;
bool chol_small_ok(int n);
template <typename T>
cudaError_t launch_chol_small(bool solve, bool row, bool up, int n, int nrhs, T *ap, int ldap,
                              T *bp, int ldbp, int V, int nm, cudaStream_t s, size_t sa_ = 0,
                              size_t sb_ = 0);

// potrs / posv (ldlt = false), sytrsnp / sysvnp (ldlt = true); fused = factor first.
// sa_ / sb_: group strides of A and B (0: the compact layout's); a strided
// dense batch is the compact layout at V = 1 with the caller's strides
template <typename T>
cudaError_t launch_sym_solve(bool ldlt, bool fused, bool row, bool up, int n, int nrhs, T *ap,
                             int ldap, T *bp, int ldbp, int V, int nm, cudaStream_t s,
                             size_t sa_ = 0, size_t sb_ = 0);

template <typename T>
cudaError_t launch_trsm(bool left, bool up, bool row, bool tran, bool unit, int m, int n, T alpha,
                        const T *ap, int ldap, T *bp, int ldbp, int V, int nm, cudaStream_t s);

template <typename T>
cudaError_t launch_geqrf(bool row, int m, int n, T *ap, int ldap, T *taup, int V, int nm,
                         cudaStream_t s);

template <typename T>
cudaError_t launch_ormqr(bool left, bool row, bool tran, int m, int n, int k, const T *ap,
                         int ldap, const T *taup, T *cp, int ldcp, int V, int nm, cudaStream_t s);

template <typename T>
cudaError_t launch_orgqr(bool row, int m, int n, int k, T *ap, int ldap, const T *taup, int V,
                         int nm, cudaStream_t s);

template <typename T>
cudaError_t launch_gels(bool row, bool tran, int m, int n, int nrhs, T *ap, int ldap, T *bp,
                        int ldbp, T *taup, int V, int nm, cudaStream_t s, size_t sa_ = 0,
                        size_t sb_ = 0);

// dense batch (matrix idx at a + idx*stride, element (i,j) at i + j*lda
// column-major or i*lda + j row-major) <-> compact; padded lanes get pad_diag
template <typename T>
cudaError_t launch_pack(bool row, int m, int n, const T *a, int lda, long long stride, T *ap,
                        int ldap, int V, int nm, T pad_diag, cudaStream_t s);
template <typename T>
cudaError_t launch_unpack(bool row, int m, int n, const T *ap, int ldap, T *a, int lda,
                          long long stride, int V, int nm, cudaStream_t s);

// mixed-precision SPD solve (cbk_kernels_refine.cu)
size_t posv_refined_lwork(int n, int nrhs, int V, int nm);
// sa_ / sb_: the scalars from one group of A / B to the next; 0 takes the
// compact layout's own (a dense batch is V = 1 with the caller's strides)
cudaError_t launch_posv_refined(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                double *bp, int ldbp, int V, int nm, int max_iter, int *iters,
                                double *berr, void *work, cudaStream_t s, size_t sa_ = 0,
                                size_t sb_ = 0);
// mixed-precision least squares (cbk_kernels_refine_gels.cu)
size_t gels_refined_lwork(int m, int n, int nrhs, int V, int nm);
int gels_refined_nmax();
// the warp-per-matrix refined least squares (m <= 64, n in {8, 16})
bool gels_refined_warp_ok(int m, int n);
cudaError_t launch_gels_refined_warp(bool row, int m, int n, int nrhs, double *ap, int ldap,
                                     double *bp, int ldbp, double *taup, int V, int nm,
                                     int max_iter, int *iters, double *berr, cudaStream_t s,
                                     size_t sa = 0, size_t sb = 0);
cudaError_t launch_gels_refined(bool row, int m, int n, int nrhs, double *ap, int ldap, double *bp,
                                int ldbp, double *taup, int V, int nm, int max_iter, int *iters,
                                double *berr, void *work, cudaStream_t s, size_t sa_ = 0,
                                size_t sb_ = 0);

// one persistent launch over a table of single-order compact buckets
// (cbk_kernels_bucketed.cu); work holds the 8-byte item counter
template <typename T>
cudaError_t launch_bucketed(bool ldlt, bool row, bool up, int nrhs, int nbuckets, const int *n,
                            const int *nm, const int *V, T *const *ap, const int *ldap,
                            T *const *bp, const int *ldbp, void *work, cudaStream_t s);

// orders 17 .. 64: one warp per matrix, no workspace (cbk_kernels_refine_warp.cu)
bool posv_refined_warp_ok(int n);
cudaError_t launch_posv_refined_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                     double *bp, int ldbp, int V, int nm, int max_iter,
                                     int *iters, double *berr, cudaStream_t s, size_t sa_ = 0,
                                     size_t sb_ = 0);
// the same with two (wpb = 2) or one (wpb = 1) matrices per block
// (cbk_kernels_refine_warp_small.cu); sa, sb: the group strides
cudaError_t launch_posv_refined_warp_small(int wpb, bool row, bool up, int n, int nrhs,
                                           double *ap, int ldap, double *bp, int ldbp, int V,
                                           int nm, int max_iter, int *iters, double *berr,
                                           cudaStream_t s, size_t sa, size_t sb);

// the refined solve on host-memory batches, copies pipelined with the solves
// (cbk_host.cpp); dwork: device workspace of posv_refined_host_lwork bytes
size_t posv_refined_host_lwork(bool row, int n, int nrhs, int ldap, int ldbp, int V, int nm);
cudaError_t posv_refined_host(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                              int ldbp, int V, int nm, int max_iter, int *iters, double *berr,
                              void *dwork, cudaStream_t caller);
// the referenced triangle of `groups` compact groups of n x n matrices
// (leading dimension ld, group stride ld n V), src -> dst in place
// (cbk_kernels_pack.cu); either pointer may be device-addressable host memory
cudaError_t launch_tri_copy(bool row, bool up, int n, int ld, int V, long groups,
                            const double *src, double *dst, cudaStream_t s);
// *count += the number of negative entries of iters[0 .. n)
cudaError_t launch_count_negative(const int *iters, int n, int *count, cudaStream_t s);

// the same with the library's own scratch array (no allocation, no
// workspace); returns 0, CBK_CUDA_NOALLOC_IN_CAPTURE or CBK_CUDA_ERROR_BASE +
// a CUDA error
int launch_posv_refined_noalloc(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                double *bp, int ldbp, int V, int nm, int max_iter, int *iters,
                                double *berr, cudaStream_t s);

} // namespace cbkcuda
