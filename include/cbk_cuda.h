#ifndef CBK_CUDA_H
#define CBK_CUDA_H

/* cbk_cuda.h -- the compact batch kernels on an NVIDIA GB300 (sm_103a): the
 * C ABI of libcbk_cuda.so.
 *
 * A drop-in for ivan-pi/cbk v0.2.0's include/cbk.h: every routine there has a
 * counterpart here with the same argument list, the same meaning of each
 * argument, the same LAPACK-style checks returning -j for an illegal j-th
 * argument (checked in argument order, before any device work), the same
 * quick returns and the same in-place results -- with three differences:
 *
 *  1. The array arguments are DEVICE pointers (cudaMalloc'd or managed
 *     memory, or device views of host-registered memory).
 *  2. Work is enqueued on a CUDA stream: the plain name uses the legacy
 *     default stream (stream 0), the _async variant takes the stream. Like
 *     cuBLAS, calls return once the work is queued; the results are ready
 *     when the stream is synchronised. A CUDA error at launch is returned as
 *     CBK_CUDA_ERROR_BASE + the cudaError_t code (always > 0).
 *  3. The interleave width V may also be any multiple of 32 up to 1024 (32
 *     lanes of a warp then read element (i,j) of 32 matrices as one coalesced
 *     access); the reference's widths 2, 4, 8 and 16 remain valid.
 *
 * Compact layout (include/cbk.h:22-29 of the reference); group g = idx/V,
 * slot v = idx%V:
 *   A_v(i,j)  = ap [ g*ldap*ncol*V + (j*ldap + i)*V + v ]   (column-major)
 *   tau_v(kk) = taup[ g*k*V         +  kk*V          + v ]
 *   B_v(i,j)  = bp [ g*ldbp*nrhs*V  + (j*ldbp + i)*V + v ]
 * Row-major swaps the in-matrix index roles (i*ld + j). Every lane of every
 * group is computed, the padded lanes of a partial last group included, as
 * the reference does: pack them with the identity (tau with zero).
 *
 * The routines never abort and never allocate: the caller owns every buffer.
 * Numerical failure (a non-SPD lane, a zero pivot, a rank-deficient R) gives
 * Inf/NaN confined to that lane, as in the reference.
 */

#ifdef __cplusplus
extern "C" {
#endif

#define CBK_CUDA_VERSION_MAJOR 0
#define CBK_CUDA_VERSION_MINOR 2
#define CBK_CUDA_VERSION_PATCH 0
#define CBK_CUDA_VERSION                                                                 \
    (CBK_CUDA_VERSION_MAJOR * 10000 + CBK_CUDA_VERSION_MINOR * 100 + CBK_CUDA_VERSION_PATCH)

/* A CUDA launch failure is reported as this base plus the cudaError_t. */
#define CBK_CUDA_ERROR_BASE 1000

/* Same type as cudaStream_t; 0 is the legacy default stream. */
typedef struct CUstream_st *cbk_stream_t;

/* Replaces cbk_get_version (include/cbk.h:76-77, src/cbk.cpp:36-39): the version
 * of the API implemented, encoded as CBK_VERSION is (0.2.0 -> 200). */
int cbk_cuda_get_version(void);

/* 1 if V is an accepted interleave width (2, 4, 8, 16, or 32*k <= 1024). */
int cbk_cuda_vlen_ok(int V);

/* A short description of a return code (0, -j, or a CUDA error). */
const char *cbk_cuda_status_string(int info);

/* The declarations below come in pairs per scalar type (d = double,
 * s = float): NAME(...) on stream 0 and NAME_async(..., stream). */

/* QR factorization (include/cbk.h:79-95). -1 layout -2 m -3 n -5 ldap -7 V -8 nm */
int cbk_cuda_dgeqrf_compact(char layout, int m, int n, double *ap, int ldap, double *taup,
                            int V, int nm);
int cbk_cuda_dgeqrf_compact_async(char layout, int m, int n, double *ap, int ldap,
                                  double *taup, int V, int nm, cbk_stream_t stream);
int cbk_cuda_sgeqrf_compact(char layout, int m, int n, float *ap, int ldap, float *taup,
                            int V, int nm);
int cbk_cuda_sgeqrf_compact_async(char layout, int m, int n, float *ap, int ldap, float *taup,
                                  int V, int nm, cbk_stream_t stream);

/* Apply Q or Q^T from either side (include/cbk.h:97-123).
 * -1 layout -2 side -3 trans -4 m -5 n -6 k -8 ldap -11 ldcp -12 V -13 nm */
int cbk_cuda_dormqr_compact(char layout, char side, char trans, int m, int n, int k,
                            const double *ap, int ldap, const double *taup, double *cp,
                            int ldcp, int V, int nm);
int cbk_cuda_dormqr_compact_async(char layout, char side, char trans, int m, int n, int k,
                                  const double *ap, int ldap, const double *taup, double *cp,
                                  int ldcp, int V, int nm, cbk_stream_t stream);
int cbk_cuda_sormqr_compact(char layout, char side, char trans, int m, int n, int k,
                            const float *ap, int ldap, const float *taup, float *cp, int ldcp,
                            int V, int nm);
int cbk_cuda_sormqr_compact_async(char layout, char side, char trans, int m, int n, int k,
                                  const float *ap, int ldap, const float *taup, float *cp,
                                  int ldcp, int V, int nm, cbk_stream_t stream);

/* Form the explicit Q in place (include/cbk.h:125-150).
 * -1 layout -2 m -3 n -4 k -6 ldap -8 V -9 nm; k = 0 writes I(:, 0:n-1) */
int cbk_cuda_dorgqr_compact(char layout, int m, int n, int k, double *ap, int ldap,
                            const double *taup, int V, int nm);
int cbk_cuda_dorgqr_compact_async(char layout, int m, int n, int k, double *ap, int ldap,
                                  const double *taup, int V, int nm, cbk_stream_t stream);
int cbk_cuda_sorgqr_compact(char layout, int m, int n, int k, float *ap, int ldap,
                            const float *taup, int V, int nm);
int cbk_cuda_sorgqr_compact_async(char layout, int m, int n, int k, float *ap, int ldap,
                                  const float *taup, int V, int nm, cbk_stream_t stream);

/* Cholesky factorization (include/cbk.h:151-170). -1 layout -2 uplo -3 n
 * -5 ldap -6 V -7 nm; the strictly-opposite triangle is never touched */
int cbk_cuda_dpotrf_compact(char layout, char uplo, int n, double *ap, int ldap, int V,
                            int nm);
int cbk_cuda_dpotrf_compact_async(char layout, char uplo, int n, double *ap, int ldap, int V,
                                  int nm, cbk_stream_t stream);
int cbk_cuda_spotrf_compact(char layout, char uplo, int n, float *ap, int ldap, int V, int nm);
int cbk_cuda_spotrf_compact_async(char layout, char uplo, int n, float *ap, int ldap, int V,
                                  int nm, cbk_stream_t stream);

/* Solve from a Cholesky factor (include/cbk.h:171-195). -1 layout -2 uplo -3 n
 * -4 nrhs -6 ldap -8 ldbp -9 V -10 nm */
int cbk_cuda_dpotrs_compact(char layout, char uplo, int n, int nrhs, const double *ap,
                            int ldap, double *bp, int ldbp, int V, int nm);
int cbk_cuda_dpotrs_compact_async(char layout, char uplo, int n, int nrhs, const double *ap,
                                  int ldap, double *bp, int ldbp, int V, int nm,
                                  cbk_stream_t stream);
int cbk_cuda_spotrs_compact(char layout, char uplo, int n, int nrhs, const float *ap, int ldap,
                            float *bp, int ldbp, int V, int nm);
int cbk_cuda_spotrs_compact_async(char layout, char uplo, int n, int nrhs, const float *ap,
                                  int ldap, float *bp, int ldbp, int V, int nm,
                                  cbk_stream_t stream);

/* Fused Cholesky factor + solve (include/cbk.h:196-212): bit-identical to
 * ?potrf then ?potrs; nrhs = 0 still factors. Codes as ?potrs. */
int cbk_cuda_dposv_compact(char layout, char uplo, int n, int nrhs, double *ap, int ldap,
                           double *bp, int ldbp, int V, int nm);
int cbk_cuda_dposv_compact_async(char layout, char uplo, int n, int nrhs, double *ap, int ldap,
                                 double *bp, int ldbp, int V, int nm, cbk_stream_t stream);
int cbk_cuda_sposv_compact(char layout, char uplo, int n, int nrhs, float *ap, int ldap,
                           float *bp, int ldbp, int V, int nm);
int cbk_cuda_sposv_compact_async(char layout, char uplo, int n, int nrhs, float *ap, int ldap,
                                 float *bp, int ldbp, int V, int nm, cbk_stream_t stream);

/* Unpivoted LDL^T factorization (include/cbk.h:213-238). Codes as ?potrf. */
int cbk_cuda_dsytrfnp_compact(char layout, char uplo, int n, double *ap, int ldap, int V,
                              int nm);
int cbk_cuda_dsytrfnp_compact_async(char layout, char uplo, int n, double *ap, int ldap, int V,
                                    int nm, cbk_stream_t stream);
int cbk_cuda_ssytrfnp_compact(char layout, char uplo, int n, float *ap, int ldap, int V,
                              int nm);
int cbk_cuda_ssytrfnp_compact_async(char layout, char uplo, int n, float *ap, int ldap, int V,
                                    int nm, cbk_stream_t stream);

/* Solve from an LDL^T factor (include/cbk.h:239-262). Codes as ?potrs. */
int cbk_cuda_dsytrsnp_compact(char layout, char uplo, int n, int nrhs, const double *ap,
                              int ldap, double *bp, int ldbp, int V, int nm);
int cbk_cuda_dsytrsnp_compact_async(char layout, char uplo, int n, int nrhs, const double *ap,
                                    int ldap, double *bp, int ldbp, int V, int nm,
                                    cbk_stream_t stream);
int cbk_cuda_ssytrsnp_compact(char layout, char uplo, int n, int nrhs, const float *ap,
                              int ldap, float *bp, int ldbp, int V, int nm);
int cbk_cuda_ssytrsnp_compact_async(char layout, char uplo, int n, int nrhs, const float *ap,
                                    int ldap, float *bp, int ldbp, int V, int nm,
                                    cbk_stream_t stream);

/* Fused LDL^T factor + solve (include/cbk.h:263-279). Codes as ?potrs. */
int cbk_cuda_dsysvnp_compact(char layout, char uplo, int n, int nrhs, double *ap, int ldap,
                             double *bp, int ldbp, int V, int nm);
int cbk_cuda_dsysvnp_compact_async(char layout, char uplo, int n, int nrhs, double *ap,
                                   int ldap, double *bp, int ldbp, int V, int nm,
                                   cbk_stream_t stream);
int cbk_cuda_ssysvnp_compact(char layout, char uplo, int n, int nrhs, float *ap, int ldap,
                             float *bp, int ldbp, int V, int nm);
int cbk_cuda_ssysvnp_compact_async(char layout, char uplo, int n, int nrhs, float *ap,
                                   int ldap, float *bp, int ldbp, int V, int nm,
                                   cbk_stream_t stream);

/* Triangular solve (include/cbk.h:280-309). -1 layout -2 side -3 uplo
 * -4 transa -5 diag -6 m -7 n -10 ldap -12 ldbp -13 V -14 nm;
 * alpha = 0 sets B := 0 without reading A */
int cbk_cuda_dtrsm_compact(char layout, char side, char uplo, char transa, char diag, int m,
                           int n, double alpha, const double *ap, int ldap, double *bp,
                           int ldbp, int V, int nm);
int cbk_cuda_dtrsm_compact_async(char layout, char side, char uplo, char transa, char diag,
                                 int m, int n, double alpha, const double *ap, int ldap,
                                 double *bp, int ldbp, int V, int nm, cbk_stream_t stream);
int cbk_cuda_strsm_compact(char layout, char side, char uplo, char transa, char diag, int m,
                           int n, float alpha, const float *ap, int ldap, float *bp, int ldbp,
                           int V, int nm);
int cbk_cuda_strsm_compact_async(char layout, char side, char uplo, char transa, char diag,
                                 int m, int n, float alpha, const float *ap, int ldap,
                                 float *bp, int ldbp, int V, int nm, cbk_stream_t stream);

/* Least squares / minimum norm (include/cbk.h:310-352). -1 layout -2 trans
 * -3 m -4 n -5 nrhs -7 ldap -9 ldbp -11 V -12 nm; min(m,n) = 0 sets B := 0,
 * nrhs = 0 does nothing */
int cbk_cuda_dgels_compact(char layout, char trans, int m, int n, int nrhs, double *ap,
                           int ldap, double *bp, int ldbp, double *taup, int V, int nm);
int cbk_cuda_dgels_compact_async(char layout, char trans, int m, int n, int nrhs, double *ap,
                                 int ldap, double *bp, int ldbp, double *taup, int V, int nm,
                                 cbk_stream_t stream);
int cbk_cuda_sgels_compact(char layout, char trans, int m, int n, int nrhs, float *ap,
                           int ldap, float *bp, int ldbp, float *taup, int V, int nm);
int cbk_cuda_sgels_compact_async(char layout, char trans, int m, int n, int nrhs, float *ap,
                                 int ldap, float *bp, int ldbp, float *taup, int V, int nm,
                                 cbk_stream_t stream);

/* The same routines on HOST arrays: the reference's own calling convention
 * (include/cbk.h:77-352, every array on the host; its MKL-style adapter,
 * src/cbk_compat.cpp:252-333, is such a layer over the kernels too) over the
 * device routines above. cbk_cuda_host_NAME_compact takes NAME's arguments
 * unchanged -- host pointers, the same -j codes in the same order, the same
 * quick returns, which touch no array and need no workspace -- plus:
 *   dwork  device memory of at least *lwork bytes (the call never allocates);
 *   lwork  in: the bytes of dwork, or a negative value to ask: the call then
 *          checks the arguments, stores the bytes it needs in *lwork (0 when
 *          there is nothing to compute) and returns, touching nothing else;
 *   stream the stream the copies and kernels run on.
 * The call copies the arrays the routine reads to dwork, runs it there,
 * copies the arrays it writes back and synchronises the stream; the host
 * arrays then hold exactly what NAME_compact_async leaves in device memory.
 * Extra codes: -(k+1) dwork NULL or *lwork too small, -(k+2) lwork NULL,
 * where k is NAME's argument count (geqrf 8, ormqr 13, orgqr 9, potrf and
 * sytrfnp 7, potrs, posv, sytrsnp and sysvnp 10, trsm 14, gels 12). */
#define CBK_CUDA_HOST_DECLS(T, p)                                                                  \
    int cbk_cuda_host_##p##geqrf_compact(char layout, int m, int n, T *ap, int ldap, T *taup,     \
                                         int V, int nm, void *dwork, long long *lwork,             \
                                         cbk_stream_t stream);                                     \
    int cbk_cuda_host_##p##ormqr_compact(char layout, char side, char trans, int m, int n, int k,  \
                                         const T *ap, int ldap, const T *taup, T *cp, int ldcp,    \
                                         int V, int nm, void *dwork, long long *lwork,             \
                                         cbk_stream_t stream);                                     \
    int cbk_cuda_host_##p##orgqr_compact(char layout, int m, int n, int k, T *ap, int ldap,        \
                                         const T *taup, int V, int nm, void *dwork,                \
                                         long long *lwork, cbk_stream_t stream);                   \
    int cbk_cuda_host_##p##potrf_compact(char layout, char uplo, int n, T *ap, int ldap, int V,    \
                                         int nm, void *dwork, long long *lwork,                    \
                                         cbk_stream_t stream);                                     \
    int cbk_cuda_host_##p##sytrfnp_compact(char layout, char uplo, int n, T *ap, int ldap, int V,  \
                                           int nm, void *dwork, long long *lwork,                  \
                                           cbk_stream_t stream);                                   \
    int cbk_cuda_host_##p##potrs_compact(char layout, char uplo, int n, int nrhs, const T *ap,     \
                                         int ldap, T *bp, int ldbp, int V, int nm, void *dwork,    \
                                         long long *lwork, cbk_stream_t stream);                   \
    int cbk_cuda_host_##p##posv_compact(char layout, char uplo, int n, int nrhs, T *ap, int ldap,  \
                                        T *bp, int ldbp, int V, int nm, void *dwork,               \
                                        long long *lwork, cbk_stream_t stream);                    \
    int cbk_cuda_host_##p##sytrsnp_compact(char layout, char uplo, int n, int nrhs, const T *ap,   \
                                           int ldap, T *bp, int ldbp, int V, int nm, void *dwork,  \
                                           long long *lwork, cbk_stream_t stream);                 \
    int cbk_cuda_host_##p##sysvnp_compact(char layout, char uplo, int n, int nrhs, T *ap,          \
                                          int ldap, T *bp, int ldbp, int V, int nm, void *dwork,   \
                                          long long *lwork, cbk_stream_t stream);                  \
    int cbk_cuda_host_##p##trsm_compact(char layout, char side, char uplo, char transa,           \
                                        char diag, int m, int n, T alpha, const T *ap, int ldap,   \
                                        T *bp, int ldbp, int V, int nm, void *dwork,               \
                                        long long *lwork, cbk_stream_t stream);                    \
    int cbk_cuda_host_##p##gels_compact(char layout, char trans, int m, int n, int nrhs, T *ap,    \
                                        int ldap, T *bp, int ldbp, T *taup, int V, int nm,         \
                                        void *dwork, long long *lwork, cbk_stream_t stream);
CBK_CUDA_HOST_DECLS(double, d)
CBK_CUDA_HOST_DECLS(float, s)
#undef CBK_CUDA_HOST_DECLS

/* Dense batch <-> compact layout on the device. No reference entry point:
 * the device form of the reference tests' pack_compact / unpack_compact
 * (tests/test_compact_util.hpp:477-531) and of mkl_?gepack_compact.
 * a holds nm m x n matrices, matrix idx at a + idx*stridea, element (i,j) at
 * i + j*lda (layout 'C') or i*lda + j ('R'); ap is the compact batch in the
 * same layout. Pack fills the padded lanes of the last group with pad_diag
 * on the diagonal and zero elsewhere (1 for matrices, 0 for right-hand sides
 * or tau); unpack writes only the nm real matrices.
 * pack:   -1 layout -2 m -3 n -5 lda (< max(1, m) 'C' / max(1, n) 'R')
 *         -6 stridea (< lda * n 'C' / lda * m 'R') -8 ldap -9 V -10 nm
 * unpack: -1 layout -2 m -3 n -5 ldap -7 lda -8 stridea -9 V -10 nm */
int cbk_cuda_dpack_compact_async(char layout, int m, int n, const double *a, int lda,
                                 long long stridea, double *ap, int ldap, int V, int nm,
                                 double pad_diag, cbk_stream_t stream);
int cbk_cuda_spack_compact_async(char layout, int m, int n, const float *a, int lda,
                                 long long stridea, float *ap, int ldap, int V, int nm,
                                 float pad_diag, cbk_stream_t stream);
int cbk_cuda_dunpack_compact_async(char layout, int m, int n, const double *ap, int ldap,
                                   double *a, int lda, long long stridea, int V, int nm,
                                   cbk_stream_t stream);
int cbk_cuda_sunpack_compact_async(char layout, int m, int n, const float *ap, int ldap,
                                   float *a, int lda, long long stridea, int V, int nm,
                                   cbk_stream_t stream);

/* Mixed-precision SPD solve A X = B: FP32 Cholesky, FP64 iterative refinement
 * of each right-hand side, FP64 fallback per matrix. No reference entry
 * point: the ?posv_compact arguments (include/cbk.h:196-212) plus the method
 * of LAPACK dsposv. Per lane: x = solve32(b); r = b - A x in FP64 until
 * ||r||_inf <= sqrt(n) eps64 ||A||_inf ||x||_inf, correcting x += solve32(r)
 * (for n <= 8 and 17 <= n <= 40 the first r, of the FP32-exact x0, is formed
 * in double-FP32 arithmetic instead: error-free products and sums, Dot2; the
 * stopping test is always taken on an FP64 residual);
 * a lane whose FP32 rounding overflows (iters = -2), whose FP32 pivot is not
 * positive (-1), or whose refinement stalls or exceeds max_iter corrections
 * (-3) is solved by the FP64 path instead and then holds its FP64 factor in
 * ap; a converged lane leaves ap unchanged. bp is overwritten with X.
 *   iters  device int[nm] or NULL: corrections used (max over the lane's
 *          right-hand sides), or the negative fallback code
 *   berr   device double[nm] or NULL: the lane's largest normwise backward
 *          error ||b - A x|| / (||A|| ||x|| + ||b||) (inf-norms), NaN when the
 *          lane fell back
 *   work   device workspace of lwork bytes, at least
 *          cbk_cuda_dposv_refined_compact_lwork(n, nrhs, V, nm): 0 for n <= 64,
 *          where the FP32 factor stays on chip (registers for n <= 16, one
 *          warp per matrix with the matrix in shared memory for 17 .. 64),
 *          and NULL is allowed then
 * Returns 0, or -j: -1 layout -2 uplo -3 n -4 nrhs -6 ldap -8 ldbp -9 V
 * -10 nm -11 max_iter (< 0) -15 lwork (too small). n = 0, nm = 0 or
 * nrhs = 0 return at once, touching nothing. */
long long cbk_cuda_dposv_refined_compact_lwork(int n, int nrhs, int V, int nm);
int cbk_cuda_dposv_refined_compact_async(char layout, char uplo, int n, int nrhs, double *ap,
                                         int ldap, double *bp, int ldbp, int V, int nm,
                                         int max_iter, int *iters, double *berr, void *work,
                                         long long lwork, cbk_stream_t stream);

/* The same solve on a strided dense batch, the layout of cuBLAS/cuSOLVER
 * batched routines: matrix k's A is column-major at a + k*stride_a with
 * leading dimension lda (the uplo triangle referenced), its B at
 * b + k*stride_b with leading dimension ldb. No reference entry point: the
 * reference's callers pack into the compact layout first
 * (tests/test_compact_util.hpp:468-531); here the kernels read and write
 * the dense arrays directly, and each matrix's results are bit-identical to
 * the compact entry point's for the same matrix. Returns 0, -1 uplo, -2 n,
 * -3 nrhs, -5 lda < max(1,n), -6 stride_a < lda*n, -8 ldb < max(1,n),
 * -9 stride_b < ldb*nrhs, -10 nm, -11 max_iter, -15 work/lwork below
 * cbk_cuda_dposv_refined_batched_lwork(n, nrhs, nm) (0 for n <= 64; -1 for
 * a negative argument), or CBK_CUDA_ERROR_BASE + a CUDA error. iters, berr
 * and the fallback are as for the compact entry point. */
long long cbk_cuda_dposv_refined_batched_lwork(int n, int nrhs, int nm);
int cbk_cuda_dposv_refined_batched_async(char uplo, int n, int nrhs, double *a, int lda,
                                         long long stride_a, double *b, int ldb,
                                         long long stride_b, int nm, int max_iter, int *iters,
                                         double *berr, void *work, long long lwork,
                                         cbk_stream_t stream);

/* The plain drivers on strided dense batches, the layout of cuBLAS/cuSOLVER
 * batched routines: matrix k's A is column-major at a + k*stride_a with
 * leading dimension lda, its B at b + k*stride_b with leading dimension ldb.
 * No reference entry point (the reference's callers pack into the compact
 * layout first, tests/test_compact_util.hpp:468-531): the kernels read and
 * write the dense arrays directly, and each matrix gets exactly the bits of
 * the compact entry point (?posv_compact, ?sysvnp_compact, ?gels_compact).
 * ?posv_batched / ?sysvnp_batched (the uplo triangle referenced; nrhs = 0
 * still factors): 0, -1 uplo, -2 n, -3 nrhs, -5 lda < max(1,n),
 * -6 stride_a < lda*n, -8 ldb < max(1,n), -9 stride_b < ldb*nrhs, -10 nm.
 * ?gels_batched (trans 'N' or 'T'; A m x n, B max(m,n) x nrhs, the min(m,n)
 * tau values of matrix k at tau + k*min(m,n)): 0, -1 trans, -2 m, -3 n,
 * -4 nrhs, -6 lda < max(1,m), -7 stride_a < lda*n, -9 ldb < max(1,m,n),
 * -10 stride_b < ldb*nrhs, -12 nm. Or CBK_CUDA_ERROR_BASE + a CUDA error. */
int cbk_cuda_dposv_batched_async(char uplo, int n, int nrhs, double *a, int lda,
                                 long long stride_a, double *b, int ldb, long long stride_b,
                                 int nm, cbk_stream_t stream);
int cbk_cuda_sposv_batched_async(char uplo, int n, int nrhs, float *a, int lda,
                                 long long stride_a, float *b, int ldb, long long stride_b, int nm,
                                 cbk_stream_t stream);
int cbk_cuda_dsysvnp_batched_async(char uplo, int n, int nrhs, double *a, int lda,
                                   long long stride_a, double *b, int ldb, long long stride_b,
                                   int nm, cbk_stream_t stream);
int cbk_cuda_ssysvnp_batched_async(char uplo, int n, int nrhs, float *a, int lda,
                                   long long stride_a, float *b, int ldb, long long stride_b,
                                   int nm, cbk_stream_t stream);
int cbk_cuda_dgels_batched_async(char trans, int m, int n, int nrhs, double *a, int lda,
                                 long long stride_a, double *b, int ldb, long long stride_b,
                                 double *tau, int nm, cbk_stream_t stream);
int cbk_cuda_sgels_batched_async(char trans, int m, int n, int nrhs, float *a, int lda,
                                 long long stride_a, float *b, int ldb, long long stride_b,
                                 float *tau, int nm, cbk_stream_t stream);

/* The same solve on batches in HOST memory (ap, bp, iters, berr are host
 * pointers; pinned memory lets the copies overlap the solves). No reference
 * entry point: the reference's own calling convention -- every array on the
 * host, as in ?posv_compact (include/cbk.h:196-212) -- over the device solve
 * above. The batch is cut into chunks of whole groups (about 192 MiB of
 * input each, at least 256 groups; the first and last about 12 MiB)
 * that pass through three device slots on three streams, so that copying one
 * chunk in, solving another and copying a third out overlap. The workspace
 * is therefore bounded whatever nm. When ap is pinned (or registered)
 * host memory, the device reads only the referenced triangle of A from it
 * directly; otherwise each chunk's A moves as one contiguous copy. B moves as
 * one contiguous copy each way. B (X) is copied back; A is copied back only for a
 * chunk in which some lane fell back (ap then holds those lanes' FP64
 * factor), so ap, bp, iters and berr end exactly as the device entry point
 * leaves them. dwork is a device workspace of at least
 * cbk_cuda_dposv_refined_compact_host_lwork(layout, n, nrhs, ldap, ldbp, V,
 * nm) bytes (0 when n, nrhs or nm is 0; -1 for an illegal argument). The call
 * returns when every copy is done; its work is ordered after the caller's
 * prior work on stream. Returns 0, the codes of
 * cbk_cuda_dposv_refined_compact_async (-15 for dwork/lwork), or
 * CBK_CUDA_ERROR_BASE + a CUDA error. */
long long cbk_cuda_dposv_refined_compact_host_lwork(char layout, int n, int nrhs, int ldap,
                                                    int ldbp, int V, int nm);
int cbk_cuda_dposv_refined_compact_host(char layout, char uplo, int n, int nrhs, double *ap,
                                        int ldap, double *bp, int ldbp, int V, int nm,
                                        int max_iter, int *iters, double *berr, void *dwork,
                                        long long lwork, cbk_stream_t stream);

/* Mixed-precision least squares min ||b - A x||, A m x n with m >= n: FP32
 * QR, FP64 refinement of the augmented system [I A; A^T 0][r; x] = [b; 0]
 * (Bjorck) per right-hand side, FP64 fallback per matrix. No reference entry
 * point: the ?gels_compact arguments (include/cbk.h:310-352) for the
 * overdetermined, non-transposed case. Per lane: x0 from the FP32 QR, then
 * f = b - r - A x and g = -A^T r in FP64, the correction from the FP32 QR,
 * until both residuals are at the FP64 rounding level of their terms
 * (||g||_inf <= sqrt(n) eps64 ||A|| (||A|| ||x|| + ||b|| + ||r||) and
 * ||f||_inf <= sqrt(n) eps64 (||A|| ||x|| + ||b|| + ||r||)). A lane whose FP32 rounding
 * overflows (iters -2) or whose refinement stalls or exceeds max_iter (-3)
 * is solved by the FP64 path, whose QR then sits in ap and taup; a converged
 * lane leaves ap and taup untouched. On exit B(0:n) holds X and B(n:m) the
 * residual's coordinates (Q^T r)(n:m) through the FP32 Q (their squared
 * norms are the residual sums of squares to FP32 accuracy).
 *   iters, berr  device int[nm] / double[nm] or NULL: corrections used, or
 *          the fallback code; the largest normal-equations residual
 *          ||A^T r||_inf / (||A||_inf (||A||_inf ||x||_inf + ||b||_inf))
 *          (NaN when the lane fell back)
 *   work   at least cbk_cuda_dgels_refined_compact_lwork(m, n, nrhs, V, nm)
 *          bytes of device memory
 * Returns 0, or -j: -1 layout -2 trans (only 'N') -3 m -4 n (< 0, > m or
 * > 64) -5 nrhs -7 ldap -9 ldbp -11 V -12 nm -13 max_iter -17 lwork.
 * nrhs = 0, nm = 0 or m = 0 return at once; n = 0 sets B := 0. */
long long cbk_cuda_dgels_refined_compact_lwork(int m, int n, int nrhs, int V, int nm);
int cbk_cuda_dgels_refined_compact_async(char layout, char trans, int m, int n, int nrhs,
                                         double *ap, int ldap, double *bp, int ldbp,
                                         double *taup, int V, int nm, int max_iter, int *iters,
                                         double *berr, void *work, long long lwork,
                                         cbk_stream_t stream);

/* The same least squares on a strided dense batch: matrix k's A (m x n) is
 * column-major at a + k*stride_a with leading dimension lda, its B (m x nrhs)
 * at b + k*stride_b with leading dimension ldb, its n tau values at
 * tau + k*n. No reference entry point (the reference's callers pack first);
 * each matrix's results are bit-identical to the compact entry point's.
 * Returns 0, -1 trans (only 'N'), -2 m, -3 n (0 <= n <= min(m, 64)), -4 nrhs,
 * -6 lda < max(1,m), -7 stride_a < lda*n, -9 ldb < max(1,m),
 * -10 stride_b < ldb*nrhs, -12 nm, -13 max_iter, -17 work/lwork below
 * cbk_cuda_dgels_refined_batched_lwork(m, n, nrhs, nm) (-1 for a negative
 * argument), or CBK_CUDA_ERROR_BASE + a CUDA error. n = 0 sets B to zero. */
long long cbk_cuda_dgels_refined_batched_lwork(int m, int n, int nrhs, int nm);
int cbk_cuda_dgels_refined_batched_async(char trans, int m, int n, int nrhs, double *a, int lda,
                                         long long stride_a, double *b, int ldb,
                                         long long stride_b, double *tau, int nm, int max_iter,
                                         int *iters, double *berr, void *work, long long lwork,
                                         cbk_stream_t stream);

/* Batches of uneven orders in one persistent launch. No reference counterpart:
 * the reference takes one order per call (?sysvnp_compact, ?posv_compact), so
 * a mixed batch is one call per order. Here the caller groups the matrices by
 * order into buckets, each an ordinary compact batch (its own n, nm, V, ap,
 * ldap, bp, ldbp, the layout of include/cbk.h), and one launch factors and
 * solves every bucket: the work is cut into 32-lane items, largest order
 * first, pulled by one wave of warps from a device counter held in `work`.
 * Each bucket's results are bit-identical to a ?sysvnp_compact
 * (?posv_compact) call on that bucket alone; nrhs = 0 factors only.
 *   work   device memory of at least CBK_CUDA_BUCKETED_LWORK bytes (the item
 *          counter; reset by the call itself -- concurrent calls need their
 *          own work)
 * Returns 0, or -j: -1 layout -2 uplo -3 nrhs (< 0) -4 nbuckets (< 0 or
 * > CBK_CUDA_MAX_BUCKETS) -5 buckets (NULL, or an entry with n < 0, nm < 0,
 * an illegal V, ldap < max(1, n), or ldbp < max(1, n) column-major /
 * max(1, nrhs) row-major) -6 work (NULL) -7 lwork (too small). */
#define CBK_CUDA_MAX_BUCKETS 64
#define CBK_CUDA_BUCKETED_LWORK 256
typedef struct {
    int n, nm, V;
    double *ap;
    int ldap;
    double *bp;
    int ldbp;
} cbk_cuda_dbucket;
typedef struct {
    int n, nm, V;
    float *ap;
    int ldap;
    float *bp;
    int ldbp;
} cbk_cuda_sbucket;
int cbk_cuda_dsysvnp_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_dbucket *buckets, void *work,
                                            long long lwork, cbk_stream_t stream);
int cbk_cuda_ssysvnp_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_sbucket *buckets, void *work,
                                            long long lwork, cbk_stream_t stream);
int cbk_cuda_dposv_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                          const cbk_cuda_dbucket *buckets, void *work,
                                          long long lwork, cbk_stream_t stream);
int cbk_cuda_sposv_compact_bucketed_async(char layout, char uplo, int nrhs, int nbuckets,
                                          const cbk_cuda_sbucket *buckets, void *work,
                                          long long lwork, cbk_stream_t stream);

/* The same launch captured once into an instantiated CUDA graph (the counter
 * reset and the persistent kernel), replayed by cbk_cuda_graph_launch on any
 * stream: one submission per replay, no host work. The buckets' pointers are
 * baked in; the graph is valid while they are. graph_create returns the
 * bucketed call's codes (-1 .. -7), or CBK_CUDA_ERROR_BASE + a CUDA error. */
typedef struct cbk_cuda_graph_st *cbk_cuda_graph;
int cbk_cuda_dsysvnp_compact_bucketed_graph(char layout, char uplo, int nrhs, int nbuckets,
                                            const cbk_cuda_dbucket *buckets, void *work,
                                            long long lwork, cbk_cuda_graph *graph);
int cbk_cuda_graph_launch(cbk_cuda_graph graph, cbk_stream_t stream);
int cbk_cuda_graph_destroy(cbk_cuda_graph graph);

/* The mixed-precision SPD solve without a workspace and without allocating.
 * No counterpart in the reference, whose routines need no scratch memory.
 * It is for callers that cannot allocate device memory at the point of the
 * call: code hosted by a framework or plugin host that owns every device
 * allocation, or a latency-bound loop that must not call cudaMalloc or
 * cudaFree. For n > 64 the FP32 factor needs scratch; here it comes from one
 * array of CBK_CUDA_NOALLOC_SCRATCH_BYTES (64 MiB) that the library reserves
 * on every GPU it is used on, for as long as the process runs. n <= 64 needs
 * none.
 * Arguments, results and return codes are those of
 * cbk_cuda_dposv_refined_compact_async without work and lwork, plus:
 *   CBK_CUDA_NOALLOC_TOO_LARGE  the batch does not fit the array:
 *          cbk_cuda_dposv_refined_compact_lwork(n, nrhs, V, nm) exceeds
 *          CBK_CUDA_NOALLOC_SCRATCH_BYTES (for n = 80, about 2,500 matrices;
 *          split larger batches into several calls); checked after the
 *          argument codes, before any device work
 *   CBK_CUDA_NOALLOC_IN_CAPTURE  the first n > 64 call in this CUDA context
 *          came on a capturing stream: nothing was enqueued
 * The first n > 64 call in each CUDA context (each device's primary context,
 * a driver-API context of the caller's, the primary context again after a
 * cudaDeviceReset) looks up the array's address in that context: make it
 * before any stream capture. Every call shares the one array, and it keeps
 * the last call's contents; nothing in it needs to start at zero. Calls that
 * overlap on the GPU -- on different streams, or from host threads without
 * ordering between them -- race on the array and give wrong results:
 * serialise them on one stream. */
#define CBK_CUDA_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define CBK_CUDA_NOALLOC_TOO_LARGE 900
#define CBK_CUDA_NOALLOC_IN_CAPTURE 901
int cbk_cuda_dposv_refined_compact_noalloc_async(char layout, char uplo, int n, int nrhs,
                                                 double *ap, int ldap, double *bp, int ldbp,
                                                 int V, int nm, int max_iter, int *iters,
                                                 double *berr, cbk_stream_t stream);

/* Autotuning, no reference counterpart. The library keeps one process-wide
 * table of launch shapes per (routine, precision, order): threads per block
 * of the lane-per-matrix kernels, the block shape of the warp-per-matrix
 * refined solve (orders 17 .. 64: variant 0 four matrices per block, 1 the
 * same at a lower register cap with one block more per SM, 2 two matrices
 * per block, 3 one), and the interleave width measured fastest
 * (advice for the caller's packing; a batch's width is the caller's). Entry
 * 0 means the built-in choice. Launch shapes never change results.
 * routine: "potrf", "sytrfnp", "potrs", "posv", "sytrsnp", "sysvnp", "trsm",
 * "geqrf", "ormqr", "orgqr", "gels", "posv_refined", "gels_refined",
 * "sysvnp_bucketed" or "posv_bucketed"; prec
 * 'd' or 's' ('d' only for the refined solves); the order is n, except m for
 * the QR routines. "gels_refined" has one entry, set by cbk_cuda_tune_set
 * (not autotuned): variant 0 runs one warp per matrix where that kernel is
 * compiled (m <= 64, n = 8 or 16), variant 1 one lane per matrix.
 * "sysvnp_bucketed" / "posv_bucketed" (keyed by the largest order of the
 * launch): variant v runs the persistent grid with one wave of warps halved
 * v times (0 .. 3) -- fewer matrices in flight keep the large orders' working
 * set in the L2 cache, against less latency hiding.
 *
 * cbk_cuda_autotune times the routine on a synthetic batch of nm matrices
 * (m x n for the QR routines, m >= n; n x n otherwise; nrhs right-hand
 * sides; for the bucketed launches nm matrices spread over the orders 4 .. n,
 * at width 32) for every candidate shape at widths 32, 64 and 128, best of
 * three CUDA-event timings each, and stores the winner. It allocates and
 * synchronises the device (not for use inside a stream capture). Returns 0,
 * -1 routine, -2 prec, -3 m, -4 n, -5 nrhs, -6 nm, or CBK_CUDA_ERROR_BASE + a
 * CUDA error (the table entry then keeps the built-in choice).
 * cbk_cuda_tune_set / _get write / read one entry (set: threads 0 or a
 * power of two 32 .. 512, variant 0 .. 3, vlen 0 or a multiple of 32 up to
 * 1024; -j for the first illegal argument). cbk_cuda_tune_save writes every
 * non-default entry as text ("routine prec n threads variant vlen" lines);
 * cbk_cuda_tune_load reads such a file and returns the number of entries, -1
 * if it cannot be read, or -(line) at the first malformed line. The
 * environment variable CBK_CUDA_TUNE_FILE names a file loaded on first use. */
typedef struct {
    int threads; /* threads per block (0: built-in) */
    int variant; /* kernel variant (0: built-in) */
    int vlen;    /* fastest interleave width measured (0: untuned) */
    double ms;   /* the chosen shape's time for the tuning batch (autotune only) */
} cbk_cuda_tune_result;
int cbk_cuda_autotune(const char *routine, char prec, int m, int n, int nrhs, int nm,
                      cbk_cuda_tune_result *out);
/* The same at one interleave width V (a multiple of 32, -7 otherwise), for a
 * caller whose layout is fixed. */
int cbk_cuda_autotune_at(const char *routine, char prec, int m, int n, int nrhs, int nm, int V,
                         cbk_cuda_tune_result *out);
int cbk_cuda_tune_set(const char *routine, char prec, int n, int threads, int variant, int vlen);
int cbk_cuda_tune_get(const char *routine, char prec, int n, cbk_cuda_tune_result *out);
void cbk_cuda_tune_reset(void);
int cbk_cuda_tune_save(const char *path);
int cbk_cuda_tune_load(const char *path);

/* The bounds-checked build, no reference counterpart. libcbk_cuda_checked.so
 * (cbk_gb300/build.py, build(checked=True)) is this library compiled with
 * CBK_CUDA_CHECKED: every element access a kernel makes through a matrix
 * view -- all of the lane-per-matrix kernels' accesses, and the warp
 * kernels' global-memory ones -- is first tested against the matrix's
 * logical extent; an access outside it is not made but counted, with the
 * (i, j) of the first. cbk_cuda_check_status reads (and, if reset, clears)
 * that count after the caller has synchronised its streams. Returns 0, -1 in
 * the normal build (count 0: nothing is checked), or CBK_CUDA_ERROR_BASE + a
 * CUDA error. Shared-memory accesses and the warp kernels' staging copies are
 * not checked. */
int cbk_cuda_check_status(unsigned long long *count, int *first_i, int *first_j, int reset);

/* Calibration, no reference counterpart: the measured fused multiply-add
 * rate of the current device in TFLOP/s (2 flops per FMA), FP64 (fp64 = 1)
 * or FP32 (fp64 = 0), from a ~10 ms synthetic kernel -- the denominator of the
 * FP64-pipe roofline that bounds the FP64 solves on a GB300. Allocates and
 * synchronises the device; not for use inside a captured stream. */
int cbk_cuda_measure_fma_rate(int fp64, double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* CBK_CUDA_H */
