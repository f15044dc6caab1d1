/* cbk_oracle.h -- TEST INFRASTRUCTURE (the oracle), not the product.
 *
 * The CPU restatement of ivan-pi/cbk v0.2.0's include/cbk.h C API that the
 * CUDA library is checked against. Same argument lists, meaning and -j error
 * codes as include/cbk.h:77-351 (host pointers), names prefixed oracle_.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 */
#ifndef CBK_ORACLE_H
#define CBK_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

int oracle_get_version(void);
int oracle_max_threads(void);
int oracle_vlen_ok(int V);

#define CBK_ORACLE_DECLARE(T, p)                                                          \
    int oracle_##p##geqrf_compact(char layout, int m, int n, T *ap, int ldap, T *taup,    \
                                  int V, int nm);                                         \
    int oracle_##p##ormqr_compact(char layout, char side, char trans, int m, int n,       \
                                  int k, const T *ap, int ldap, const T *taup, T *cp,     \
                                  int ldcp, int V, int nm);                               \
    int oracle_##p##orgqr_compact(char layout, int m, int n, int k, T *ap, int ldap,      \
                                  const T *taup, int V, int nm);                          \
    int oracle_##p##potrf_compact(char layout, char uplo, int n, T *ap, int ldap, int V,  \
                                  int nm);                                                \
    int oracle_##p##potrs_compact(char layout, char uplo, int n, int nrhs, const T *ap,   \
                                  int ldap, T *bp, int ldbp, int V, int nm);              \
    int oracle_##p##posv_compact(char layout, char uplo, int n, int nrhs, T *ap,          \
                                 int ldap, T *bp, int ldbp, int V, int nm);               \
    int oracle_##p##sytrfnp_compact(char layout, char uplo, int n, T *ap, int ldap,       \
                                    int V, int nm);                                       \
    int oracle_##p##sytrsnp_compact(char layout, char uplo, int n, int nrhs,              \
                                    const T *ap, int ldap, T *bp, int ldbp, int V,        \
                                    int nm);                                              \
    int oracle_##p##sysvnp_compact(char layout, char uplo, int n, int nrhs, T *ap,        \
                                   int ldap, T *bp, int ldbp, int V, int nm);             \
    int oracle_##p##trsm_compact(char layout, char side, char uplo, char transa,          \
                                 char diag, int m, int n, T alpha, const T *ap,           \
                                 int ldap, T *bp, int ldbp, int V, int nm);               \
    int oracle_##p##gels_compact(char layout, char trans, int m, int n, int nrhs, T *ap,  \
                                 int ldap, T *bp, int ldbp, T *taup, int V, int nm);

CBK_ORACLE_DECLARE(double, d)
CBK_ORACLE_DECLARE(float, s)

#undef CBK_ORACLE_DECLARE

#ifdef __cplusplus
}
#endif

#endif /* CBK_ORACLE_H */
