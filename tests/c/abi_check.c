/* A C caller of include/cbk_cuda.h, as a C program that used include/cbk.h
 * would become: argument checks, quick returns and workspace queries, which
 * all return before any device work, so it runs without a GPU. Exit code 0
 * when every call returns what the header documents. */
#include <stdio.h>

#include "cbk_cuda.h"

static int fails = 0;

#define EXPECT(expr, want)                                                        \
    do {                                                                          \
        const long long got_ = (long long)(expr);                                 \
        if (got_ != (long long)(want)) {                                          \
            printf("FAIL %s: %lld, expected %lld\n", #expr, got_, (long long)(want)); \
            ++fails;                                                              \
        }                                                                         \
    } while (0)

int main(void)
{
    double a[4] = {0}, b[4] = {0}, t[4] = {0};
    EXPECT(cbk_cuda_get_version() > 0, 1);
    EXPECT(cbk_cuda_vlen_ok(32), 1);
    EXPECT(cbk_cuda_vlen_ok(8), 1);
    EXPECT(cbk_cuda_vlen_ok(48), 0);
    /* the reference's routines: -j for the first illegal argument, in order */
    EXPECT(cbk_cuda_dposv_compact('X', 'L', 8, 1, a, 8, b, 8, 32, 64), -1);
    EXPECT(cbk_cuda_dposv_compact('C', 'X', 8, 1, a, 8, b, 8, 32, 64), -2);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', -1, 1, a, 8, b, 8, 32, 64), -3);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', 8, -1, a, 8, b, 8, 32, 64), -4);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', 8, 1, a, 7, b, 8, 32, 64), -6);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', 8, 1, a, 8, b, 7, 32, 64), -8);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', 8, 1, a, 8, b, 8, 48, 64), -9);
    EXPECT(cbk_cuda_dposv_compact('C', 'L', 8, 1, a, 8, b, 8, 32, -1), -10);
    EXPECT(cbk_cuda_dposv_compact('c', 'l', 0, 1, a, 1, b, 1, 32, 64), 0);
    EXPECT(cbk_cuda_dgels_compact('C', 'X', 8, 4, 1, a, 8, b, 8, t, 32, 64), -2);
    EXPECT(cbk_cuda_dgels_compact('C', 'N', 8, 4, 1, a, 8, b, 8, t, 32, 0), 0);
    /* the mixed-precision solves and their workspace queries */
    EXPECT(cbk_cuda_dposv_refined_compact_lwork(48, 1, 32, 1000), 0);
    EXPECT(cbk_cuda_dposv_refined_compact_lwork(8, 1, 48, 1000), -1);
    EXPECT(cbk_cuda_dposv_refined_compact_async('C', 'L', 8, 1, a, 8, b, 8, 32, 64, -1, 0, 0, 0,
                                                0, 0),
           -11);
    EXPECT(cbk_cuda_dposv_refined_batched_lwork(48, 1, 1000), 0);
    EXPECT(cbk_cuda_dposv_refined_batched_async('L', 8, 1, a, 8, 63, b, 8, 8, 10, 10, 0, 0, 0, 0,
                                                0),
           -6);
    EXPECT(cbk_cuda_dgels_refined_batched_async('N', 8, 4, 1, a, 8, 32, b, 8, 8, t, 10, 10, 0, 0,
                                                0, 0, 0),
           -17);
    EXPECT(cbk_cuda_dgels_refined_batched_lwork(-1, 1, 1, 1), -1);
    /* the plain drivers on strided dense batches, both precisions */
    {
        float fa[4] = {0}, fb[4] = {0}, ft[4] = {0};
        EXPECT(cbk_cuda_dposv_batched_async('X', 8, 1, a, 8, 64, b, 8, 8, 10, 0), -1);
        EXPECT(cbk_cuda_dposv_batched_async('L', 8, 1, a, 8, 63, b, 8, 8, 10, 0), -6);
        EXPECT(cbk_cuda_sposv_batched_async('U', 8, 2, fa, 8, 64, fb, 8, 15, 10, 0), -9);
        EXPECT(cbk_cuda_dsysvnp_batched_async('L', 8, 1, a, 8, 64, b, 7, 8, 10, 0), -8);
        EXPECT(cbk_cuda_ssysvnp_batched_async('L', 0, 1, fa, 1, 0, fb, 1, 1, 10, 0), 0);
        EXPECT(cbk_cuda_dgels_batched_async('N', 8, 4, 1, a, 8, 31, b, 8, 8, t, 10, 0), -7);
        EXPECT(cbk_cuda_sgels_batched_async('T', 4, 8, 1, fa, 4, 32, fb, 4, 8, ft, 10, 0), -9);
        EXPECT(cbk_cuda_sgels_batched_async('N', 8, 4, 1, fa, 8, 32, fb, 8, 8, ft, -1, 0), -12);
    }
    if (fails == 0) printf("c abi ok\n");
    return fails != 0;
}
