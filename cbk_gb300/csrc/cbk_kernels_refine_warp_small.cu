// cbk_kernels_refine_warp_small.cu -- the mixed-precision SPD solve for
// orders 17 .. 64 (the kernel: cbk_refine_warp.cuh) with two matrices or one
// matrix per block: the autotuner's variants 2 and 3 of posv_refined. The
// resident warps per SM are those of the four-matrix shape (the register cap
// of each shape is set for the same count), so only the grain changes: a
// smaller block frees its shared memory as soon as its own matrices are done,
// at the cost of staging loads that fill half or a quarter of a 32-byte sector.
#include "cbk_refine_warp.cuh"

namespace cbkcuda {

cudaError_t launch_posv_refined_warp_small(int wpb, bool row, bool up, int n, int nrhs,
                                           double *ap, int ldap, double *bp, int ldbp, int V,
                                           int nm, int max_iter, int *iters, double *berr,
                                           cudaStream_t s, size_t sa, size_t sb)
{
    const WarpOut out{iters, berr, nm, max_iter};
    // B: the four-matrix shape's blocks per SM; 32 blocks is the SM's limit
#define CBK_WARP(N, B)                                                                             \
    return wpb == 2 ? launch_warp<N, 2, 2 * B>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s, \
                                               sa, sb)                                             \
                    : launch_warp<N, 1, (4 * B < 32 ? 4 * B : 32)>(row, up, n, nrhs, ap, ldap, bp,  \
                                                                   ldbp, V, nm, out, s, sa, sb)
    switch ((n + 7) / 8) {
    case 3: CBK_WARP(24, 6);
    case 4: CBK_WARP(32, 7);
    case 5: CBK_WARP(40, 4);
    case 6: CBK_WARP(48, 4);
    case 7: CBK_WARP(56, 3);
    default: CBK_WARP(64, 3);
    }
#undef CBK_WARP
}

} // namespace cbkcuda
