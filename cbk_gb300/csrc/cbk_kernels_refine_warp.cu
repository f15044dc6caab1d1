// cbk_kernels_refine_warp.cu -- launches of the mixed-precision SPD solve for
// orders 17 .. 64, one warp per matrix (the kernel: cbk_refine_warp.cuh), with
// four matrices per block; the two-matrix and one-matrix block shapes are
// compiled in cbk_kernels_refine_warp_small.cu (a separate translation unit,
// so that the two compile in parallel).
#include "cbk_refine_warp.cuh"

namespace cbkcuda {

// orders the warp-per-matrix variant takes
bool posv_refined_warp_ok(int n)
{
    return n > 16 && n <= 64;
}

cudaError_t launch_posv_refined_warp(bool row, bool up, int n, int nrhs, double *ap, int ldap,
                                     double *bp, int ldbp, int V, int nm, int max_iter,
                                     int *iters, double *berr, cudaStream_t s, size_t sa_,
                                     size_t sb_)
{
    const WarpOut out{iters, berr, nm, max_iter};
    const size_t sa = sa_ ? sa_ : gstride(row, ldap, n, n, V);
    const size_t sb = sb_ ? sb_ : gstride(row, ldbp, n, nrhs, V);
    // The tuned variant picks the block shape; every shape gives the same bits.
    //   0: four matrices per block (the staging loads then fill 32-byte
    //      sectors), the last template argument capping the registers for the
    //      resident blocks wanted (measured: at n = 32 seven blocks beat six
    //      and five despite spills, at n = 48 four beat five);
    //   1: the same with one block more per SM (fewer registers per thread);
    //   2: two matrices per block, twice the blocks (a block's shared memory
    //      is freed as soon as its two matrices are done);
    //   3: one matrix per block.
    // The order is padded to a multiple of 8.
    const int variant = variant_for(R_POSV_REFINED, n, 8);
    if (variant >= 2)
        return launch_posv_refined_warp_small(variant == 2 ? 2 : 1, row, up, n, nrhs, ap, ldap, bp,
                                              ldbp, V, out.nm, out.max_iter, out.iters, out.berr,
                                              s, sa, sb);
    const bool more = variant == 1;
#define CBK_WARP(N, B)                                                                             \
    return more ? launch_warp<N, 4, B + 1>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s, sa, \
                                           sb)                                                     \
                : launch_warp<N, 4, B>(row, up, n, nrhs, ap, ldap, bp, ldbp, V, nm, out, s, sa, sb)
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
