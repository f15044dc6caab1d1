// cbk_kernels_bucketed.cu -- one persistent launch for batches of uneven
// orders: LDL^T factor + solve (?sysvnp) and Cholesky factor + solve (?posv)
// over a table of buckets, each bucket an ordinary compact batch of one order.
//
// No counterpart in the reference, which takes one order per call
// (src/cbk_sysvnp_compact.hpp:38-65); a batch of mixed orders there is one
// call per order. Here the work of every bucket is cut into 32-lane items
// (one warp each), ordered largest order first, and a grid of one wave of
// warps (SMs x resident warps) pulls items from a device counter until none
// are left: the costliest items start first and the short ones fill the tail,
// so no SM idles while another still has a large matrix to factor. The loop
// ends when the counter passes the item count -- there is no waiting on other
// warps and nothing to hang on. Each lane runs the same per-lane code as the
// single-order kernels, so a bucket's results are bit-identical to a
// ?sysvnp_compact (?posv_compact) call on that bucket alone.
#include "../../include/cbk_cuda.h"
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace cbkcuda {
using namespace cbkdev;

namespace {

constexpr int MAX_BUCKETS = CBK_CUDA_MAX_BUCKETS;

template <typename T> struct BucketTable {
    int nb;               // buckets, sorted by decreasing order
    long items;           // total 32-lane items
    long first[MAX_BUCKETS + 1]; // first item of each bucket
    int n[MAX_BUCKETS], V[MAX_BUCKETS], ldap[MAX_BUCKETS], ldbp[MAX_BUCKETS];
    long lanes[MAX_BUCKETS];     // padded lanes of the bucket
    size_t sa[MAX_BUCKETS], sb[MAX_BUCKETS];
    T *ap[MAX_BUCKETS];
    T *bp[MAX_BUCKETS];
};

template <typename T, bool LDLT>
__global__ void __launch_bounds__(128) k_bucketed(const __grid_constant__ BucketTable<T> tab,
                                                  bool row, bool up, int nrhs,
                                                  unsigned long long *counter)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(counter, 1ull);
        item = __shfl_sync(0xffffffffu, item, 0);
        if ((long)item >= tab.items) return;
        int b = 0;
        while (b + 1 < tab.nb && (long)item >= tab.first[b + 1])
            ++b;
        const long l = ((long)item - tab.first[b]) * 32 + lane;
        if (l >= tab.lanes[b]) continue;
        const int V = tab.V[b], n = tab.n[b];
        const long g = l / V;
        const int v = (int)(l - g * V);
        LV<T> A = lv_make<T>(tab.ap[b] + g * tab.sa[b] + v, row, tab.ldap[b], V, n, n);
        if (up) A = A.t();
        // FP32: the in-memory panel sweep (the same bits), which keeps this
        // kernel at its former 128 registers (the register sweep took it to
        // 168 with spills in the Cholesky instance)
        factor_lane<T, LDLT, sizeof(T) == 4>(n, A);
        if (nrhs > 0)
            sym_solve_lane<T, LDLT>(n, nrhs, A,
                                    lv_make<T>(tab.bp[b] + g * tab.sb[b] + v, row, tab.ldbp[b], V, n, nrhs));
    }
}

template <typename T, bool LDLT>
int resident_warps()
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bucketed<T, LDLT>, 128, 0);
    return sms * std::max(1, per_sm) * 4;
}

} // namespace

template <typename T>
cudaError_t launch_bucketed(bool ldlt, bool row, bool up, int nrhs, int nbuckets, const int *n,
                            const int *nm, const int *V, T *const *ap, const int *ldap,
                            T *const *bp, const int *ldbp, void *work, cudaStream_t s)
{
    std::vector<int> order;
    for (int b = 0; b < nbuckets; ++b)
        if (n[b] > 0 && nm[b] > 0) order.push_back(b);
    if (order.empty()) return cudaSuccess;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
    BucketTable<T> tab;
    std::memset(&tab, 0, sizeof(tab));
    tab.nb = (int)order.size();
    long items = 0;
    for (int k = 0; k < tab.nb; ++k) {
        const int b = order[k];
        const long lanes = (((long)nm[b] + V[b] - 1) / V[b]) * V[b];
        tab.first[k] = items;
        items += (lanes + 31) / 32;
        tab.n[k] = n[b];
        tab.V[k] = V[b];
        tab.ldap[k] = ldap[b];
        tab.ldbp[k] = ldbp[b];
        tab.lanes[k] = lanes;
        tab.sa[k] = gstride(row, ldap[b], n[b], n[b], V[b]);
        tab.sb[k] = gstride(row, ldbp[b], n[b], nrhs, V[b]);
        tab.ap[k] = ap[b];
        tab.bp[k] = bp[b];
    }
    tab.first[tab.nb] = items;
    tab.items = items;
    auto *counter = static_cast<unsigned long long *>(work);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    // the persistent grid: one wave of warps, or that halved `variant` times
    // (fewer matrices in flight: a smaller working set in the L2 cache for the
    // large orders, against less latency hiding); the variant is tuned per
    // largest order
    const int variant = variant_for(ldlt ? R_SYSVNP_BUCKETED : R_POSV_BUCKETED, tab.n[0],
                                    (int)sizeof(T));
    const int warps = (ldlt ? resident_warps<T, true>() : resident_warps<T, false>()) >> variant;
    const long want = std::min<long>(items, std::max(warps, 4));
    const unsigned blocks = (unsigned)((want + 3) / 4);
    if (ldlt)
        k_bucketed<T, true><<<blocks, 128, 0, s>>>(tab, row, up, nrhs, counter);
    else
        k_bucketed<T, false><<<blocks, 128, 0, s>>>(tab, row, up, nrhs, counter);
    return cudaGetLastError();
}

template cudaError_t launch_bucketed<float>(bool, bool, bool, int, int, const int *, const int *,
                                            const int *, float *const *, const int *,
                                            float *const *, const int *, void *, cudaStream_t);
template cudaError_t launch_bucketed<double>(bool, bool, bool, int, int, const int *, const int *,
                                             const int *, double *const *, const int *,
                                             double *const *, const int *, void *, cudaStream_t);

} // namespace cbkcuda
