// cbk_host.cpp -- the refined SPD solve on host-memory batches: the copies
// in and out pipelined with the solves.
//
// The reference's calling convention keeps every array in host memory
// (include/cbk.h:196-212, its MKL-style adapter src/cbk_compat.cpp copies
// nothing because its kernels run on the CPU). Here a host batch is cut into
// chunks of whole groups that flow through NBUF device slots, each slot on its
// own stream: while one chunk is solved, the next one is copied in and the
// previous one out, so the time is close to that of the copies alone.
// When A is in pinned host memory the device reads it directly: a kernel
// gathers only the referenced triangle (half of A's bytes) over the host link,
// which its 16-byte loads of whole contiguous runs drive at the link's full
// rate (2-D copies of the same runs by the copy engine measured three times
// slower). Otherwise (pageable memory) a chunk's groups, contiguous in the
// compact layout, move as one copy. B moves as one contiguous copy each way.
// A goes back to the host only for a chunk in which some lane fell back to
// the FP64 path (those lanes then hold the FP64 factor, the others the
// unchanged input) -- by the same triangle kernel when A is pinned -- so the
// results in host memory are exactly the device entry point's.
#include "cbk_launch.h"

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

namespace cbkcuda {

namespace {

constexpr int NBUF = 3;
// A chunk moves about CHUNK_BYTES over the link (A's triangle and B), and
// holds at least MIN_CHUNK_GROUPS groups, so its solve fills the GPU. Each
// chunk costs the copy stream some tens of microseconds beyond its bytes
// (launch, the copy kernel's tail, the DMA of B), so chunks are large:
// measured at 262,144 matrices, 192 MiB chunks took n = 32 from 6.51 to
// 6.31 ms and n = 48 from 13.3 to 13.0 ms against 48 MiB ones. The first and
// the last chunk move about RAMP_BYTES (at least MIN_RAMP_GROUPS groups): the
// first solve starts after a short copy, and the last copy leaves a short
// solve.
constexpr size_t CHUNK_BYTES = (size_t)192 << 20;
constexpr size_t RAMP_BYTES = (size_t)12 << 20;
constexpr long MIN_CHUNK_GROUPS = 256;
constexpr long MIN_RAMP_GROUPS = 64;

inline size_t align256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

struct Plan {
    long ngroups, chunk, ramp; // groups in the batch, per chunk (a slot), in the first and last
    size_t ga, gb;             // bytes of one group of A and of B
    size_t a, b, it, be, cnt, ws, slot; // bytes of each part of one slot

    // the size of the chunk that starts at group g0: the first is `ramp`,
    // then `chunk` while more than chunk + ramp remain, then the rest but
    // `ramp`, then `ramp`
    long at(long g0) const
    {
        const long left = ngroups - g0;
        if (g0 == 0 || left <= ramp) return std::min(left, ramp);
        if (left > chunk + ramp) return chunk;
        return left - ramp;
    }
};

Plan plan(bool row, int n, int nrhs, int ldap, int ldbp, int V, int nm)
{
    Plan p{};
    p.ngroups = ((long)nm + V - 1) / V;
    p.ga = (size_t)ldap * n * V * sizeof(double);
    p.gb = (size_t)ldbp * (row ? n : nrhs) * V * sizeof(double);
    const size_t moved = (size_t)n * (n + 1) / 2 * V * sizeof(double) + p.gb;
    const long want = (long)((CHUNK_BYTES + moved - 1) / moved);
    p.chunk = std::min(p.ngroups, std::max(MIN_CHUNK_GROUPS, want));
    p.ramp = std::min(p.chunk, std::max(MIN_RAMP_GROUPS, (long)((RAMP_BYTES + moved - 1) / moved)));
    // CBK_CUDA_HOST_CHUNK_GROUPS=g (read on every call, and by the workspace
    // query): chunks of g groups, the first and last g / 4 -- for tests of
    // the pipeline's chunking on small batches, or a caller's own tuning
    if (const char *e = std::getenv("CBK_CUDA_HOST_CHUNK_GROUPS")) {
        const long g = std::strtol(e, nullptr, 10);
        if (g > 0) {
            p.chunk = std::min(p.ngroups, g);
            p.ramp = std::min(p.chunk, std::max(1L, g / 4));
        }
    }
    const size_t lanes = (size_t)p.chunk * V;
    p.a = align256(p.chunk * p.ga);
    p.b = align256(p.chunk * p.gb);
    p.it = align256(lanes * sizeof(int));
    p.be = align256(lanes * sizeof(double));
    p.cnt = 256;
    p.ws = align256(posv_refined_lwork(n, nrhs, V, (int)lanes));
    p.slot = p.a + p.b + p.it + p.be + p.cnt + p.ws;
    return p;
}

} // namespace

size_t posv_refined_host_lwork(bool row, int n, int nrhs, int ldap, int ldbp, int V, int nm)
{
    if (n <= 0 || nrhs <= 0 || nm <= 0) return 0;
    return (size_t)NBUF * plan(row, n, nrhs, ldap, ldbp, V, nm).slot;
}

cudaError_t posv_refined_host(bool row, bool up, int n, int nrhs, double *ap, int ldap, double *bp,
                              int ldbp, int V, int nm, int max_iter, int *iters, double *berr,
                              void *dwork, cudaStream_t caller)
{
    const Plan p = plan(row, n, nrhs, ldap, ldbp, V, nm);
    char *const ha = reinterpret_cast<char *>(ap);
    char *const hb = reinterpret_cast<char *>(bp);
    // pinned (or registered) A, 16-byte aligned: the device address the
    // triangle kernel reads with 16-byte moves (every chunk starts a whole
    // number of groups on, a multiple of 16 bytes since V is even); an A
    // that is only 8-byte aligned goes by the copy engine
    double *zc = nullptr;
    {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, ap) == cudaSuccess && at.type == cudaMemoryTypeHost &&
            at.devicePointer != nullptr && reinterpret_cast<uintptr_t>(at.devicePointer) % 16 == 0)
            zc = static_cast<double *>(at.devicePointer);
        cudaGetLastError(); // a pageable pointer is not an error
    }
    const size_t ga_doubles = p.ga / sizeof(double);

    struct Slot {
        cudaStream_t s = nullptr;
        cudaEvent_t ready = nullptr; // the chunk's inputs are in the slot
        double *a, *b, *be;
        int *it, *cnt;
        void *ws;
        long g0 = -1, groups = 0; // the chunk in the slot (-1: none)
    } slot[NBUF];
    char *base = static_cast<char *>(dwork);
    for (int k = 0; k < NBUF; ++k) {
        char *q = base + (size_t)k * p.slot;
        slot[k].a = reinterpret_cast<double *>(q);
        slot[k].b = reinterpret_cast<double *>(q + p.a);
        slot[k].it = reinterpret_cast<int *>(q + p.a + p.b);
        slot[k].be = reinterpret_cast<double *>(q + p.a + p.b + p.it);
        slot[k].cnt = reinterpret_cast<int *>(q + p.a + p.b + p.it + p.be);
        slot[k].ws = p.ws ? q + p.a + p.b + p.it + p.be + p.cnt : nullptr;
    }

    cudaError_t err = cudaSuccess;
    cudaEvent_t start = nullptr, solved = nullptr;
    auto keep = [&](cudaError_t e) {
        if (err == cudaSuccess && e != cudaSuccess) err = e;
        return err == cudaSuccess;
    };
    // The inputs move on one stream of the highest priority, the solves and
    // the outputs on one stream per slot: a solve launched first would
    // otherwise keep the GPU until its last block is dispatched, and the copy
    // of the next chunk (a persistent kernel) must get the resources its
    // blocks free. All streams start after the caller's prior work on its
    // stream.
    cudaStream_t in = nullptr;
    int lo_prio = 0, hi_prio = 0;
    keep(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    keep(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    keep(cudaEventCreateWithFlags(&solved, cudaEventDisableTiming));
    if (err == cudaSuccess) keep(cudaEventRecord(start, caller));
    if (err == cudaSuccess &&
        keep(cudaStreamCreateWithPriority(&in, cudaStreamNonBlocking, hi_prio)))
        keep(cudaStreamWaitEvent(in, start, 0));
    for (int k = 0; k < NBUF && err == cudaSuccess; ++k)
        if (keep(cudaStreamCreateWithFlags(&slot[k].s, cudaStreamNonBlocking)) &&
            keep(cudaEventCreateWithFlags(&slot[k].ready, cudaEventDisableTiming)))
            keep(cudaStreamWaitEvent(slot[k].s, start, 0));

    // a chunk is finished once its stream is idle; if one of its lanes fell
    // back, its A goes back to the host too
    auto finish = [&](Slot &sl) {
        if (sl.g0 < 0) return;
        if (!keep(cudaStreamSynchronize(sl.s))) return;
        int fell = 0;
        if (keep(cudaMemcpyAsync(&fell, sl.cnt, sizeof(int), cudaMemcpyDeviceToHost, sl.s)) &&
            keep(cudaStreamSynchronize(sl.s)) && fell > 0) {
            if (zc)
                keep(launch_tri_copy(row, up, n, ldap, V, sl.groups, sl.a,
                                     zc + (size_t)sl.g0 * ga_doubles, sl.s));
            else
                keep(cudaMemcpyAsync(ha + (size_t)sl.g0 * p.ga, sl.a, (size_t)sl.groups * p.ga,
                                     cudaMemcpyDeviceToHost, sl.s));
            keep(cudaStreamSynchronize(sl.s));
        }
        sl.g0 = -1;
    };

    for (long g0 = 0, c = 0, groups = 0; g0 < p.ngroups && err == cudaSuccess;
         g0 += groups, ++c) {
        Slot &sl = slot[c % NBUF];
        finish(sl);
        if (err != cudaSuccess) break;
        groups = p.at(g0);
        const long lane0 = g0 * V;
        const int nmc = (int)std::min((long)nm - lane0, groups * V);
        // the slot is idle (finish), so its inputs may be overwritten now
        keep(cudaMemsetAsync(sl.cnt, 0, sizeof(int), in));
        if (zc)
            keep(launch_tri_copy(row, up, n, ldap, V, groups, zc + (size_t)g0 * ga_doubles, sl.a,
                                 in));
        else
            keep(cudaMemcpyAsync(sl.a, ha + (size_t)g0 * p.ga, (size_t)groups * p.ga,
                                 cudaMemcpyHostToDevice, in));
        keep(cudaMemcpyAsync(sl.b, hb + (size_t)g0 * p.gb, (size_t)groups * p.gb,
                             cudaMemcpyHostToDevice, in));
        keep(cudaEventRecord(sl.ready, in));
        keep(cudaStreamWaitEvent(sl.s, sl.ready, 0));
        // the solves run one after another in chunk order: solves that
        // overlap each finish late, and a slot is free only when its chunk is
        if (c > 0) keep(cudaStreamWaitEvent(sl.s, solved, 0));
        keep(launch_posv_refined(row, up, n, nrhs, sl.a, ldap, sl.b, ldbp, V, nmc, max_iter, sl.it,
                                 berr ? sl.be : nullptr, sl.ws, sl.s));
        keep(launch_count_negative(sl.it, nmc, sl.cnt, sl.s));
        keep(cudaEventRecord(solved, sl.s));
        keep(cudaMemcpyAsync(hb + (size_t)g0 * p.gb, sl.b, (size_t)groups * p.gb,
                             cudaMemcpyDeviceToHost, sl.s));
        if (iters)
            keep(cudaMemcpyAsync(iters + lane0, sl.it, (size_t)nmc * sizeof(int),
                                 cudaMemcpyDeviceToHost, sl.s));
        if (berr)
            keep(cudaMemcpyAsync(berr + lane0, sl.be, (size_t)nmc * sizeof(double),
                                 cudaMemcpyDeviceToHost, sl.s));
        sl.g0 = g0;
        sl.groups = groups;
    }
    for (int k = 0; k < NBUF; ++k)
        if (err == cudaSuccess) finish(slot[k]);
    if (in) {
        cudaStreamSynchronize(in);
        cudaStreamDestroy(in);
    }
    for (int k = 0; k < NBUF; ++k) {
        if (slot[k].s) {
            cudaStreamSynchronize(slot[k].s);
            cudaStreamDestroy(slot[k].s);
        }
        if (slot[k].ready) cudaEventDestroy(slot[k].ready);
    }
    if (start) cudaEventDestroy(start);
    if (solved) cudaEventDestroy(solved);
    return err;
}

} // namespace cbkcuda
