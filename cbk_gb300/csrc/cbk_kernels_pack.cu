// cbk_kernels_pack.cu -- device conversion between a dense batch (one matrix
// after another, LAPACK storage) and the compact layout, the device-side form
// of the reference tests' pack_compact / unpack_compact
// (tests/test_compact_util.hpp:477-531): padded lanes of a partial last group
// receive pad_diag on the diagonal and zero elsewhere.
//
// Memory-bound transposes. A block stages a 32-lane x 32-element tile in
// shared memory: the dense side is read (or written) 32 consecutive elements
// of one matrix at a time, the compact side 32 consecutive lanes of one
// element at a time, so both sides are coalesced. Elements are numbered in the
// dense matrix's own storage order (column-major: e = i + j*m; row-major:
// e = i*n + j), which keeps the dense side contiguous when lda is the
// matrix's extent.
#include "cbk_device.cuh"
#include "cbk_launch.h"

#include <algorithm>

namespace cbkcuda {

namespace {

constexpr int TILE = 32;
constexpr int ROWS = 8; // block = TILE x ROWS threads

struct PackGeom {
    int m, n, lda, ldap, V, nm;
    long long stride;
    bool row;
    long nelem;  // m * n
    long nlanes; // padded lane count
    size_t gs;   // scalars per compact group
};

// Element e -> (i, j) in the dense storage order.
__device__ __forceinline__ void elem_ij(const PackGeom &G, long e, int &i, int &j)
{
    if (G.row) {
        i = (int)(e / G.n);
        j = (int)(e - (long)i * G.n);
    }
    else {
        j = (int)(e / G.m);
        i = (int)(e - (long)j * G.m);
    }
}

__device__ __forceinline__ size_t dense_off(const PackGeom &G, long mat, int i, int j)
{
    return (size_t)mat * (size_t)G.stride +
           (G.row ? (size_t)i * G.lda + j : (size_t)j * G.lda + i);
}

__device__ __forceinline__ size_t compact_off(const PackGeom &G, long lane, int i, int j)
{
    const long g = lane / G.V;
    const int v = (int)(lane - g * G.V);
    const size_t in = G.row ? (size_t)i * G.ldap + j : (size_t)j * G.ldap + i;
    return (size_t)g * G.gs + in * (size_t)G.V + v;
}

// grid: x over lane tiles, y over element tiles
template <typename T>
__global__ void k_pack(PackGeom G, const T *__restrict__ a, T *__restrict__ ap, T pad_diag)
{
    __shared__ T tile[TILE][TILE + 1];
    const long e0 = (long)blockIdx.y * TILE;
    const long l0 = (long)blockIdx.x * TILE;
    // read: lane l0+r, elements e0 .. e0+31 (consecutive threads, consecutive elements)
    for (int r = threadIdx.y; r < TILE; r += ROWS) {
        const long lane = l0 + r;
        const long e = e0 + threadIdx.x;
        T x = T(0);
        if (lane < G.nlanes && e < G.nelem) {
            int i, j;
            elem_ij(G, e, i, j);
            if (lane < G.nm)
                x = a[dense_off(G, lane, i, j)];
            else
                x = (i == j) ? pad_diag : T(0);
        }
        tile[r][threadIdx.x] = x;
    }
    __syncthreads();
    // write: element e0+r, lanes l0 .. l0+31 (consecutive threads, consecutive lanes)
    for (int r = threadIdx.y; r < TILE; r += ROWS) {
        const long e = e0 + r;
        const long lane = l0 + threadIdx.x;
        if (lane < G.nlanes && e < G.nelem) {
            int i, j;
            elem_ij(G, e, i, j);
            ap[compact_off(G, lane, i, j)] = tile[threadIdx.x][r];
        }
    }
}

template <typename T>
__global__ void k_unpack(PackGeom G, const T *__restrict__ ap, T *__restrict__ a)
{
    __shared__ T tile[TILE][TILE + 1];
    const long e0 = (long)blockIdx.y * TILE;
    const long l0 = (long)blockIdx.x * TILE;
    for (int r = threadIdx.y; r < TILE; r += ROWS) {
        const long e = e0 + r;
        const long lane = l0 + threadIdx.x;
        T x = T(0);
        if (lane < G.nm && e < G.nelem) {
            int i, j;
            elem_ij(G, e, i, j);
            x = ap[compact_off(G, lane, i, j)];
        }
        tile[threadIdx.x][r] = x;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < TILE; r += ROWS) {
        const long lane = l0 + r;
        const long e = e0 + threadIdx.x;
        if (lane < G.nm && e < G.nelem) {
            int i, j;
            elem_ij(G, e, i, j);
            a[dense_off(G, lane, i, j)] = tile[r][threadIdx.x];
        }
    }
}

PackGeom make_geom(bool row, int m, int n, int lda, long long stride, int ldap, int V, int nm)
{
    PackGeom G;
    G.m = m;
    G.n = n;
    G.lda = lda;
    G.ldap = ldap;
    G.V = V;
    G.nm = nm;
    G.stride = stride;
    G.row = row;
    G.nelem = (long)m * n;
    G.nlanes = (((long)nm + V - 1) / V) * V;
    G.gs = cbkdev::gstride(row, ldap, m, n, V);
    return G;
}

// The referenced triangle of every n x n matrix of `groups` compact groups:
// run k (a column of a column-major lower / row-major upper triangle from the
// diagonal on, or of the opposite pair up to the diagonal) is contiguous, so a
// warp copies it with 16-byte moves, four loads in flight per lane before
// their stores; dst has src's layout. Either side may be host memory the
// device can address (pinned): the copy then runs over the host link at its
// full rate with half the bytes of the whole matrices. Over the link a load
// takes microseconds, so the bytes in flight set the rate, and with four per
// lane one block per two SMs fills the link. The grid is that small and
// persistent: it runs beside a solve that fills the rest of the GPU (a grid
// of one block per run would wait for the solve's blocks to drain), and it
// takes few of the solve's SM slots (measured: two blocks per SM slowed the
// solves beside it until they, not the link, set the pace).
__global__ void __launch_bounds__(256)
    k_tri_copy(const double *__restrict__ src, double *__restrict__ dst, bool from_diag, int n,
               int ld, int V, long groups, long gstride)
{
    constexpr int UNROLL = 4;
    const long runs = groups * n;
    const int lane = threadIdx.x & 31;
    const long wpb = blockDim.x >> 5;
    for (long b = blockIdx.x * wpb + (threadIdx.x >> 5); b < runs; b += gridDim.x * wpb) {
        const long g = b / n;
        const int k = (int)(b - g * n);
        const long start = ((long)k * ld + (from_diag ? k : 0)) * V;
        const long len2 = (long)(from_diag ? n - k : k + 1) * V / 2; // V is even
        const double2 *s = reinterpret_cast<const double2 *>(src + g * gstride + start);
        double2 *d = reinterpret_cast<double2 *>(dst + g * gstride + start);
        for (long i = lane; i < len2; i += 32 * UNROLL) {
            double2 v[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u)
                if (i + 32 * u < len2) v[u] = s[i + 32 * u];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u)
                if (i + 32 * u < len2) d[i + 32 * u] = v[u];
        }
    }
}

} // namespace

cudaError_t launch_tri_copy(bool row, bool up, int n, int ld, int V, long groups,
                            const double *src, double *dst, cudaStream_t s)
{
    if (groups <= 0 || n <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long blocks = std::min<long>(groups * n, std::max(sms / 2, 1));
    k_tri_copy<<<(unsigned)blocks, 256, 0, s>>>(src, dst, row == up, n, ld, V, groups,
                                                (long)ld * n * V);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pack(bool row, int m, int n, const T *a, int lda, long long stride, T *ap,
                        int ldap, int V, int nm, T pad_diag, cudaStream_t s)
{
    const PackGeom G = make_geom(row, m, n, lda, stride, ldap, V, nm);
    const dim3 grid((unsigned)((G.nlanes + TILE - 1) / TILE), (unsigned)((G.nelem + TILE - 1) / TILE));
    k_pack<T><<<grid, dim3(TILE, ROWS), 0, s>>>(G, a, ap, pad_diag);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_unpack(bool row, int m, int n, const T *ap, int ldap, T *a, int lda,
                          long long stride, int V, int nm, cudaStream_t s)
{
    const PackGeom G = make_geom(row, m, n, lda, stride, ldap, V, nm);
    const dim3 grid((unsigned)((nm + TILE - 1) / TILE), (unsigned)((G.nelem + TILE - 1) / TILE));
    k_unpack<T><<<grid, dim3(TILE, ROWS), 0, s>>>(G, ap, a);
    return cudaGetLastError();
}

template cudaError_t launch_pack<float>(bool, int, int, const float *, int, long long, float *, int,
                                        int, int, float, cudaStream_t);
template cudaError_t launch_pack<double>(bool, int, int, const double *, int, long long, double *,
                                         int, int, int, double, cudaStream_t);
template cudaError_t launch_unpack<float>(bool, int, int, const float *, int, float *, int,
                                          long long, int, int, cudaStream_t);
template cudaError_t launch_unpack<double>(bool, int, int, const double *, int, double *, int,
                                           long long, int, int, cudaStream_t);

} // namespace cbkcuda
