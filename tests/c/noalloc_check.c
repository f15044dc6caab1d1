/* The no-allocation refined solve: its refusal to make a first address
 * lookup under stream capture, and its results in more than one CUDA context
 * of a device.
 *
 * A caller that cannot allocate may also own its CUDA contexts (a driver-API
 * host makes its own with cuCtxCreate). The library's scratch array has a
 * different address in each context, so each context's first n > 64 call
 * must look it up there. This program solves the same order-80 batch:
 *   1. in the device's primary context, first on a stream being captured --
 *      before any n > 64 call, so the call must return
 *      CBK_CUDA_NOALLOC_IN_CAPTURE and enqueue nothing -- then outside it;
 *   2. there again, through the workspace entry point (the reference result),
 *      and once more through the no-allocation one;
 *   3. in a second context of the same device made current by cuCtxCreate,
 *      where the GPU allows one (a device in exclusive-process compute mode
 *      does not: that step is then reported and skipped).
 * Every solution, iteration count and backward error must equal the
 * workspace entry point's bit for bit. The driver functions are resolved
 * through the runtime (no link-time libcuda). Exit code 0 and "noalloc ok"
 * when every check passes. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "cbk_cuda.h"

enum { N = 80, V = 32, NM = 300 };
#define NG ((NM + V - 1) / V)
#define ASZ ((size_t)NG * N * N * V)
#define BSZ ((size_t)NG * N * V)

typedef int (*ctx_create_fn)(void **ctx, unsigned int flags, int dev);
typedef int (*ctx_destroy_fn)(void *ctx);

static double next(unsigned long long *s)
{
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(*s >> 11) / 9007199254740992.0 - 0.5;
}

#define CK(x)                                                                            \
    do {                                                                                 \
        cudaError_t e_ = (x);                                                            \
        if (e_ != cudaSuccess) {                                                         \
            printf("%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_));    \
            exit(2);                                                                     \
        }                                                                                \
    } while (0)

struct result {
    double x[BSZ];
    int it[NM];
    double be[NM];
};

/* one solve of the host batch (A, B) in the current context; noalloc selects
 * the entry point; capture: begin a capture first and expect the refusal */
static int solve(const double *A, const double *B, int noalloc, int capture, struct result *r)
{
    double *da, *db, *dberr;
    int *dit;
    void *work = NULL;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaMalloc((void **)&da, ASZ * sizeof(double)));
    CK(cudaMalloc((void **)&db, BSZ * sizeof(double)));
    CK(cudaMalloc((void **)&dit, NM * sizeof(int)));
    CK(cudaMalloc((void **)&dberr, NM * sizeof(double)));
    CK(cudaMemcpy(da, A, ASZ * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(db, B, BSZ * sizeof(double), cudaMemcpyHostToDevice));
    const long long lw = cbk_cuda_dposv_refined_compact_lwork(N, 1, V, NM);
    int info;
    if (capture) {
        cudaGraph_t g = NULL;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        info = cbk_cuda_dposv_refined_compact_noalloc_async('C', 'L', N, 1, da, N, db, N, V, NM,
                                                            10, dit, dberr, st);
        CK(cudaStreamEndCapture(st, &g));
        if (g) CK(cudaGraphDestroy(g));
        if (info != CBK_CUDA_NOALLOC_IN_CAPTURE) {
            printf("capture: expected %d, got %d\n", CBK_CUDA_NOALLOC_IN_CAPTURE, info);
            return 1;
        }
    }
    if (noalloc) {
        info = cbk_cuda_dposv_refined_compact_noalloc_async('C', 'L', N, 1, da, N, db, N, V, NM,
                                                            10, dit, dberr, st);
    }
    else {
        CK(cudaMalloc(&work, (size_t)lw));
        info = cbk_cuda_dposv_refined_compact_async('C', 'L', N, 1, da, N, db, N, V, NM, 10, dit,
                                                    dberr, work, lw, st);
    }
    CK(cudaStreamSynchronize(st));
    CK(cudaMemcpy(r->x, db, BSZ * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r->it, dit, NM * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r->be, dberr, NM * sizeof(double), cudaMemcpyDeviceToHost));
    if (work) CK(cudaFree(work));
    CK(cudaFree(da));
    CK(cudaFree(db));
    CK(cudaFree(dit));
    CK(cudaFree(dberr));
    CK(cudaStreamDestroy(st));
    if (info != 0) printf("solve: info %d (%s)\n", info, cbk_cuda_status_string(info));
    return info != 0;
}

static int same(const char *what, const struct result *a, const struct result *b)
{
    if (memcmp(a->x, b->x, sizeof a->x) || memcmp(a->it, b->it, sizeof a->it) ||
        memcmp(a->be, b->be, sizeof a->be)) {
        printf("%s: results differ from the workspace entry point's\n", what);
        return 1;
    }
    return 0;
}

int main(void)
{
    static double A[ASZ], B[BSZ];
    static struct result ref, got;
    unsigned long long s = 2027;
    /* diagonally dominant SPD batch, compact column-major, padded lanes I */
    for (int k = 0; k < NG * V; ++k) {
        const int g = k / V, v = k % V;
        for (int j = 0; j < N; ++j)
            for (int i = j; i < N; ++i) {
                const double a = k < NM ? (i == j ? 2.0 * N : next(&s)) : (i == j ? 1.0 : 0.0);
                A[(size_t)g * N * N * V + ((size_t)j * N + i) * V + v] = a;
                A[(size_t)g * N * N * V + ((size_t)i * N + j) * V + v] = a;
            }
        for (int i = 0; i < N; ++i) B[(size_t)g * N * V + (size_t)i * V + v] = k < NM ? next(&s) : 0;
    }
    int bad = 0;
    CK(cudaSetDevice(0));
    {   /* initialise the library's runtime with a call that needs no scratch:
         * one 1 x 1 system in a group of width 2, A = (4, pad 1), B = (2, 0) */
        double *one;
        CK(cudaMalloc((void **)&one, 4 * sizeof(double)));
        const double h[4] = {4.0, 1.0, 2.0, 0.0};
        CK(cudaMemcpy(one, h, sizeof h, cudaMemcpyHostToDevice));
        if (cbk_cuda_dposv_compact('C', 'L', 1, 1, one, 1, one + 2, 1, 2, 1) != 0) bad = 1;
        CK(cudaDeviceSynchronize());
        CK(cudaFree(one));
    }
    bad |= solve(A, B, 1, 1, &got);
    bad |= solve(A, B, 0, 0, &ref);
    bad |= same("primary context, after a refused capture", &ref, &got);
    bad |= solve(A, B, 1, 0, &got) || same("primary context, second call", &ref, &got);

    ctx_create_fn create = NULL;
    ctx_destroy_fn destroy = NULL;
    enum cudaDriverEntryPointQueryResult q;
    CK(cudaGetDriverEntryPointByVersion("cuCtxCreate", (void **)&create, 12000, cudaEnableDefault,
                                        &q));
    CK(cudaGetDriverEntryPointByVersion("cuCtxDestroy", (void **)&destroy, 12000,
                                        cudaEnableDefault, &q));
    if (!create || !destroy) {
        printf("driver context functions unavailable\n");
        return 3;
    }
    void *c2 = NULL;
    const int rc = create(&c2, 0, 0);
    if (rc != 0) {
        printf("note: no second context on this device (cuCtxCreate %d): step 3 skipped\n", rc);
    }
    else {
        bad |= solve(A, B, 1, 0, &got) || same("second context", &ref, &got);
        bad |= solve(A, B, 1, 0, &got) || same("second context, second call", &ref, &got);
        destroy(c2);
        bad |= solve(A, B, 1, 0, &got) || same("primary context again", &ref, &got);
    }
    if (bad) return 1;
    printf("noalloc ok\n");
    return 0;
}
