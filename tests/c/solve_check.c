/* A C caller moving a cbk_dposv_compact call site to the GPU: a compact
 * batch built on the host (include/cbk.h's layout), copied to the device,
 * solved by cbk_cuda_dposv_compact and by the mixed-precision
 * cbk_cuda_dposv_refined_compact, copied back and checked on the host by its
 * normwise backward error. Exit code 0 when both solves meet 8 n eps. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "cbk_cuda.h"

enum { N = 12, NRHS = 2, V = 32, NM = 100 };

/* element (i, j) of matrix k in the compact column-major layout, ld = N */
static size_t at(int k, int i, int j, int cols)
{
    const int g = k / V, v = k % V;
    return (size_t)g * N * cols * V + ((size_t)j * N + i) * V + v;
}

static double next(unsigned long long *s)
{
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(*s >> 11) / 9007199254740992.0 - 0.5;
}

static int check(const char *what, const double *A, const double *B, const double *X)
{
    int bad = 0;
    for (int k = 0; k < NM; ++k)
        for (int c = 0; c < NRHS; ++c) {
            double rmax = 0, anorm = 0, xmax = 0, bmax = 0;
            for (int i = 0; i < N; ++i) {
                double r = B[at(k, i, c, NRHS)], rs = 0;
                for (int j = 0; j < N; ++j) {
                    const double a = A[at(k, i, j, N)];
                    r -= a * X[at(k, j, c, NRHS)];
                    rs += fabs(a);
                }
                rmax = fmax(rmax, fabs(r));
                anorm = fmax(anorm, rs);
                xmax = fmax(xmax, fabs(X[at(k, i, c, NRHS)]));
                bmax = fmax(bmax, fabs(B[at(k, i, c, NRHS)]));
            }
            if (!(rmax <= 8.0 * N * 2.220446049250313e-16 * (anorm * xmax + bmax))) ++bad;
        }
    printf("%s: %d of %d solutions above the bound\n", what, bad, NM * NRHS);
    return bad;
}

int main(void)
{
    const int ng = (NM + V - 1) / V;
    const size_t na = (size_t)ng * N * N * V, nb = (size_t)ng * N * NRHS * V;
    double *A = calloc(na, sizeof(double)), *B = calloc(nb, sizeof(double));
    double *X = calloc(nb, sizeof(double));
    unsigned long long s = 12345;
    for (int k = 0; k < ng * V; ++k) {
        /* A = G G^T + N I (padded lanes: the identity), B ~ U(-0.5, 0.5) */
        double G[N][N];
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                G[i][j] = next(&s);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                double a = 0;
                for (int l = 0; l < N; ++l)
                    a += G[i][l] * G[j][l];
                A[at(k, i, j, N)] = k < NM ? a + (i == j ? N : 0) : (i == j);
            }
        for (int i = 0; i < N; ++i)
            for (int c = 0; c < NRHS; ++c)
                B[at(k, i, c, NRHS)] = k < NM ? next(&s) : 0;
    }
    double *da, *db;
    if (cudaMalloc((void **)&da, na * sizeof(double)) || cudaMalloc((void **)&db, nb * sizeof(double))) {
        printf("cudaMalloc failed\n");
        return 2;
    }
    int bad = 0;
    for (int pass = 0; pass < 2; ++pass) {
        cudaMemcpy(da, A, na * sizeof(double), cudaMemcpyHostToDevice);
        cudaMemcpy(db, B, nb * sizeof(double), cudaMemcpyHostToDevice);
        int info;
        if (pass == 0) {
            info = cbk_cuda_dposv_compact('C', 'L', N, NRHS, da, N, db, N, V, NM);
        }
        else {
            const long long lw = cbk_cuda_dposv_refined_compact_lwork(N, NRHS, V, NM);
            info = cbk_cuda_dposv_refined_compact_async('C', 'L', N, NRHS, da, N, db, N, V, NM, 10,
                                                        NULL, NULL, NULL, lw, NULL);
        }
        if (info != 0 || cudaDeviceSynchronize() != cudaSuccess) {
            printf("pass %d: info %d\n", pass, info);
            return 3;
        }
        cudaMemcpy(X, db, nb * sizeof(double), cudaMemcpyDeviceToHost);
        bad += check(pass == 0 ? "cbk_cuda_dposv_compact" : "cbk_cuda_dposv_refined_compact", A,
                     B, X);
    }
    cudaFree(da);
    cudaFree(db);
    free(A);
    free(B);
    free(X);
    if (bad == 0) printf("c solve ok\n");
    return bad != 0;
}
