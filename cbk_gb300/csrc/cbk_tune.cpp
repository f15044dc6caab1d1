// cbk_tune.cpp -- launch-shape table of the kernels.
//
// threads_for(routine, n, dsize) gives the threads per block of a
// lane-per-matrix kernel for a routine at order n and scalar size dsize;
// variant_for(...) picks between a kernel's compiled shapes where it has more
// than one (for the warp-per-matrix refined solve: registers per thread
// against resident blocks). Both default to the built-in choice (0); the
// autotuner (cbk_cuda_autotune, cbk_autotune.cpp) overwrites entries with
// measured winners, and CBK_CUDA_THREADS=<t> / CBK_CUDA_VARIANT=<v> force one
// value everywhere.
#include "cbk_launch.h"

#include <atomic>
#include <cstdlib>

namespace cbkcuda {

namespace {

constexpr int NMAX = 65; // orders 0..64 tuned individually, larger share slot 64
std::atomic<int> g_table[R_COUNT][2][NMAX];
std::atomic<int> g_variant[R_COUNT][2][NMAX];
std::atomic<int> g_forced{-1};
std::atomic<int> g_forced_variant{-2};

int forced()
{
    int f = g_forced.load(std::memory_order_relaxed);
    if (f < 0) {
        const char *e = std::getenv("CBK_CUDA_THREADS");
        int v = e ? std::atoi(e) : 0;
        if (v != 32 && v != 64 && v != 128 && v != 256 && v != 512) v = 0;
        g_forced.store(v, std::memory_order_relaxed);
        f = v;
    }
    return f;
}

int forced_variant()
{
    int f = g_forced_variant.load(std::memory_order_relaxed);
    if (f < -1) {
        const char *e = std::getenv("CBK_CUDA_VARIANT");
        int v = e ? std::atoi(e) : -1;
        if (v < 0 || v >= MAX_VARIANTS) v = -1;
        g_forced_variant.store(v, std::memory_order_relaxed);
        f = v;
    }
    return f;
}

int slot_of(int n)
{
    return n < 0 ? 0 : (n >= NMAX ? NMAX - 1 : n);
}

} // namespace

int threads_for(int routine, int n, int dsize)
{
    if (int f = forced()) return f;
    const int slot = slot_of(n);
    const int t = (routine >= 0 && routine < R_COUNT)
                      ? g_table[routine][dsize == 8 ? 1 : 0][slot].load(std::memory_order_relaxed)
                      : 0;
    return t > 0 ? t : 128;
}

void set_threads(int routine, int n, int dsize, int threads)
{
    if (routine < 0 || routine >= R_COUNT) return;
    g_table[routine][dsize == 8 ? 1 : 0][slot_of(n)].store(threads, std::memory_order_relaxed);
}

int variant_for(int routine, int n, int dsize)
{
    const int f = forced_variant();
    if (f >= 0) return f;
    if (routine < 0 || routine >= R_COUNT) return 0;
    return g_variant[routine][dsize == 8 ? 1 : 0][slot_of(n)].load(std::memory_order_relaxed);
}

void set_variant(int routine, int n, int dsize, int variant)
{
    if (routine < 0 || routine >= R_COUNT || variant < 0 || variant >= MAX_VARIANTS) return;
    g_variant[routine][dsize == 8 ? 1 : 0][slot_of(n)].store(variant, std::memory_order_relaxed);
}

} // namespace cbkcuda
