// cbk_tune.cpp -- launch-shape table of the lane-per-matrix kernels.
//
// threads_for(routine, n, dsize) gives the threads per block for a routine at
// order n and scalar size dsize. The defaults come from the table below; the
// autotuner (cbk_cuda_autotune, cbk_autotune.cu) overwrites entries with
// measured winners, and CBK_CUDA_THREADS=<t> forces one value everywhere.
#include "cbk_launch.h"

#include <atomic>
#include <cstdlib>

namespace cbkcuda {

namespace {

constexpr int NMAX = 65; // orders 0..64 tuned individually, larger share slot 64
std::atomic<int> g_table[R_COUNT][2][NMAX];
std::atomic<int> g_forced{-1};

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

} // namespace

int threads_for(int routine, int n, int dsize)
{
    if (int f = forced()) return f;
    const int slot = n < 0 ? 0 : (n >= NMAX ? NMAX - 1 : n);
    const int t = (routine >= 0 && routine < R_COUNT)
                      ? g_table[routine][dsize == 8 ? 1 : 0][slot].load(std::memory_order_relaxed)
                      : 0;
    return t > 0 ? t : 128;
}

void set_threads(int routine, int n, int dsize, int threads)
{
    if (routine < 0 || routine >= R_COUNT) return;
    const int slot = n < 0 ? 0 : (n >= NMAX ? NMAX - 1 : n);
    g_table[routine][dsize == 8 ? 1 : 0][slot].store(threads, std::memory_order_relaxed);
}

} // namespace cbkcuda
