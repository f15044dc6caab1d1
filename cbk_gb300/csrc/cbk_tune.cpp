// cbk_tune.cpp -- launch-shape table of the kernels.
//
// threads_for(routine, n, dsize) gives the threads per block of a
// lane-per-matrix kernel for a routine at order n and scalar size dsize;
// variant_for(...) picks between a kernel's compiled shapes where it has more
// than one (for the warp-per-matrix refined solve: registers per thread
// against resident blocks; for the refined least squares: 0 one warp per
// matrix where compiled, 1 one lane per matrix); vlen_for(...) is the interleave width the
// autotuner measured fastest (advice for the caller's layout: the width of a
// batch is the caller's). All default to 0 (the built-in choice); the
// autotuner (cbk_cuda_autotune, cbk_autotune.cu) overwrites entries with
// measured winners, cbk_cuda_tune_load reads a saved table, and
// CBK_CUDA_THREADS=<t> / CBK_CUDA_VARIANT=<v> force one value everywhere.
// CBK_CUDA_TUNE_FILE=<path> loads a saved table on first use.
//
// The table is the only global state of the library; entries are atomics
// (a launch reads a consistent value even while another thread tunes), and
// results never depend on it: every launch shape computes the same bits.
#include "../../include/cbk_cuda.h"
#include "cbk_launch.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace cbkcuda {

namespace {

constexpr int NMAX = 65; // orders 0..64 tuned individually, larger share slot 64
std::atomic<int> g_table[R_COUNT][2][NMAX];
std::atomic<int> g_variant[R_COUNT][2][NMAX];
std::atomic<int> g_vlen[R_COUNT][2][NMAX];
std::once_flag g_env_once;

void load_env_file()
{
    std::call_once(g_env_once, [] {
        if (const char *f = std::getenv("CBK_CUDA_TUNE_FILE")) cbk_cuda_tune_load(f);
    });
}
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

int threads_or(int routine, int n, int dsize, int dflt)
{
    if (int f = forced()) return f;
    load_env_file();
    const int slot = slot_of(n);
    const int t = (routine >= 0 && routine < R_COUNT)
                      ? g_table[routine][dsize == 8 ? 1 : 0][slot].load(std::memory_order_relaxed)
                      : 0;
    return t > 0 ? t : dflt;
}

int threads_for(int routine, int n, int dsize)
{
    return threads_or(routine, n, dsize, 128);
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
    load_env_file();
    return g_variant[routine][dsize == 8 ? 1 : 0][slot_of(n)].load(std::memory_order_relaxed);
}

void set_variant(int routine, int n, int dsize, int variant)
{
    if (routine < 0 || routine >= R_COUNT || variant < 0 || variant >= MAX_VARIANTS) return;
    g_variant[routine][dsize == 8 ? 1 : 0][slot_of(n)].store(variant, std::memory_order_relaxed);
}

int vlen_for(int routine, int n, int dsize)
{
    if (routine < 0 || routine >= R_COUNT) return 0;
    load_env_file();
    return g_vlen[routine][dsize == 8 ? 1 : 0][slot_of(n)].load(std::memory_order_relaxed);
}

void set_vlen(int routine, int n, int dsize, int V)
{
    if (routine < 0 || routine >= R_COUNT) return;
    g_vlen[routine][dsize == 8 ? 1 : 0][slot_of(n)].store(V, std::memory_order_relaxed);
}

namespace {

struct Name {
    const char *name;
    int routine;
};
constexpr Name NAMES[] = {
    {"potrf", R_POTRF},   {"sytrfnp", R_SYTRFNP}, {"potrs", R_POTRS},
    {"posv", R_POSV},     {"sytrsnp", R_SYTRSNP}, {"sysvnp", R_SYSVNP},
    {"trsm", R_TRSM},     {"geqrf", R_GEQRF},     {"ormqr", R_ORMQR},
    {"orgqr", R_ORGQR},   {"gels", R_GELS},       {"posv_refined", R_POSV_REFINED},
    {"gels_refined", R_GELS_REFINED}, {"sysvnp_bucketed", R_SYSVNP_BUCKETED},
    {"posv_bucketed", R_POSV_BUCKETED},
};

} // namespace

int routine_of(const char *name)
{
    if (!name) return -1;
    for (const Name &e : NAMES)
        if (std::strcmp(e.name, name) == 0) return e.routine;
    return -1;
}

const char *routine_name(int routine)
{
    for (const Name &e : NAMES)
        if (e.routine == routine) return e.name;
    return nullptr;
}

int tune_slots()
{
    return NMAX;
}

} // namespace cbkcuda

using namespace cbkcuda;

extern "C" {

int cbk_cuda_tune_set(const char *routine, char prec, int n, int threads, int variant, int vlen)
{
    const int r = routine_of(routine);
    if (r < 0) return -1;
    if (prec != 'd' && prec != 's') return -2;
    if (n < 0) return -3;
    if (threads != 0 && threads != 32 && threads != 64 && threads != 128 && threads != 256 &&
        threads != 512)
        return -4;
    if (variant < 0 || variant >= MAX_VARIANTS) return -5;
    if (vlen != 0 && (vlen < 32 || vlen > 1024 || vlen % 32 != 0)) return -6;
    const int ds = prec == 'd' ? 8 : 4;
    set_threads(r, n, ds, threads);
    set_variant(r, n, ds, variant);
    set_vlen(r, n, ds, vlen);
    return 0;
}

int cbk_cuda_tune_get(const char *routine, char prec, int n, cbk_cuda_tune_result *out)
{
    const int r = routine_of(routine);
    if (r < 0) return -1;
    if (prec != 'd' && prec != 's') return -2;
    if (n < 0) return -3;
    if (out == nullptr) return -4;
    const int ds = prec == 'd' ? 8 : 4;
    const int slot = n >= NMAX ? NMAX - 1 : n;
    out->threads = g_table[r][ds == 8][slot].load(std::memory_order_relaxed);
    out->variant = g_variant[r][ds == 8][slot].load(std::memory_order_relaxed);
    out->vlen = g_vlen[r][ds == 8][slot].load(std::memory_order_relaxed);
    out->ms = 0.0;
    return 0;
}

void cbk_cuda_tune_reset(void)
{
    for (int r = 0; r < R_COUNT; ++r)
        for (int p = 0; p < 2; ++p)
            for (int k = 0; k < NMAX; ++k) {
                g_table[r][p][k].store(0, std::memory_order_relaxed);
                g_variant[r][p][k].store(0, std::memory_order_relaxed);
                g_vlen[r][p][k].store(0, std::memory_order_relaxed);
            }
}

// text, one tuned entry per line: routine prec n threads variant vlen
int cbk_cuda_tune_save(const char *path)
{
    if (!path) return -1;
    std::FILE *f = std::fopen(path, "w");
    if (!f) return -1;
    std::fprintf(f, "# cbk_gb300 tuning table: routine prec n threads variant vlen\n");
    for (const Name &e : NAMES)
        for (int p = 0; p < 2; ++p)
            for (int k = 0; k < NMAX; ++k) {
                const int t = g_table[e.routine][p][k].load(std::memory_order_relaxed);
                const int v = g_variant[e.routine][p][k].load(std::memory_order_relaxed);
                const int w = g_vlen[e.routine][p][k].load(std::memory_order_relaxed);
                if (t || v || w)
                    std::fprintf(f, "%s %c %d %d %d %d\n", e.name, p ? 'd' : 's', k, t, v, w);
            }
    return std::fclose(f) == 0 ? 0 : -1;
}

// returns the number of entries read, or -1 (unreadable file) / -(line) for
// the first malformed line (entries before it are kept)
int cbk_cuda_tune_load(const char *path)
{
    if (!path) return -1;
    std::FILE *f = std::fopen(path, "r");
    if (!f) return -1;
    char line[256];
    int count = 0, lineno = 0;
    while (std::fgets(line, sizeof line, f)) {
        ++lineno;
        if (line[0] == '#' || line[0] == '\n') continue;
        char name[64], prec;
        int n, t, v, w;
        if (std::sscanf(line, "%63s %c %d %d %d %d", name, &prec, &n, &t, &v, &w) != 6 ||
            cbk_cuda_tune_set(name, prec, n, t, v, w) != 0) {
            std::fclose(f);
            return -lineno;
        }
        ++count;
    }
    std::fclose(f);
    return count;
}

} // extern "C"
