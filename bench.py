#!/usr/bin/env python
"""Benchmark: mixed-precision (FP32 factor + FP64 refinement) vs plain FP64
compact SPD solves on one or more GB300s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cbk|reference]

Workload (the mixed-precision dposv configuration): for each n in
{8, 16, 32, 48}, 262,144 SPD matrices A = U diag(s) U^T (U Haar-random, the Q
of a seeded Gaussian's QR with R's diagonal signs folded in; s log-uniform
from 1 to 1/kappa, log10 kappa uniform in [1, 6]), one right-hand side
b ~ N(0,1), compact layout with V = 32, column-major, lower triangle. A step
solves all four batches (1,048,576 systems). Synthetic data stands in for a
dataset; the seed is in the JSON line.

value      refined solves/s with the inputs resident in HBM (CUDA events around
           the solve launches; inputs restored and L2 flushed untimed before
           every step); the plain FP64 dposv_compact is timed the same way on
           the same matrices and both paths' worst normwise backward error is
           reported against the common bound 8 n eps64 ("equal FP64 error")
e2e        the same solves through the C ABI from pinned host buffers: the H2D
           copy of every A and b, the solves and the D2H copy of every x inside
           the timed region
roofline   HBM roofline of the dominant launch (the largest order): algorithmic
           bytes (lower triangle of A read once, b read, x written) over its
           measured duration; fp64_pipe the same launch's FP64 work over the
           measured FP64 FMA rate -- the pipe that binds on this part
cpu_baseline  the reference's own dposv_compact (its src/cbk.cpp built -O3 for
           the host's native vector ISA, OpenMP over groups, every host core)
           on this run's matrices copied to the host, at the fastest of the
           reference's widths 2/4/8

With --gpus N > 1 (torchrun, one rank per GPU) every rank solves its own full
replica of the workload: value = all ranks' solves / the slowest rank's time.
--impl reference times the reference's own CPU build on the same workload
instead (rank 0 only; the port of it where the reference could not be built).

The other configurations are measured after the headline and reported in its
line under "configs" (each with its own roofline and a cpu_baseline through
the reference's own build on the same matrices): c1 plain dposv n = 8 on
65,536 matrices; c2 dgels 16 x 8 (nrhs 4) and dorgqr on 1,048,576; c4 the
uneven-order dsysvnp in one CUDA-graph launch against one launch per order;
c5 the mixed-precision least squares 64 x 16 (nrhs 8) against plain dgels;
lay the layout / triangle / side / transpose forms of posv (plain and
refined), trsm and ormqr, each against its column-major lower / left form.
--config NAME prints one of them (or c3d: the headline's refined solve on
strided dense batches against the compact layout) on its own line; --no-extra
leaves them out. --case KIND N NM runs one small solve for a profiler
capture.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s & HBM GB/s, n=8-48: refined FP32 vs plain FP64 at equal FP64 error"
UNIT = "solves/s"
SIZES = (8, 16, 32, 48)
NM = 262144
V = 32
NRHS = 1
SEED = 0x5EED
LOG10_KAPPA = (1.0, 6.0)
WORKLOAD = ("mixed-precision dposv_compact: n in {8,16,32,48}, nrhs=1, 262144 SPD matrices "
            "per n (kappa log-uniform 1e1..1e6), compact V=32 column-major lower")
DATA = ("synthetic (seed 0x5EED): A = U diag(s) U^T, U Haar (sign-fixed QR of a Gaussian), "
        "s log-uniform with log10 kappa ~ U[1,6]; b ~ N(0,1)")


def bytes_per_matrix(n: int) -> int:
    """Algorithmic HBM bytes of one solve: the lower triangle of A read once,
    b read and x written (FP64)."""
    return 8 * (n * (n + 1) // 2 + 2 * n * NRHS)


def plain_bytes_per_matrix(n: int, nrhs: int = NRHS) -> int:
    """Algorithmic HBM bytes of one plain FP64 dposv: the lower triangle of A
    read once and its factor written back, b read and x written."""
    return 8 * (2 * (n * (n + 1) // 2) + 2 * n * nrhs)


def plain_flops(n: int) -> float:
    """FP64 flops of the plain factor + solve: n^3/3 + n^2/2 + n/6 + 2 n^2 nrhs."""
    return n ** 3 / 3 + n * n / 2 + n / 6 + 2 * n * n * NRHS


# ---------------------------------------------------------------------------
# process setup
# ---------------------------------------------------------------------------

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def slowest_rank(times_ms, device=None):
    """Each timing's maximum over ranks (the slowest rank decides): an
    all-reduce MAX when torch.distributed runs more than one rank, the values
    themselves otherwise. device: where the reduction tensor lives (a CUDA
    device under NCCL, the CPU under gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(t) for t in times_ms]
    tt = torch.tensor([float(t) for t in times_ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return [float(x) for x in tt]


def job_throughput(units_per_rank, t_ms, ws):
    """Whole-job throughput of weak-scaled replicas: every rank's units over
    the slowest rank's time."""
    return ws * units_per_rank / (t_ms * 1e-3)


class Clocks:
    """nvidia-smi sampler over the timed region (clocks, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20", "-i", str(self.idx)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# CPU implementation (the reference arm, and the cpu_baseline of ours)
# ---------------------------------------------------------------------------

CPU_WIDTHS = (2, 4, 8)  # the reference's widths: NEON holds 2 doubles, AVX-512 8


def cpu_lib():
    """(library, kind): the reference's own src/cbk.cpp in its performance build
    (oracle/_ref/libcbk_ref_fast.so: -O3, the host's native vector ISA,
    OpenMP), or, where the reference could not be built, the oracle's port."""
    from oracle import oracle as O
    lib = O.reference(fast=True)
    if lib is not None:
        return lib, "reference"
    return O.oracle(fast=True), "port"


def cpu_threads():
    """OpenMP threads a parallel region of the CPU library gets."""
    import ctypes
    try:
        gomp = ctypes.CDLL("libgomp.so.1")
        gomp.omp_get_max_threads.restype = ctypes.c_int
        return int(gomp.omp_get_max_threads())
    except OSError:
        return os.cpu_count()


def cpu_info():
    import platform
    info = {"machine": platform.machine(), "logical_cpus": os.cpu_count(),
            "omp_threads": cpu_threads()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                info["model"] = ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


def cpu_pass(lib, packed, Vc, nm):
    """One step over `packed` [(n, a, b)] with the library's dposv_compact at
    width Vc; the inputs are restored from the pristine arrays untimed before
    each call (the reference benches' method). Returns seconds per order."""
    import numpy as np
    out = []
    for n, a0, b0, a, b in packed:
        np.copyto(a, a0)
        np.copyto(b, b0)
        t0 = time.perf_counter()
        info = lib.call("posv", np.float64, "C", "L", n, NRHS, a, n, b, n, Vc, nm)
        out.append(time.perf_counter() - t0)
        assert info == 0, info
    return out


def cpu_packed(dense, Vc):
    """[(n, A, B)] dense -> [(n, a0, b0, a, b)] compact at width Vc (pristine
    and working copies)."""
    from oracle import oracle as O
    out = []
    for n, A, B in dense:
        a0, b0 = O.pack(A, Vc), O.pack(B, Vc, pad_diag=0.0)
        out.append((n, a0, b0, a0.copy(), b0.copy()))
    return out


def cpu_pick_width(lib, dense, nm, reps=2):
    """The fastest of the reference's widths on `dense` (best of reps passes
    each); returns (V, {V: ms per pass})."""
    times = {}
    for Vc in CPU_WIDTHS:
        packed = cpu_packed(dense, Vc)
        cpu_pass(lib, packed, Vc, nm)
        times[Vc] = 1e3 * min(sum(cpu_pass(lib, packed, Vc, nm)) for _ in range(reps))
        del packed
    return min(times, key=times.get), times


def _gen_chunk(task):
    """A chunk of the headline workload for one order, packed at width Vc
    (a spawned worker of the reference arm's input generation)."""
    n, count, seed, Vc = task
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as C
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    A, _ = C.gen_spd_cond(rng, count, n, LOG10_KAPPA)
    B = rng.standard_normal((count, n, NRHS))
    return O.pack(A, Vc), O.pack(B, Vc, pad_diag=0.0)


def cpu_workload(Vc, per_n=NM, chunk=16384):
    """The full headline workload on the host, packed at width Vc: for every
    order per_n matrices from the same distribution as the GPU arm's, made by
    a pool of spawned single-threaded workers (one seeded chunk each).
    Returns [(n, a0, b0, a, b)]."""
    import multiprocessing as mp

    import numpy as np
    seeds = np.random.SeedSequence(SEED).spawn(len(SIZES) * (per_n // chunk))
    tasks = [(n, chunk, seeds[k * (per_n // chunk) + c], Vc)
             for k, n in enumerate(SIZES) for c in range(per_n // chunk)]
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")}
    os.environ.update(OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    try:
        pool = mp.get_context("spawn").Pool(processes=max(1, min(32, os.cpu_count() or 1)))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    with pool:
        parts = pool.map(_gen_chunk, tasks, chunksize=1)
    out = []
    per = per_n // chunk
    for k, n in enumerate(SIZES):
        a0 = np.concatenate([parts[k * per + c][0] for c in range(per)])
        b0 = np.concatenate([parts[k * per + c][1] for c in range(per)])
        out.append((n, a0, b0, a0.copy(), b0.copy()))
    return out


def cpu_baseline_from(dense_fn, steps=3):
    """cpu_baseline of our arm: the reference's dposv_compact (its performance
    build) on the GPU run's own matrices, copied to the host, at the fastest
    of its widths; best of `steps` passes. dense_fn() gives [(n, A, B)]."""
    lib, kind = cpu_lib()
    dense = dense_fn()
    nm = dense[0][1].shape[0]
    Vc, wtimes = cpu_pick_width(lib, [(n, A[:16384], B[:16384]) for n, A, B in dense], 16384)
    packed = cpu_packed(dense, Vc)
    del dense
    cpu_pass(lib, packed, Vc, nm)  # warm-up
    best = min(sum(cpu_pass(lib, packed, Vc, nm)) for _ in range(steps))
    return {"value": nm * len(SIZES) / best, "unit": UNIT, "cores": cpu_threads(), "kind": kind,
            "V": Vc, "width_ms_16384_per_n": wtimes, "host": cpu_info(),
            "sample": (f"the GPU run's own matrices, all {nm} per n in {{8,16,32,48}}, "
                       f"dposv_compact at V={Vc} (fastest of {CPU_WIDTHS} on 16384 per n), "
                       f"best of {steps} passes ({best * 1e3:.1f} ms per pass)")}


def run_reference(args):
    """--impl reference: the reference's own CPU implementation (its
    performance build) on the same workload and config as the GPU arm, rank 0
    alone; the other ranks exit without work."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    import numpy as np
    lib, kind = cpu_lib()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as C
    per_n = args.ref_per_n
    nsub = min(16384, per_n)
    rng = np.random.default_rng(SEED)
    sub = []
    for n in SIZES:
        A, _ = C.gen_spd_cond(rng, nsub, n, LOG10_KAPPA)
        sub.append((n, A, rng.standard_normal((nsub, n, NRHS))))
    Vc, wtimes = cpu_pick_width(lib, sub, nsub)
    wtimes = {f"{v} ({nsub} per n)": t for v, t in wtimes.items()}
    del sub
    t0 = time.perf_counter()
    packed = cpu_workload(Vc, per_n, chunk=nsub)
    gen_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        cpu_pass(lib, packed, Vc, per_n)
    per = [cpu_pass(lib, packed, Vc, per_n) for _ in range(args.steps)]
    tot = [sum(p) for p in per]
    solves = per_n * len(SIZES)
    ms = 1e3 * sum(tot) / len(tot)
    value = solves / (ms * 1e-3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA,
        "config": {"workload": WORKLOAD, "nm_per_n": per_n, "n": list(SIZES), "nrhs": NRHS,
                   "V": Vc, "parallelism": "OpenMP over groups of V (the reference's own)"},
        "per_n_ms": {str(n): 1e3 * statistics.mean(p[k] for p in per)
                     for k, n in enumerate(SIZES)},
        "best_ms_per_step": 1e3 * min(tot),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_threads(), "kind": kind,
                         "V": Vc, "width_ms": wtimes, "host": cpu_info(),
                         "sample": (f"the whole workload every step: {per_n} matrices per n, "
                                    f"dposv_compact at V={Vc} (fastest of {CPU_WIDTHS}); "
                                    f"inputs made by a spawned pool in {gen_s:.0f} s, "
                                    f"restored untimed before every call")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def haar_dev(cbk, n, nm, gen, device):
    """Haar-random orthogonal U (nm, n, n) on the device: the Q of a Gaussian's
    QR with the signs of R's diagonal folded in (Mezzadri 2007), the QR taken
    by this library's own dgeqrf_compact + dorgqr_compact."""
    import torch
    G = torch.randn(nm, n, n, dtype=torch.float64, device=device, generator=gen)
    gp = pack_dev(cbk, G)
    del G
    tau = torch.empty(((nm + V - 1) // V) * V * n, dtype=torch.float64, device=device)
    cbk.check("geqrf", cbk.dgeqrf_compact("C", n, n, gp, n, tau, V, nm))
    ng = (nm + V - 1) // V
    d = torch.sign(gp.view(ng, n, n, V)[:, torch.arange(n), torch.arange(n), :])  # (ng, n, V)
    d[d == 0] = 1
    cbk.check("orgqr", cbk.dorgqr_compact("C", n, n, n, gp, n, tau, V, nm))
    Q = gp.view(ng, n, n, V).permute(0, 3, 2, 1).reshape(ng * V, n, n)[:nm]  # [k, i, j]
    return Q * d.permute(0, 2, 1).reshape(ng * V, n)[:nm, None, :]


def gen_batch(n, nm, gen, device):
    """Dense A (nm, n, n) FP64 on the device and b (nm, n, 1), as the docstring
    describes."""
    import torch

    import cbk_gb300 as cbk
    f64 = torch.float64
    U = haar_dev(cbk, n, nm, gen, device)
    lk = torch.empty(nm, dtype=f64, device=device).uniform_(*LOG10_KAPPA, generator=gen)
    u = torch.sort(torch.rand(nm, n, dtype=f64, device=device, generator=gen), dim=1).values
    if n > 1:
        u[:, 0] = 0
        u[:, -1] = 1
    s = torch.pow(10.0, -lk[:, None] * u)
    A = (U * s[:, None, :]) @ U.transpose(1, 2)
    del U
    A = torch.tril(A) + torch.tril(A, -1).transpose(1, 2)
    B = torch.randn(nm, n, NRHS, dtype=f64, device=device, generator=gen)
    return A, B


def pack_dev(cbk, M):
    """Dense (nm, r, c) FP64 -> compact V=32 column-major, on the device."""
    import torch
    nm, r, c = M.shape
    ng = (nm + V - 1) // V
    out = torch.empty(ng * r * c * V, dtype=M.dtype, device=M.device)
    colmajor = M.transpose(1, 2).contiguous()
    pad = 1.0 if r == c else 0.0
    cbk.check("pack", cbk.call("d", "pack", "C", r, c, colmajor, r, r * c, out, r, V, nm, pad))
    return out


def x_dense(bp, n, nm):
    """Compact (V=32, col-major, ld=n) n x 1 batch -> dense (nm, n, 1)."""
    ng = (nm + V - 1) // V
    return bp.view(ng, n, V).permute(0, 2, 1).reshape(ng * V, n)[:nm].unsqueeze(2)


def berr_max(A, X, B):
    """Largest normwise backward error over the batch, FP64 on the device."""
    import torch
    R = B - torch.bmm(A, X)
    an = A.abs().sum(dim=2).amax(dim=1)
    rn = R.abs().amax(dim=(1, 2))
    xn = X.abs().amax(dim=(1, 2))
    bn = B.abs().amax(dim=(1, 2))
    return float((rn / (an * xn + bn)).max())


def run_case(args):
    """One small solve for a profiler to capture: the headline's batch for one
    order (--case refined|plain N NM), solved twice (the second launch is the
    one a capture skips to); prints a line, times nothing."""
    import torch

    import cbk_gb300 as cbk
    kind, n, nm = args.case[0], int(args.case[1]), int(args.case[2])
    if kind not in ("refined", "plain", "gels_refined", "gels"):
        raise SystemExit("--case takes refined|plain|gels_refined|gels N NM")
    dev = torch.device("cuda", 0)
    if kind.startswith("gels"):
        return run_gels_case(kind, n, nm, dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    A, B = gen_batch(n, nm, gen, dev)
    ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
    del A, B
    ap, bp = ap0.clone(), bp0.clone()
    work = torch.empty(max(1, cbk.dposv_refined_lwork(n, NRHS, V, nm)), dtype=torch.uint8,
                       device=dev)
    for _ in range(2):
        ap.copy_(ap0)
        bp.copy_(bp0)
        if kind == "refined":
            info = cbk.dposv_refined_compact("C", "L", n, NRHS, ap, n, bp, n, V, nm, 10, None,
                                             None, work)
        else:
            info = cbk.dposv_compact("C", "L", n, NRHS, ap, n, bp, n, V, nm)
        assert info == 0, info
    torch.cuda.synchronize()
    print("case", kind, n, nm, "ok")


def ls_batch(m, n, nrhs, nm, dev):
    """The least-squares batch: A = U diag(s) V^T with kappa in 1e1 .. 1e4,
    B = A X + 1e-3 N(0,1), packed at width V on the device; also A and B
    unpacked (device) for the error checks."""
    import numpy as np
    import torch
    rng = np.random.default_rng(SEED)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as C
    from oracle import oracle as O
    A, Bm, _, _ = C.gen_ls_cond(rng, nm, m, n, nrhs)
    ap0 = torch.from_numpy(O.pack(A, V)).to(dev)
    bp0 = torch.from_numpy(O.pack(Bm, V, pad_diag=0.0)).to(dev)
    return ap0, bp0, torch.from_numpy(A).to(dev), torch.from_numpy(Bm).to(dev)


def ls_normal_residual(A, bp, B, m, n, nrhs, nm):
    """max over matrices and right-hand sides of ||A^T (b - A x)||_inf /
    (||A||_inf (||A||_inf ||x||_inf + ||b||_inf)), x read from the packed B."""
    X = bp.view(nm // V, nrhs, m, V).permute(0, 3, 2, 1).reshape(nm, m, nrhs)[:, :n]
    G = A.transpose(1, 2) @ (B - A @ X)
    an = A.abs().sum(dim=2).amax(dim=1)[:, None]
    den = an * (an * X.abs().amax(dim=1) + B.abs().amax(dim=1))
    return float((G.abs().amax(dim=1) / den).amax())


def run_gels_case(kind, n, nm, dev):
    """--case gels_refined|gels N NM: the least-squares configuration's shape
    (m = 4 N, nrhs = 8) on NM matrices, solved twice."""
    import torch

    import cbk_gb300 as cbk
    m, nrhs = 4 * n, 8
    ap0, bp0, _, _ = ls_batch(m, n, nrhs, nm, dev)
    ap, bp = ap0.clone(), bp0.clone()
    tau = torch.empty(nm * n, dtype=torch.float64, device=dev)
    work = torch.empty(max(1, cbk.dgels_refined_lwork(m, n, nrhs, V, nm)), dtype=torch.uint8,
                       device=dev)
    for _ in range(2):
        ap.copy_(ap0)
        bp.copy_(bp0)
        if kind == "gels_refined":
            info = cbk.dgels_refined_compact("C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm, 10,
                                             None, None, work)
        else:
            info = cbk.dgels_compact("C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm)
        assert info == 0, info
    torch.cuda.synchronize()
    print("case", kind, n, nm, "ok")


def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    import cbk_gb300 as cbk
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + rank)

    def barrier():
        if ws > 1:
            dist.barrier()

    # launch shapes from the library's autotuner, at this layout's width, for
    # both paths (untimed setup; shapes never change results)
    tuned = {}
    if not args.no_tune:
        for n in SIZES:
            for routine in ("posv_refined", "posv"):
                info, r = cbk.autotune_at(routine, "d", n, n, NRHS, NM, V)
                assert info == 0, (routine, n, info)
                tuned[f"{routine} n={n}"] = {"threads": r["threads"], "variant": r["variant"]}

    batches = []
    for n in SIZES:
        A, B = gen_batch(n, NM, gen, dev)
        ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
        batches.append(dict(n=n, A=A, B=B, ap0=ap0, bp0=bp0, ap=torch.empty_like(ap0),
                            bp=torch.empty_like(bp0),
                            work=torch.empty(max(1, cbk.dposv_refined_lwork(n, NRHS, V, NM)),
                                             dtype=torch.uint8, device=dev),
                            iters=torch.empty(NM, dtype=torch.int32, device=dev),
                            berr=torch.empty(NM, dtype=torch.float64, device=dev)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB of L2
    torch.cuda.synchronize()

    def refined(b, stream=None):
        return cbk.dposv_refined_compact("C", "L", b["n"], NRHS, b["ap"], b["n"], b["bp"], b["n"],
                                         V, NM, 10, b["iters"], b["berr"], b["work"],
                                         stream=stream)

    def plain(b, stream=None):
        return cbk.dposv_compact("C", "L", b["n"], NRHS, b["ap"], b["n"], b["bp"], b["n"], V, NM,
                                 stream=stream)

    def restore():
        for b in batches:
            b["ap"].copy_(b["ap0"])
            b["bp"].copy_(b["bp0"])
        flush.fill_(1)

    def step(fn):
        """One timed step: per-launch events; returns (total ms, [ms per n])."""
        restore()
        torch.cuda.synchronize()
        barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(batches) + 1)]
        ev[0].record()
        for k, b in enumerate(batches):
            info = fn(b)
            assert info == 0, info
            ev[k + 1].record()
        torch.cuda.synchronize()
        barrier()
        per = [ev[k].elapsed_time(ev[k + 1]) for k in range(len(batches))]
        return ev[0].elapsed_time(ev[-1]), per

    def run_path(fn, K, W):
        for _ in range(W):
            step(fn)
        tot, per = [], []
        for _ in range(K):
            t, p = step(fn)
            tot.append(t)
            per.append(p)
        return tot, per

    # The job's step: the four orders are independent batches, so each goes
    # on its own stream, the largest first (its long launch starts at once and
    # the short ones fill the SMs that its last waves leave idle), joined by
    # events on the timing stream. Measured: 7.85 against 7.95 ms one after
    # another on one stream.
    streams = [torch.cuda.Stream(device=dev) for _ in batches]
    order = sorted(range(len(batches)), key=lambda k: -batches[k]["n"])

    def step_concurrent(fn):
        """One timed step of the whole job; returns ms."""
        restore()
        torch.cuda.synchronize()
        barrier()
        main = torch.cuda.current_stream()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(main)
        for k in order:
            streams[k].wait_event(e0)
            info = fn(batches[k], streams[k])
            assert info == 0, info
        for st in streams:
            main.wait_stream(st)
        e1.record(main)
        torch.cuda.synchronize()
        barrier()
        return e0.elapsed_time(e1)

    # the headline path, with the clocks sampled over its timed steps
    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0]) \
        if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else local
    for _ in range(args.warmup):
        step_concurrent(refined)
    with Clocks(gpu_index) as clk:
        ref_tot = [step_concurrent(refined) for _ in range(args.steps)]
    clocks = clk.summary()
    # per order, one launch at a time (the per-n table and the roofline)
    _, ref_per = run_path(refined, args.steps, 1)
    # outcomes of the refined path (from the last step) and its backward error
    ref_stats = {}
    worst_ref = 0.0
    for b in batches:
        it = b["iters"]
        conv = it >= 0
        ref_stats[b["n"]] = {
            "converged_frac": float(conv.float().mean()),
            "mean_corrections": float(it[conv].float().mean()) if bool(conv.any()) else None,
            "fallbacks": {str(c): int((it == c).sum()) for c in (-1, -2, -3)},
        }
        e = berr_max(b["A"], x_dense(b["bp"], b["n"], NM), b["B"])
        ref_stats[b["n"]]["max_berr_over_n_eps"] = e / (b["n"] * 2.220446049250313e-16)
        worst_ref = max(worst_ref, ref_stats[b["n"]]["max_berr_over_n_eps"])
    # the plain FP64 path on the same matrices, the same two ways
    for _ in range(max(1, args.warmup // 2)):
        step_concurrent(plain)
    pl_tot = [step_concurrent(plain) for _ in range(args.steps)]
    _, pl_per = run_path(plain, args.steps, 0)
    worst_plain = 0.0
    for b in batches:
        e = berr_max(b["A"], x_dense(b["bp"], b["n"], NM), b["B"])
        ref_stats[b["n"]]["plain_max_berr_over_n_eps"] = e / (b["n"] * 2.220446049250313e-16)
        worst_plain = max(worst_plain, ref_stats[b["n"]]["plain_max_berr_over_n_eps"])

    solves = NM * len(SIZES)
    t_ref = sum(ref_tot) / len(ref_tot)
    t_pl = sum(pl_tot) / len(pl_tot)
    t_ref, t_pl = slowest_rank([t_ref, t_pl], dev)
    value = job_throughput(solves, t_ref, ws)
    plain_value = job_throughput(solves, t_pl, ws)

    per_n = {}
    for k, b in enumerate(batches):
        n = b["n"]
        r_ms = statistics.mean(p[k] for p in ref_per)
        p_ms = statistics.mean(p[k] for p in pl_per)
        per_n[str(n)] = dict(ref_stats[n], refined_ms=r_ms, plain_ms=p_ms,
                             speedup=p_ms / r_ms,
                             refined_gbs=NM * bytes_per_matrix(n) / (r_ms * 1e-3) / 1e9,
                             plain_gbs=NM * bytes_per_matrix(n) / (p_ms * 1e-3) / 1e9)

    # roofline of the dominant launch (the longest: the largest order)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    hbm_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    kdom = max(range(len(batches)), key=lambda k: statistics.mean(p[k] for p in ref_per))
    ndom = batches[kdom]["n"]
    dom_ms = statistics.mean(p[kdom] for p in ref_per)
    achieved = NM * bytes_per_matrix(ndom) / (dom_ms * 1e-3) / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tr = json.load(f)
        per_matrix = tr.get(f"posv_refined_n{ndom}", {}).get("dram_bytes_per_matrix")
        traffic = per_matrix * NM if per_matrix else None
    except (OSError, ValueError):
        pass
    rate = ctypes_fma_rate(cbk)
    # FP64 work of the dominant refined launch: (corrections + 1) residuals of
    # n^2 FMAs per right-hand side, plus the fallbacks' plain solves
    it = batches[kdom]["iters"]
    conv = it >= 0
    ncorr = float(it[conv].double().sum()) + float(conv.sum())
    nfall = int((~conv).sum())
    fp64_flops = 2.0 * ndom * ndom * ncorr + plain_flops(ndom) * nfall
    pl_dom_ms = statistics.mean(p[kdom] for p in pl_per)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ref, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor + f64 refinement (f64 results)", "data": DATA,
        "config": {"workload": WORKLOAD, "nm_per_n": NM, "n": list(SIZES), "nrhs": NRHS, "V": V,
                   "max_iter": 10, "l2": "flushed (256 MiB write) before every timed step",
                   "inputs": "restored untimed before every step", "parallelism": "replicas",
                   "launch": "the four orders on four streams, largest first, joined by events "
                             "on the timing stream; per_n from a second pass, one launch at a "
                             "time",
                   "launch_shapes": tuned or "built-in defaults (--no-tune)"},
        "plain_fp64": {"value": plain_value, "unit": UNIT, "ms_per_step": t_pl},
        "speedup_refined_vs_plain": plain_value and value / plain_value,
        "equal_error": {"bound": "berr <= 8 n eps64 (normwise, inf-norm)",
                        "refined_max_berr_over_n_eps": worst_ref,
                        "plain_max_berr_over_n_eps": worst_plain,
                        "both_within_bound": worst_ref <= 8 and worst_plain <= 8},
        "per_n": per_n,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "binding": "the FP64 pipe, not HBM (see fp64_pipe)",
                     "fp64_frac": (fp64_flops / (dom_ms * 1e-3) / 1e12) / rate if rate else None,
                     "kernel": f"k_posv_refined_warp<{ndom}> (n={ndom})" if 16 < ndom <= 64
                     else f"k_posv_refined (n={ndom})",
                     "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)"},
        "fp64_pipe": {"kernel": f"k_posv_refined_warp<{ndom}> (n={ndom})" if 16 < ndom <= 64
                      else f"k_posv_refined (n={ndom})", "unit": "TFLOP/s",
                      "achieved": fp64_flops / (dom_ms * 1e-3) / 1e12,
                      "plain_achieved": NM * plain_flops(ndom) / (pl_dom_ms * 1e-3) / 1e12,
                      "peak": rate, "peak_source": "measured FP64 FMA rate "
                      "(cbk_cuda_measure_fma_rate, this run)"},
        "gpu_launches": len(SIZES) * args.steps,
        "clocks": clocks,
    }
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_from(
            lambda: [(b["n"], b["A"].cpu().numpy(), b["B"].cpu().numpy()) for b in batches])
    if not args.no_e2e:
        line["e2e"] = e2e(args, cbk, batches, barrier, ws)
    # free the device, then the other configurations (1 GPU only)
    del batches
    torch.cuda.empty_cache()
    if ws == 1 and not args.no_extra:
        t0 = time.perf_counter()
        line["configs"] = config_lines(("c1", "c2", "c4", "c5", "lay"), args, cbk, dev,
                                       with_cpu=not args.no_cpu)
        line["configs_wall_s"] = time.perf_counter() - t0
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def ctypes_fma_rate(cbk):
    import ctypes
    out = ctypes.c_double(0)
    f = cbk.lib().cbk_cuda_measure_fma_rate
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    return out.value if f(1, ctypes.byref(out)) == 0 else None


def e2e(args, cbk, batches, barrier, ws):
    """The solves through the public C ABI on host memory: every step,
    cbk_cuda_dposv_refined_compact_host copies each batch's A (the referenced
    triangle) and b in from pinned host buffers, solves and copies x out --
    the copies pipelined with the solves by the library, all inside the timed
    region."""
    import torch
    host = []
    for b in batches:
        n = b["n"]
        host.append(dict(n=n, ap0=b["ap0"].cpu().pin_memory(), bp0=b["bp0"].cpu().pin_memory(),
                         ap=torch.empty_like(b["ap0"], device="cpu").pin_memory(),
                         bp=torch.empty_like(b["bp0"], device="cpu").pin_memory(),
                         dwork=torch.empty(cbk.dposv_refined_host_lwork("C", n, NRHS, n, n,
                                                                        V, NM),
                                           dtype=torch.uint8, device=b["ap0"].device)))
    del b
    groups = (NM + V - 1) // V
    # pinned A: the library reads only its lower triangle over the host link
    h2d = sum(groups * V * 8 * (h["n"] * (h["n"] + 1) // 2 + h["n"] * NRHS) for h in host)
    d2h = sum(groups * V * 8 * h["n"] * NRHS for h in host)

    # The four batches are independent, so the four calls go from four host
    # threads at once, the largest order first (the library's host entry point
    # is re-entrant: each call has its own streams and workspace; ctypes
    # releases the GIL for the call). Their fixed costs and pipeline ramps
    # then overlap on the host link: 21.5 against 22.4 ms for the calls one
    # after another, with the same bits.
    from concurrent.futures import ThreadPoolExecutor
    dev = batches[0]["ap"].device
    # each worker makes this rank's GPU its current device (a new thread
    # starts on device 0; the library runs on the caller's current device)
    pool = ThreadPoolExecutor(len(host), initializer=torch.cuda.set_device, initargs=(dev,))
    by_size = sorted(host, key=lambda h: -h["n"])

    def call(h):
        t = time.perf_counter()
        info = cbk.dposv_refined_compact_host("C", "L", h["n"], NRHS, h["ap"], h["n"], h["bp"],
                                              h["n"], V, NM, 10, None, None, h["dwork"])
        h["t"] = (time.perf_counter() - t) * 1e3
        return info

    def one():
        for h in host:  # fresh inputs, untimed
            h["ap"].copy_(h["ap0"])
            h["bp"].copy_(h["bp0"])
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        infos = list(pool.map(call, by_size))
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) * 1e3
        assert all(i == 0 for i in infos), infos
        barrier()
        per.append([h["t"] for h in host])
        return t

    per = []

    # as many untimed steps as the headline (at least two), and Python's
    # garbage collected first: the first calls after the CPU baseline's
    # multi-GB host arrays were freed have shown one-time stalls of tens of ms
    import gc
    gc.collect()
    for _ in range(max(2, args.warmup)):
        one()
    ts = [one() for _ in range(args.steps)]
    pool.shutdown()
    t = slowest_rank([sum(ts) / len(ts)], batches[0]["ap"].device)[0]
    per = per[-len(ts):]
    per_n_ms = {str(h["n"]): statistics.mean(p[k] for p in per) for k, h in enumerate(host)}
    return {"value": job_throughput(NM * len(SIZES), t, ws), "unit": UNIT, "ms_per_step": t,
            "per_n_ms": per_n_ms,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "path": "cbk_cuda_dposv_refined_compact_host per n: pinned host A (its lower "
                    "triangle, read by the device) and b in, x out, pipelined with the solves "
                    "in 3 device slots; the four calls from four host threads at once, largest "
                    "order first; host wall clock around them (per_n_ms: each call's own wall "
                    "time, the calls overlapping)"}


# ---------------------------------------------------------------------------
# the other configurations (--config): one JSON line each, same timing rules
# ---------------------------------------------------------------------------

def _timer(dev):
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run(fn, restore, K, W):
        ts = []
        for k in range(W + K):
            restore()
            flush.fill_(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            n_launch = fn()
            e1.record()
            torch.cuda.synchronize()
            if k >= W:
                ts.append(e0.elapsed_time(e1))
        return sum(ts) / len(ts), n_launch
    return run


def cpu_best_width(timer, sample_fn, widths=CPU_WIDTHS):
    """The fastest of the reference's widths for one configuration: timer(Vc,
    packed) -> seconds for one pass, sample_fn(Vc) -> the packed sample."""
    t = {}
    for Vc in widths:
        pk = sample_fn(Vc)
        timer(Vc, pk)
        t[Vc] = min(timer(Vc, pk) for _ in range(2))
    return min(t, key=t.get), {str(k): 1e3 * v for k, v in t.items()}


def cpu_config_baseline(kind, dense, unit, steps=3):
    """The reference's own CPU build (its performance build, every host core)
    on one configuration's matrices, copied to the host: the fastest width of
    2/4/8 on a 16384-matrix sample, then the whole batch, best of `steps`
    passes with the inputs restored untimed before each call. dense holds
    the configuration's host arrays; kind selects the calls:
      posv  dense = (A, B): dposv_compact
      gels  dense = (A, B): dgels_compact ('N')
      sysvnp  dense = [(A_n, B_n) per order]: one dsysvnp_compact per order
    Returns the cpu_baseline object (units: matrices per second)."""
    import numpy as np
    from oracle import oracle as O
    lib, lkind = cpu_lib()

    def pack_all(Vc, limit=None):
        out = []
        for A, B in (dense if kind == "sysvnp" else [dense]):
            A_, B_ = (A, B) if limit is None else (A[:limit], B[:limit])
            if A_.shape[0] == 0:
                continue
            a0, b0 = O.pack(A_, Vc), O.pack(B_, Vc, pad_diag=0.0)
            out.append((A_.shape, B_.shape, a0, b0, a0.copy(), b0.copy()))
        return out

    def one_pass(Vc, packed):
        t = 0.0
        for (sa, sb, a0, b0, a, b) in packed:
            np.copyto(a, a0)
            np.copyto(b, b0)
            nm, m, n = sa
            nrhs = sb[2]
            t0 = time.perf_counter()
            if kind == "gels":
                tau = np.zeros(O.compact_size(nm, n, 1, n, Vc))
                info = lib.call("gels", np.float64, "C", "N", m, n, nrhs, a, m, b, m, tau, Vc, nm)
            else:
                info = lib.call(kind, np.float64, "C", "L", n, nrhs, a, n, b, n, Vc, nm)
            t += time.perf_counter() - t0
            assert info == 0, info
        return t

    per = 16384 if kind != "sysvnp" else 1024
    Vc, wms = cpu_best_width(one_pass, lambda Vc: pack_all(Vc, per))
    packed = pack_all(Vc)
    total = sum(p[0][0] for p in packed)
    one_pass(Vc, packed)
    best = min(one_pass(Vc, packed) for _ in range(steps))
    return {"value": total / best, "unit": unit, "cores": cpu_threads(), "kind": lkind, "V": Vc,
            "width_ms_sample": wms, "ms_per_pass": 1e3 * best,
            "sample": f"this configuration's own {total} matrices, copied to the host; "
                      f"fastest width of {CPU_WIDTHS} on {per} per call; best of {steps}"}


def fp64_peak(cbk):
    """The measured FP64 FMA rate in TFLOP/s (cbk_cuda_measure_fma_rate)."""
    return ctypes_fma_rate(cbk)


def config_lines(names, args, cbk, dev, with_cpu=True):
    """The other configurations' measurements, one dict per name (c1, c2, c4,
    c5, c3d), each with its own roofline against the pipe that binds it (FP64
    work over the measured FP64 FMA rate; algorithmic bytes over the measured
    HBM copy rate) and, for c1 / c2 / c4 / c5, a cpu_baseline through the
    reference's own build on the same matrices."""
    import numpy as np
    import torch
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    timed = _timer(dev)
    f64 = torch.float64
    rate = fp64_peak(cbk)
    hbm = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm = json.load(f).get("hbm_gbs")
    except OSError:
        pass
    hbm_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0

    def roof(flops, nbytes, ms, kernel):
        tf = flops / (ms * 1e-3) / 1e12
        gb = nbytes / (ms * 1e-3) / 1e9
        return {"kernel": kernel, "bound": "fp64 pipe", "fp64_tflops": tf, "fp64_peak": rate,
                "fp64_frac": tf / rate if rate else None, "hbm_gbs": gb, "hbm_peak": hbm,
                "hbm_frac": gb / hbm, "peak_source": f"FP64: measured FMA rate this run; HBM: "
                                                     f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)"}

    out = {}
    base = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "config": {"workload": None, "l2": "flushed (256 MiB write) before every timed step",
                       "inputs": "restored untimed before every step"}}
    for name in names:
        line = json.loads(json.dumps(base))
        if name == "c1":
            n, nm = 8, 65536
            G = torch.randn(nm, n, n, dtype=f64, device=dev, generator=gen)
            A = G @ G.transpose(1, 2) + n * torch.eye(n, dtype=f64, device=dev)
            B = torch.randn(nm, n, 1, dtype=f64, device=dev, generator=gen)
            ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
            ap, bp = ap0.clone(), bp0.clone()

            def restore():
                ap.copy_(ap0)
                bp.copy_(bp0)
            t, _ = timed(lambda: cbk.check("posv", cbk.dposv_compact(
                "C", "L", n, 1, ap, n, bp, n, V, nm)) or 1, restore, args.steps, args.warmup)
            berr = berr_max(A, x_dense(bp, n, nm), B) / (n * 2.220446049250313e-16)
            it = torch.empty(nm, dtype=torch.int32, device=dev)
            tr, _ = timed(lambda: cbk.check("posv_refined", cbk.dposv_refined_compact(
                "C", "L", n, 1, ap, n, bp, n, V, nm, 10, it)) or 1, restore, args.steps,
                args.warmup)
            line.update(metric="dposv_compact FP64 n=8 nrhs=1 solves/s", value=nm / (t * 1e-3),
                        unit=UNIT, ms_per_step=t, dtype="f64",
                        data="synthetic: A = G G^T + n I, G, B ~ N(0,1), seed 0x5EED",
                        max_berr_over_n_eps=berr, refined_value=nm / (tr * 1e-3),
                        gbs=nm * plain_bytes_per_matrix(n, 1) / (t * 1e-3) / 1e9,
                        roofline=roof(nm * plain_flops(n), nm * plain_bytes_per_matrix(n, 1), t,
                                      "k_chol_small<double,8,1>"),
                        gpu_launches=args.steps)
            line["config"]["workload"] = "dposv_compact n=8 nrhs=1, 65536 matrices, V=32"
            if with_cpu:
                line["cpu_baseline"] = cpu_config_baseline(
                    "posv", (A.cpu().numpy(), B.cpu().numpy()), UNIT)
            del A, B, G, ap0, bp0, ap, bp
        elif name == "c2":
            m, n, nrhs, nm = 16, 8, 4, 1 << 20
            A = torch.randn(nm, m, n, dtype=f64, device=dev, generator=gen)
            B = torch.randn(nm, m, nrhs, dtype=f64, device=dev, generator=gen)
            ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
            ap, bp = ap0.clone(), bp0.clone()
            tau = torch.empty(nm * n, dtype=f64, device=dev)

            def restore():
                ap.copy_(ap0)
                bp.copy_(bp0)
            t, _ = timed(lambda: cbk.check("gels", cbk.dgels_compact(
                "C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm)) or 1, restore, args.steps,
                args.warmup)
            geq = ap.clone()  # the QR left by the last gels, for orgqr

            def restore_q():
                ap.copy_(geq)
            tq, _ = timed(lambda: cbk.check("orgqr", cbk.dorgqr_compact(
                "C", m, n, n, ap, m, tau, V, nm)) or 1, restore_q, args.steps, args.warmup)
            ng = nm // V
            Q = ap.view(ng, n, m, V).permute(0, 3, 2, 1).reshape(nm, m, n)
            orth = float((Q.transpose(1, 2) @ Q - torch.eye(n, dtype=f64, device=dev)).abs()
                         .amax()) / 2.220446049250313e-16
            del Q, geq
            line.update(metric="dgels_compact FP64 16x8 nrhs=4 solves/s", value=nm / (t * 1e-3),
                        unit=UNIT, ms_per_step=t, dtype="f64", data="synthetic: A, B ~ N(0,1)",
                        gbs=nm * 3136 / (t * 1e-3) / 1e9, dorgqr_ms=tq,
                        dorgqr_per_s=nm / (tq * 1e-3), dorgqr_orthogonality_over_eps=orth,
                        roofline=roof(nm * 3499.0, nm * 3136.0, t, "k_gels<double>"),
                        dorgqr_roofline=roof(nm * 1707.0, nm * 2112.0, tq, "k_orgqr<double>"),
                        gpu_launches=args.steps)
            line["config"]["workload"] = "dgels_compact m=16 n=8 nrhs=4 + dorgqr, 1048576, V=32"
            if with_cpu:
                line["cpu_baseline"] = cpu_config_baseline(
                    "gels", (A.cpu().numpy(), B.cpu().numpy()), UNIT)
            del A, B, ap0, bp0, ap, bp, tau
        elif name == "c4":
            nrhs, total = 2, 1 << 20
            rng = np.random.default_rng(SEED)
            counts = np.bincount(rng.integers(4, 49, total), minlength=49)[4:]
            bks, host = [], []
            flops = nbytes = 0.0
            for k, n in enumerate(range(4, 49)):
                nm = int(counts[k])
                G = torch.randn(nm, n, n, dtype=f64, device=dev, generator=gen)
                S = (G + G.transpose(1, 2)) / 2 + 2 * n * torch.eye(n, dtype=f64, device=dev)
                Bm = torch.randn(nm, n, nrhs, dtype=f64, device=dev, generator=gen)
                a0, b0 = pack_dev(cbk, S), pack_dev(cbk, Bm)
                bks.append(dict(n=n, nm=nm, a0=a0, b0=b0, a=a0.clone(), b=b0.clone()))
                if with_cpu:
                    host.append((S.cpu().numpy(), Bm.cpu().numpy()))
                flops += nm * (n ** 3 / 3 + 2 * n * n * nrhs + n * nrhs)
                nbytes += nm * 8 * (n * (n + 1) + 2 * n * nrhs)
                del G, S, Bm

            def restore():
                for b in bks:
                    b["a"].copy_(b["a0"])
                    b["b"].copy_(b["b0"])
            # the persistent grid from the library's autotuner on a batch of
            # this workload's size (untimed; the graph bakes the launch in at
            # capture). A smaller tuning batch misleads: at 2^17 matrices the
            # halved grid can measure faster, at 2^20 it is 30 % slower.
            tuned = None
            if not args.no_tune:
                info, tuned = cbk.autotune("sysvnp_bucketed", "d", 48, 48, nrhs, total)
                assert info == 0, info
            work = torch.empty(cbk.BUCKETED_LWORK, dtype=torch.uint8, device=dev)
            tup = [(b["n"], b["nm"], V, b["a"], b["n"], b["b"], b["n"]) for b in bks]
            graph = cbk.BucketedGraph("C", "L", nrhs, tup, work)
            tg, _ = timed(lambda: cbk.check("graph", graph.launch()) or 1, restore, args.steps,
                          args.warmup)

            def per_size():
                for b in bks:
                    cbk.check("sysvnp", cbk.dsysvnp_compact("C", "L", b["n"], nrhs, b["a"],
                                                            b["n"], b["b"], b["n"], V, b["nm"]))
                return len(bks)
            tp, _ = timed(per_size, restore, args.steps, args.warmup)
            graph.close()
            line.update(metric="uneven-size dsysvnp solves/s (n~U{4..48}, nrhs=2)",
                        value=total / (tg * 1e-3), unit=UNIT, ms_per_step=tg, dtype="f64",
                        data="synthetic: symmetric N(0,1) + 2n I, B ~ N(0,1)",
                        per_size_launches={"value": total / (tp * 1e-3), "ms_per_step": tp,
                                           "launches": len(bks)},
                        speedup_graph_vs_per_size=tp / tg,
                        launch_shape=({"variant": tuned["variant"],
                                       "grid": "one wave of warps halved 'variant' times"}
                                      if tuned else "built-in (--no-tune)"),
                        roofline=roof(flops, nbytes, tg, "k_bucketed<double,true>"),
                        gpu_launches=args.steps)
            line["config"]["workload"] = ("dsysvnp_compact, 1048576 matrices, n uniform in "
                                          "4..48, 45 buckets, V=32: one persistent CUDA-graph "
                                          "launch")
            if with_cpu:
                line["cpu_baseline"] = cpu_config_baseline("sysvnp", host, UNIT)
                line["cpu_baseline"]["sample"] += " (one call per order, as the reference takes)"
            del bks, host, work
        elif name == "c3d":
            # the headline batches as strided dense column-major arrays (lda =
            # n, stride n^2): the refined solve reads and writes them in place,
            # against the compact path on the same matrices
            per, td_all, tc_all, same = {}, 0.0, 0.0, True
            for n in SIZES:
                A, B = gen_batch(n, NM, gen, dev)
                a0, b0 = A.contiguous(), B.contiguous()
                ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
                del A, B
                a, b, ap, bp = a0.clone(), b0.clone(), ap0.clone(), bp0.clone()
                it = torch.empty(NM, dtype=torch.int32, device=dev)

                def rd():
                    a.copy_(a0)
                    b.copy_(b0)

                def rc():
                    ap.copy_(ap0)
                    bp.copy_(bp0)
                td, _ = timed(lambda: cbk.check("batched", cbk.dposv_refined_batched(
                    "L", n, NRHS, a, n, n * n, b, n, n * NRHS, NM, 10, it)) or 1, rd,
                    args.steps, args.warmup)
                tc, _ = timed(lambda: cbk.check("posv_refined", cbk.dposv_refined_compact(
                    "C", "L", n, NRHS, ap, n, bp, n, V, NM, 10, it)) or 1, rc, args.steps,
                    args.warmup)
                same = same and torch.equal(b.view(NM, n), x_dense(bp, n, NM).view(NM, n))
                per[str(n)] = {"dense_ms": td, "compact_ms": tc}
                td_all += td
                tc_all += tc
                del a0, b0, ap0, bp0, a, b, ap, bp
            line.update(metric="mixed-precision dposv on strided dense batches solves/s, n=8-48",
                        value=NM * len(SIZES) / (td_all * 1e-3), unit=UNIT, ms_per_step=td_all,
                        dtype="f32 factor + f64 refinement (f64 results)",
                        data="synthetic: the headline's matrices (seed 0x5EED), dense "
                             "column-major",
                        compact={"value": NM * len(SIZES) / (tc_all * 1e-3),
                                 "ms_per_step": tc_all},
                        per_n=per, x_bit_identical_to_compact=bool(same),
                        gpu_launches=len(SIZES) * args.steps)
            line["config"]["workload"] = ("dposv_refined_batched: n in {8,16,32,48}, 262144 "
                                          "matrices each, A column-major lda = n, stride n^2, "
                                          "nrhs = 1")
        elif name == "c5":
            m, n, nrhs, nm = 64, 16, 8, 131072
            ap0, bp0, Ad, Bd = ls_batch(m, n, nrhs, nm, dev)
            ap, bp = ap0.clone(), bp0.clone()
            tau = torch.empty(nm * n, dtype=f64, device=dev)
            it = torch.empty(nm, dtype=torch.int32, device=dev)
            work = torch.empty(cbk.dgels_refined_lwork(m, n, nrhs, V, nm), dtype=torch.uint8,
                               device=dev)

            def restore():
                ap.copy_(ap0)
                bp.copy_(bp0)
            tr, _ = timed(lambda: cbk.check("gels_refined", cbk.dgels_refined_compact(
                "C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm, 10, it, None, work)) or 1,
                restore, args.steps, args.warmup)
            itc = it.cpu().numpy()
            ne_ref = ls_normal_residual(Ad, bp, Bd, m, n, nrhs, nm)
            tpl, _ = timed(lambda: cbk.check("gels", cbk.dgels_compact(
                "C", "N", m, n, nrhs, ap, m, bp, m, tau, V, nm)) or 1, restore, args.steps,
                args.warmup)
            ne_pl = ls_normal_residual(Ad, bp, Bd, m, n, nrhs, nm)
            steps = float(itc[itc >= 0].mean())
            # FP64 work of the refined solve: per right-hand side and step the
            # residuals f = b - r - A x (2mn, skipped at the first step) and
            # g = -A^T r (2mn); plain: geqrf + Q^T B + R^-1
            fl_ref = nm * nrhs * (4.0 * m * n * (steps + 1) - 2.0 * m * n)
            fl_pl = nm * (2 * m * n * n - 2 * n ** 3 / 3 + 4 * m * nrhs * n - 2 * nrhs * n * n +
                          n * n * nrhs)
            by = nm * 8 * (m * n + 2 * m * nrhs)
            eps = 2.220446049250313e-16
            line.update(metric="least squares 64x16 nrhs=8 solves/s: refined FP32 vs plain FP64",
                        value=nm / (tr * 1e-3), unit=UNIT, ms_per_step=tr,
                        dtype="f32 QR + f64 refinement", data="synthetic: A = U diag(s) V^T, "
                        "kappa 1e1..1e4, B = A X + 1e-3 N(0,1)",
                        plain_fp64={"value": nm / (tpl * 1e-3), "ms_per_step": tpl,
                                    "roofline": roof(fl_pl, nm * 8 * (2 * m * n + n + 2 * m *
                                                                     nrhs), tpl, "k_gels<double>")},
                        speedup_refined_vs_plain=tpl / tr,
                        max_normal_residual_over_n_eps={"refined": ne_ref / (n * eps),
                                                        "plain": ne_pl / (n * eps)},
                        refinement={"converged_frac": float((itc >= 0).mean()),
                                    "mean_steps": steps},
                        roofline=roof(fl_ref, by, tr, "k_gels_refined_warp<2,16,4,3>"),
                        gpu_launches=args.steps)
            line["config"]["workload"] = "dgels m=64 n=16 nrhs=8, 131072 matrices, V=32"
            if with_cpu:
                line["cpu_baseline"] = cpu_config_baseline(
                    "gels", (Ad.cpu().numpy(), Bd.cpu().numpy()), UNIT)
                line["cpu_baseline"]["sample"] += " (the reference's plain FP64 dgels_compact)"
            del ap0, bp0, Ad, Bd, ap, bp, tau, work
        elif name == "lay":
            # The layout, triangle, side and transpose variants that the
            # configurations above run in one form only: each routine timed in
            # every form on the same bytes (a symmetric matrix reads the same in
            # either layout and triangle; a random square one is a valid
            # triangular or QR input in any of them), against its column-major
            # lower / left form.
            variants = {}

            def ratio_table(key, times):
                base = times[next(iter(times))]
                variants[key] = {"ms": times, "worst_over_first": max(times.values()) / base}
            for n in (16, 48):
                nm = 65536
                G = torch.randn(nm, n, n, dtype=f64, device=dev, generator=gen)
                A = G @ G.transpose(1, 2) + n * torch.eye(n, dtype=f64, device=dev)
                B = torch.randn(nm, n, 1, dtype=f64, device=dev, generator=gen)
                ap0, bp0 = pack_dev(cbk, A), pack_dev(cbk, B)
                ap, bp = ap0.clone(), bp0.clone()
                work = torch.empty(max(1, cbk.dposv_refined_lwork(n, 1, V, nm)),
                                   dtype=torch.uint8, device=dev)

                def restore():
                    ap.copy_(ap0)
                    bp.copy_(bp0)
                for kind in ("posv", "posv_refined"):
                    times = {}
                    for lay, uplo in (("C", "L"), ("C", "U"), ("R", "L"), ("R", "U")):
                        if kind == "posv":
                            fn = (lambda lay=lay, uplo=uplo: cbk.check("posv", cbk.dposv_compact(
                                lay, uplo, n, 1, ap, n, bp, 1 if lay == "R" else n, V, nm)) or 1)
                        else:
                            fn = (lambda lay=lay, uplo=uplo: cbk.check(
                                "posv_refined", cbk.dposv_refined_compact(
                                    lay, uplo, n, 1, ap, n, bp, 1 if lay == "R" else n, V, nm, 10,
                                    None, None, work)) or 1)
                        times[f"{lay},{uplo}"], _ = timed(fn, restore, args.steps, args.warmup)
                    ratio_table(f"d{kind} n={n} (layout,uplo)", times)
                del G, A, B, ap0, bp0, ap, bp, work
            m, nm = 16, 1 << 18
            T0 = torch.randn(nm, m, m, dtype=f64, device=dev, generator=gen)
            T0 = T0 + 4.0 * m * torch.eye(m, dtype=f64, device=dev)
            C0 = torch.randn(nm, m, m, dtype=f64, device=dev, generator=gen)
            tp0, cp0 = pack_dev(cbk, T0), pack_dev(cbk, C0)
            tp, cp = tp0.clone(), cp0.clone()

            def restore_c():
                cp.copy_(cp0)
            times = {}
            for lay in ("C", "R"):
                for side in ("L", "R"):
                    for tr in ("N", "T"):
                        times[f"{lay},{side},{tr}"], _ = timed(
                            lambda lay=lay, side=side, tr=tr: cbk.check("trsm", cbk.dtrsm_compact(
                                lay, side, "L", tr, "N", m, m, 1.0, tp, m, cp, m, V, nm)) or 1,
                            restore_c, args.steps, args.warmup)
            ratio_table("dtrsm 16x16, 16 right-hand sides (layout,side,trans)", times)
            times = {}
            k = 8
            tau = torch.empty(nm * k, dtype=f64, device=dev)
            for lay in ("C", "R"):
                tp.copy_(tp0)
                lda = m if lay == "C" else k  # the QR of the leading 16 x 8 block
                cbk.check("geqrf", cbk.dgeqrf_compact(lay, m, k, tp, lda, tau, V, nm))
                for side, tr in (("L", "T"), ("R", "N")):
                    times[f"{lay},{side},{tr}"], _ = timed(
                        lambda lay=lay, side=side, tr=tr, lda=lda: cbk.check(
                            "ormqr", cbk.dormqr_compact(lay, side, tr, m, m, k, tp, lda, tau, cp,
                                                        m, V, nm)) or 1,
                        restore_c, args.steps, args.warmup)
            ratio_table("dormqr 16x16, k=8 (layout,side,trans)", times)
            del T0, C0, tp0, cp0, tp, cp, tau
            line.update(metric="layout / triangle / side variants against the first form (ms)",
                        value=max(v["worst_over_first"] for v in variants.values()),
                        unit="worst time ratio", higher_is_better=False, dtype="f64",
                        data="synthetic: SPD G G^T + n I; triangular T + 4m I; C ~ N(0,1)",
                        variants=variants, gpu_launches=args.steps)
            line["config"]["workload"] = ("dposv (plain, refined) n=16/48 x 65536, dtrsm and "
                                          "dormqr 16x16 x 262144, V=32, every form")
        torch.cuda.empty_cache()
        out[name] = line
    return out


def run_config(args):
    import torch

    import cbk_gb300 as cbk
    dev = torch.device("cuda", 0)
    line = config_lines([args.config], args, cbk, dev, with_cpu=not args.no_cpu)[args.config]
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("cbk", "reference"), default="cbk")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the built-in launch shapes instead of autotuning them first")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the other configurations (c1, c2, c4, c5) in the headline line")
    ap.add_argument("--ref-per-n", type=int, default=NM,
                    help="--impl reference: matrices per order (default: the whole workload)")
    ap.add_argument("--config", choices=("c3", "c1", "c2", "c4", "c5", "c3d", "lay"),
                    default="c3",
                    help="c3 (default) is the headline; the others print their own line")
    ap.add_argument("--case", nargs=3, metavar=("KIND", "N", "NM"),
                    help="no timing: solve one batch (refined|plain, order N, NM matrices) "
                         "twice, for a profiler capture")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3  # at least three untimed warm-up steps
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config != "c3":
        run_config(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
