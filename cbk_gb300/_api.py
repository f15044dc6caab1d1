"""The reference's C API (include/cbk.h) as Python functions over the GPU.

Each function has the reference's name and argument list; arrays are CUDA
tensors (or device pointers). They return the info code (0 or -j, or a CUDA
error as CBK_CUDA_ERROR_BASE + code) exactly as the C entry points do, and
accept an optional ``stream=`` (default: torch's current stream).
"""
from __future__ import annotations

from ._abi import call

__all__ = []


def _make(prefix: str, routine: str):
    def f(*args, stream=None):
        return call(prefix, routine, *args, stream=stream)

    f.__name__ = f"{prefix}{routine}_compact"
    f.__doc__ = (f"{prefix}{routine}_compact -- include/cbk.h's routine on the GPU; "
                 f"returns info (0 or -j).")
    return f


for _r in ("geqrf", "ormqr", "orgqr", "potrf", "potrs", "posv", "sytrfnp", "sytrsnp", "sysvnp",
           "trsm", "gels", "pack", "unpack"):
    for _p in ("d", "s"):
        _name = f"{_p}{_r}_compact"
        globals()[_name] = _make(_p, _r)
        __all__.append(_name)


def dposv_refined_lwork(n: int, nrhs: int, V: int, nm: int) -> int:
    """Workspace bytes of dposv_refined_compact (0 for n <= 16)."""
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_dposv_refined_compact_lwork
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_int] * 4
    return int(f(n, nrhs, V, nm))


def dposv_refined_compact(layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter=10,
                          iters=None, berr=None, work=None, lwork=None, stream=None):
    """Mixed-precision dposv (FP32 factor + FP64 refinement, FP64 fallback per
    matrix). iters / berr: optional int32 / float64 CUDA tensors of nm entries.
    work: a CUDA tensor of at least dposv_refined_lwork(...) bytes, allocated
    here when None (the C entry point itself never allocates)."""
    import ctypes

    from ._abi import _ptr, _stream, lib
    need = dposv_refined_lwork(n, nrhs, V, nm) if (n > 0 and nm > 0 and V > 0) else 0
    if work is None and need > 0:
        import torch
        work = torch.empty(need, dtype=torch.uint8, device="cuda")
    f = lib().cbk_cuda_dposv_refined_compact_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_longlong, ctypes.c_void_p]

    def raw(t):
        if t is None or isinstance(t, int):
            return t
        return t.data_ptr()
    wbytes = lwork if lwork is not None else (work.numel() * work.element_size()
                                              if work is not None and not isinstance(work, int)
                                              else 0)
    return f(layout.encode(), uplo.encode(), n, nrhs, _ptr(ap, "d"), ldap, _ptr(bp, "d"), ldbp,
             V, nm, max_iter, raw(iters), raw(berr), raw(work), wbytes,
             _stream(stream) if (ap is not None and not isinstance(ap, int)) or stream else None)


__all__ += ["dposv_refined_compact", "dposv_refined_lwork"]


def dposv_refined_batched_lwork(n: int, nrhs: int, nm: int) -> int:
    """Workspace bytes of dposv_refined_batched (0 for n <= 64; -1: illegal)."""
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_dposv_refined_batched_lwork
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_int] * 3
    return f(n, nrhs, nm)


def dposv_refined_batched(uplo, n, nrhs, a, lda, stride_a, b, ldb, stride_b, nm, max_iter=10,
                          iters=None, berr=None, work=None, lwork=None, stream=None):
    """The mixed-precision dposv on a strided dense batch: matrix k's A
    column-major at a + k stride_a (leading dimension lda), its B at
    b + k stride_b. Results per matrix equal dposv_refined_compact's."""
    import ctypes

    from ._abi import _ptr, _stream, lib
    need = dposv_refined_batched_lwork(n, nrhs, nm) if (n > 0 and nm > 0) else 0
    if work is None and need > 0:
        import torch
        work = torch.empty(need, dtype=torch.uint8, device="cuda")
    f = lib().cbk_cuda_dposv_refined_batched_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong,
                  ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_longlong, ctypes.c_void_p]

    def raw(t):
        if t is None or isinstance(t, int):
            return t
        return t.data_ptr()
    wbytes = lwork if lwork is not None else (work.numel() * work.element_size()
                                              if work is not None and not isinstance(work, int)
                                              else 0)
    return f(uplo.encode(), n, nrhs, _ptr(a, "d"), lda, stride_a, _ptr(b, "d"), ldb, stride_b, nm,
             max_iter, raw(iters), raw(berr), raw(work), wbytes,
             _stream(stream) if (a is not None and not isinstance(a, int)) or stream else None)


__all__ += ["dposv_refined_batched", "dposv_refined_batched_lwork"]


def _plain_batched(prefix, routine):
    """?posv_batched / ?sysvnp_batched (uplo, n, nrhs, a, lda, stride_a, b,
    ldb, stride_b, nm) and ?gels_batched (trans, m, n, nrhs, a, lda,
    stride_a, b, ldb, stride_b, tau, nm): the plain drivers on strided dense
    batches (arrays: CUDA tensors or device pointers)."""
    import ctypes

    def f(*args, stream=None):
        from ._abi import _ptr, _stream, lib
        fn = getattr(lib(), f"cbk_cuda_{prefix}{routine}_batched_async")
        fn.restype = ctypes.c_int
        P, I, L = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        if routine == "gels":
            trans, m, n, nrhs, a, lda, sa, b, ldb, sb, tau, nm = args
            fn.argtypes = [ctypes.c_char, I, I, I, P, I, L, P, I, L, P, I, P]
            arrays = (a, b, tau)
            return fn(trans.encode(), m, n, nrhs, _ptr(a, prefix), lda, sa, _ptr(b, prefix), ldb,
                      sb, _ptr(tau, prefix), nm,
                      _stream(stream) if any(t is not None and not isinstance(t, int)
                                             for t in arrays) or stream else None)
        uplo, n, nrhs, a, lda, sa, b, ldb, sb, nm = args
        fn.argtypes = [ctypes.c_char, I, I, P, I, L, P, I, L, I, P]
        return fn(uplo.encode(), n, nrhs, _ptr(a, prefix), lda, sa, _ptr(b, prefix), ldb, sb, nm,
                  _stream(stream) if (a is not None and not isinstance(a, int)) or stream
                  else None)

    f.__name__ = f"{prefix}{routine}_batched"
    return f


for _r in ("posv", "sysvnp", "gels"):
    for _p in ("d", "s"):
        globals()[f"{_p}{_r}_batched"] = _plain_batched(_p, _r)
        __all__.append(f"{_p}{_r}_batched")


def dgels_refined_batched_lwork(m: int, n: int, nrhs: int, nm: int) -> int:
    """Workspace bytes of dgels_refined_batched (-1: illegal argument)."""
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_dgels_refined_batched_lwork
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_int] * 4
    return f(m, n, nrhs, nm)


def dgels_refined_batched(trans, m, n, nrhs, a, lda, stride_a, b, ldb, stride_b, tau, nm,
                          max_iter=10, iters=None, berr=None, work=None, lwork=None,
                          stream=None):
    """The mixed-precision least squares on a strided dense batch: matrix k's
    A column-major at a + k stride_a, B at b + k stride_b, tau at tau + k n.
    Results per matrix equal dgels_refined_compact's."""
    import ctypes

    from ._abi import _ptr, _stream, lib
    need = dgels_refined_batched_lwork(m, n, nrhs, nm) if min(m, n, nm) > 0 else 0
    if work is None and need > 0:
        import torch
        work = torch.empty(need, dtype=torch.uint8, device="cuda")
    f = lib().cbk_cuda_dgels_refined_batched_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                  ctypes.c_void_p]

    def raw(t):
        if t is None or isinstance(t, int):
            return t
        return t.data_ptr()
    wbytes = lwork if lwork is not None else (work.numel() * work.element_size()
                                              if work is not None and not isinstance(work, int)
                                              else 0)
    return f(trans.encode(), m, n, nrhs, _ptr(a, "d"), lda, stride_a, _ptr(b, "d"), ldb,
             stride_b, _ptr(tau, "d"), nm, max_iter, raw(iters), raw(berr), raw(work), wbytes,
             _stream(stream) if (a is not None and not isinstance(a, int)) or stream else None)


__all__ += ["dgels_refined_batched", "dgels_refined_batched_lwork"]


def dposv_refined_host_lwork(layout: str, n: int, nrhs: int, ldap: int, ldbp: int, V: int,
                             nm: int) -> int:
    """Device workspace bytes of dposv_refined_compact_host (-1: illegal argument)."""
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_dposv_refined_compact_host_lwork
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char] + [ctypes.c_int] * 6
    return int(f(layout.encode(), n, nrhs, ldap, ldbp, V, nm))


def _host_ptr(a):
    """Address of a host array: a numpy array, a CPU torch tensor, an int or None."""
    if a is None or isinstance(a, int):
        return a
    if hasattr(a, "ctypes"):
        return a.ctypes.data
    if getattr(a, "is_cuda", False):
        raise ValueError("dposv_refined_compact_host takes host arrays")
    return a.data_ptr()


def dposv_refined_compact_host(layout, uplo, n, nrhs, ap, ldap, bp, ldbp, V, nm, max_iter=10,
                               iters=None, berr=None, dwork=None, lwork=None, stream=None):
    """The mixed-precision dposv on batches in host memory (numpy arrays or
    CPU tensors; pinned memory lets the copies overlap the solves). dwork: a
    CUDA tensor of at least dposv_refined_host_lwork(...) bytes, allocated
    here when None. Returns info once every copy is done."""
    import ctypes

    from ._abi import _stream, lib
    need = (dposv_refined_host_lwork(layout, n, nrhs, ldap, ldbp, V, nm)
            if (n > 0 and nm > 0 and V > 0) else 0)
    if dwork is None and need > 0:
        import torch
        dwork = torch.empty(need, dtype=torch.uint8, device="cuda")
    f = lib().cbk_cuda_dposv_refined_compact_host
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_longlong, ctypes.c_void_p]
    dptr = dwork if (dwork is None or isinstance(dwork, int)) else dwork.data_ptr()
    wbytes = lwork if lwork is not None else (
        dwork.numel() * dwork.element_size() if dwork is not None and not isinstance(dwork, int)
        else 0)
    st = _stream(stream) if (stream is not None or (dwork is not None and
                                                     not isinstance(dwork, int))) else None
    return f(layout.encode(), uplo.encode(), n, nrhs, _host_ptr(ap), ldap, _host_ptr(bp), ldbp, V,
             nm, max_iter, _host_ptr(iters), _host_ptr(berr), dptr, wbytes, st)


__all__ += ["dposv_refined_compact_host", "dposv_refined_host_lwork"]


# ---------------------------------------------------------------------------
# uneven orders: bucketed launches and their CUDA graphs
# ---------------------------------------------------------------------------

def _bucket_struct(scalar):
    import ctypes

    class Bucket(ctypes.Structure):
        _fields_ = [("n", ctypes.c_int), ("nm", ctypes.c_int), ("V", ctypes.c_int),
                    ("ap", ctypes.c_void_p), ("ldap", ctypes.c_int), ("bp", ctypes.c_void_p),
                    ("ldbp", ctypes.c_int)]
    return Bucket


_BUCKET = {}


def _buckets(prefix, buckets):
    """A ctypes array of bucket descriptors from (n, nm, V, ap, ldap, bp, ldbp)
    tuples whose ap / bp are CUDA tensors or device pointers."""
    from ._abi import _ptr
    if prefix not in _BUCKET:
        _BUCKET[prefix] = _bucket_struct(prefix)
    B = _BUCKET[prefix]
    arr = (B * max(1, len(buckets)))()
    for k, (n, nm, V, ap, ldap, bp, ldbp) in enumerate(buckets):
        arr[k] = B(n, nm, V, _ptr(ap, prefix), ldap, _ptr(bp, prefix), ldbp)
    return arr


BUCKETED_LWORK = 256


def bucketed_compact(routine, prefix, layout, uplo, nrhs, buckets, work=None, stream=None):
    """One persistent launch over buckets of single-order compact batches:
    routine 'sysvnp' or 'posv', prefix 'd' or 's'. buckets: a list of
    (n, nm, V, ap, ldap, bp, ldbp). work: >= 256 bytes of device memory
    (allocated here when None). Returns the info code."""
    import ctypes

    from ._abi import _stream, lib
    if work is None:
        import torch
        work = torch.empty(BUCKETED_LWORK, dtype=torch.uint8, device="cuda")
    f = getattr(lib(), f"cbk_cuda_{prefix}{routine}_compact_bucketed_async")
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    arr = _buckets(prefix, buckets)
    wptr = work if isinstance(work, int) else work.data_ptr()
    wlen = BUCKETED_LWORK if isinstance(work, int) else work.numel() * work.element_size()
    return f(layout.encode(), uplo.encode(), nrhs, len(buckets), ctypes.addressof(arr), wptr,
             wlen, _stream(stream))


class BucketedGraph:
    """cbk_cuda_dsysvnp_compact_bucketed_graph: the bucketed launch captured
    once into a CUDA graph; launch() replays it on a stream."""

    def __init__(self, layout, uplo, nrhs, buckets, work):
        import ctypes

        from ._abi import check, lib
        self._lib = lib()
        f = self._lib.cbk_cuda_dsysvnp_compact_bucketed_graph
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_longlong, ctypes.POINTER(ctypes.c_void_p)]
        arr = _buckets("d", buckets)
        self._work = work
        self.handle = ctypes.c_void_p()
        check("dsysvnp_compact_bucketed_graph",
              f(layout.encode(), uplo.encode(), nrhs, len(buckets), ctypes.addressof(arr),
                work.data_ptr(), work.numel() * work.element_size(), ctypes.byref(self.handle)))

    def launch(self, stream=None):
        import ctypes

        from ._abi import _stream
        f = self._lib.cbk_cuda_graph_launch
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        return f(self.handle, _stream(stream))

    def close(self):
        if self.handle:
            import ctypes
            f = self._lib.cbk_cuda_graph_destroy
            f.argtypes = [ctypes.c_void_p]
            f(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ += ["bucketed_compact", "BucketedGraph", "BUCKETED_LWORK"]


def dgels_refined_lwork(m: int, n: int, nrhs: int, V: int, nm: int) -> int:
    """Workspace bytes of dgels_refined_compact."""
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_dgels_refined_compact_lwork
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_int] * 5
    return int(f(m, n, nrhs, V, nm))


def dgels_refined_compact(layout, trans, m, n, nrhs, ap, ldap, bp, ldbp, taup, V, nm,
                          max_iter=10, iters=None, berr=None, work=None, stream=None):
    """Mixed-precision dgels for m >= n, trans 'N' (FP32 QR + FP64 refinement of
    the augmented system, FP64 fallback per matrix). work is allocated here
    when None (the C entry point itself never allocates)."""
    import ctypes

    from ._abi import _ptr, _stream, lib
    need = dgels_refined_lwork(m, n, nrhs, V, nm) if min(m, n, nm, V) > 0 else 0
    if work is None and need > 0:
        import torch
        work = torch.empty(need, dtype=torch.uint8, device="cuda")
    f = lib().cbk_cuda_dgels_refined_compact_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char] + [ctypes.c_int] * 3 + [
        ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]

    def raw(t):
        return t if (t is None or isinstance(t, int)) else t.data_ptr()
    wbytes = 0 if work is None else (need if isinstance(work, int)
                                     else work.numel() * work.element_size())
    live = ap is not None and not isinstance(ap, int)
    return f(layout.encode(), trans.encode(), m, n, nrhs, _ptr(ap, "d"), ldap, _ptr(bp, "d"),
             ldbp, _ptr(taup, "d"), V, nm, max_iter, raw(iters), raw(berr), raw(work), wbytes,
             _stream(stream) if live or stream else None)


__all__ += ["dgels_refined_compact", "dgels_refined_lwork"]


# ---------------------------------------------------------------------------
# autotuning
# ---------------------------------------------------------------------------

def _tune_struct():
    import ctypes

    class TuneResult(ctypes.Structure):
        _fields_ = [("threads", ctypes.c_int), ("variant", ctypes.c_int), ("vlen", ctypes.c_int),
                    ("ms", ctypes.c_double)]
    return TuneResult


_TUNE = []


def _tr():
    if not _TUNE:
        _TUNE.append(_tune_struct())
    return _TUNE[0]


def autotune(routine: str, prec: str, m: int, n: int, nrhs: int, nm: int):
    """Time the routine's launch shapes and widths on a synthetic batch and
    keep the fastest in the library's table. Returns (info, dict)."""
    import ctypes

    from ._abi import lib
    TR = _tr()
    f = lib().cbk_cuda_autotune
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_char] + [ctypes.c_int] * 4 + [ctypes.POINTER(TR)]
    r = TR()
    info = f(routine.encode(), prec.encode(), m, n, nrhs, nm, ctypes.byref(r))
    return info, {"threads": r.threads, "variant": r.variant, "vlen": r.vlen, "ms": r.ms}


def autotune_at(routine: str, prec: str, m: int, n: int, nrhs: int, nm: int, V: int):
    """autotune at one interleave width V. Returns (info, dict)."""
    import ctypes

    from ._abi import lib
    TR = _tr()
    f = lib().cbk_cuda_autotune_at
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_char] + [ctypes.c_int] * 5 + [ctypes.POINTER(TR)]
    r = TR()
    info = f(routine.encode(), prec.encode(), m, n, nrhs, nm, V, ctypes.byref(r))
    return info, {"threads": r.threads, "variant": r.variant, "vlen": r.vlen, "ms": r.ms}


def tune_set(routine: str, prec: str, n: int, threads: int = 0, variant: int = 0,
             vlen: int = 0) -> int:
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_tune_set
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_char] + [ctypes.c_int] * 4
    return f(routine.encode(), prec.encode(), n, threads, variant, vlen)


def tune_get(routine: str, prec: str, n: int):
    """(info, {"threads", "variant", "vlen"}) of one table entry."""
    import ctypes

    from ._abi import lib
    TR = _tr()
    f = lib().cbk_cuda_tune_get
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_char, ctypes.c_int, ctypes.POINTER(TR)]
    r = TR()
    info = f(routine.encode(), prec.encode(), n, ctypes.byref(r))
    return info, {"threads": r.threads, "variant": r.variant, "vlen": r.vlen}


def tune_reset() -> None:
    from ._abi import lib
    lib().cbk_cuda_tune_reset()


def tune_save(path: str) -> int:
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_tune_save
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p]
    return f(path.encode())


def tune_load(path: str) -> int:
    import ctypes

    from ._abi import lib
    f = lib().cbk_cuda_tune_load
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p]
    return f(path.encode())


__all__ += ["autotune", "autotune_at", "tune_set", "tune_get", "tune_reset", "tune_save",
            "tune_load"]
