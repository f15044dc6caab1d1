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
