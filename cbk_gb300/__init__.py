"""cbk_gb300 -- the compact batch kernels on an NVIDIA GB300.

Python mirror of ivan-pi/cbk's include/cbk.h API over libcbk_cuda.so (the C
ABI declared in include/cbk_cuda.h). Every routine keeps the reference's name,
argument list, argument meaning and -j error codes; the array arguments are
CUDA tensors (or raw device pointers as ints) and the work is enqueued on the
current torch stream, or on ``stream=`` when given.

    import cbk_gb300 as cbk
    info = cbk.dposv_compact('C', 'L', n, nrhs, ap, n, bp, n, V, nm)

There is no CPU fallback: importing the package loads libcbk_cuda.so and
raises if it is missing or fails to load (build it with
``python -m cbk_gb300.build`` or ``__graft_entry__.build()``).
"""
from __future__ import annotations

from ._abi import (  # noqa: F401
    CBK_CUDA_ERROR_BASE,
    SIGNATURES,
    CbkError,
    call,
    check,
    lib,
    lib_path,
    status_string,
    version,
    vlen_ok,
)
from ._api import *  # noqa: F401,F403
from ._api import __all__ as _api_all

__all__ = ["lib", "lib_path", "call", "check", "CbkError", "version", "vlen_ok",
           "status_string", "SIGNATURES"] + list(_api_all)
