"""ctypes binding of the host-pointer layer, cbk_cuda_host_<p><routine>_compact
(test infrastructure): the routine's arguments with numpy host arrays, then
dwork (a device pointer or None), lwork (in/out) and the stream."""
import ctypes

import numpy as np

import cases as C
from oracle import oracle as O


def fn(dtype, routine):
    import cbk_gb300
    p = "d" if np.dtype(dtype) == np.float64 else "s"
    f = getattr(cbk_gb300.lib(), f"cbk_cuda_host_{p}{routine}_compact")
    scalar = ctypes.c_double if p == "d" else ctypes.c_float
    kinds = O.SIGNATURES[routine]
    f.argtypes = [{"c": ctypes.c_char, "i": ctypes.c_int, "P": ctypes.c_void_p, "S": scalar}[k]
                  for k in kinds] + [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                     ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f, kinds


def call(dtype, routine, args, dwork, lwork, stream=None):
    """args: the routine's arguments (numpy arrays or None for the arrays);
    lwork: a ctypes.c_longlong or None. Returns the info code."""
    f, kinds = fn(dtype, routine)
    conv = []
    for k, a in zip(kinds, args):
        if k == "c":
            conv.append(a.encode() if isinstance(a, str) else a)
        elif k == "P":
            conv.append(None if a is None else a.ctypes.data)
        else:
            conv.append(a)
    ptr = None if lwork is None else ctypes.byref(lwork)
    return f(*conv, dwork, ptr, stream)


def run_case(case, stream=None):
    """A compact case through the host layer: size query, a device workspace
    of that size, the call; returns (info, the case after)."""
    import torch
    c = case.copy()
    args = c.args()
    lw = ctypes.c_longlong(-1)
    info = call(c.dtype, c.routine, args, None, lw)
    if info != 0:
        return info, c
    work = torch.empty(max(1, lw.value), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream
    info = call(c.dtype, c.routine, args, work.data_ptr() if lw.value else None, lw, s)
    return info, c
