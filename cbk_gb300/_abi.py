"""ctypes binding of libcbk_cuda.so (include/cbk_cuda.h)."""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
CBK_CUDA_ERROR_BASE = 1000

# argument kinds of each routine, in include/cbk.h order:
# c char, i int, L long long, P array (device pointer), S scalar of the routine's type
SIGNATURES = {
    "geqrf": "ciiPiPii",
    "ormqr": "ccciiiPiPPiii",
    "orgqr": "ciiiPiPii",
    "potrf": "cciPiii",
    "potrs": "cciiPiPiii",
    "posv": "cciiPiPiii",
    "sytrfnp": "cciPiii",
    "sytrsnp": "cciiPiPiii",
    "sysvnp": "cciiPiPiii",
    "trsm": "ccccciiSPiPiii",
    "gels": "cciiiPiPiPii",
    "pack": "ciiPiLPiiiS",
    "unpack": "ciiPiPiLii",
}

_lib = None


class CbkError(RuntimeError):
    """A nonzero return code: -j (illegal j-th argument) or a CUDA error."""

    def __init__(self, routine: str, info: int):
        self.info = info
        super().__init__(f"{routine}: info={info} ({status_string(info)})")


def lib_path() -> str:
    return os.environ.get("CBK_CUDA_LIB", os.path.join(_HERE, "libcbk_cuda.so"))


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError(
                f"libcbk_cuda.so not found at {path}: build it with `python -m cbk_gb300.build`")
        _lib = ctypes.CDLL(path)
        _lib.cbk_cuda_status_string.restype = ctypes.c_char_p
        _lib.cbk_cuda_status_string.argtypes = [ctypes.c_int]
    return _lib


def version() -> int:
    return lib().cbk_cuda_get_version()


def vlen_ok(V: int) -> bool:
    return bool(lib().cbk_cuda_vlen_ok(int(V)))


def status_string(info: int) -> str:
    return lib().cbk_cuda_status_string(int(info)).decode()


_fns: dict = {}


def _fn(prefix: str, routine: str):
    key = (prefix, routine)
    if key not in _fns:
        name = f"cbk_cuda_{prefix}{routine}_compact_async"
        f = getattr(lib(), name)
        scalar = ctypes.c_double if prefix == "d" else ctypes.c_float
        kinds = SIGNATURES[routine]
        f.argtypes = [{"c": ctypes.c_char, "i": ctypes.c_int, "L": ctypes.c_longlong,
                       "P": ctypes.c_void_p, "S": scalar}[k] for k in kinds] + [ctypes.c_void_p]
        f.restype = ctypes.c_int
        _fns[key] = (f, kinds)
    return _fns[key]


def _ptr(a, prefix):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    # a torch tensor: must live on the GPU with the routine's scalar type
    import torch
    want = torch.float64 if prefix == "d" else torch.float32
    if not a.is_cuda:
        raise TypeError("array arguments must be CUDA tensors (device pointers)")
    if a.dtype != want:
        raise TypeError(f"array dtype {a.dtype} does not match the routine's {want}")
    return a.data_ptr()


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def call(prefix: str, routine: str, *args, stream=None) -> int:
    """Call cbk_cuda_<prefix><routine>_compact_async; returns the info code.
    Array arguments: CUDA tensors or device pointers (int); chars as str."""
    f, kinds = _fn(prefix, routine)
    if len(args) != len(kinds):
        raise TypeError(f"{prefix}{routine}_compact takes {len(kinds)} arguments, got {len(args)}")
    conv = []
    for k, a in zip(kinds, args):
        if k == "c":
            conv.append(a.encode() if isinstance(a, str) else a)
        elif k == "P":
            conv.append(_ptr(a, prefix))
        else:
            conv.append(a)
    # the stream is only touched when there is device work: argument errors
    # and quick returns never need one
    needs_stream = any(k == "P" and a is not None and not isinstance(a, int)
                       for k, a in zip(kinds, args))
    conv.append(_stream(stream) if (needs_stream or stream is not None) else None)
    return f(*conv)


def check(routine: str, info: int) -> int:
    if info != 0:
        raise CbkError(routine, info)
    return info
