"""TEST INFRASTRUCTURE (the oracle), not the product.

ctypes binding of the CPU oracle (oracle/liboracle*.so, the C restatement of
ivan-pi/cbk's compact batch kernels) and, where it was built, of the
reference itself (oracle/_ref/libcbk_ref.so, compiled from the reference's own
src/cbk.cpp). Both export include/cbk.h's 22 entry points -- the oracle with
an ``oracle_`` prefix -- with host pointers.

Also numpy helpers that pack dense batches into the compact layout of
include/cbk.h:22-29 and back (the test-side pack_compact / unpack_compact /
pack_tau of tests/test_compact_util.hpp:477-562: padded slots carry the
identity, tau padding is zero).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# argument kinds: c char, i int, P array, S scalar of the routine's type
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
    "trsm": "cccccIISPiPiii".replace("I", "i"),
    "gels": "cciiiPiPiPii",
}

_LIBS: dict = {}


def build(ref: bool = False) -> None:
    """Compile the oracle (and the reference, if asked and present) with make."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class CbkLib:
    """One loaded library exposing the cbk.h entry points under a prefix."""

    def __init__(self, path: str, prefix: str):
        self.path = path
        self.prefix = prefix
        self.lib = ctypes.CDLL(path)
        self._fns = {}

    def fn(self, dtype, routine):
        key = (np.dtype(dtype).char, routine)
        if key in self._fns:
            return self._fns[key]
        p = "d" if np.dtype(dtype) == np.float64 else "s"
        f = getattr(self.lib, f"{self.prefix}{p}{routine}_compact")
        scalar = ctypes.c_double if p == "d" else ctypes.c_float
        kinds = SIGNATURES[routine]
        f.argtypes = [
            {"c": ctypes.c_char, "i": ctypes.c_int, "P": ctypes.c_void_p, "S": scalar}[k]
            for k in kinds
        ]
        f.restype = ctypes.c_int
        self._fns[key] = (f, kinds)
        return self._fns[key]

    def call(self, routine, dtype, *args):
        """Call routine with numpy arrays for the array arguments (modified in
        place) and Python scalars/str for the rest; returns the info code."""
        f, kinds = self.fn(dtype, routine)
        conv = []
        for k, a in zip(kinds, args):
            if k == "c":
                conv.append(a.encode() if isinstance(a, str) else a)
            elif k == "P":
                if a is None:
                    conv.append(None)
                else:
                    assert isinstance(a, np.ndarray) and a.dtype == np.dtype(dtype)
                    assert a.flags["C_CONTIGUOUS"]
                    conv.append(a.ctypes.data)
            else:
                conv.append(a)
        return f(*conv)


def oracle(fast: bool = False) -> CbkLib:
    """The oracle: liboracle.so (no contraction, the checker) or
    liboracle_fast.so (the CPU-baseline build)."""
    name = "liboracle_fast.so" if fast else "liboracle.so"
    path = os.path.join(HERE, name)
    if name not in _LIBS:
        if not os.path.exists(path):
            build()
        _LIBS[name] = CbkLib(path, "oracle_")
    return _LIBS[name]


def reference(fast: bool = False) -> CbkLib | None:
    """The reference's own build, or None where it was not built: the pin
    build (no contraction) or, fast=True, its performance build (-O3, the
    host's native vector ISA, OpenMP), the timed CPU baseline."""
    name = "libcbk_ref_fast.so" if fast else "libcbk_ref.so"
    path = os.path.join(HERE, "_ref", name)
    if not os.path.exists(path):
        return None
    if name not in _LIBS:
        _LIBS[name] = CbkLib(path, "")
    return _LIBS[name]


def max_threads() -> int:
    lib = oracle().lib
    lib.oracle_max_threads.restype = ctypes.c_int
    return lib.oracle_max_threads()


# ---------------------------------------------------------------------------
# compact layout helpers (numpy, host)
# ---------------------------------------------------------------------------

def group_stride(rowmajor: bool, ld: int, rows: int, cols: int, V: int) -> int:
    """Scalars per group of V interleaved rows x cols matrices."""
    return ld * (rows if rowmajor else cols) * V


def compact_size(nm: int, rows: int, cols: int, ld: int, V: int, rowmajor=False) -> int:
    ng = (nm + V - 1) // V
    return max(1, ng * group_stride(rowmajor, ld, rows, cols, V))


def pack(mats: np.ndarray, V: int, ld: int | None = None, rowmajor: bool = False,
         pad_diag: float = 1.0) -> np.ndarray:
    """Dense (nm, rows, cols) batch -> flat compact buffer. Padded slots of the
    last group carry pad_diag on the diagonal and zero elsewhere; rows beyond
    the matrix inside the leading dimension are zero."""
    nm, rows, cols = mats.shape
    if ld is None:
        ld = max(1, cols if rowmajor else rows)
    ng = (nm + V - 1) // V
    out = np.zeros(compact_size(nm, rows, cols, ld, V, rowmajor), dtype=mats.dtype)
    if ng == 0 or rows == 0 or cols == 0:
        return out
    full = np.zeros((ng * V, rows, cols), dtype=mats.dtype)
    full[:nm] = mats
    if ng * V > nm:
        k = min(rows, cols)
        full[nm:, np.arange(k), np.arange(k)] = pad_diag
    g = full.reshape(ng, V, rows, cols)
    if rowmajor:
        view = out[: ng * rows * ld * V].reshape(ng, rows, ld, V)
        view[:, :, :cols, :] = g.transpose(0, 2, 3, 1)
    else:
        view = out[: ng * cols * ld * V].reshape(ng, cols, ld, V)
        view[:, :, :rows, :] = g.transpose(0, 3, 2, 1)
    return out


def unpack(buf: np.ndarray, nm: int, rows: int, cols: int, V: int, ld: int | None = None,
           rowmajor: bool = False) -> np.ndarray:
    """Flat compact buffer -> dense (nm, rows, cols) batch."""
    if ld is None:
        ld = max(1, cols if rowmajor else rows)
    ng = (nm + V - 1) // V
    if ng == 0 or rows == 0 or cols == 0:
        return np.zeros((nm, rows, cols), dtype=buf.dtype)
    if rowmajor:
        view = buf[: ng * rows * ld * V].reshape(ng, rows, ld, V)[:, :, :cols, :]
        g = view.transpose(0, 3, 1, 2)
    else:
        view = buf[: ng * cols * ld * V].reshape(ng, cols, ld, V)[:, :, :rows, :]
        g = view.transpose(0, 3, 2, 1)
    return np.ascontiguousarray(g.reshape(ng * V, rows, cols)[:nm])


def pack_tau(tau: np.ndarray, V: int) -> np.ndarray:
    """(nm, k) reflector scalars -> compact tau buffer (padding zero)."""
    nm, k = tau.shape
    return pack(tau.reshape(nm, k, 1), V, ld=max(1, k), pad_diag=0.0)


def unpack_tau(buf: np.ndarray, nm: int, k: int, V: int) -> np.ndarray:
    return unpack(buf, nm, k, 1, V, ld=max(1, k)).reshape(nm, k)
