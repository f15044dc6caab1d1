"""The C ABI of libcbk_cuda.so on the host (CPU, no GPU needed).

The library must load, export every function include/cbk_cuda.h declares,
and return the reference's -j argument codes and quick returns before any
device work: those paths never touch a pointer or the GPU.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import abi_tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(cbk_cuda_\w+)\s*\(", text))
            # declarations written once per scalar type by a macro
            for stem in re.findall(r"\b(cbk_cuda_\w+?)_##p##(\w+)\s*\(", text):
                names |= {f"{stem[0]}_{p}{stem[1]}" for p in "ds"}
    return sorted(names)


def test_library_loads():
    import cbk_gb300
    lib = cbk_gb300.lib()
    assert isinstance(lib, ctypes.CDLL)
    assert cbk_gb300.version() == 200  # the API of the reference's v0.2.0


def test_every_declared_symbol_is_exported():
    import cbk_gb300
    lib = cbk_gb300.lib()
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_interleave_widths():
    import cbk_gb300
    ok = [V for V in range(0, 1100) if cbk_gb300.vlen_ok(V)]
    assert ok[:4] == [2, 4, 8, 16]
    assert ok[4:] == list(range(32, 1025, 32))


@pytest.mark.parametrize("routine", ["potrf", "sytrfnp", "potrs", "posv", "sytrsnp", "sysvnp",
                                     "trsm", "geqrf", "ormqr", "orgqr", "gels"])
def test_argument_checks(routine, oracle_lib):
    """Every row's code is the expected one, identical in the CUDA library and
    in the oracle (whose checks are pinned to the reference's)."""
    import cbk_gb300
    n = 0
    for r, dt, args, code in abi_tables.rows_with_codes():
        if r != routine:
            continue
        p = "d" if dt == np.float64 else "s"
        got = cbk_gb300.call(p, r, *args)
        assert got == code, (r, dt, args, got, code)
        assert oracle_lib.call(r, dt, *args) == code, (r, dt, args)
        n += 1
    assert n > 20


def test_pack_argument_checks():
    import cbk_gb300
    N = None
    # (layout, m, n, a, lda, stridea, ap, ldap, V, nm, pad)
    b = dict(layout="C", m=4, n=3, a=N, lda=4, stride=12, ap=N, ldap=4, V=32, nm=5, pad=1.0)
    order = ["layout", "m", "n", "a", "lda", "stride", "ap", "ldap", "V", "nm", "pad"]
    rows = [(dict(b, layout="X"), -1), (dict(b, m=-1), -2), (dict(b, n=-1), -3),
            (dict(b, lda=3), -5), (dict(b, stride=11), -6), (dict(b, ldap=3), -8),
            (dict(b, V=7), -9), (dict(b, nm=-1), -10), (dict(b, nm=0), 0), (dict(b, m=0), 0),
            (dict(b, layout="R", lda=2, stride=12, ldap=3, nm=0), -5)]
    for p in "ds":
        for kw, code in rows:
            assert cbk_gb300.call(p, "pack", *[kw[k] for k in order]) == code, (kw, code)
    # unpack: (layout, m, n, ap, ldap, a, lda, stridea, V, nm)
    u = dict(layout="C", m=4, n=3, ap=N, ldap=4, a=N, lda=4, stride=12, V=32, nm=5)
    uorder = ["layout", "m", "n", "ap", "ldap", "a", "lda", "stride", "V", "nm"]
    urows = [(dict(u, layout="X"), -1), (dict(u, ldap=3), -5), (dict(u, lda=3), -7),
             (dict(u, stride=10), -8), (dict(u, V=33), -9), (dict(u, nm=-2), -10),
             (dict(u, n=0), 0)]
    for p in "ds":
        for kw, code in urows:
            assert cbk_gb300.call(p, "unpack", *[kw[k] for k in uorder]) == code, (kw, code)


def test_status_strings():
    import cbk_gb300
    assert cbk_gb300.status_string(0) == "success"
    assert "illegal" in cbk_gb300.status_string(-3)
    assert cbk_gb300.status_string(1002)  # a CUDA error text


def test_bucketed_argument_checks():
    """The bucketed entry points check their table before any device work."""
    import ctypes

    import cbk_gb300
    from cbk_gb300._api import _buckets
    f = cbk_gb300.lib().cbk_cuda_dsysvnp_compact_bucketed_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    ok = _buckets("d", [(8, 40, 32, 0, 8, 0, 8), (5, 3, 32, 0, 5, 0, 5)])
    bad_ld = _buckets("d", [(8, 40, 32, 0, 8, 0, 8), (5, 3, 32, 0, 4, 0, 5)])
    bad_v = _buckets("d", [(8, 40, 24, 0, 8, 0, 8)])
    empty = _buckets("d", [(0, 40, 32, 0, 1, 0, 1), (6, 0, 32, 0, 6, 0, 6)])
    a = ctypes.addressof
    fake_work = 1 << 40  # never dereferenced: every row returns before device work
    assert f(b"X", b"L", 2, 2, a(ok), fake_work, 256, None) == -1
    assert f(b"C", b"X", 2, 2, a(ok), fake_work, 256, None) == -2
    assert f(b"C", b"L", -1, 2, a(ok), fake_work, 256, None) == -3
    assert f(b"C", b"L", 2, 65, a(ok), fake_work, 256, None) == -4
    assert f(b"C", b"L", 2, 2, None, fake_work, 256, None) == -5
    assert f(b"C", b"L", 2, 2, a(bad_ld), fake_work, 256, None) == -5
    assert f(b"C", b"L", 2, 1, a(bad_v), fake_work, 256, None) == -5
    assert f(b"C", b"L", 2, 2, a(ok), None, 256, None) == -6
    assert f(b"C", b"L", 2, 2, a(ok), fake_work, 255, None) == -7
    assert f(b"C", b"L", 2, 2, a(empty), fake_work, 256, None) == 0
    assert f(b"C", b"L", 2, 0, None, fake_work, 256, None) == 0


def test_refined_host_entry_validates_before_any_device_work():
    """cbk_cuda_dposv_refined_compact_host checks its arguments in order and
    returns before touching a pointer or the device (here: no GPU at all)."""
    import cbk_gb300
    f = cbk_gb300.dposv_refined_compact_host
    assert f("X", "L", 8, 1, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == -1
    assert f("C", "Q", 8, 1, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == -2
    assert f("C", "L", -1, 1, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == -3
    assert f("C", "L", 8, -1, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == -4
    assert f("C", "L", 8, 1, None, 7, None, 8, 32, 64, dwork=0, lwork=0) == -6
    assert f("C", "L", 8, 1, None, 8, None, 7, 32, 64, dwork=0, lwork=0) == -8
    assert f("C", "L", 8, 1, None, 8, None, 8, 33, 64, dwork=0, lwork=0) == -9
    assert f("C", "L", 8, 1, None, 8, None, 8, 32, -1, dwork=0, lwork=0) == -10
    assert f("C", "L", 8, 1, None, 8, None, 8, 32, 64, max_iter=-1, dwork=0, lwork=0) == -11
    assert f("C", "L", 8, 1, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == -15
    assert f("C", "L", 8, 0, None, 8, None, 8, 32, 64, dwork=0, lwork=0) == 0
    lw = cbk_gb300.dposv_refined_host_lwork
    assert lw("C", 8, 1, 8, 8, 32, 0) == 0 and lw("C", 8, 1, 8, 8, 33, 64) == -1
    assert lw("X", 8, 1, 8, 8, 32, 64) == -1 and lw("C", 8, 1, 7, 8, 32, 64) == -1
    # three slots, each with a chunk of at least 256 groups (or the batch)
    assert lw("C", 48, 1, 48, 48, 32, 64) >= 3 * 32 * 48 * 48 * 8
    assert lw("C", 48, 1, 50, 48, 32, 64) > lw("C", 48, 1, 48, 48, 32, 64)
    assert lw("C", 48, 1, 48, 48, 32, 10 ** 3) < lw("C", 48, 1, 48, 48, 32, 10 ** 5)
    # chunks are sized by bytes moved (about 192 MiB of A's triangle and B,
    # 643 groups at n = 48): the workspace stops growing with nm
    big = lw("C", 48, 1, 48, 48, 32, 10 ** 6)
    assert big == lw("C", 48, 1, 48, 48, 32, 2 * 10 ** 6)
    assert big < 3 * 700 * 32 * 48 * 48 * 8 + (64 << 20)
    assert lw("C", 8, 1, 8, 8, 32, 10 ** 7) == lw("C", 8, 1, 8, 8, 32, 2 * 10 ** 7)


def test_refined_batched_argument_checks():
    """The strided dense batch entry point: -j in argument order, quick
    returns, the workspace query (CPU only: no device work)."""
    import cbk_gb300
    f = cbk_gb300.dposv_refined_batched
    assert f("X", 8, 1, None, 8, 64, None, 8, 8, 10) == -1
    assert f("L", -1, 1, None, 8, 64, None, 8, 8, 10) == -2
    assert f("L", 8, -1, None, 8, 64, None, 8, 8, 10) == -3
    assert f("L", 8, 1, None, 7, 64, None, 8, 8, 10) == -5
    assert f("L", 8, 1, None, 8, 63, None, 8, 8, 10) == -6
    assert f("L", 8, 1, None, 8, 64, None, 7, 8, 10) == -8
    assert f("L", 8, 2, None, 8, 64, None, 8, 15, 10) == -9
    assert f("L", 8, 1, None, 8, 64, None, 8, 8, -1) == -10
    assert f("L", 8, 1, None, 8, 64, None, 8, 8, 10, max_iter=-1) == -11
    assert f("L", 80, 1, None, 80, 6400, None, 80, 80, 10, work=0, lwork=0) == -15
    assert f("L", 8, 0, None, 8, 64, None, 8, 8, 10) == 0
    assert f("U", 0, 1, None, 1, 0, None, 1, 1, 10) == 0
    lw = cbk_gb300.dposv_refined_batched_lwork
    assert lw(48, 1, 1000) == 0 and lw(80, 1, 100) > 0 and lw(-1, 1, 1) == -1


def test_refined_gels_batched_argument_checks():
    """The least squares' strided dense entry point: -j in argument order
    (CPU only: every row returns before device work)."""
    import cbk_gb300

    def f(*a, **k):
        k.setdefault("work", 0)
        k.setdefault("lwork", 0)
        return cbk_gb300.dgels_refined_batched(*a, **k)
    assert f("T", 8, 4, 1, None, 8, 32, None, 8, 8, None, 10) == -1
    assert f("N", -1, 4, 1, None, 8, 32, None, 8, 8, None, 10) == -2
    assert f("N", 8, 9, 1, None, 8, 72, None, 8, 8, None, 10) == -3
    assert f("N", 80, 70, 1, None, 80, 5600, None, 80, 80, None, 10) == -3
    assert f("N", 8, 4, -1, None, 8, 32, None, 8, 8, None, 10) == -4
    assert f("N", 8, 4, 1, None, 7, 32, None, 8, 8, None, 10) == -6
    assert f("N", 8, 4, 1, None, 8, 31, None, 8, 8, None, 10) == -7
    assert f("N", 8, 4, 1, None, 8, 32, None, 7, 8, None, 10) == -9
    assert f("N", 8, 4, 2, None, 8, 32, None, 8, 15, None, 10) == -10
    assert f("N", 8, 4, 1, None, 8, 32, None, 8, 8, None, -1) == -12
    assert f("N", 8, 4, 1, None, 8, 32, None, 8, 8, None, 10, max_iter=-1) == -13
    assert f("N", 8, 4, 1, None, 8, 32, None, 8, 8, None, 10) == -17
    assert f("N", 8, 4, 0, None, 8, 32, None, 8, 8, None, 10) == 0
    assert cbk_gb300.dgels_refined_batched_lwork(-1, 1, 1, 1) == -1


@pytest.mark.parametrize("p", ["d", "s"])
@pytest.mark.parametrize("routine", ["posv", "sysvnp"])
def test_plain_batched_argument_checks(p, routine):
    """?posv_batched / ?sysvnp_batched on strided dense batches: -j in
    argument order and the quick returns (CPU only: no device work)."""
    import cbk_gb300
    f = getattr(cbk_gb300, f"{p}{routine}_batched")
    assert f("X", 8, 1, None, 8, 64, None, 8, 8, 10) == -1
    assert f("L", -1, 1, None, 8, 64, None, 8, 8, 10) == -2
    assert f("L", 8, -1, None, 8, 64, None, 8, 8, 10) == -3
    assert f("L", 8, 1, None, 7, 64, None, 8, 8, 10) == -5
    assert f("L", 8, 1, None, 8, 63, None, 8, 8, 10) == -6
    assert f("L", 8, 1, None, 8, 64, None, 7, 8, 10) == -8
    assert f("L", 8, 2, None, 8, 64, None, 8, 15, 10) == -9
    assert f("L", 8, 1, None, 8, 64, None, 8, 8, -1) == -10
    assert f("U", 0, 1, None, 1, 0, None, 1, 1, 10) == 0
    assert f("L", 8, 1, None, 8, 64, None, 8, 8, 0) == 0


@pytest.mark.parametrize("p", ["d", "s"])
def test_plain_gels_batched_argument_checks(p):
    """?gels_batched on strided dense batches: -j in argument order (B holds
    max(m, n) rows) and the quick returns (CPU only: no device work)."""
    import cbk_gb300
    f = getattr(cbk_gb300, f"{p}gels_batched")
    assert f("X", 8, 4, 1, None, 8, 32, None, 8, 8, None, 10) == -1
    assert f("N", -1, 4, 1, None, 8, 32, None, 8, 8, None, 10) == -2
    assert f("N", 8, -1, 1, None, 8, 32, None, 8, 8, None, 10) == -3
    assert f("N", 8, 4, -1, None, 8, 32, None, 8, 8, None, 10) == -4
    assert f("N", 8, 4, 1, None, 7, 32, None, 8, 8, None, 10) == -6
    assert f("N", 8, 4, 1, None, 8, 31, None, 8, 8, None, 10) == -7
    assert f("T", 4, 8, 1, None, 4, 32, None, 4, 8, None, 10) == -9
    assert f("N", 8, 4, 2, None, 8, 32, None, 8, 15, None, 10) == -10
    assert f("N", 8, 4, 1, None, 8, 32, None, 8, 8, None, -1) == -12
    assert f("N", 8, 4, 0, None, 8, 32, None, 8, 0, None, 10) == 0
    assert f("N", 0, 0, 1, None, 1, 0, None, 1, 1, None, 10) == 0
    assert f("N", 8, 4, 1, None, 8, 32, None, 8, 8, None, 0) == 0


def _noalloc_fn():
    import ctypes

    import cbk_gb300
    f = cbk_gb300.lib().cbk_cuda_dposv_refined_compact_noalloc_async
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_entry_validates_before_any_device_work():
    """The no-allocation refined solve: the argument codes of the workspace
    entry point, the quick returns, and CBK_CUDA_NOALLOC_TOO_LARGE (900) --
    distinct from -10, an illegal nm -- for a batch beyond the 64 MiB array;
    all before any device work (here: no GPU at all, null pointers)."""
    import cbk_gb300
    f = _noalloc_fn()
    scratch = 64 << 20  # CBK_CUDA_NOALLOC_SCRATCH_BYTES
    n, V = 80, 32
    lw = cbk_gb300.dposv_refined_lwork
    fits = max(nm for nm in range(32, 20000, 32) if lw(n, 1, V, nm) <= scratch)
    assert lw(n, 1, V, fits + 32) > scratch
    assert f(b"X", b"L", n, 1, None, n, None, n, V, 64, 10, None, None, None) == -1
    assert f(b"C", b"Q", n, 1, None, n, None, n, V, 64, 10, None, None, None) == -2
    assert f(b"C", b"L", -1, 1, None, n, None, n, V, 64, 10, None, None, None) == -3
    assert f(b"C", b"L", n, -1, None, n, None, n, V, 64, 10, None, None, None) == -4
    assert f(b"C", b"L", n, 1, None, n - 1, None, n, V, 64, 10, None, None, None) == -6
    assert f(b"C", b"L", n, 1, None, n, None, n - 1, V, 64, 10, None, None, None) == -8
    assert f(b"C", b"L", n, 1, None, n, None, n, 33, 64, 10, None, None, None) == -9
    assert f(b"C", b"L", n, 1, None, n, None, n, V, -1, 10, None, None, None) == -10
    assert f(b"C", b"L", n, 1, None, n, None, n, V, 64, -1, None, None, None) == -11
    assert f(b"C", b"L", n, 1, None, n, None, n, V, fits + 32, 10, None, None, None) == 900
    assert f(b"C", b"L", n, 1, None, n, None, n, V, 0, 10, None, None, None) == 0
    assert f(b"C", b"L", n, 0, None, n, None, n, V, 10 ** 6, 10, None, None, None) == 0
    assert f(b"C", b"L", 0, 1, None, 1, None, 1, V, 10 ** 6, 10, None, None, None) == 0
    assert "too large" in cbk_gb300.status_string(900)
    assert "capturing" in cbk_gb300.status_string(901)


def test_normal_build_reports_no_checking():
    """cbk_cuda_check_status in the normal build: -1 (nothing is checked),
    count 0, no device work."""
    import ctypes

    import cbk_gb300
    f = cbk_gb300.lib().cbk_cuda_check_status
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    count = ctypes.c_ulonglong(7)
    assert f(ctypes.byref(count), None, None, 0) == -1 and count.value == 0


def test_host_layer_argument_codes_and_quick_returns():
    """The host-pointer layer returns every routine's -j codes and quick
    returns before touching an array (null host pointers, no workspace), and
    a size query of a quick return answers 0."""
    import ctypes

    import abi_tables
    import host_layer as H
    for routine, dtype, args, code in abi_tables.rows_with_codes():
        lw = ctypes.c_longlong(-1)
        assert H.call(dtype, routine, args, None, lw) == code, (routine, args, code)
        if code == 0:
            assert lw.value == 0, (routine, args)


def test_host_layer_workspace_query_and_codes():
    """Size query: the arrays the routine touches, each 256-byte aligned; then
    -(k+1) for a missing or small workspace and -(k+2) for a null lwork (k the
    routine's argument count) -- all before any device work."""
    import ctypes

    import host_layer as H
    a = np.zeros(2 * 8 * 8 * 32)
    b = np.zeros(2 * 8 * 32)
    args = ["C", "L", 8, 1, a, 8, b, 8, 32, 64]
    lw = ctypes.c_longlong(-1)
    assert H.call(np.float64, "posv", args, None, lw) == 0
    assert lw.value == 2 * 8 * 8 * 32 * 8 + 2 * 8 * 1 * 32 * 8
    small = ctypes.c_longlong(lw.value - 1)
    assert H.call(np.float64, "posv", args, 1 << 40, small) == -11
    assert H.call(np.float64, "posv", args, None, ctypes.c_longlong(lw.value)) == -11
    assert H.call(np.float64, "posv", args, None, None) == -12
    # potrs reads A and writes B; trsm with alpha = 0 never reads A
    lw = ctypes.c_longlong(-1)
    assert H.call(np.float64, "trsm", ["C", "L", "U", "N", "N", 8, 2, 0.0, None, 8,
                                       np.zeros(2 * 8 * 2 * 32), 8, 32, 64], None, lw) == 0
    assert lw.value == 2 * 8 * 2 * 32 * 8
    lw = ctypes.c_longlong(-1)  # gels 16 x 8: A, B and tau
    assert H.call(np.float32, "gels", ["C", "N", 16, 8, 4, None, 16, None, 16, None, 32, 40],
                  None, lw) == 0
    assert lw.value == 2 * 16 * 8 * 32 * 4 + 2 * 16 * 4 * 32 * 4 + 2 * 8 * 32 * 4


def test_host_chunk_override_in_the_size_query(monkeypatch):
    """CBK_CUDA_HOST_CHUNK_GROUPS sets the host pipeline's chunk (in groups),
    read by the workspace query as by the call: three slots of g groups; an
    unset, zero or unparsable value keeps the default chunking."""
    import cbk_gb300
    lw = cbk_gb300.dposv_refined_host_lwork
    monkeypatch.delenv("CBK_CUDA_HOST_CHUNK_GROUPS", raising=False)
    default = lw("C", 16, 1, 16, 16, 32, 32 * 1000)
    monkeypatch.setenv("CBK_CUDA_HOST_CHUNK_GROUPS", "5")
    five = lw("C", 16, 1, 16, 16, 32, 32 * 1000)
    monkeypatch.setenv("CBK_CUDA_HOST_CHUNK_GROUPS", "10")
    ten = lw("C", 16, 1, 16, 16, 32, 32 * 1000)
    assert 0 < five < ten < default
    for bad in ("0", "-3", "chunks"):
        monkeypatch.setenv("CBK_CUDA_HOST_CHUNK_GROUPS", bad)
        assert lw("C", 16, 1, 16, 16, 32, 32 * 1000) == default
