"""The host-pointer layer on the GPU: every routine, both precisions, both
layouts, called with host arrays through cbk_cuda_host_<p><routine>_compact,
leaves exactly what the device entry point leaves in device memory -- bit for
bit, padded lanes and leading-dimension padding included -- and meets the
oracle's bound."""
import numpy as np
import pytest

import cases as C
import gpu_util as G
import host_layer as H

pytestmark = pytest.mark.gpu


def _cases():
    out = []
    seed = 7000
    for dt in (np.float64, np.float32):
        for lay in "CR":
            for r, kw in (("potrf", {}), ("sytrfnp", {}), ("potrs", {"nrhs": 3}),
                          ("posv", {"nrhs": 2}), ("sytrsnp", {"nrhs": 1}),
                          ("sysvnp", {"nrhs": 2}), ("posv", {"nrhs": 0}),
                          ("trsm", {"m": 9, "side": "L", "transa": "T", "alpha": 0.5}),
                          ("trsm", {"m": 5, "side": "R", "alpha": 0.0}),
                          ("geqrf", {"m": 16}), ("orgqr", {"m": 16, "k": 5}),
                          ("ormqr", {"m": 16, "k": 6, "side": "L", "trans": "T"}),
                          ("gels", {"m": 16, "nrhs": 4}), ("gels", {"m": 5, "nrhs": 2})):
                seed += 1
                n = 8 if r not in ("trsm",) else 4
                out.append(C.make_case(r, dt, seed, 32, 45, lay, "L" if seed % 2 else "U", n,
                                       **{**dict(ldpad=seed % 2), **kw}))
    return out


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c.label)
def test_host_layer_equals_device_entry_point(case, cuda, oracle_lib):
    hi, h = H.run_case(case)
    di, d = G.run_gpu(case)
    assert hi == di == 0, (hi, di)
    for k in C.ARRAYS:
        if k in h.kw:
            assert np.array_equal(h.kw[k].view(np.uint8), d.kw[k].view(np.uint8)), k
    oi, o = C.run(oracle_lib, case)
    r = G.lane_ratios_scaled(h, o, case)
    assert all(v <= 8 * G.order_of(case) for v in r.values()), r
