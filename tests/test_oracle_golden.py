"""The oracle against the golden fixtures made by the reference (CPU).

tests/golden/cbk_ref_golden.npz holds inputs and the reference's outputs
(tests/golden/make_golden.py). The oracle, rebuilt wherever the tests run,
must reproduce every output buffer bit for bit: this pins the oracle on
machines that do not have the reference's sources.
"""
import numpy as np

import cases as C
import make_golden


def test_oracle_reproduces_golden(oracle_lib):
    bad = []
    fixtures = make_golden.load()
    assert len(fixtures) > 300
    for cin, cout, info in fixtures:
        i, got = C.run(oracle_lib, cin)
        if i != info or not C.outputs_equal(got, cout):
            bad.append(cin.label)
    assert not bad, f"{len(bad)} fixtures differ, e.g. {bad[:5]}"


def test_golden_pins_the_benchmark_orders():
    """Orders above the sweep's 33 (the benchmark configurations' 48 and the
    64 x 16 least squares) are among the reference-made fixtures."""
    fx = make_golden.load()
    assert any(c.routine == "posv" and c.kw["n"] == 48 for c, _, _ in fx)
    assert any(c.routine == "sysvnp" and c.kw["n"] == 48 for c, _, _ in fx)
    assert any(c.routine == "gels" and c.kw["m"] == 64 and c.kw["n"] == 16 for c, _, _ in fx)


def test_golden_covers_every_routine():
    seen = {(c.routine, c.dtype) for c, _, _ in make_golden.load()}
    for r in C.ARGS:
        for dt in (np.float64, np.float32):
            assert (r, dt) in seen, (r, dt)
