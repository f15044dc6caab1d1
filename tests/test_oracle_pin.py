"""The oracle against the reference itself, bit for bit (CPU).

oracle/_ref/libcbk_ref.so is ivan-pi/cbk's own src/cbk.cpp compiled from its
sources (oracle/Makefile); oracle/liboracle.so is the C restatement in
oracle/cbk_oracle.c. Both are built without floating-point contraction, so
every output buffer -- factors, solutions, reflectors, tau, and the padded
lanes and untouched triangles -- must agree to the last bit, over every
routine, both precisions, the reference's widths 2/4/8/16 and (by
re-interleaving at 16 lanes) the GPU widths 32/64.

Skipped where the reference's sources are absent: the golden fixtures carry
the pin there (test_oracle_golden.py).
"""
import numpy as np
import pytest

import cases as C
from oracle import oracle as O


def _ref():
    ref = O.reference()
    if ref is None:
        try:
            O.build(ref=True)
        except Exception:
            pass
        ref = O.reference()
    if ref is None:
        pytest.skip("the reference's sources are not present here")
    return ref


@pytest.mark.parametrize("V", [2, 4, 8, 16])
def test_oracle_equals_reference(V, oracle_lib):
    ref = _ref()
    bad = []
    cases = C.sweep(V_list=(V,))
    for c in cases:
        i1, a = C.run(ref, c)
        i2, b = C.run(oracle_lib, c)
        if i1 != i2 or not C.outputs_equal(a, b):
            bad.append(c.label)
    assert not bad, f"{len(bad)}/{len(cases)} cases differ, e.g. {bad[:5]}"


@pytest.mark.parametrize("V", [32, 64])
def test_oracle_equals_reference_gpu_widths(V, oracle_lib):
    ref = _ref()
    bad = []
    cases = C.sweep(V_list=(V,), quick=True)
    for c in cases:
        i1, a = C.run_any_width(ref, c)
        i2, b = C.run(oracle_lib, c)
        if i1 != i2 or not C.outputs_equal(a, b):
            bad.append(c.label)
    assert not bad, f"{len(bad)}/{len(cases)} cases differ, e.g. {bad[:5]}"


def test_pin_detects_a_planted_difference(oracle_lib):
    """A one-ulp change to one input element must show up as a difference."""
    ref = _ref()
    c = C.make_case("posv", np.float64, 7, 8, 19, "C", "L", 9, 2)
    _, a = C.run(ref, c)
    c2 = c.copy()
    c2.kw["A"][5] = np.nextafter(c2.kw["A"][5], np.inf)
    _, b = C.run(oracle_lib, c2)
    assert not C.outputs_equal(a, b)


def test_argument_checks_equal_reference(oracle_lib):
    """The -j codes of the restated checks equal the reference's over a table
    of illegal and degenerate arguments (src/cbk.cpp:46-320)."""
    ref = _ref()
    import abi_tables
    for routine, dtype, args in abi_tables.rows(reference_widths=True):
        assert ref.call(routine, dtype, *args) == oracle_lib.call(routine, dtype, *args), \
            (routine, args)
