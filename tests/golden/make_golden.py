"""Generate the golden fixtures from the reference itself (test infrastructure).

Runs ivan-pi/cbk's own src/cbk.cpp (compiled by oracle/Makefile into
oracle/_ref/libcbk_ref.so; that needs the reference sources, so this script
runs only where they are) on a fixed subset of the seeded cases of
tests/cases.py and stores inputs, outputs and return codes in
tests/golden/cbk_ref_golden.npz. Cases at GPU interleave widths (32, 64) are
run through the reference at width 16 by re-interleaving every lane
(tests/cases.py:reinterleave), which computes exactly the same lanes.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402

import cases as C  # noqa: E402

OUT = os.path.join(HERE, "cbk_ref_golden.npz")


MAX_BYTES = 24_000  # per case, inputs only: keeps the fixture file small


def select():
    """Every routine over both dtypes, layouts, triangles / sides / transposes,
    the small dimensions and a panel-crossing order, at the reference width 4
    and the GPU width 32: a deterministic thinning of the quick sweep."""
    picked = []
    for V, stride in ((4, 5), (32, 7)):
        count = {}
        for c in C.sweep(V_list=(V,), quick=True):
            size = sum(c.kw[k].nbytes for k in C.ARRAYS if k in c.kw)
            if size > MAX_BYTES:
                continue
            k = count.get(c.routine, 0)
            count[c.routine] = k + 1
            if k % stride == 0:
                picked.append(c)
    # the benchmark configurations' orders and shapes (n = 32 / 48, 64 x 16),
    # at the reference's width 2 with one padded lane: above the size cap, so
    # kept to three matrices each
    picked += C.benchmark_shapes(V=2, nm=3)
    return picked


def main():
    ref = O.reference()
    if ref is None:
        O.build(ref=True)
        ref = O.reference()
    if ref is None:
        raise SystemExit("the reference could not be built (its sources are needed)")
    cases = select()
    meta = []
    arrays = {}
    for i, c in enumerate(cases):
        info, out = C.run_any_width(ref, c)
        kw = {k: v for k, v in c.kw.items() if k not in C.ARRAYS}
        meta.append({"routine": c.routine, "dtype": np.dtype(c.dtype).name, "kw": kw,
                     "arrays": sorted(k for k in c.kw if k in C.ARRAYS), "info": int(info)})
        for k in C.ARRAYS:
            if k in c.kw:
                arrays[f"c{i}_in_{k}"] = c.kw[k]
                arrays[f"c{i}_out_{k}"] = out.kw[k]
    np.savez_compressed(OUT, meta=np.array(json.dumps(meta)), **arrays)
    print(f"{len(cases)} cases -> {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB)")


def load():
    """The fixtures as a list of (Case with the inputs, Case with the
    reference's outputs, info)."""
    z = np.load(OUT)
    meta = json.loads(str(z["meta"]))
    res = []
    for i, m in enumerate(meta):
        dt = np.dtype(m["dtype"]).type
        kin = dict(m["kw"])
        kout = dict(m["kw"])
        for k in m["arrays"]:
            kin[k] = z[f"c{i}_in_{k}"]
            kout[k] = z[f"c{i}_out_{k}"]
        res.append((C.Case(m["routine"], dt, kin), C.Case(m["routine"], dt, kout), m["info"]))
    return res


if __name__ == "__main__":
    main()
