"""The bounds-checked build on the GPU: libcbk_cuda_checked.so (the library
compiled with CBK_CUDA_CHECKED, every matrix-view access tested against the
matrix's logical extent before it is made) runs the routine sweep, the
benchmark orders, the mixed-precision solves on all their kernels, the
bucketed launch and pack / unpack (tests/checked_run.py, in a process of its
own); no access may be refused, and every result must still be the oracle's.
This is the out-of-bounds read and write detection that replaces a
sanitizer, which these tests cannot run."""
import os
import re
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_checked_build_refuses_no_access(cuda):
    from cbk_gb300 import build as B
    path = B.build(checked=True)
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_run.py")],
                       capture_output=True, text=True, timeout=1200,
                       env=dict(os.environ, CBK_CUDA_LIB=path))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    m = re.search(r"checked: (\d+) (-?\d+) (-?\d+) rc=(-?\d+) failures=(.*)", r.stdout)
    assert m, r.stdout[-2000:]
    count, i, j, rc, failures = int(m[1]), int(m[2]), int(m[3]), int(m[4]), m[5]
    assert rc == 0
    assert count == 0, f"{count} view accesses outside their matrix, the first at ({i}, {j})"
    assert failures == "[]", failures

