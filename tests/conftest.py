"""pytest configuration: the `gpu` marker and import paths.

Tests marked gpu run the CUDA library on a GPU and call it through the C ABI
(include/cbk_cuda.h); everything else runs on the CPU: the oracle and its pin
against the reference, the golden fixtures, the host-side argument checks and
the library's exported symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    return O.oracle()


@pytest.fixture(scope="session")
def cuda():
    """The CUDA library on a live device; the product path has no CPU fallback,
    so a GPU test fails (does not skip) when the library cannot load."""
    import torch
    import cbk_gb300
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    cbk_gb300.lib()
    return cbk_gb300
