import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (the GB300 parity tests)")


def _build_native():
    """Build the CUDA library and the oracle before the tests import them
    (nvcc cross-compiles here; on a GPU machine build() has usually run)."""
    from fluids2d_gb300 import build as product_build
    from oracle import build as oracle_build
    product_build.build()
    oracle_build.build()


_build_native()
