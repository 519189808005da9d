"""pytest configuration: the `gpu` marker and import paths.

Tests marked gpu need a CUDA device and the built library; everything else runs
on a CPU-only machine (the oracle, host logic, and the library's exports).
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "scale-dg-kernel-extraction_gb300"):
    path = os.path.join(ROOT, sub)
    if path not in sys.path:
        sys.path.insert(0, path)


def _ensure_built():
    """Builds the CUDA library (nvcc cross-compiles without a GPU) and the
    oracle when they are missing or older than their sources."""
    import build as product_build  # scale-dg-kernel-extraction_gb300/build.py
    import oracle
    product_build.build()
    oracle.build()


_ensure_built()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
