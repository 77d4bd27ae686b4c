"""Test configuration: import paths, the `gpu` marker, shared fixtures.

Tests marked `gpu` need a CUDA device; everything else runs on the CPU
(the oracle, the host store, the C-ABI library's exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "opencl-sph_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _ensure_built():
    lib = os.path.join(PKG, "lib", "libsph_gb300.so")
    if not os.path.exists(lib):
        sys.path.insert(0, PKG)
        import build
        build.build()
    from oracle import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()


_ensure_built()
