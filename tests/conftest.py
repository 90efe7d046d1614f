"""Shared pytest setup: the gpu marker and import paths.

``-m gpu`` tests call the CUDA library through its C ABI and compare with
the FP64 CPU oracle; ``-m "not gpu"`` tests cover the oracle against the
reference's known answers, the host logic, and that the C-ABI library
exports every symbol its header declares.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "geostat-rs_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
