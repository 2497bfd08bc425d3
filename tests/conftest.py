"""Shared pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built C-ABI library; the CPU
suite (`-m "not gpu"`) covers the oracle against the reference's known-answer
tests and golden vectors, the host-side logic, and the library's exports.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "gridaphybrid.jl_gb300")
for p in (ROOT, PKG_DIR, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")
