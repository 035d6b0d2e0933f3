"""Shared test set-up: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the CUDA library (libscft.so) built
for sm_103a; everything else runs on the CPU.  The oracle under oracle/ is
used only to check results against.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the sm_103a build of libscft")
