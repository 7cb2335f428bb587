"""Shared pytest configuration: the gpu marker and import paths."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_DIR = ROOT / "copss-hydrodynamics-private_gb300"
for p in (ROOT, ROOT / "oracle", PKG_DIR):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
