import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    import torch
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


INTR = (525.0, 525.0, 319.5, 239.5)


def _ensure_built():
    lib = ROOT / "superscanner_gb300" / "libss.so"
    shim = ROOT / "superscanner_gb300" / "_build" / "shim_roundtrip"
    if not lib.exists() or not shim.exists():
        import __graft_entry__
        __graft_entry__.build()


_ensure_built()
