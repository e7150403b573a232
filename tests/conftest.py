"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the built product library; all
others run on a CPU-only host (the oracle, host-side logic, the C-ABI export
list, and the multi-process paths over gloo).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "shadow-channel_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built product library")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
