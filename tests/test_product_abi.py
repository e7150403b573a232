"""The product library loads on a CPU-only host and exports the C ABI.

No compute calls here (no GPU); the parity tests are in test_gpu_parity.py.
"""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "c_channel.h"
LIB = ROOT / "shadow-channel_gb300" / "libc_channel.so"


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(c_[A-Za-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not LIB.exists():
        import sys
        sys.path.insert(0, str(ROOT / "shadow-channel_gb300"))
        import build  # noqa: F401
        build.build()
    return ctypes.CDLL(str(LIB))


def test_header_declares_reference_entry_points():
    names = set(_declared())
    # channel/channel.i:17-229
    for n in ["c_init", "c_destroy", "c_primal", "c_tangent", "c_adjoint", "c_ddt_project", "c_getsoln",
              "c_getincresoln", "c_spec2phys", "c_read_solution", "c_save_solution", "c_quad", "c_qpts",
              "c_dimR", "c_dimQ", "c_Nx", "c_Nz", "c_nsteps"]:
        assert n in names, n


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_no_cpu_fallback_symbols(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB)], capture_output=True, text=True).stdout
    assert "cport_" not in out and "offt_" not in out  # the oracle is never linked in


def test_getters_before_init(lib):
    lib.c_qpts.restype = ctypes.c_int
    assert lib.c_qpts() == 0
