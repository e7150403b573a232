"""The FP64 noise floor of the reference algorithm itself.

The reference path is built twice -- the oracle port as pinned (no FMA
contraction) and the same source with FMA contraction allowed -- and the two
builds run the same seeded case.  Both are valid FP64 evaluations; their
difference is the reproducibility any reimplementation can be held to.  The
implicit fourth-order operators amplify rounding, so this floor is ~1e-12
per step at 16x33x16 and ~1e-11 at 32x65x32.  tests/test_gpu_parity.py
bounds the GPU at a small multiple of it.
"""
import ctypes
import platform
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O

HERE = Path(__file__).resolve().parent.parent / "oracle"


def _build_fma(tmp_path):
    out = tmp_path / "libchanport_fma.so"
    flags = ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", *flags, "-o", str(out),
                    str(HERE / "chan_port.c"), str(HERE / "fft.c"), "-lm"], check=True)
    return out


def _run(lib_path, args):
    saved = (O.PortChannel._lib, O.PORT_LIB)
    try:
        O.PortChannel._lib = None
        O.PORT_LIB = Path(lib_path)
        ch = O.PortChannel(*args)
        n = args[-1]
        C = O.synthetic_state(*args[:3], seed=0)
        ch.primal(0, C)
        traj = [ch.getsoln(i) for i in range(n + 1)]
        IC = O.synthetic_state(*args[:3], seed=3, laminar=False)
        ch.tangent(0, n, IC, 1)
        AC = O.synthetic_state(*args[:3], seed=4, laminar=False)
        ch.adjoint(n, 0, AC, 0, 0.0)
        ch.close()
        return traj, IC, AC
    finally:
        O.PortChannel._lib, O.PORT_LIB = saved


def test_fp64_noise_floor_16(tmp_path):
    args = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 6)
    O.build_port()
    a = _run(O.PORT_LIB, args)
    b = _run(_build_fma(tmp_path), args)
    rel = lambda x, y: np.linalg.norm(x - y) / np.linalg.norm(y)
    per_step = [rel(a[0][i], b[0][i]) for i in range(1, args[-1] + 1)]
    # the two evaluations differ, and by an amount far above one rounding
    assert max(per_step) > 1e-13
    assert max(per_step) < 5e-11
    assert rel(a[2], b[2]) < 1e-9
