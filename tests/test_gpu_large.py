"""Grids whose padded planes exceed one block's shared memory run their 2D
transforms as separate z and x passes (csrc/phys.cu, split transforms).

- The split passes are the fused FFT kernels' 1D transforms on the same
  data, so forcing them (CHN_SPLIT_TRANSFORMS=1, each block-size / chunk
  variant the autotuner chooses from) at 32x65x32 must reproduce the fused
  FFT results bit for bit through primal, tangents, the coupled adjoint and
  the exact adjoint (CHN_TRANSFORMS_FP64=1 keeps the inverse on the FFT
  kernels in both runs; the tensor-core inverse is compared with them in
  test_gpu_recon_tc.py).
- 48x97x48 (113 KB per plane) and 128x129x128 (no plane fits a block:
  split transforms) against the oracle, one step each way, and the exact
  adjoint's dot-product identity.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

# One step each way at these sizes, the oracle built with and without FMA
# contraction differs by (primal, tangent, adjoint) 3.2e-11, 1.7e-10,
# 8.8e-11 at 48x97x48 and 3.1e-10, 1.6e-9, 9.7e-10 at 128x129x128 (the
# implicit fourth-order operators amplify rounding with the mode count): the
# GPU is held to twice that floor.
TOL = {48: (7e-11, 4e-10, 2e-10), 128: (7e-10, 4e-9, 2e-9)}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


@pytest.fixture(scope="module")
def gpu():
    if not has_gpu():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_split_transforms_bitwise_equal_fused(gpu, variant):
    code = r"""
import ctypes, json, sys, numpy as np
sys.path.insert(0, 'shadow-channel_gb300'); sys.path.insert(0, 'oracle')
from channel import c_channel as cc
from channel.synthetic import synthetic_state
args = (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 3)
assert cc.c_init(*args) == 0
lib = cc.lib
assert lib.c_batch_init(2, 2, 1) == 0
C = np.stack([synthetic_state(32, 65, 32, seed=s) for s in range(2)])
IC = np.stack([np.stack([synthetic_state(32, 65, 32, seed=10 + 2 * s + j, laminar=False) for j in range(2)])
               for s in range(2)])
AC = np.stack([synthetic_state(32, 65, 32, seed=20 + s, laminar=False) for s in range(2)])
inh = (ctypes.c_int * 2)(0, 1)
assert lib.c_batch_forward(0, 3, C.ctypes.data, IC.ctypes.data, inh) == 0, cc.c_last_error_message()
assert lib.c_batch_adjoint(3, 0, AC.ctypes.data, 1.0) == 0, cc.c_last_error_message()
AE = np.stack([synthetic_state(32, 65, 32, seed=30 + s, laminar=False) for s in range(2)])
assert lib.c_batch_adjoint_exact(3, 0, AE.ctypes.data) == 0, cc.c_last_error_message()
flow = np.zeros((3, 48, 97, 48))
cc.c_spec2phys(np.ascontiguousarray(C[0]), flow)
print(json.dumps({k: v.view(np.float64).ravel().tolist() for k, v in
                  (("C", C), ("IC", IC), ("AC", AC), ("AE", AE), ("flow", flow))}))
"""
    root = O.HERE.parent
    outs = []
    for split in ("0", "1"):
        env = dict(os.environ, CHN_SPLIT_TRANSFORMS=split, CHN_SPLIT_VARIANT=str(variant), CHN_AUTOTUNE="0",
                   CHN_TRANSFORMS_FP64="1")
        r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(next(ln for ln in r.stdout.splitlines() if ln.startswith("{"))))
    for key in ("C", "IC", "AC", "AE", "flow"):
        assert np.array_equal(np.array(outs[0][key]), np.array(outs[1][key])), key


@pytest.mark.parametrize("grid", [(48, 97, 48), (128, 129, 128)])
def test_large_grid_one_step_each_way(gpu, grid):
    from channel import c_channel as cc
    Nx, Ny, Nz = grid
    big = Nx == 128
    Lx, Lz = (4 * np.pi, 2 * np.pi) if big else (2 * np.pi, np.pi)
    dt = 0.002 if big else 0.005
    args = (Nx, Ny, Nz, Lx, Lz, 3300.0, 2.0, dt, 1)
    C0 = O.synthetic_state(Nx, Ny, Nz, seed=1, Lx=Lx, Lz=Lz)
    IC0 = O.synthetic_state(Nx, Ny, Nz, seed=2, laminar=False, Lx=Lx, Lz=Lz)
    AC0 = O.synthetic_state(Nx, Ny, Nz, seed=3, laminar=False, Lx=Lx, Lz=Lz)
    port = O.PortChannel(*args)
    assert cc.c_init(*args) == 0, cc.c_last_error_message()
    res = {}
    for who, ch in (("gpu", cc), ("ref", port)):
        C, IC, AC = C0.copy(), IC0.copy(), AC0.copy()
        if who == "gpu":
            cc.c_primal(0, C)
            cc.c_tangent(0, 1, IC, 1)
            cc.c_adjoint(1, 0, AC, 0, 1.0)
        else:
            port.primal(0, C)
            port.tangent(0, 1, IC, 1)
            port.adjoint(1, 0, AC, 0, 1.0)
        res[who] = (C, IC, AC)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    tp, tt, ta = TOL[Nx]
    assert rel(res["gpu"][0], res["ref"][0]) <= tp
    assert rel(res["gpu"][1], res["ref"][1]) <= tt
    assert rel(res["gpu"][2], res["ref"][2]) <= ta
    # the exact adjoint: the dot-product identity with the homogeneous
    # tangent on the GPU, and the oracle's transpose within the tangent floor
    v, lam = IC0.copy(), AC0.copy()
    cc.c_tangent(0, 1, v, 0)
    cc.c_adjoint_exact(1, 0, lam)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    d = lambda a, b: float(np.sum(a.real * b.real + a.imag * b.imag))
    lhs, rhs = d(AC0, v), d(lam, IC0)
    assert abs(lhs - rhs) <= 1e-11 * np.linalg.norm(AC0) * np.linalg.norm(v), (lhs, rhs)
    ref = AC0.copy()
    assert port.adjoint_exact(1, 0, ref) == 0
    assert rel(lam, ref) <= tt
