"""The contractions on the tensor cores (csrc/tc_common.cuh: base-256 digit
products in bf16 mma with exact FP32 level sums, recombined in 64-bit
integers and rounded once) -- the reconstruction (csrc/recon_tc.cu), the
quadrature right-hand sides of the implicit solve (quad_rhs_tc,
csrc/recon_solve.cu) and the inverse transforms as DFT GEMMs
(csrc/phys_tc.cu) -- against the FP64 kernels (CHN_RECON_FP64=1 and
CHN_TRANSFORMS_FP64=1 switch them back: k_recon, quad_rhs, the FFTs).

Both evaluate the same contractions; the digit form is the correctly
rounded value of the 56-bit truncated operands' exact sum, the FP64 form
accumulates K rounded products.  spec2phys (reconstruction + inverse
transforms) of one state must agree to 1e-14 of the field scale on every
grid shape class (16x33x16, 32x65x32, 48x97x48 with two kx tiles,
12x17x24 with a partial tile, 16x33x18 with an odd padded z length, where
the inverse's z stage is not split radix-2); a few primal, tangent and adjoint steps stay
within the parity tolerances of test_gpu_parity.py (the difference is
rounding, amplified by the implicit operators like any FP64 reordering).
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

CODE = r"""
import json, sys, numpy as np
sys.path.insert(0, 'shadow-channel_gb300'); sys.path.insert(0, 'oracle')
from channel import c_channel as cc
from channel.synthetic import synthetic_state
Nx, Ny, Nz, n = [int(v) for v in sys.argv[1:5]]
args = (Nx, Ny, Nz, 2 * np.pi, np.pi, 2000.0, 2.0, 0.004, n)
assert cc.c_init(*args) == 0, cc.c_last_error_message()
C = synthetic_state(Nx, Ny, Nz, seed=1)
flow = np.zeros((3, 3 * Nx // 2, cc.c_qpts(), 3 * Nz // 2))
cc.c_spec2phys(C.copy(), flow)
cc.c_primal(0, C)
IC = synthetic_state(Nx, Ny, Nz, seed=2, laminar=False)
cc.c_tangent(0, n, IC, 1)
AC = synthetic_state(Nx, Ny, Nz, seed=3, laminar=False)
cc.c_adjoint(n, 0, AC, 0, 1.0)
assert cc.c_last_error() == 0, cc.c_last_error_message()
print(json.dumps({k: v.view(np.float64).ravel().tolist() for k, v in
                  (("flow", flow), ("C", C), ("IC", IC), ("AC", AC))}))
"""


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("grid", [(16, 33, 16, 3), (32, 65, 32, 3), (48, 97, 48, 1), (12, 17, 24, 3), (16, 33, 18, 3)])
def test_tensor_core_reconstruction_matches_fp64(grid):
    if not has_gpu():
        pytest.skip("no CUDA device")
    root = O.HERE.parent
    outs = []
    for fp64 in ("0", "1"):
        env = dict(os.environ, CHN_RECON_FP64=fp64, CHN_TRANSFORMS_FP64=fp64)
        r = subprocess.run([sys.executable, "-c", CODE, *map(str, grid)], cwd=root, env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append({k: np.array(v) for k, v in
                     json.loads(next(ln for ln in r.stdout.splitlines() if ln.startswith("{"))).items()})
    tc, ref = outs
    scale = np.abs(ref["flow"]).max()
    assert np.abs(tc["flow"] - ref["flow"]).max() <= 1e-14 * scale
    n = grid[3]
    # per-step tolerances: those of test_gpu_parity.py, and at 48x97x48 the
    # one-step FMA/no-FMA floors of test_gpu_large.py (3.2e-11, 1.7e-10,
    # 8.8e-11, held at twice that)
    tp, tt, ta = (7e-11, 4e-10, 2e-10) if grid[0] >= 48 else ((2e-11 if grid[0] >= 32 else 5e-12), 1e-11, 3e-11)
    assert rel(tc["C"], ref["C"]) <= tp * n
    assert rel(tc["IC"], ref["IC"]) <= tt * n
    assert rel(tc["AC"], ref["AC"]) <= ta * n
