"""Long-run statistics: the time-mean streamwise velocity profile and the
time-mean wall shear of a 400-step run (16x33x16, Re 2000) from the GPU and
from the oracle agree.  Both are FP64 evaluations of one chaotic system; the
per-step difference (~1e-12) grows with the flow's instability but stays far
below the sampling error of such short means (held here to 1e-8 relative)."""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 400)


def test_mean_profile_and_wall_shear(tmp_path):
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel as cc
    n = ARGS[-1]
    C0 = O.synthetic_state(*ARGS[:3], seed=11, amp=5e-2)
    port = O.PortChannel(*ARGS)
    port.primal(0, C0.copy())
    assert cc.c_init(*ARGS) == 0
    cc.c_primal(0, C0.copy())
    # GPU statistics from the device (mean mode of the stored coefficients)
    u_gpu = cc.c_mean_profile(0, 0, 0, n).mean(axis=0)
    tau_gpu = cc.c_wall_shear(0, 0, n)[:, 0].mean()
    # oracle: the reference's way, spec2phys of every step averaged over x, z
    u_ref = np.mean([port.spec2phys(np.ascontiguousarray(port.getsoln(i)))[0].mean(2).mean(0)
                     for i in range(0, n, 1)], axis=0)
    R = ARGS[1] - 2
    P = np.zeros(R)
    P[0], P[1] = 1.0, -1.0
    for k in range(1, R - 1):
        P[k + 1] = ((2 * k + 1) * (-P[k]) - k * P[k - 1]) / (k + 1)
    rp0 = np.array([2.0] + [k * P[k - 1] + (k + 2.0) * P[k] for k in range(1, R)])
    tau_ref = np.mean([rp0 @ port.getsoln(i)[0, 0, :, 0].real for i in range(n)])
    assert np.abs(u_gpu - u_ref).max() <= 1e-8 * np.abs(u_ref).max()
    assert abs(tau_gpu - tau_ref) <= 1e-8 * abs(tau_ref)
