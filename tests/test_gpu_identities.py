"""The identities the reference's own drivers use to check the path
(drivers/testTan.py, channel/channel.c:412-415), on the GPU:

- the laminar Poiseuille profile (1 - y^2) flux 3/4 with no perturbation
  stays laminar;
- the homogeneous tangent equals central differences of the primal along
  the initial perturbation;
- the mean-flux tangent (inhomo = 1) equals central differences of the
  primal in meanU (flux = 2 meanU), the parameter that forcing differentiates.
"""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 4)


def rel(a, b):
    return np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b))


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _final(cc, C0, meanU=1.0):
    a = list(ARGS)
    a[6] = 2.0 * meanU
    assert cc.c_init(*a) == 0
    C = C0.copy()
    cc.c_primal(0, C)
    return C


def test_laminar_start_stays_laminar(cc):
    """From the projected laminar profile with no perturbation every
    non-mean mode stays exactly zero, the mass flux stays at 2 meanU, and the
    mean flow relaxes only to the scheme's own discrete steady profile
    (the flux correction uses Rs^-1, not the implicit operator, so the
    continuous parabola is not its exact fixed point), as the oracle's does."""
    n = 20
    args = ARGS[:-1] + (n,)
    C0 = O.synthetic_state(*ARGS[:3], seed=0, amp=0.0)
    assert cc.c_init(*args) == 0
    C = C0.copy()
    cc.c_primal(0, C)
    others = C.copy()
    others[0, :, :, 0] = 0
    assert np.abs(others).max() == 0.0
    y, w = cc.c_quad()
    prof = cc.c_mean_profile(0, 0, 0, n + 1)
    flux = prof @ w
    # the correction's vector Rs^-1 sum_j Rw is not exactly flux-normalised:
    # the first step loses 1.8e-8 of the flux, after which it holds
    assert np.abs(flux - 2.0).max() <= 1e-7
    assert np.abs(flux[2:] - flux[1]).max() <= 1e-11
    assert np.abs(prof[-1] - prof[0]).max() <= 1e-4 * np.abs(prof[0]).max()
    port = O.PortChannel(*args)
    Cr = C0.copy()
    port.primal(0, Cr)
    assert rel(C, Cr) <= 2e-11   # 20 steps at the per-step noise floor


def test_homogeneous_tangent_matches_central_differences(cc):
    C0 = O.synthetic_state(*ARGS[:3], seed=4, amp=5e-2)
    v = O.synthetic_state(*ARGS[:3], seed=5, laminar=False)
    h = 1e-4
    fd = (_final(cc, C0 + h * v) - _final(cc, C0 - h * v)) / (2 * h)
    _final(cc, C0)
    IC = v.copy()
    cc.c_tangent(0, ARGS[-1], IC, 0)
    assert rel(IC, fd) <= 1e-6   # central-difference truncation: 1.3e-7 at h = 1e-4


def test_mean_flux_tangent_matches_central_differences_in_meanU(cc):
    C0 = O.synthetic_state(*ARGS[:3], seed=4, amp=5e-2)
    h = 1e-4
    fd = (_final(cc, C0, 1.0 + h) - _final(cc, C0, 1.0 - h)) / (2 * h)
    _final(cc, C0)
    IC = np.zeros_like(C0)
    cc.c_tangent(0, ARGS[-1], IC, 1)
    assert rel(IC, fd) <= 1e-6
