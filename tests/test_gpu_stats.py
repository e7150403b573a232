"""GPU parity of the device statistics (c_mean_profile, c_mean_product,
c_wall_shear and the channel / channel.sensitivities functions built on
them) against the reference's way of computing them: spec2phys of each
stored step on the oracle, then the x-z average (channel/__init__.py:203-299,
drivers/sensitivities.py).

The device statistics read the mean Fourier mode (and Parseval sums) from
the coefficients; the oracle averages transformed fields.  Both are FP64
evaluations of the same sums: held to 1e-12 relative to the field scale.
"""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 6)
TOL = 1e-12


@pytest.fixture(scope="module")
def both():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel as cc
    port = O.PortChannel(*ARGS)
    C0 = O.synthetic_state(*ARGS[:3], seed=0)
    port.primal(0, C0.copy())
    assert cc.c_init(*ARGS) == 0
    cc.c_primal(0, C0.copy())
    IC = O.synthetic_state(*ARGS[:3], seed=3, laminar=False)
    port.tangent(0, ARGS[-1], IC.copy(), 1)
    cc.c_tangent(0, ARGS[-1], IC.copy(), 1)
    return cc, port


def _flows(port, inc):
    get = port.getincresoln if inc else port.getsoln
    return [port.spec2phys(np.ascontiguousarray(get(i))) for i in range(ARGS[-1] + 1)]


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= TOL * scale, np.abs(a - b).max() / scale


@pytest.mark.parametrize("inc", [0, 1])
def test_mean_profiles(both, inc):
    cc, port = both
    n = ARGS[-1]
    flows = _flows(port, inc)
    for comp in range(3):
        got = cc.c_mean_profile(inc, comp, 0, n + 1)
        ref = np.stack([f[comp].mean(2).mean(0) for f in flows])
        if comp == 1:
            assert np.abs(ref).max() <= 1e-13 * np.abs(flows[0][0]).max()
            assert not got.any()
        else:
            _close(got, ref)


def test_mean_products(both):
    cc, port = both
    n = ARGS[-1]
    fp, ft = _flows(port, 0), _flows(port, 1)
    for (ia, ca, ib, cb) in [(0, 0, 0, 0), (0, 2, 0, 1), (0, 0, 1, 0), (1, 1, 1, 1)]:
        fa = fp if ia == 0 else ft
        fb = fp if ib == 0 else ft
        got = cc.c_mean_product(ia, ca, ib, cb, 1, n + 1)
        ref = np.stack([(fa[i][ca] * fb[i][cb]).mean(2).mean(0) for i in range(1, n + 1)])
        _close(got, ref)


def test_wall_shear(both):
    """Uxb = Rp0 . a with Rp0 = R'(-1) (channel/RsQs.c:158-186)."""
    cc, port = both
    n = ARGS[-1]
    R = ARGS[1] - 2
    P = np.zeros(R)
    P[0], P[1] = 1.0, -1.0
    for k in range(1, R - 1):
        P[k + 1] = ((2 * k + 1) * (-1.0 * P[k]) - k * P[k - 1]) / (k + 1)
    rp0 = np.array([2.0] + [k * P[k - 1] - (k + 2.0) * (-1.0 * P[k]) for k in range(1, R)])
    got = cc.c_wall_shear(0, 0, n + 1)
    # the kernel against the formula on the library's own coefficients
    own = np.array([[rp0 @ cc.c_getsoln(i)[0, v, :, 0].real for v in (0, 1)] for i in range(n + 1)])
    _close(got, own)
    # against the oracle trajectory: the wall derivative weighs the high
    # Legendre modes (|R'_n(-1)| ~ n), so it carries the trajectories' own
    # per-step difference (<= 5e-12 per step) amplified a few times
    ref = np.array([[rp0 @ port.getsoln(i)[0, v, :, 0].real for v in (0, 1)] for i in range(n + 1)])
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()
    # a laminar-like profile: the shear at the lower wall is positive
    assert got[0, 0] > 0


def test_python_statistics(both):
    """channel.velAvg / IvelAvg / uavgGrad and channel.sensitivities against
    the reference formulas evaluated on oracle fields."""
    cc, port = both
    import channel
    from channel import sensitivities as sens
    channel.dt, channel.Re = ARGS[7], ARGS[5]
    n = ARGS[-1]
    T = n * ARGS[7]
    fp, ft = _flows(port, 0), _flows(port, 1)
    mean = lambda f: f.mean(2).mean(0)
    ref_u = sum((ARGS[7] / T) * mean(fp[i][0]) for i in range(n))
    _close(channel.velAvg(0, n, T), ref_u)
    assert abs(channel.velAvg(0, n, T, profile=False) - ref_u[channel.c_channel.c_qpts() // 2 + 1]) \
        <= TOL * np.abs(ref_u).max()
    ref_v = sum((ARGS[7] / T) * mean(ft[i][0]) for i in range(n))
    _close(channel.IvelAvg(0, n, T), ref_v)
    zeta = np.array([0.3, -0.2])
    nb = [0, 3, 6]
    ref_g = sum(sum((ARGS[7] / T) * mean(ft[i][0]) for i in range(nb[k], nb[k + 1]))
                + (1. / T) * zeta[k] * (mean(fp[nb[k + 1]][0]) - ref_u) for k in range(2))
    _close(channel.uavgGrad(2, nb, T, ref_u, zeta), ref_g)
    inv = 1. / (ARGS[5] ** 2)
    ref_du2 = sum((ARGS[7] / T) * mean(2 * fp[i][2] * inv * ft[i][2]) for i in range(n))
    _close(sens.dvel2Avg(2, 0, n, T), ref_du2)
    ref_u2 = sum((ARGS[7] / T) * mean(fp[i][0] * fp[i][0]) for i in range(n))
    _close(sens.vel2Avg(0, 0, n, T), ref_u2)
