"""The Re-sensitivity tangent forcings of the oracle (oracle/chan_port.c,
cport_tangent_forcing) against central finite differences of the primal in Re.

kind 3 is the exact derivative of the discrete RK3 step with respect to Re,
so it must match central differences to the differencing error: at Re = 500
the error is 4e-8 at h = 0.1 (truncation grows as h^2: 1e-6 at h = 0.5;
rounding as 1/h: 1e-6 at h = 0.01).
kind 2 is the reference's own forcing (channel/tangent_forcing.c,
tangent_forcing0.c, increproject.c:61-104) reconnected: a first-order
approximation, applied once per step at the first substage, so it agrees
only to O(dt).
"""
import numpy as np

import oracle as O

ARGS = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 3)


def _final(Re, C0):
    a = list(ARGS)
    a[5] = Re
    p = O.PortChannel(*a)
    C = C0.copy()
    p.primal(0, C)
    return C


def _tangent(kind, C0):
    p = O.PortChannel(*ARGS)
    p.primal(0, C0.copy())
    IC = np.zeros(p.coef_shape, complex)
    p.tangent_forcing(0, ARGS[-1], IC, kind)
    return IC


def test_exact_re_forcing_matches_central_differences():
    C0 = O.synthetic_state(*ARGS[:3], seed=2, amp=5e-2)
    h = 0.1
    fd = (_final(ARGS[5] + h, C0) - _final(ARGS[5] - h, C0)) / (2 * h)
    tan = _tangent(3, C0)
    assert np.linalg.norm(fd) > 0
    assert np.linalg.norm(tan - fd) <= 1e-6 * np.linalg.norm(fd)


def test_reference_re_forcing_is_first_order():
    C0 = O.synthetic_state(*ARGS[:3], seed=2, amp=5e-2)
    h = 0.1
    fd = (_final(ARGS[5] + h, C0) - _final(ARGS[5] - h, C0)) / (2 * h)
    tan = _tangent(2, C0)
    err = np.linalg.norm(tan - fd) / np.linalg.norm(fd)
    assert err < 0.3
    assert np.vdot(tan.ravel(), fd.ravel()).real > 0.9 * np.linalg.norm(tan) * np.linalg.norm(fd)


def test_forcing_kinds_0_and_1_are_the_reference_tangent():
    C0 = O.synthetic_state(*ARGS[:3], seed=2)
    IC0 = O.synthetic_state(*ARGS[:3], seed=5, laminar=False)
    p = O.PortChannel(*ARGS)
    p.primal(0, C0.copy())
    for kind in (0, 1):
        a, b = IC0.copy(), IC0.copy()
        p.tangent(0, ARGS[-1], a, kind)
        p.tangent_forcing(0, ARGS[-1], b, kind)
        assert np.array_equal(a, b)
