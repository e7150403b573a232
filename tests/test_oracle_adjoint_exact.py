"""The oracle's exact discrete adjoint (oracle/chan_port.c, cport_adjoint_exact):
the transpose of the homogeneous tangent step (cport_tangent_forcing with
forcing 0, the restatement of channel/channel.c:483-590).

The dot-product identity <lambda, T v> = <T^T lambda, v> pins it: both
sides are FP64 evaluations of one bilinear form.  Their difference,
normalised by |lambda| |T v|, is the rounding of the two sweeps (measured
4e-16 .. 7e-14 on these grids, 3e-13 at 32x65x32; it grows with the
condition of the fourth-order implicit operators).  For random lambda and v
the inner product itself is only a few 1e-2 of that norm product, so the
plain relative difference is checked on a correlated pair
lambda = T v + noise.  Linearity, composition of sub-ranges, the untouched
primal trajectory and a laminar start without run-up (where the tangent
linearises about a re-advanced primal, not the stored one) are checked too.
"""
import numpy as np
import pytest

import oracle as O

GRIDS = [
    (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 2),
    (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 3),
    (12, 17, 24, 2 * np.pi, np.pi, 1000.0, 2.0, 0.01, 3),
]


def dot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def nrm(a):
    return float(np.linalg.norm(a.ravel()))


def _check_pair(p, args, n, v, lam):
    Tv = v.copy()
    assert p.tangent(0, n, Tv, 0) == 0
    Tl = lam.copy()
    assert p.adjoint_exact(n, 0, Tl) == 0
    lhs, rhs = dot(lam, Tv), dot(Tl, v)
    assert abs(lhs - rhs) <= 1e-12 * nrm(lam) * nrm(Tv), (lhs, rhs)
    lam2 = Tv + 0.1 * lam * (nrm(Tv) / nrm(lam))
    Tl2 = lam2.copy()
    assert p.adjoint_exact(n, 0, Tl2) == 0
    lhs, rhs = dot(lam2, Tv), dot(Tl2, v)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs), (lhs, rhs)


@pytest.mark.parametrize("args", GRIDS)
def test_dot_product_identity(args):
    n = args[-1]
    p = O.PortChannel(*args)
    p.primal(0, O.synthetic_state(*args[:3], seed=0))
    mc = np.stack([p.getsoln(i).copy() for i in range(n + 1)])
    for seeds in ((5, 6), (7, 8)):
        _check_pair(p, args, n, O.synthetic_state(*args[:3], seed=seeds[0], laminar=False),
                    O.synthetic_state(*args[:3], seed=seeds[1], laminar=False))
    # sub-ranges compose, up to rounding (the split folds the velocity
    # cotangent into the state cotangent at step 1)
    lam = O.synthetic_state(*args[:3], seed=9, laminar=False)
    whole = lam.copy()
    p.adjoint_exact(n, 0, whole)
    part = lam.copy()
    p.adjoint_exact(n, 1, part)
    p.adjoint_exact(1, 0, part)
    assert nrm(part - whole) <= 1e-11 * nrm(whole)
    # the primal trajectory is read, not written
    assert np.array_equal(np.stack([p.getsoln(i) for i in range(n + 1)]), mc)


def test_laminar_start_without_run_up():
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 3)
    p = O.PortChannel(*args)
    O.libc_srand(2)
    p.primal(0, None)
    _check_pair(p, args, args[-1], O.synthetic_state(*args[:3], seed=3, laminar=False),
                O.synthetic_state(*args[:3], seed=4, laminar=False))


def test_linearity_and_errors():
    args = GRIDS[0]
    n = args[-1]
    p = O.PortChannel(*args)
    p.primal(0, O.synthetic_state(*args[:3], seed=0))
    a = O.synthetic_state(*args[:3], seed=1, laminar=False)
    b = O.synthetic_state(*args[:3], seed=2, laminar=False)
    ta, tb, tab = a.copy(), b.copy(), (2.0 * a - 3.0 * b)
    p.adjoint_exact(n, 0, ta)
    p.adjoint_exact(n, 0, tb)
    p.adjoint_exact(n, 0, tab)
    ref = 2.0 * ta - 3.0 * tb
    assert nrm(tab - ref) <= 1e-13 * nrm(ref)
    assert p.adjoint_exact(0, n, a.copy()) == -2
