"""CPU checks of the LSS driver restatement (oracle/lss_oracle.py)."""
import numpy as np

import oracle as O
from lss_oracle import Wrapper, par_minres


def test_par_minres_solves_symmetric_indefinite():
    rng = np.random.default_rng(0)
    Q, _ = np.linalg.qr(rng.standard_normal((40, 40)))
    A = Q @ np.diag(np.linspace(-3.0, 5.0, 40) + 0.05) @ Q.T
    b = rng.standard_normal(40)
    x, (info, it) = par_minres(lambda v: A @ v, b, np.zeros(40), np.dot, tol=1e-12, maxiter=400)
    assert info == 0 and it <= 400
    assert np.linalg.norm(A @ x - b) <= 1e-9 * np.linalg.norm(b)


def test_wrapper_matvec_is_linear_for_homogeneous_tangents():
    """KKT(a x + y) = a KKT(x) + KKT(y) with inhomo = 0 (the tangent, adjoint
    and ddt_project are linear), on the tiny grid."""
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 4)
    port = O.PortChannel(*args)
    port.primal(0, O.synthetic_state(*args[:3], seed=1))
    wr = Wrapper(port, [0, 2, 4])
    m = int(np.prod(port.coef_shape))

    def vec(seed):
        parts = [O.synthetic_state(*args[:3], seed=seed + j, laminar=False) for j in range(3)]
        return np.concatenate([p.ravel() for p in parts]).view(np.float64).copy()

    x, y = vec(10), vec(20)
    assert x.size == 2 * m * 3
    lhs = wr.matvec(2.5 * x + y, 0)
    rhs = 2.5 * wr.matvec(x, 0) + wr.matvec(y, 0)
    assert np.linalg.norm(lhs - rhs) <= 1e-10 * np.linalg.norm(rhs)
