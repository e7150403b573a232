"""channel.autograd.TimeMeanWallShear: the checkpointed differentiable
objective.  Its gradients (dJ/dRe, dJ/dmeanU and dJ/dC0 from one exact-adjoint
sweep) must match central finite differences of the objective to 1e-6 and
the forced tangent sweeps (Re forcing kind 3, mean-flux forcing kind 1) to
rounding, and checkpointing must not change the results."""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

GRID = dict(Nx=16, Ny=33, Nz=16, Lx=2 * np.pi, Lz=np.pi, dt=0.01)
RE, MEANU, NSTEPS = 2000.0, 1.0, 12


@pytest.fixture(scope="module")
def mod():
    if not has_gpu():
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    from channel import autograd as ag
    return torch, ag


def _cfg(checkpoint):
    C0 = O.synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=7, amp=5e-2)
    return {"grid": GRID, "C0": C0, "nsteps": NSTEPS, "checkpoint": checkpoint}


def _J(ag, Re, U, checkpoint=4):
    return ag.primal_objective(GRID, Re, U, _cfg(checkpoint)["C0"], NSTEPS, checkpoint)[0]


def test_gradients_match_central_differences(mod):
    torch, ag = mod
    Re = torch.tensor(RE, dtype=torch.float64, requires_grad=True)
    U = torch.tensor(MEANU, dtype=torch.float64, requires_grad=True)
    cfg = _cfg(4)
    J = ag.TimeMeanWallShear.apply(Re, U, cfg)
    J.backward()
    hR, hU = 0.4, 2e-4
    fdR = (_J(ag, RE + hR, MEANU) - _J(ag, RE - hR, MEANU)) / (2 * hR)
    fdU = (_J(ag, RE, MEANU + hU) - _J(ag, RE, MEANU - hU)) / (2 * hU)
    assert abs(float(Re.grad) - fdR) <= 1e-6 * abs(fdR), (float(Re.grad), fdR)
    assert abs(float(U.grad) - fdU) <= 1e-6 * abs(fdU), (float(U.grad), fdU)
    assert cfg["report"]["forward_s"] > 0 and cfg["report"]["backward_s"] > 0


def test_adjoint_parameter_gradients_match_tangent_sweeps(mod):
    """the single reverse sweep's dJ/dRe, dJ/dmeanU against one forced
    tangent sweep per parameter over the same checkpoint intervals"""
    torch, ag = mod
    cfg = _cfg(5)
    J, ckpts, chunks = ag.primal_objective(GRID, RE, MEANU, cfg["C0"], NSTEPS, 5)
    _, dU, dRe = ag.adjoint_gradients(GRID, RE, MEANU, ckpts, chunks, NSTEPS)
    t = ag.tangent_gradients(GRID, RE, MEANU, ckpts, chunks, NSTEPS)
    assert abs(dRe - t[3]) <= 1e-9 * abs(t[3]), (dRe, t[3])
    assert abs(dU - t[1]) <= 1e-9 * abs(t[1]), (dU, t[1])


def test_checkpoint_spacing_does_not_change_results(mod):
    torch, ag = mod
    out = []
    for ck in (3, 5, NSTEPS):
        Re = torch.tensor(RE, dtype=torch.float64, requires_grad=True)
        U = torch.tensor(MEANU, dtype=torch.float64, requires_grad=True)
        J = ag.TimeMeanWallShear.apply(Re, U, _cfg(ck))
        J.backward()
        out.append((float(J.detach()), float(Re.grad), float(U.grad)))
    for o in out[1:]:
        for a, b in zip(o, out[0]):
            assert abs(a - b) <= 1e-12 * abs(b)


def test_state_gradient_matches_central_differences(mod):
    """dJ/dC0 from the exact discrete adjoint (one reverse sweep per
    checkpoint interval) against central differences of J along two random
    directions, to 1e-6; checkpoint spacing leaves it unchanged to rounding."""
    torch, ag = mod
    C0 = _cfg(4)["C0"]
    grads = []
    for ck in (4, NSTEPS):
        Re = torch.tensor(RE, dtype=torch.float64)
        U = torch.tensor(MEANU, dtype=torch.float64)
        Ct = torch.from_numpy(C0.view(np.float64).reshape(C0.shape + (2,)).copy()).requires_grad_(True)
        J = ag.time_mean_wall_shear(Re, U, _cfg(ck), Ct)
        J.backward()
        assert Re.grad is None and Ct.grad is not None
        grads.append(Ct.grad.numpy().copy())
    g = grads[0]
    assert np.linalg.norm(grads[1] - g) <= 1e-12 * np.linalg.norm(g)
    for seed in (11, 12):
        d = O.synthetic_state(GRID["Nx"], GRID["Ny"], GRID["Nz"], seed=seed, laminar=False)
        d *= 1e-2 * np.linalg.norm(C0) / np.linalg.norm(d)
        h = 1e-2
        Jp = ag.primal_objective(GRID, RE, MEANU, C0 + h * d, NSTEPS, 4)[0]
        Jm = ag.primal_objective(GRID, RE, MEANU, C0 - h * d, NSTEPS, 4)[0]
        fd = (Jp - Jm) / (2 * h)
        an = float(np.sum(g * d.view(np.float64).reshape(g.shape)))
        assert abs(an - fd) <= 1e-6 * abs(fd), (an, fd)
