"""Pin the CPU oracle before trusting it.

1. The C restatement (oracle/chan_port.c) against the golden fixtures made
   from the reference itself (tests/golden/make_golden.py): bit-exact on the
   build host, and within 1e-13 relative on any other host (the GPU host's
   compiler may round the odd libm call differently).
2. Where the reference tree exists, the port against the reference compiled
   in place, bit for bit, on fresh seeded inputs.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / den


def _replay(cls, g):
    args = tuple(g["args"])
    Nx, Ny, Nz = (int(v) for v in args[:3])
    n = int(args[-1])
    ch = cls(Nx, Ny, Nz, *args[3:8], n)
    out = {}
    C = g["C0"].copy()
    ch.primal(0, C)
    out["C"] = C
    out["traj"] = np.stack([ch.mc_sub(k) for k in range(3 * n + 1)])
    IC = g["IC0"].copy()
    ch.tangent(0, n, IC, 1)
    out["IC_inh"] = IC
    IC = g["IC_hom0"].copy()
    ch.tangent(0, n, IC, 0)
    out["IC_hom"] = IC
    out["mic"] = np.stack([ch.mic_sub(k) for k in range(3 * n + 1)])
    AC = g["AC0"].copy()
    ch.adjoint(n, 0, AC, 0, 0.5)
    out["AC"] = AC
    AC = g["AC0b"].copy()
    ch.adjoint(n, 1, AC, 0, 0.0)
    out["ACb"] = AC
    V = g["V0"].copy()
    out["proj"] = ch.ddt_project(1, V)
    out["V"] = V
    out["flow"] = ch.spec2phys(out["C"])
    out["y"], out["w"] = ch.quad()
    if hasattr(ch, "close"):
        ch.close()
    O.libc_srand(1)
    ch2 = cls(Nx, Ny, Nz, *args[3:8], n)
    ch2.primal(0, None)
    out["laminar_srand1"] = np.stack([ch2.getsoln(i) for i in range(n + 1)])
    if hasattr(ch2, "close"):
        ch2.close()
    return out


@pytest.mark.parametrize("case", ["tiny", "cfg0"])
def test_port_matches_golden(case):
    g = dict(np.load(GOLD / f"golden_{case}.npz"))
    out = _replay(O.PortChannel, g)
    for key in ("C", "IC_inh", "IC_hom", "AC", "ACb", "V", "y", "w"):
        assert _rel(out[key], g[key]) <= 1e-13, key
    assert abs(out["proj"] - float(g["proj"])) <= 1e-13 * max(1.0, abs(float(g["proj"])))
    traj, mic, lam = out["traj"], out["mic"], out["laminar_srand1"]
    if "traj_idx" in g:
        traj = traj[g["traj_idx"]]
        mic = mic[g["mic_idx"]]
        lam = lam[[0, -1]]
    assert _rel(traj, g["traj"]) <= 1e-13
    assert _rel(mic, g["mic"]) <= 1e-13
    assert _rel(lam, g["laminar_srand1"]) <= 1e-13
    if "flow" in g:
        assert _rel(out["flow"], g["flow"]) <= 1e-13


@pytest.mark.skipif(not O.RefChannel.available(), reason="reference tree not present on this host")
@pytest.mark.parametrize("seed", [11, 12])
def test_port_bitwise_equals_reference(seed):
    """Fresh inputs, every entry point, bit-for-bit equality."""
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz = 8, 13, 8
    n = 3
    args = (Nx, Ny, Nz, 2 * np.pi, np.pi, 1000.0 + 500 * rng.random(), 2.0, 0.01, n)
    g = dict(args=np.array(args),
             C0=O.synthetic_state(Nx, Ny, Nz, seed=seed),
             IC0=O.synthetic_state(Nx, Ny, Nz, seed=seed + 1, laminar=False),
             IC_hom0=O.synthetic_state(Nx, Ny, Nz, seed=seed + 2, laminar=False),
             AC0=O.synthetic_state(Nx, Ny, Nz, seed=seed + 3, laminar=False),
             AC0b=O.synthetic_state(Nx, Ny, Nz, seed=seed + 4, laminar=False),
             V0=O.synthetic_state(Nx, Ny, Nz, seed=seed + 5, laminar=False))
    ref = _replay(O.RefChannel, g)
    port = _replay(O.PortChannel, g)
    for key in ref:
        assert np.array_equal(np.asarray(ref[key]), np.asarray(port[key])), key


def test_port_reentrant_instances():
    """Two live port instances do not share state (the reference cannot do this)."""
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 2)
    a = O.PortChannel(*args)
    b = O.PortChannel(*args)
    Ca = O.synthetic_state(8, 9, 8, seed=1)
    Cb = O.synthetic_state(8, 9, 8, seed=2)
    Ca2, Cb2 = Ca.copy(), Cb.copy()
    a.primal(0, Ca)
    b.primal(0, Cb)
    c = O.PortChannel(*args)
    c.primal(0, Ca2)
    assert np.array_equal(Ca, Ca2)
    assert not np.array_equal(Ca, Cb)


def test_init_rejects_bad_sizes():
    with pytest.raises(ValueError):
        O.PortChannel(10, 9, 8, 1.0, 1.0, 100.0, 2.0, 0.01, 1)  # Nx % 4 != 0
    with pytest.raises(ValueError):
        O.PortChannel(8, 9, 7, 1.0, 1.0, 100.0, 2.0, 0.01, 1)  # Nz odd
    with pytest.raises(ValueError):
        O.PortChannel(8, 3, 8, 1.0, 1.0, 100.0, 2.0, 0.01, 1)  # Ny < 4
