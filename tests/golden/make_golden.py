"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own channel/*.c (compiled in place by ``make -C oracle
ref`` against the FFTW-2 shim) through its entry points on small seeded
cases and stores inputs and outputs as compressed .npz files.  The reference
tree only exists on the build host, so the fixtures are committed; tests on
any host compare the oracle port and the GPU product against them.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import oracle as O  # noqa: E402

CASES = {
    # name: (Nx, Ny, Nz, Lx, Lz, Re, flux, dt, nsteps)
    "tiny": (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 3),
    "cfg0": (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 3),
}


def run_case(name, args):
    Nx, Ny, Nz = args[:3]
    n = args[-1]
    ch = O.RefChannel(*args)
    C0 = O.synthetic_state(Nx, Ny, Nz, seed=0, amp=1e-2)
    C = C0.copy()
    ch.primal(0, C)
    traj = np.stack([ch.mc_sub(k) for k in range(3 * n + 1)])
    IC0 = O.synthetic_state(Nx, Ny, Nz, seed=1, laminar=False)
    IC_inh = IC0.copy()
    ch.tangent(0, n, IC_inh, 1)
    IC_hom0 = O.synthetic_state(Nx, Ny, Nz, seed=2, laminar=False)
    IC_hom = IC_hom0.copy()
    ch.tangent(0, n, IC_hom, 0)
    mic = np.stack([ch.mic_sub(k) for k in range(3 * n + 1)])
    AC0 = O.synthetic_state(Nx, Ny, Nz, seed=3, laminar=False)
    AC = AC0.copy()
    ch.adjoint(n, 0, AC, 0, 0.5)
    AC0b = O.synthetic_state(Nx, Ny, Nz, seed=5, laminar=False)
    ACb = AC0b.copy()
    ch.adjoint(n, 1, ACb, 0, 0.0)
    V0 = O.synthetic_state(Nx, Ny, Nz, seed=4, laminar=False)
    V = V0.copy()
    proj = ch.ddt_project(1, V)
    flow = ch.spec2phys(C)
    y, w = ch.quad()
    O.libc_srand(1)
    ch2 = O.RefChannel(*args)
    ch2.primal(0, None)
    lam = np.stack([ch2.getsoln(i) for i in range(n + 1)])
    ch2.close()
    out = dict(args=np.array(args, dtype=np.float64), C0=C0, C=C, traj=traj, IC0=IC0, IC_inh=IC_inh,
               IC_hom0=IC_hom0, IC_hom=IC_hom, mic=mic, AC0=AC0, AC=AC, AC0b=AC0b, ACb=ACb,
               V0=V0, V=V, proj=np.array(proj), y=y, w=w, laminar_srand1=lam)
    if name == "tiny":
        out["flow"] = flow
    else:
        # keep the committed file small: substages of the first step, the end states
        sel = np.array([0, 1, 2, 3, 3 * n])
        out["traj_idx"] = sel
        out["traj"] = traj[sel]
        out["mic_idx"] = np.array([0, 3 * n])
        out["mic"] = mic[[0, 3 * n]]
        out["laminar_srand1"] = lam[[0, n]]
    np.savez_compressed(HERE / f"golden_{name}.npz", **out)
    print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    for name, args in CASES.items():
        run_case(name, args)
