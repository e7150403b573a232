"""Seeded synthetic coefficient states (the reference ships no restart files).

``synthetic_state`` builds a laminar Poiseuille profile plus seeded random
low modes: complex normal noise of amplitude amp*exp(-n/3) on kx index
0..kmax, kz in {0..kmax, Nz-kmax..Nz-1} and Legendre index n < nmax of both
alpha (v) and beta (wall-normal vorticity); alpha rows >= Ny-4 zero away
from the mean mode; the kz = Nz/2 line zero; Hermitian symmetry on the
kx = 0 plane with a real mean line.  The Q and R bases make any such set
divergence-free and no-slip, so it is a valid initial state.
"""
import numpy as np


def laminar_mean(Ny, flux):
    """R-basis coefficients of u = (1 - y^2) * flux * 3/4: a_0 = 3 flux / 4."""
    out = np.zeros((2, Ny - 2))
    out[0, 0] = 0.75 * flux
    return out


def synthetic_state(Nx, Ny, Nz, seed=0, amp=1e-2, kmax=4, nmax=8, flux=2.0, laminar=True):
    R, D, X = Ny - 2, Ny - 4, Nx // 2
    rng = np.random.default_rng(seed)
    C = np.zeros((Nz, 2, R, X), np.complex128)
    nmax = min(nmax, R)
    scale = amp * np.exp(-np.arange(nmax) / 3.0)
    for z in list(range(0, kmax + 1)) + list(range(Nz - kmax, Nz)):
        for x in range(min(kmax + 1, X)):
            for v in range(2):
                C[z, v, :nmax, x] = scale * (rng.normal(size=nmax) + 1j * rng.normal(size=nmax))
    keep = C[0, 0, D:, 0].copy()
    C[:, 0, D:, :] = 0
    C[0, 0, D:, 0] = keep
    C[Nz // 2] = 0
    for z in range(1, Nz // 2):
        C[Nz - z, :, :, 0] = np.conj(C[z, :, :, 0])
    C[0, :, :, 0] = C[0, :, :, 0].real
    if laminar:
        C[0, :, :, 0] += laminar_mean(Ny, flux)
    return C
