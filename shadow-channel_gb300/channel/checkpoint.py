"""Long-horizon forward + adjoint with checkpointing (the reference keeps the
whole primal trajectory MC in memory, channel/channel.c:429-431, which at
128x129x128 is 33 MB per substage: 5000 steps would need 500 GB).

``forward_adjoint`` runs the primal over ``nsteps`` steps keeping only a
checkpoint (one coefficient array, host memory) every ``spacing`` steps, then
the adjoint backwards one interval at a time: the interval's primal is
recomputed from its checkpoint on the GPU (bit-identical to the forward
pass) and the adjoint state is carried across interval boundaries.  The
result equals ``c_adjoint(nsteps, 0, ...)`` on a fully stored trajectory bit
for bit (strength 0: no tangent coupling).

``spacing=None`` picks the largest interval whose trajectory and working set
fit in the given fraction of the free HBM.  The returned report gives the
times of the forward pass, the recomputation and the adjoint, and the
recomputation overhead (recompute / forward).
"""
import time

import numpy as np

from . import c_channel


def _init(grid, steps):
    rc = c_channel.c_init(int(grid["Nx"]), int(grid["Ny"]), int(grid["Nz"]), float(grid["Lx"]),
                          float(grid["Lz"]), float(grid["Re"]), float(grid["flux"]), float(grid["dt"]), int(steps))
    if rc != 0:
        raise RuntimeError("c_init failed: " + c_channel.c_last_error_message())


def bytes_per_step(grid):
    """HBM of one stored step of the single-trajectory working set: three
    substage states of MC and MIC and three substages of the primal field
    cache (six physical fields on the padded grid)."""
    Nx, Ny, Nz = int(grid["Nx"]), int(grid["Ny"]), int(grid["Nz"])
    coef = Nz * 2 * (Ny - 2) * (Nx // 2) * 16
    q = 3 * Ny // 2
    phys = 6 * q * (3 * Nz // 2) * (3 * Nx // 2) * 8
    return 3 * (2 * coef + phys)


def choose_spacing(grid, nsteps, fraction=0.5):
    """Largest checkpoint interval whose per-step storage fits in ``fraction``
    of the free device memory (at least 1, at most nsteps)."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    k = int(fraction * free // bytes_per_step(grid))
    return max(1, min(int(nsteps), k))


def forward_adjoint(grid, C0, nsteps, AC_final, spacing=None, fraction=0.5):
    """Primal from C0 over nsteps, then the adjoint from AC_final at step
    nsteps back to step 0.  Returns (C_final, AC_0, report)."""
    nsteps = int(nsteps)
    if spacing is None:
        spacing = choose_spacing(grid, nsteps, fraction)
    spacing = max(1, min(int(spacing), nsteps))
    chunks, n = [], 0
    while n < nsteps:
        k = min(spacing, nsteps - n)
        chunks.append(k)
        n += k
    current = [None]

    def ensure(k):  # the engine holds k stored steps; re-initialised only when k changes
        if current[0] != k:
            _init(grid, k)
            current[0] = k

    t0 = time.perf_counter()
    C = np.ascontiguousarray(C0, dtype=np.complex128).copy()
    ckpts = []
    for k in chunks:
        ckpts.append(C.copy())
        ensure(k)
        c_channel.c_primal(0, C)
        if c_channel.c_last_error() & 1:
            raise FloatingPointError("CFL limit exceeded in the primal")
    t_fwd = time.perf_counter() - t0
    AC = np.ascontiguousarray(AC_final, dtype=np.complex128).copy()
    t_re = t_adj = 0.0
    for Cc, k in zip(reversed(ckpts), reversed(chunks)):
        t1 = time.perf_counter()
        ensure(k)
        c_channel.c_primal(0, Cc.copy())
        c_channel.c_synchronize()
        t2 = time.perf_counter()
        c_channel.c_adjoint(k, 0, AC, 0, 0.0)
        t3 = time.perf_counter()
        t_re += t2 - t1
        t_adj += t3 - t2
    report = {"nsteps": nsteps, "spacing": spacing, "checkpoints": len(ckpts),
              "checkpoint_bytes_host": int(len(ckpts) * C.nbytes),
              "trajectory_bytes_device_per_interval": int(spacing * bytes_per_step(grid)),
              "forward_s": t_fwd, "recompute_s": t_re, "adjoint_s": t_adj,
              "recompute_overhead": t_re / t_fwd if t_fwd > 0 else None}
    return C, AC, report
