"""Differentiable channel objectives for PyTorch.

``TimeMeanWallShear`` is a ``torch.autograd.Function`` whose forward runs the
primal (FP64, on the GPU through libc_channel.so) for ``nsteps`` steps and
returns the time-mean wall shear

    J = (1/N) sum_{n=0}^{N-1} dU/dy(y = -1) at step n

(the reference's Uxb of the mean flow, channel/project0.c:224-234), and
whose backward returns dJ/dRe and dJ/dmeanU.  The derivatives are exact
derivatives of the discrete RK3 scheme: tangent sweeps with the Re forcing
(c_tangent_forcing kind 3) and the mean-flux forcing (kind 1, the
reference's inhomogeneous tangent), whose wall shear is read from the
stored tangent trajectory.  For a scalar parameter the tangent sweep costs
what one adjoint sweep costs and carries no transposition error.

Memory: the primal is checkpointed every ``checkpoint`` steps (one
coefficient array per checkpoint, host memory); the backward recomputes the
trajectory one checkpoint interval at a time, so only ``checkpoint`` steps of
trajectory live in HBM however long the horizon.  ``ctx.report`` records the
forward and backward wall times (the recomputation overhead).
"""
import time

import numpy as np
import torch

from . import c_channel


def _init(grid, Re, meanU, steps):
    rc = c_channel.c_init(int(grid["Nx"]), int(grid["Ny"]), int(grid["Nz"]), float(grid["Lx"]),
                          float(grid["Lz"]), float(Re), float(2.0 * meanU), float(grid["dt"]), int(steps))
    if rc != 0:
        raise RuntimeError("c_init failed: " + c_channel.c_last_error_message())


def _chunks(nsteps, checkpoint):
    out, n = [], 0
    while n < nsteps:
        k = min(checkpoint, nsteps - n)
        out.append(k)
        n += k
    return out


def primal_objective(grid, Re, meanU, C0, nsteps, checkpoint):
    """J and the checkpoints [C at step 0, checkpoint, 2 checkpoint, ...]."""
    chunks = _chunks(nsteps, checkpoint)
    C = np.ascontiguousarray(C0, dtype=np.complex128).copy()
    ckpts, J = [], 0.0
    for k in chunks:
        ckpts.append(C.copy())
        _init(grid, Re, meanU, k)
        c_channel.c_primal(0, C)
        if c_channel.c_last_error() & 1:
            raise FloatingPointError("CFL limit exceeded in the primal")
        J += c_channel.c_wall_shear(0, 0, k)[:, 0].sum()
    return J / nsteps, ckpts, chunks


def tangent_gradients(grid, Re, meanU, ckpts, chunks, nsteps, kinds=(3, 1)):
    """dJ/dparameter for each tangent forcing kind (3: Re, 1: meanU),
    recomputing each checkpoint interval's primal from its checkpoint."""
    shape = ckpts[0].shape
    v = {k: np.zeros(shape, np.complex128) for k in kinds}
    dJ = {k: 0.0 for k in kinds}
    for C, k in zip(ckpts, chunks):
        _init(grid, Re, meanU, k)
        c_channel.c_primal(0, C.copy())
        for kind in kinds:
            c_channel.c_tangent_forcing(0, k, v[kind], kind)
            dJ[kind] += c_channel.c_wall_shear(1, 0, k)[:, 0].sum()
    return {kind: dJ[kind] / nsteps for kind in kinds}


class TimeMeanWallShear(torch.autograd.Function):
    """J(Re, meanU) = time-mean lower-wall shear of the primal from C0.

    Usage: ``J = TimeMeanWallShear.apply(Re, meanU, cfg)`` with Re, meanU
    0-d float64 tensors and cfg a dict: grid (Nx, Ny, Nz, Lx, Lz, dt), C0
    (complex [Nz, 2, Ny-2, Nx/2]), nsteps, checkpoint.
    """

    @staticmethod
    def forward(ctx, Re, meanU, cfg):
        t0 = time.perf_counter()
        J, ckpts, chunks = primal_objective(cfg["grid"], float(Re), float(meanU), cfg["C0"], int(cfg["nsteps"]),
                                            int(cfg["checkpoint"]))
        ctx.cfg = cfg
        ctx.params = (float(Re), float(meanU))
        ctx.ckpts, ctx.chunks = ckpts, chunks
        ctx.report = {"forward_s": time.perf_counter() - t0}
        cfg.setdefault("report", {}).update(ctx.report)
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        t0 = time.perf_counter()
        Re, meanU = ctx.params
        d = tangent_gradients(ctx.cfg["grid"], Re, meanU, ctx.ckpts, ctx.chunks, int(ctx.cfg["nsteps"]))
        ctx.cfg["report"]["backward_s"] = time.perf_counter() - t0
        g = float(gJ)
        return (torch.tensor(g * d[3], dtype=torch.float64), torch.tensor(g * d[1], dtype=torch.float64), None)


def time_mean_wall_shear(Re, meanU, cfg):
    """Functional form of TimeMeanWallShear.apply."""
    return TimeMeanWallShear.apply(Re, meanU, cfg)
