"""Differentiable channel objectives for PyTorch.

``TimeMeanWallShear`` is a ``torch.autograd.Function`` whose forward runs the
primal (FP64, on the GPU through libc_channel.so) for ``nsteps`` steps and
returns the time-mean wall shear

    J = (1/N) sum_{n=0}^{N-1} dU/dy(y = -1) at step n

(the reference's Uxb of the mean flow, channel/project0.c:224-234), and
whose backward returns dJ/dRe, dJ/dmeanU and, when the initial state is
passed as a tensor, dJ/dC0.  The derivatives are exact derivatives of the
discrete RK3 scheme, all three from ONE reverse sweep of the exact discrete
adjoint (c_adjoint_exact_grad, the transpose of the tangent) with the
wall-shear weights as its per-step source:
    dJ/dC0 = (1/N) sum_n T(0 -> n)^T g,   g = Rp0 on Re C[0, 0, :, 0],
and dJ/dRe, dJ/dmeanU from the cotangents of the exact Re forcing
(c_tangent_forcing kind 3) and of the mean-flux forcing (kind 1, the
reference's inhomogeneous tangent) at every substage of the same sweep.
``tangent_gradients`` gives the two parameter derivatives by the forced
tangent sweeps instead (one sweep per parameter), as a cross-check.

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


def adjoint_gradients(grid, Re, meanU, ckpts, chunks, nsteps):
    """(dJ/dC0, dJ/dmeanU, dJ/dRe) from one exact-adjoint sweep, one
    checkpoint interval at a time from the last: each interval's primal is
    recomputed from its checkpoint, its transposed tangent carries lambda
    back with the source g / nsteps added at every step, and the interval's
    parameter gradients (the forcings' cotangents along it) add up."""
    shape = ckpts[0].shape
    lam = np.zeros(shape, np.complex128)
    src = None
    gU = gRe = 0.0
    for C, k in zip(reversed(ckpts), reversed(chunks)):
        _init(grid, Re, meanU, k)
        c_channel.c_primal(0, C.copy())
        if src is None:
            src = np.zeros(shape, np.complex128)
            src[0, 0, :, 0] = c_channel.c_wall_shear_weights() / nsteps
        u, r = c_channel.c_adjoint_exact_grad(k, 0, lam, src)
        if c_channel.c_last_error() != 0:
            raise RuntimeError("adjoint sweep failed: " + c_channel.c_last_error_message())
        gU += u
        gRe += r
    return lam, gU, gRe


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
    """J(Re, meanU, C0) = time-mean lower-wall shear of the primal from C0.

    Usage: ``J = TimeMeanWallShear.apply(Re, meanU, cfg[, C0])`` with Re,
    meanU 0-d float64 tensors and cfg a dict: grid (Nx, Ny, Nz, Lx, Lz, dt),
    C0 (complex [Nz, 2, Ny-2, Nx/2]), nsteps, checkpoint.  The optional
    tensor C0 (float64 [Nz, 2, Ny-2, Nx/2, 2], the real view of the complex
    state, e.g. ``torch.view_as_real``) replaces cfg["C0"] and receives
    dJ/dC0 when it requires grad.
    """

    @staticmethod
    def forward(ctx, Re, meanU, cfg, C0=None):
        t0 = time.perf_counter()
        c0 = cfg["C0"] if C0 is None else \
            np.ascontiguousarray(C0.detach().cpu().numpy()).view(np.complex128)[..., 0]
        J, ckpts, chunks = primal_objective(cfg["grid"], float(Re), float(meanU), c0, int(cfg["nsteps"]),
                                            int(cfg["checkpoint"]))
        ctx.cfg = cfg
        ctx.params = (float(Re), float(meanU))
        ctx.ckpts, ctx.chunks = ckpts, chunks
        ctx.c0_meta = None if C0 is None else (C0.shape, C0.dtype, C0.device)
        ctx.report = {"forward_s": time.perf_counter() - t0}
        cfg.setdefault("report", {}).update(ctx.report)
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        t0 = time.perf_counter()
        Re, meanU = ctx.params
        g = float(gJ)
        nsteps = int(ctx.cfg["nsteps"])
        gRe = gU = gC = None
        lam, dU, dRe = adjoint_gradients(ctx.cfg["grid"], Re, meanU, ctx.ckpts, ctx.chunks, nsteps)
        if ctx.needs_input_grad[0]:
            gRe = torch.tensor(g * dRe, dtype=torch.float64)
        if ctx.needs_input_grad[1]:
            gU = torch.tensor(g * dU, dtype=torch.float64)
        if ctx.c0_meta is not None and len(ctx.needs_input_grad) > 3 and ctx.needs_input_grad[3]:
            shape, dtype, device = ctx.c0_meta
            gC = torch.from_numpy(np.ascontiguousarray(lam).view(np.float64).reshape(shape) * g).to(
                device=device, dtype=dtype)
        ctx.cfg["report"]["backward_s"] = time.perf_counter() - t0
        return gRe, gU, None, gC


def time_mean_wall_shear(Re, meanU, cfg, C0=None):
    """Functional form of TimeMeanWallShear.apply."""
    if C0 is None:
        return TimeMeanWallShear.apply(Re, meanU, cfg)
    return TimeMeanWallShear.apply(Re, meanU, cfg, C0)
