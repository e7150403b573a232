"""TEST INFRASTRUCTURE ONLY -- CPU restatement of the reference's LSS driver
layer, run on the oracle's single-trajectory entry points.

* ``Wrapper`` restates drivers/wrapper.py:5-54 (the KKT matvec over time
  segments ``nb[i]..nb[i+1]`` of one stored primal trajectory), in Python 3.
* ``par_minres`` restates drivers/pariter.py:63-125 (unpreconditioned
  MINRES with a caller-supplied inner product).

Both are checkers for the device LSS operator (channel/lss.py); the product
never imports this module.
"""
from __future__ import annotations

import math

import numpy as np


class Wrapper:
    """drivers/wrapper.py:5-54 on an oracle channel object ``ch`` (PortChannel
    or RefChannel) whose primal covers steps 0..nb[-1]."""

    def __init__(self, ch, nb):
        self.ch = ch
        self.nb = list(nb)
        self.n = len(self.nb) - 1
        self.shape = ch.coef_shape
        self.m = int(np.prod(self.shape))
        self.zeta = np.zeros(self.n)

    def forward(self, i, v0, inhomo):
        # wrapper.py:14-21
        v1 = v0.copy()
        self.ch.ddt_project(self.nb[i], v1)
        self.ch.tangent(self.nb[i], self.nb[i + 1], v1, inhomo)
        eta = self.ch.ddt_project(self.nb[i + 1], v1)
        return v1, eta

    def backward(self, i, w0, strength):
        # wrapper.py:23-30
        w1 = w0.copy()
        self.ch.ddt_project(self.nb[i + 1], w1)
        self.ch.adjoint(self.nb[i + 1], self.nb[i], w1, 0, strength)
        self.ch.ddt_project(self.nb[i], w1)
        return w1

    def matvec(self, x, inhomo=0):
        # wrapper.py:33-54: per segment forward then backward, so each
        # adjoint couples to the tangent trajectory of its own segment
        n_v = self.m * self.n
        n_w = self.m * (self.n - 1)
        assert x.shape == (2 * n_v + 2 * n_w,)
        z = x[::2] + 1j * x[1::2]
        v = z[:n_v].reshape((-1,) + self.shape)
        w = np.concatenate([z[n_v:].reshape((-1,) + self.shape), np.zeros((1,) + self.shape, complex)])
        R_w = np.zeros((self.n - 1,) + self.shape, complex)
        R_v = np.zeros((self.n,) + self.shape, complex)
        self.zeta = np.zeros(self.n)
        for i in range(self.n):
            vip, eta = self.forward(i, np.ascontiguousarray(v[i]), inhomo)
            self.zeta[i] = -eta
            wim = self.backward(i, np.ascontiguousarray(w[i]), 1.0)
            if i < self.n - 1:
                R_w[i] = v[i + 1] - vip
            if i > 0:
                R_v[i] = w[i - 1] - wim
            else:
                R_v[i] = -wim
        return np.hstack([R_v.ravel(), R_w.ravel()]).view(np.float64)


def par_minres(matvec, b, x, dot, tol=1e-5, maxiter=None):
    """drivers/pariter.py:63-125; x is updated in place and returned with
    (info, iterations), info 0 when |eta|/r0 < tol."""
    if maxiter is None:
        maxiter = len(b) * 10
    vi = b - matvec(x)
    vim = np.zeros_like(vi)
    betai = math.sqrt(dot(vi, vi))
    r0 = betai
    eta = betai
    gammai = gammaim = 1.0
    sigmai = sigmaim = 0.0
    wi = np.zeros_like(vi)
    wim = np.zeros_like(vi)
    for k in range(maxiter):
        vi = vi / betai
        Avi = matvec(vi)
        alphai = dot(vi, Avi)
        vip = Avi - alphai * vi - betai * vim
        betaip = math.sqrt(dot(vip, vip))
        delta = gammai * alphai - gammaim * sigmai * betai
        p1 = math.sqrt(delta * delta + betaip * betaip)
        p2 = sigmai * alphai + gammaim * gammai * betai
        p3 = sigmaim * betai
        gammaip = delta / p1
        sigmaip = betaip / p1
        wip = (vi - p3 * wim - p2 * wi) / p1
        x += gammaip * eta * wip
        eta *= -sigmaip
        betai = betaip
        sigmaim, sigmai = sigmai, sigmaip
        gammaim, gammai = gammai, gammaip
        wim, wi = wi, wip
        vim, vi = vi, vip
        if abs(eta) / r0 < tol:
            return x, (0, k + 1)
    return x, (1, maxiter)
