"""Least-squares shadowing (LSS) on the GPU.

The reference solves the LSS KKT system with ``Wrapper.matvec``
(drivers/wrapper.py:5-54) around the single-trajectory tangent / adjoint /
ddt_project calls and scipy's or its own MINRES (drivers/pariter.py:63-125),
one time segment after another.  ``KKT`` here keeps that interface but
advances every segment at once: the segments are the windows of one primal
trajectory, held as a chained batch on the device, and the matvec, the inner
products and the MINRES iteration run in libc_channel.so.

Vectors are float64 arrays of length 2*m*(2n-1) (m = Nx*(Ny-2)*Nz complex
coefficients per state, n segments), the reference's layout: the float view
of [v_0 .. v_{n-1}, w_0 .. w_{n-2}].  numpy arrays (host) and CUDA torch
tensors (device, no copies) are both accepted.
"""
import ctypes

import numpy as np

from . import c_channel

_lib = c_channel.lib


def _torch():
    import torch
    return torch


class KKT:
    """The LSS KKT operator of ``nseg`` windows of ``window_steps`` steps.

    starts: complex128 [nseg, Nz, 2, Ny-2, Nx/2], the primal state at each
    window start (window i starts where window i-1 ends); c_init must have
    run on the grid.  The windows' primal trajectories are recomputed on the
    device from these states.
    """

    def __init__(self, starts, window_steps):
        torch = _torch()
        starts = np.ascontiguousarray(starts, dtype=np.complex128)
        self.nseg, self.L = int(starts.shape[0]), int(window_steps)
        self.m = int(np.prod(starts.shape[1:]))
        self.state_shape = tuple(starts.shape[1:])
        assert self.nseg >= 1 and self.L >= 1
        rc = _lib.c_batch_init_steps(self.nseg, 1, 0, self.L)
        assert rc == 0, c_channel.c_last_error_message()
        assert _lib.c_batch_set_chain(self.L) == 0, c_channel.c_last_error_message()
        self.dev = torch.device("cuda")
        C = torch.from_numpy(starts.view(np.float64).copy()).to(self.dev)
        torch.cuda.synchronize()
        rc = _lib.c_batch_primal_dev(0, C.data_ptr())
        assert rc == 0, c_channel.c_last_error_message()
        self.size = 2 * self.m * (2 * self.nseg - 1)
        self.zeta = np.zeros(self.nseg)
        self._zeta_dev = torch.zeros(self.nseg, dtype=torch.float64, device=self.dev)

    # ---- vectors ----
    def _to_dev(self, x):
        torch = _torch()
        if isinstance(x, torch.Tensor):
            assert x.is_cuda and x.dtype == torch.float64 and x.is_contiguous()
            return x, False
        x = np.ascontiguousarray(x, dtype=np.float64)
        t = torch.from_numpy(x).to(self.dev)
        torch.cuda.synchronize()
        return t, True

    def _check(self, x):
        assert tuple(x.shape) == (self.size,), (tuple(x.shape), self.size)

    def dot(self, a, b):
        """Euclidean inner product of two vectors (device, deterministic)."""
        a, _ = self._to_dev(a)
        b, _ = self._to_dev(b)
        out = ctypes.c_double()
        assert _lib.c_lss_dot_dev(a.numel(), a.data_ptr(), b.data_ptr(), ctypes.byref(out)) == 0
        return out.value

    # ---- the reference's Wrapper interface ----
    def matvec(self, x, inhomo=0):
        """KKT x (drivers/wrapper.py:27-54); also sets self.zeta (the time
        dilation terms, minus the window-end projection coefficients)."""
        self._check(x)
        xd, host = self._to_dev(x)
        torch = _torch()
        y = torch.empty_like(xd)
        rc = _lib.c_lss_matvec_dev(xd.data_ptr(), y.data_ptr(), int(inhomo), self._zeta_dev.data_ptr())
        assert rc == 0, c_channel.c_last_error_message()
        assert _lib.c_synchronize() == 0
        self.zeta = self._zeta_dev.cpu().numpy().copy()
        return y.cpu().numpy() if host else y

    def rhs(self, host=True):
        """-matvec(0, 1) - matvec(0, 0), the right-hand side of drivers/wrapper.py:100
        (a numpy array, or a CUDA tensor with host=False)."""
        torch = _torch()
        z = torch.zeros(self.size, dtype=torch.float64, device=self.dev)
        b = -self.matvec(z, 1) - self.matvec(z, 0)
        return b.cpu().numpy() if host else b

    def minres(self, b, x0=None, tol=1e-5, maxiter=None):
        """MINRES on the device (drivers/pariter.py:63-125); returns
        (x, (info, iterations)), info 0 when converged."""
        self._check(b)
        bd, host = self._to_dev(b)
        torch = _torch()
        if x0 is None:
            x = torch.zeros_like(bd)
        else:
            x, _ = self._to_dev(x0)
            x = x.clone()
        maxiter = self.size * 10 if maxiter is None else int(maxiter)
        it = ctypes.c_int()
        res = ctypes.c_double()
        rc = _lib.c_lss_minres_dev(bd.data_ptr(), x.data_ptr(), float(tol), maxiter, ctypes.byref(it),
                                   ctypes.byref(res))
        assert rc in (0, 1), c_channel.c_last_error_message()
        self.rel_residual = res.value
        return (x.cpu().numpy() if host else x), (rc, it.value)

    def vw(self, x):
        """Split a vector into v [nseg, ...] and w [nseg-1, ...] complex arrays (host)."""
        torch = _torch()
        if isinstance(x, torch.Tensor):
            x = x.cpu().numpy()
        z = np.asarray(x).view(np.complex128)
        nv = self.nseg * self.m
        return (z[:nv].reshape((self.nseg,) + self.state_shape),
                z[nv:].reshape((self.nseg - 1,) + self.state_shape))

    def close(self):
        _lib.c_batch_destroy()
