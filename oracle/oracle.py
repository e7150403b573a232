"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the channel-flow time step.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker (or as the timed CPU baseline).  The
product library never loads it.

Two interchangeable backends with the reference's entry-point semantics
(channel/channel.i:17-229, channel/channel.c:207-780):

* ``PortChannel`` -- oracle/chan_port.c, a reentrant C restatement of the
  reference path.  Builds anywhere (``make -C oracle port``) and is what the
  GPU host uses.
* ``RefChannel``  -- the reference's own channel/*.c compiled in place against
  the FFTW-2 shim (``make -C oracle ref``).  Needs the reference tree, so it
  exists only where that tree exists; it pins the port (tests/test_oracle_pin.py).

Arrays: coefficients are complex128 [Nz, 2, Ny-2, Nx/2]; physical flow is
float64 [3, 3Nx/2, qpts, 3Nz/2].
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libchanport.so"
REF_LIB = HERE / "_ref" / "libref_channel.so"
# The reference's channel/ directory: $SHADOW_CHANNEL_REFERENCE (the root of
# a reference checkout), else a checkout named "reference" beside this
# repository; absent on hosts that only run the port.
REF_DIR = Path(os.environ["SHADOW_CHANNEL_REFERENCE"]) / "channel" if os.environ.get(
    "SHADOW_CHANNEL_REFERENCE") else HERE.parent.parent / "reference" / "channel"

_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p


def build_port() -> Path:
    """Compile the C restatement (fast; a few seconds)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def build_ref() -> Path | None:
    """Compile the reference sources in place, when the reference tree exists."""
    if not REF_DIR.is_dir():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_DIR={REF_DIR}"],
                   check=True, stdout=subprocess.DEVNULL)
    return REF_LIB


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _check_coef(C: np.ndarray, shape) -> None:
    if C.dtype != np.complex128 or C.shape != tuple(shape) or not C.flags["C_CONTIGUOUS"]:
        raise ValueError(f"coefficient array must be C-contiguous complex128 {tuple(shape)}, "
                         f"got {C.dtype} {C.shape}")


class _Base:
    Nx: int
    Ny: int
    Nz: int
    nsteps: int

    @property
    def coef_shape(self):
        return (self.Nz, 2, self.Ny - 2, self.Nx // 2)

    @property
    def flow_shape(self):
        return (3, 3 * self.Nx // 2, self.qpts, 3 * self.Nz // 2)

    @property
    def qpts(self):
        return 3 * self.Ny // 2

    def spec2phys(self, C: np.ndarray) -> np.ndarray:
        C = np.ascontiguousarray(C, dtype=np.complex128)
        flow = np.zeros(self.flow_shape, np.float64)
        self._spec2phys(C, flow)
        return flow


class PortChannel(_Base):
    """The C restatement; several instances may coexist (one per segment)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not PORT_LIB.exists():
                build_port()
            L = ctypes.CDLL(str(PORT_LIB))
            L.cport_init.restype = _vp
            L.cport_init.argtypes = [_c_int] * 3 + [_c_dbl] * 5 + [_c_int]
            L.cport_destroy.argtypes = [_vp]
            L.cport_primal.argtypes = [_vp, _c_int, _vp]
            L.cport_tangent.argtypes = [_vp, _c_int, _c_int, _vp, _c_int]
            L.cport_tangent_forcing.argtypes = [_vp, _c_int, _c_int, _vp, _c_int]
            L.cport_adjoint_exact.argtypes = [_vp, _c_int, _c_int, _vp]
            L.cport_adjoint.argtypes = [_vp, _c_int, _c_int, _vp, _c_int, _c_dbl]
            L.cport_ddt_project.argtypes = [_vp, _c_int, _vp]
            L.cport_ddt_project.restype = _c_dbl
            L.cport_spec2phys.argtypes = [_vp, _vp, _vp]
            for f in ("cport_mc", "cport_mic", "cport_mc_sub", "cport_mic_sub"):
                getattr(L, f).restype = _vp
                getattr(L, f).argtypes = [_vp, _c_int]
            L.cport_qy.restype = _vp
            L.cport_qy.argtypes = [_vp]
            L.cport_w.restype = _vp
            L.cport_w.argtypes = [_vp]
            L.cport_table.restype = _vp
            L.cport_table.argtypes = [_vp, _c_int]
            cls._lib = L
        return cls._lib

    def __init__(self, Nx, Ny, Nz, Lx, Lz, Re, flux, dt, nsteps):
        L = self.lib()
        self.Nx, self.Ny, self.Nz, self.nsteps = int(Nx), int(Ny), int(Nz), int(nsteps)
        self.Lx, self.Lz, self.Re, self.flux, self.dt = float(Lx), float(Lz), float(Re), float(flux), float(dt)
        self._h = L.cport_init(self.Nx, self.Ny, self.Nz, self.Lx, self.Lz, self.Re,
                               self.flux, self.dt, self.nsteps)
        if not self._h:
            raise ValueError("cport_init rejected the parameters")

    def close(self):
        if getattr(self, "_h", None):
            self.lib().cport_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def primal(self, ru_steps: int, C: np.ndarray | None) -> int:
        if C is None:
            return self.lib().cport_primal(self._h, int(ru_steps), None)
        _check_coef(C, self.coef_shape)
        return self.lib().cport_primal(self._h, int(ru_steps), _ptr(C))

    def tangent(self, start, end, IC, inhomo) -> int:
        _check_coef(IC, self.coef_shape)
        return self.lib().cport_tangent(self._h, int(start), int(end), _ptr(IC), int(inhomo))

    def tangent_forcing(self, start, end, IC, forcing) -> int:
        """forcing 0 none, 1 mean flux, 2 Re (the reference's forcing
        reconnected), 3 Re (exact derivative of the discrete step)."""
        _check_coef(IC, self.coef_shape)
        return self.lib().cport_tangent_forcing(self._h, int(start), int(end), _ptr(IC), int(forcing))

    def adjoint(self, start, end, AC, inhomo, strength) -> int:
        _check_coef(AC, self.coef_shape)
        return self.lib().cport_adjoint(self._h, int(start), int(end), _ptr(AC), int(inhomo), float(strength))

    def adjoint_exact(self, start, end, AC) -> int:
        """The transpose of the homogeneous tangent from end to start
        (start > end) applied to AC in place."""
        _check_coef(AC, self.coef_shape)
        return self.lib().cport_adjoint_exact(self._h, int(start), int(end), _ptr(AC))

    def ddt_project(self, i_step, IC) -> float:
        _check_coef(IC, self.coef_shape)
        return self.lib().cport_ddt_project(self._h, int(i_step), _ptr(IC))

    def _spec2phys(self, C, flow):
        self.lib().cport_spec2phys(self._h, _ptr(C), _ptr(flow))

    def _view(self, fn, i) -> np.ndarray:
        p = fn(self._h, int(i))
        n = int(np.prod(self.coef_shape))
        buf = (ctypes.c_double * (2 * n)).from_address(p)
        return np.frombuffer(buf, dtype=np.complex128).reshape(self.coef_shape)

    def getsoln(self, i_step) -> np.ndarray:
        return self._view(self.lib().cport_mc, i_step).copy()

    def getincresoln(self, i_step) -> np.ndarray:
        return self._view(self.lib().cport_mic, i_step).copy()

    def mc_sub(self, count) -> np.ndarray:
        return self._view(self.lib().cport_mc_sub, count).copy()

    def mic_sub(self, count) -> np.ndarray:
        return self._view(self.lib().cport_mic_sub, count).copy()

    def quad(self):
        q = self.qpts
        y = np.frombuffer((ctypes.c_double * q).from_address(self.lib().cport_qy(self._h)), np.float64).copy()
        w = np.frombuffer((ctypes.c_double * q).from_address(self.lib().cport_w(self._h)), np.float64).copy()
        return y, w

    def table(self, which: int) -> np.ndarray:
        q, R, D = self.qpts, self.Ny - 2, self.Ny - 4
        shapes = [(q, D), (q, D), (q, D), (q, R), (q, R), (D, q), (D, q), (D, q), (R, q), (R, q),
                  (D, 9), (D, 9), (D, 9), (R, 5), (R, 5)]
        shp = shapes[which]
        p = self.lib().cport_table(self._h, int(which))
        return np.frombuffer((ctypes.c_double * int(np.prod(shp))).from_address(p), np.float64).reshape(shp).copy()


class RefChannel(_Base):
    """The reference's own C, compiled here.  Process-global state: one live
    instance at a time, exactly as in the reference."""

    _lib = None
    _live = None

    @classmethod
    def available(cls) -> bool:
        return REF_LIB.exists() or REF_DIR.is_dir()

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not REF_LIB.exists():
                if build_ref() is None:
                    raise RuntimeError("reference tree not present; RefChannel unavailable")
            L = ctypes.CDLL(str(REF_LIB))
            L.init.argtypes = [_c_int] * 3 + [_c_dbl] * 5 + [_c_int]
            L.init.restype = _c_int
            L.destroy.argtypes = [_c_int]
            L.primal.argtypes = [_c_int, _vp]
            L.tangent.argtypes = [_c_int, _c_int, _vp, _c_int]
            L.adjoint.argtypes = [_c_int, _c_int, _vp, _c_int, _c_dbl]
            L.ddt_project.argtypes = [_c_int, _vp]
            L.ddt_project.restype = _c_dbl
            L.spec2phys.argtypes = [_vp, _vp]
            cls._lib = L
        return cls._lib

    def __init__(self, Nx, Ny, Nz, Lx, Lz, Re, flux, dt, nsteps):
        L = self.lib()
        if RefChannel._live is not None:
            RefChannel._live.close()
        self.Nx, self.Ny, self.Nz, self.nsteps = int(Nx), int(Ny), int(Nz), int(nsteps)
        self.dt = float(dt)
        rc = L.init(self.Nx, self.Ny, self.Nz, float(Lx), float(Lz), float(Re), float(flux), float(dt), self.nsteps)
        if rc != 0:
            raise ValueError("reference init() failed")
        RefChannel._live = self

    def close(self):
        if RefChannel._live is self:
            self.lib().destroy(0xffffffff)
            RefChannel._live = None

    def primal(self, ru_steps, C):
        if C is None:
            self.lib().primal(int(ru_steps), None)
        else:
            _check_coef(C, self.coef_shape)
            self.lib().primal(int(ru_steps), _ptr(C))
        return 0

    def tangent(self, start, end, IC, inhomo):
        _check_coef(IC, self.coef_shape)
        self.lib().tangent(int(start), int(end), _ptr(IC), int(inhomo))
        return 0

    def adjoint(self, start, end, AC, inhomo, strength):
        _check_coef(AC, self.coef_shape)
        self.lib().adjoint(int(start), int(end), _ptr(AC), int(inhomo), float(strength))
        return 0

    def ddt_project(self, i_step, IC):
        _check_coef(IC, self.coef_shape)
        return self.lib().ddt_project(int(i_step), _ptr(IC))

    def _spec2phys(self, C, flow):
        self.lib().spec2phys(_ptr(C), _ptr(flow))

    def _traj(self, name, count) -> np.ndarray:
        p = ctypes.c_void_p.in_dll(self.lib(), name).value
        for _ in range(4):  # mcomplex***** -> contiguous base
            p = ctypes.cast(p, ctypes.POINTER(ctypes.c_void_p))[0]
        n = int(np.prod(self.coef_shape))
        base = p + int(count) * n * 16
        buf = (ctypes.c_double * (2 * n)).from_address(base)
        return np.frombuffer(buf, dtype=np.complex128).reshape(self.coef_shape).copy()

    def getsoln(self, i_step):
        return self._traj("MC", 3 * int(i_step))

    def getincresoln(self, i_step):
        return self._traj("MIC", 3 * int(i_step))

    def mc_sub(self, count):
        return self._traj("MC", count)

    def mic_sub(self, count):
        return self._traj("MIC", count)

    def quad(self):
        q = self.qpts
        L = self.lib()
        y = np.frombuffer((ctypes.c_double * q).from_address(ctypes.c_void_p.in_dll(L, "Qy").value), np.float64).copy()
        w = np.frombuffer((ctypes.c_double * q).from_address(ctypes.c_void_p.in_dll(L, "W").value), np.float64).copy()
        return y, w


def libc_srand(seed: int) -> None:
    """Seed the C library's rand(), which the laminar start (channel.c:417-420) draws from."""
    libc = ctypes.CDLL(None)
    libc.srand(ctypes.c_uint(seed))


# ----------------------------------------------------------------------------
# synthetic states (the reference ships no restart files)
# ----------------------------------------------------------------------------

def synthetic_state(Nx, Ny, Nz, seed=0, amp=1e-2, kmax=4, nmax=8, flux=2.0, Lx=2 * np.pi,
                    Lz=np.pi, laminar=True):
    """Laminar Poiseuille coefficients plus seeded random low modes.

    Complex normal noise of amplitude amp*exp(-n/3) on kx index 0..kmax,
    kz in {0..kmax, Nz-kmax..Nz-1}, Legendre index n < nmax of both alpha and
    beta; alpha rows >= Ny-4 zero off the mean mode; kz = Nz/2 zero; the kx = 0
    plane Hermitian and the (0,0) line real.  The Q and R bases make any such
    set divergence-free and no-slip.
    """
    R, D, X = Ny - 2, Ny - 4, Nx // 2
    rng = np.random.default_rng(seed)
    C = np.zeros((Nz, 2, R, X), np.complex128)
    zs = list(range(0, kmax + 1)) + list(range(Nz - kmax, Nz))
    nmax = min(nmax, R)
    n = np.arange(nmax)
    scale = amp * np.exp(-n / 3.0)
    for z in zs:
        for x in range(min(kmax + 1, X)):
            for v in range(2):
                C[z, v, :nmax, x] = scale * (rng.normal(size=nmax) + 1j * rng.normal(size=nmax))
    keep = C[0, 0, D:, 0].copy()      # the (0,0) line uses all dimR rows
    C[:, 0, D:, :] = 0                  # alpha rows >= Ny-4 unused elsewhere
    C[0, 0, D:, 0] = keep
    C[Nz // 2] = 0
    # Hermitian symmetry on kx = 0
    for z in range(1, Nz // 2):
        C[Nz - z, :, :, 0] = np.conj(C[z, :, :, 0])
    C[0, :, :, 0] = C[0, :, :, 0].real
    if laminar:
        C[0, :, :, 0] += laminar_mean(Ny, flux)
    return C


def laminar_mean(Ny, flux):
    """Legendre coefficients of the laminar profile u = (1 - y^2) * flux * 3/4
    in the R basis: R_0 = (1 - y^2) P_0, so a_0 = 3 flux / 4 and the rest 0."""
    R = Ny - 2
    out = np.zeros((2, R))
    out[0, 0] = 0.75 * flux
    return out
