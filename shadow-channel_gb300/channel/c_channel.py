"""ctypes binding of libc_channel.so with the call signatures of the SWIG
module ``c_channel`` (channel/channel.i), so code written against the
reference's extension keeps working:

    c_init(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, nsteps) -> int
    c_primal(ru_steps, C)                  C: complex128 [Nz, 2, Ny-2, Nx/2], in place
    c_tangent(start, end, IC, inhomo)
    c_adjoint(start, end, AC, inhomo, strength)
    c_adjoint_exact(start, end, AC)        transpose of the homogeneous tangent (no SWIG counterpart)
    c_ddt_project(i_step, IC) -> float
    c_getsoln(i_step) / c_getincresoln(i_step) -> ndarray (library-owned buffer)
    c_spec2phys(C, flow)                   flow: float64 [3, 3Nx/2, qpts, 3Nz/2]
    c_read_solution(filename, C) / c_save_solution(filename, C)
    c_quad() -> (y, w)
    c_qpts(), c_dimR(), c_dimQ(), c_Nx(), c_Nz(), c_nsteps()

SWIG's INPLACE_ARRAY4 typemaps reject arrays that are not C-contiguous
complex128; so does this module (TypeError).  The library has no CPU code
path: if the shared library is missing this module raises ImportError.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent.parent
_LIBPATH = Path(os.environ.get("CHN_LIBRARY", _PKG / "libc_channel.so"))

if not _LIBPATH.exists():
    raise ImportError(f"libc_channel.so not found at {_LIBPATH}; build it with "
                      f"`python shadow-channel_gb300/build.py` (needs nvcc, sm_103a)")

_lib = ctypes.CDLL(str(_LIBPATH))

_i, _d, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
_pp = ctypes.POINTER(ctypes.c_void_p)
_ip = ctypes.POINTER(ctypes.c_int)

_lib.c_init.argtypes = [_i, _i, _i, _d, _d, _d, _d, _d, _i]
_lib.c_init.restype = _i
_lib.c_destroy.argtypes = []
_lib.c_destroy.restype = None
_lib.c_primal.argtypes = [_i, _vp, _i, _i, _i, _i]
_lib.c_primal.restype = None
_lib.c_tangent.argtypes = [_i, _i, _vp, _i, _i, _i, _i, _i]
_lib.c_tangent.restype = None
_lib.c_adjoint.argtypes = [_i, _i, _vp, _i, _i, _i, _i, _i, _d]
_lib.c_adjoint.restype = None
_lib.c_adjoint_exact.argtypes = [_i, _i, _vp, _i, _i, _i, _i]
_lib.c_adjoint_exact.restype = None
_lib.c_adjoint_exact_source.argtypes = [_i, _i, _vp, _vp, _i, _i, _i, _i]
_lib.c_adjoint_exact_source.restype = None
_lib.c_adjoint_exact_grad.argtypes = [_i, _i, _vp, _vp, _vp]
_lib.c_adjoint_exact_grad.restype = _i
_lib.c_ddt_project.argtypes = [_i, _vp, _i, _i, _i, _i]
_lib.c_ddt_project.restype = _d
_lib.c_getsoln.argtypes = [_i, _pp, _ip, _ip, _ip, _ip]
_lib.c_getsoln.restype = None
_lib.c_getincresoln.argtypes = [_i, _pp, _ip, _ip, _ip, _ip]
_lib.c_getincresoln.restype = None
_lib.c_spec2phys.argtypes = [_vp, _i, _i, _i, _i, _vp, _i, _i, _i, _i]
_lib.c_spec2phys.restype = None
_lib.c_read_solution.argtypes = [ctypes.c_char_p, _vp, _i, _i, _i, _i]
_lib.c_read_solution.restype = None
_lib.c_save_solution.argtypes = [ctypes.c_char_p, _vp, _i, _i, _i, _i]
_lib.c_save_solution.restype = None
_lib.c_quad.argtypes = [ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), _ip,
                        ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), _ip]
_lib.c_quad.restype = None
for _n in ("c_qpts", "c_dimR", "c_dimQ", "c_Nx", "c_Nz", "c_nsteps", "c_last_error",
           "c_batch_destroy", "c_synchronize"):
    getattr(_lib, _n).argtypes = []
    getattr(_lib, _n).restype = _i
_lib.c_last_error_message.argtypes = []
_lib.c_last_error_message.restype = ctypes.c_char_p
_lib.c_last_cfl.argtypes = []
_lib.c_last_cfl.restype = _d
_lib.c_launch_count.argtypes = []
_lib.c_launch_count.restype = ctypes.c_longlong
_lib.c_fp64_peak_tflops.argtypes = []
_lib.c_fp64_peak_tflops.restype = _d
_lib.c_pipe_peak_tflops.argtypes = [_i]
_lib.c_pipe_peak_tflops.restype = _d
_lib.c_autotune_report.argtypes = []
_lib.c_autotune_report.restype = ctypes.c_char_p
_lib.c_batch_init.argtypes = [_i, _i, _i]
_lib.c_batch_init.restype = _i
_lib.c_batch_primal.argtypes = [_i, _vp]
_lib.c_batch_primal.restype = _i
_lib.c_batch_tangent.argtypes = [_i, _i, _vp, _vp]
_lib.c_batch_tangent.restype = _i
_lib.c_batch_forward.argtypes = [_i, _i, _vp, _vp, _vp]
_lib.c_batch_forward.restype = _i
_lib.c_batch_adjoint.argtypes = [_i, _i, _vp, _d]
_lib.c_batch_adjoint.restype = _i
_lib.c_batch_adjoint_exact.argtypes = [_i, _i, _vp]
_lib.c_batch_adjoint_exact.restype = _i
_lib.c_batch_getsoln.argtypes = [_i, _i, _vp]
_lib.c_batch_getsoln.restype = _i
_lib.c_batch_getincresoln.argtypes = [_i, _i, _vp]
_lib.c_batch_getincresoln.restype = _i
for _n in ("c_batch_primal_dev",):
    getattr(_lib, _n).argtypes = [_i, _vp]
    getattr(_lib, _n).restype = _i
_lib.c_batch_tangent_dev.argtypes = [_i, _i, _vp, _vp]
_lib.c_batch_tangent_dev.restype = _i
_lib.c_batch_forward_dev.argtypes = [_i, _i, _vp, _vp, _vp]
_lib.c_batch_forward_dev.restype = _i
_lib.c_batch_adjoint_dev.argtypes = [_i, _i, _vp, _d]
_lib.c_batch_adjoint_dev.restype = _i
_lib.c_batch_adjoint_exact_dev.argtypes = [_i, _i, _vp]
_lib.c_batch_adjoint_exact_dev.restype = _i
_lib.c_batch_adjoint_exact_source_dev.argtypes = [_i, _i, _vp, _vp]
_lib.c_batch_adjoint_exact_source_dev.restype = _i
_lib.c_batch_adjoint_exact_grad_dev.argtypes = [_i, _i, _vp, _vp, _vp]
_lib.c_batch_adjoint_exact_grad_dev.restype = _i

_lib.c_stream.argtypes = []
_lib.c_stream.restype = _vp
_lib.c_batch_kernel_ms.argtypes = [_i, _i]
_lib.c_batch_kernel_ms.restype = _d

_lib.c_spec2phys_noalloc.argtypes = [_vp, _vp]
_lib.c_spec2phys_noalloc.restype = _i

_ipc = ctypes.POINTER(ctypes.c_int)
_dpc = ctypes.POINTER(ctypes.c_double)
_lib.c_multi_init.argtypes = [_i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i]
_lib.c_multi_init.restype = _i
_lib.c_multi_destroy.argtypes = []
_lib.c_multi_destroy.restype = _i
_lib.c_multi_coef_elems.argtypes = [_i]
_lib.c_multi_coef_elems.restype = ctypes.c_longlong
_lib.c_multi_primal.argtypes = [_i, _vp]
_lib.c_multi_primal.restype = _i
_lib.c_multi_forward.argtypes = [_i, _i, _vp, _vp, _vp]
_lib.c_multi_forward.restype = _i
_lib.c_multi_adjoint.argtypes = [_i, _i, _vp, _d]
_lib.c_multi_adjoint.restype = _i
_lib.c_multi_adjoint_exact.argtypes = [_i, _i, _vp]
_lib.c_multi_adjoint_exact.restype = _i
_lib.c_multi_getsoln.argtypes = [_i, _i, _vp]
_lib.c_multi_getsoln.restype = _i
_lib.c_tangent_forcing.argtypes = [_i, _i, _vp, _i, _i, _i, _i, _i]
_lib.c_tangent_forcing.restype = None
_lib.c_mean_profile.argtypes = [_i, _i, _i, _i, _vp]
_lib.c_mean_profile.restype = _i
_lib.c_wall_shear_weights.argtypes = [_vp]
_lib.c_wall_shear_weights.restype = _i
_lib.c_wall_shear.argtypes = [_i, _i, _i, _vp]
_lib.c_wall_shear.restype = _i
_lib.c_mean_product.argtypes = [_i, _i, _i, _i, _i, _i, _vp]
_lib.c_mean_product.restype = _i
_lib.c_batch_mean_profile.argtypes = [_i, _i, _i, _i, _vp]
_lib.c_batch_mean_profile.restype = _i
for _n in ("c_batch_mean_profile_dev",):
    getattr(_lib, _n).argtypes = [_i, _i, _i, _i, _vp]
    getattr(_lib, _n).restype = _i
_lib.c_batch_wall_shear_dev.argtypes = [_i, _i, _i, _vp]
_lib.c_batch_wall_shear_dev.restype = _i
_lib.c_batch_mean_product_dev.argtypes = [_i, _i, _i, _i, _i, _i, _vp]
_lib.c_batch_mean_product_dev.restype = _i

_lib.c_batch_init_steps.argtypes = [_i, _i, _i, _i]
_lib.c_batch_init_steps.restype = _i
_lib.c_batch_set_chain.argtypes = [_i]
_lib.c_batch_set_chain.restype = _i
_lib.c_batch_ddt_project.argtypes = [_i, _vp, _vp]
_lib.c_batch_ddt_project.restype = _i
_lib.c_batch_ddt_project_dev.argtypes = [_i, _vp, _vp]
_lib.c_batch_ddt_project_dev.restype = _i
_lib.c_lss_matvec_dev.argtypes = [_vp, _vp, _i, _vp]
_lib.c_lss_matvec_dev.restype = _i
_lib.c_lss_dot_dev.argtypes = [ctypes.c_longlong, _vp, _vp, _vp]
_lib.c_lss_dot_dev.restype = _i
_lib.c_lss_minres_dev.argtypes = [_vp, _vp, _d, _i, _ip, ctypes.POINTER(_d)]
_lib.c_lss_minres_dev.restype = _i

LIBRARY_PATH = str(_LIBPATH)
lib = _lib


def _inplace4(a, dtype, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or a.ndim != 4 or not a.flags["C_CONTIGUOUS"] \
            or not a.flags["WRITEABLE"]:
        raise TypeError(f"{name}: expected a writeable C-contiguous {np.dtype(dtype).name} array of rank 4")
    return a.ctypes.data, a.shape


def c_init(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, nstep):
    return _lib.c_init(int(Nx), int(Ny), int(Nz), float(Lx), float(Lz), float(Re), float(flux),
                       float(dt), int(nstep))


def c_destroy():
    _lib.c_destroy()


def c_primal(ru_steps, C_given):
    p, s = _inplace4(C_given, np.complex128, "c_primal")
    _lib.c_primal(int(ru_steps), p if C_given.size else None, *s)


def c_tangent(start_step, end_step, IC_given, inhomo):
    p, s = _inplace4(IC_given, np.complex128, "c_tangent")
    _lib.c_tangent(int(start_step), int(end_step), p, *s, int(inhomo))


def c_tangent_forcing(start_step, end_step, IC_given, forcing):
    """c_tangent with forcing 0 none, 1 mean flux, 2 Re (the reference's
    forcing reconnected), 3 Re (exact derivative of the discrete step)."""
    ptr, shp = _inplace4(IC_given, np.complex128, "IC_given")
    _lib.c_tangent_forcing(int(start_step), int(end_step), ptr, *shp, int(forcing))


def c_adjoint(start_step, end_step, AC_given, inhomo, strength):
    p, s = _inplace4(AC_given, np.complex128, "c_adjoint")
    _lib.c_adjoint(int(start_step), int(end_step), p, *s, int(inhomo), float(strength))


def c_adjoint_exact(start_step, end_step, AC_given):
    """The transpose of the homogeneous tangent from end_step to start_step
    (start_step > end_step), applied to AC_given in place: <AC, T v> equals
    <T^T AC, v> for every v, with T v = c_tangent(end_step, start_step, v, 0)."""
    p, s = _inplace4(AC_given, np.complex128, "c_adjoint_exact")
    _lib.c_adjoint_exact(int(start_step), int(end_step), p, *s)


def c_adjoint_exact_source(start_step, end_step, AC_given, src):
    """c_adjoint_exact with src added after every step (lambda_n = T_n^T
    lambda_{n+1} + src): the gradient of a per-step sum of <src, C_n>."""
    p, s = _inplace4(AC_given, np.complex128, "c_adjoint_exact_source")
    q, t = _inplace4(src, np.complex128, "src")
    if t != s:
        raise ValueError("src must have the shape of AC_given")
    _lib.c_adjoint_exact_source(int(start_step), int(end_step), p, q, *s)


def c_adjoint_exact_grad(start_step, end_step, AC_given, src=None):
    """c_adjoint_exact_source (src None: no source) returning
    (dJ/dmeanU, dJ/dRe) of J = <AC, C_start> + sum_n <src, C_n> from the same
    reverse sweep (the cotangents of the mean-flux and exact Re forcings)."""
    p, s = _inplace4(AC_given, np.complex128, "c_adjoint_exact_grad")
    q = None
    if src is not None:
        q, t = _inplace4(src, np.complex128, "src")
        if t != s:
            raise ValueError("src must have the shape of AC_given")
    grad = np.zeros(2)
    rc = _lib.c_adjoint_exact_grad(int(start_step), int(end_step), p, q, grad.ctypes.data)
    if rc < 0:
        raise RuntimeError("c_adjoint_exact_grad: " + c_last_error_message())
    return float(grad[0]), float(grad[1])


def c_ddt_project(i_step, IC_given):
    p, s = _inplace4(IC_given, np.complex128, "c_ddt_project")
    return _lib.c_ddt_project(int(i_step), p, *s)


def _traj(fn, i_step):
    ptr = ctypes.c_void_p()
    d = [ctypes.c_int() for _ in range(4)]
    fn(int(i_step), ctypes.byref(ptr), *[ctypes.byref(v) for v in d])
    shape = tuple(v.value for v in d)
    n = int(np.prod(shape))
    buf = (ctypes.c_double * (2 * n)).from_address(ptr.value)
    return np.frombuffer(buf, dtype=np.complex128).reshape(shape)


def c_getsoln(i_step):
    return _traj(_lib.c_getsoln, i_step)


def c_getincresoln(i_step):
    return _traj(_lib.c_getincresoln, i_step)


def c_spec2phys(C_ptr, flow_ptr):
    pc, sc = _inplace4(C_ptr, np.complex128, "c_spec2phys")
    pf, sf = _inplace4(flow_ptr, np.float64, "c_spec2phys")
    _lib.c_spec2phys(pc, *sc, pf, *sf)


def c_read_solution(filename, C_ptr):
    p, s = _inplace4(C_ptr, np.complex128, "c_read_solution")
    _lib.c_read_solution(str(filename).encode(), p, *s)


def c_save_solution(filename, C_ptr):
    p, s = _inplace4(C_ptr, np.complex128, "c_save_solution")
    _lib.c_save_solution(str(filename).encode(), p, *s)


def c_mean_profile(inc, comp, start_step, end_step):
    """x-z mean of velocity component comp (0 u, 1 v, 2 w) of MC (inc 0) or
    MIC (inc 1) at steps start..end-1: float64 [end-start, qpts]."""
    out = np.zeros((end_step - start_step, c_qpts()))
    _check(_lib.c_mean_profile(int(inc), int(comp), int(start_step), int(end_step), out.ctypes.data))
    return out


def c_wall_shear(inc, start_step, end_step):
    """dU/dy, dW/dy of the mean flow at y = -1 per step: float64 [end-start, 2]."""
    out = np.zeros((end_step - start_step, 2))
    _check(_lib.c_wall_shear(int(inc), int(start_step), int(end_step), out.ctypes.data))
    return out


def c_wall_shear_weights():
    """Rp0 = R'(-1), float64 [dimR]: dU/dy at y = -1 is Rp0 . Re(C[0, 0, :, 0])."""
    out = np.zeros(c_dimR())
    _check(_lib.c_wall_shear_weights(out.ctypes.data))
    return out


def c_mean_product(inc_a, comp_a, inc_b, comp_b, start_step, end_step):
    """x-z mean of the product of two velocity components per step: [end-start, qpts]."""
    out = np.zeros((end_step - start_step, c_qpts()))
    _check(_lib.c_mean_product(int(inc_a), int(comp_a), int(inc_b), int(comp_b), int(start_step),
                               int(end_step), out.ctypes.data))
    return out


def _check(rc):
    if rc != 0:
        raise RuntimeError(c_last_error_message())


def c_quad():
    y = ctypes.POINTER(ctypes.c_double)()
    w = ctypes.POINTER(ctypes.c_double)()
    n1, n2 = ctypes.c_int(), ctypes.c_int()
    _lib.c_quad(ctypes.byref(y), ctypes.byref(n1), ctypes.byref(w), ctypes.byref(n2))
    return (np.ctypeslib.as_array(y, shape=(n1.value,)), np.ctypeslib.as_array(w, shape=(n2.value,)))


def c_qpts():
    return _lib.c_qpts()


def c_dimR():
    return _lib.c_dimR()


def c_dimQ():
    return _lib.c_dimQ()


def c_Nx():
    return _lib.c_Nx()


def c_Nz():
    return _lib.c_Nz()


def c_nsteps():
    return _lib.c_nsteps()


# ---- additions ---------------------------------------------------------------

def c_last_error():
    return _lib.c_last_error()


def c_last_error_message():
    return _lib.c_last_error_message().decode()


def c_last_cfl():
    return _lib.c_last_cfl()


def c_launch_count():
    return _lib.c_launch_count()


def c_fp64_peak_tflops():
    return _lib.c_fp64_peak_tflops()


def c_synchronize():
    return _lib.c_synchronize()
