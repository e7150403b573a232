"""Channel-flow DNS with tangent and adjoint solvers on a GB300.

Python 3 counterpart of the reference package ``channel`` (channel/__init__.py):
same module parameters, same functions, same array shapes.  The work happens
in libc_channel.so (FP64 CUDA kernels for sm_103a) through ``c_channel``.

Coefficient arrays are complex128 [Nz, 2, Ny-2, Nx/2]; physical fields are
float64 [3, 3Nx/2, qpts, 3Nz/2] with qpts = 3Ny/2.
"""
import numpy as np

from . import c_channel

# global lock (per process), channel/__init__.py:6
__is_initialized__ = False

# default parameters, channel/__init__.py:10-26
Nx = 16
Ny = 33
Nz = 16
Lx = 1.6
Lz = 1.6
dt = .01
meanU = 1.
Re = 5000


def _shape():
    return (c_channel.c_Nz(), 2, c_channel.c_dimR(), c_channel.c_Nx() // 2)


def quad():
    y, w = c_channel.c_quad()
    return y.copy(), w.copy()


def save_solution(filename, C, fmt="raw"):
    """Save the solution C (and the last tangent) to ``filename``.

    fmt "raw": the library's container (8 bytes "SCHNRAW1", int32 Nx, Ny,
    Nz, 0, float64 dt, 1/Re, mpg, then alpha, beta, ialpha, ibeta as
    [dimR][Nz][Nx/2] complex records); fmt "npz": a numpy archive with the
    reference's HDF5 dataset names and shapes (data_alpha, data_beta,
    data_ialpha, data_ibeta [dimR, Nz, Nx/2] complex128; data_Nx, data_Ny,
    data_Nz int32 [1]; data_dt, data_Re (= 1/Re), data_mpg float64 [1];
    channel/channel.c:889-1028).  HDF5 itself is not part of this build.
    Must be called after init()."""
    if not filename.endswith('.hd5'):
        filename += '.hd5'
    assert C.shape == _shape()
    if fmt == "raw":
        c_channel.c_save_solution(filename, C)
        return
    assert fmt == "npz", fmt
    import os
    import tempfile
    fd, tmp = tempfile.mkstemp(suffix=".raw")
    os.close(fd)
    try:
        c_channel.c_save_solution(tmp, C)
        d = _read_raw(tmp)
    finally:
        os.unlink(tmp)
    with open(filename, "wb") as f:
        np.savez(f, **d)


def _read_raw(path):
    with open(path, "rb") as f:
        head = f.read(8)
        assert head == b"SCHNRAW1", "not a SCHNRAW1 solution file"
        nx, ny, nz, _ = np.frombuffer(f.read(16), "<i4")
        dt_, re_, mpg = np.frombuffer(f.read(24), "<f8")
        shp = (int(ny) - 2, int(nz), int(nx) // 2)
        n = int(np.prod(shp))
        arrs = [np.frombuffer(f.read(16 * n), "<c16").reshape(shp).copy() for _ in range(4)]
    d = {k: v for k, v in zip(("data_alpha", "data_beta", "data_ialpha", "data_ibeta"), arrs)}
    d.update(data_Nx=np.array([nx], np.int32), data_Ny=np.array([ny], np.int32),
             data_Nz=np.array([nz], np.int32), data_dt=np.array([dt_]), data_Re=np.array([re_]),
             data_mpg=np.array([mpg]))
    return d


def _write_raw(path, d):
    with open(path, "wb") as f:
        f.write(b"SCHNRAW1")
        f.write(np.array([d["data_Nx"][0], d["data_Ny"][0], d["data_Nz"][0], 0], "<i4").tobytes())
        f.write(np.array([d["data_dt"][0], d["data_Re"][0], d["data_mpg"][0]], "<f8").tobytes())
        for k in ("data_alpha", "data_beta", "data_ialpha", "data_ibeta"):
            f.write(np.ascontiguousarray(d[k], "<c16").tobytes())


def read_solution(filename):
    """Read a solution written by save_solution (either format); returns
    complex [Nz, 2, dimR, Nx/2]."""
    if not filename.endswith('.hd5'):
        filename += '.hd5'
    C = np.zeros(_shape(), complex)
    with open(filename, "rb") as f:
        is_npz = f.read(2) == b"PK"
    if not is_npz:
        c_channel.c_read_solution(str(filename), C)
        return C
    import os
    import tempfile
    with np.load(filename) as z:
        d = {k: z[k] for k in z.files}
    fd, tmp = tempfile.mkstemp(suffix=".raw")
    os.close(fd)
    try:
        _write_raw(tmp, d)
        c_channel.c_read_solution(tmp, C)
    finally:
        os.unlink(tmp)
    return C


def get_solution(i_step, copy=True):
    """Primal solution at step i_step (not counting run-up steps)."""
    C = c_channel.c_getsoln(int(i_step))
    assert C.shape == _shape()
    if copy:
        C = C.copy()
    return C


def init(n_steps, ru_steps=0, restart=None):
    """Must be called before any other call of this module; runs the primal.
    restart: None (perturbed laminar start) or a solution file name."""
    global __is_initialized__
    assert not __is_initialized__
    __is_initialized__ = True
    assert n_steps >= 0 and ru_steps >= 0
    rc = c_channel.c_init(int(Nx), int(Ny), int(Nz), float(Lx), float(Lz), float(Re),
                          float(meanU * 2), float(dt), int(n_steps))
    if rc != 0:
        __is_initialized__ = False
        raise RuntimeError("c_init failed: " + c_channel.c_last_error_message())
    if restart is None:
        c_channel.c_primal(int(ru_steps), np.zeros([0, 0, 0, 0], complex))
    else:
        C = read_solution(restart)
        assert C.shape == _shape()
        c_channel.c_primal(int(ru_steps), C)


def para_init(n_steps, C):
    """Like init, but from the given coefficient array (parallel LSS)."""
    global __is_initialized__
    assert not __is_initialized__
    __is_initialized__ = True
    assert n_steps >= 0
    rc = c_channel.c_init(int(Nx), int(Ny), int(Nz), float(Lx), float(Lz), float(Re),
                          float(meanU * 2), float(dt), int(n_steps))
    if rc != 0:
        __is_initialized__ = False
        raise RuntimeError("c_init failed: " + c_channel.c_last_error_message())
    assert C.shape == _shape()
    c_channel.c_primal(0, C)


def destroy():
    global __is_initialized__
    assert __is_initialized__
    __is_initialized__ = False
    c_channel.c_destroy()


def primal(C_init):
    """Run the primal from C_init for nsteps; C_init holds the final state after."""
    assert C_init.shape == _shape()
    c_channel.c_primal(0, C_init)


def tangent(start_step, end_step, IC_init, inhomo):
    """Tangent from start_step to end_step; IC_init updated in place.
    inhomo != 0 adds the mean-flux (meanU) forcing (channel/increproject0.c:209-214)."""
    assert IC_init.shape == _shape()
    assert 0 <= start_step <= end_step <= c_channel.c_nsteps()
    c_channel.c_tangent(int(start_step), int(end_step), IC_init, int(inhomo))


def tangent_forcing(start_step, end_step, IC_init, forcing):
    """Tangent with a chosen forcing: 0 none, 1 mean flux (meanU), 2 Re with
    the reference's forcing reconnected (channel/tangent_forcing*.c; first
    order in dt), 3 Re, exact derivative of the discrete step."""
    assert IC_init.shape == _shape()
    assert 0 <= start_step <= end_step <= c_channel.c_nsteps()
    c_channel.c_tangent_forcing(int(start_step), int(end_step), IC_init, int(forcing))


def adjoint(start_step, end_step, AC_init, inhomo, strength):
    assert AC_init.shape == _shape()
    assert 0 <= end_step <= start_step <= c_channel.c_nsteps()
    c_channel.c_adjoint(int(start_step), int(end_step), AC_init, int(inhomo), float(strength))


def spec2phys(solution):
    if isinstance(solution, str):
        solution = read_solution(solution)
    if isinstance(solution, int):
        solution = get_solution(solution, copy=False)
    assert solution.dtype == complex
    assert solution.shape == _shape()
    flow = np.zeros([3, int(c_channel.c_Nx() * 3 // 2), c_channel.c_qpts(),
                     int(c_channel.c_Nz() * 3 // 2)], np.float64)
    c_channel.c_spec2phys(np.ascontiguousarray(solution), flow)
    return flow


def ddt_project(i_step, v):
    """Project v against the primal time derivative at i_step; v updated in
    place; returns the removed component (channel/channel.c:704-780)."""
    return c_channel.c_ddt_project(int(i_step), v)


def vel(i_step):
    """Streamwise velocity field at step i_step."""
    return spec2phys(get_solution(i_step, copy=True))[0]


def _centre(profile_values):
    return profile_values[..., c_channel.c_qpts() // 2 + 1]


def velAvg(start_step, end_step, T, profile=True):
    """Time-averaged streamwise velocity profile (or its value at quadrature
    point qpts/2 + 1), channel/__init__.py:217-236.  The x-z average of each
    step's field is the mean Fourier mode, computed on the device from the
    stored coefficients (c_mean_profile) instead of spec2phys per step."""
    assert 0 <= start_step <= end_step <= c_channel.c_nsteps()
    uavg = np.zeros(c_channel.c_qpts()) if profile else 0.0
    if end_step > start_step:
        prof = c_channel.c_mean_profile(0, 0, start_step, end_step)
        for u in prof:
            uavg = uavg + (dt / T) * (u if profile else _centre(u))
    return uavg


def wallShear(start_step, end_step):
    """dU/dy of the mean streamwise flow at the wall y = -1 for each step in
    start_step..end_step-1 (the reference's Uxb, channel/project0.c:224-234)."""
    return c_channel.c_wall_shear(0, start_step, end_step)[:, 0].copy()


def wallShearAvg(start_step, end_step, T):
    """Time-averaged wall shear dU/dy(-1) over steps start_step..end_step-1."""
    tau = 0.0
    for t in wallShear(start_step, end_step):
        tau = tau + (dt / T) * t
    return tau


def Ivel(i_step, project=False):
    """Incremental (tangent) streamwise velocity at step i_step."""
    IC = c_channel.c_getincresoln(int(i_step)).copy()
    assert IC.shape == _shape()
    if project:
        ddt_project(i_step, IC)
    return spec2phys(IC)[0]


def IvelAvg(start_step, end_step, T, profile=True):
    """Time-averaged mean tangent streamwise velocity (channel/__init__.py:253-273),
    from the stored tangent trajectory on the device."""
    assert 0 <= start_step <= end_step <= c_channel.c_nsteps()
    vavg = np.zeros(c_channel.c_qpts()) if profile else 0.0
    if end_step > start_step:
        prof = c_channel.c_mean_profile(1, 0, start_step, end_step)
        for v in prof:
            vavg = vavg + (dt / T) * (v if profile else _centre(v))
    return vavg


def uavgGrad(n_chunk, chunk_bounds, T, uavg, zeta, profile=True):
    """Time-averaged sensitivity of the mean streamwise profile to the mass
    flux, with the LSS time-dilation terms zeta (channel/__init__.py:275-299)."""
    grad = np.zeros(c_channel.c_qpts()) if profile else 0.0
    for i in range(n_chunk):
        start_step = chunk_bounds[i]
        end_step = chunk_bounds[i + 1]
        vavg = IvelAvg(start_step, end_step, T, profile)
        uEnd = c_channel.c_mean_profile(0, 0, end_step, end_step + 1)[0]
        if not profile:
            uEnd = _centre(uEnd)
        grad = grad + vavg + (1. / T) * zeta[i] * (uEnd - uavg)
    return grad
