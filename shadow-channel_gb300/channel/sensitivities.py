"""Mean-velocity statistics and their sensitivities (drivers/sensitivities.py),
Python 3, with the x-z averages computed on the device from the stored
trajectories (c_mean_profile, c_mean_product) instead of spec2phys per step.

dirc is the velocity component (0 streamwise, 1 wall-normal, 2 spanwise).
The tangent fields carry the reference's 1/Re^2 factor (sensitivities.py:58).
"""
import numpy as np

from . import c_channel
import channel as _ch


def _steps(start_step, end_step):
    assert 0 <= start_step <= end_step <= c_channel.c_nsteps()
    return end_step > start_step


def vel(dirc, i_step):
    """Velocity component dirc at step i_step (physical field)."""
    return _ch.spec2phys(_ch.get_solution(i_step, copy=True))[dirc]


def velAvg(dirc, start_step, end_step, T):
    """Time-averaged x-z mean profile of component dirc."""
    uavg = np.zeros(c_channel.c_qpts())
    if _steps(start_step, end_step):
        for u in c_channel.c_mean_profile(0, dirc, start_step, end_step):
            uavg = uavg + (_ch.dt / T) * u
    return uavg


def vel2Avg(dirc, start_step, end_step, T):
    """Time-averaged x-z mean of the squared component dirc."""
    u2avg = np.zeros(c_channel.c_qpts())
    if _steps(start_step, end_step):
        for u2 in c_channel.c_mean_product(0, dirc, 0, dirc, start_step, end_step):
            u2avg = u2avg + (_ch.dt / T) * u2
    return u2avg


def I_vel(dirc, i_step, project=False):
    """Tangent velocity component dirc at step i_step, times 1/Re^2."""
    IC = c_channel.c_getincresoln(int(i_step)).copy()
    if project:
        _ch.ddt_project(i_step, IC)
    return (1. / (_ch.Re * _ch.Re)) * _ch.spec2phys(IC)[dirc]


def dvelAvg(dirc, start_step, end_step, T):
    """Time-averaged x-z mean of the tangent component dirc, times 1/Re^2."""
    vavg = np.zeros(c_channel.c_qpts())
    if _steps(start_step, end_step):
        for v in c_channel.c_mean_profile(1, dirc, start_step, end_step):
            vavg = vavg + (_ch.dt / T) * ((1. / (_ch.Re * _ch.Re)) * v)
    return vavg


def dvel2Avg(dirc, start_step, end_step, T):
    """Time-averaged x-z mean of 2 u v (u primal, v tangent / Re^2) for component dirc."""
    du2avg = np.zeros(c_channel.c_qpts())
    if _steps(start_step, end_step):
        for uv in c_channel.c_mean_product(0, dirc, 1, dirc, start_step, end_step):
            du2avg = du2avg + (_ch.dt / T) * (2 * (1. / (_ch.Re * _ch.Re)) * uv)
    return du2avg


def uBarGrad(dirc, n_chunk, chunk_bounds, T, uavg, zeta):
    """Sensitivity of the time-averaged mean profile to Re with the LSS
    time-dilation terms zeta (sensitivities.py:96-115)."""
    grad = np.zeros(c_channel.c_qpts())
    for i in range(n_chunk):
        start_step, end_step = chunk_bounds[i], chunk_bounds[i + 1]
        duAvg = dvelAvg(dirc, start_step, end_step, T)
        uEnd = c_channel.c_mean_profile(0, dirc, end_step, end_step + 1)[0]
        grad = grad + duAvg + (1. / T) * (1. / (_ch.Re * _ch.Re)) * zeta[i] * (uEnd - uavg)
    return grad


def u2BarGrad(dirc, n_chunk, chunk_bounds, T, u2avg, zeta):
    """The same for the mean square profile (sensitivities.py:117-137); as in
    the reference, the end value is the square of the mean profile."""
    grad = np.zeros(c_channel.c_qpts())
    for i in range(n_chunk):
        start_step, end_step = chunk_bounds[i], chunk_bounds[i + 1]
        du2Avg = dvel2Avg(dirc, start_step, end_step, T)
        uEnd = c_channel.c_mean_profile(0, dirc, end_step, end_step + 1)[0]
        u2End = uEnd * uEnd
        grad = grad + du2Avg + (1. / T) * (1. / (_ch.Re * _ch.Re)) * zeta[i] * (u2End - u2avg)
    return grad
