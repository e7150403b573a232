"""GPU parity: the product (libc_channel.so, FP64 CUDA) against the CPU oracle.

Every call goes through the C ABI via the c_channel ctypes module, exactly
like the reference's SWIG module is driven by channel/__init__.py.  The
oracle is the C restatement (oracle/chan_port.c), itself pinned bit-exact to
the reference (tests/test_oracle_pin.py), and the golden fixtures made from
the reference (tests/golden).

Tolerances.  Two valid FP64 evaluations of the reference's own algorithm
(its C built with and without FMA contraction) differ by up to ~7e-12 per
step at 16x33x16 and ~1.3e-11 at 32x65x32 for the primal, ~1e-11 for the
adjoint at 16x33x16 (tests/test_oracle_noise_floor.py measures this): the
implicit fourth-order operators amplify rounding.  The GPU path is held to
that floor: per-step primal error <= 5e-12 (16x33x16) and 3e-11 (32x65x32),
tangent 1e-11, adjoint 3e-11, physical fields 1e-12.  At 32x65x32 the
tensor-core contractions (exact sums of 56-bit truncated operands, rounded
once) sit at 6e-12 .. 2.0e-11 per step against the oracle over 10 steps
(the FP64 kernels: 5e-12 .. 1.05e-11), within about twice the reference's
own FMA/no-FMA difference; the bound is three times it.
"""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

TOL = 1e-12          # physical fields, quadrature
TOL_STEP = {16: 5e-12, 32: 3e-11, 8: 5e-12, 12: 5e-12}   # primal, per time step (see module docstring)
TOL_TAN = 1e-11
TOL_ADJ = 3e-11


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _init_both(cc, args):
    Nx, Ny, Nz, Lx, Lz, Re, flux, dt, n = args
    assert cc.c_init(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, n) == 0, cc.c_last_error_message()
    return O.PortChannel(*args)


CFG_TINY = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 4)
CFG0 = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 10)
# Nz = 10: an odd padded length pz = 15, where the tensor-core inverse keeps
# its z stage as one class (no radix-2 split)
CFG_ODD = (12, 17, 10, 2 * np.pi, np.pi, 1000.0, 2.0, 0.008, 4)


@pytest.mark.parametrize("args", [CFG_TINY, CFG0, CFG_ODD])
def test_quadrature_and_spec2phys(cc, args):
    ref = _init_both(cc, args)
    y, w = cc.c_quad()
    yr, wr = ref.quad()
    assert np.abs(y - yr).max() <= 4e-16 and np.abs(w - wr).max() <= 1e-15
    C = O.synthetic_state(*args[:3], seed=7)
    flow = np.zeros(ref.flow_shape)
    cc.c_spec2phys(C, flow)
    assert rel(flow, ref.spec2phys(C)) <= TOL


CFG1 = (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 10)


@pytest.mark.parametrize("args", [CFG_TINY, CFG0, CFG1, CFG_ODD])
def test_primal_per_step(cc, args):
    """Per-step relative L2 error at the FP64 floor over every stored step (10 steps)."""
    ref = _init_both(cc, args)
    n = args[-1]
    tol = TOL_STEP[args[0]]
    C0 = O.synthetic_state(*args[:3], seed=0)
    Cg, Cr = C0.copy(), C0.copy()
    cc.c_primal(0, Cg)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    ref.primal(0, Cr)
    assert np.array_equal(cc.c_getsoln(0), ref.getsoln(0))
    for i in range(1, n + 1):
        assert rel(cc.c_getsoln(i), ref.getsoln(i)) <= tol, i
    assert rel(Cg, Cr) <= tol


def test_primal_matches_golden(cc):
    g = dict(np.load(O.HERE.parent / "tests" / "golden" / "golden_cfg0.npz"))
    args = tuple(g["args"])
    args = tuple(int(a) if i in (0, 1, 2, 8) else float(a) for i, a in enumerate(args))
    assert cc.c_init(*args) == 0
    C = g["C0"].copy()
    cc.c_primal(0, C)
    assert rel(C, g["C"]) <= TOL_STEP[16]
    IC = g["IC0"].copy()
    cc.c_tangent(0, args[-1], IC, 1)
    assert rel(IC, g["IC_inh"]) <= TOL_TAN
    AC = g["AC0b"].copy()
    cc.c_adjoint(args[-1], 1, AC, 0, 0.0)
    assert rel(AC, g["ACb"]) <= TOL_ADJ


@pytest.mark.parametrize("inhomo", [0, 1])
def test_tangent(cc, inhomo):
    args = CFG0
    ref = _init_both(cc, args)
    n = args[-1]
    C0 = O.synthetic_state(*args[:3], seed=0)
    cc.c_primal(0, C0.copy())
    ref.primal(0, C0.copy())
    IC0 = O.synthetic_state(*args[:3], seed=3, laminar=False)
    ICg, ICr = IC0.copy(), IC0.copy()
    cc.c_tangent(2, n, ICg, inhomo)
    ref.tangent(2, n, ICr, inhomo)
    assert rel(ICg, ICr) <= TOL_TAN
    for i in range(2, n + 1):
        assert rel(cc.c_getincresoln(i), ref.getincresoln(i)) <= TOL_TAN, i


@pytest.mark.parametrize("strength", [0.0, 0.8])
def test_adjoint(cc, strength):
    args = CFG0
    ref = _init_both(cc, args)
    n = args[-1]
    C0 = O.synthetic_state(*args[:3], seed=0)
    cc.c_primal(0, C0.copy())
    ref.primal(0, C0.copy())
    IC0 = O.synthetic_state(*args[:3], seed=3, laminar=False)
    cc.c_tangent(0, n, IC0.copy(), 1)
    ref.tangent(0, n, IC0.copy(), 1)
    AC0 = O.synthetic_state(*args[:3], seed=4, laminar=False)
    ACg, ACr = AC0.copy(), AC0.copy()
    cc.c_adjoint(n, 1, ACg, 0, strength)
    ref.adjoint(n, 1, ACr, 0, strength)
    assert rel(ACg, ACr) <= TOL_ADJ


def test_ddt_project(cc):
    args = CFG0
    ref = _init_both(cc, args)
    C0 = O.synthetic_state(*args[:3], seed=0)
    cc.c_primal(0, C0.copy())
    ref.primal(0, C0.copy())
    for i in (0, 3):
        V0 = O.synthetic_state(*args[:3], seed=9 + i, laminar=False)
        Vg, Vr = V0.copy(), V0.copy()
        rg = cc.c_ddt_project(i, Vg)
        rr = ref.ddt_project(i, Vr)
        assert abs(rg - rr) <= 1e-12 * max(1.0, abs(rr))
        assert rel(Vg, Vr) <= 1e-10   # V - r dC/dt cancels; floor 3.5e-11 (noise-floor test)


def test_laminar_start_with_rand(cc):
    args = CFG_TINY
    ref = O.PortChannel(*args)
    O.libc_srand(1)
    ref.primal(0, None)
    assert cc.c_init(*args) == 0
    O.libc_srand(1)
    cc.c_primal(0, np.zeros((0, 0, 0, 0), complex))
    for i in range(args[-1] + 1):
        assert rel(cc.c_getsoln(i), ref.getsoln(i)) <= TOL_STEP[8], i


def test_cfl_stop(cc):
    """A step too large for the CFL limit stops the loop with the state kept,
    like channel/pass1.c:133-137 + channel/channel.c:448-452."""
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.5, 3)
    ref = _init_both(cc, args)
    C0 = O.synthetic_state(*args[:3], seed=1)
    Cg, Cr = C0.copy(), C0.copy()
    cc.c_primal(0, Cg)
    assert cc.c_last_error() & 1
    assert cc.c_last_cfl() >= 2.8
    assert ref.primal(0, Cr) == -1
    assert rel(Cg, Cr) <= TOL
    for i in range(args[-1] + 1):
        assert rel(cc.c_getsoln(i), ref.getsoln(i)) <= TOL


def test_deterministic_rerun(cc):
    args = CFG_TINY
    assert cc.c_init(*args) == 0
    C0 = O.synthetic_state(*args[:3], seed=5)
    a, b = C0.copy(), C0.copy()
    cc.c_primal(0, a)
    cc.c_primal(0, b)
    assert np.array_equal(a, b)


def test_dot_product_terms_match_reference(cc):
    """testAdj.py pattern (drivers/testAdj.py:22-56): <lambda_0, T v_0> and
    <T* lambda_0, v_0> in the physical quadrature inner product.  The
    reference's adjoint (reversed RK coefficients, channel/adjproject.c:34-38)
    is not the exact transpose of its tangent: the two sides differ by ~2e-4
    relative at this size.  The drop-in must reproduce both sides."""
    args = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 6)
    ref = _init_both(cc, args)
    n = args[-1]
    C0 = O.synthetic_state(*args[:3], seed=0)
    cc.c_primal(0, C0.copy())
    ref.primal(0, C0.copy())
    y, w = cc.c_quad()

    def sides(T, A, P):
        IC = O.synthetic_state(*args[:3], seed=22, laminar=False)
        IC0 = IC.copy()
        T(1, n - 1, IC, 0)
        AC = O.synthetic_state(*args[:3], seed=23, laminar=False)
        AC0 = AC.copy()
        A(n - 1, 1, AC, 0, 0.0)
        return (P(AC0) * P(IC) * w[:, None]).sum(), (P(AC) * P(IC0) * w[:, None]).sum()

    def gphys(C):
        f = np.zeros(ref.flow_shape)
        cc.c_spec2phys(np.ascontiguousarray(C), f)
        return f

    lg, rg = sides(cc.c_tangent, cc.c_adjoint, gphys)
    lr, rr = sides(ref.tangent, ref.adjoint, ref.spec2phys)
    assert abs(lg - lr) <= 1e-10 * abs(lr)
    assert abs(rg - rr) <= 1e-10 * abs(rr)


def test_field_cache_off_matches(cc):
    """The physical-field caches are an optimisation only: a separate process
    with CHN_NO_FIELD_CACHE=1 gives the same tangent (bit for bit) and adjoint
    (the cached coupling forms dC/dt's fields as a difference of transforms
    instead of the transform of a difference: equal up to rounding)."""
    import json
    import os
    import subprocess
    import sys
    code = r"""
import json, sys, numpy as np
sys.path.insert(0, 'shadow-channel_gb300'); sys.path.insert(0, 'oracle')
from channel import c_channel as cc
from channel.synthetic import synthetic_state
args = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 5)
assert cc.c_init(*args) == 0
cc.c_primal(0, synthetic_state(16, 33, 16, seed=0))
IC = synthetic_state(16, 33, 16, seed=3, laminar=False); cc.c_tangent(0, 5, IC, 1)
AC = synthetic_state(16, 33, 16, seed=4, laminar=False); cc.c_adjoint(5, 0, AC, 0, 0.5)
print(json.dumps({"IC": IC.view(np.float64).tolist(), "AC": AC.view(np.float64).tolist()}))
"""
    root = O.HERE.parent
    outs = []
    for off in ("0", "1"):
        env = dict(os.environ, CHN_NO_FIELD_CACHE=off)
        r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(next(ln for ln in r.stdout.splitlines() if ln.startswith("{"))))
    a, b = np.array(outs[0]["IC"]), np.array(outs[1]["IC"])
    assert np.array_equal(a, b)
    a, b = np.array(outs[0]["AC"]), np.array(outs[1]["AC"])
    assert np.linalg.norm(a - b) <= 1e-11 * np.linalg.norm(b)   # measured 2.8e-12
