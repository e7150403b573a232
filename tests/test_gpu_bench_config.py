"""The benchmarked batched path at its own configuration, against the oracle.

bench.py times c_batch_forward_dev + c_batch_adjoint_dev on 64 LSS segments
of a 32x65x32 channel (Re 3300, dt 0.005): per segment a primal, two
homogeneous tangents, one mean-flux tangent (the coupled one) and an adjoint
coupled to it with strength 1.  Here the same calls run on 4 such segments
over 10 steps, through the host-array and the device-array entry points, and
every segment's stored primal and tangent steps and its final tangent and
adjoint states are compared with the oracle run segment by segment through
the reference's single-trajectory sequence (channel/channel.c:399-780):
primal, the tangents (the coupled one last, so MIC is its trajectory),
adjoint.  At this grid the product and transform kernels take their tensor-
core forms (k_products_tc, k_phys_inverse_tc), as in the benchmark.

The oracle runs in a pool of spawned processes, one segment each, started
before the first GPU call.  It runs twice: as pinned (no FMA contraction)
and built with FMA contraction.  The two builds are equally valid FP64
evaluations of the reference; over these 10 steps they differ by up to
~4e-11 (the implicit fourth-order solves amplify rounding at this grid).
The GPU is held to twice that difference, measured in the same run, and to
an absolute cap.

Measured on a GB300: primal 1.7e-11, coupled tangent steps 5.8e-12, final
tangents 5.6e-11, adjoint 3.1e-11 relative to the pinned oracle.
"""
import platform
import subprocess
from pathlib import Path
import ctypes
import multiprocessing as mp

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 10)
NSEG, NTAN, COUPLE = 4, 3, 2
INHOMO = [0, 0, 1]
STRENGTH = 1.0
RUNUP = 200

FLOOR_FACTOR = 2.0   # x the reference's own FMA / no-FMA difference over the same steps
CAP = 2e-10


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def port_lib_fma(tmp):
    """the oracle port built with FMA contraction"""
    out = Path(tmp) / "libchanport_fma.so"
    flags = ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", *flags, "-o", str(out),
                    str(O.HERE / "chan_port.c"), str(O.HERE / "fft.c"), "-lm"], check=True)
    return str(out)


def oracle_segment(C, IC, AC, lib=None):
    """the reference sequence for one segment (with the given build of the
    port, default the pinned one); returns its stored steps and end states"""
    target = Path(lib) if lib is not None else O.HERE / "_build" / "libchanport.so"
    if O.PORT_LIB != target or O.PortChannel._lib is None:
        O.PortChannel._lib, O.PORT_LIB = None, target
    if lib is None and not target.exists():
        O.build_port()
    n = ARGS[-1]
    ref = O.PortChannel(*ARGS)
    c = C.copy()
    ref.primal(0, c)
    ic = IC.copy()
    for j in [j for j in range(NTAN) if j != COUPLE] + [COUPLE]:
        t = ic[j].copy()
        ref.tangent(0, n, t, INHOMO[j])
        ic[j] = t
    ac = AC.copy()
    ref.adjoint(n, 0, ac, 0, STRENGTH)
    out = {"MC": np.stack([ref.getsoln(i) for i in range(n + 1)]),
           "MIC": np.stack([ref.getincresoln(i) for i in range(n + 1)]), "C": c, "IC": ic, "AC": ac}
    ref.close()
    return out


@pytest.fixture(scope="module")
def pool():
    if not has_gpu():
        pytest.skip("no CUDA device")
    ctx = mp.get_context("spawn")
    p = ctx.Pool(NSEG)
    yield p
    p.close()
    p.join()


@pytest.fixture(scope="module")
def cc(pool):
    from channel import c_channel
    return c_channel


@pytest.fixture(scope="module")
def case(cc, pool, tmp_path_factory):
    """segment states as the benchmark makes them (run-up parent + seeded
    1e-3 perturbations), and the oracle's results for them"""
    from channel.synthetic import synthetic_state
    Nx, Ny, Nz = ARGS[:3]
    assert cc.c_init(*ARGS[:-1], 1) == 0, cc.c_last_error_message()
    Cp = synthetic_state(Nx, Ny, Nz, seed=0)
    cc.c_primal(RUNUP, Cp)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    cc.c_destroy()
    C = np.stack([Cp + synthetic_state(Nx, Ny, Nz, seed=1000 + s, amp=1e-3, laminar=False) for s in range(NSEG)])
    IC = np.stack([np.stack([synthetic_state(Nx, Ny, Nz, seed=2000 + NTAN * s + j, laminar=False)
                             for j in range(NTAN)]) for s in range(NSEG)])
    AC = np.stack([synthetic_state(Nx, Ny, Nz, seed=5000 + s, laminar=False) for s in range(NSEG)])
    refs = pool.starmap(oracle_segment, [(C[s], IC[s], AC[s]) for s in range(NSEG)])
    fma = port_lib_fma(tmp_path_factory.mktemp("fma"))
    alt = pool.starmap(oracle_segment, [(C[s], IC[s], AC[s], fma) for s in range(NSEG)])
    floor = _errors(refs, [a["MC"] for a in alt], [a["MIC"] for a in alt], [a["IC"] for a in alt],
                    [a["AC"] for a in alt])
    print(f"\nreference FMA vs no-FMA over the same steps: {floor}")
    return C, IC, AC, refs, floor


def _inh():
    return (ctypes.c_int * NTAN)(*INHOMO)


def _errors(refs, MC, MIC, IC, AC):
    """max relative errors over the segments against the pinned oracle"""
    worst = {"primal": 0.0, "tangent_steps": 0.0, "tangent": 0.0, "adjoint": 0.0}
    for s in range(NSEG):
        for i in range(ARGS[-1] + 1):
            worst["primal"] = max(worst["primal"], rel(MC[s][i], refs[s]["MC"][i]))
            worst["tangent_steps"] = max(worst["tangent_steps"], rel(MIC[s][i], refs[s]["MIC"][i]))
        for j in range(NTAN):
            worst["tangent"] = max(worst["tangent"], rel(IC[s][j], refs[s]["IC"][j]))
        worst["adjoint"] = max(worst["adjoint"], rel(AC[s], refs[s]["AC"]))
    return worst


def _compare(cc, hIC, hAC, refs, floor):
    lib = cc.lib
    n = ARGS[-1]
    MC, MIC = [], []
    for s in range(NSEG):
        mc, mic = [], []
        for i in range(n + 1):
            out = np.zeros(refs[0]["C"].shape, np.complex128)
            assert lib.c_batch_getsoln(s, i, out.ctypes.data) == 0
            mc.append(out.copy())
            assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
            mic.append(out.copy())
        MC.append(mc)
        MIC.append(mic)
    worst = _errors(refs, MC, MIC, hIC, hAC)
    print(f"\nbatched 32x65x32 vs oracle (max over {NSEG} segments, {n} steps): {worst}")
    for k, v in worst.items():
        assert v <= FLOOR_FACTOR * floor[k] + 1e-13, (k, worst, floor)
        assert v <= CAP, (k, worst, floor)
    return worst


def test_bench_config_host_api(cc, case):
    C, IC, AC, refs, floor = case
    n = ARGS[-1]
    assert cc.c_init(*ARGS) == 0, cc.c_last_error_message()
    lib = cc.lib
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0, cc.c_last_error_message()
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        assert lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, _inh()) == 0, cc.c_last_error_message()
        assert lib.c_batch_adjoint(n, 0, hAC.ctypes.data, STRENGTH) == 0, cc.c_last_error_message()
        assert cc.c_last_error() == 0, cc.c_last_error_message()
        _compare(cc, hIC, hAC, refs, floor)
        for s in range(NSEG):
            assert rel(hC[s], refs[s]["C"]) <= FLOOR_FACTOR * floor["primal"] + 1e-13, s
    finally:
        lib.c_batch_destroy()
        cc.c_destroy()


def test_bench_config_device_api(cc, case):
    """the device-array calls the benchmark times give the host-array results bit for bit"""
    torch = pytest.importorskip("torch")
    C, IC, AC, refs, floor = case
    n = ARGS[-1]
    assert cc.c_init(*ARGS) == 0, cc.c_last_error_message()
    lib = cc.lib
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0, cc.c_last_error_message()
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        assert lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, _inh()) == 0
        assert lib.c_batch_adjoint(n, 0, hAC.ctypes.data, STRENGTH) == 0
        dev = torch.device("cuda:0")
        dC = torch.from_numpy(C.view(np.float64)).to(dev)
        dIC = torch.from_numpy(IC.view(np.float64)).to(dev)
        dAC = torch.from_numpy(AC.view(np.float64)).to(dev)
        torch.cuda.synchronize()
        assert lib.c_batch_forward_dev(0, n, dC.data_ptr(), dIC.data_ptr(), _inh()) == 0
        assert lib.c_batch_adjoint_dev(n, 0, dAC.data_ptr(), STRENGTH) == 0
        assert lib.c_synchronize() == 0
        gIC = dIC.cpu().numpy().view(np.complex128)
        gAC = dAC.cpu().numpy().view(np.complex128)
        assert np.array_equal(gIC, hIC)
        assert np.array_equal(gAC, hAC)
        _compare(cc, gIC, gAC, refs, floor)
    finally:
        lib.c_batch_destroy()
        cc.c_destroy()
