"""The allocation-free spec2phys entry point (c_spec2phys_noalloc).

Callers that cannot allocate device memory at the point of use -- code
running while a stream is captured into a CUDA graph, or real-time loops
kept off the allocator -- pass their own device arrays for the input and
the output; the library's intermediate arrays come from fixed device
storage shared by every call.  This checks, through the C ABI:

* two calls in a row reproduce the regular c_spec2phys result;
* a call after one whose input was all NaN (every scratch entry it wrote is
  NaN) still gives the exact result: no scratch entry is read before the
  current call writes it;
* a smaller grid after a larger one (the scratch laid out differently);
* the same with the FP64 kernels (CHN_RECON_FP64=1, CHN_TRANSFORMS_FP64=1),
  in a fresh process because the kernel choice is made at c_init;
* a grid beyond the fixed capacity is refused.

Kept in a file of its own that pytest collects last.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import has_gpu

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
G32 = (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 1)
G16 = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 1)
TOL = 1e-12


def _check(cc, args, seeds, poison_first=False):
    """relative errors of c_spec2phys_noalloc against c_spec2phys for the
    given seeds (calls in a row), optionally after an all-NaN call"""
    import torch
    from channel.synthetic import synthetic_state
    assert cc.c_init(*args) == 0, cc.c_last_error_message()
    Nx, Ny, Nz = args[:3]
    flow_shape = (3, 3 * Nx // 2, 3 * Ny // 2, 3 * Nz // 2)
    errs = []
    try:
        if poison_first:
            bad = np.full((Nz, 2, Ny - 2, Nx // 2), complex(np.nan, np.nan))
            dC = torch.from_numpy(bad.view(np.float64)).cuda()
            dflow = torch.zeros(flow_shape, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            assert cc.lib.c_spec2phys_noalloc(dC.data_ptr(), dflow.data_ptr()) == 0, cc.c_last_error_message()
            assert cc.c_synchronize() == 0
            assert torch.isnan(dflow).any().item()
        for seed in seeds:
            C = synthetic_state(Nx, Ny, Nz, seed=seed)
            ref = np.zeros(flow_shape)
            cc.c_spec2phys(C, ref)
            dC = torch.from_numpy(C.view(np.float64)).cuda()
            dflow = torch.full(flow_shape, float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            assert cc.lib.c_spec2phys_noalloc(dC.data_ptr(), dflow.data_ptr()) == 0, cc.c_last_error_message()
            assert cc.c_synchronize() == 0
            got = dflow.cpu().numpy()
            assert np.isfinite(got).all()
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    finally:
        cc.c_destroy()
    return errs


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def test_noalloc_matches_spec2phys_twice(cc):
    errs = _check(cc, G32, (3, 4))
    assert max(errs) <= TOL, errs


def test_noalloc_after_a_poisoned_call(cc):
    errs = _check(cc, G32, (5,), poison_first=True)
    assert max(errs) <= TOL, errs


def test_noalloc_smaller_grid_after_larger(cc):
    errs = _check(cc, G32, (6,)) + _check(cc, G16, (7, 8)) + _check(cc, G32, (9,), poison_first=True)
    assert max(errs) <= TOL, errs


_FP64_SCRIPT = r"""
import json, sys
sys.path[:0] = [sys.argv[1], sys.argv[2]]
import numpy as np
import test_zz_no_alloc as T
from channel import c_channel as cc
errs = T._check(cc, T.G32, (3, 4), poison_first=True) + T._check(cc, T.G16, (5,), poison_first=True)
print("RESULT " + json.dumps(errs))
"""


def test_noalloc_fp64_kernels_in_fresh_process(cc):
    env = dict(os.environ, CHN_RECON_FP64="1", CHN_TRANSFORMS_FP64="1")
    r = subprocess.run([sys.executable, "-c", _FP64_SCRIPT, str(ROOT / "tests"), str(ROOT / "shadow-channel_gb300")],
                       env=env, capture_output=True, text=True, timeout=600)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")]
    assert r.returncode == 0 and line, r.stdout[-2000:] + r.stderr[-2000:]
    errs = json.loads(line[0][7:])
    assert max(errs) <= TOL, errs


def test_noalloc_rejects_grids_beyond_capacity(cc):
    assert cc.c_init(48, 97, 48, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 1) == 0
    assert cc.lib.c_spec2phys_noalloc(None, None) == -5
    assert "capacity" in cc.c_last_error_message()
    cc.c_destroy()
