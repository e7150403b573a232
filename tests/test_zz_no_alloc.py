"""The allocation-free spec2phys entry point (c_spec2phys_noalloc).

Callers that cannot allocate device memory at the point of use -- code
running while a stream is captured into a CUDA graph, or real-time loops
kept off the allocator -- pass their own device arrays for the input and
the output; the library's intermediate arrays come from fixed device
storage.  This checks, through the C ABI, that two calls in a row reproduce
the regular c_spec2phys result, and that an oversized grid is refused.

Kept in a file of its own that pytest collects last.
"""
import numpy as np
import pytest

from conftest import has_gpu
from channel.synthetic import synthetic_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def test_noalloc_matches_spec2phys_twice(cc):
    import torch
    args = (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 1)
    assert cc.c_init(*args) == 0, cc.c_last_error_message()
    Nx, Ny, Nz = args[:3]
    flow_shape = (3, 3 * Nx // 2, 3 * Ny // 2, 3 * Nz // 2)
    for seed in (3, 4):
        C = synthetic_state(Nx, Ny, Nz, seed=seed)
        ref = np.zeros(flow_shape)
        cc.c_spec2phys(C, ref)
        dC = torch.from_numpy(C.view(np.float64)).cuda()
        dflow = torch.full(flow_shape, float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert cc.lib.c_spec2phys_noalloc(dC.data_ptr(), dflow.data_ptr()) == 0, cc.c_last_error_message()
        assert cc.c_synchronize() == 0
        got = dflow.cpu().numpy()
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= 1e-12, err
    cc.c_destroy()


def test_noalloc_rejects_grids_beyond_capacity(cc):
    assert cc.c_init(48, 97, 48, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 1) == 0
    assert cc.lib.c_spec2phys_noalloc(None, None) == -5
    assert "capacity" in cc.c_last_error_message()
    cc.c_destroy()
