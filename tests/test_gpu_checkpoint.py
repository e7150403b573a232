"""channel.checkpoint.forward_adjoint: the checkpointed long-horizon adjoint
equals the adjoint on a fully stored trajectory bit for bit, for any
checkpoint spacing; the HBM-sized spacing is positive and bounded."""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

GRID = dict(Nx=16, Ny=33, Nz=16, Lx=2 * np.pi, Lz=np.pi, Re=2000.0, flux=2.0, dt=0.01)
N = 10


@pytest.fixture(scope="module")
def mods():
    if not has_gpu():
        pytest.skip("no CUDA device")
    pytest.importorskip("torch")
    from channel import c_channel, checkpoint
    return c_channel, checkpoint


def test_checkpointed_adjoint_equals_stored(mods):
    cc, ck = mods
    C0 = O.synthetic_state(16, 33, 16, seed=6, amp=5e-2)
    AC0 = O.synthetic_state(16, 33, 16, seed=7, laminar=False)
    ck._init(GRID, N)
    C = C0.copy()
    cc.c_primal(0, C)
    AC = AC0.copy()
    cc.c_adjoint(N, 0, AC, 0, 0.0)
    for spacing in (1, 3, 4, N):
        Cf, ACk, rep = ck.forward_adjoint(GRID, C0, N, AC0, spacing=spacing)
        assert np.array_equal(Cf, C), spacing
        assert np.array_equal(ACk, AC), spacing
        assert rep["checkpoints"] == -(-N // spacing)
        assert rep["forward_s"] > 0 and rep["recompute_overhead"] is not None


def test_hbm_sized_spacing(mods):
    cc, ck = mods
    k = ck.choose_spacing(dict(GRID, Nx=128, Ny=129, Nz=128), 5000, fraction=0.5)
    assert 1 <= k <= 5000
    assert k * ck.bytes_per_step(dict(GRID, Nx=128, Ny=129, Nz=128)) <= 300e9
