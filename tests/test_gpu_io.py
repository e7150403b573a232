"""Solution files (channel.save_solution / read_solution; c_save_solution,
c_read_solution): the raw container and the npz twin that carries the
reference's HDF5 dataset names and shapes (channel/channel.c:791-1028)."""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 3)


@pytest.fixture(scope="module")
def ch():
    if not has_gpu():
        pytest.skip("no CUDA device")
    import channel
    from channel import c_channel as cc
    assert cc.c_init(*ARGS) == 0
    C = O.synthetic_state(*ARGS[:3], seed=0)
    cc.c_primal(0, C)
    IC = O.synthetic_state(*ARGS[:3], seed=3, laminar=False)
    cc.c_tangent(0, ARGS[-1], IC, 0)
    return channel, C, IC


@pytest.mark.parametrize("fmt", ["raw", "npz"])
def test_round_trip(ch, tmp_path, fmt):
    channel, C, IC = ch
    name = str(tmp_path / f"state_{fmt}")
    channel.save_solution(name, C, fmt=fmt)
    back = channel.read_solution(name)
    assert np.array_equal(back, C)


def test_npz_datasets(ch, tmp_path):
    channel, C, IC = ch
    name = str(tmp_path / "state")
    channel.save_solution(name, C, fmt="npz")
    with np.load(name + ".hd5") as z:
        R, X = ARGS[1] - 2, ARGS[0] // 2
        for k in ("data_alpha", "data_beta", "data_ialpha", "data_ibeta"):
            assert z[k].shape == (R, ARGS[2], X) and z[k].dtype == np.complex128
        # [dimR][Nz][Nx/2] transposition of C[Nz][alpha|beta][dimR][Nx/2]
        assert np.array_equal(z["data_alpha"], C[:, 0].transpose(1, 0, 2))
        assert np.array_equal(z["data_beta"], C[:, 1].transpose(1, 0, 2))
        assert np.array_equal(z["data_ialpha"], IC[:, 0].transpose(1, 0, 2))
        assert (int(z["data_Nx"][0]), int(z["data_Ny"][0]), int(z["data_Nz"][0])) == ARGS[:3]
        assert z["data_dt"][0] == ARGS[7]
        assert abs(z["data_Re"][0] - 1.0 / ARGS[5]) <= 1e-18
