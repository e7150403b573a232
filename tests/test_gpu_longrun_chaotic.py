"""Long-run statistics in a chaotic regime, against the reference's.

The case (tests/golden/make_longrun.py): a 16x33x16 channel at Re 3300,
dt 0.01, run up 4000 steps into sustained turbulence, where two
trajectories 1e-8 apart separate to O(1) in a few thousand steps.  From the
same saved state the GPU runs the 12000 steps the reference ran; rounding
differences grow until the two trajectories are unrelated, so only their
statistics can agree.  Compared: the time means of the first eight
mean-flow Legendre coefficients, the lower-wall shear and the perturbation
energy, each with its sampling error from 12 batch means per run.

* the two runs decorrelate (end states O(1) apart: the comparison is
  statistical, not a trajectory match);
* every mean agrees within 3.5 combined sampling errors, and the sum of the
  squared z-scores stays below the 99.9% point of chi-square with 10
  degrees of freedom (29.6);
* a biased scheme is caught: the same run at Re x 1.3 fails the check.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import has_gpu

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_longrun as ML  # noqa: E402

Z_MAX = 3.5
CHI2_999_10 = 29.59


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


@pytest.fixture(scope="module")
def fix():
    return dict(np.load(GOLDEN / "longrun_16x33x16_re3300.npz"))


def _run(cc, grid, C0, nstat, chunk=500):
    assert cc.c_init(*grid, chunk) == 0, cc.c_last_error_message()
    C = C0.copy()
    series = []
    for _ in range(nstat // chunk):
        cc.c_primal(0, C)
        assert cc.c_last_error() == 0, cc.c_last_error_message()
        for i in range(1, chunk + 1):
            series.append(ML.stats_of(cc.c_getsoln(i)))
    cc.c_destroy()
    return C, ML.batch_means(series, ML.NBATCH)


def _zscores(bm_a, bm_b):
    n = bm_a.shape[0]
    sa = bm_a.std(0, ddof=1) / np.sqrt(n)
    sb = bm_b.std(0, ddof=1) / np.sqrt(bm_b.shape[0])
    return (bm_a.mean(0) - bm_b.mean(0)) / np.sqrt(sa ** 2 + sb ** 2)


def _grid(fix, re_factor=1.0):
    g = [float(v) for v in fix["grid"]]
    g[0], g[1], g[2] = int(g[0]), int(g[1]), int(g[2])
    g[5] *= re_factor
    return tuple(g)


def test_statistics_match_reference_after_decorrelation(cc, fix):
    C_end, bm = _run(cc, _grid(fix), fix["C0"], int(fix["nstat"]))
    sep = np.linalg.norm(C_end - fix["C_end"]) / np.linalg.norm(fix["C_end"])
    z = _zscores(bm, fix["batch_means"])
    print(f"\nend-state separation {sep:.3f}; z-scores {np.round(z, 2)}; chi2 {np.sum(z ** 2):.1f}")
    print(f"means GPU {bm.mean(0)}\n  reference {fix['batch_means'].mean(0)}")
    assert sep > 0.1, sep
    assert np.all(np.abs(z) < Z_MAX), z
    assert np.sum(z ** 2) < CHI2_999_10


def test_biased_scheme_fails_the_check(cc, fix):
    _, bm = _run(cc, _grid(fix, 1.3), fix["C0"], int(fix["nstat"]))
    z = _zscores(bm, fix["batch_means"])
    print(f"\nRe x 1.3: z-scores {np.round(z, 2)}; chi2 {np.sum(z ** 2):.1f}")
    assert np.any(np.abs(z) >= Z_MAX) or np.sum(z ** 2) >= CHI2_999_10
