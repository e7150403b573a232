"""Generate tests/golden/longrun_16x33x16_re3300.npz: long-run statistics of
the reference in a chaotic regime.

Run here, where the reference compiles (the reference's own channel/*.c,
oracle/_ref; the oracle port, bit-identical to it, where it does not):

    python tests/golden/make_longrun.py

Case: 16x33x16 channel, 2pi x 2 x pi, Re 3300, dt 0.01, flux 2.  From the
seeded synthetic state (seed 0, amplitude 5e-2) the flow becomes turbulent
and stays so; two trajectories started 1e-8 apart separate to O(1) within
~4000 steps and stay O(1) apart (chaos).  After RUNUP steps the state C0 is
saved; the statistics run covers NSTAT further steps in NBATCH batches.
Per step the statistics are linear functionals of the mean flow and the
perturbation energy (stats_of); the fixture keeps their batch means, from
which a test takes the time means and their sampling errors.
"""
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

GRID = (16, 33, 16, 2 * np.pi, np.pi, 3300.0, 2.0, 0.01)
SEED, AMP = 0, 5e-2
RUNUP = 4000
NSTAT, NBATCH = 12000, 12
CHUNK = 500
NA = 8  # mean-flow coefficients kept


def stats_of(C):
    """Per-state statistics: the first NA Legendre coefficients a_n of the
    mean streamwise velocity (C[0, 0, n, 0], R basis), the lower-wall shear
    dU/dy(-1) = sum_n a_n R_n'(-1) = 2 sum_n (-1)^n a_n (R_n = (1 - y^2) P_n),
    and the perturbation energy sum |C|^2 over every mode but (0, 0)."""
    a = C[0, 0, :, 0].real
    n = np.arange(a.size)
    shear = 2.0 * np.sum(np.where(n % 2 == 0, 1.0, -1.0) * a)
    e = float(np.sum(np.abs(C) ** 2) - np.sum(np.abs(C[0, :, :, 0]) ** 2))
    return np.concatenate([a[:NA], [shear, e]])


def batch_means(series, nbatch):
    s = np.asarray(series)
    return s[: (len(s) // nbatch) * nbatch].reshape(nbatch, -1, s.shape[1]).mean(axis=1)


def main():
    import oracle as O
    use_ref = O.RefChannel.available()
    if use_ref:
        O.build_ref()
    Ch = O.RefChannel if use_ref else O.PortChannel
    t0 = time.time()
    ch = Ch(*GRID, CHUNK)
    C = O.synthetic_state(*GRID[:3], seed=SEED, amp=AMP)
    for _ in range(RUNUP // CHUNK):
        assert ch.primal(0, C) == 0
    C0 = C.copy()
    series = []
    for _ in range(NSTAT // CHUNK):
        assert ch.primal(0, C) == 0
        for i in range(1, CHUNK + 1):
            series.append(stats_of(ch.getsoln(i)))
    bm = batch_means(series, NBATCH)
    np.savez_compressed(HERE / "longrun_16x33x16_re3300.npz", grid=np.array(GRID), C0=C0, C_end=C,
                        batch_means=bm, nstat=NSTAT, nbatch=NBATCH, runup=RUNUP, seed=SEED, amp=AMP,
                        source=np.array("reference channel/*.c" if use_ref else "oracle port"))
    print(f"done in {time.time() - t0:.0f} s; means {bm.mean(0)}; sampling errors {bm.std(0, ddof=1) / np.sqrt(NBATCH)}")


if __name__ == "__main__":
    main()
