"""The batched multi-shot 2D engine on the GPU: every shot of one persistent
launch is bit-identical to the same shot run alone through a single-shot
handle (same per-cell arithmetic), and matches the FP64 oracle."""
import numpy as np
import pytest

from seismic_cpml_gb300.batch import Batch
from seismic_cpml_gb300.solver import Solver
from seismic_cpml_gb300.workloads import batch2d_shots
from oracle import oracle_c

pytestmark = pytest.mark.gpu


def small_shots():
    return batch2d_shots(nshots=6, seed=11, interior=(24, 70), npml=8, record_s=0.25, nrec=7)


TUNINGS = [(1, 8), (2, 8), (2, 16), (3, 16)]


@pytest.mark.parametrize("tuning", TUNINGS, ids=["d1", "d2t8", "d2t16", "d3t16"])
def test_batch_equals_single_shots_bitwise(tuning):
    """Every temporal-blocking depth and tile height: shots of odd and even
    NSTEP (a last phase of fewer steps than the depth), homogeneous and
    per-cell models, receivers in the C-PML and the interior, bit-identical
    seismograms and final fields to single-shot handles."""
    shots = small_shots()
    assert len({p.nstep for p, _, _ in shots}) > 1          # uneven lengths
    assert {p.nstep % 2 for p, _, _ in shots} == {0, 1} and {p.nstep % 3 for p, _, _ in shots} >= {1, 2}
    models = [m if s % 2 == 0 else None for s, (_, m, _) in enumerate(shots)]
    with Batch([p for p, _, _ in shots], models=models, receivers=[r for _, _, r in shots]) as b:
        b.set_tuning(*tuning)
        assert b.tuning() == tuning
        b.run()
        for s, (p, m, rec) in enumerate(shots):
            with Solver(p, rec, model=models[s]) as one:
                one.run()
                vx1, vy1, _ = one.seismograms()
                f1 = {n: one.field(n) for n in ("vx", "vy", "sxx", "syy", "sxy")}
            vx, vy = b.seismograms(s)
            assert np.array_equal(vx, vx1) and np.array_equal(vy, vy1), s
            for n, f in f1.items():
                assert np.array_equal(b.field(s, n), f), (s, n)


def test_batch_autotune_keeps_results_exact():
    shots = small_shots()[:4]
    args = ([p for p, _, _ in shots], [m for _, m, _ in shots], [r for _, _, r in shots])
    with Batch(*args) as ref:
        ref.run()
        want = [ref.seismograms(s) for s in range(4)]
    with Batch(*args) as b:
        best = b.autotune(trial_steps=40)
        assert (best["depth"], best["tile_y"]) in TUNINGS and best["ms_per_step"] > 0
        assert b.tuning() == (best["depth"], best["tile_y"])
        b.run()
        for s in range(4):
            vx, vy = b.seismograms(s)
            assert np.array_equal(vx, want[s][0]) and np.array_equal(vy, want[s][1])


def test_batch_matches_oracle():
    shots = small_shots()[:2]
    with Batch([p for p, _, _ in shots], models=[m for _, m, _ in shots],
               receivers=[r for _, _, r in shots]) as b:
        b.run()
        for s, (p, m, rec) in enumerate(shots):
            ref = oracle_c.run(p, rec=rec, lam=m[0], mu=m[1], rho=m[2])
            vx, vy = b.seismograms(s)
            err = np.linalg.norm(np.concatenate([vx, vy]) - np.concatenate([ref.sisvx, ref.sisvy])) / \
                np.linalg.norm(np.concatenate([ref.sisvx, ref.sisvy]))
            assert err <= 1e-5, err


def test_batch_rerun_is_deterministic():
    shots = small_shots()[:3]
    with Batch([p for p, _, _ in shots], receivers=[r for _, _, r in shots]) as b:
        b.run()
        a = [b.seismograms(s)[0].copy() for s in range(3)]
        b.run()
        for s in range(3):
            assert np.array_equal(b.seismograms(s)[0], a[s])


def test_barrier_timeout_is_reported_and_the_next_run_is_clean():
    """A grid-barrier wait bound of one cycle runs out at the first barrier:
    every CTA returns, cpml_batch_run reports CPML_ERR_TIMEOUT, and with the
    default bound the same batch runs again to the exact results of a fresh
    batch (the context stays usable; nothing faults or hangs)."""
    from seismic_cpml_gb300.lib import CpmlError
    shots = small_shots()[:3]
    args = ([p for p, _, _ in shots], None, [r for _, _, r in shots])
    with Batch(*args) as ref:
        ref.run()
        want = [ref.seismograms(s)[0].copy() for s in range(3)]
    with Batch(*args) as b:
        b.set_wait_limit(1)
        with pytest.raises(CpmlError) as e:
            b.run()
        assert e.value.status == -5                         # CPML_ERR_TIMEOUT
        b.set_wait_limit(0)
        b.run()
        for s in range(3):
            assert np.array_equal(b.seismograms(s)[0], want[s])
