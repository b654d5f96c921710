"""Re-planning a handle releases the device buffers it replaces: after a larger
receiver set, a new per-cell model or a new tuning, and after a rebuilt batch
schedule, the device memory in use is that of the current plan, not the sum of
every plan made; the results stay those of a fresh handle."""
import numpy as np
import pytest
import torch

from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.batch import Batch
from seismic_cpml_gb300.solver import Solver
from seismic_cpml_gb300.workloads import batch2d_shots

pytestmark = pytest.mark.gpu

MB = 1 << 20


def used_bytes():
    torch.cuda.synchronize()
    free, total = torch.cuda.mem_get_info()
    return total - free


def receiver_grid(p, n):
    rng = np.random.default_rng(n)
    return [(int(i), int(j)) for i, j in zip(rng.integers(1, p.nx + 1, n), rng.integers(1, p.ny + 1, n))]


def test_growing_receiver_sets_release_the_old_seismogram_buffer():
    p, rec = P.small_2d(nx=48, ny=64, nstep=2000)
    small, big = receiver_grid(p, 10_000), receiver_grid(p, 20_000)   # 240 MB and 480 MB of traces
    with Solver(p, rec) as s:
        s.set_receivers(small)
        base = used_bytes()
        s.set_receivers(big)
        grown = used_bytes() - base
        # the 480 MB buffer replaces the 240 MB one: +240 MB, not +480 MB
        assert grown < 300 * MB, grown / MB
        s.run(200)
        vx, _, _ = s.seismograms()
    with Solver(p, big) as fresh:
        fresh.run(200)
        assert np.array_equal(vx[:, :200], fresh.seismograms()[0][:, :200])


def test_repeated_retuning_does_not_grow_device_memory():
    p, rec = P.small_3d(n=(40, 36, 36), nstep=60)
    with Solver(p, rec) as s:
        s.set_tuning(0, 8, 16, 2)
        base = used_bytes()
        for _ in range(6):
            for ty, lz in ((8, 24), (16, 16), (8, 16)):
                s.set_tuning(0, ty, lz, 2)
        assert used_bytes() - base < 8 * MB
        s.run()
        vx = s.seismograms()[0]
    with Solver(p, rec, tuning=(0, 8, 16, 2)) as fresh:
        fresh.run()
        assert np.array_equal(vx, fresh.seismograms()[0])


def test_batch_schedule_rebuild_releases_the_old_schedule():
    shots = batch2d_shots(nshots=3, seed=2, interior=(24, 40), npml=8, record_s=0.25, nrec=7)
    big = [receiver_grid(p, 40_000) for p, _, _ in shots]
    with Batch([p for p, _, _ in shots], receivers=big) as b:
        b.run()
        a = b.seismograms(1)[0].copy()
        base = used_bytes()
        for _ in range(4):                      # each call marks the schedule for a rebuild
            b.set_wait_limit(0)
            b.run()
        assert used_bytes() - base < 8 * MB
        assert np.array_equal(b.seismograms(1)[0], a)
