"""The seeded synthetic workloads against their specifications (CPU).

batch2d_shots (the 256-shot batched workload) and the large 3D model
generator define what the benchmarks run: per-shot sizes, models, time
steps and receivers. Checked here on small draws: each value range and
relation the workload specifies, and seeded determinism.
"""
import math

import numpy as np
import pytest

from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.earth import layered_model, layered_model_3d_device
from seismic_cpml_gb300.workloads import batch2d_shots


def velocities(lam, mu, rho):
    lam, mu, rho = (np.asarray(a, np.float64) for a in (lam, mu, rho))
    return np.sqrt((lam + 2.0 * mu) / rho), np.sqrt(mu / rho)


@pytest.fixture(scope="module")
def shots():
    return batch2d_shots(nshots=6, seed=4)


def test_batch_shots_follow_their_specification(shots):
    for p, (lam, mu, rho), rec in shots:
        nxi, nyi = p.nx - 40, p.ny - 40
        assert 200 <= nxi <= 1200 and 200 <= nyi <= 1200 and p.npoints_pml == 20
        assert p.deltax == p.deltay == 5.0 and list(p.use_pml) == [1, 1, 1, 1, 0, 0]
        assert lam.shape == (p.ny, p.nx) and lam.dtype == np.float32
        cp, cs = velocities(lam, mu, rho)
        # cp in [1500, 4500] times three anomalies of up to +/-10 % each (they
        # may overlap); cs = cp / sqrt(3); Gardner density
        assert cp.min() >= 1500.0 * 0.9 ** 3 * (1 - 1e-6) and cp.max() <= 4500.0 * 1.1 ** 3 * (1 + 1e-6)
        assert np.allclose(cs, cp / math.sqrt(3.0), rtol=1e-5)
        assert np.allclose(rho, 310.0 * cp ** 0.25, rtol=1e-5)
        # the shot's fastest P velocity sets cp, the C-PML and a Courant number of 0.5
        assert p.cp == pytest.approx(cp.max(), rel=1e-6)
        assert p.courant() == pytest.approx(0.5, rel=1e-12)
        assert p.nstep == math.ceil(2.0 / p.deltat)           # a 2 s record
        assert 8.0 <= p.f0 <= 25.0 and p.t0 == pytest.approx(1.2 / p.f0)
        assert p.stf == P.STF_RICKER and p.angle_force == 0.0
        assert 21 <= p.isource <= p.nx - 20 and p.jsource == p.ny - 20 - 3
        assert len(rec) == 128 and {j for _, j in rec} == {p.ny - 20 - 1}
        assert rec[0][0] == 21 and rec[-1][0] == 20 + nxi


def test_batch_shots_are_seeded(shots):
    again = batch2d_shots(nshots=6, seed=4)
    for (p, m, rec), (q, n, rec2) in zip(shots, again):
        assert (p.nx, p.ny, p.nstep, p.f0, p.isource) == (q.nx, q.ny, q.nstep, q.f0, q.isource)
        assert all(np.array_equal(a, b) for a, b in zip(m, n)) and rec == rec2
    other = batch2d_shots(nshots=2, seed=5)
    assert (other[0][0].nx, other[0][0].ny) != (shots[0][0].nx, shots[0][0].ny) or \
        not np.array_equal(other[0][1][0], shots[0][1][0])


def test_layered_model_layers_along_y():
    (lam, mu, rho), cpmax = layered_model((50, 40), 5, 2000.0, 4000.0, seed=9)
    cp, _ = velocities(lam, mu, rho)
    assert np.allclose(cp, cp[:, :1], rtol=1e-6)                 # constant along x
    assert len(np.unique(np.round(cp[:, 0], 3))) <= 5             # at most 5 layers along y
    assert cpmax == pytest.approx(cp.max(), rel=1e-6)


def test_large_3d_model_follows_its_specification():
    """The 3D large workload's generator, run small on the CPU: 6 layers
    along y with cp in [1800, 5000], each of 8 anomalies scaling cp by up to
    +/-15 %, cs = cp / sqrt(3), Gardner density, the same model for the same
    seed."""
    torch = pytest.importorskip("torch")
    shape = (12, 30, 14)
    lam, mu, rho = (t.numpy() for t in layered_model_3d_device(shape, anomalies=0, device="cpu"))
    cp, cs = velocities(lam, mu, rho)
    assert np.allclose(cp, cp[:1, :, :1], rtol=1e-6)             # a function of y alone
    assert len(np.unique(np.round(cp[0, :, 0], 2))) <= 6
    assert cp.min() >= 1800.0 * (1 - 1e-6) and cp.max() <= 5000.0 * (1 + 1e-6)
    assert np.allclose(cs, cp / math.sqrt(3.0), rtol=1e-5)
    assert np.allclose(rho, 310.0 * cp ** 0.25, rtol=1e-5)
    a = [t.numpy() for t in layered_model_3d_device(shape, device="cpu")]
    b = [t.numpy() for t in layered_model_3d_device(shape, device="cpu")]
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    # the anomalies multiply the layered model by 1 +/- 0.15 g (0 < g <= 1)
    # each; on a grid this small all eight overlap
    cpa, _ = velocities(*a)
    ratio = cpa / cp
    assert ratio.min() >= 0.85 ** 8 * (1 - 1e-5) and ratio.max() <= 1.15 ** 8 * (1 + 1e-5)
    assert np.abs(ratio - 1.0).max() > 0.01
    assert torch is not None
