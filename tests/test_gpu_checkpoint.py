"""Checkpoint / restart through the C ABI (cpml_save_state / cpml_load_state).

The state a restart of the reference time loop needs is the step counter,
the wavefields and the 18 (3D) or 8 (2D) C-PML memory variables, plus what
has been recorded so far (3D:720-756, 2D:522-544 initialise exactly these).
A run of N steps must equal, bit for bit, a run that stops after M steps,
saves, and continues in a FRESH handle (same parameters, model and
receivers) after loading the snapshot: in 2D and 3D, on every step kernel,
at an odd and an even M (the fused 3D step alternates two buffer sets).
"""
import numpy as np
import pytest

from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.lib import CpmlError
from seismic_cpml_gb300.solver import Solver
from tests.models import layered_2d, layered_3d

pytestmark = pytest.mark.gpu

NAMES_2D = ["vx", "vy", "sxx", "syy", "sxy"]
NAMES_3D = ["vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"]


def _case(name):
    if name.startswith("2d"):
        p, rec = P.small_2d(nstep=160)
        if "order4" in name:
            p.order = 4
            p.deltat = 1.0e-3
        if "split" in name:
            p.scheme = P.SCHEME_SPLIT
        model = layered_2d(p, seed=9) if "het" in name else None
        tuning = (3, 8, 32, 2) if "persistent" in name else (1, 8, 32, 2)
        return p, rec, model, tuning, NAMES_2D
    p, rec = P.small_3d(n=(40, 36, 30), nstep=150)
    model = layered_3d(p, seed=9) if "het" in name else None
    tuning = (1, 8, 32, 2) if "two_sweep" in name else (2, 8, 12, 2)
    return p, rec, model, tuning, NAMES_3D


def _results(s, names):
    vx, vy, vz = s.seismograms()
    ek, ep = s.energy()
    out = dict(vx=vx, vy=vy, vz=vz, ek=ek, ep=ep, status=s.status())
    out.update({"field_" + n: s.field(n) for n in names})
    return out


CASES = ["2d", "2d_het", "2d_persistent", "2d_order4_het", "2d_split", "3d_fused", "3d_fused_het",
         "3d_two_sweep"]


@pytest.mark.parametrize("m", [63, 64])
@pytest.mark.parametrize("case", CASES)
def test_restart_from_a_snapshot_is_bitwise(case, m):
    p, rec, model, tuning, names = _case(case)
    with Solver(p, rec, model=model, tuning=tuning) as a:
        a.run()
        full = _results(a, names)
    with Solver(p, rec, model=model, tuning=tuning) as b:
        b.run(m)
        snap = b.save_state()
    with Solver(p, rec, model=model, tuning=tuning) as c:
        c.load_state(snap)
        assert c.status()[0] == m
        c.run()
        resumed = _results(c, names)
    for k, v in full.items():
        if v is None:
            assert resumed[k] is None
        elif k == "status":
            assert resumed[k] == v
        else:
            assert np.array_equal(resumed[k], v), (case, m, k)
    assert np.abs(full["vx"]).max() > 0


def test_snapshot_moves_between_step_kernels():
    """A snapshot of the fused 3D step continues on the two-sweep kernels
    (the same time loop; the two kernels agree to FP32 rounding)."""
    p, rec, _, _, names = _case("3d_fused")
    with Solver(p, rec, tuning=(2, 16, 8, 2)) as a:
        a.run()
        full = _results(a, names)
    with Solver(p, rec, tuning=(2, 16, 8, 2)) as b:
        b.run(71)
        snap = b.save_state()
    with Solver(p, rec, tuning=(1, 8, 32, 2)) as c:
        c.load_state(snap)
        c.run()
        r = _results(c, names)
    t_full = np.concatenate([full["vx"], full["vy"], full["vz"]])
    t_r = np.concatenate([r["vx"], r["vy"], r["vz"]])
    assert np.linalg.norm(t_r - t_full) / np.linalg.norm(t_full) < 2e-6


def test_snapshot_rejected_by_a_different_handle():
    p, rec, _, tuning, _ = _case("3d_fused")
    with Solver(p, rec, tuning=tuning) as b:
        b.run(20)
        snap = b.save_state()
    q = p.copy()
    q.f0 = p.f0 * 1.1                                   # another source: another run
    with Solver(q, rec, tuning=tuning) as c:
        with pytest.raises(CpmlError) as e:
            c.load_state(snap)
        assert e.value.status == -1
    with Solver(p, rec[:2], tuning=tuning) as c:        # other receivers
        with pytest.raises(CpmlError):
            c.load_state(snap)
    with Solver(p, rec, model=layered_3d(p, seed=9), tuning=tuning) as c:   # another model
        with pytest.raises(CpmlError):
            c.load_state(snap)
    with Solver(p, rec, tuning=tuning) as c:            # truncated snapshot
        with pytest.raises(CpmlError):
            c.load_state(snap[:-8])
        c.load_state(snap)                              # the intact one loads
        assert c.status()[0] == 20
