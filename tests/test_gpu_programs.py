"""GPU parity of the two other 2D programs on the path, through the C ABI:

  seismic_CPML_2D_isotropic_fourth_order.f90  (order = 4: the 27/24 staggered
      operator, a ghost layer read as zero, the K_y correction of 2D4:596 and
      the one-cell-wider energy interior of 2D4:696-712)
  seismic_PML_Collino_2D_isotropic.f90        (scheme = split: the classical
      split-field PML the reference compares its C-PML against, 2D:764-777)

Both against the FP64 oracle restatements (oracle/cpml_oracle.cpp, checked
against oracle/oracle_np.py), at the programs' own shipped sizes through the
golden fixtures and on small grids with whole fields. Tolerances as in
test_gpu_parity: traces <= 1e-5 and energy <= 1e-6 relative L2.
"""
import numpy as np
import pytest

from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.lib import CpmlError
from seismic_cpml_gb300.solver import Solver
from oracle import oracle_c
from tests.models import layered_2d
from tests.test_gpu_parity import check, run_gpu

pytestmark = pytest.mark.gpu


def _fixture_case(golden, name, params):
    g0 = golden(name)
    p = params()
    rec = [tuple(r) for r in g0["rec"]]
    assert rec == P.reference_receivers_2d(p)
    g = run_gpu(p, rec)

    class R:
        sisvx, sisvy, sisvz, ek, ep = g0["sisvx"], g0["sisvy"], None, g0["ek"], g0["ep"]
    et, ee = check(g, R)
    # max|v| at the last display step, as the program prints it
    assert abs(g["vmax"] - g0["vmax"][-1]) <= 1e-4 * g0["vmax"][-1]
    return et, ee, g


def test_fourth_order_program_as_shipped(golden):
    """101 x 641, 4000 steps of 1 ms (2D4:132-190), first derivative of a
    Gaussian at (80, 428), 135 degrees, receivers at (70, 231), (81, 31)."""
    et, ee, _ = _fixture_case(golden, "ref2d_fourth", P.default_2d_fourth)
    print(f"fourth-order program: trace rel-L2 {et:.3e}, energy rel-L2 {ee:.3e}")


def test_split_pml_program_as_shipped(golden):
    """The classical split-field PML program (PML:96-141), 2000 steps."""
    et, ee, _ = _fixture_case(golden, "ref2d_split", P.default_2d_split)
    print(f"split-PML program: trace rel-L2 {et:.3e}, energy rel-L2 {ee:.3e}")


@pytest.mark.parametrize("het", [False, True])
def test_fourth_order_small_with_fields(het):
    p, rec = P.small_2d(nstep=300)
    p.order = 4
    p.deltat = 1.0e-3
    model = layered_2d(p, seed=3) if het else None
    kw = dict(lam=model[0], mu=model[1], rho=model[2]) if het else {}
    ref = oracle_c.run(p, rec=rec, keep_fields=True, **kw)
    ref32 = oracle_c.run(p, rec=rec, keep_fields=True, double=False, **kw)
    g = run_gpu(p, rec, model)
    check(g, ref, ref.fields, ref32.fields)
    # a different program than the second-order one on the same grid
    q = p.copy()
    q.order = 2
    other = oracle_c.run(q, rec=rec, **kw)
    assert np.linalg.norm(g["vx"] - other.sisvx) > 1e-3 * np.linalg.norm(other.sisvx)


def test_split_small_with_fields():
    p, rec = P.small_2d(nstep=300)
    p.scheme = P.SCHEME_SPLIT
    ref = oracle_c.run(p, rec=rec, keep_fields=True)
    ref32 = oracle_c.run(p, rec=rec, keep_fields=True, double=False)
    g = run_gpu(p, rec)
    check(g, ref, ref.fields, ref32.fields)


def test_cpml_against_split_pml_energy(golden):
    """The reference's comparison (plot_comparison, 2D:764-777): the total
    energy of the C-PML run and of the split-field PML run of the same
    source, receivers and grid, each from the GPU; after the wave has left
    the interior, the C-PML leaves less energy behind."""
    g_c = run_gpu(P.default_2d(), P.reference_receivers_2d(P.default_2d()))
    g_s = run_gpu(P.default_2d_split(), P.reference_receivers_2d(P.default_2d_split()))
    e_c = g_c["ek"] + g_c["ep"]
    e_s = g_s["ek"] + g_s["ep"]
    ref_c, ref_s = golden("ref2d_default"), golden("ref2d_split")
    assert np.linalg.norm(e_c - (ref_c["ek"] + ref_c["ep"])) <= 1e-6 * np.linalg.norm(ref_c["ek"] + ref_c["ep"])
    assert np.linalg.norm(e_s - (ref_s["ek"] + ref_s["ep"])) <= 1e-6 * np.linalg.norm(ref_s["ek"] + ref_s["ep"])
    late = slice(1500, 2000)
    assert e_c[late].mean() < e_s[late].mean(), (e_c[late].mean(), e_s[late].mean())


def test_kernel_choices_of_the_other_programs():
    for mk in (P.default_2d_fourth, P.default_2d_split):
        p = mk()
        p.nstep = 20
        with Solver(p, []) as s:
            assert s.tuning()[0] == 1 and s.launches_per_step() == (2, 2)   # two-sweep
            with pytest.raises(CpmlError):
                s.set_tuning(3, 8, 32, 2)        # the persistent kernel is the second-order program's
            with pytest.raises(CpmlError):
                s.set_tuning(4, 8, 32, 2)        # and so is the on-chip cluster kernel
    p = P.default_2d_split()
    p.nstep = 20
    with Solver(p, []) as s:
        lam = np.full((p.ny, p.nx), 1e9, np.float32)
        with pytest.raises(CpmlError):
            s.set_model(lam, lam, lam)           # the split-field program is homogeneous
