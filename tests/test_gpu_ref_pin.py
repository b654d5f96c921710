"""The GPU path against the reference programs' own outputs.

tests/golden/refpin_*.npz hold the reference programs' outputs, from their
Fortran statements translated to C by oracle/ref_f90c.py and run
(tests/golden/make_ref_vectors.py). libcpml (FP32 CUDA kernels for sm_103a,
called through the C ABI) runs the same parameters. The set includes cases
the other GPU tests do not:
  - one PML face off in 2D;
  - the Ricker and Gaussian wavelets of the programs' alternative lines;
  - receiver lines of three points;
  - the fourth-order program with its x-min face off;
  - 3D with the x-min and z-max faces off;
  - per-cell models in the second- and fourth-order programs.
Tolerances (relative L2, the reference's FP64 run as truth): seismograms
1e-5, energy curve 1e-6. The 3D program records vx and vy only.
"""
import pytest

from seismic_cpml_gb300.solver import Solver
from tests.test_ref_pin import SHIPPED, SMALL, compare_fp32, load, model_of, params_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", SMALL + SHIPPED)
def test_gpu_matches_reference(name):
    fx = load(name)
    p, rec = params_of(fx)
    with Solver(p, rec, model=model_of(fx)) as s:
        s.run()
        vx, vy, _ = s.seismograms()
        ek, ep = s.energy()
    et, ee = compare_fp32(fx, vx, vy, ek, ep)
    print(f"{name}: trace rel-L2 {et:.3e}, energy rel-L2 {ee:.3e}")
