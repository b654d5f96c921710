"""The allocation-free energy entry point, checked on the GPU.

cpml_energy3d_noalloc serves callers that own their wavefields on the device
and cannot allocate device memory mid-run (a pool allocator or fixed memory
budget, where cudaMalloc would synchronise the device or fail). Its scratch is
a static device array inside the library. This test calls it through the C
ABI on fields produced by a solver handle and compares the result with the
energy the handle itself recorded for the same time step, twice in a row
(the second call reuses the scratch the first one left behind). It lives in
its own file so that it runs after every other test.
"""
import ctypes

import numpy as np
import pytest

from seismic_cpml_gb300 import lib as L
from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.solver import Solver

pytestmark = pytest.mark.gpu

ENERGY_TOL = 1e-6   # relative, the tolerance the parity tests use for energy
NAMES = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")


def _reference_energy_and_fields(flags):
    p, rec = P.small_3d(n=(44, 38, 34), nstep=90)
    p.flags = flags
    with Solver(p, rec) as s:
        s.run()
        ek, ep = s.energy()
        fields = [s.field(n) for n in NAMES]
    return p, ek[-1], ep[-1], fields


@pytest.mark.parametrize("flags", [P.FLAG_ENERGY, P.FLAG_ENERGY | P.FLAG_EP_PHYSICAL])
def test_noalloc_energy_matches_solver_energy(flags):
    import torch
    lib = L.load()
    p, ek_ref, ep_ref, fields = _reference_energy_and_fields(flags)
    dev = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in fields]
    ptrs = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in dev])
    lam = p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs)
    mu = p.rho * p.cs * p.cs
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.cpml_energy3d_noalloc(ptrs, p.nx, p.ny, p.nz, p.nx, p.npoints_pml, lam, mu, p.rho,
                                       None, None, None, flags, out.data_ptr(), stream)
        assert st == 0, L.strerror(st)
        torch.cuda.synchronize()
        ek, ep = out.cpu().numpy()
        assert abs(ek - ek_ref) <= ENERGY_TOL * abs(ek_ref), (ek, ek_ref)
        assert abs(ep - ep_ref) <= ENERGY_TOL * abs(ep_ref), (ep, ep_ref)


def test_noalloc_rejects_too_many_planes():
    lib = L.load()
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    st = lib.cpml_energy3d_noalloc(ptrs, 8, 8, 8193, 8, 2, 1.0e9, 1.0e9, 2000.0,
                                   None, None, None, 0, 1, None)
    assert st == -9   # CPML_ERR_RANGE: the static scratch holds 8192 planes
