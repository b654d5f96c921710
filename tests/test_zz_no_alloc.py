"""The allocation-free energy entry point, checked on the GPU.

cpml_energy3d_noalloc serves callers that own their wavefields on the device
and cannot allocate device memory mid-run (a pool allocator or fixed memory
budget, where cudaMalloc would synchronise the device or fail). Its scratch is
a static device array inside the library. These tests call it through the C
ABI on fields produced by a solver handle and compare the result with the
energy the handle itself recorded for the same time step, twice in a row
(the second call reuses the scratch the first one left behind): for the
homogeneous model, for a per-cell model passed as device arrays, and for
fields copied into a padded row pitch. It lives in its own file so that it
runs after every other test.
"""
import ctypes

import numpy as np
import pytest

from seismic_cpml_gb300 import lib as L
from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.solver import Solver
from tests.models import layered_3d

pytestmark = pytest.mark.gpu

ENERGY_TOL = 1e-6   # relative, the tolerance the parity tests use for energy
NAMES = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")


def _reference_energy_and_fields(flags, model=None):
    p, rec = P.small_3d(n=(44, 38, 34), nstep=90)
    p.flags = flags
    with Solver(p, rec, model=model) as s:
        s.run()
        ek, ep = s.energy()
        fields = [s.field(n) for n in NAMES]
    return p, ek[-1], ep[-1], fields


def _to_device(arrays, pitch):
    """float32 [nz][ny][nx] host arrays -> device tensors [nz][ny][pitch] (pad zero)."""
    import torch
    out = []
    for a in arrays:
        nz, ny, nx = a.shape
        t = torch.zeros((nz, ny, pitch), dtype=torch.float32, device="cuda")
        t[:, :, :nx] = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
        out.append(t)
    return out


def _call_twice(p, fields, pitch, flags, ek_ref, ep_ref, model=None):
    import torch
    lib = L.load()
    dev = _to_device(fields, pitch)
    ptrs = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in dev])
    cells = [None, None, None]
    if model is not None:
        mdev = _to_device(model, pitch)
        cells = [t.data_ptr() for t in mdev]
    lam = p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs)
    mu = p.rho * p.cs * p.cs
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.cpml_energy3d_noalloc(ptrs, p.nx, p.ny, p.nz, pitch, p.npoints_pml, lam, mu, p.rho,
                                       *cells, flags, out.data_ptr(), stream)
        assert st == 0, L.strerror(st)
        torch.cuda.synchronize()
        ek, ep = out.cpu().numpy()
        assert abs(ek - ek_ref) <= ENERGY_TOL * abs(ek_ref), (ek, ek_ref)
        assert abs(ep - ep_ref) <= ENERGY_TOL * abs(ep_ref), (ep, ep_ref)


@pytest.mark.parametrize("flags", [P.FLAG_ENERGY, P.FLAG_ENERGY | P.FLAG_EP_PHYSICAL])
def test_noalloc_energy_matches_solver_energy(flags):
    p, ek_ref, ep_ref, fields = _reference_energy_and_fields(flags)
    _call_twice(p, fields, p.nx, flags, ek_ref, ep_ref)


def test_noalloc_padded_pitch_matches_solver_energy():
    """Fields laid out with a row pitch of nx + 8 floats (the padding holds
    zeros the interior never reaches)."""
    p, ek_ref, ep_ref, fields = _reference_energy_and_fields(P.FLAG_ENERGY)
    _call_twice(p, fields, p.nx + 8, P.FLAG_ENERGY, ek_ref, ep_ref)


@pytest.mark.parametrize("pitch_pad", [0, 8])
def test_noalloc_per_cell_model_matches_solver_energy(pitch_pad):
    """A per-cell model (lambda, mu, rho device arrays in the fields' layout):
    the same model drives the handle's run, whose recorded energy uses the
    unaveraged per-cell values of the energy interior (3D:1131-1180)."""
    p0, _ = P.small_3d(n=(44, 38, 34), nstep=90)
    model = layered_3d(p0, seed=11)
    p, ek_ref, ep_ref, fields = _reference_energy_and_fields(P.FLAG_ENERGY, model=model)
    _call_twice(p, fields, p.nx + pitch_pad, P.FLAG_ENERGY, ek_ref, ep_ref, model=model)


def test_noalloc_rejects_too_many_planes():
    lib = L.load()
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    st = lib.cpml_energy3d_noalloc(ptrs, 8, 8, 8193, 8, 2, 1.0e9, 1.0e9, 2000.0,
                                   None, None, None, 0, 1, None)
    assert st == -9   # CPML_ERR_RANGE: the static scratch holds 8192 planes
