"""CPU checks of the oracle (the FP64 restatements of the reference programs).

The oracle is pinned to the reference's own outputs in tests/test_ref_pin.py.
Here it is held by (1) two independent restatements that must agree, C++
(oracle/cpml_oracle.cpp) and numpy (oracle/oracle_np.py); (2) the committed
golden fixtures (tests/golden/, made by make_golden.py); (3) physical
properties the reference's own diagnostics rely on (energy decay in the
C-PML, 2D:741-777; source wavelet shapes, 2D:644-654).
"""
import math

import numpy as np
import pytest

from oracle import oracle_c, oracle_np
from seismic_cpml_gb300 import params as P
from tests.models import layered_2d, layered_3d


def rl2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("het", [False, True])
def test_two_restatements_agree(ndim, het):
    p, rec = (P.small_2d(nstep=150) if ndim == 2 else P.small_3d(nstep=60))
    model = None
    if het:
        model = layered_2d(p, seed=9) if ndim == 2 else layered_3d(p, seed=9)
    kw = {} if model is None else dict(lam=model[0], mu=model[1], rho=model[2])
    a = oracle_c.run(p, rec=rec, keep_fields=True, **kw)
    b = (oracle_np.run2d if ndim == 2 else oracle_np.run3d)(p, rec=rec, keep_fields=True, **kw)
    for name, f in b.fields.items():
        assert np.array_equal(a.fields[name], f), name       # identical loop nests, same rounding
    assert np.array_equal(a.sisvx, b.sisvx) and np.array_equal(a.sisvy, b.sisvy)
    assert np.allclose(a.ek, b.ek, rtol=1e-12, atol=0) and np.allclose(a.ep, b.ep, rtol=1e-12, atol=0)


@pytest.mark.parametrize("program", ["fourth_order", "fourth_order_het", "split_pml"])
def test_two_restatements_agree_on_the_other_2d_programs(program):
    """seismic_CPML_2D_isotropic_fourth_order.f90 and
    seismic_PML_Collino_2D_isotropic.f90: the C++ restatement (ghost reads
    through a bounds test; split parts as separate arrays) and the numpy one
    (arrays held with the reference's ghost layer; sliced updates) agree."""
    p, rec = P.small_2d(nstep=150)
    kw = {}
    if program.startswith("fourth"):
        p.order = 4
        p.deltat = 1.0e-3
        if program.endswith("het"):
            m = layered_2d(p, seed=4)
            kw = dict(lam=m[0], mu=m[1], rho=m[2])
        b = oracle_np.run2d4(p, rec=rec, keep_fields=True, **kw)
    else:
        p.scheme = P.SCHEME_SPLIT
        b = oracle_np.run_split(p, rec=rec, keep_fields=True)
    a = oracle_c.run(p, rec=rec, keep_fields=True, **kw)
    for name, f in b.fields.items():
        assert np.array_equal(a.fields[name], f), name
    assert np.array_equal(a.sisvx, b.sisvx) and np.array_equal(a.sisvy, b.sisvy)
    assert np.abs(a.sisvx).max() > 0
    assert np.allclose(a.ek, b.ek, rtol=1e-12, atol=0) and np.allclose(a.ep, b.ep, rtol=1e-12, atol=0)


def test_fourth_order_program_details():
    """The fourth-order program's y profile starts its high-side C-PML one
    cell further out (2D4:401) and its x profile does not; a split-field
    handle refuses a per-cell model."""
    p = P.default_2d_fourth()
    q = P.default_2d()
    y4, y2 = oracle_c.profile(p, 1), oracle_c.profile(q, 1)
    x4, x2 = oracle_c.profile(p, 0), oracle_c.profile(q, 0)
    assert np.array_equal(x4["d"], x2["d"])
    assert np.array_equal(y4["d"][:100], y2["d"][:100])
    assert not np.array_equal(y4["d"][-12:], y2["d"][-12:])
    n = p.ny
    assert y4["d"][n - 1] < y2["d"][n - 1] and y4["d"][n - 10] == 0.0 < y2["d"][n - 10]
    s = P.default_2d_split()
    s.nx, s.ny, s.nstep = 30, 30, 2
    s.isource, s.jsource = 15, 15
    with pytest.raises(RuntimeError):
        oracle_c.run(s, lam=np.ones((30, 30)))


def test_restatements_agree_on_reference_flags():
    """3D energy quirk (3D:1170-1171) and its physical variant, both oracles."""
    p, rec = P.small_3d(nstep=40)
    for flags in (P.FLAG_ENERGY, P.FLAG_ENERGY | P.FLAG_EP_PHYSICAL):
        q = p.copy()
        q.flags = flags
        a = oracle_c.run(q, rec=rec)
        b = oracle_np.run3d(q, rec=rec)
        assert np.allclose(a.ep, b.ep, rtol=1e-12)
    a = oracle_c.run(p, rec=rec)
    q = p.copy()
    q.flags = P.FLAG_ENERGY | P.FLAG_EP_PHYSICAL
    b = oracle_c.run(q, rec=rec)
    assert not np.allclose(a.ep, b.ep)        # the quirk changes Ep
    assert np.array_equal(a.ek, b.ek)         # but not Ek


@pytest.mark.parametrize("name", ["ref2d_default", "config_2d_plain", "small2d_het", "small3d_hom",
                                  "small3d_het"])
def test_oracle_matches_golden(golden, name):
    g = golden(name)
    mk = {"ref2d_default": lambda: (P.default_2d(), None), "config_2d_plain": P.config_2d_plain,
          "small2d_het": P.small_2d, "small3d_hom": P.small_3d, "small3d_het": P.small_3d}[name]
    p, _ = mk()
    rec = [tuple(r) for r in g["rec"]]
    kw = {}
    if "lam" in g:
        kw = dict(lam=g["lam"], mu=g["mu"], rho=g["rho"])
    r = oracle_c.run(p, rec=rec, **kw)
    assert rl2(r.sisvx, g["sisvx"]) < 1e-12 and rl2(r.sisvy, g["sisvy"]) < 1e-12
    assert rl2(r.ek + r.ep, g["ek"] + g["ep"]) < 1e-12


def test_fp32_floor_is_below_the_tolerance():
    """The algorithm in FP32 (oracle's float build) stays within the parity
    bounds against FP64: this is the floor any FP32 implementation inherits."""
    p, rec = P.small_2d()
    a = oracle_c.run(p, rec=rec)
    b = oracle_c.run(p, rec=rec, double=False)
    assert rl2(np.concatenate([b.sisvx, b.sisvy]), np.concatenate([a.sisvx, a.sisvy])) < 1e-5
    assert rl2(b.ek + b.ep, a.ek + a.ep) < 1e-6


def test_energy_decays_in_the_pml(golden):
    """The C-PML absorbs: after the wave has left, total energy falls far
    below its peak (the reference's energy.dat check, 2D:741-762)."""
    g = golden("ref2d_default")
    e = g["ek"] + g["ep"]
    assert e.max() > 0
    assert e[-1] < 1e-3 * e.max()


def test_source_wavelets():
    p = P.default_2d()
    a = math.pi ** 2 * p.f0 ** 2
    it0 = int(round(p.t0 / p.deltat)) + 1   # step whose time is closest to t0
    p.stf = P.STF_RICKER
    assert abs(oracle_c.source_term(p, it0) - p.factor) < 1e-3 * p.factor
    p.stf = P.STF_GAUSSIAN
    assert abs(oracle_c.source_term(p, it0) - p.factor) < 1e-3 * p.factor
    p.stf = P.STF_DGAUSSIAN
    t = (it0 - 1) * p.deltat - p.t0
    assert abs(oracle_c.source_term(p, it0) - (-p.factor * 2 * a * t * math.exp(-a * t * t))) < 1e-6


def test_profiles_follow_the_reference_formulas():
    p = P.default_2d()
    for axis, n in ((0, p.nx), (1, p.ny)):
        pr = oracle_c.profile(p, axis)
        prn = oracle_np.pml_profile(n, 10.0, 10, True, True, p.cp, p.f0, p.deltat)
        for k in pr:
            assert np.array_equal(pr[k], prn[k]), k
        d0 = -(2.0 + 1) * p.cp * math.log(0.001) / (2.0 * 100.0)     # 2D:296
        assert abs(pr["d"][0] - d0) < 1e-9 * d0
        # a is nonzero only inside the PML: NPML points per side, and one
        # more half point on the high side
        nzf = np.nonzero(pr["a"])[0]
        nzh = np.nonzero(pr["a_half"])[0]
        assert list(nzf) == list(range(0, 10)) + list(range(n - 10, n))
        assert list(nzh) == list(range(0, 10)) + list(range(n - 11, n))
        assert np.all(pr["b"] > 0) and np.all(pr["b"] <= 1)
        assert np.all(pr["K"] == 1.0)          # K_MAX_PML = 1 (2D:217)


def test_profile_disabled_side_has_no_pml():
    p = P.default_2d()
    p.use_pml[3] = 0                          # no PML at y max
    pr = oracle_c.profile(p, 1)
    assert np.all(pr["a"][p.ny // 2:] == 0) and np.all(pr["a_half"][p.ny // 2:] == 0)


def test_nearest_gridpoint_rules():
    rng = np.random.default_rng(0)
    for _ in range(20):
        x, y = rng.uniform(-20, 1020), rng.uniform(-20, 6420)
        assert P.nearest_gridpoint(101, 641, 10.0, 10.0, x, y) == \
            oracle_np.nearest_gridpoint(101, 641, 10.0, 10.0, x, y)
    # exact ties go to the first point in i-fastest order (strict < in 2D:500)
    assert oracle_np.nearest_gridpoint(101, 641, 10.0, 10.0, 15.0, 25.0) == (2, 3)
    assert P.reference_receivers_2d(P.default_2d()) == [(70, 231), (80, 31)]


def test_3d_source_plane_semantics():
    """The 3D program injects on the cut plane k = NZ/2 and records there
    (3D:1080, 1126); the default parameter block puts ksource there."""
    p = P.default_3d()
    assert p.ksource == p.nz // 2
    q, rec = P.small_3d(nstep=30)
    r = oracle_c.run(q, rec=[(q.isource, q.jsource, q.ksource)])
    assert np.abs(r.sisvx).max() > 0
