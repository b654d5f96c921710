"""GPU parity: libcpml (FP32 CUDA kernels for sm_103a, called through the C
ABI) against the FP64 oracle restatement of the reference programs.

Tolerances (relative L2, the reference's double-precision run as truth):
  seismograms, all receivers and components together   <= 1e-5
  energy curve Ek+Ep over all steps                     <= 1e-6
The FP32 rounding floor of the algorithm itself, measured with the oracle's
FP32 instantiation, is ~4e-6 on traces and ~1e-7 on energy for the 2000-step
2D runs, so these bounds leave room only for rounding-level differences.
"""
import numpy as np
import pytest

from seismic_cpml_gb300 import params as P
from seismic_cpml_gb300.lib import CpmlError
from seismic_cpml_gb300.solver import Solver
from oracle import oracle_c
from tests.models import layered_2d, layered_3d

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
ENERGY_TOL = 1e-6
# Whole-field comparisons: after the wave has left through the PML the fields
# hold small residuals whose FP32 rounding floor (oracle FP32 build vs FP64)
# reaches 1e-4 relative; a field passes at <= max(1e-5, 4 x that floor).
FIELD_TOL = 1e-5
FIELD_FLOOR_FACTOR = 4.0


def rl2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def traces(*comps):
    return np.concatenate([c for c in comps if c is not None])


def run_gpu(p, rec, model=None, nsteps=None, tuning=None):
    with Solver(p, rec, model=model, tuning=tuning) as s:
        s.run(nsteps)
        vx, vy, vz = s.seismograms()
        ek, ep = s.energy()
        names = ["vx", "vy", "sxx", "syy", "sxy"] if p.ndim == 2 else \
            ["vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"]
        fields = {n: s.field(n) for n in names}
        it, vmax = s.status()
    return dict(vx=vx, vy=vy, vz=vz, ek=ek, ep=ep, fields=fields, it=it, vmax=vmax)


def check(g, ref, fields=None, floor=None, trace_tol=TRACE_TOL, energy_tol=ENERGY_TOL):
    et = rl2(traces(g["vx"], g["vy"], g["vz"]), traces(ref.sisvx, ref.sisvy, ref.sisvz))
    ee = rl2(g["ek"] + g["ep"], ref.ek + ref.ep)
    assert et <= trace_tol, f"trace rel-L2 {et:.3e}"
    assert ee <= energy_tol, f"energy rel-L2 {ee:.3e}"
    if fields:
        for n, f in fields.items():
            ef = rl2(g["fields"][n], f)
            tol = FIELD_TOL
            if floor is not None:
                tol = max(tol, FIELD_FLOOR_FACTOR * rl2(floor[n], f))
            assert ef <= tol, f"field {n} rel-L2 {ef:.3e} > {tol:.3e}"
    return et, ee


CLUSTER_CASES = {"small": lambda: P.small_2d(), "small_tall": lambda: P.small_2d(nx=40, ny=300, nstep=200),
                 "reference_2d": lambda: (P.default_2d(), P.reference_receivers_2d(P.default_2d())),
                 "config_2d_plain": P.config_2d_plain}


@pytest.mark.parametrize("het", [False, True])
@pytest.mark.parametrize("case", list(CLUSTER_CASES))
def test_2d_cluster_kernel_is_bitwise_two_sweep(case, het):
    """The on-chip cluster kernel (the whole grid in the shared memory of one
    cluster, halo rows through distributed shared memory) gives bit-identical
    seismograms and fields to the two-sweep kernels, on grids whose bands
    hold the source, receivers, both y slabs and a short last band; its
    energy is summed per CTA (compensated FP32 sums over a few cells per
    thread) instead of one cell per thread and tile, equal to ~1e-8."""
    p, rec = CLUSTER_CASES[case]()
    if case in ("reference_2d", "config_2d_plain"):
        p.nstep = 600
    model = layered_2d(p, seed=8) if het else None
    a = run_gpu(p, rec, model, tuning=(4, 8, 32, 2))
    b = run_gpu(p, rec, model, tuning=(1, 8, 32, 2))
    for k in ("vx", "vy"):
        assert np.array_equal(a[k], b[k]), k
    for n in a["fields"]:
        assert np.array_equal(a["fields"][n], b["fields"][n]), n
    e_a, e_b = a["ek"] + a["ep"], b["ek"] + b["ep"]
    assert np.abs(e_a - e_b).max() <= 1e-7 * np.abs(e_b).max()
    assert a["it"] == b["it"] == p.nstep and np.abs(a["vx"]).max() > 0


@pytest.mark.parametrize("het", [False, True])
def test_2d_small(het):
    p, rec = P.small_2d()
    model = layered_2d(p, seed=3) if het else None
    kw = dict(lam=model[0], mu=model[1], rho=model[2]) if het else {}
    ref = oracle_c.run(p, rec=rec, keep_fields=True, **kw)
    ref32 = oracle_c.run(p, rec=rec, keep_fields=True, double=False, **kw)
    check(run_gpu(p, rec, model), ref, ref.fields, ref32.fields)


@pytest.mark.parametrize("het", [False, True])
@pytest.mark.parametrize("shape", [(48, 64, 300), (4000, 400, 120)], ids=["tile_per_cta", "tiles_per_cta"])
def test_2d_persistent_is_bitwise_two_sweep(het, shape):
    """The persistent 2D kernel (the steps of a chunk in one cooperative launch)
    gives bit-identical seismograms, energies and fields to the two-sweep
    kernels: on a grid with one tile per CTA, and on one (6250 tiles) larger
    than the resident grid, where each CTA takes several tiles. Chunks of 5,
    45 and 50 steps (IT_DISPLAY = 50) exercise several cached graphs."""
    nx, ny, nstep = shape
    p, rec = P.small_2d(nx=nx, ny=ny, nstep=nstep)
    model = layered_2d(p, seed=5) if het else None
    a = run_gpu(p, rec, model, tuning=(3, 8, 32, 2))
    b = run_gpu(p, rec, model, tuning=(1, 8, 32, 2))
    for k in ("vx", "vy", "ek", "ep"):
        assert np.array_equal(a[k], b[k]), k
    assert np.abs(a["vx"]).max() > 0 and a["ek"][-1] > 0
    for n in a["fields"]:
        assert np.array_equal(a["fields"][n], b["fields"][n]), n
    assert a["it"] == b["it"] == nstep and a["vmax"] == b["vmax"]


def test_2d_kernel_choice_and_launch_accounting():
    p, rec = P.small_2d()                            # 16 tiles: one resident wave
    with Solver(p, rec) as s:                        # automatic: two-sweep
        assert s.tuning()[0] == 1 and s.launches_per_step() == (2, 2)
    with Solver(p, rec, tuning=(4, 8, 32, 2)) as s:  # on request: the on-chip cluster kernel
        assert s.tuning()[0] == 4 and s.launches_per_step() == (0, 3)
    with Solver(p, rec, tuning=(3, 8, 32, 2)) as s:
        assert s.tuning()[0] == 3 and s.launches_per_step() == (0, 3)
    pb, recb = P.small_2d(nx=4000, ny=400, nstep=20)  # 6250 tiles: more than the resident CTAs
    with Solver(pb, recb) as s:                      # automatic: still two-sweep
        assert s.tuning()[0] == 1 and s.launches_per_step() == (2, 2)
    with Solver(pb, recb, tuning=(3, 8, 32, 2)) as s:
        assert s.tuning()[0] == 3 and s.launches_per_step() == (0, 3)
    with Solver(p, rec) as s:
        with pytest.raises(RuntimeError):
            s.set_tuning(2, 8, 32, 2)                # the fused kernel is 3D only
    p3, rec3 = P.small_3d()
    with Solver(p3, rec3) as s:
        with pytest.raises(RuntimeError):
            s.set_tuning(3, 8, 32, 2)                # the persistent kernel is 2D only
        with pytest.raises(RuntimeError):
            s.set_tuning(4, 8, 32, 2)                # so is the cluster kernel


def test_failed_replan_blocks_runs_until_a_valid_one():
    """A tuning request whose plan cannot be built (the cluster kernel on a
    grid too large for one cluster's shared memory) leaves the handle
    refusing to run (CPML_ERR_NOT_READY) instead of running a half-built
    plan; the next valid request restores it, with the same results as a
    handle that never failed."""
    p, rec = P.small_2d(nx=600, ny=600, nstep=40)
    with Solver(p, rec) as ref:
        ref.run()
        want = ref.seismograms()
    with Solver(p, rec) as s:
        with pytest.raises(CpmlError) as e:
            s.set_tuning(4, 8, 32, 2)
        assert e.value.status == -1                  # CPML_ERR_INVALID
        with pytest.raises(CpmlError) as e:
            s.run()
        assert e.value.status == -7                  # CPML_ERR_NOT_READY
        s.set_tuning(1, 8, 32, 2)
        s.run()
        got = s.seismograms()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


TUNINGS_3D = [(1, 8, 32, 2), (2, 16, 32, 2), (2, 8, 7, 2), (2, 16, 5, 2), (2, 8, 9, 2), (2, 8, 11, 2)]


@pytest.mark.parametrize("het", [False, True])
@pytest.mark.parametrize("tuning", TUNINGS_3D, ids=["two_sweep", "f16z32", "f8z7", "f16z5", "f8z9", "f8z11"])
def test_3d_small(het, tuning):
    p, rec = P.small_3d()
    model = layered_3d(p, seed=5) if het else None
    kw = dict(lam=model[0], mu=model[1], rho=model[2]) if het else {}
    ref = oracle_c.run(p, rec=rec, keep_fields=True, **kw)
    ref32 = oracle_c.run(p, rec=rec, keep_fields=True, double=False, **kw)
    g = run_gpu(p, rec, model, tuning=tuning)
    check(g, ref, ref.fields, ref32.fields)


def test_2d_reference_default(golden):
    """The 2D program as shipped (2D:138-218): 101 x 641, 2000 steps, first
    derivative of a Gaussian at (80, 428), 135 degrees."""
    g0 = golden("ref2d_default")
    p = P.default_2d()
    rec = [tuple(r) for r in g0["rec"]]
    g = run_gpu(p, rec)

    class R:
        sisvx, sisvy, sisvz, ek, ep = g0["sisvx"], g0["sisvy"], None, g0["ek"], g0["ep"]
    check(g, R)
    # reference prints max|v| at it = 2000 (2D:718); same value within FP32
    assert abs(g["vmax"] - g0["vmax"][-1]) <= 1e-4 * g0["vmax"][-1]


def test_2d_plain_config(golden):
    """2D plain workload: Ricker at the centre, 45 degrees, no PML on top."""
    g0 = golden("config_2d_plain")
    p, rec = P.config_2d_plain()
    g = run_gpu(p, rec)

    class R:
        sisvx, sisvy, sisvz, ek, ep = g0["sisvx"], g0["sisvy"], None, g0["ek"], g0["ep"]
    check(g, R)


def test_small_het_fixtures(golden):
    for name, mk in (("small2d_het", P.small_2d), ("small3d_het", P.small_3d)):
        g0 = golden(name)
        p, _ = mk()
        rec = [tuple(r) for r in g0["rec"]]
        g = run_gpu(p, rec, model=(g0["lam"], g0["mu"], g0["rho"]))

        class R:
            sisvx, sisvy, ek, ep = g0["sisvx"], g0["sisvy"], g0["ek"], g0["ep"]
            sisvz = g0.get("sisvz")
        check(g, R)


def test_3d_reference_quirk_and_physical_energy():
    """Ep of the 3D reference counts eps_yy*sigma_yy twice and drops the zz
    term (3D:1170-1171); CPML_FLAG_EP_PHYSICAL switches to the textbook sum."""
    p, rec = P.small_3d(nstep=80)
    for flags in (P.FLAG_ENERGY, P.FLAG_ENERGY | P.FLAG_EP_PHYSICAL):
        q = p.copy()
        q.flags = flags
        ref = oracle_c.run(q, rec=rec)
        check(run_gpu(q, rec), ref)


@pytest.mark.parametrize("tuning", [(1, 8, 32, 2), (2, 16, 32, 2), (2, 8, 12, 2), (2, 8, 20, 2)])
def test_3d_mid_size_vs_oracle(tuning):
    """A 3D case with more than one tile in every direction and a z extent
    spanning several z-chunks, 300 steps."""
    p, rec = P.small_3d(n=(70, 52, 44), nstep=300)
    p.npoints_pml = 10
    ref = oracle_c.run(p, rec=rec)
    check(run_gpu(p, rec, tuning=tuning), ref)


INTERIOR_TUNINGS = [(2, 8, 16, 2), (2, 8, 48, 2), (2, 16, 24, 2), (2, 16, 64, 2)]


@pytest.mark.parametrize("tuning", INTERIOR_TUNINGS, ids=["f8z16", "f8z48", "f16z24", "f16z64"])
def test_3d_interior_class_vs_oracle(tuning):
    """The lean interior kernel (homogeneous model: the class and the model
    the 3D plain workload runs) against the FP64 oracle. At 108 x 100 x 96
    with a 10-point C-PML the grid has interior tiles in x, y and z, so all
    five step kernels launch (interior + X, Y, Z and mixed general classes);
    the source and a receiver line lie inside interior tiles. 400 steps, the
    wave crosses the grid and leaves through the C-PML (3D:836-1180)."""
    p, _ = P.small_3d(n=(108, 100, 96), nstep=400)
    p.npoints_pml = 10
    c = (p.nx // 2, p.ny // 2 + 1, p.nz // 2)
    rec = [(i, c[1], c[2]) for i in range(12, p.nx - 10, 7)] + \
          [(c[0], j, c[2] + 3) for j in range(14, p.ny - 10, 9)] + [(7, 8, 9), (p.nx - 7, p.ny - 6, c[2] + 2)]
    ref = oracle_c.run(p, rec=rec, keep_fields=True)
    ref32 = oracle_c.run(p, rec=rec, keep_fields=True, double=False)
    with Solver(p, rec, tuning=tuning) as s:
        assert s.tuning()[0] == 2
        assert s.launches_per_step()[0] == 5, s.launches_per_step()   # interior items exist
        s.run()
        vx, vy, vz = s.seismograms()
        ek, ep = s.energy()
        fields = {n: s.field(n) for n in ref.fields}
    g = dict(vx=vx, vy=vy, vz=vz, ek=ek, ep=ep, fields=fields)
    et, ee = check(g, ref, ref.fields, ref32.fields)
    print(f"interior class {tuning}: trace rel-L2 {et:.3e}, energy rel-L2 {ee:.3e}")


@pytest.mark.parametrize("tuning", [None, (2, 8, 48, 2), (2, 16, 32, 2)], ids=["auto", "f8z48", "f16z32"])
def test_3d_plain_config_full_size_vs_fixture(golden, tuning):
    """The 3D plain workload itself (276^3, 2500 steps, 64 receivers: what the
    benchmark times) against the FP64 oracle's run of the same parameters
    (tests/golden/config_3d_plain.npz): traces within 1e-5 and the energy
    curve within 1e-6 relative L2 after every one of the 2500 steps."""
    g0 = golden("config_3d_plain")
    p, rec = P.config_3d_plain()
    assert [tuple(r) for r in g0["rec"]] == [tuple(r) for r in rec]
    with Solver(p, rec, tuning=tuning) as s:
        assert s.tuning()[0] == 2                                    # the fused one-sweep step
        assert s.launches_per_step()[0] == 5, s.launches_per_step()
        s.run()
        vx, vy, vz = s.seismograms()
        ek, ep = s.energy()

    class R:
        sisvx, sisvy, sisvz, ek, ep = g0["sisvx"], g0["sisvy"], g0["sisvz"], g0["ek"], g0["ep"]
    et, ee = check(dict(vx=vx, vy=vy, vz=vz, ek=ek, ep=ep), R)
    print(f"3d_plain full size {tuning}: trace rel-L2 {et:.3e}, energy rel-L2 {ee:.3e}")


def test_fused_is_the_default_3d_step():
    """The fused step must be available (its tensor-map encoder found through
    the runtime's versioned driver entry point): a 3D handle that silently took
    the two-sweep kernels would move 108 instead of 72 B per cell."""
    p, rec = P.small_3d()
    with Solver(p, rec) as s:
        assert s.tuning()[0] == 2


def test_fused_equals_two_sweep_traces():
    """Both 3D step kernels agree with each other to FP32 rounding."""
    p, rec = P.small_3d(n=(40, 36, 30), nstep=150)
    a = run_gpu(p, rec, tuning=(1, 8, 32, 2))
    b = run_gpu(p, rec, tuning=(2, 16, 8, 2))
    assert rl2(traces(b["vx"], b["vy"], b["vz"]), traces(a["vx"], a["vy"], a["vz"])) < 2e-6


def test_chunked_run_equals_single_run():
    """Running in pieces (different chunk lengths and CUDA graphs) gives the
    bitwise-identical result of one call."""
    p, rec = P.small_3d(nstep=150)
    a = run_gpu(p, rec)
    with Solver(p, rec) as s:
        for n in (3, 1, 40, 6, 100):
            s.run(n)
        vx, vy, vz = s.seismograms()
        ek, ep = s.energy()
    assert np.array_equal(vx, a["vx"]) and np.array_equal(vz, a["vz"])
    assert np.array_equal(ek, a["ek"]) and np.array_equal(ep, a["ep"])


def test_determinism_and_reset():
    p, rec = P.small_2d(nstep=120)
    with Solver(p, rec) as s:
        s.run()
        x1 = s.seismograms()[0].copy()
        e1 = s.energy()[0].copy()
        s.reset()
        s.run()
        assert np.array_equal(s.seismograms()[0], x1)
        assert np.array_equal(s.energy()[0], e1)


def test_linearity_in_source_amplitude():
    """The scheme is linear: doubling `factor` doubles every trace (a
    size-independent property, checked on the full 276^3 plain 3D grid)."""
    p, rec = P.config_3d_plain(nstep=60)
    a = run_gpu(p, rec)
    q = p.copy()
    q.factor = 2.0 * p.factor
    b = run_gpu(q, rec)
    assert rl2(b["vx"], 2.0 * a["vx"]) < 1e-6
    assert rl2(b["ek"], 4.0 * a["ek"]) < 1e-6


def test_unstable_is_reported():
    """A NaN planted in the wavefield is caught at the next display step and
    reported as CPML_ERR_UNSTABLE (2D:724 stops there)."""
    from seismic_cpml_gb300.lib import CpmlError
    p, rec = P.small_2d(nstep=120)
    with Solver(p, rec) as s:
        s.run(10)
        vx = s.field("vx")
        vx[30, 20] = np.nan
        s.set_field("vx", vx)
        with pytest.raises(CpmlError) as e:
            s.run(60)
        assert e.value.status == -4
        it, _ = s.status()
        assert it == 50   # stopped at the display step (it_display = 50)


def test_plane_and_field_agree():
    p, rec = P.small_3d(nstep=40)
    with Solver(p, rec) as s:
        s.run()
        f = s.field("vy")
        assert np.array_equal(s.plane("vy", 2, 7), f[6])
        assert np.array_equal(s.plane("vy", 1, 5), f[:, 4, :])
        assert np.array_equal(s.plane("vy", 0, 9), f[:, :, 8])


def test_autotune_picks_a_candidate_and_keeps_results_exact(tmp_path):
    """The autotuner leaves the handle reset on the fastest shape; results
    under the chosen shape still match the oracle; the cache file round-trips."""
    p, rec = P.small_3d(n=(70, 52, 44), nstep=120)
    cache = str(tmp_path / "tune.txt")
    with Solver(p, rec) as s:
        best = s.autotune(trial_steps=8, cache_path=cache)
        assert best["kernel"] in (1, 2) and best["ms_per_step"] > 0
        assert s.status()[0] == 0
        s.run()
        vx, vy, vz = s.seismograms()
    ref = oracle_c.run(p, rec=rec)
    assert rl2(traces(vx, vy, vz), traces(ref.sisvx, ref.sisvy, ref.sisvz)) <= TRACE_TOL
    assert open(cache).read().split()[:4] == ["3", "70", "52", "44"]
    with Solver(p, rec) as s2:   # second handle of the same class: served from the cache
        again = s2.autotune(trial_steps=8, cache_path=cache)
        assert again == best


def test_large_config_generator_at_reduced_size_vs_oracle():
    """The 820^3 heterogeneous workload's parameters and model generator at
    140^3 (120^3 interior, same DELTA, DELTAT, source, receiver-grid layout):
    traces and energy against the FP64 oracle."""
    from seismic_cpml_gb300.earth import layered_model_3d_device
    p, rec = P.config_3d_large(n_interior=120, nstep=150, nrec_side=11)
    lam, mu, rho = (t.cpu().numpy() for t in layered_model_3d_device((p.nz, p.ny, p.nx), radius=(3.0, 12.0)))
    g = run_gpu(p, rec, model=(lam, mu, rho))
    ref = oracle_c.run(p, rec=rec, lam=lam, mu=mu, rho=rho)
    check(g, ref)


def test_concurrent_autotune_of_two_handles_shares_one_cache(tmp_path):
    """Handles are independent: two threads autotune two handles of one shape
    class at once (ctypes releases the GIL in the calls), sharing the process
    cache and one cache file; both get a valid choice and the file stays
    well-formed."""
    import threading
    p, rec = P.small_3d(n=(40, 36, 36), nstep=60)
    cache = str(tmp_path / "tune.txt")
    res, err = [None, None], []

    def work(k):
        try:
            with Solver(p, rec) as s:
                res[k] = s.autotune(trial_steps=4, cache_path=cache)
                s.run()
        except Exception as e:   # surfaced below: a thread's exception does not propagate
            err.append(e)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not err, err
    assert all(r is not None and r["kernel"] in (1, 2) and r["ms_per_step"] > 0 for r in res)
    lines = open(cache).read().splitlines()
    assert 1 <= len(lines) <= 2 and all(len(ln.split()) == 12 for ln in lines)


def test_autotune_2d_times_both_kernels_and_keeps_results_exact():
    p, rec = P.small_2d(nx=1200, ny=900, nstep=60)   # 4275 tiles: both 2D kernels are candidates
    with Solver(p, rec) as s:
        best = s.autotune(trial_steps=8)
        assert best["kernel"] in (1, 3, 4) and best["ms_per_step"] > 0
        assert s.tuning()[0] == best["kernel"] and s.status()[0] == 0
        s.run()
        vx, vy, _ = s.seismograms()
    with Solver(p, rec, tuning=(1, 8, 32, 2)) as t:
        t.run()
        tx, ty, _ = t.seismograms()
    assert np.array_equal(vx, tx) and np.array_equal(vy, ty)


def test_launch_accounting():
    p, rec = P.small_3d()
    with Solver(p, rec, tuning=(2, 8, 16, 2)) as s:
        k, c = s.launches_per_step()
        assert 2 <= k <= 5 and c == 2
    with Solver(p, rec, tuning=(1, 8, 16, 2)) as s:
        assert s.launches_per_step() == (2, 2)
