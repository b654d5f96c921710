"""The oracle against the reference programs themselves (CPU).

tests/golden/refpin_*.npz hold what the reference programs compute. Each
program's own Fortran statements were translated to C by oracle/ref_f90c.py,
compiled with gcc, and run, the 3D program on 2, 4 and 12 emulated MPI ranks
(tests/golden/make_ref_vectors.py). Here the C++ oracle runs the same
parameters and must reproduce those outputs:
  - bit for bit: fields, seismograms, and the 2D energies, which the oracle
    sums in the programs' order;
  - the 3D total energy within 1e-14 relative on the small grids and 1e-12
    on the 276^3 grid. The program reduces its per-rank sums over MPI
    (3D:1179), while the oracle sums plane partials in z order.
The full-size 3D plain fixture (config_3d_plain.npz, made by the oracle) is
checked against the reference's run of the same workload. So the GPU tests,
which compare the product with the oracle, are anchored to the reference.

The last tests check the translator itself on a small program written for
this file, and, where the reference sources exist, regenerate two of the
vectors from them.
"""
from __future__ import annotations

import hashlib
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle_c, oracle_np, ref_f90c
from seismic_cpml_gb300 import params as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_DIR = ref_f90c.DEFAULT_REF_DIR
SMALL = ["refpin_2d_small", "refpin_2d4_small", "refpin_pml2d_small", "refpin_3d_2ranks",
         "refpin_3d_4ranks", "refpin_2d_profiles", "refpin_2d4_profiles", "refpin_3d_profiles",
         "refpin_2d_het", "refpin_2d4_het"]
SHIPPED = ["refpin_2d_shipped", "refpin_2d4_shipped", "refpin_pml2d_shipped", "refpin_2d_plain"]
STF = {"ricker": P.STF_RICKER, "gaussian": P.STF_GAUSSIAN, "program default": P.STF_DGAUSSIAN}


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def params_of(fx):
    """CpmlParams for the run a fixture records, from the parameter values
    the program itself evaluated."""
    prog = str(fx["program"])
    g = lambda k: fx["p_" + k].item()  # noqa: E731
    three_d = "3D" in prog
    if "fourth" in prog:
        p = P.default_2d_fourth()
    elif "Collino" in prog:
        p = P.default_2d_split()
    elif three_d:
        p = P.default_3d()
    else:
        p = P.default_2d()
    p.nx, p.ny, p.nstep, p.npoints_pml = g("nx"), g("ny"), g("nstep"), g("npoints_pml")
    p.cp, p.cs, p.deltat, p.f0, p.t0, p.factor = (g(k) for k in ("cp", "cs", "deltat", "f0",
                                                                  "t0", "factor"))
    p.isource, p.jsource, p.angle_force = g("isource"), g("jsource"), g("angle_force")
    p.it_display = g("it_display")
    p.stf = STF[str(fx["stf"])]
    if "Collino" in prog:
        p.deltax = p.deltay = g("h")
        p.rho = g("rho")
    else:
        p.deltax, p.deltay = g("deltax"), g("deltay")
        p.rho = g("rho") if three_d else g("density")
        faces = ["xmin", "xmax", "ymin", "ymax"] + (["zmin", "zmax"] if three_d else [])
        p.use_pml[:] = [int(g("use_pml_" + f)) for f in faces] + [0] * (6 - len(faces))
    if "p_npower" in fx:      # the C-PML profile parameters (the split program has none)
        p.npower, p.k_max_pml = g("npower"), g("k_max_pml")
        amax = g("alpha_max_pml")
        # the programs' own value 2 pi (f0 / 2) is the oracle's default (-1)
        p.alpha_max_pml = -1.0 if amax == 2.0 * math.pi * (p.f0 / 2.0) else amax
    rec = [tuple(int(v) for v in r) for r in fx["rec"]]
    if three_d:
        p.nz, p.deltaz = g("nz"), g("deltaz")
        p.ksource = p.nz // 2                      # the cut plane, 3D:346, 1080
        rec = [(i, j, p.nz // 2) for i, j in rec]  # recorded on the cut plane, 3D:1126
    return p, rec


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def check(fx, r):
    assert np.array_equal(r.sisvx, fx["sisvx"]), "vx seismograms differ"
    assert np.array_equal(r.sisvy, fx["sisvy"]), "vy seismograms differ"
    if "energy" in fx:
        e = r.ek + r.ep
        rel = np.abs(e - fx["energy"]).max() / np.abs(fx["energy"]).max()
        assert rel <= 1e-14, rel
    else:
        assert np.array_equal(r.ek, fx["ek"]), "kinetic energy differs"
        assert np.array_equal(r.ep, fx["ep"]), "potential energy differs"
    for k in fx:
        if k.startswith("f_"):
            assert np.array_equal(r.fields[k[2:]], fx[k]), f"field {k[2:]} differs"
        if k.startswith("sha_"):
            assert digest(r.fields[k[4:]]) == str(fx[k]), f"field {k[4:]} differs"


def model_of(fx):
    """The per-cell model (lambda, mu, rho) a fixture's run read in, or None."""
    return (fx["lam"], fx["mu"], fx["rho"]) if "lam" in fx else None


@pytest.mark.parametrize("name", SMALL + SHIPPED)
def test_oracle_reproduces_reference(name):
    fx = load(name)
    p, rec = params_of(fx)
    m = model_of(fx)
    kw = dict(lam=m[0], mu=m[1], rho=m[2]) if m else {}
    check(fx, oracle_c.run(p, rec=rec, keep_fields=True, **kw))


@pytest.mark.parametrize("name", ["refpin_2d_small", "refpin_2d4_small", "refpin_pml2d_small",
                                  "refpin_3d_2ranks", "refpin_3d_4ranks", "refpin_2d_het",
                                  "refpin_2d4_het", "refpin_2d_profiles", "refpin_2d4_profiles",
                                  "refpin_3d_profiles"])
def test_numpy_restatement_reproduces_reference(name):
    fx = load(name)
    p, rec = params_of(fx)
    run = oracle_np.run3d if p.ndim == 3 else (
        oracle_np.run2d4 if p.order == 4 else
        oracle_np.run_split if p.scheme == P.SCHEME_SPLIT else oracle_np.run2d)
    m = model_of(fx)
    r = run(p, rec=rec, **(dict(lam=m[0], mu=m[1], rho=m[2]) if m else {}))
    assert np.array_equal(r.sisvx, fx["sisvx"])
    assert np.array_equal(r.sisvy, fx["sisvy"])
    e_ref = fx["energy"] if "energy" in fx else fx["ek"] + fx["ep"]
    assert np.abs(r.ek + r.ep - e_ref).max() <= 1e-14 * np.abs(e_ref).max()


def test_shipped_fixtures_are_the_reference():
    """The oracle's fixtures of the programs as shipped and of the 2D plain
    workload (used by the GPU tests) equal the reference's own outputs."""
    for ours, ref in (("ref2d_default", "refpin_2d_shipped"), ("ref2d_fourth", "refpin_2d4_shipped"),
                      ("ref2d_split", "refpin_pml2d_shipped"), ("config_2d_plain", "refpin_2d_plain")):
        a, b = load(ours), load(ref)
        assert np.array_equal(a["rec"][:, :2], b["rec"]), ours
        for k in ("sisvx", "sisvy", "ek", "ep"):
            assert np.array_equal(a[k], b[k]), (ours, k)


def test_full_size_3d_plain_fixture_is_the_reference():
    """config_3d_plain.npz (276^3, 2500 steps, 64 receivers; the fixture the
    GPU run of the benchmarked kernels is compared with) against the
    reference's own run of that workload on 12 ranks."""
    a, b = load("config_3d_plain"), load("refpin_3d_plain_full")
    assert np.array_equal(a["rec"][:, :2], b["rec"])
    assert int(b["p_nx"]) == int(b["p_ny"]) == int(b["p_nz"]) == 276
    assert int(b["p_nstep"]) == 2500 and str(b["stf"]) == "ricker"
    for k in ("sisvx", "sisvy"):
        if k in b:
            assert np.array_equal(a[k], b[k]), k
        else:
            assert digest(a[k]) == str(b["sha_" + k]), k
    # 16.7 M interior cells summed in another order (12 per-rank sums and an
    # MPI reduction against per-plane partials): 8e-14 measured
    e = a["ek"] + a["ep"]
    assert np.abs(e - b["energy"]).max() <= 1e-12 * np.abs(b["energy"]).max()


# ---------------------------------------------------------------------------
# the translator itself
# ---------------------------------------------------------------------------
SELF_TEST = """\
program selftest
  implicit none
  include 'mpif.h'
  integer, parameter :: N = 5, M = 2 * N / 3 + 1
  double precision, parameter :: X = 1.d0 / 3.d0, BIG = 1.d+30
  double precision, dimension(0:N,2) :: a
  double precision, dimension(4) :: buf
  double precision :: s, mx, e, part, tot
  real :: r
  integer :: i, k, cnt, rank, nprocs, code, left, right
  call MPI_INIT(code)
  call MPI_COMM_SIZE(MPI_COMM_WORLD, nprocs, code)
  call MPI_COMM_RANK(MPI_COMM_WORLD, rank, code)
  do i = 0, N
    a(i,1) = dble(i) * X - 2.d0**2  ! comment
    a(i,2) = - a(i,1)**2
  enddo
  s = sum(a(1:N,1))
  mx = maxval(abs(a))
  r = 0.1
  e = r
  k = -7 / 2
  cnt = 0
  do i = 10, 1, -3
    cnt = cnt + 1
  end do
  if (k == -3 .and. .not. (cnt /= 4)) then
    a(0,1) = BIG
  else if (k > 0) then
    a(0,1) = 1
  else
    a(0,1) = 2
  endif
  a(:,2) = a(:,2) / 2.d0
  left = rank - 1
  right = rank + 1
  if (rank == 0) left = MPI_PROC_NULL
  if (rank == nprocs - 1) right = MPI_PROC_NULL
  buf(:) = 0.d0
  buf(1:2) = dble(rank + 1)
  call MPI_SENDRECV(buf(1:2),2,MPI_DOUBLE_PRECISION,right,0,buf(3:4),2, &
         MPI_DOUBLE_PRECISION,left,0,MPI_COMM_WORLD,i,code)
  part = dble(rank + 1) / 7.d0
  call MPI_REDUCE(part + 0.d0,tot,1,MPI_DOUBLE_PRECISION,MPI_SUM,0,MPI_COMM_WORLD,code)
  call MPI_FINALIZE(code)
end program selftest
"""


@pytest.fixture(scope="module")
def selftest(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    d = tmp_path_factory.mktemp("ref")
    src = d / "selftest.f90"
    src.write_text(SELF_TEST)
    code, manifest = ref_f90c.translate_file(str(src), {"N": 6}, ["a", "s", "mx", "e", "k", "cnt",
                                                                    "m", "buf", "tot"])
    c = d / "selftest.c"
    c.write_text(code)
    exe = d / "selftest"
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-w", "-o", str(exe), str(c),
                    ref_f90c.MPI_RUNTIME, "-lm", "-lpthread"], check=True)
    return ref_f90c.RefProgram(str(exe), manifest)


def test_translator_semantics(selftest):
    d = selftest.run(nprocs=1)[0]
    n = 6                                              # the overridden parameter
    assert int(d["m"]) == 2 * n // 3 + 1
    x = 1.0 / 3.0
    col = np.array([float(i) * x - 4.0 for i in range(n + 1)])
    s = 0.0
    for v in col[1:]:                                  # SUM in element order
        s = s + v
    assert d["s"] == s
    assert d["mx"] == max(np.abs(col).max(), (col ** 2).max())
    assert d["e"] == float(np.float32(0.1))            # 0.1 is a single-precision literal
    assert int(d["k"]) == -3                           # integer division truncates
    assert int(d["cnt"]) == 4                          # 10, 7, 4, 1
    assert d["a"][0, 0] == 1.0e30                      # the IF branch taken
    assert np.array_equal(d["a"][1:, 1], -(col[1:] ** 2) / 2.0)
    assert d["a"].shape == (n + 1, 2)


def test_mpi_stand_in(selftest):
    out = selftest.run(nprocs=3)
    for r, d in enumerate(out):
        assert list(d["buf"][:2]) == [r + 1.0] * 2
        assert list(d["buf"][2:]) == ([0.0, 0.0] if r == 0 else [float(r)] * 2)
    tot = 0.0
    for r in range(3):                                 # rank order
        tot = tot + (r + 1) / 7.0
    assert out[0]["tot"] == tot


def test_translator_rejects_what_it_does_not_know(tmp_path):
    src = tmp_path / "bad.f90"
    src.write_text("program bad\n  implicit none\n  integer :: i\n  i = 1\n  goto 10\n"
                   "end program bad\n")
    with pytest.raises(ref_f90c.TranslateError, match="line 5"):
        ref_f90c.translate_file(str(src))
    with pytest.raises(ref_f90c.TranslateError, match="not parameters"):
        src.write_text("program ok\n  implicit none\n  integer :: i\n  i = 1\nend program ok\n")
        ref_f90c.translate_file(str(src), {"NX": 3})


IO_TEST = """\
program iotest
  implicit none
  integer :: k
  character(len=20) :: fname
  k = 42
  write(fname,"('out',i3.3,'.txt')") k
  open(unit=12, file=fname, status='unknown')
  write(12,"(i3,' ',i2,' x',i6.4)") 7, 123, -42
  write(12,"('no items ',i4,' after')")
  write(12,*) k, -3
  write(12,*) 'abc'
  write(12,*) 1.5d0, 0.1
  close(12)
end program iotest
"""


def test_translator_io(tmp_path):
    """WRITE with I editing (the standard's rules: right-justified, at least
    m digits, asterisks when the field is too narrow), output that stops at
    the first data edit without an item, internal WRITE into a file name,
    OPEN/CLOSE, and list-directed integers and strings."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    src = tmp_path / "iotest.f90"
    src.write_text(IO_TEST)
    code, manifest = ref_f90c.translate_file(str(src), io=True)
    (tmp_path / "iotest.c").write_text(code)
    exe = tmp_path / "iotest"
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-w", "-o", str(exe), str(tmp_path / "iotest.c"),
                    ref_f90c.MPI_RUNTIME, "-lm", "-lpthread"], check=True)
    out = ref_f90c.RefProgram(str(exe), manifest).run(files=["out042.txt"])[0]["files"]["out042.txt"]
    lines = out.splitlines()
    assert lines[:4] == ["  7 ** x -0042", "no items ", "          42          -3", " abc"]
    # list-directed reals: digits enough to read the value back exactly
    d, r = (float(v) for v in lines[4].split())
    assert d == 1.5 and np.float32(r) == np.float32(0.1) and r != 0.1


@pytest.mark.skipif(not os.path.isdir(REF_DIR) or shutil.which("gcc") is None,
                    reason="needs the reference sources and gcc")
def test_pnm_vectors_regenerate_from_reference_source(tmp_path):
    import sys
    sys.path.insert(0, GOLD)
    import make_ref_vectors as M
    a, b = dict(np.load(M.generate_pnm(REF_DIR, str(tmp_path)))), load("refpin_pnm")
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def _regenerable():
    import sys
    sys.path.insert(0, GOLD)
    import make_ref_vectors as M
    return [n for n in M.CASES if not n.endswith("_full")]


@pytest.mark.skipif(not os.path.isdir(REF_DIR) or shutil.which("gcc") is None,
                    reason="needs the reference sources and gcc")
def test_file_vectors_regenerate_from_reference_source(tmp_path):
    import sys
    sys.path.insert(0, GOLD)
    import make_ref_vectors as M
    a, b = dict(np.load(M.generate_files(REF_DIR, str(tmp_path)))), load("refpin_files")
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.skipif(not os.path.isdir(REF_DIR) or shutil.which("gcc") is None,
                    reason="needs the reference sources and gcc")
@pytest.mark.parametrize("name", _regenerable())
def test_vectors_regenerate_from_reference_source(name, tmp_path):
    import sys
    sys.path.insert(0, GOLD)
    import make_ref_vectors as M
    path = M.generate(name, REF_DIR, str(tmp_path))
    a, b = dict(np.load(path)), load(name)
    assert sorted(a) == sorted(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


# ---------------------------------------------------------------------------
# FP32 runs against the reference (the GPU twin is test_gpu_ref_pin.py)
# ---------------------------------------------------------------------------
TRACE_TOL = 1e-5     # relative L2 over all receivers and recorded components
ENERGY_TOL = 1e-6    # relative L2 of the energy curve


def rl2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def compare_fp32(fx, vx, vy, ek, ep):
    """Trace and energy rel-L2 of an FP32 run against a reference fixture.
    The 3D program records vx and vy only (3D:1126-1127)."""
    et = rl2(np.concatenate([vx, vy]), np.concatenate([fx["sisvx"], fx["sisvy"]]))
    e_ref = fx["energy"] if "energy" in fx else fx["ek"] + fx["ep"]
    ee = rl2(ek + ep, e_ref)
    assert et <= TRACE_TOL, f"trace rel-L2 {et:.3e}"
    assert ee <= ENERGY_TOL, f"energy rel-L2 {ee:.3e}"
    return et, ee


@pytest.mark.parametrize("name", SMALL)
def test_fp32_restatement_within_tolerance_of_reference(name):
    """The algorithm in FP32 (the oracle's float instantiation) stays within
    the GPU tolerances of the reference's FP64 outputs: the same check the
    GPU runs, here on the CPU."""
    fx = load(name)
    p, rec = params_of(fx)
    m = model_of(fx)
    r = oracle_c.run(p, rec=rec, double=False, **(dict(lam=m[0], mu=m[1], rho=m[2]) if m else {}))
    compare_fp32(fx, r.sisvx, r.sisvy, r.ek, r.ep)


# ---------------------------------------------------------------------------
# PNM snapshots
# ---------------------------------------------------------------------------
PNM_CASES = ["vx_small", "vy_corner", "vx_fourth", "sxy_split", "seeded", "zero"]


@pytest.fixture(scope="module")
def cpml_lib():
    from seismic_cpml_gb300 import lib as L
    from seismic_cpml_gb300.build import build
    build()
    return L.load()


@pytest.mark.parametrize("case", PNM_CASES)
def test_pnm_writer_reproduces_reference(case, cpml_lib, tmp_path):
    """cpml_write_pnm against the programs' own create_color_image
    (2D:861-999, translated and run on the same plane; refpin_pnm.npz).
    The pixel records, written with the explicit format (i3,' ',i3,' ',i3),
    must match byte for byte. The header lines are list-directed, whose
    spacing is the compiler's choice, so only their tokens are compared."""
    import ctypes
    fx = load("refpin_pnm")
    plane, rec = fx[case + "_plane"], fx[case + "_rec"]
    par = dict(zip([str(n) for n in fx["par_names"]], (int(v) for v in fx[case + "_par"])))
    ny, nx = plane.shape
    use = np.array([par[k] for k in ("UXMIN", "UXMAX", "UYMIN", "UYMAX")], np.int32)
    ix, iy = np.ascontiguousarray(rec[:, 0]), np.ascontiguousarray(rec[:, 1])
    ip = ctypes.POINTER(ctypes.c_int)
    st = cpml_lib.cpml_write_pnm(str(tmp_path).encode(),
                                 plane.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), nx, ny,
                                 par["IT"], par["ISRC"], par["JSRC"], ix.ctypes.data_as(ip),
                                 iy.ctypes.data_as(ip), len(rec), par["NPML"], use.ctypes.data_as(ip),
                                 par["FIELD"])
    assert st == 0
    ours = (tmp_path / str(fx[case + "_file"])).read_text().splitlines()
    ref = bytes(fx[case + "_pnm"]).decode().splitlines()
    assert [ln.split() for ln in ours[:3]] == [ln.split() for ln in ref[:3]]
    assert len(ours) == len(ref) == 3 + nx * ny
    bad = [k for k in range(3, len(ref)) if ours[k] != ref[k]]
    assert not bad, f"{len(bad)} pixels differ, first at record {bad[0]}: {ours[bad[0]]!r} vs {ref[bad[0]]!r}"



def test_blow_up_stops_where_the_reference_stops():
    """The stop rule (2D:716-726): a per-cell model 1.6x faster than the cp
    of the Courant check runs unstable. The reference program stops at the
    first display step (it = 5 or a multiple of IT_DISPLAY) where
    max |v| > 1e25. The oracle's max |v| crosses the threshold at that same
    step, and its traces equal the reference's up to it."""
    fx = load("refpin_2d_blowup")
    p, rec = params_of(fx)
    m = model_of(fx)
    stop = int(fx["stop_it"])
    assert "blew up" in str(fx["stop"])
    r = oracle_c.run(p, rec=rec, vmax=True, lam=m[0], mu=m[1], rho=m[2])
    display = [it for it in range(1, p.nstep + 1) if it % p.it_display == 0 or it == 5]
    first = next(it for it in display if r.vmax[it - 1] > 1e25)
    assert first == stop
    for k in ("sisvx", "sisvy"):
        assert np.array_equal(getattr(r, k)[:, :stop], fx[k][:, :stop]), k
    assert np.array_equal(r.ek[:stop], fx["ek"][:stop]) and np.array_equal(r.ep[:stop], fx["ep"][:stop])


PROFILE_CASES = [n for n in SMALL + SHIPPED if n != "refpin_3d_plain_full"] + ["refpin_2d_blowup"]


@pytest.mark.parametrize("name", PROFILE_CASES)
def test_pml_profiles_reproduce_reference(name, cpml_lib):
    """R1 at the C ABI: cpml_pml_profile (FP64 d, K, alpha, a, b at grid and
    half points per axis, what the device tables are rounded from) against
    the reference program's own profile arrays, bit for bit. For the
    split-field program: its damping profiles divided by two.

    One documented exception: the reference clamps alpha >= 0 along x only
    (2D:383-384, 3D:514-515). On y and z, the half point past the last grid
    point (j = NY, k = NZ, which lies outside the layer) keeps a negative
    alpha, and the a_half and b_half computed from it. No loop of the
    programs reads that entry (half-point arrays are read up to N - 1). Here
    every axis is clamped, so at that one entry alpha_half is max(alpha, 0)."""
    import ctypes
    fx = load(name)
    p, _ = params_of(fx)
    dp = ctypes.POINTER(ctypes.c_double)
    for axis, ax in enumerate("xyz"[:p.ndim]):
        if "prof_" + ax not in fx:
            continue
        ref = fx["prof_" + ax]
        n = ref.shape[1]
        arrs = [np.zeros(n) for _ in range(10)]
        assert cpml_lib.cpml_pml_profile(ctypes.byref(p), axis, n, *[a.ctypes.data_as(dp) for a in arrs]) == 0
        ours = np.stack([arrs[0], arrs[5]]) if p.scheme == P.SCHEME_SPLIT else np.stack(arrs)
        keep = np.ones(n, bool)
        if p.scheme != P.SCHEME_SPLIT and ax != "x" and ref[7][-1] < 0:
            assert ours[7][-1] == 0.0                # clamped here, not in the reference
            keep[-1] = False
        for q in range(ref.shape[0]):
            assert np.array_equal(ours[q][keep], ref[q][keep]), (ax, q, np.abs(ours[q] - ref[q]).max())


@pytest.mark.parametrize("name", PROFILE_CASES)
def test_courant_number_reproduces_reference(name, cpml_lib):
    """R4: cpml_courant equals the Courant number each program computes for
    its check (2D:513, 2D4:514, 3D:712, PML:304: the split-field program's
    is one-dimensional, cp * DELTAT / h), bit for bit."""
    import ctypes
    fx = load(name)
    p, _ = params_of(fx)
    cpml_lib.cpml_courant.restype = ctypes.c_double
    cpml_lib.cpml_courant.argtypes = [ctypes.c_void_p, ctypes.c_double]
    assert cpml_lib.cpml_courant(ctypes.byref(p), p.cp) == fx["courant"].item()



@pytest.mark.parametrize("key, case", [("d2", "refpin_2d_small"), ("d3", "refpin_3d_2ranks")])
def test_output_files_reproduce_reference(key, case, cpml_lib, tmp_path):
    """The seismogram files and energy.dat (2D:826-857, 741-746;
    3D:1253-1257): cpml_write_seismograms and cpml_write_energy, given the
    reference run's own seismograms and energies, write the same files as
    the programs' own WRITE statements. Same names, same lines, and every
    number the same when read back: single precision for the time stamps,
    the traces and the 2D energies, double for the 3D total energy. The
    list-directed spacing is the compiler's choice and is not compared."""
    import ctypes
    files, fx = load("refpin_files"), load(case)
    p, _ = params_of(fx)
    nrec, nt = fx["sisvx"].shape
    dp = ctypes.POINTER(ctypes.c_double)
    vx, vy = np.ascontiguousarray(fx["sisvx"]), np.ascontiguousarray(fx["sisvy"])
    d = str(tmp_path).encode()
    assert cpml_lib.cpml_write_seismograms(d, vx.ctypes.data_as(dp), vy.ctypes.data_as(dp), None, nt,
                                           nrec, ctypes.c_double(p.deltat)) == 0
    if key == "d3":
        ek, ep = np.ascontiguousarray(fx["energy"]), np.zeros(nt)
    else:
        ek, ep = np.ascontiguousarray(fx["ek"]), np.ascontiguousarray(fx["ep"])
    assert cpml_lib.cpml_write_energy(d, ek.ctypes.data_as(dp), ep.ctypes.data_as(dp), nt,
                                      ctypes.c_double(p.deltat), 2 if key == "d3" else 4) == 0
    ref_names = sorted(k[len(key) + 2:] for k in files if k.startswith(key + "__") and k.endswith("_dat"))
    ours = sorted(f.name.replace(".", "_") for f in tmp_path.iterdir())
    assert ours == ref_names
    for n in ref_names:
        ref = np.loadtxt(bytes(files[f"{key}__{n}"]).decode().splitlines(), ndmin=2)
        got = np.loadtxt(tmp_path / n.replace("_dat", ".dat"), ndmin=2)
        assert ref.shape == got.shape == (nt, ref.shape[1]), n
        single = [0] if (key == "d3" and n == "energy_dat") else list(range(ref.shape[1]))
        for c in range(ref.shape[1]):   # REAL(4) columns compared as the floats they hold
            a, b = (ref[:, c].astype(np.float32), got[:, c].astype(np.float32)) if c in single \
                else (ref[:, c], got[:, c])
            assert np.array_equal(a, b), (n, c, np.abs(ref[:, c] - got[:, c]).max())


@pytest.mark.parametrize("fn, name", [("cpml_params_default_2d", "refpin_2d_shipped"),
                                      ("cpml_params_default_2d_fourth", "refpin_2d4_shipped"),
                                      ("cpml_params_default_2d_split", "refpin_pml2d_shipped")])
def test_default_parameter_blocks_are_the_shipped_programs(fn, name, cpml_lib):
    """The C ABI's default parameter blocks are the shipped programs' own
    (2D:138-218, 2D4:132-190, PML:96-141): every value equals what the
    program evaluated when run as shipped."""
    import ctypes
    q = P.CpmlParams()
    assert getattr(cpml_lib, fn)(ctypes.byref(q)) == 0
    p, _ = params_of(load(name))
    for f, _t in P.CpmlParams._fields_:
        if f.startswith("reserved") or f in ("flags", "ksource", "nz", "deltaz"):
            continue
        a, b = getattr(q, f), getattr(p, f)
        if f == "use_pml":
            a, b = list(a)[:4], list(b)[:4]
        assert a == b, (f, a, b)


def test_default_3d_block_is_the_shipped_program(cpml_lib, tmp_path):
    """cpml_params_default_3d against the shipped 3D program's parameter
    block (3D:124-218) as cpml_program evaluates it from the source (that
    evaluator is pinned against the program's own evaluation above), with
    the source and receivers on the cut plane NZ/2."""
    import ctypes
    from seismic_cpml_gb300.build import PROGRAM, build
    if not os.path.isdir(REF_DIR):
        pytest.skip("needs the reference sources")
    build()
    src = os.path.join(REF_DIR, ref_f90c.REFERENCE_PROGRAMS["cpml3d"])
    r = subprocess.run([PROGRAM, "3d", src, str(tmp_path), "--print-params"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = dict(ln.split(" = ", 1) for ln in r.stdout.splitlines() if " = " in ln and not ln.startswith((" ", "!")))
    q = P.CpmlParams()
    assert cpml_lib.cpml_params_default_3d(ctypes.byref(q)) == 0
    amax = 2.0 * math.pi * (q.f0 / 2.0) if q.alpha_max_pml < 0 else q.alpha_max_pml
    want = {"NX": q.nx, "NY": q.ny, "NZ": q.nz, "NSTEP": q.nstep, "NPOINTS_PML": q.npoints_pml,
            "IT_DISPLAY": q.it_display, "DELTAX": q.deltax, "DELTAY": q.deltay, "DELTAZ": q.deltaz,
            "DELTAT": q.deltat, "cp": q.cp, "cs": q.cs, "rho": q.rho, "f0": q.f0, "t0": q.t0,
            "factor": q.factor, "ANGLE_FORCE": q.angle_force, "ISOURCE": q.isource,
            "JSOURCE": q.jsource, "KSOURCE": q.ksource, "NPOWER": q.npower, "K_MAX_PML": q.k_max_pml,
            "ALPHA_MAX_PML": amax, "RCOEF": q.rcoef}
    for k, v in want.items():
        assert float(got[k]) == float(v), (k, got[k], v)
    for k, face in zip(["XMIN", "XMAX", "YMIN", "YMAX", "ZMIN", "ZMAX"], q.use_pml):
        assert got["USE_PML_" + k] == (".true." if face else ".false."), k


RECEIVER_CASES = PROFILE_CASES + ["refpin_2d_receivers"]


@pytest.mark.parametrize("name", RECEIVER_CASES)
def test_nearest_gridpoint_reproduces_reference(name, cpml_lib):
    """R3: cpml_nearest_gridpoint, given each program's receiver targets in
    metres, returns the grid points the program chose (2D:483-509,
    3D:683-706), ties included: refpin_2d_receivers puts 41 targets on
    half-cell positions, where the strict < keeps the first minimum."""
    import ctypes
    fx = load(name)
    p, _ = params_of(fx)
    i, j = ctypes.c_int(), ctypes.c_int()
    for (x, y), (ri, rj) in zip(fx["rec_xy"], fx["rec"]):
        assert cpml_lib.cpml_nearest_gridpoint(p.nx, p.ny, ctypes.c_double(p.deltax),
                                               ctypes.c_double(p.deltay), ctypes.c_double(x),
                                               ctypes.c_double(y), ctypes.byref(i), ctypes.byref(j)) == 0
        assert (i.value, j.value) == (int(ri), int(rj)), (x, y)



SEMANTICS_TEST = """\
program semantics
  implicit none
  real :: x, y
  double precision :: d, e
  double precision, dimension(-2:3) :: a
  integer :: i, n1, n2, n3, n4, m1, m2, trips, mx, mn
  logical :: p, q, r
  x = 0.1
  y = x * 3.0 + 1.0e-3
  d = x * 3.0d0
  e = 0.1d0 * 3.0d0
  n1 = nint(2.5d0)
  n2 = nint(-2.5d0)
  n3 = nint(0.49999997)
  n4 = int(-3.7d0)
  m1 = mod(-7, 3)
  m2 = mod(7, -3)
  mx = max(3, -1, 8, 2)
  mn = min(3, -1, 8, 2)
  trips = 0
  do i = 5, 4
    trips = trips + 1
  enddo
  a(:) = 0.d0
  a(-1:1) = 2.d0
  a(3) = sum(a(-2:2)) / 4.d0
  p = .true.
  q = (n1 == 3) .eqv. (n2 == -3)
  r = p .neqv. q
  if (q) then
    if (.not. r) n4 = n4 * 10
  endif
end program semantics
"""


def test_translator_arithmetic_semantics(tmp_path):
    """Fortran's rules as the translation keeps them: single-precision
    arithmetic rounds every operation to float, mixed kinds promote to
    double, NINT rounds halves away from zero, INT and MOD truncate, a DO
    loop whose range is empty runs no trip, sections keep declared lower
    bounds, .EQV./.NEQV. compare logicals."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    src = tmp_path / "semantics.f90"
    src.write_text(SEMANTICS_TEST)
    names = ["x", "y", "d", "e", "a", "n1", "n2", "n3", "n4", "m1", "m2", "mx", "mn", "trips", "q", "r"]
    code, manifest = ref_f90c.translate_file(str(src), dump=names)
    (tmp_path / "s.c").write_text(code)
    exe = tmp_path / "s"
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-w", "-o", str(exe), str(tmp_path / "s.c"),
                    ref_f90c.MPI_RUNTIME, "-lm", "-lpthread"], check=True)
    v = ref_f90c.RefProgram(str(exe), manifest).run()[0]
    f = np.float32
    assert v["x"] == f(0.1)
    assert v["y"] == f(f(f(0.1) * f(3.0)) + f(1.0e-3))         # every step rounded to float
    assert v["d"] == float(f(0.1)) * 3.0 and v["d"] != 0.1 * 3.0  # the float 0.1, promoted
    assert v["e"] == 0.1 * 3.0
    assert (int(v["n1"]), int(v["n2"]), int(v["n3"])) == (3, -3, 0)
    assert (int(v["m1"]), int(v["m2"])) == (-1, 1)              # sign of the first operand
    assert (int(v["mx"]), int(v["mn"]), int(v["trips"])) == (8, -1, 0)
    assert v["a"].tolist() == [0.0, 2.0, 2.0, 2.0, 0.0, 1.5]   # a(-2..3)
    assert int(v["q"]) == 1 and int(v["r"]) == 0
    assert int(v["n4"]) == -30                                  # INT truncates; nested IF taken
