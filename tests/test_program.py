"""cpml_program, the C++ host program that replaces the reference programs'
main units: parameter file with the Fortran names, stop conditions, and the
reference's output files."""
import subprocess

import numpy as np
import pytest

from seismic_cpml_gb300.build import PROGRAM, build


@pytest.fixture(scope="module")
def program():
    build()
    return PROGRAM


def test_courant_violation_stops_like_the_reference(program, tmp_path):
    par = tmp_path / "p.par"
    par.write_text("NX = 60\nNY = 80\nDELTAT = 5.d-3   ! Courant 2.3\n")
    r = subprocess.run([program, "2d", str(par), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 3
    assert "time step is too large, simulation will be unstable" in r.stdout    # 2D:516


def test_fortran_double_literals_are_read(program, tmp_path):
    """DELTAT = 1.6d-3 is 0.0016 s (Courant 0.75: the program goes on to the
    device, which a CPU-only run does not have, or runs to the end on a GPU),
    not 1.6 s, which would stop on the Courant check (2D:516)."""
    par = tmp_path / "p.par"
    par.write_text("NX = 60\nNY = 80\nNSTEP = 40\nIT_DISPLAY = 20\nDELTAT = 1.6d-3\n")
    r = subprocess.run([program, "2d", str(par), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode != 3 and "too large" not in r.stdout, r.stdout
    assert r.returncode in (0, 4), r.stdout + r.stderr


def test_non_numeric_value_is_rejected(program, tmp_path):
    par = tmp_path / "p.par"
    par.write_text("NX = sixty\n")
    r = subprocess.run([program, "2d", str(par), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 2 and "bad value for NX" in r.stderr


def test_unknown_parameter_is_rejected(program, tmp_path):
    par = tmp_path / "p.par"
    par.write_text("NXX = 60\n")
    r = subprocess.run([program, "2d", str(par), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown parameter" in r.stderr


@pytest.mark.gpu
def test_program_2d_default_outputs(program, tmp_path, golden):
    """The shipped 2D program: same receivers, seismogram files within FP32
    parity of the FP64 fixture, energy.dat with 4 columns, snapshots at the
    display steps, gnuplot scripts."""
    r = subprocess.run([program, "2d", "-", str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "closest grid point found in i,j = 70 231" in r.stdout
    g = golden("ref2d_default")
    vx = np.stack([np.loadtxt(tmp_path / f"Vx_file_{k:03d}.dat")[:, 1] for k in (1, 2)])
    err = np.linalg.norm(vx - g["sisvx"]) / np.linalg.norm(g["sisvx"])
    assert err < 1e-5, err
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape == (2000, 4)
    for it in (5, 100, 2000):
        assert (tmp_path / f"image{it:06d}_Vx.pnm").exists()
        assert (tmp_path / f"image{it:06d}_Vy.pnm").exists()
    assert (tmp_path / "plotgnu").exists() and (tmp_path / "plot_energy").exists()
    cmp_script = (tmp_path / "plot_comparison").read_text()   # 2D:764-777
    assert '"../collino/energy.dat" us 1:4' in cmp_script and "compare_total_energy_semilog.eps" in cmp_script


@pytest.mark.gpu
@pytest.mark.parametrize("mode, fixture, nstep, display", [("2d4", "ref2d_fourth", 4000, 200),
                                                           ("2dpml", "ref2d_split", 2000, 100)])
def test_program_other_2d_programs(program, tmp_path, golden, mode, fixture, nstep, display):
    """The fourth-order and split-field PML programs as shipped, run by
    cpml_program: seismogram files within FP32 parity of the FP64 fixtures
    (equal to the reference's own outputs), energy.dat, snapshots."""
    r = subprocess.run([program, mode, "-", str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    g = golden(fixture)
    for comp, key in (("Vx", "sisvx"), ("Vy", "sisvy")):
        tr = np.stack([np.loadtxt(tmp_path / f"{comp}_file_{k:03d}.dat")[:, 1] for k in (1, 2)])
        err = np.linalg.norm(tr - g[key]) / np.linalg.norm(g[key])
        assert err < 1e-5, (comp, err)
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape == (nstep, 4)
    tot = g["ek"] + g["ep"]
    assert np.linalg.norm(e[:, 3] - tot) / np.linalg.norm(tot) < 1e-6
    for it in (5, display, nstep):
        assert (tmp_path / f"image{it:06d}_Vx.pnm").exists()
    # each program's own scripts: the split-field program names its energy
    # plot after Collino and writes no comparison script (PML:562-606)
    energy_plot = (tmp_path / "plot_energy").read_text()
    if mode == "2dpml":
        assert "collino_total_energy_semilog.eps" in energy_plot
        assert not (tmp_path / "plot_comparison").exists()
    else:
        assert "cpml_total_energy_semilog.eps" in energy_plot
        assert (tmp_path / "plot_comparison").exists()


@pytest.mark.gpu
def test_program_3d_outputs(program, tmp_path):
    """The 3D program on a small grid: progress and elapsed-time lines, a
    timestamp file per display step (3D:1197-1228), snapshots of the cut
    plane, 2-column energy.dat (3D:1255), vx and vy files but no vz ones,
    which its gnuplot script names nonetheless (3D:1293-1296, 1330-1364)."""
    par = tmp_path / "p.par"
    par.write_text("NX = 40\nNY = 40\nNZ = 36\nNSTEP = 120\nIT_DISPLAY = 50\n"
                   "YDEB = 300.d0\nYFIN = 100.d0\n")
    r = subprocess.run([program, "3d", str(par), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Elapsed time in hh:mm:ss" in r.stdout
    for it in (5, 50, 100):
        ts = (tmp_path / f"timestamp{it:06d}").read_text()
        assert f"Time step # {it}" in ts and "Mean elapsed time per time step" in ts
        assert (tmp_path / f"image{it:06d}_Vx.pnm").exists()
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape == (120, 2) and np.isfinite(e).all() and e[:, 1].max() > 0
    assert (tmp_path / "Vx_file_001.dat").exists() and (tmp_path / "Vy_file_002.dat").exists()
    assert not (tmp_path / "Vz_file_001.dat").exists()
    assert "Vz_file_001.dat" in (tmp_path / "plotgnu").read_text()


# ---------------------------------------------------------------------------
# the reference program's own source as the parameter file
# ---------------------------------------------------------------------------
REF_CASES = ["refpin_2d_shipped", "refpin_2d_small", "refpin_2d_profiles", "refpin_2d_plain",
             "refpin_2d4_shipped", "refpin_2d4_small", "refpin_2d4_profiles",
             "refpin_pml2d_shipped", "refpin_pml2d_small",
             "refpin_3d_2ranks", "refpin_3d_4ranks", "refpin_3d_profiles", "refpin_3d_plain_full"]
MODE = {"cpml2d": "2d", "cpml2d4": "2d4", "pml2d": "2dpml", "cpml3d": "3d"}


def edited_source(src, overrides, stf):
    """The program's text with its parameter lines edited as a user edits
    them, and the chosen wavelet line active."""
    import re
    from oracle import ref_f90c
    lines = open(src, encoding="latin-1").read().split("\n")
    for name, value in overrides.items():
        rx = re.compile(r"(?i)(\b%s\s*=\s*)([^,!]+)" % re.escape(name))
        for k, ln in enumerate(lines):
            if not ln.lstrip().startswith("!") and "parameter" in ln.lower() and rx.search(ln):
                lines[k] = rx.sub(lambda m: m.group(1) + str(value) + " ", ln, count=1)
                break
        else:
            raise AssertionError(f"no parameter line for {name}")
    if stf is not None:
        lines = ref_f90c.select_source_time_function(lines, stf)
    return "\n".join(lines)


@pytest.mark.parametrize("name", REF_CASES)
def test_reference_source_as_parameter_file(program, tmp_path, name):
    """cpml_program reads a reference program's .f90 file as its parameter
    file. Every parameter it resolves, and every receiver point, equals what
    the program itself evaluated when translated and run (the p_* values and
    receivers of the reference vectors), bit for bit."""
    import ast
    import os
    import sys
    from oracle import ref_f90c
    if not os.path.isdir(ref_f90c.DEFAULT_REF_DIR):
        pytest.skip("needs the reference sources")
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, gold)
    import make_ref_vectors as M
    prog, overrides, stf = M.CASES[name][:3]
    fx = dict(np.load(os.path.join(gold, name + ".npz")))
    src = tmp_path / "program.f90"
    src.write_text(edited_source(os.path.join(ref_f90c.DEFAULT_REF_DIR, M.PROGRAMS[prog]), overrides, stf))
    three_d, split = prog == "cpml3d", prog == "pml2d"
    r = subprocess.run([program, MODE[prog], str(src), str(tmp_path), "--print-params"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = {}
    for ln in r.stdout.splitlines():
        if " = " in ln and not ln.startswith(" "):
            k, v = ln.split(" = ", 1)
            got[k.lower()] = v.strip()
    rho = "rho" if three_d or split else "density"
    pairs = {"nx": "nx", "ny": "ny", "nstep": "nstep", "npoints_pml": "npoints_pml",
             "it_display": "it_display", "deltat": "deltat",
             "cp": "cp", "cs": "cs", "rho": rho, "f0": "f0", "t0": "t0", "factor": "factor",
             "angle_force": "angle_force", "isource": "isource", "jsource": "jsource", "nrec": "nrec"}
    if split:        # one grid spacing h, PML on every edge (PML:100)
        pairs.update(deltax="h", deltay="h")
    else:
        pairs.update(deltax="deltax", deltay="deltay", use_pml_xmin="use_pml_xmin",
                     use_pml_xmax="use_pml_xmax", use_pml_ymin="use_pml_ymin", use_pml_ymax="use_pml_ymax")
    if "p_npower" in fx:
        pairs.update(npower="npower", k_max_pml="k_max_pml", alpha_max_pml="alpha_max_pml")
    if three_d:
        pairs.update(nz="nz", deltaz="deltaz", use_pml_zmin="use_pml_zmin", use_pml_zmax="use_pml_zmax")
    for ours, theirs in pairs.items():
        want = fx["p_" + theirs].item()
        v = got[ours]
        have = {".true.": 1, ".false.": 0}.get(v, None)
        have = ast.literal_eval(v) if have is None else have
        assert float(have) == float(want), (ours, v, want)
    stf_name = {"ricker": "ricker", "gaussian": "gaussian", "program default": "derivative_of_gaussian"}
    assert got["source_time_function"] == stf_name[str(fx["stf"])]
    recs = [tuple(int(x) for x in ln.split("=")[1].split()) for ln in r.stdout.splitlines()
            if "closest grid point found in i,j" in ln]
    assert recs == [tuple(int(v) for v in rr) for rr in fx["rec"]]


def test_fortran_parameter_file_errors(program, tmp_path):
    """An expression naming something undefined, or a program whose
    source_term lines are all commented out, stops with a message before
    any device call."""
    base = ("program p\n  implicit none\n  integer, parameter :: NX = 2**5 + 8, NY = 50\n"
            "  double precision, parameter :: DELTAX = 10.d0, DELTAT = 1.d-3\n"
            "  integer, parameter :: NSTEP = 10, NPOINTS_PML = 5, ISOURCE = NX / 2, JSOURCE = 2 * NY / 3\n"
            "  double precision, parameter :: cp = 3000.d0, cs = cp / 1.732d0, density = 2000.d0\n"
            "  double precision, parameter :: f0 = 10.d0, factor = 1.d7, ANGLE_FORCE = 0.d0\n")
    src = tmp_path / "bad.f90"
    src.write_text(base + "  double precision, parameter :: t0 = 1.2d0 / fzero\n"
                   "  source_term = factor\nend program p\n")
    r = subprocess.run([program, "2d", str(src), str(tmp_path), "--print-params"], capture_output=True,
                       text=True)
    assert r.returncode == 2 and "unknown name fzero" in r.stderr
    src.write_text(base + "! source_term = factor\nend program p\n")
    r = subprocess.run([program, "2d", str(src), str(tmp_path), "--print-params"], capture_output=True,
                       text=True)
    assert r.returncode == 2 and "one active source_term line, found 0" in r.stderr
    src.write_text(base + "  source_term = factor * exp(-a*(t-t0)**2)\nend program p\n")
    r = subprocess.run([program, "2d", str(src), str(tmp_path), "--print-params"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert "NX = 40" in r.stdout                                           # 2**5 + 8
    assert "ISOURCE = 20" in r.stdout and "JSOURCE = 33" in r.stdout      # integer division
    assert "SOURCE_TIME_FUNCTION = gaussian" in r.stdout


SCRIPT_CASES = {"refpin_2d_small": "d2", "refpin_3d_2ranks": "d3", "refpin_2d4_small": "d24",
                "refpin_pml2d_small": "dpml"}


@pytest.mark.parametrize("name", list(SCRIPT_CASES))
def test_gnuplot_scripts_reproduce_reference(program, tmp_path, name):
    """The gnuplot scripts cpml_program writes equal the ones each program
    writes itself (translated with its WRITE statements; refpin_files.npz),
    line for line. Only the leading blank of a list-directed record, the
    compiler's choice, is not compared."""
    import os
    import sys
    from oracle import ref_f90c
    if not os.path.isdir(ref_f90c.DEFAULT_REF_DIR):
        pytest.skip("needs the reference sources")
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, gold)
    import make_ref_vectors as M
    prog, overrides, stf = M.CASES[name][:3]
    src = tmp_path / "program.f90"
    src.write_text(edited_source(os.path.join(ref_f90c.DEFAULT_REF_DIR, M.PROGRAMS[prog]), overrides, stf))
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([program, MODE[prog], str(src), str(out), "--scripts-only"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    files = dict(np.load(os.path.join(gold, "refpin_files.npz")))
    key = SCRIPT_CASES[name]
    norm = lambda t: [ln[1:].rstrip() if ln.startswith(" ") else ln.rstrip() for ln in t.splitlines()]  # noqa: E731
    for script in M.SCRIPTS[prog]:
        ref = norm(bytes(files[f"{key}__{script}"]).decode())
        ours = norm((out / script).read_text())
        assert ours == ref, (script, [(a, b) for a, b in zip(ours, ref) if a != b][:3], len(ours), len(ref))
    extra = {f.name for f in out.iterdir()} - set(M.SCRIPTS[prog])
    assert not extra, extra
