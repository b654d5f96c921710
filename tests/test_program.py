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
