"""Generate tests/golden/refpin_*.npz: golden vectors from the reference itself.

The reference programs are Fortran, and no Fortran compiler exists on either
machine this project runs on. oracle/ref_f90c.py translates each program's
own source, read where it lies, into C. gcc compiles it, and oracle/ref_mpi.c
runs it on emulated MPI ranks. This script runs those programs and saves:
  - the parameters each run used (as the program evaluated them);
  - the receiver grid points from the program's own nearest-point search;
  - the seismograms and energies;
  - SHA-256 digests of the final wavefields. The small 2D cases also keep
    the fields themselves. For the full-size 3D case only digests of the
    traces are kept: they equal config_3d_plain.npz's bit for bit.
tests/test_ref_pin.py checks the C++ oracle against these vectors, bit for
bit where the arithmetic order is the same.

Parameters are overridden as a user edits the `parameter` lines, and the
source-time function is chosen among the program's three `source_term`
lines. Nothing else in the programs changes.

refpin_files.npz holds the seismogram files, energy.dat and the gnuplot
scripts the four programs write themselves (their WRITE statements
translated too).
refpin_pnm.npz holds PNM snapshots from the programs' create_color_image
subroutine (2D:861-999, the same in all four programs), run by a small
driver of this project's own on planes given to it.

Run (needs the reference sources and gcc):
    python tests/golden/make_ref_vectors.py [--ref-dir DIR] [name ...]
The full-size 3D case (276^3 x 2500 steps on 12 ranks) takes several
minutes. The other cases take seconds.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_f90c  # noqa: E402

PROGRAMS = ref_f90c.REFERENCE_PROGRAMS

_COMMON = ["nx", "ny", "npoints_pml", "cp", "cs", "nstep", "deltat", "f0", "t0", "factor",
           "isource", "jsource", "angle_force", "nrec", "it_display"]
PARAMS = {
    "cpml2d": _COMMON + ["deltax", "deltay", "density", "use_pml_xmin", "use_pml_xmax",
                         "use_pml_ymin", "use_pml_ymax"],
    "pml2d": _COMMON + ["h", "rho"],
    "cpml3d": _COMMON + ["nz", "nproc", "deltax", "deltay", "deltaz", "rho", "use_pml_xmin",
                         "use_pml_xmax", "use_pml_ymin", "use_pml_ymax", "use_pml_zmin",
                         "use_pml_zmax"],
}
for _k in ("cpml2d", "cpml3d"):
    PARAMS[_k] += ["npower", "k_max_pml", "alpha_max_pml"]
PARAMS["cpml2d4"] = PARAMS["cpml2d"]

# final wavefields: oracle name -> the program's array name(s); the split
# program's total field is the sum of its two parts (PML:153-159)
FIELDS = {
    "cpml2d": {"vx": ["vx"], "vy": ["vy"], "sxx": ["sigma_xx"], "syy": ["sigma_yy"],
               "sxy": ["sigma_xy"]},
    "cpml2d4": {"vx": ["vx"], "vy": ["vy"], "sxx": ["sigmaxx"], "syy": ["sigmayy"],
                "sxy": ["sigmaxy"]},
    "pml2d": {"vx": ["vx_1", "vx_2"], "vy": ["vy_1", "vy_2"], "sxx": ["sigmaxx_1", "sigmaxx_2"],
              "syy": ["sigmayy_1", "sigmayy_2"], "sxy": ["sigmaxy_1", "sigmaxy_2"]},
    "cpml3d": {"vx": ["vx"], "vy": ["vy"], "vz": ["vz"], "sxx": ["sigmaxx"], "syy": ["sigmayy"],
               "szz": ["sigmazz"], "sxy": ["sigmaxy"], "sxz": ["sigmaxz"], "syz": ["sigmayz"]},
}

# the C-PML profiles (R1, 2D:283-465, 3D:399-667) per axis, in the order the
# C ABI's cpml_pml_profile returns them; the split-field program's damping
# profiles divided by two (PML:180-250)
_PROF = ["d", "k", "alpha", "a", "b"]
PROFILES = {
    "cpml2d": {ax: [f"{q}_{ax}" for q in _PROF] + [f"{q}_{ax}_half" for q in _PROF] for ax in "xy"},
    "cpml3d": {ax: [f"{q}_{ax}" for q in _PROF] + [f"{q}_{ax}_half" for q in _PROF] for ax in "xyz"},
    "pml2d": {ax: [f"d{ax}_over_two", f"d{ax}_half_over_two"] for ax in "xy"},
}
PROFILES["cpml2d4"] = PROFILES["cpml2d"]

# name -> (program, overrides, source-time function or None for the
#          program's active line, emulated ranks, keep full fields
#          [, options: "model" seed of a per-cell model read in after the
#           material fill, "scale" of its lambda and mu, "stop": the run is
#           expected to end on a STOP])
CASES = {
    # the programs exactly as shipped
    "refpin_2d_shipped": ("cpml2d", {}, None, 1, False),
    "refpin_2d4_shipped": ("cpml2d4", {}, None, 1, False),
    "refpin_pml2d_shipped": ("pml2d", {}, None, 1, False),
    # the 2D plain workload (101 x 641, 2000 steps): Ricker at the centre
    # (51, 321), 45 degrees, no PML on the top edge, receivers by the
    # program's own rule relative to that source
    "refpin_2d_plain": ("cpml2d", {"ISOURCE": 51, "JSOURCE": 321, "ANGLE_FORCE": "45.d0",
                                   "USE_PML_YMAX": ".false."}, "ricker", 1, False),
    # small grids with the parameters moved: one PML face off, another
    # angle, three receivers, the Ricker wavelet (as in the 2D plain workload)
    "refpin_2d_small": ("cpml2d", {"NX": 41, "NY": 61, "NSTEP": 400, "USE_PML_YMAX": ".false.",
                                   "ANGLE_FORCE": "45.d0", "NREC": 3, "xdeb": "60.d0",
                                   "ydeb": "450.d0", "xfin": "330.d0", "yfin": "120.d0"},
                        "ricker", 1, True),
    "refpin_2d4_small": ("cpml2d4", {"NX": 43, "NY": 57, "NSTEP": 600, "USE_PML_XMIN": ".false.",
                                     "ANGLE_FORCE": "20.d0", "ydeb": "400.d0",
                                     "yfin": "150.d0"}, "gaussian", 1, True),
    "refpin_pml2d_small": ("pml2d", {"NX": 41, "NY": 61, "NSTEP": 400, "ydeb": "400.d0",
                                     "yfin": "150.d0"}, None, 1, True),
    # the C-PML profile parameters moved (R1): K_MAX_PML > 1 (the 1/K terms),
    # other NPOWER (non-integer: pow), ALPHA_MAX_PML = 0 (classical PML
    # profile), unequal grid spacings, another PML width
    "refpin_2d_profiles": ("cpml2d", {"NX": 47, "NY": 53, "NSTEP": 500, "NPOINTS_PML": 8,
                                      "DELTAY": "7.5d0", "DELTAT": "1.d-3", "NPOWER": "3.d0",
                                      "K_MAX_PML": "7.d0", "ALPHA_MAX_PML": "0.d0", "f0": "12.d0",
                                      "cp": "2800.d0", "density": "2200.d0", "ydeb": "300.d0",
                                      "yfin": "100.d0"}, None, 1, True),
    "refpin_2d4_profiles": ("cpml2d4", {"NX": 45, "NY": 51, "NSTEP": 700, "DELTAX": "9.d0",
                                        "NPOWER": "1.5d0", "K_MAX_PML": "3.d0", "ydeb": "300.d0",
                                        "yfin": "100.d0"}, "ricker", 1, True),
    "refpin_3d_profiles": ("cpml3d", {"NX": 34, "NY": 30, "NZ": 36, "NPROC": 2, "NSTEP": 220,
                                      "DELTAY": "9.d0", "ONE_OVER_DELTAY": "1.d0 / DELTAY",
                                      "DELTAZ": "8.d0", "ONE_OVER_DELTAZ": "1.d0 / DELTAZ",
                                      "DELTAT": "1.2d-3", "NPOWER": "2.5d0", "K_MAX_PML": "4.d0",
                                      "NPOINTS_PML": 9, "ANGLE_FORCE": "200.d0", "ydeb": "220.d0",
                                      "yfin": "80.d0"}, "gaussian", 2, False),
    # per-cell models (the programs' lambda, mu and rho arrays, 2D:204, with
    # their averaging rules, 2D:560-562, 586, 627): a seeded layered model
    # with anomalies, read in after the programs' homogeneous fill
    "refpin_2d_het": ("cpml2d", {"NX": 61, "NY": 73, "NSTEP": 600, "DELTAT": "1.5d-3",
                                 "ydeb": "500.d0", "yfin": "200.d0"}, "ricker", 1, True, {"model": 11}),
    "refpin_2d4_het": ("cpml2d4", {"NX": 57, "NY": 65, "NSTEP": 800, "ydeb": "450.d0",
                                   "yfin": "150.d0"}, None, 1, True, {"model": 12}),
    # the receiver rule (2D:483-509): 41 targets on half-cell positions,
    # equidistant from two or four grid points, where the strict < keeps the
    # first minimum in the program's scan order (j outer, i inner)
    "refpin_2d_receivers": ("cpml2d", {"NX": 41, "NY": 31, "NSTEP": 5, "NREC": 41,
                                       "xdeb": "5.d0", "xfin": "405.d0", "ydeb": "5.d0",
                                       "yfin": "305.d0"}, None, 1, False),
    # the blow-up stop (2D:716-726): a model 1.6x faster than the cp the
    # Courant check sees (2D:513-516), so the run passes that check and then
    # grows without bound; the program stops at the first display step
    # (it = 5 or a multiple of IT_DISPLAY) where max |v| exceeds 1e25
    "refpin_2d_blowup": ("cpml2d", {"NX": 51, "NY": 61, "NSTEP": 600, "IT_DISPLAY": 50,
                                    "ydeb": "450.d0", "yfin": "150.d0"}, None, 1, False,
                         {"model": 13, "scale": 2.56, "stop": True}),
    # 3D on 2 and 4 ranks: the z-slab exchanges of 3D:811-823 and 951-963 run
    "refpin_3d_2ranks": ("cpml3d", {"NX": 36, "NY": 40, "NZ": 40, "NPROC": 2, "NSTEP": 200,
                                    "ydeb": "300.d0", "yfin": "100.d0"}, None, 2, False),
    "refpin_3d_4ranks": ("cpml3d", {"NX": 30, "NY": 34, "NZ": 48, "NPROC": 4, "NSTEP": 240,
                                    "USE_PML_ZMAX": ".false.", "USE_PML_XMIN": ".false.",
                                    "ANGLE_FORCE": "60.d0", "NREC": 3, "xdeb": "40.d0",
                                    "ydeb": "250.d0", "xfin": "200.d0", "yfin": "90.d0"},
                         "ricker", 4, False),
    # the 3D plain workload at full size: 276^3, 2500 steps, Ricker at the
    # centre, 64 receivers on the x line through it
    "refpin_3d_plain_full": ("cpml3d", ref_f90c.plain_3d_overrides(2500), "ricker",
                             ref_f90c.PLAIN_3D_RANKS, False),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def fill_end_line(src: str) -> int:
    """Source line of the END DO that closes the 2D programs' homogeneous
    material fill (the loop nest that sets rho(i,j) = density, 2D:467-473)."""
    lines = open(src, encoding="latin-1").read().split("\n")
    start = next(k for k, ln in enumerate(lines) if re.match(r"\s*rho\(i,j\)\s*=\s*density", ln, re.I))
    ends = [k for k in range(start, len(lines)) if re.match(r"\s*end\s*do\s*$", lines[k], re.I)]
    return ends[1] + 1


def model_2d(nx, ny, seed):
    """Seeded float32 lambda, mu, rho of shape (ny, nx) (tests/models.py)."""
    from types import SimpleNamespace
    from tests.models import layered_2d
    return layered_2d(SimpleNamespace(nx=nx, ny=ny, cp=3300.0), seed)


def generate(name: str, ref_dir: str, out_dir: str = HERE) -> str:
    prog, overrides, stf, nprocs, keep, *opt = CASES[name]
    opt = opt[0] if opt else {}
    src = os.path.join(ref_dir, PROGRAMS[prog])
    three_d = prog == "cpml3d"
    fields = FIELDS[prog]
    arrays = sorted({a for parts in fields.values() for a in parts})
    outs = ["sisvx", "sisvy", "ix_rec", "iy_rec"]
    outs += ["total_energy", "rank_cut_plane"] if three_d else ["total_energy_kinetic",
                                                               "total_energy_potential"]
    big = name.endswith("_full")
    stop = opt.get("stop", False)
    profiles = {} if big else PROFILES[prog]
    dump = outs + PARAMS[prog] + ([] if big or stop else arrays) + (["it"] if stop else []) \
        + [n for names in profiles.values() for n in names] \
        + ([] if big else ["courant_number", "xrec", "yrec"])
    t0 = time.time()
    model, load_after, inputs = None, None, None
    if "model" in opt:      # the model goes into the program's own arrays after its fill
        model = model_2d(int(overrides["NX"]), int(overrides["NY"]), opt["model"])
        if "scale" in opt:   # faster waves: lambda and mu scaled, rho kept
            model = (model[0] * np.float32(opt["scale"]), model[1] * np.float32(opt["scale"]), model[2])
        load_after = (fill_end_line(src), ["lambda", "mu", "rho"])
        # the fourth-order program's arrays are (0:NX+1, 0:NY+1): its fill
        # leaves the halo cells at their static zero, which no update reads
        pad = 1 if prog == "cpml2d4" else 0
        inputs = {k: np.pad(m.T.astype(np.float64), pad) for k, m in zip(load_after[1], model)}
    exe = ref_f90c.build(src, name, overrides, dump, bounds=not big, stf=stf,
                         load_after=load_after)
    ranks = exe.run(nprocs=nprocs, timeout=7200, inputs=inputs, allow_stop=stop)
    cut = int(ranks[0]["rank_cut_plane"]) if three_d else 0
    d = ranks[cut]
    if stop != ("stop" in d):
        raise RuntimeError(f"{name}: the run {'did not stop' if stop else 'stopped: ' + d['stop']}")
    out = {"program": np.array(PROGRAMS[prog]), "stf": np.array(stf or "program default"),
           "nprocs": np.array(nprocs),
           "overrides": np.array(repr(sorted(overrides.items())))}
    for k in PARAMS[prog]:
        out["p_" + k] = np.array(d[k])
    out["rec"] = np.stack([d["ix_rec"], d["iy_rec"]], axis=1).astype(np.int32)
    for k in ("sisvx", "sisvy"):
        tr = np.ascontiguousarray(d[k].T)
        if big:   # 64 x 2500 traces: their digest (config_3d_plain.npz holds the values)
            out["sha_" + k] = np.array(digest(tr))
        else:
            out[k] = tr
    for ax, names in profiles.items():
        out["prof_" + ax] = np.stack([d[n] for n in names])
    if not big:
        out["courant"] = np.array(d["courant_number"])
        out["rec_xy"] = np.stack([d["xrec"], d["yrec"]], axis=1)   # the targets, in metres
    if model is not None:
        out["lam"], out["mu"], out["rho"] = model
    if stop:     # where the program stopped, and why
        out["stop"], out["stop_it"] = np.array(d["stop"]), np.array(int(d["it"]))
    if three_d:
        out["energy"] = d["total_energy"]
    else:
        out["ek"] = d["total_energy_kinetic"]
        out["ep"] = d["total_energy_potential"]
    if not big and not stop:
        for fname, parts in fields.items():
            if three_d:   # local planes 1..NZ_LOCAL of every rank, in rank order
                full = np.concatenate([r[parts[0]][:, :, 1:-1] for r in ranks], axis=2)
                c = full.transpose(2, 1, 0)
            else:
                a = d[parts[0]] if len(parts) == 1 else d[parts[0]] + d[parts[1]]
                nx, ny = int(d["nx"]), int(d["ny"])
                lo = 1 if a.shape[0] == nx + 2 else 0   # 0:NX+1 arrays of the 4th-order program
                c = a[lo:lo + nx, lo:lo + ny].T
            out["sha_" + fname] = np.array(digest(c))
            if keep:
                out["f_" + fname] = np.ascontiguousarray(c)
    path = os.path.join(out_dir, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"wrote {name} in {time.time() - t0:.1f} s")
    return path


# ---------------------------------------------------------------------------
# PNM snapshots (2D:861-999; the same subroutine in all four programs)
# ---------------------------------------------------------------------------
# A driver of this project's own that hands one plane to the programs'
# create_color_image subroutine, translated from the reference source; the
# plane and the receiver indices are loaded from files before it runs.
PNM_HARNESS = """\
program pnm_harness
  implicit none
  integer, parameter :: NX = 8, NY = 8, NREC = 1, IT = 1, ISRC = 4, JSRC = 4, NPML = 2
  integer, parameter :: FIELD = 1
  logical, parameter :: UXMIN = .true., UXMAX = .true., UYMIN = .true., UYMAX = .true.
  double precision, dimension(NX,NY) :: plane
  integer, dimension(NREC) :: ix_rec, iy_rec
  call create_color_image(plane,NX,NY,IT,ISRC,JSRC,ix_rec,iy_rec,NREC,NPML, &
                          UXMIN,UXMAX,UYMIN,UYMAX,FIELD)
end program pnm_harness
"""


def pnm_cases():
    """(name, plane [ny][nx] float32, parameters, receivers) per snapshot: wavefields of the
    small reference runs and seeded planes, with sources and receivers on and
    off the frame, each PML face off in turn, both fields, and an all-zero
    plane (0/0 normalisation)."""
    g = lambda n: dict(np.load(os.path.join(HERE, n + ".npz")))  # noqa: E731
    a, b, c = g("refpin_2d_small"), g("refpin_2d4_small"), g("refpin_pml2d_small")
    rng = np.random.default_rng(7)
    syn = (rng.standard_normal((29, 37)) * 3.0).astype(np.float32)
    syn[10, 10], syn[20, 30] = 7.0, -7.0                  # the extremes: +-1 after normalising
    syn[5, 5:9] = np.float32(0.07)                        # about the 1 % cut
    out = []
    def case(name, plane, it, isrc, jsrc, npml, field, use, rec):
        out.append((name, np.ascontiguousarray(plane, np.float32),
                    dict(IT=it, ISRC=isrc, JSRC=jsrc, NPML=npml, FIELD=field, UXMIN=use[0],
                         UXMAX=use[1], UYMIN=use[2], UYMAX=use[3]), np.asarray(rec, np.int32)))
    case("vx_small", a["f_vx"], 400, int(a["p_isource"]), int(a["p_jsource"]), 10, 1, (1, 1, 1, 0),
         a["rec"])
    case("vy_corner", a["f_vy"], 400, 3, 4, 10, 2, (0, 1, 1, 1), [[4, 6], [1, 1], [40, 60]])
    case("vx_fourth", b["f_vx"], 600, int(b["p_isource"]), int(b["p_jsource"]), 7, 1, (1, 0, 0, 1),
         b["rec"])
    case("sxy_split", c["f_sxy"], 5, 30, 50, 10, 2, (1, 1, 1, 1), c["rec"])
    case("seeded", syn, 123456, 20, 14, 4, 1, (1, 1, 0, 1), [[10, 10]])
    case("zero", np.zeros((23, 19), np.float32), 0, 9, 11, 3, 2, (1, 1, 1, 1), [[2, 2], [17, 21]])
    return out


def generate_pnm(ref_dir: str, out_dir: str = HERE) -> str:
    import tempfile
    t0 = time.time()
    with tempfile.TemporaryDirectory() as tmp:
        harness = os.path.join(tmp, "pnm_harness.f90")
        with open(harness, "w") as f:
            f.write(PNM_HARNESS)
        out = {}
        for name, plane, par, rec in pnm_cases():
            ny, nx = plane.shape
            ov = {"NX": nx, "NY": ny, "NREC": len(rec)}
            ov.update({k: (".true." if v else ".false.") if k.startswith("U") else v
                       for k, v in par.items()})
            exe = ref_f90c.build(harness, "pnm_" + name, ov, (), load=["plane", "ix_rec", "iy_rec"],
                                 subroutines=[(os.path.join(ref_dir, PROGRAMS["cpml2d"]),
                                               "create_color_image")])
            fname = f"image{par['IT']:06d}_{'Vx' if par['FIELD'] == 1 else 'Vy'}.pnm"
            r = exe.run(inputs={"plane": plane.T.astype(np.float64),
                                "ix_rec": rec[:, 0].copy(), "iy_rec": rec[:, 1].copy()},
                        files=[fname])
            out[name + "_plane"] = plane
            out[name + "_rec"] = rec
            out[name + "_par"] = np.array([par[k] for k in PNM_PAR], np.int32)
            out[name + "_file"] = np.array(fname)
            out[name + "_pnm"] = np.frombuffer(r[0]["files"][fname].encode(), np.uint8)
    out["par_names"] = np.array(PNM_PAR)
    path = os.path.join(out_dir, "refpin_pnm.npz")
    np.savez_compressed(path, **out)
    print(f"wrote refpin_pnm in {time.time() - t0:.1f} s")
    return path


PNM_PAR = ["IT", "ISRC", "JSRC", "NPML", "FIELD", "UXMIN", "UXMAX", "UYMIN", "UYMAX"]


# ---------------------------------------------------------------------------
# output files: the programs' seismogram files (write_seismograms, 2D:826-857)
# and energy.dat (2D:741-746, 3D:1253-1257), written by the programs' own
# WRITE statements; the runs of refpin_2d_small and refpin_3d_2ranks
# ---------------------------------------------------------------------------
FILE_CASES = {"d2": "refpin_2d_small", "d3": "refpin_3d_2ranks", "d24": "refpin_2d4_small",
              "dpml": "refpin_pml2d_small"}
# the gnuplot scripts each program writes (2D:748-808, 3D:1258-1312, PML:560-606)
SCRIPTS = {"cpml2d": ["plot_energy", "plot_comparison", "plotgnu"],
           "cpml2d4": ["plot_energy", "plot_comparison", "plotgnu"],
           "cpml3d": ["plot_energy", "plotgnu"], "pml2d": ["plot_energy", "plotgnu"]}


def generate_files(ref_dir: str, out_dir: str = HERE) -> str:
    t0 = time.time()
    out = {}
    for key, case in FILE_CASES.items():
        prog, overrides, stf, nprocs = CASES[case][:4]
        src = os.path.join(ref_dir, PROGRAMS[prog])
        exe = ref_f90c.build(src, "files_" + case, overrides, ["nrec"], stf=stf, io=True,
                             subroutines=[(src, "write_seismograms")])
        nrec = int(dict(np.load(os.path.join(HERE, case + ".npz")))["p_nrec"])
        names = [f"{c}_file_{r:03d}.dat" for c in ("Vx", "Vy") for r in range(1, nrec + 1)]
        names += ["energy.dat"] + SCRIPTS[prog]
        r = exe.run(nprocs=nprocs, files=names)
        for n in names:
            out[f"{key}__{n.replace('.', '_')}"] = np.frombuffer(r[0]["files"][n].encode(), np.uint8)
    path = os.path.join(out_dir, "refpin_files.npz")
    np.savez_compressed(path, **out)
    print(f"wrote refpin_files in {time.time() - t0:.1f} s")
    return path


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=ref_f90c.DEFAULT_REF_DIR)
    ap.add_argument("names", nargs="*")
    a = ap.parse_args()
    for n in a.names or list(CASES) + ["refpin_pnm", "refpin_files"]:
        if n == "refpin_pnm":
            generate_pnm(a.ref_dir)
        elif n == "refpin_files":
            generate_files(a.ref_dir)
        else:
            generate(n, a.ref_dir)


if __name__ == "__main__":
    main()
