"""CPU checks of the C ABI library (libcpml.so): it loads, exports every entry
point include/cpml.h declares, and its host-only entry points (parameter
blocks, Courant number, receiver placement, FP64 profiles, validation, output
writers) behave like the reference. No compute call is made without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle_c, oracle_np
from seismic_cpml_gb300 import lib as L
from seismic_cpml_gb300 import params as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


@pytest.fixture(scope="module")
def lib():
    from seismic_cpml_gb300.build import build
    build()
    return L.load()


def header_functions():
    txt = open(os.path.join(ROOT, "include", "cpml.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cpml_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in L.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_fortran_binding_module_matches_the_library(lib):
    """include/cpml_gpu.f90 (not compiled here: no Fortran compiler): every
    function it binds is exported, and its cpml_params type lists the C
    struct's fields in order with the same kinds and array lengths."""
    src = open(os.path.join(ROOT, "include", "cpml_gpu.f90")).read().lower()
    names = re.findall(r"(?:function|subroutine)\s+(cpml_\w+)\s*\(", src)
    assert len(names) > 30
    for n in names:
        assert hasattr(lib, n), n
    body = src[src.index("type, bind(c) :: cpml_params"):src.index("end type")]
    fields = []
    for line in body.splitlines()[1:]:
        if "::" not in line:
            continue
        kind = "int" if "integer(c_int32_t)" in line else "double"
        for item in line.split("::")[1].split(","):
            item = item.strip()
            m = re.match(r"(\w+)(?:\((\d+)\))?", item)
            fields.append((m.group(1), kind, int(m.group(2) or 1)))
    want = []
    for name, ctype in P.CpmlParams._fields_:
        n = getattr(ctype, "_length_", 1)
        base = ctype._type_ if hasattr(ctype, "_length_") else ctype
        want.append((name, "int" if base is ctypes.c_int32 else "double", n))
    assert fields == want


def test_default_parameter_blocks_match_the_mirror(lib):
    for fn, mirror in ((lib.cpml_params_default_2d, P.default_2d),
                       (lib.cpml_params_default_3d, P.default_3d),
                       (lib.cpml_params_default_2d_fourth, P.default_2d_fourth),
                       (lib.cpml_params_default_2d_split, P.default_2d_split)):
        c = P.CpmlParams()
        assert fn(ctypes.byref(c)) == 0
        m = mirror()
        for name, _ in P.CpmlParams._fields_:
            a, b = getattr(c, name), getattr(m, name)
            if hasattr(a, "__len__"):
                a, b = list(a), list(b)
            assert a == b, name


def test_courant_and_nearest_gridpoint(lib):
    p = P.default_2d()
    assert abs(lib.cpml_courant(ctypes.byref(p), p.cp) - p.courant()) < 1e-15
    assert abs(p.courant() - 0.9333809511662428) < 1e-12        # 2D:513 with the defaults
    i, j = ctypes.c_int(), ctypes.c_int()
    rng = np.random.default_rng(1)
    for _ in range(5):
        x, y = rng.uniform(0, 1000), rng.uniform(0, 6400)
        assert lib.cpml_nearest_gridpoint(101, 641, 10.0, 10.0, x, y, ctypes.byref(i), ctypes.byref(j)) == 0
        assert (i.value, j.value) == oracle_np.nearest_gridpoint(101, 641, 10.0, 10.0, x, y)


def test_pml_profile_matches_oracle(lib):
    p = P.default_3d()
    p.nx, p.ny, p.nz = 40, 50, 60
    for axis, n in enumerate((p.nx, p.ny, p.nz)):
        arrs = [np.zeros(n) for _ in range(10)]
        assert lib.cpml_pml_profile(ctypes.byref(p), axis, n, *[a.ctypes.data_as(_dp) for a in arrs]) == 0
        ref = oracle_c.profile(p, axis)
        keys = ["d", "K", "alpha", "a", "b", "d_half", "K_half", "alpha_half", "a_half", "b_half"]
        for q, k in enumerate(keys):
            assert np.array_equal(arrs[q], ref[k]), (axis, k)


@pytest.mark.parametrize("program", ["fourth_order", "split_pml"])
def test_pml_profile_of_the_other_2d_programs(lib, program):
    """The host profile entry point follows each program's own profile: the
    fourth-order y origin (2D4:401) and the split-field damping divided by two
    (PML:180-250), against both oracle restatements."""
    p = P.default_2d_fourth() if program == "fourth_order" else P.default_2d_split()
    for axis, n in enumerate((p.nx, p.ny)):
        arrs = [np.zeros(n) for _ in range(10)]
        assert lib.cpml_pml_profile(ctypes.byref(p), axis, n, *[a.ctypes.data_as(_dp) for a in arrs]) == 0
        if program == "fourth_order":
            ref = oracle_c.profile(p, axis)
            keys = ["d", "K", "alpha", "a", "b", "d_half", "K_half", "alpha_half", "a_half", "b_half"]
            for q, k in enumerate(keys):
                assert np.array_equal(arrs[q], ref[k]), (axis, k)
            pn = oracle_np.pml_profile(n, 10.0, p.npoints_pml, True, True, p.cp, p.f0, p.deltat,
                                       high_origin_cells=n if axis == 1 else None)
            assert np.allclose(arrs[0], pn["d"], rtol=1e-14, atol=0)
        else:
            f, g = oracle_np.split_profile(n, 10.0, p.npoints_pml, p.cp, p.rcoef)
            assert np.allclose(arrs[0], f, rtol=1e-14, atol=0) and np.allclose(arrs[5], g, rtol=1e-14, atol=0)
            assert np.all(arrs[1] == 1.0) and np.all(arrs[3] == 0.0) and f[0] > 0 and f[50] == 0


def test_create_validates_the_other_2d_programs(lib):
    h = ctypes.c_void_p()
    for mk, field, value in ((P.default_2d_fourth, "order", 3), (P.default_2d_split, "scheme", 2),
                             (P.default_2d_split, "deltay", 12.0), (P.default_2d_split, "order", 4),
                             (P.default_3d, "order", 4), (P.default_3d, "scheme", 1)):
        q = mk()
        setattr(q, field, value)
        assert lib.cpml_create(ctypes.byref(q), ctypes.byref(h)) == -1, (mk.__name__, field)


def test_strerror_covers_all_codes(lib):
    for code in range(0, -10, -1):
        assert lib.cpml_strerror(code).decode() not in ("", "unknown status")
    assert lib.cpml_strerror(-99).decode() == "unknown status"


def test_create_validates_before_touching_the_device(lib):
    h = ctypes.c_void_p()
    p = P.default_2d()
    p.deltat = 4e-3                     # Courant 1.87 > 1: the reference stops (2D:516)
    assert lib.cpml_create(ctypes.byref(p), ctypes.byref(h)) == -2
    for field, value in (("nx", 2), ("npoints_pml", 0), ("isource", 0), ("ndim", 4), ("rcoef", 1.5),
                         ("it_display", 0), ("stf", 3), ("stf", -1)):
        q = P.default_2d()
        setattr(q, field, value)
        assert lib.cpml_create(ctypes.byref(q), ctypes.byref(h)) == -1, field
    assert lib.cpml_create(None, ctypes.byref(h)) == -1


def test_batch_create_validates_before_touching_the_device(lib):
    """Every shot is checked first; the batched engine runs the second-order
    C-PML program only, so fourth-order and split-field shots are refused
    rather than run as another program."""
    b = ctypes.c_void_p()
    ok = P.default_2d()
    for field, value in (("stf", 5), ("order", 4), ("scheme", P.SCHEME_SPLIT), ("isource", 0)):
        q = P.default_2d()
        setattr(q, field, value)
        arr = (P.CpmlParams * 2)(ok, q)
        assert lib.cpml_batch_create(2, arr, ctypes.byref(b)) == -1, field
    q = P.default_2d()
    q.deltat = 4e-3
    assert lib.cpml_batch_create(1, (P.CpmlParams * 1)(q), ctypes.byref(b)) == -2


def test_create_without_gpu_reports_cuda(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    p = P.default_2d()
    assert lib.cpml_create(ctypes.byref(p), ctypes.byref(h)) == -6


def test_noalloc_rejects_oversize_before_any_device_call(lib):
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    assert lib.cpml_energy3d_noalloc(ptrs, 8, 8, 9000, 8, 2, 1e9, 1e9, 2e3, None, None, None, 0,
                                     1, None) == -9
    assert lib.cpml_energy3d_noalloc(None, 8, 8, 8, 8, 2, 1e9, 1e9, 2e3, None, None, None, 0,
                                     1, None) == -1


@pytest.mark.parametrize("dims", [(1, 8, 30), (8, 4, 30), (8, 8, 4), (20, 20, 20)])
def test_noalloc_rejects_an_empty_energy_interior(lib, dims):
    """2*npml >= nx, ny or nz leaves no interior cell: CPML_ERR_INVALID before
    any device call (the fake pointers are never dereferenced)."""
    nx, ny, nz = dims
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    assert lib.cpml_energy3d_noalloc(ptrs, nx, ny, nz, nx, 10 if nx == 20 else 2, 1e9, 1e9, 2e3,
                                     None, None, None, 0, 1, None) == -1


def test_noalloc_rejects_a_partial_model_triple(lib):
    ptrs = (ctypes.c_void_p * 9)(*([1] * 9))
    for cells in ((1, None, None), (None, 1, None), (1, 1, None), (None, None, 1)):
        assert lib.cpml_energy3d_noalloc(ptrs, 8, 8, 8, 8, 2, 1e9, 1e9, 2e3, *cells, 0, 1, None) == -1


def test_su_seismogram_writer(lib, tmp_path):
    """seisVx.su / seisVy.su / seisVz.su: per receiver 120 int16 header words
    (word 58 = samples, word 59 = interval in microseconds) and the samples as
    REAL(4), the layout of the reference's SU output."""
    nt, nrec, dt = 11, 3, 4.0e-4
    vx = np.arange(nt * nrec, dtype=np.float64).reshape(nrec, nt) * 1e-3 - 0.01
    vy, vz = -vx, 2.0 * vx
    d = str(tmp_path).encode()
    assert lib.cpml_write_seismograms_su(d, vx.ctypes.data_as(_dp), vy.ctypes.data_as(_dp),
                                         vz.ctypes.data_as(_dp), nt, nrec, dt) == 0
    rec_t = np.dtype([("head", "<i2" if np.little_endian else ">i2", (120,)), ("data", "=f4", (nt,))])
    for name, ref in (("seisVx.su", vx), ("seisVy.su", vy), ("seisVz.su", vz)):
        raw = (tmp_path / name).read_bytes()
        assert len(raw) == nrec * (240 + 4 * nt)
        recs = np.frombuffer(raw, dtype=rec_t)
        assert np.all(recs["head"][:, 57] == nt) and np.all(recs["head"][:, 58] == 400)
        assert np.count_nonzero(recs["head"]) == 2 * nrec
        assert np.array_equal(recs["data"], ref.astype(np.float32))
    assert lib.cpml_write_seismograms_su(d, vx.ctypes.data_as(_dp), vy.ctypes.data_as(_dp), None,
                                         40000, 1, dt) == -9


def test_seismogram_and_energy_writers(lib, tmp_path):
    nt, nrec, dt = 7, 2, 2e-3
    vx = np.arange(nt * nrec, dtype=np.float64).reshape(nrec, nt) * 1e-3 - 0.004
    vy = -vx
    d = str(tmp_path).encode()
    assert lib.cpml_write_seismograms(d, vx.ctypes.data_as(_dp), vy.ctypes.data_as(_dp), None,
                                      nt, nrec, dt) == 0
    for r in range(nrec):
        for comp, ref in (("Vx", vx), ("Vy", vy)):
            arr = np.loadtxt(tmp_path / f"{comp}_file_{r + 1:03d}.dat")
            assert arr.shape == (nt, 2)
            assert np.allclose(arr[:, 0], np.arange(nt) * dt, rtol=1e-6)
            assert np.allclose(arr[:, 1], ref[r], rtol=1e-6, atol=1e-12)
    assert not (tmp_path / "Vz_file_001.dat").exists()
    ek = np.linspace(1, 2, nt)
    ep = np.linspace(3, 4, nt)
    assert lib.cpml_write_energy(d, ek.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), nt, dt, 4) == 0
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape == (nt, 4) and np.allclose(e[:, 3], ek + ep, rtol=1e-6)
    assert lib.cpml_write_energy(d, ek.ctypes.data_as(_dp), ep.ctypes.data_as(_dp), nt, dt, 2) == 0
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape == (nt, 2) and np.allclose(e[:, 1], ek + ep, rtol=1e-12)


def test_pnm_writer_follows_the_colour_rules(lib, tmp_path):
    nx, ny = 30, 40
    data = np.zeros((ny, nx), np.float32)
    data[20, 15] = 1.0                 # positive peak -> red 255
    data[25, 15] = -0.5                # negative -> blue
    data[22, 22] = 0.001               # below the 1 % cut -> white
    ix = np.array([5], np.int32)
    iy = np.array([30], np.int32)
    use = np.array([1, 1, 1, 1], np.int32)
    assert lib.cpml_write_pnm(str(tmp_path).encode(), data.ctypes.data_as(_fp), nx, ny, 100,
                              15, 10, ix.ctypes.data_as(_ip), iy.ctypes.data_as(_ip), 1, 4,
                              use.ctypes.data_as(_ip), 1) == 0
    tok = (tmp_path / "image000100_Vx.pnm").read_text().split()
    assert tok[0] == "P3" and tok[1:4] == ["30", "40", "255"]
    px = np.array(tok[4:], int).reshape(ny, nx, 3)   # rows from the top (iy = NY first)
    row = lambda iy1: ny - iy1                       # 1-based iy -> row index
    assert tuple(px[row(21), 15]) == (255, 0, 0)     # data[20, 15] is (ix=16, iy=21)
    assert px[row(26), 15][2] == round(255 * 0.5 ** 0.3) and px[row(26), 15][0] == 0
    assert tuple(px[row(23), 22]) == (255, 255, 255)
    assert tuple(px[row(10), 15]) == (255, 157, 0)   # source cross at (15, 10)
    assert tuple(px[row(30), 5]) == (30, 180, 60)    # receiver square
    assert tuple(px[0, 0]) == (0, 0, 0)              # frame


def test_split_program_courant_check_is_its_own(lib):
    """The split-field program checks cp * DELTAT / h (PML:304): 0.9 passes
    that check (its 2D number is 1.27) and goes on to the device, 1.1 stops."""
    h = ctypes.c_void_p()
    p = P.default_2d_split()
    p.deltat = 0.9 * p.deltax / p.cp
    st = lib.cpml_create(ctypes.byref(p), ctypes.byref(h))
    assert st != -2
    if st == 0:
        lib.cpml_destroy(h)
    p.deltat = 1.1 * p.deltax / p.cp
    assert lib.cpml_create(ctypes.byref(p), ctypes.byref(h)) == -2
