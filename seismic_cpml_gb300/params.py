"""Python mirror of ``cpml_params`` (include/cpml.h) and the reference's
parameter blocks.

The reference programs are configured by editing compile-time Fortran
``parameter`` constants (seismic_CPML_2D_isotropic_second_order.f90:138-218,
seismic_CPML_3D_isotropic_MPI_OpenMP.f90:124-218). Here the same constants are
fields of a C struct passed to ``cpml_create``; the field names follow the
Fortran names.
"""
from __future__ import annotations

import ctypes
import math

STF_DGAUSSIAN, STF_GAUSSIAN, STF_RICKER = 0, 1, 2
SCHEME_CPML, SCHEME_SPLIT = 0, 1
FLAG_ENERGY, FLAG_EP_PHYSICAL, FLAG_NO_STABILITY = 0x1, 0x2, 0x4

FIELDS = {"vx": 0, "vy": 1, "vz": 2, "sxx": 3, "syy": 4, "szz": 5,
          "sxy": 6, "sxz": 7, "syz": 8}


class CpmlParams(ctypes.Structure):
    """Byte-for-byte twin of ``struct cpml_params``."""
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("nstep", ctypes.c_int32),
        ("npoints_pml", ctypes.c_int32),
        ("use_pml", ctypes.c_int32 * 6),
        ("isource", ctypes.c_int32), ("jsource", ctypes.c_int32), ("ksource", ctypes.c_int32),
        ("stf", ctypes.c_int32),
        ("it_display", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("scheme", ctypes.c_int32),
        ("reserved_i", ctypes.c_int32 * 2),
        ("deltax", ctypes.c_double), ("deltay", ctypes.c_double), ("deltaz", ctypes.c_double),
        ("deltat", ctypes.c_double),
        ("cp", ctypes.c_double), ("cs", ctypes.c_double), ("rho", ctypes.c_double),
        ("f0", ctypes.c_double), ("t0", ctypes.c_double), ("factor", ctypes.c_double),
        ("angle_force", ctypes.c_double),
        ("npower", ctypes.c_double),
        ("k_max_pml", ctypes.c_double),
        ("alpha_max_pml", ctypes.c_double),
        ("rcoef", ctypes.c_double),
        ("reserved_d", ctypes.c_double * 4),
    ]

    def copy(self) -> "CpmlParams":
        c = CpmlParams()
        ctypes.pointer(c)[0] = self
        return c

    @property
    def ncell(self) -> int:
        return self.nx * self.ny * (self.nz if self.ndim == 3 else 1)

    def courant(self, cp_max: float | None = None) -> float:
        """Courant number (2D:513, 3D:712)."""
        cp = self.cp if cp_max is None else cp_max
        s = 1.0 / self.deltax ** 2 + 1.0 / self.deltay ** 2
        if self.ndim == 3:
            s += 1.0 / self.deltaz ** 2
        return cp * self.deltat * math.sqrt(s)

    def __repr__(self) -> str:  # pragma: no cover - debugging aid
        keys = [f[0] for f in self._fields_ if not f[0].startswith("reserved")]
        out = []
        for k in keys:
            v = getattr(self, k)
            if k == "use_pml":
                v = list(v)
            out.append(f"{k}={v}")
        return "CpmlParams(" + ", ".join(out) + ")"


def default_2d() -> CpmlParams:
    """The 2D program's parameter block (2D:138-218)."""
    p = CpmlParams()
    p.ndim = 2
    p.nx, p.ny, p.nz = 101, 641, 1
    p.deltax = p.deltay = p.deltaz = 10.0
    p.use_pml[:] = [1, 1, 1, 1, 0, 0]
    p.npoints_pml = 10
    p.cp = 3300.0
    p.cs = 3300.0 / 1.732
    p.rho = 2800.0
    p.nstep = 2000
    p.deltat = 2.0e-3
    p.f0 = 7.0
    p.t0 = 1.20 / p.f0
    p.factor = 1.0e7
    p.isource = p.nx - 2 * p.npoints_pml - 1          # 2D:171
    p.jsource = 2 * p.ny // 3 + 1                      # 2D:172
    p.ksource = 1
    p.angle_force = 135.0
    p.stf = STF_DGAUSSIAN
    p.it_display = 100
    p.flags = FLAG_ENERGY
    p.npower = 2.0
    p.k_max_pml = 1.0
    p.alpha_max_pml = -1.0            # => 2*pi*(f0/2) (2D:218)
    p.rcoef = 0.001
    return p


def default_2d_fourth() -> CpmlParams:
    """seismic_CPML_2D_isotropic_fourth_order.f90:132-190: the second-order
    program's block with the 27/24 fourth-order operator, DELTAT halved and
    NSTEP, IT_DISPLAY doubled."""
    p = default_2d()
    p.order = 4
    p.nstep = 2000 * 2
    p.deltat = 2.0e-3 / 2
    p.it_display = 100 * 2
    return p


def default_2d_split() -> CpmlParams:
    """seismic_PML_Collino_2D_isotropic.f90:96-141: classical split-field PML,
    homogeneous, h = 10 m, 2000 steps of 2 ms, first derivative of a
    Gaussian at (80, 428), 135 degrees."""
    p = default_2d()
    p.scheme = SCHEME_SPLIT
    return p


def default_3d() -> CpmlParams:
    """The 3D program's parameter block (3D:124-218), one domain of NZ planes,
    source and receivers on global plane NZ/2."""
    p = default_2d()
    p.ndim = 3
    p.nx, p.ny, p.nz = 101, 641, 640
    p.use_pml[:] = [1, 1, 1, 1, 1, 1]
    p.nstep = 2500
    p.deltat = 1.6e-3
    p.isource = p.nx - 2 * p.npoints_pml - 1
    p.jsource = 2 * p.ny // 3 + 1
    p.ksource = p.nz // 2
    return p


def reference_receivers_2d(p: CpmlParams, nrec: int = 2):
    """Receiver targets in metres of 2D:180-183 / 3D:175-178, on the line from
    (xsource-100, 2300) to (xsource, 300), resolved to grid points by the
    reference's nearest-point rule."""
    xsource = (p.isource - 1) * p.deltax
    xdeb, ydeb, xfin, yfin = xsource - 100.0, 2300.0, xsource, 300.0
    xs = (xfin - xdeb) / float(nrec - 1)
    ys = (yfin - ydeb) / float(nrec - 1)
    out = []
    for r in range(nrec):
        x = xdeb + float(r) * xs
        y = ydeb + float(r) * ys
        out.append(nearest_gridpoint(p.nx, p.ny, p.deltax, p.deltay, x, y))
    return out


def nearest_gridpoint(nx, ny, dx, dy, x, y):
    """First grid point at minimum distance in i-fastest order (2D:486-509).
    Closed form of the brute-force scan: the scan's winner is the smallest
    (j, i) whose distance equals the minimum; separable rounding with ties to
    the lower index gives that point."""
    def axis(n, d, v):
        best, bd = 1, None
        for i in range(1, n + 1):
            dd = abs(d * float(i - 1) - v)
            if bd is None or dd < bd:
                best, bd = i, dd
        return best
    # brute force in the same order as the reference for exact tie rules
    dist = 1.0e30
    bi, bj = 1, 1
    ci, cj = axis(nx, dx, x), axis(ny, dy, y)
    # the minimum lies within one cell of the separable minimum; scan a
    # neighbourhood in reference order to keep the first-minimum rule exact
    for j in range(max(1, cj - 2), min(ny, cj + 2) + 1):
        for i in range(max(1, ci - 2), min(nx, ci + 2) + 1):
            dv = math.sqrt((dx * float(i - 1) - x) ** 2 + (dy * float(j - 1) - y) ** 2)
            if dv < dist:
                dist, bi, bj = dv, i, j
    return bi, bj


# ---------------------------------------------------------------------------
# Benchmark workloads (synthetic, seeded)
# ---------------------------------------------------------------------------
def config_2d_plain() -> tuple[CpmlParams, list]:
    """2D plain: 101 x 641, 10-point PML on all edges but the top (y max),
    homogeneous cp=3300, Ricker f0=7 Hz at (NX/2, NY/2), 45 degrees, 2000
    steps; receivers by the reference's rule relative to this source."""
    p = default_2d()
    p.use_pml[:] = [1, 1, 1, 0, 0, 0]
    p.isource = p.nx // 2 + 1        # 1-based centre (51, 321)
    p.jsource = p.ny // 2 + 1
    p.angle_force = 45.0
    p.stf = STF_RICKER
    return p, reference_receivers_2d(p)


def config_3d_plain(n_interior: int = 256, nstep: int = 2500) -> tuple[CpmlParams, list]:
    """3D plain: (256 + 2*10)^3, DELTA=10 m, homogeneous cp=3300, DELTAT=1.6 ms,
    2500 steps, Ricker f0=7 Hz at the centre, 135 degrees in x-y, 64 receivers
    on the x line through the centre."""
    p = default_3d()
    n = n_interior + 2 * p.npoints_pml
    p.nx = p.ny = p.nz = n
    p.nstep = nstep
    p.deltat = 1.6e-3
    p.stf = STF_RICKER
    c = n // 2
    p.isource = p.jsource = p.ksource = c
    nrec = 64
    rec = []
    for r in range(nrec):
        i = p.npoints_pml + 1 + int(round(r * (n_interior - 1) / (nrec - 1)))
        rec.append((i, c, c))
    return p, rec


def config_3d_large(n_interior: int = 800, nstep: int = 4000, deltat: float = 4.0e-4,
                    nrec_side: int = 201) -> tuple[CpmlParams, list]:
    """3D large: (800 + 2*10)^3, DELTA = 5 m, Ricker f0 = 12 Hz at the
    centre, NSTEP = 4000, a 201 x 201 receiver grid on the plane one below
    the top interior plane in y (y is the vertical axis), at i, k = 11 + 4 m.
    The per-cell layered model comes from earth.layered_model_3d_device.
    DELTAT is 0.4 ms: with cp up to 5000 m/s and +15 % anomalies, 0.8 ms
    would give a Courant number of 1.39-1.59 and the reference's check
    (3D:712-717) would stop."""
    p = default_3d()
    n = n_interior + 2 * p.npoints_pml
    p.nx = p.ny = p.nz = n
    p.deltax = p.deltay = p.deltaz = 5.0
    p.nstep = nstep
    p.deltat = deltat
    p.stf = STF_RICKER
    p.f0 = 12.0
    p.t0 = 1.2 / p.f0
    p.cp = 5000.0 * 1.15             # C-PML d0 and the Courant check use the fastest cp
    p.cs = p.cp / 1.7320508075688772
    p.rho = 310.0 * p.cp ** 0.25
    c = n // 2
    p.isource, p.jsource, p.ksource = c, c, c
    p.it_display = 100
    jr = n - p.npoints_pml - 1                       # 1-based
    step = (n_interior - 1) / (nrec_side - 1)
    idx = [p.npoints_pml + 1 + int(round(m * step)) for m in range(nrec_side)]
    rec = [(i, jr, k) for k in idx for i in idx]
    return p, rec


def small_2d(nx=48, ny=64, nstep=300) -> tuple[CpmlParams, list]:
    """A small 2D case that finishes in seconds on the oracles."""
    p = default_2d()
    p.nx, p.ny, p.nstep = nx, ny, nstep
    p.npoints_pml = 8
    p.isource = nx // 2
    p.jsource = ny // 2 + 3
    p.deltat = 1.5e-3
    p.f0 = 12.0
    p.t0 = 1.2 / p.f0
    p.it_display = 50
    rec = [(nx // 2 - 5, ny // 2 - 10), (12, 15), (nx - 12, ny - 14)]
    return p, rec


def small_3d(n=(28, 24, 20), nstep=120) -> tuple[CpmlParams, list]:
    """A small 3D case that finishes in seconds on the oracles."""
    p = default_3d()
    p.nx, p.ny, p.nz = n
    p.nstep = nstep
    p.npoints_pml = 5
    p.deltat = 1.2e-3
    p.f0 = 15.0
    p.t0 = 1.2 / p.f0
    p.isource, p.jsource, p.ksource = n[0] // 2, n[1] // 2 + 1, n[2] // 2
    p.it_display = 40
    rec = [(n[0] // 2 - 4, n[1] // 2, n[2] // 2), (7, 8, 9), (n[0] - 7, n[1] - 6, n[2] // 2 + 2)]
    return p, rec
