"""Vectorised numpy restatement of the two reference programs.

TEST INFRASTRUCTURE ONLY. This module is an oracle: the tests, the smoke
check and the CPU-baseline leg of the benchmark use it as a checker. The
product never imports it, calls it or falls back to it.

It restates, loop nest by loop nest, the time loop of
  seismic_CPML_2D_isotropic_second_order.f90      (2D:283-744)
  seismic_CPML_3D_isotropic_MPI_OpenMP.f90        (3D:399-1180)
with the index ranges and operation order of the Fortran, on 0-based numpy
arrays laid out [j, i] (2D) and [k, j, i] (3D), i fastest (the Fortran memory
order). Every loop of the reference updates cells that no other iteration of
the same loop reads, so each loop nest is one vectorised slice expression.

The 3D program is restated with single-domain semantics: one domain of NZ
planes equals the union of the MPI slabs (3D:771-796 exchange one halo plane
per field before each half step; k2begin/kminus1end trim the global first and
last plane), with the source and receivers on global plane k = NZ/2 (the last
local plane of rank nb_procs/2-1, 3D:346, 1080-1081, 1126-1127).

Parity of this restatement is cross-checked against the independent C++
restatement in oracle/cpml_oracle.cpp, and both are checked against the
reference programs' own statements. oracle/ref_f90c.py translated those
from their Fortran source and gcc ran them (tests/test_ref_pin.py). This
file reproduces their seismograms bit for bit, and their energies to
summation order.

`dtype=np.float32` runs the identical algorithm in single precision (profiles
still built in float64 and rounded), which measures the FP32 rounding floor
that any FP32 implementation inherits.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PI = 3.141592653589793238462643
STF_DGAUSSIAN, STF_GAUSSIAN, STF_RICKER = 0, 1, 2
FLAG_ENERGY, FLAG_EP_PHYSICAL = 0x1, 0x2


# ---------------------------------------------------------------------------
# C-PML profiles: 2D:283-465 (x and y), 3D:560-667 (z). FP64 host loops.
# ---------------------------------------------------------------------------
def pml_profile(n, delta, npml, use_min, use_max, cp, f0, deltat,
                npower=2.0, k_max=1.0, alpha_max=None, rcoef=0.001, high_origin_cells=None):
    """Return dict of d, K, alpha, a, b and their *_half twins (length n).
    high_origin_cells: the high-side origin sits at that many cells minus the
    thickness (default n - 1; the fourth-order program's y axis uses n,
    2D4:401)."""
    if alpha_max is None or alpha_max < 0:
        alpha_max = 2.0 * PI * (f0 / 2.0)                       # 2D:218
    thickness = npml * delta                                   # 2D:285
    d0 = -(npower + 1) * cp * math.log(rcoef) / (2.0 * thickness)  # 2D:296
    d = np.zeros(n); dh = np.zeros(n)
    K = np.ones(n); Kh = np.ones(n)
    al = np.zeros(n); alh = np.zeros(n)
    a = np.zeros(n); ah = np.zeros(n)
    b = np.zeros(n); bh = np.zeros(n)
    origin_left = thickness
    origin_right = ((n - 1) if high_origin_cells is None else high_origin_cells) * delta - thickness
    for i in range(1, n + 1):
        val = delta * float(i - 1)
        ii = i - 1
        if use_min:                                            # 2D:329-351
            absc = origin_left - val
            if absc >= 0.0:
                nrm = absc / thickness
                d[ii] = d0 * nrm ** npower
                K[ii] = 1.0 + (k_max - 1.0) * nrm ** npower
                al[ii] = alpha_max * (1.0 - nrm)
            absc = origin_left - (val + delta / 2.0)
            if absc >= 0.0:
                nrm = absc / thickness
                dh[ii] = d0 * nrm ** npower
                Kh[ii] = 1.0 + (k_max - 1.0) * nrm ** npower
                alh[ii] = alpha_max * (1.0 - nrm)
        if use_max:                                            # 2D:354-376
            absc = val - origin_right
            if absc >= 0.0:
                nrm = absc / thickness
                d[ii] = d0 * nrm ** npower
                K[ii] = 1.0 + (k_max - 1.0) * nrm ** npower
                al[ii] = alpha_max * (1.0 - nrm)
            absc = val + delta / 2.0 - origin_right
            if absc >= 0.0:
                nrm = absc / thickness
                dh[ii] = d0 * nrm ** npower
                Kh[ii] = 1.0 + (k_max - 1.0) * nrm ** npower
                alh[ii] = alpha_max * (1.0 - nrm)
        if al[ii] < 0.0:                                       # 2D:383-384
            al[ii] = 0.0
        if alh[ii] < 0.0:
            alh[ii] = 0.0
        b[ii] = math.exp(-(d[ii] / K[ii] + al[ii]) * deltat)   # 2D:386-387
        bh[ii] = math.exp(-(dh[ii] / Kh[ii] + alh[ii]) * deltat)
        if abs(d[ii]) > 1e-6:                                  # 2D:390-392
            a[ii] = d[ii] * (b[ii] - 1.0) / (K[ii] * (d[ii] + K[ii] * al[ii]))
        if abs(dh[ii]) > 1e-6:
            ah[ii] = dh[ii] * (bh[ii] - 1.0) / (Kh[ii] * (dh[ii] + Kh[ii] * alh[ii]))
    return dict(d=d, K=K, alpha=al, a=a, b=b,
                d_half=dh, K_half=Kh, alpha_half=alh, a_half=ah, b_half=bh)


def source_term(p, it):
    """Source time function at step it (1-based), 2D:644-654 / 3D:1058-1072."""
    a = PI * PI * p.f0 * p.f0
    t = float(it - 1) * p.deltat
    tt = t - p.t0
    if p.stf == STF_GAUSSIAN:
        return p.factor * math.exp(-a * tt ** 2)
    if p.stf == STF_RICKER:
        return p.factor * (1.0 - 2.0 * a * tt ** 2) * math.exp(-a * tt ** 2)
    return -p.factor * 2.0 * a * tt * math.exp(-a * tt ** 2)


def nearest_gridpoint(nx, ny, dx, dy, x, y):
    """Brute-force nearest grid point, first minimum in i-fastest order
    (2D:486-509). Returns 1-based (i, j)."""
    dist = 1.0e30
    best = (1, 1)
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            dv = math.sqrt((dx * float(i - 1) - x) ** 2 + (dy * float(j - 1) - y) ** 2)
            if dv < dist:
                dist = dv
                best = (i, j)
    return best


@dataclass
class Result:
    sisvx: np.ndarray            # [nrec, nstep]
    sisvy: np.ndarray
    sisvz: np.ndarray | None
    ek: np.ndarray               # [nstep]
    ep: np.ndarray
    fields: dict = field(default_factory=dict)
    vmax: list = field(default_factory=list)   # (it, max|v|) at display steps


def _prof(p, axis, n, delta, dt_np):
    pr = pml_profile(n, delta, p.npoints_pml, bool(p.use_pml[2 * axis]),
                     bool(p.use_pml[2 * axis + 1]), p.cp, p.f0, p.deltat,
                     p.npower, p.k_max_pml, p.alpha_max_pml, p.rcoef)
    return {k: v.astype(dt_np) for k, v in pr.items()}


# ---------------------------------------------------------------------------
# 2D time loop: 2D:550-735
# ---------------------------------------------------------------------------
def run2d(p, nsteps=None, lam=None, mu=None, rho=None, rec=None,
          dtype=np.float64, keep_fields=False):
    """Run the 2D program. lam/mu/rho: [ny, nx] arrays (default homogeneous,
    2D:468-474). rec: list of 1-based (ix, iy)."""
    T = np.dtype(dtype).type
    NX, NY = p.nx, p.ny
    nsteps = p.nstep if nsteps is None else nsteps
    if rho is None:
        rho = np.full((NY, NX), p.rho)
    if mu is None:
        mu = np.full((NY, NX), p.rho * p.cs * p.cs)
    if lam is None:
        lam = np.full((NY, NX), p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs))
    lam = np.asarray(lam, dtype); mu = np.asarray(mu, dtype); rho = np.asarray(rho, dtype)
    px = _prof(p, 0, NX, p.deltax, dtype)
    py = _prof(p, 1, NY, p.deltay, dtype)
    DX, DY, DT = T(p.deltax), T(p.deltay), T(p.deltat)
    half, two, quarter = T(0.5), T(2.0), T(0.25)

    z = lambda: np.zeros((NY, NX), dtype)
    vx, vy, sxx, syy, sxy = z(), z(), z(), z(), z()
    m_dvx_dx, m_dvx_dy, m_dvy_dx, m_dvy_dy = z(), z(), z(), z()
    m_dsxx_dx, m_dsyy_dy, m_dsxy_dx, m_dsxy_dy = z(), z(), z(), z()
    rec = rec or []
    nrec = len(rec)
    sisvx = np.zeros((nrec, nsteps)); sisvy = np.zeros((nrec, nsteps))
    ek = np.zeros(nsteps); ep = np.zeros(nsteps)
    vmax = []

    bx, ax, Kx = px["b"][None, :], px["a"][None, :], px["K"][None, :]
    bxh, axh, Kxh = px["b_half"][None, :], px["a_half"][None, :], px["K_half"][None, :]
    by, ay, Ky = py["b"][:, None], py["a"][:, None], py["K"][:, None]
    byh, ayh, Kyh = py["b_half"][:, None], py["a_half"][:, None], py["K_half"][:, None]

    # staggered material, constant over time (2D:559-562, 586, 627)
    lam_hx = half * (lam[1:, 1:] + lam[1:, :-1])
    mu_hx = half * (mu[1:, 1:] + mu[1:, :-1])
    l2m_hx = lam_hx + two * mu_hx
    mu_hy = half * (mu[1:, 1:] + mu[:-1, 1:])
    rho_hxhy = quarter * (rho[:-1, :-1] + rho[:-1, 1:] + rho[1:, 1:] + rho[1:, :-1])
    npml = p.npoints_pml
    isrc, jsrc = p.isource - 1, p.jsource - 1
    ang = p.angle_force * (PI / 180.0)

    for it in range(1, nsteps + 1):
        # sigma_xx, sigma_yy: j=2..NY, i=1..NX-1 (2D:556-580)
        R = (slice(1, NY), slice(0, NX - 1))
        dvx_dx = (vx[1:, 1:] - vx[1:, :-1]) / DX
        dvy_dy = (vy[1:, :-1] - vy[:-1, :-1]) / DY
        m_dvx_dx[R] = bxh[:, :-1] * m_dvx_dx[R] + axh[:, :-1] * dvx_dx
        m_dvy_dy[R] = by[1:] * m_dvy_dy[R] + ay[1:] * dvy_dy
        dvx_dx = dvx_dx / Kxh[:, :-1] + m_dvx_dx[R]
        dvy_dy = dvy_dy / Ky[1:] + m_dvy_dy[R]
        sxx[R] = sxx[R] + (l2m_hx * dvx_dx + lam_hx * dvy_dy) * DT
        syy[R] = syy[R] + (lam_hx * dvx_dx + l2m_hx * dvy_dy) * DT

        # sigma_xy: j=1..NY-1, i=2..NX (2D:582-600)
        R = (slice(0, NY - 1), slice(1, NX))
        dvy_dx = (vy[:-1, 1:] - vy[:-1, :-1]) / DX
        dvx_dy = (vx[1:, 1:] - vx[:-1, 1:]) / DY
        m_dvy_dx[R] = bx[:, 1:] * m_dvy_dx[R] + ax[:, 1:] * dvy_dx
        m_dvx_dy[R] = byh[:-1] * m_dvx_dy[R] + ayh[:-1] * dvx_dy
        dvy_dx = dvy_dx / Kx[:, 1:] + m_dvy_dx[R]
        dvx_dy = dvx_dy / Kyh[:-1] + m_dvx_dy[R]
        sxy[R] = sxy[R] + mu_hy * (dvy_dx + dvx_dy) * DT

        # v_x: j=2..NY, i=2..NX (2D:606-621)
        R = (slice(1, NY), slice(1, NX))
        dsxx_dx = (sxx[1:, 1:] - sxx[1:, :-1]) / DX
        dsxy_dy = (sxy[1:, 1:] - sxy[:-1, 1:]) / DY
        m_dsxx_dx[R] = bx[:, 1:] * m_dsxx_dx[R] + ax[:, 1:] * dsxx_dx
        m_dsxy_dy[R] = by[1:] * m_dsxy_dy[R] + ay[1:] * dsxy_dy
        dsxx_dx = dsxx_dx / Kx[:, 1:] + m_dsxx_dx[R]
        dsxy_dy = dsxy_dy / Ky[1:] + m_dsxy_dy[R]
        vx[R] = vx[R] + (dsxx_dx + dsxy_dy) * DT / rho[1:, 1:]

        # v_y: j=1..NY-1, i=1..NX-1 (2D:623-641)
        R = (slice(0, NY - 1), slice(0, NX - 1))
        dsxy_dx = (sxy[:-1, 1:] - sxy[:-1, :-1]) / DX
        dsyy_dy = (syy[1:, :-1] - syy[:-1, :-1]) / DY
        m_dsxy_dx[R] = bxh[:, :-1] * m_dsxy_dx[R] + axh[:, :-1] * dsxy_dx
        m_dsyy_dy[R] = byh[:-1] * m_dsyy_dy[R] + ayh[:-1] * dsyy_dy
        dsxy_dx = dsxy_dx / Kxh[:, :-1] + m_dsxy_dx[R]
        dsyy_dy = dsyy_dy / Kyh[:-1] + m_dsyy_dy[R]
        vy[R] = vy[R] + (dsxy_dx + dsyy_dy) * DT / rho_hxhy

        # source (2D:644-667)
        st = source_term(p, it)
        fx = T(math.sin(ang) * st)
        fy = T(math.cos(ang) * st)
        rs = quarter * (rho[jsrc, isrc] + rho[jsrc, isrc + 1] + rho[jsrc + 1, isrc + 1]
                        + rho[jsrc + 1, isrc])
        vx[jsrc, isrc] = vx[jsrc, isrc] + fx * DT / rho[jsrc, isrc]
        vy[jsrc, isrc] = vy[jsrc, isrc] + fy * DT / rs

        # Dirichlet edges (2D:670-680)
        for f in (vx, vy):
            f[:, 0] = 0; f[:, NX - 1] = 0; f[0, :] = 0; f[NY - 1, :] = 0

        # seismograms (2D:683-686)
        for r, (ix, iy) in enumerate(rec):
            sisvx[r, it - 1] = vx[iy - 1, ix - 1]
            sisvy[r, it - 1] = vy[iy - 1, ix - 1]

        # energy over the non-PML interior (2D:694-713)
        I = (slice(npml, NY - npml), slice(npml, NX - npml))
        ek[it - 1] = 0.5 * np.sum(rho[I].astype(np.float64) * (
            vx[I].astype(np.float64) ** 2 + vy[I].astype(np.float64) ** 2))
        l, m_ = lam[I].astype(np.float64), mu[I].astype(np.float64)
        s1, s2, s3 = (sxx[I].astype(np.float64), syy[I].astype(np.float64),
                      sxy[I].astype(np.float64))
        exx = ((l + 2.0 * m_) * s1 - l * s2) / (4.0 * m_ * (l + m_))
        eyy = ((l + 2.0 * m_) * s2 - l * s1) / (4.0 * m_ * (l + m_))
        exy = s3 / (2.0 * m_)
        ep[it - 1] = np.sum(0.5 * (exx * s1 + eyy * s2 + 2.0 * exy * s3))

        if it % p.it_display == 0 or it == 5:                      # 2D:716-718
            vmax.append((it, float(np.max(np.sqrt(vx.astype(np.float64) ** 2
                                                  + vy.astype(np.float64) ** 2)))))
    res = Result(sisvx, sisvy, None, ek, ep, vmax=vmax)
    if keep_fields:
        res.fields = dict(vx=vx, vy=vy, sxx=sxx, syy=syy, sxy=sxy)
    return res


# ---------------------------------------------------------------------------
# 2D fourth-order program: seismic_CPML_2D_isotropic_fourth_order.f90 (2D4)
# ---------------------------------------------------------------------------
def run2d4(p, nsteps=None, lam=None, mu=None, rho=None, rec=None, dtype=np.float64,
           keep_fields=False):
    """The fourth-order program's time loop (2D4:553-745). Every array is
    held with the reference's ghost layer, shape (NY+2, NX+2) for Fortran
    0:NX+1 x 0:NY+1 (2D4:205, 223): Fortran (i, j) is element [j, i]; the
    ghost layer is never written and stays zero."""
    T = np.dtype(dtype).type
    NX, NY = p.nx, p.ny
    nsteps = p.nstep if nsteps is None else nsteps
    g = lambda: np.zeros((NY + 2, NX + 2), dtype)

    def padded(a, default):
        out = g()
        out[:, :] = default   # the reference fills the whole 0:NX+1 array (2D4:468-474)
        if a is not None:
            out[1:NY + 1, 1:NX + 1] = np.asarray(a, dtype)
        return out
    rho = padded(rho, p.rho)
    mu = padded(mu, p.rho * p.cs * p.cs)
    lam = padded(lam, p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs))
    px = {k: np.concatenate([[0.0], v, [0.0]]).astype(dtype) for k, v in _prof(p, 0, NX, p.deltax, np.float64).items()}
    pr = pml_profile(NY, p.deltay, p.npoints_pml, bool(p.use_pml[2]), bool(p.use_pml[3]), p.cp, p.f0,
                     p.deltat, p.npower, p.k_max_pml, p.alpha_max_pml, p.rcoef, high_origin_cells=NY)
    py = {k: np.concatenate([[0.0], v, [0.0]]).astype(dtype) for k, v in pr.items()}
    DX, DY, DT = T(p.deltax), T(p.deltay), T(p.deltat)
    c27, c24 = T(27.0), T(24.0)
    half, two, quarter = T(0.5), T(2.0), T(0.25)
    vx, vy, sxx, syy, sxy = g(), g(), g(), g(), g()
    m_dvx_dx, m_dvx_dy, m_dvy_dx, m_dvy_dy = g(), g(), g(), g()
    m_dsxx_dx, m_dsyy_dy, m_dsxy_dx, m_dsxy_dy = g(), g(), g(), g()
    rec = rec or []
    sisvx = np.zeros((len(rec), nsteps)); sisvy = np.zeros((len(rec), nsteps))
    ek = np.zeros(nsteps); ep = np.zeros(nsteps)
    vmax = []
    col = lambda d, k: d[k][None, :]
    row = lambda d, k: d[k][:, None]
    npml = p.npoints_pml
    ang = p.angle_force * (PI / 180.0)

    def S(i0, i1, j0, j1, di=0, dj=0):
        """Fortran i = i0..i1, j = j0..j1 shifted by (di, dj), as a padded-array slice."""
        return (slice(j0 + dj, j1 + dj + 1), slice(i0 + di, i1 + di + 1))

    def D(f, r, axis_h, p1, p0, p2, m1):
        # (27 f(p1) - 27 f(p0) - f(p2) + f(m1)) / (24 h); p* are (di, dj) offsets
        a = lambda o: f[S(*r, *o)]
        return (c27 * a(p1) - c27 * a(p0) - a(p2) + a(m1)) / (c24 * axis_h)

    for it in range(1, nsteps + 1):
        r = (1, NX - 1, 2, NY)                                     # 2D4:557-580
        R = S(*r)
        lhx = half * (lam[S(*r, 1, 0)] + lam[R]); mhx = half * (mu[S(*r, 1, 0)] + mu[R])
        l2m = lhx + two * mhx
        dvx_dx = D(vx, r, DX, (1, 0), (0, 0), (2, 0), (-1, 0))
        dvy_dy = D(vy, r, DY, (0, 0), (0, -1), (0, 1), (0, -2))
        m_dvx_dx[R] = col(px, "b_half")[:, 1:NX] * m_dvx_dx[R] + col(px, "a_half")[:, 1:NX] * dvx_dx
        m_dvy_dy[R] = row(py, "b")[2:NY + 1] * m_dvy_dy[R] + row(py, "a")[2:NY + 1] * dvy_dy
        dvx_dx = dvx_dx / col(px, "K_half")[:, 1:NX] + m_dvx_dx[R]
        dvy_dy = dvy_dy / row(py, "K")[2:NY + 1] + m_dvy_dy[R]
        sxx[R] = sxx[R] + (l2m * dvx_dx + lhx * dvy_dy) * DT
        syy[R] = syy[R] + (lhx * dvx_dx + l2m * dvy_dy) * DT

        r = (2, NX, 1, NY - 1)                                     # 2D4:582-600
        R = S(*r)
        mhy = half * (mu[S(*r, 0, 1)] + mu[R])
        dvy_dx = D(vy, r, DX, (0, 0), (-1, 0), (1, 0), (-2, 0))
        dvx_dy = D(vx, r, DY, (0, 1), (0, 0), (0, 2), (0, -1))
        m_dvy_dx[R] = col(px, "b")[:, 2:NX + 1] * m_dvy_dx[R] + col(px, "a")[:, 2:NX + 1] * dvy_dx
        m_dvx_dy[R] = row(py, "b_half")[1:NY] * m_dvx_dy[R] + row(py, "a_half")[1:NY] * dvx_dy
        dvy_dx = dvy_dx / col(px, "K")[:, 2:NX + 1] + m_dvy_dx[R]
        dvx_dy = dvx_dy / row(py, "K")[1:NY] + m_dvx_dy[R]        # K_y (2D4:596)
        sxy[R] = sxy[R] + mhy * (dvy_dx + dvx_dy) * DT

        r = (2, NX, 2, NY)                                         # 2D4:606-621
        R = S(*r)
        d1 = D(sxx, r, DX, (0, 0), (-1, 0), (1, 0), (-2, 0))
        d2 = D(sxy, r, DY, (0, 0), (0, -1), (0, 1), (0, -2))
        m_dsxx_dx[R] = col(px, "b")[:, 2:NX + 1] * m_dsxx_dx[R] + col(px, "a")[:, 2:NX + 1] * d1
        m_dsxy_dy[R] = row(py, "b")[2:NY + 1] * m_dsxy_dy[R] + row(py, "a")[2:NY + 1] * d2
        d1 = d1 / col(px, "K")[:, 2:NX + 1] + m_dsxx_dx[R]
        d2 = d2 / row(py, "K")[2:NY + 1] + m_dsxy_dy[R]
        vx[R] = vx[R] + (d1 + d2) * DT / rho[R]

        r = (1, NX - 1, 1, NY - 1)                                 # 2D4:623-641
        R = S(*r)
        rhh = quarter * (rho[R] + rho[S(*r, 1, 0)] + rho[S(*r, 1, 1)] + rho[S(*r, 0, 1)])
        d1 = D(sxy, r, DX, (1, 0), (0, 0), (2, 0), (-1, 0))
        d2 = D(syy, r, DY, (0, 1), (0, 0), (0, 2), (0, -1))
        m_dsxy_dx[R] = col(px, "b_half")[:, 1:NX] * m_dsxy_dx[R] + col(px, "a_half")[:, 1:NX] * d1
        m_dsyy_dy[R] = row(py, "b_half")[1:NY] * m_dsyy_dy[R] + row(py, "a_half")[1:NY] * d2
        d1 = d1 / col(px, "K_half")[:, 1:NX] + m_dsxy_dx[R]
        d2 = d2 / row(py, "K_half")[1:NY] + m_dsyy_dy[R]
        vy[R] = vy[R] + (d1 + d2) * DT / rhh

        st = source_term(p, it)                                    # 2D4:644-680
        fx, fy = T(math.sin(ang) * st), T(math.cos(ang) * st)
        i, j = p.isource, p.jsource
        rs = quarter * (rho[j, i] + rho[j, i + 1] + rho[j + 1, i + 1] + rho[j + 1, i])
        vx[j, i] = vx[j, i] + fx * DT / rho[j, i]
        vy[j, i] = vy[j, i] + fy * DT / rs
        for f in (vx, vy):                                         # 2D4:683-693, whole 0:N+1 lines
            f[:, 1] = 0; f[:, NX] = 0; f[1, :] = 0; f[NY, :] = 0
        for q, (ix, iy) in enumerate(rec):
            sisvx[q, it - 1] = vx[iy, ix]
            sisvy[q, it - 1] = vy[iy, ix]
        I = S(npml, NX - npml + 1, npml, NY - npml + 1)            # 2D4:696-712
        ek[it - 1] = 0.5 * np.sum(rho[I].astype(np.float64) * (
            vx[I].astype(np.float64) ** 2 + vy[I].astype(np.float64) ** 2))
        l, m_ = lam[I].astype(np.float64), mu[I].astype(np.float64)
        s1, s2, s3 = sxx[I].astype(np.float64), syy[I].astype(np.float64), sxy[I].astype(np.float64)
        exx = ((l + 2.0 * m_) * s1 - l * s2) / (4.0 * m_ * (l + m_))
        eyy = ((l + 2.0 * m_) * s2 - l * s1) / (4.0 * m_ * (l + m_))
        ep[it - 1] = np.sum(0.5 * (exx * s1 + eyy * s2 + 2.0 * (s3 / (2.0 * m_)) * s3))
        if it % p.it_display == 0 or it == 5:
            vmax.append((it, float(np.max(np.sqrt(vx.astype(np.float64) ** 2 + vy.astype(np.float64) ** 2)))))
    res = Result(sisvx, sisvy, None, ek, ep, vmax=vmax)
    if keep_fields:
        inner = (slice(1, NY + 1), slice(1, NX + 1))
        res.fields = dict(vx=vx[inner], vy=vy[inner], sxx=sxx[inner], syy=syy[inner], sxy=sxy[inner])
    return res


# ---------------------------------------------------------------------------
# classical split-field PML: seismic_PML_Collino_2D_isotropic.f90 (PML)
# ---------------------------------------------------------------------------
def split_profile(n, h, npml, cp, rcoef):
    """Damping d/2 at grid and half points (PML:180-250)."""
    delta = npml * h
    d0 = 3.0 * cp * math.log(1.0 / rcoef) / (2.0 * delta)
    ol, orr = delta, (n - 1) * h - delta
    f = np.zeros(n); g = np.zeros(n)
    for i in range(1, n + 1):
        x = h * float(i - 1)
        if x < ol:
            f[i - 1] = d0 * ((ol - x) / delta) ** 2
            g[i - 1] = d0 * ((ol - x - h / 2.0) / delta) ** 2
        elif x >= 0.9999 * orr:
            f[i - 1] = d0 * ((x - orr) / delta) ** 2
            g[i - 1] = d0 * ((x + h / 2.0 - orr) / delta) ** 2
    return f / 2.0, g / 2.0


def run_split(p, nsteps=None, rec=None, dtype=np.float64, keep_fields=False):
    """The split-field PML program's time loop (PML:337-533): every field is
    the sum of an x and a y part, each damped by its own axis's profile."""
    T = np.dtype(dtype).type
    NX, NY = p.nx, p.ny
    nsteps = p.nstep if nsteps is None else nsteps
    h, odt = T(p.deltax), T(1.0 / p.deltat)
    rho = T(p.rho)
    mu = T(p.rho * p.cs * p.cs)
    lam = T(p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs))
    l2m = T(p.rho * p.cp * p.cp)
    dx2, dxh2 = (a.astype(dtype)[None, :] for a in split_profile(NX, p.deltax, p.npoints_pml, p.cp, p.rcoef))
    dy2, dyh2 = (a.astype(dtype)[:, None] for a in split_profile(NY, p.deltay, p.npoints_pml, p.cp, p.rcoef))
    z = lambda: np.zeros((NY, NX), dtype)
    vx1, vx2, vy1, vy2 = z(), z(), z(), z()
    sxx1, sxx2, syy1, syy2, sxy1, sxy2 = z(), z(), z(), z(), z(), z()
    rec = rec or []
    sisvx = np.zeros((len(rec), nsteps)); sisvy = np.zeros((len(rec), nsteps))
    ek = np.zeros(nsteps); ep = np.zeros(nsteps)
    vmax = []
    ang = p.angle_force * (PI / 180.0)
    npml = p.npoints_pml
    upd = lambda old, d, rhs: (old * (odt - d) + rhs) / (odt + d)
    for it in range(1, nsteps + 1):
        R = (slice(1, NY), slice(0, NX - 1))                        # PML:344-364
        vdx = (vx1[1:, 1:] - vx1[1:, :-1]) / h + (vx2[1:, 1:] - vx2[1:, :-1]) / h
        vdy = (vy1[1:, :-1] - vy1[:-1, :-1]) / h + (vy2[1:, :-1] - vy2[:-1, :-1]) / h
        d = dxh2[:, :-1]
        sxx1[R] = upd(sxx1[R], d, l2m * vdx)
        syy1[R] = upd(syy1[R], d, lam * vdx)
        d = dy2[1:]
        sxx2[R] = upd(sxx2[R], d, lam * vdy)
        syy2[R] = upd(syy2[R], d, l2m * vdy)
        R = (slice(0, NY - 1), slice(1, NX))                        # PML:366-383
        vdx = (vy1[:-1, 1:] - vy1[:-1, :-1]) / h + (vy2[:-1, 1:] - vy2[:-1, :-1]) / h
        vdy = (vx1[1:, 1:] - vx1[:-1, 1:]) / h + (vx2[1:, 1:] - vx2[:-1, 1:]) / h
        sxy1[R] = upd(sxy1[R], dx2[:, 1:], mu * vdx)
        sxy2[R] = upd(sxy2[R], dyh2[:-1], mu * vdy)
        R = (slice(1, NY), slice(1, NX))                            # PML:389-406
        sdx = (sxx1[1:, 1:] - sxx1[1:, :-1]) / h + (sxx2[1:, 1:] - sxx2[1:, :-1]) / h
        sdy = (sxy1[1:, 1:] - sxy1[:-1, 1:]) / h + (sxy2[1:, 1:] - sxy2[:-1, 1:]) / h
        vx1[R] = upd(vx1[R], dx2[:, 1:], sdx / rho)
        vx2[R] = upd(vx2[R], dy2[1:], sdy / rho)
        R = (slice(0, NY - 1), slice(0, NX - 1))                    # PML:408-425
        sdx = (sxy1[:-1, 1:] - sxy1[:-1, :-1]) / h + (sxy2[:-1, 1:] - sxy2[:-1, :-1]) / h
        sdy = (syy1[1:, :-1] - syy1[:-1, :-1]) / h + (syy2[1:, :-1] - syy2[:-1, :-1]) / h
        vy1[R] = upd(vy1[R], dxh2[:, :-1], sdx / rho)
        vy2[R] = upd(vy2[R], dyh2[:-1], sdy / rho)
        st = source_term(p, it)                                     # PML:428-451
        i, j = p.isource - 1, p.jsource - 1
        vx1[j, i] = vx1[j, i] + T(math.sin(ang) * st) * T(p.deltat) / rho
        vy1[j, i] = vy1[j, i] + T(math.cos(ang) * st) * T(p.deltat) / rho
        for f in (vx1, vy1, vx2, vy2):                              # PML:453-478
            f[:, 0] = 0; f[:, NX - 1] = 0; f[0, :] = 0; f[NY - 1, :] = 0
        vxt = vx1.astype(np.float64) + vx2.astype(np.float64)
        vyt = vy1.astype(np.float64) + vy2.astype(np.float64)
        for q, (ix, iy) in enumerate(rec):                          # PML:481-484
            sisvx[q, it - 1] = vxt[iy - 1, ix - 1]
            sisvy[q, it - 1] = vyt[iy - 1, ix - 1]
        I = (slice(npml, NY - npml), slice(npml, NX - npml))        # PML:486-515
        ek[it - 1] = 0.5 * np.sum(float(rho) * (vxt[I] ** 2 + vyt[I] ** 2))
        l, m_ = float(lam), float(mu)
        s1 = (sxx1.astype(np.float64) + sxx2)[I]
        s2 = (syy1.astype(np.float64) + syy2)[I]
        s3 = (sxy1.astype(np.float64) + sxy2)[I]
        exx = ((l + 2.0 * m_) * s1 - l * s2) / (4.0 * m_ * (l + m_))
        eyy = ((l + 2.0 * m_) * s2 - l * s1) / (4.0 * m_ * (l + m_))
        ep[it - 1] = np.sum(0.5 * (exx * s1 + eyy * s2 + 2.0 * (s3 / (2.0 * m_)) * s3))
        if it % p.it_display == 0 or it == 5:
            vmax.append((it, float(np.max(np.sqrt(vxt ** 2 + vyt ** 2)))))
    res = Result(sisvx, sisvy, None, ek, ep, vmax=vmax)
    if keep_fields:
        res.fields = dict(vx=vx1 + vx2, vy=vy1 + vy2, sxx=sxx1 + sxx2, syy=syy1 + syy2, sxy=sxy1 + sxy2)
    return res


# ---------------------------------------------------------------------------
# 3D time loop: 3D:802-1180 (single-domain semantics)
# ---------------------------------------------------------------------------
def run3d(p, nsteps=None, lam=None, mu=None, rho=None, rec=None,
          dtype=np.float64, keep_fields=False):
    """Run the 3D program. Homogeneous scalars by default (3D:139-144);
    lam/mu/rho [nz, ny, nx] arrays select the per-cell extension, whose
    staggered averages follow the 2D program's rules (2D:560-562, 586, 627)
    extended to z. rec: list of 1-based (ix, iy, iz)."""
    T = np.dtype(dtype).type
    NX, NY, NZ = p.nx, p.ny, p.nz
    nsteps = p.nstep if nsteps is None else nsteps
    px = _prof(p, 0, NX, p.deltax, dtype)
    py = _prof(p, 1, NY, p.deltay, dtype)
    pz = _prof(p, 2, NZ, p.deltaz, dtype)
    DT = T(p.deltat)
    odx, ody, odz = T(1.0 / p.deltax), T(1.0 / p.deltay), T(1.0 / p.deltaz)
    hetero = lam is not None or mu is not None or rho is not None
    half, quarter, eighth = T(0.5), T(0.25), T(0.125)
    if hetero:
        shp = (NZ, NY, NX)
        lam = np.asarray(lam if lam is not None else np.full(shp, p.rho * (p.cp ** 2 - 2 * p.cs ** 2)), dtype)
        mu = np.asarray(mu if mu is not None else np.full(shp, p.rho * p.cs ** 2), dtype)
        rho = np.asarray(rho if rho is not None else np.full(shp, p.rho), dtype)
        lam_hx = half * (lam[1:, 1:, 1:] + lam[1:, 1:, :-1])
        mu_hx = half * (mu[1:, 1:, 1:] + mu[1:, 1:, :-1])
        DT_lam = DT * lam_hx
        DT_l2m = DT * (lam_hx + T(2.0) * mu_hx)
        DT_mu_xy = DT * (half * (mu[:, 1:, 1:] + mu[:, :-1, 1:]))
        DT_mu_xz = DT * (half * (mu[1:, :, 1:] + mu[:-1, :, 1:]))
        DT_mu_yz = None                       # computed by _dtmu_yz
        DT_rho_x = DT / rho[1:, 1:, 1:]
        DT_rho_y = DT / (quarter * (rho[1:, :-1, :-1] + rho[1:, :-1, 1:] + rho[1:, 1:, 1:] + rho[1:, 1:, :-1]))
        DT_rho_z = DT / (quarter * (rho[:-1, 1:, :-1] + rho[:-1, 1:, 1:] + rho[1:, 1:, 1:] + rho[1:, 1:, :-1]))
        DT_mu_yz = _dtmu_yz(mu, DT, eighth)
        rho_s = lambda k, j, i: rho[k, j, i]
    else:
        lam_s = p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs)        # 3D:142-144
        mu_s = p.rho * p.cs * p.cs
        l2m_s = p.rho * p.cp * p.cp
        DT_lam, DT_mu, DT_l2m = T(p.deltat * lam_s), T(p.deltat * mu_s), T(p.deltat * l2m_s)
        DT_mu_xy = DT_mu_xz = DT_mu_yz = DT_mu
        DT_rho_x = DT_rho_y = DT_rho_z = T(p.deltat / p.rho)       # 3D:300
        rho_s = lambda k, j, i: p.rho

    z = lambda: np.zeros((NZ, NY, NX), dtype)
    vx, vy, vz = z(), z(), z()
    sxx, syy, szz, sxy, sxz, syz = z(), z(), z(), z(), z(), z()
    names = ["dvx_dx", "dvx_dy", "dvx_dz", "dvy_dx", "dvy_dy", "dvy_dz", "dvz_dx",
             "dvz_dy", "dvz_dz", "dsxx_dx", "dsyy_dy", "dszz_dz", "dsxy_dx", "dsxy_dy",
             "dsxz_dx", "dsxz_dz", "dsyz_dy", "dsyz_dz"]
    M = {n: z() for n in names}
    rec = rec or []
    nrec = len(rec)
    sisvx = np.zeros((nrec, nsteps)); sisvy = np.zeros((nrec, nsteps)); sisvz = np.zeros((nrec, nsteps))
    ek = np.zeros(nsteps); ep = np.zeros(nsteps)
    vmax = []

    X = lambda pr, key: pr[key][None, None, :]
    Y = lambda pr, key: pr[key][None, :, None]
    Zp = lambda pr, key: pr[key][:, None, None]
    bx, ax, Kx = X(px, "b"), X(px, "a"), X(px, "K")
    bxh, axh, Kxh = X(px, "b_half"), X(px, "a_half"), X(px, "K_half")
    by, ay, Ky = Y(py, "b"), Y(py, "a"), Y(py, "K")
    byh, ayh, Kyh = Y(py, "b_half"), Y(py, "a_half"), Y(py, "K_half")
    bz, az, Kz = Zp(pz, "b"), Zp(pz, "a"), Zp(pz, "K")
    bzh, azh, Kzh = Zp(pz, "b_half"), Zp(pz, "a_half"), Zp(pz, "K_half")

    def upd(name, R, b, a, val, K):
        M[name][R] = b * M[name][R] + a * val
        return val / K + M[name][R]

    npml = p.npoints_pml
    isrc, jsrc, ksrc = p.isource - 1, p.jsource - 1, p.ksource - 1
    ang = p.angle_force * (PI / 180.0)
    q1 = not (p.flags & FLAG_EP_PHYSICAL)

    for it in range(1, nsteps + 1):
        # normal stresses: k=2..NZ, j=2..NY, i=1..NX-1 (3D:836-863)
        R = (slice(1, NZ), slice(1, NY), slice(0, NX - 1))
        dvx_dx = (vx[1:, 1:, 1:] - vx[1:, 1:, :-1]) * odx
        dvy_dy = (vy[1:, 1:, :-1] - vy[1:, :-1, :-1]) * ody
        dvz_dz = (vz[1:, 1:, :-1] - vz[:-1, 1:, :-1]) * odz
        dvx_dx = upd("dvx_dx", R, bxh[..., :-1], axh[..., :-1], dvx_dx, Kxh[..., :-1])
        dvy_dy = upd("dvy_dy", R, by[:, 1:], ay[:, 1:], dvy_dy, Ky[:, 1:])
        dvz_dz = upd("dvz_dz", R, bz[1:], az[1:], dvz_dz, Kz[1:])
        sxx[R] = DT_l2m * dvx_dx + DT_lam * (dvy_dy + dvz_dz) + sxx[R]
        syy[R] = DT_lam * (dvx_dx + dvz_dz) + DT_l2m * dvy_dy + syy[R]
        szz[R] = DT_lam * (dvx_dx + dvy_dy) + DT_l2m * dvz_dz + szz[R]

        # sigma_xy: k=1..NZ, j=1..NY-1, i=2..NX (3D:877-894)
        R = (slice(0, NZ), slice(0, NY - 1), slice(1, NX))
        dvy_dx = (vy[:, :-1, 1:] - vy[:, :-1, :-1]) * odx
        dvx_dy = (vx[:, 1:, 1:] - vx[:, :-1, 1:]) * ody
        dvy_dx = upd("dvy_dx", R, bx[..., 1:], ax[..., 1:], dvy_dx, Kx[..., 1:])
        dvx_dy = upd("dvx_dy", R, byh[:, :-1], ayh[:, :-1], dvx_dy, Kyh[:, :-1])
        sxy[R] = DT_mu_xy * (dvy_dx + dvx_dy) + sxy[R]

        # sigma_xz: k=1..NZ-1, j=1..NY, i=2..NX (3D:908-925)
        R = (slice(0, NZ - 1), slice(0, NY), slice(1, NX))
        dvz_dx = (vz[:-1, :, 1:] - vz[:-1, :, :-1]) * odx
        dvx_dz = (vx[1:, :, 1:] - vx[:-1, :, 1:]) * odz
        dvz_dx = upd("dvz_dx", R, bx[..., 1:], ax[..., 1:], dvz_dx, Kx[..., 1:])
        dvx_dz = upd("dvx_dz", R, bzh[:-1], azh[:-1], dvx_dz, Kzh[:-1])
        sxz[R] = DT_mu_xz * (dvz_dx + dvx_dz) + sxz[R]

        # sigma_yz: k=1..NZ-1, j=1..NY-1, i=1..NX (3D:927-942)
        R = (slice(0, NZ - 1), slice(0, NY - 1), slice(0, NX))
        dvz_dy = (vz[:-1, 1:, :] - vz[:-1, :-1, :]) * ody
        dvy_dz = (vy[1:, :-1, :] - vy[:-1, :-1, :]) * odz
        dvz_dy = upd("dvz_dy", R, byh[:, :-1], ayh[:, :-1], dvz_dy, Kyh[:, :-1])
        dvy_dz = upd("dvy_dz", R, bzh[:-1], azh[:-1], dvy_dz, Kzh[:-1])
        syz[R] = DT_mu_yz * (dvz_dy + dvy_dz) + syz[R]

        # v_x: k=2..NZ, j=2..NY, i=2..NX (3D:976-993)
        R = (slice(1, NZ), slice(1, NY), slice(1, NX))
        a1 = (sxx[1:, 1:, 1:] - sxx[1:, 1:, :-1]) * odx
        a2 = (sxy[1:, 1:, 1:] - sxy[1:, :-1, 1:]) * ody
        a3 = (sxz[1:, 1:, 1:] - sxz[:-1, 1:, 1:]) * odz
        a1 = upd("dsxx_dx", R, bx[..., 1:], ax[..., 1:], a1, Kx[..., 1:])
        a2 = upd("dsxy_dy", R, by[:, 1:], ay[:, 1:], a2, Ky[:, 1:])
        a3 = upd("dsxz_dz", R, bz[1:], az[1:], a3, Kz[1:])
        vx[R] = DT_rho_x * (a1 + a2 + a3) + vx[R]

        # v_y: k=2..NZ, j=1..NY-1, i=1..NX-1 (3D:995-1014)
        R = (slice(1, NZ), slice(0, NY - 1), slice(0, NX - 1))
        a1 = (sxy[1:, :-1, 1:] - sxy[1:, :-1, :-1]) * odx
        a2 = (syy[1:, 1:, :-1] - syy[1:, :-1, :-1]) * ody
        a3 = (syz[1:, :-1, :-1] - syz[:-1, :-1, :-1]) * odz
        a1 = upd("dsxy_dx", R, bxh[..., :-1], axh[..., :-1], a1, Kxh[..., :-1])
        a2 = upd("dsyy_dy", R, byh[:, :-1], ayh[:, :-1], a2, Kyh[:, :-1])
        a3 = upd("dsyz_dz", R, bz[1:], az[1:], a3, Kz[1:])
        vy[R] = DT_rho_y * (a1 + a2 + a3) + vy[R]

        # v_z: k=1..NZ-1, j=2..NY, i=1..NX-1 (3D:1031-1052)
        R = (slice(0, NZ - 1), slice(1, NY), slice(0, NX - 1))
        a1 = (sxz[:-1, 1:, 1:] - sxz[:-1, 1:, :-1]) * odx
        a2 = (syz[:-1, 1:, :-1] - syz[:-1, :-1, :-1]) * ody
        a3 = (szz[1:, 1:, :-1] - szz[:-1, 1:, :-1]) * odz
        a1 = upd("dsxz_dx", R, bxh[..., :-1], axh[..., :-1], a1, Kxh[..., :-1])
        a2 = upd("dsyz_dy", R, by[:, 1:], ay[:, 1:], a2, Ky[:, 1:])
        a3 = upd("dszz_dz", R, bzh[:-1], azh[:-1], a3, Kzh[:-1])
        vz[R] = DT_rho_z * (a1 + a2 + a3) + vz[R]

        # source on plane ksource with plain rho (3D:1055-1083)
        st = source_term(p, it)
        fx = math.sin(ang) * st
        fy = math.cos(ang) * st
        r0 = rho_s(ksrc, jsrc, isrc)
        vx[ksrc, jsrc, isrc] = vx[ksrc, jsrc, isrc] + T(fx * p.deltat / r0) if not hetero else \
            vx[ksrc, jsrc, isrc] + T(fx) * DT / r0
        vy[ksrc, jsrc, isrc] = vy[ksrc, jsrc, isrc] + T(fy * p.deltat / r0) if not hetero else \
            vy[ksrc, jsrc, isrc] + T(fy) * DT / r0

        # Dirichlet on the six faces (3D:1087-1121)
        for f in (vx, vy, vz):
            f[:, :, 0] = 0; f[:, :, NX - 1] = 0
            f[:, 0, :] = 0; f[:, NY - 1, :] = 0
            f[0, :, :] = 0; f[NZ - 1, :, :] = 0

        # seismograms (3D:1124-1129; the reference records no vz)
        for r, (ix, iy, iz) in enumerate(rec):
            sisvx[r, it - 1] = vx[iz - 1, iy - 1, ix - 1]
            sisvy[r, it - 1] = vy[iz - 1, iy - 1, ix - 1]
            sisvz[r, it - 1] = vz[iz - 1, iy - 1, ix - 1]

        # energy (3D:1131-1180)
        I = (slice(npml, NZ - npml), slice(npml, NY - npml), slice(npml, NX - npml))
        f64 = lambda a_: a_[I].astype(np.float64)
        if hetero:
            r_, l, m_ = f64(rho), f64(lam), f64(mu)
        else:
            r_, l, m_ = p.rho, lam_s, mu_s
        ek[it - 1] = np.sum(0.5 * r_ * (f64(vx) ** 2 + f64(vy) ** 2 + f64(vz) ** 2))
        s_xx, s_yy, s_zz, s_xy, s_xz, s_yz = (f64(sxx), f64(syy), f64(szz), f64(sxy),
                                              f64(sxz), f64(syz))
        den = 2.0 * m_ * (3.0 * l + 2.0 * m_)
        exx = (2.0 * (l + m_) * s_xx - l * s_yy - l * s_zz) / den
        eyy = (2.0 * (l + m_) * s_yy - l * s_xx - l * s_zz) / den
        ezz = (2.0 * (l + m_) * s_zz - l * s_xx - l * s_yy) / den
        exy = s_xy / (2.0 * m_); exz = s_xz / (2.0 * m_); eyz = s_yz / (2.0 * m_)
        third = eyy * s_yy if q1 else ezz * s_zz
        ep[it - 1] = np.sum(0.5 * (exx * s_xx + eyy * s_yy + third + 2.0 * exy * s_xy
                                   + 2.0 * exz * s_xz + 2.0 * eyz * s_yz))

        if it % p.it_display == 0 or it == 5:                       # 3D:1183-1186
            vmax.append((it, float(np.max(np.sqrt(vx.astype(np.float64) ** 2
                                                  + vy.astype(np.float64) ** 2
                                                  + vz.astype(np.float64) ** 2)))))
    res = Result(sisvx, sisvy, sisvz, ek, ep, vmax=vmax)
    if keep_fields:
        res.fields = dict(vx=vx, vy=vy, vz=vz, sxx=sxx, syy=syy, szz=szz, sxy=sxy,
                          sxz=sxz, syz=syz)
    return res


def _dtmu_yz(mu, DT, eighth):
    """DT*mu at the sigma_yz points (rows k<NZ, j<NY, all i) of the per-cell
    3D extension."""
    # 8-point average at (i+1/2, j+1/2, k+1/2); for the last column i = NX the
    # i+1 neighbour does not exist and the column i itself is used instead.
    m = mu
    mi1 = np.concatenate([m[:, :, 1:], m[:, :, -1:]], axis=2)
    s = (m[:-1, :-1, :] + mi1[:-1, :-1, :] + m[:-1, 1:, :] + mi1[:-1, 1:, :]
         + m[1:, :-1, :] + mi1[1:, :-1, :] + m[1:, 1:, :] + mi1[1:, 1:, :])
    return DT * (eighth * s)
