// cpml_oracle.cpp -- C++ restatement of the two reference programs.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle: tests, the smoke check and
// the CPU-baseline leg of the benchmark use it as a checker and as the timed
// CPU implementation. The product library never links, calls or falls back
// to it.
//
// It follows, loop nest by loop nest and in the reference's operation order:
//   seismic_CPML_2D_isotropic_second_order.f90   2D:283-744
//   seismic_CPML_2D_isotropic_fourth_order.f90   2D4:325-745 (order = 4)
//   seismic_PML_Collino_2D_isotropic.f90         PML:180-533 (scheme = split)
//   seismic_CPML_3D_isotropic_MPI_OpenMP.f90     3D:399-1180
// with full-grid memory arrays as in the reference (2D:221-230, 3D:228-247)
// and OpenMP over the outer loop index as in 3D:825. The 3D program is
// restated for one domain of NZ planes: the union of the MPI slabs, whose
// one-plane halo exchanges (3D:811-823, 951-963) make the sweep ranges
// k = 2..NZ (k2begin on rank 0) and k = 1..NZ-1 (kminus1end on the last
// rank); the source and receivers sit on global plane ksource (NZ/2 in the
// reference, 3D:1080, 1126).
//
// Templated on the arithmetic type: double is the oracle, float measures the
// FP32 rounding floor. Built with -ffp-contract=off so results do not depend
// on the host ISA's FMA contraction.
//
// Pinned to the reference: tests/test_ref_pin.py checks this file against the
// reference programs' own statements. oracle/ref_f90c.py translated them from
// their Fortran source and gcc ran them, the 3D program on 2, 4 and 12
// emulated MPI ranks (tests/golden/refpin_*.npz). Fields, seismograms and 2D
// energies agree bit for bit. The 3D total energy agrees to summation order,
// because the reference reduces per-rank sums over MPI. The file is also
// cross-checked against the independent numpy restatement
// (oracle/oracle_np.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/cpml.h"

namespace {

const double PI = 3.141592653589793238462643;

struct Profile {
  std::vector<double> d, K, alpha, a, b, dh, Kh, alphah, ah, bh;
};

// 2D:283-394 (x), 2D:396-465 (y), 3D:560-667 (z)
// The fourth-order program puts the high-side origin of the y profile one
// cell further out: yorigintop = NY*DELTAY - thickness (2D4:401) where the
// second-order program has (NY-1)*DELTAY (2D:400).
Profile build_profile(const cpml_params* p, int axis, int n, double delta) {
  const bool top_shift = p->ndim == 2 && p->order == 4 && axis == 1;
  Profile P;
  P.d.assign(n, 0.0); P.dh.assign(n, 0.0);
  P.K.assign(n, 1.0); P.Kh.assign(n, 1.0);
  P.alpha.assign(n, 0.0); P.alphah.assign(n, 0.0);
  P.a.assign(n, 0.0); P.ah.assign(n, 0.0);
  P.b.assign(n, 0.0); P.bh.assign(n, 0.0);
  const bool use_min = p->use_pml[2 * axis] != 0;
  const bool use_max = p->use_pml[2 * axis + 1] != 0;
  const double npower = p->npower;
  const double kmax = p->k_max_pml;
  const double amax = p->alpha_max_pml < 0 ? 2.0 * PI * (p->f0 / 2.0) : p->alpha_max_pml;
  const double thickness = p->npoints_pml * delta;
  const double d0 = -(npower + 1) * p->cp * std::log(p->rcoef) / (2.0 * thickness);
  const double oleft = thickness;
  const double oright = (top_shift ? n : n - 1) * delta - thickness;
  for (int i = 1; i <= n; ++i) {
    const double val = delta * double(i - 1);
    const int ii = i - 1;
    if (use_min) {
      double ab = oleft - val;
      if (ab >= 0.0) {
        double nr = ab / thickness;
        P.d[ii] = d0 * std::pow(nr, npower);
        P.K[ii] = 1.0 + (kmax - 1.0) * std::pow(nr, npower);
        P.alpha[ii] = amax * (1.0 - nr);
      }
      ab = oleft - (val + delta / 2.0);
      if (ab >= 0.0) {
        double nr = ab / thickness;
        P.dh[ii] = d0 * std::pow(nr, npower);
        P.Kh[ii] = 1.0 + (kmax - 1.0) * std::pow(nr, npower);
        P.alphah[ii] = amax * (1.0 - nr);
      }
    }
    if (use_max) {
      double ab = val - oright;
      if (ab >= 0.0) {
        double nr = ab / thickness;
        P.d[ii] = d0 * std::pow(nr, npower);
        P.K[ii] = 1.0 + (kmax - 1.0) * std::pow(nr, npower);
        P.alpha[ii] = amax * (1.0 - nr);
      }
      ab = val + delta / 2.0 - oright;
      if (ab >= 0.0) {
        double nr = ab / thickness;
        P.dh[ii] = d0 * std::pow(nr, npower);
        P.Kh[ii] = 1.0 + (kmax - 1.0) * std::pow(nr, npower);
        P.alphah[ii] = amax * (1.0 - nr);
      }
    }
    if (P.alpha[ii] < 0.0) P.alpha[ii] = 0.0;
    if (P.alphah[ii] < 0.0) P.alphah[ii] = 0.0;
    P.b[ii] = std::exp(-(P.d[ii] / P.K[ii] + P.alpha[ii]) * p->deltat);
    P.bh[ii] = std::exp(-(P.dh[ii] / P.Kh[ii] + P.alphah[ii]) * p->deltat);
    if (std::fabs(P.d[ii]) > 1e-6)
      P.a[ii] = P.d[ii] * (P.b[ii] - 1.0) / (P.K[ii] * (P.d[ii] + P.K[ii] * P.alpha[ii]));
    if (std::fabs(P.dh[ii]) > 1e-6)
      P.ah[ii] = P.dh[ii] * (P.bh[ii] - 1.0) / (P.Kh[ii] * (P.dh[ii] + P.Kh[ii] * P.alphah[ii]));
  }
  return P;
}

// Source time function at 1-based step it (2D:644-654).
double source_term(const cpml_params* p, int it) {
  const double a = PI * PI * p->f0 * p->f0;
  const double t = double(it - 1) * p->deltat;
  const double tt = t - p->t0;
  const double tt2 = tt * tt;
  if (p->stf == CPML_STF_GAUSSIAN) return p->factor * std::exp(-(a * tt2));
  if (p->stf == CPML_STF_RICKER) return p->factor * (1.0 - 2.0 * a * tt2) * std::exp(-(a * tt2));
  return -(p->factor * 2.0 * a * tt * std::exp(-(a * tt2)));
}

template <typename R>
struct Prof1 {  // one axis, rounded to the arithmetic type
  std::vector<R> a, b, K, ah, bh, Kh;
  explicit Prof1(const Profile& P) {
    auto cv = [](const std::vector<double>& v) { return std::vector<R>(v.begin(), v.end()); };
    a = cv(P.a); b = cv(P.b); K = cv(P.K); ah = cv(P.ah); bh = cv(P.bh); Kh = cv(P.Kh);
  }
};

struct Out {
  int nsteps, nrec;
  const int *ix, *iy, *iz;
  double *sisvx, *sisvy, *sisvz, *ek, *ep, *vmax;
};

// ---------------------------------------------------------------------------
// 2D program, time loop 2D:550-735
// ---------------------------------------------------------------------------
template <typename R>
struct State2D {
  const cpml_params* p;
  int NX, NY;
  size_t N;
  std::vector<R> lam, mu, rho;
  Prof1<R> X, Y;
  R DX, DY, DT;
  std::vector<R> vx, vy, sxx, syy, sxy;
  std::vector<R> m_dvx_dx, m_dvx_dy, m_dvy_dx, m_dvy_dy;
  std::vector<R> m_dsxx_dx, m_dsyy_dy, m_dsxy_dx, m_dsxy_dy;
  int npml;
  double sa, ca;
  State2D(const cpml_params* p_, const double* lam_in, const double* mu_in, const double* rho_in)
      : p(p_), NX(p_->nx), NY(p_->ny), N(size_t(p_->nx) * p_->ny),
        X(build_profile(p_, 0, p_->nx, p_->deltax)), Y(build_profile(p_, 1, p_->ny, p_->deltay)) {
    lam.resize(N); mu.resize(N); rho.resize(N);
    const double lam0 = p->rho * (p->cp * p->cp - 2.0 * p->cs * p->cs);
    const double mu0 = p->rho * p->cs * p->cs;
    for (size_t c = 0; c < N; ++c) {                               // 2D:468-474
      rho[c] = R(rho_in ? rho_in[c] : p->rho);
      mu[c] = R(mu_in ? mu_in[c] : mu0);
      lam[c] = R(lam_in ? lam_in[c] : lam0);
    }
    DX = R(p->deltax); DY = R(p->deltay); DT = R(p->deltat);
    for (auto* v : {&vx, &vy, &sxx, &syy, &sxy, &m_dvx_dx, &m_dvx_dy, &m_dvy_dx, &m_dvy_dy, &m_dsxx_dx,
                    &m_dsyy_dy, &m_dsxy_dx, &m_dsxy_dy})
      v->assign(N, R(0));
    npml = p->npoints_pml;
    const double ang = p->angle_force * (PI / 180.0);
    sa = std::sin(ang); ca = std::cos(ang);
  }
  size_t at(int i, int j) const { return size_t(j - 1) * NX + (i - 1); }  // 1-based
  void step(int it, const Out& o);
  void step4(int it, const Out& o);
  void advance(int it, const Out& o) { if (p->order == 4) step4(it, o); else step(it, o); }
  void fields(double* out) const {
    const std::vector<R>* F[5] = {&vx, &vy, &sxx, &syy, &sxy};
    for (int f = 0; f < 5; ++f)
      for (size_t c = 0; c < N; ++c) out[f * N + c] = double((*F[f])[c]);
  }
};

// one pass of the time loop 2D:550-735
template <typename R>
void State2D<R>::step(int it, const Out& o) {
    // sigma_xx, sigma_yy (2D:556-580)
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j);
        R lam_hx = R(0.5) * (lam[at(i + 1, j)] + lam[c]);
        R mu_hx = R(0.5) * (mu[at(i + 1, j)] + mu[c]);
        R l2m = lam_hx + R(2.0) * mu_hx;
        R dvx_dx = (vx[at(i + 1, j)] - vx[c]) / DX;
        R dvy_dy = (vy[c] - vy[at(i, j - 1)]) / DY;
        m_dvx_dx[c] = X.bh[i - 1] * m_dvx_dx[c] + X.ah[i - 1] * dvx_dx;
        m_dvy_dy[c] = Y.b[j - 1] * m_dvy_dy[c] + Y.a[j - 1] * dvy_dy;
        dvx_dx = dvx_dx / X.Kh[i - 1] + m_dvx_dx[c];
        dvy_dy = dvy_dy / Y.K[j - 1] + m_dvy_dy[c];
        sxx[c] = sxx[c] + (l2m * dvx_dx + lam_hx * dvy_dy) * DT;
        syy[c] = syy[c] + (lam_hx * dvx_dx + l2m * dvy_dy) * DT;
      }
    // sigma_xy (2D:582-600)
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j);
        R mu_hy = R(0.5) * (mu[at(i, j + 1)] + mu[c]);
        R dvy_dx = (vy[c] - vy[at(i - 1, j)]) / DX;
        R dvx_dy = (vx[at(i, j + 1)] - vx[c]) / DY;
        m_dvy_dx[c] = X.b[i - 1] * m_dvy_dx[c] + X.a[i - 1] * dvy_dx;
        m_dvx_dy[c] = Y.bh[j - 1] * m_dvx_dy[c] + Y.ah[j - 1] * dvx_dy;
        dvy_dx = dvy_dx / X.K[i - 1] + m_dvy_dx[c];
        dvx_dy = dvx_dy / Y.Kh[j - 1] + m_dvx_dy[c];
        sxy[c] = sxy[c] + mu_hy * (dvy_dx + dvx_dy) * DT;
      }
    // v_x (2D:606-621)
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j);
        R d1 = (sxx[c] - sxx[at(i - 1, j)]) / DX;
        R d2 = (sxy[c] - sxy[at(i, j - 1)]) / DY;
        m_dsxx_dx[c] = X.b[i - 1] * m_dsxx_dx[c] + X.a[i - 1] * d1;
        m_dsxy_dy[c] = Y.b[j - 1] * m_dsxy_dy[c] + Y.a[j - 1] * d2;
        d1 = d1 / X.K[i - 1] + m_dsxx_dx[c];
        d2 = d2 / Y.K[j - 1] + m_dsxy_dy[c];
        vx[c] = vx[c] + (d1 + d2) * DT / rho[c];
      }
    // v_y (2D:623-641)
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j);
        R rhh = R(0.25) * (rho[c] + rho[at(i + 1, j)] + rho[at(i + 1, j + 1)] + rho[at(i, j + 1)]);
        R d1 = (sxy[at(i + 1, j)] - sxy[c]) / DX;
        R d2 = (syy[at(i, j + 1)] - syy[c]) / DY;
        m_dsxy_dx[c] = X.bh[i - 1] * m_dsxy_dx[c] + X.ah[i - 1] * d1;
        m_dsyy_dy[c] = Y.bh[j - 1] * m_dsyy_dy[c] + Y.ah[j - 1] * d2;
        d1 = d1 / X.Kh[i - 1] + m_dsxy_dx[c];
        d2 = d2 / Y.Kh[j - 1] + m_dsyy_dy[c];
        vy[c] = vy[c] + (d1 + d2) * DT / rhh;
      }
    // source (2D:644-667)
    {
      const double st = source_term(p, it);
      const R fx = R(sa * st), fy = R(ca * st);
      const int i = p->isource, j = p->jsource;
      R rhh = R(0.25) * (rho[at(i, j)] + rho[at(i + 1, j)] + rho[at(i + 1, j + 1)] + rho[at(i, j + 1)]);
      vx[at(i, j)] = vx[at(i, j)] + fx * DT / rho[at(i, j)];
      vy[at(i, j)] = vy[at(i, j)] + fy * DT / rhh;
    }
    // Dirichlet (2D:670-680)
    for (int j = 1; j <= NY; ++j) {
      vx[at(1, j)] = 0; vx[at(NX, j)] = 0; vy[at(1, j)] = 0; vy[at(NX, j)] = 0;
    }
    for (int i = 1; i <= NX; ++i) {
      vx[at(i, 1)] = 0; vx[at(i, NY)] = 0; vy[at(i, 1)] = 0; vy[at(i, NY)] = 0;
    }
    // seismograms (2D:683-686)
    for (int r = 0; r < o.nrec; ++r) {
      o.sisvx[size_t(r) * o.nsteps + it - 1] = double(vx[at(o.ix[r], o.iy[r])]);
      o.sisvy[size_t(r) * o.nsteps + it - 1] = double(vy[at(o.ix[r], o.iy[r])]);
    }
    // energy (2D:694-713), in double whatever R is, sequential i-fastest order
    if (o.ek || o.ep) {
      double ek = 0.0, ep = 0.0;
      for (int j = npml + 1; j <= NY - npml; ++j)
        for (int i = npml + 1; i <= NX - npml; ++i) {
          const size_t c = at(i, j);
          const double vxx = vx[c], vyy = vy[c];
          ek = ek + double(rho[c]) * (vxx * vxx + vyy * vyy);
          const double l = lam[c], m = mu[c];
          const double s1 = sxx[c], s2 = syy[c], s3 = sxy[c];
          const double exx = ((l + 2.0 * m) * s1 - l * s2) / (4.0 * m * (l + m));
          const double eyy = ((l + 2.0 * m) * s2 - l * s1) / (4.0 * m * (l + m));
          const double exy = s3 / (2.0 * m);
          ep = ep + 0.5 * (exx * s1 + eyy * s2 + 2.0 * exy * s3);
        }
      if (o.ek) o.ek[it - 1] = 0.5 * ek;
      if (o.ep) o.ep[it - 1] = ep;
    }
    if (o.vmax) {
      double vm = 0.0;
      for (size_t c = 0; c < N; ++c)
        vm = std::max(vm, std::sqrt(double(vx[c]) * vx[c] + double(vy[c]) * vy[c]));
      o.vmax[it - 1] = vm;
    }
  }

// one pass of the fourth-order program's time loop (2D4:553-745): the same
// sweeps with the 27/24 staggered operator, arrays 0:NX+1 x 0:NY+1 whose
// ghost layer is never written (zero), dvx_dy corrected with K_y rather than
// K_y_half (2D4:596), and the energy over [NPML, N-NPML+1] (2D4:696-712)
template <typename R>
void State2D<R>::step4(int it, const Out& o) {
    auto G = [&](const std::vector<R>& v, int i, int j) -> R {
      return (i < 1 || i > NX || j < 1 || j > NY) ? R(0) : v[at(i, j)];
    };
    const R c27 = R(27.0), dx24 = R(24.0) * DX, dy24 = R(24.0) * DY;
    // 27/24 difference of a staggered pair: (27 f(p1) - 27 f(p0) - f(p2) + f(m1)) / (24 h)
    auto D = [&](R p1, R p0, R p2, R m1, R h24) { return (c27 * p1 - c27 * p0 - p2 + m1) / h24; };
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j);
        R lam_hx = R(0.5) * (lam[at(i + 1, j)] + lam[c]);
        R mu_hx = R(0.5) * (mu[at(i + 1, j)] + mu[c]);
        R l2m = lam_hx + R(2.0) * mu_hx;
        R dvx_dx = D(G(vx, i + 1, j), G(vx, i, j), G(vx, i + 2, j), G(vx, i - 1, j), dx24);
        R dvy_dy = D(G(vy, i, j), G(vy, i, j - 1), G(vy, i, j + 1), G(vy, i, j - 2), dy24);
        m_dvx_dx[c] = X.bh[i - 1] * m_dvx_dx[c] + X.ah[i - 1] * dvx_dx;
        m_dvy_dy[c] = Y.b[j - 1] * m_dvy_dy[c] + Y.a[j - 1] * dvy_dy;
        dvx_dx = dvx_dx / X.Kh[i - 1] + m_dvx_dx[c];
        dvy_dy = dvy_dy / Y.K[j - 1] + m_dvy_dy[c];
        sxx[c] = sxx[c] + (l2m * dvx_dx + lam_hx * dvy_dy) * DT;
        syy[c] = syy[c] + (lam_hx * dvx_dx + l2m * dvy_dy) * DT;
      }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j);
        R mu_hy = R(0.5) * (mu[at(i, j + 1)] + mu[c]);
        R dvy_dx = D(G(vy, i, j), G(vy, i - 1, j), G(vy, i + 1, j), G(vy, i - 2, j), dx24);
        R dvx_dy = D(G(vx, i, j + 1), G(vx, i, j), G(vx, i, j + 2), G(vx, i, j - 1), dy24);
        m_dvy_dx[c] = X.b[i - 1] * m_dvy_dx[c] + X.a[i - 1] * dvy_dx;
        m_dvx_dy[c] = Y.bh[j - 1] * m_dvx_dy[c] + Y.ah[j - 1] * dvx_dy;
        dvy_dx = dvy_dx / X.K[i - 1] + m_dvy_dx[c];
        dvx_dy = dvx_dy / Y.K[j - 1] + m_dvx_dy[c];   // K_y, as 2D4:596 has it
        sxy[c] = sxy[c] + mu_hy * (dvy_dx + dvx_dy) * DT;
      }
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j);
        R d1 = D(G(sxx, i, j), G(sxx, i - 1, j), G(sxx, i + 1, j), G(sxx, i - 2, j), dx24);
        R d2 = D(G(sxy, i, j), G(sxy, i, j - 1), G(sxy, i, j + 1), G(sxy, i, j - 2), dy24);
        m_dsxx_dx[c] = X.b[i - 1] * m_dsxx_dx[c] + X.a[i - 1] * d1;
        m_dsxy_dy[c] = Y.b[j - 1] * m_dsxy_dy[c] + Y.a[j - 1] * d2;
        d1 = d1 / X.K[i - 1] + m_dsxx_dx[c];
        d2 = d2 / Y.K[j - 1] + m_dsxy_dy[c];
        vx[c] = vx[c] + (d1 + d2) * DT / rho[c];
      }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j);
        R rhh = R(0.25) * (rho[c] + rho[at(i + 1, j)] + rho[at(i + 1, j + 1)] + rho[at(i, j + 1)]);
        R d1 = D(G(sxy, i + 1, j), G(sxy, i, j), G(sxy, i + 2, j), G(sxy, i - 1, j), dx24);
        R d2 = D(G(syy, i, j + 1), G(syy, i, j), G(syy, i, j + 2), G(syy, i, j - 1), dy24);
        m_dsxy_dx[c] = X.bh[i - 1] * m_dsxy_dx[c] + X.ah[i - 1] * d1;
        m_dsyy_dy[c] = Y.bh[j - 1] * m_dsyy_dy[c] + Y.ah[j - 1] * d2;
        d1 = d1 / X.Kh[i - 1] + m_dsxy_dx[c];
        d2 = d2 / Y.Kh[j - 1] + m_dsyy_dy[c];
        vy[c] = vy[c] + (d1 + d2) * DT / rhh;
      }
    {  // source (2D4:672-680)
      const double st = source_term(p, it);
      const R fx = R(sa * st), fy = R(ca * st);
      const int i = p->isource, j = p->jsource;
      R rhh = R(0.25) * (rho[at(i, j)] + rho[at(i + 1, j)] + rho[at(i + 1, j + 1)] + rho[at(i, j + 1)]);
      vx[at(i, j)] = vx[at(i, j)] + fx * DT / rho[at(i, j)];
      vy[at(i, j)] = vy[at(i, j)] + fy * DT / rhh;
    }
    for (int j = 1; j <= NY; ++j) {   // rigid edges (2D4:683-693)
      vx[at(1, j)] = 0; vx[at(NX, j)] = 0; vy[at(1, j)] = 0; vy[at(NX, j)] = 0;
    }
    for (int i = 1; i <= NX; ++i) {
      vx[at(i, 1)] = 0; vx[at(i, NY)] = 0; vy[at(i, 1)] = 0; vy[at(i, NY)] = 0;
    }
    for (int r = 0; r < o.nrec; ++r) {
      o.sisvx[size_t(r) * o.nsteps + it - 1] = double(vx[at(o.ix[r], o.iy[r])]);
      o.sisvy[size_t(r) * o.nsteps + it - 1] = double(vy[at(o.ix[r], o.iy[r])]);
    }
    if (o.ek || o.ep) {   // one cell wider than the second-order program's interior
      double ek = 0.0, ep = 0.0;
      for (int j = npml; j <= NY - npml + 1; ++j)
        for (int i = npml; i <= NX - npml + 1; ++i) {
          const size_t c = at(i, j);
          const double vxx = vx[c], vyy = vy[c];
          ek = ek + double(rho[c]) * (vxx * vxx + vyy * vyy);
          const double l = lam[c], m = mu[c];
          const double s1 = sxx[c], s2 = syy[c], s3 = sxy[c];
          const double exx = ((l + 2.0 * m) * s1 - l * s2) / (4.0 * m * (l + m));
          const double eyy = ((l + 2.0 * m) * s2 - l * s1) / (4.0 * m * (l + m));
          const double exy = s3 / (2.0 * m);
          ep = ep + 0.5 * (exx * s1 + eyy * s2 + 2.0 * exy * s3);
        }
      if (o.ek) o.ek[it - 1] = 0.5 * ek;
      if (o.ep) o.ep[it - 1] = ep;
    }
    if (o.vmax) {
      double vm = 0.0;
      for (size_t c = 0; c < N; ++c)
        vm = std::max(vm, std::sqrt(double(vx[c]) * vx[c] + double(vy[c]) * vy[c]));
      o.vmax[it - 1] = vm;
    }
  }

// ---------------------------------------------------------------------------
// classical split-field PML program (Collino and Tsogka), PML:180-533
// ---------------------------------------------------------------------------
// Damping profile divided by two at grid and half points of one axis
// (PML:204-226 for x, 228-250 for y): d0 = 3 cp ln(1/Rcoef) / (2 delta),
// quadratic, with the reference's 0.9999 factor on the high-side test.
void split_profile(const cpml_params* p, int n, double h, std::vector<double>& full,
                   std::vector<double>& half) {
  const double delta = p->npoints_pml * h;
  const double d0 = 3.0 * p->cp * std::log(1.0 / p->rcoef) / (2.0 * delta);
  const double ol = delta, orr = (n - 1) * h - delta;
  full.assign(n, 0.0);
  half.assign(n, 0.0);
  for (int i = 1; i <= n; ++i) {
    const double xval = h * double(i - 1);
    double f = 0.0, g = 0.0;
    if (xval < ol) {
      f = d0 * std::pow((ol - xval) / delta, 2);
      g = d0 * std::pow((ol - xval - h / 2.0) / delta, 2);
    } else if (xval >= 0.9999 * orr) {
      f = d0 * std::pow((xval - orr) / delta, 2);
      g = d0 * std::pow((xval + h / 2.0 - orr) / delta, 2);
    }
    full[i - 1] = f / 2.0;
    half[i - 1] = g / 2.0;
  }
}

template <typename R>
struct StateSplit {
  const cpml_params* p;
  int NX, NY;
  size_t N;
  R h, odt, rho, lam, mu, l2m;
  std::vector<R> dx2, dxh2, dy2, dyh2;
  std::vector<R> vx1, vx2, vy1, vy2, sxx1, sxx2, syy1, syy2, sxy1, sxy2;
  int npml;
  double sa, ca;
  explicit StateSplit(const cpml_params* p_)
      : p(p_), NX(p_->nx), NY(p_->ny), N(size_t(p_->nx) * p_->ny) {
    h = R(p->deltax);
    odt = R(1.0 / p->deltat);                             // ONE_OVER_DELTAT (PML:118)
    rho = R(p->rho);
    mu = R(p->rho * p->cs * p->cs);                       // PML:108-110
    lam = R(p->rho * (p->cp * p->cp - 2.0 * p->cs * p->cs));
    l2m = R(p->rho * p->cp * p->cp);
    std::vector<double> f, g;
    auto cv = [](const std::vector<double>& v) { return std::vector<R>(v.begin(), v.end()); };
    split_profile(p, NX, p->deltax, f, g); dx2 = cv(f); dxh2 = cv(g);
    split_profile(p, NY, p->deltay, f, g); dy2 = cv(f); dyh2 = cv(g);
    for (auto* v : {&vx1, &vx2, &vy1, &vy2, &sxx1, &sxx2, &syy1, &syy2, &sxy1, &sxy2}) v->assign(N, R(0));
    npml = p->npoints_pml;
    const double ang = p->angle_force * (PI / 180.0);
    sa = std::sin(ang); ca = std::cos(ang);
  }
  size_t at(int i, int j) const { return size_t(j - 1) * NX + (i - 1); }
  void advance(int it, const Out& o);
  void fields(double* out) const {   // total fields vx vy sxx syy sxy
    const std::vector<R>* A[5] = {&vx1, &vy1, &sxx1, &syy1, &sxy1};
    const std::vector<R>* B[5] = {&vx2, &vy2, &sxx2, &syy2, &sxy2};
    for (int f = 0; f < 5; ++f)
      for (size_t c = 0; c < N; ++c) out[f * N + c] = double((*A[f])[c]) + double((*B[f])[c]);
  }
};

// one pass of PML:337-533
template <typename R>
void StateSplit<R>::advance(int it, const Out& o) {
    auto upd = [&](R old, R d, R rhs) { return (old * (odt - d) + rhs) / (odt + d); };
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)            // PML:344-364
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j), e = at(i + 1, j), s_ = at(i, j - 1);
        const R vdx = (vx1[e] - vx1[c]) / h + (vx2[e] - vx2[c]) / h;
        const R vdy = (vy1[c] - vy1[s_]) / h + (vy2[c] - vy2[s_]) / h;
        R d = dxh2[i - 1];
        sxx1[c] = upd(sxx1[c], d, l2m * vdx);
        syy1[c] = upd(syy1[c], d, lam * vdx);
        d = dy2[j - 1];
        sxx2[c] = upd(sxx2[c], d, lam * vdy);
        syy2[c] = upd(syy2[c], d, l2m * vdy);
      }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)        // PML:366-383
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j), w = at(i - 1, j), n_ = at(i, j + 1);
        const R vdx = (vy1[c] - vy1[w]) / h + (vy2[c] - vy2[w]) / h;
        const R vdy = (vx1[n_] - vx1[c]) / h + (vx2[n_] - vx2[c]) / h;
        sxy1[c] = upd(sxy1[c], dx2[i - 1], mu * vdx);
        sxy2[c] = upd(sxy2[c], dyh2[j - 1], mu * vdy);
      }
#pragma omp parallel for schedule(static)
    for (int j = 2; j <= NY; ++j)            // PML:389-406
      for (int i = 2; i <= NX; ++i) {
        const size_t c = at(i, j), w = at(i - 1, j), s_ = at(i, j - 1);
        const R sdx = (sxx1[c] - sxx1[w]) / h + (sxx2[c] - sxx2[w]) / h;
        const R sdy = (sxy1[c] - sxy1[s_]) / h + (sxy2[c] - sxy2[s_]) / h;
        vx1[c] = upd(vx1[c], dx2[i - 1], sdx / rho);
        vx2[c] = upd(vx2[c], dy2[j - 1], sdy / rho);
      }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY - 1; ++j)        // PML:408-425
      for (int i = 1; i <= NX - 1; ++i) {
        const size_t c = at(i, j), e = at(i + 1, j), n_ = at(i, j + 1);
        const R sdx = (sxy1[e] - sxy1[c]) / h + (sxy2[e] - sxy2[c]) / h;
        const R sdy = (syy1[n_] - syy1[c]) / h + (syy2[n_] - syy2[c]) / h;
        vy1[c] = upd(vy1[c], dxh2[i - 1], sdx / rho);
        vy2[c] = upd(vy2[c], dyh2[j - 1], sdy / rho);
      }
    {  // source on the first split component (PML:428-451)
      const double st = source_term(p, it);
      const size_t c = at(p->isource, p->jsource);
      vx1[c] = vx1[c] + R(sa * st) * R(p->deltat) / rho;
      vy1[c] = vy1[c] + R(ca * st) * R(p->deltat) / rho;
    }
    for (int j = 1; j <= NY; ++j)            // rigid edges, both components (PML:453-478)
      for (auto* v : {&vx1, &vy1, &vx2, &vy2}) { (*v)[at(1, j)] = 0; (*v)[at(NX, j)] = 0; }
    for (int i = 1; i <= NX; ++i)
      for (auto* v : {&vx1, &vy1, &vx2, &vy2}) { (*v)[at(i, 1)] = 0; (*v)[at(i, NY)] = 0; }
    for (int r = 0; r < o.nrec; ++r) {       // PML:481-484
      const size_t c = at(o.ix[r], o.iy[r]);
      o.sisvx[size_t(r) * o.nsteps + it - 1] = double(vx1[c]) + double(vx2[c]);
      o.sisvy[size_t(r) * o.nsteps + it - 1] = double(vy1[c]) + double(vy2[c]);
    }
    if (o.ek || o.ep) {                      // PML:486-515
      const double l = double(lam), m = double(mu), r = double(rho);
      double ek = 0.0, ep = 0.0;
      for (int j = npml + 1; j <= NY - npml; ++j)
        for (int i = npml + 1; i <= NX - npml; ++i) {
          const size_t c = at(i, j);
          const double vxt = double(vx1[c]) + double(vx2[c]), vyt = double(vy1[c]) + double(vy2[c]);
          ek = ek + r * (vxt * vxt + vyt * vyt);
          const double s1 = double(sxx1[c]) + double(sxx2[c]);
          const double s2 = double(syy1[c]) + double(syy2[c]);
          const double s3 = double(sxy1[c]) + double(sxy2[c]);
          const double exx = ((l + 2.0 * m) * s1 - l * s2) / (4.0 * m * (l + m));
          const double eyy = ((l + 2.0 * m) * s2 - l * s1) / (4.0 * m * (l + m));
          const double exy = s3 / (2.0 * m);
          ep = ep + 0.5 * (exx * s1 + eyy * s2 + 2.0 * exy * s3);
        }
      if (o.ek) o.ek[it - 1] = 0.5 * ek;
      if (o.ep) o.ep[it - 1] = ep;
    }
    if (o.vmax) {
      double vm = 0.0;
      for (size_t c = 0; c < N; ++c) {
        const double a = double(vx1[c]) + double(vx2[c]), b = double(vy1[c]) + double(vy2[c]);
        vm = std::max(vm, std::sqrt(a * a + b * b));
      }
      o.vmax[it - 1] = vm;
    }
  }

template <typename R>
int run_split(const cpml_params* p, const Out& o, double* fields_out) {
  StateSplit<R> S(p);
  for (int it = 1; it <= o.nsteps; ++it) S.advance(it, o);
  if (fields_out) S.fields(fields_out);
  return CPML_OK;
}

template <typename R>
int run2d(const cpml_params* p, const double* lam_in, const double* mu_in,
          const double* rho_in, const Out& o, double* fields_out) {
  State2D<R> S(p, lam_in, mu_in, rho_in);
  for (int it = 1; it <= o.nsteps; ++it) S.advance(it, o);
  if (fields_out) S.fields(fields_out);
  return CPML_OK;
}

// ---------------------------------------------------------------------------
// 3D program, time loop 3D:802-1180, one domain of NZ planes
// ---------------------------------------------------------------------------
template <typename R>
struct State3D {
  const cpml_params* p;
  int NX, NY, NZ;
  size_t N, SX, SY, SZ;
  bool het;
  double lam0, mu0, l2m0;
  std::vector<R> lam, mu, rho;
  Prof1<R> X, Y, Z;
  R DT, odx, ody, odz, DT_lam0, DT_mu0, DT_l2m0, DT_rho0;
  std::vector<R> vx, vy, vz, sxx, syy, szz, sxy, sxz, syz;
  std::vector<R> m_dvx_dx, m_dvx_dy, m_dvx_dz, m_dvy_dx, m_dvy_dy, m_dvy_dz, m_dvz_dx, m_dvz_dy,
      m_dvz_dz, m_dsxx_dx, m_dsyy_dy, m_dszz_dz, m_dsxy_dx, m_dsxy_dy, m_dsxz_dx, m_dsxz_dz,
      m_dsyz_dy, m_dsyz_dz;
  int npml;
  double sa, ca;
  bool q1;
  std::vector<double> ekk, epk;
  State3D(const cpml_params* p_, const double* lam_in, const double* mu_in, const double* rho_in)
      : p(p_), NX(p_->nx), NY(p_->ny), NZ(p_->nz), N(size_t(p_->nx) * p_->ny * p_->nz), SX(1),
        SY(size_t(p_->nx)), SZ(size_t(p_->nx) * p_->ny), het(lam_in || mu_in || rho_in),
        X(build_profile(p_, 0, p_->nx, p_->deltax)), Y(build_profile(p_, 1, p_->ny, p_->deltay)),
        Z(build_profile(p_, 2, p_->nz, p_->deltaz)) {
    lam0 = p->rho * (p->cp * p->cp - 2.0 * p->cs * p->cs);  // 3D:142-144
    mu0 = p->rho * p->cs * p->cs;
    l2m0 = p->rho * p->cp * p->cp;
    if (het) {
      lam.resize(N); mu.resize(N); rho.resize(N);
      for (size_t c = 0; c < N; ++c) {
        lam[c] = R(lam_in ? lam_in[c] : lam0);
        mu[c] = R(mu_in ? mu_in[c] : mu0);
        rho[c] = R(rho_in ? rho_in[c] : p->rho);
      }
    }
    DT = R(p->deltat);
    odx = R(1.0 / p->deltax); ody = R(1.0 / p->deltay); odz = R(1.0 / p->deltaz);
    DT_lam0 = R(p->deltat * lam0); DT_mu0 = R(p->deltat * mu0);   // 3D:296-300
    DT_l2m0 = R(p->deltat * l2m0); DT_rho0 = R(p->deltat / p->rho);
    for (auto* v : {&vx, &vy, &vz, &sxx, &syy, &szz, &sxy, &sxz, &syz, &m_dvx_dx, &m_dvx_dy,
                    &m_dvx_dz, &m_dvy_dx, &m_dvy_dy, &m_dvy_dz, &m_dvz_dx, &m_dvz_dy, &m_dvz_dz,
                    &m_dsxx_dx, &m_dsyy_dy, &m_dszz_dz, &m_dsxy_dx, &m_dsxy_dy, &m_dsxz_dx,
                    &m_dsxz_dz, &m_dsyz_dy, &m_dsyz_dz})
      v->assign(N, R(0));
    npml = p->npoints_pml;
    const double ang = p->angle_force * (PI / 180.0);
    sa = std::sin(ang); ca = std::cos(ang);
    q1 = !(p->flags & CPML_FLAG_EP_PHYSICAL);
    ekk.assign(NZ + 1, 0.0); epk.assign(NZ + 1, 0.0);
  }
  size_t at(int i, int j, int k) const { return size_t(k - 1) * SZ + size_t(j - 1) * SY + (i - 1); }
  void step(int it, const Out& o);
  void fields(double* out) const {
    const std::vector<R>* F[9] = {&vx, &vy, &vz, &sxx, &syy, &szz, &sxy, &sxz, &syz};
    for (int f = 0; f < 9; ++f)
      for (size_t c = 0; c < N; ++c) out[f * N + c] = double((*F[f])[c]);
  }
};

// one pass of the time loop 3D:802-1180
template <typename R>
void State3D<R>::step(int it, const Out& o) {
    // normal stresses: k = 2..NZ, j = 2..NY, i = 1..NX-1 (3D:836-863)
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= NZ; ++k)
      for (int j = 2; j <= NY; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = at(i, j, k);
          R dvx_dx = (vx[c + SX] - vx[c]) * odx;
          R dvy_dy = (vy[c] - vy[c - SY]) * ody;
          R dvz_dz = (vz[c] - vz[c - SZ]) * odz;
          m_dvx_dx[c] = X.bh[i - 1] * m_dvx_dx[c] + X.ah[i - 1] * dvx_dx;
          m_dvy_dy[c] = Y.b[j - 1] * m_dvy_dy[c] + Y.a[j - 1] * dvy_dy;
          m_dvz_dz[c] = Z.b[k - 1] * m_dvz_dz[c] + Z.a[k - 1] * dvz_dz;
          dvx_dx = dvx_dx / X.Kh[i - 1] + m_dvx_dx[c];
          dvy_dy = dvy_dy / Y.K[j - 1] + m_dvy_dy[c];
          dvz_dz = dvz_dz / Z.K[k - 1] + m_dvz_dz[c];
          R DTl = DT_lam0, DTl2m = DT_l2m0;
          if (het) {
            R lhx = R(0.5) * (lam[c + SX] + lam[c]);
            R mhx = R(0.5) * (mu[c + SX] + mu[c]);
            DTl = DT * lhx;
            DTl2m = DT * (lhx + R(2.0) * mhx);
          }
          sxx[c] = DTl2m * dvx_dx + DTl * (dvy_dy + dvz_dz) + sxx[c];
          syy[c] = DTl * (dvx_dx + dvz_dz) + DTl2m * dvy_dy + syy[c];
          szz[c] = DTl * (dvx_dx + dvy_dy) + DTl2m * dvz_dz + szz[c];
        }
    // sigma_xy: k = 1..NZ, j = 1..NY-1, i = 2..NX (3D:877-894)
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 2; i <= NX; ++i) {
          const size_t c = at(i, j, k);
          R dvy_dx = (vy[c] - vy[c - SX]) * odx;
          R dvx_dy = (vx[c + SY] - vx[c]) * ody;
          m_dvy_dx[c] = X.b[i - 1] * m_dvy_dx[c] + X.a[i - 1] * dvy_dx;
          m_dvx_dy[c] = Y.bh[j - 1] * m_dvx_dy[c] + Y.ah[j - 1] * dvx_dy;
          dvy_dx = dvy_dx / X.K[i - 1] + m_dvy_dx[c];
          dvx_dy = dvx_dy / Y.Kh[j - 1] + m_dvx_dy[c];
          R DTm = het ? DT * (R(0.5) * (mu[c + SY] + mu[c])) : DT_mu0;
          sxy[c] = DTm * (dvy_dx + dvx_dy) + sxy[c];
        }
    // sigma_xz and sigma_yz: k = 1..NZ-1 (3D:908-943)
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k) {
      for (int j = 1; j <= NY; ++j)
        for (int i = 2; i <= NX; ++i) {
          const size_t c = at(i, j, k);
          R dvz_dx = (vz[c] - vz[c - SX]) * odx;
          R dvx_dz = (vx[c + SZ] - vx[c]) * odz;
          m_dvz_dx[c] = X.b[i - 1] * m_dvz_dx[c] + X.a[i - 1] * dvz_dx;
          m_dvx_dz[c] = Z.bh[k - 1] * m_dvx_dz[c] + Z.ah[k - 1] * dvx_dz;
          dvz_dx = dvz_dx / X.K[i - 1] + m_dvz_dx[c];
          dvx_dz = dvx_dz / Z.Kh[k - 1] + m_dvx_dz[c];
          R DTm = het ? DT * (R(0.5) * (mu[c + SZ] + mu[c])) : DT_mu0;
          sxz[c] = DTm * (dvz_dx + dvx_dz) + sxz[c];
        }
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 1; i <= NX; ++i) {
          const size_t c = at(i, j, k);
          R dvz_dy = (vz[c + SY] - vz[c]) * ody;
          R dvy_dz = (vy[c + SZ] - vy[c]) * odz;
          m_dvz_dy[c] = Y.bh[j - 1] * m_dvz_dy[c] + Y.ah[j - 1] * dvz_dy;
          m_dvy_dz[c] = Z.bh[k - 1] * m_dvy_dz[c] + Z.ah[k - 1] * dvy_dz;
          dvz_dy = dvz_dy / Y.Kh[j - 1] + m_dvz_dy[c];
          dvy_dz = dvy_dz / Z.Kh[k - 1] + m_dvy_dz[c];
          R DTm = DT_mu0;
          if (het) {
            // sigma_yz sits at (i+1/2, j+1/2, k+1/2): 8-point average; on the
            // last column (never read by the velocity sweeps) i+1 is clamped.
            const size_t di = (i < NX) ? SX : 0;
            const R s = ((((((mu[c] + mu[c + di]) + mu[c + SY]) + mu[c + SY + di]) + mu[c + SZ]) +
                          mu[c + SZ + di]) + mu[c + SZ + SY]) + mu[c + SZ + SY + di];
            DTm = DT * (R(0.125) * s);
          }
          syz[c] = DTm * (dvz_dy + dvy_dz) + syz[c];
        }
    }
    // v_x and v_y: k = 2..NZ (3D:976-1017)
#pragma omp parallel for schedule(static)
    for (int k = 2; k <= NZ; ++k) {
      for (int j = 2; j <= NY; ++j)
        for (int i = 2; i <= NX; ++i) {
          const size_t c = at(i, j, k);
          R d1 = (sxx[c] - sxx[c - SX]) * odx;
          R d2 = (sxy[c] - sxy[c - SY]) * ody;
          R d3 = (sxz[c] - sxz[c - SZ]) * odz;
          m_dsxx_dx[c] = X.b[i - 1] * m_dsxx_dx[c] + X.a[i - 1] * d1;
          m_dsxy_dy[c] = Y.b[j - 1] * m_dsxy_dy[c] + Y.a[j - 1] * d2;
          m_dsxz_dz[c] = Z.b[k - 1] * m_dsxz_dz[c] + Z.a[k - 1] * d3;
          d1 = d1 / X.K[i - 1] + m_dsxx_dx[c];
          d2 = d2 / Y.K[j - 1] + m_dsxy_dy[c];
          d3 = d3 / Z.K[k - 1] + m_dsxz_dz[c];
          R f = het ? DT / rho[c] : DT_rho0;
          vx[c] = f * (d1 + d2 + d3) + vx[c];
        }
      for (int j = 1; j <= NY - 1; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = at(i, j, k);
          R d1 = (sxy[c + SX] - sxy[c]) * odx;
          R d2 = (syy[c + SY] - syy[c]) * ody;
          R d3 = (syz[c] - syz[c - SZ]) * odz;
          m_dsxy_dx[c] = X.bh[i - 1] * m_dsxy_dx[c] + X.ah[i - 1] * d1;
          m_dsyy_dy[c] = Y.bh[j - 1] * m_dsyy_dy[c] + Y.ah[j - 1] * d2;
          m_dsyz_dz[c] = Z.b[k - 1] * m_dsyz_dz[c] + Z.a[k - 1] * d3;
          d1 = d1 / X.Kh[i - 1] + m_dsxy_dx[c];
          d2 = d2 / Y.Kh[j - 1] + m_dsyy_dy[c];
          d3 = d3 / Z.K[k - 1] + m_dsyz_dz[c];
          R f = DT_rho0;
          if (het) f = DT / (R(0.25) * (rho[c] + rho[c + SX] + rho[c + SX + SY] + rho[c + SY]));
          vy[c] = f * (d1 + d2 + d3) + vy[c];
        }
    }
    // v_z: k = 1..NZ-1, j = 2..NY, i = 1..NX-1 (3D:1031-1052)
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ - 1; ++k)
      for (int j = 2; j <= NY; ++j)
        for (int i = 1; i <= NX - 1; ++i) {
          const size_t c = at(i, j, k);
          R d1 = (sxz[c + SX] - sxz[c]) * odx;
          R d2 = (syz[c] - syz[c - SY]) * ody;
          R d3 = (szz[c + SZ] - szz[c]) * odz;
          m_dsxz_dx[c] = X.bh[i - 1] * m_dsxz_dx[c] + X.ah[i - 1] * d1;
          m_dsyz_dy[c] = Y.b[j - 1] * m_dsyz_dy[c] + Y.a[j - 1] * d2;
          m_dszz_dz[c] = Z.bh[k - 1] * m_dszz_dz[c] + Z.ah[k - 1] * d3;
          d1 = d1 / X.Kh[i - 1] + m_dsxz_dx[c];
          d2 = d2 / Y.K[j - 1] + m_dsyz_dy[c];
          d3 = d3 / Z.Kh[k - 1] + m_dszz_dz[c];
          R f = DT_rho0;
          if (het) f = DT / (R(0.25) * (rho[c] + rho[c + SX] + rho[c + SX + SZ] + rho[c + SZ]));
          vz[c] = f * (d1 + d2 + d3) + vz[c];
        }
    // source on plane ksource, plain rho (3D:1055-1083)
    {
      const double st = source_term(p, it);
      const double fx = sa * st, fy = ca * st;
      const size_t c = at(p->isource, p->jsource, p->ksource);
      if (het) {
        vx[c] = vx[c] + R(fx) * DT / rho[c];
        vy[c] = vy[c] + R(fy) * DT / rho[c];
      } else {
        vx[c] = vx[c] + R(fx * p->deltat / p->rho);
        vy[c] = vy[c] + R(fy * p->deltat / p->rho);
      }
    }
    // Dirichlet on the six faces (3D:1087-1121)
    std::vector<R>* V[3] = {&vx, &vy, &vz};
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= NZ; ++k)
      for (int f = 0; f < 3; ++f) {
        std::vector<R>& a = *V[f];
        for (int j = 1; j <= NY; ++j) { a[at(1, j, k)] = 0; a[at(NX, j, k)] = 0; }
        for (int i = 1; i <= NX; ++i) { a[at(i, 1, k)] = 0; a[at(i, NY, k)] = 0; }
        if (k == 1 || k == NZ)
          for (int j = 1; j <= NY; ++j)
            for (int i = 1; i <= NX; ++i) a[at(i, j, k)] = 0;
      }
    // seismograms (3D:1124-1129)
    for (int r = 0; r < o.nrec; ++r) {
      const size_t c = at(o.ix[r], o.iy[r], o.iz[r]);
      o.sisvx[size_t(r) * o.nsteps + it - 1] = double(vx[c]);
      o.sisvy[size_t(r) * o.nsteps + it - 1] = double(vy[c]);
      if (o.sisvz) o.sisvz[size_t(r) * o.nsteps + it - 1] = double(vz[c]);
    }
    // energy (3D:1131-1180): per-plane partials, summed in k order
    if (o.ek || o.ep) {
#pragma omp parallel for schedule(static)
      for (int k = npml + 1; k <= NZ - npml; ++k) {
        double ek = 0.0, ep = 0.0;
        for (int j = npml + 1; j <= NY - npml; ++j)
          for (int i = npml + 1; i <= NX - npml; ++i) {
            const size_t c = at(i, j, k);
            const double r = het ? double(rho[c]) : p->rho;
            const double l = het ? double(lam[c]) : lam0;
            const double m = het ? double(mu[c]) : mu0;
            const double a = vx[c], b = vy[c], cc = vz[c];
            ek = ek + 0.5 * r * (a * a + b * b + cc * cc);
            const double s1 = sxx[c], s2 = syy[c], s3 = szz[c];
            const double s4 = sxy[c], s5 = sxz[c], s6 = syz[c];
            const double den = 2.0 * m * (3.0 * l + 2.0 * m);
            const double exx = (2.0 * (l + m) * s1 - l * s2 - l * s3) / den;
            const double eyy = (2.0 * (l + m) * s2 - l * s1 - l * s3) / den;
            const double ezz = (2.0 * (l + m) * s3 - l * s1 - l * s2) / den;
            const double exy = s4 / (2.0 * m), exz = s5 / (2.0 * m), eyz = s6 / (2.0 * m);
            const double third = q1 ? eyy * s2 : ezz * s3;
            ep = ep + 0.5 * (exx * s1 + eyy * s2 + third + 2.0 * exy * s4 + 2.0 * exz * s5 +
                             2.0 * eyz * s6);
          }
        ekk[k] = ek; epk[k] = ep;
      }
      double ek = 0.0, ep = 0.0;
      for (int k = npml + 1; k <= NZ - npml; ++k) { ek += ekk[k]; ep += epk[k]; }
      if (o.ek) o.ek[it - 1] = ek;
      if (o.ep) o.ep[it - 1] = ep;
    }
    if (o.vmax) {
      double vm = 0.0;
#pragma omp parallel for reduction(max : vm) schedule(static)
      for (long long c = 0; c < (long long)N; ++c)
        vm = std::max(vm, std::sqrt(double(vx[c]) * vx[c] + double(vy[c]) * vy[c] +
                                    double(vz[c]) * vz[c]));
      o.vmax[it - 1] = vm;
    }
  }

template <typename R>
int run3d(const cpml_params* p, const double* lam_in, const double* mu_in,
          const double* rho_in, const Out& o, double* fields_out) {
  State3D<R> S(p, lam_in, mu_in, rho_in);
  for (int it = 1; it <= o.nsteps; ++it) S.step(it, o);
  if (fields_out) S.fields(fields_out);
  return CPML_OK;
}

}  // namespace

extern "C" {

// Run the restated program for nsteps steps.
//   use_double: 1 = FP64 oracle, 0 = FP32 floor study.
//   lam/mu/rho: per-cell model (NULL = homogeneous), [k][j][i] doubles.
//   receivers: 1-based (ix, iy, iz); iz ignored in 2D.
//   sisv*: [nrec][nsteps]; ek/ep/vmax: [nsteps]; any output may be NULL.
//   fields_out: 5 (2D) or 9 (3D) fields x ncell doubles, in the order
//   vx vy (vz) sxx syy (szz) sxy (sxz syz); may be NULL.
//   nthreads <= 0 keeps the OpenMP default.
int oracle_run(const cpml_params* p, int nsteps, int use_double, const double* lam,
               const double* mu, const double* rho, int nrec, const int* ix, const int* iy,
               const int* iz, double* sisvx, double* sisvy, double* sisvz, double* ek,
               double* ep, double* vmax, double* fields_out, int nthreads) {
  if (!p || nsteps < 0 || (p->ndim != 2 && p->ndim != 3)) return CPML_ERR_INVALID;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  std::vector<double> sx, sy;
  if (nrec > 0 && !sisvx) { sx.resize(size_t(nrec) * nsteps); sisvx = sx.data(); }
  if (nrec > 0 && !sisvy) { sy.resize(size_t(nrec) * nsteps); sisvy = sy.data(); }
  Out o{nsteps, nrec, ix, iy, iz, sisvx, sisvy, sisvz, ek, ep, vmax};
  if (p->ndim == 2 && p->scheme == CPML_SCHEME_SPLIT) {
    if (lam || mu || rho) return CPML_ERR_INVALID;   // the split-PML program is homogeneous
    return use_double ? run_split<double>(p, o, fields_out) : run_split<float>(p, o, fields_out);
  }
  if (p->ndim == 2)
    return use_double ? run2d<double>(p, lam, mu, rho, o, fields_out)
                      : run2d<float>(p, lam, mu, rho, o, fields_out);
  return use_double ? run3d<double>(p, lam, mu, rho, o, fields_out)
                    : run3d<float>(p, lam, mu, rho, o, fields_out);
}

// A persistent run for timing the reference's time loop without its set-up:
// create (allocates and zeroes like 2D:522-544 / 3D:720-756), then advance.
struct Session {
  cpml_params p;
  State2D<double>* s2 = nullptr;
  State3D<double>* s3 = nullptr;
  int it = 0;
  std::vector<double> ek, ep;
};

void* oracle_session_create(const cpml_params* p, const double* lam, const double* mu,
                            const double* rho, int nthreads) {
  if (!p || (p->ndim != 2 && p->ndim != 3)) return nullptr;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  Session* S = new Session();
  S->p = *p;
  if (p->ndim == 2) S->s2 = new State2D<double>(&S->p, lam, mu, rho);
  else S->s3 = new State3D<double>(&S->p, lam, mu, rho);
  return S;
}

// Advance nsteps steps with the reference's per-step energy; returns steps done.
int oracle_session_run(void* h, int nsteps) {
  Session* S = static_cast<Session*>(h);
  if (!S || nsteps < 0) return CPML_ERR_INVALID;
  S->ek.resize(S->it + nsteps);
  S->ep.resize(S->it + nsteps);
  Out o{S->it + nsteps, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
        S->ek.data(), S->ep.data(), nullptr};
  for (int q = 0; q < nsteps; ++q) {
    ++S->it;
    if (S->s2) S->s2->advance(S->it, o);
    else S->s3->step(S->it, o);
  }
  return S->it;
}

void oracle_session_destroy(void* h) {
  Session* S = static_cast<Session*>(h);
  if (!S) return;
  delete S->s2;
  delete S->s3;
  delete S;
}

// The FP64 profiles of one axis (for tests).
int oracle_profile(const cpml_params* p, int axis, int n, double delta, double* out10) {
  Profile P = build_profile(p, axis, n, delta);
  const std::vector<double>* v[10] = {&P.d, &P.K, &P.alpha, &P.a, &P.b,
                                      &P.dh, &P.Kh, &P.alphah, &P.ah, &P.bh};
  for (int q = 0; q < 10; ++q) std::memcpy(out10 + size_t(q) * n, v[q]->data(), sizeof(double) * n);
  return CPML_OK;
}

double oracle_source_term(const cpml_params* p, int it) { return source_term(p, it); }

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
