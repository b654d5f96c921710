// kernels2d_ext.cu -- the two other 2D programs of the path, two-sweep form.
//
//   stress2d4 / velocity2d4 -- seismic_CPML_2D_isotropic_fourth_order.f90
//       (2D4:553-745): the C-PML time loop of the second-order program with
//       the 27/24 fourth-order staggered operator. The reference holds every
//       array as 0:NX+1 x 0:NY+1 and never writes the ghost layer, so a read
//       outside the grid returns zero here. Its quirks are kept: dvx_dy of
//       sigma_xy is corrected with K_y, not K_y_half (2D4:596), and the energy
//       interior is one cell wider, [NPML, N-NPML+1] (2D4:696-712). The
//       memory variables use the slab layout of the second-order kernels.
//   stress_split / velocity_split -- seismic_PML_Collino_2D_isotropic.f90
//       (PML:337-533): the classical split-field PML. Every field is the sum
//       of an x part (StepArgs::f) and a y part (StepArgs::g), each relaxed by
//       its own axis's damping: new = (old (1/dt - d) + rhs) / (1/dt + d),
//       with d the profile divided by two; the axis tables hold
//       a = 1/dt - d and b = 1/dt + d at grid points, ah/bh at half points.
//       Homogeneous model, one grid spacing h.
// Both use the 32 x 8 tiles of kernels2d.cu, so the per-block energy
// partials and the chunk reduction are shared.
#include "cpml_internal.cuh"
#include "kutil.cuh"
#include "cell2d.cuh"

namespace cpml {

constexpr int E2X = 32, E2Y = 8;

// --------------------------------------------------------------------------
// fourth order
// --------------------------------------------------------------------------
struct Grid2 {
  const int nx, ny;
  const long long px;
  // value of f at (i, j), zero in the reference's ghost layer
  __device__ __forceinline__ float at(const float* __restrict__ f, int i, int j) const {
    return (i >= 0 && i < nx && j >= 0 && j < ny) ? f[(long long)j * px + i] : 0.f;
  }
};

// (27 f(p1) - 27 f(p0) - f(p2) + f(m1)) / (24 h), h given as 1/(24 h)
__device__ __forceinline__ float d4(float p1, float p0, float p2, float m1, float o24h) {
  return __fmul_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fmul_rn(27.f, p1), __fmul_rn(27.f, p0)), p2), m1), o24h);
}

__device__ __forceinline__ void record_receivers2d_ext(const StepArgs& s, int it, long long gtid,
                                                       long long gsize) {
  const size_t slab = (size_t)s.nrec * s.nstep;
  for (long long r = gtid; r < s.nrec; r += gsize) {
    const long long c = s.rec_cell[r];
    const size_t o = (size_t)r * s.nstep + (size_t)(it - 1);
    s.seis[o] = s.split ? __fadd_rn(s.f.vx[c], s.g.vx[c]) : s.f.vx[c];
    s.seis[slab + o] = s.split ? __fadd_rn(s.f.vy[c], s.g.vy[c]) : s.f.vy[c];
  }
}

template <bool HET>
__global__ void __launch_bounds__(E2X* E2Y) stress2d4(StepArgs a, int ls) {
  const int tid = threadIdx.x + threadIdx.y * E2X;
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  if (ls > 0)
    record_receivers2d_ext(a, *a.it_base + ls, blin * (E2X * E2Y) + tid,
                           (long long)gridDim.x * gridDim.y * (E2X * E2Y));
  const int i = blockIdx.x * E2X + threadIdx.x;
  const int j = blockIdx.y * E2Y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const Grid2 g{a.nx, a.ny, a.px};
  const Shot2D s = shot_from_args(a);
  const int sx = s.ax.slab(i), sy = s.ay.slab(j);
  const long long c = (long long)j * g.px + i;
  const long long mx = (long long)j * s.ax.width() + sx;
  const long long my = (long long)sy * g.px + i;
  const float ox = a.o24dx, oy = a.o24dy;
  // sigma_xx, sigma_yy: j = 2..NY, i = 1..NX-1 (2D4:557-580)
  if (j >= 1 && i <= a.nx - 2) {
    float d1 = d4(g.at(s.vx, i + 1, j), g.at(s.vx, i, j), g.at(s.vx, i + 2, j), g.at(s.vx, i - 1, j), ox);
    float d2 = d4(g.at(s.vy, i, j), g.at(s.vy, i, j - 1), g.at(s.vy, i, j + 1), g.at(s.vy, i, j - 2), oy);
    d1 = pml2(d1, sx, s.mx[0], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml2(d2, sy, s.my[1], my, s.ay.a, s.ay.b, s.ay.ik, j);
    float dl = s.dt_lam, dl2m = s.dt_l2m;
    if (HET) {
      const float lh = __fmul_rn(0.5f, __fadd_rn(s.lam[c + 1], s.lam[c]));
      const float mh = __fmul_rn(0.5f, __fadd_rn(s.mu[c + 1], s.mu[c]));
      dl = __fmul_rn(s.dt, lh);
      dl2m = __fmul_rn(s.dt, fmaf(2.0f, mh, lh));
    }
    s.sxx[c] = __fadd_rn(s.sxx[c], fmaf(dl2m, d1, __fmul_rn(dl, d2)));
    s.syy[c] = __fadd_rn(s.syy[c], fmaf(dl, d1, __fmul_rn(dl2m, d2)));
  }
  // sigma_xy: j = 1..NY-1, i = 2..NX (2D4:582-600)
  if (j <= a.ny - 2 && i >= 1) {
    float d1 = d4(g.at(s.vy, i, j), g.at(s.vy, i - 1, j), g.at(s.vy, i + 1, j), g.at(s.vy, i - 2, j), ox);
    float d2 = d4(g.at(s.vx, i, j + 1), g.at(s.vx, i, j), g.at(s.vx, i, j + 2), g.at(s.vx, i, j - 1), oy);
    d1 = pml2(d1, sx, s.mx[1], mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml2(d2, sy, s.my[0], my, s.ay.ah, s.ay.bh, s.ay.ik, j);   // K_y, as 2D4:596
    const float dm = HET ? __fmul_rn(s.dt, __fmul_rn(0.5f, __fadd_rn(s.mu[c + g.px], s.mu[c]))) : s.dt_mu;
    s.sxy[c] = fmaf(dm, __fadd_rn(d1, d2), s.sxy[c]);
  }
}

template <bool HET>
__global__ void __launch_bounds__(E2X* E2Y) velocity2d4(StepArgs a, int ls) {
  const int it = *a.it_base + ls + 1;
  const int i = blockIdx.x * E2X + threadIdx.x;
  const int j = blockIdx.y * E2Y + threadIdx.y;
  float ek = 0.f, ep = 0.f, vm2 = 0.f;
  int bad = 0;
  if (i < a.nx && j < a.ny) {
    const Grid2 g{a.nx, a.ny, a.px};
    const Shot2D s = shot_from_args(a);
    const int sx = s.ax.slab(i), sy = s.ay.slab(j);
    const long long px = g.px;
    const long long c = (long long)j * px + i;
    const long long mx = (long long)j * s.ax.width() + sx;
    const long long my = (long long)sy * px + i;
    const float ox = a.o24dx, oy = a.o24dy;
    float vx = s.vx[c], vy = s.vy[c];
    const float sxx = s.sxx[c], syy = s.syy[c], sxy = s.sxy[c];
    // v_x: j = 2..NY, i = 2..NX (2D4:606-621)
    if (j >= 1 && i >= 1) {
      float d1 = d4(sxx, g.at(s.sxx, i - 1, j), g.at(s.sxx, i + 1, j), g.at(s.sxx, i - 2, j), ox);
      float d2 = d4(sxy, g.at(s.sxy, i, j - 1), g.at(s.sxy, i, j + 1), g.at(s.sxy, i, j - 2), oy);
      d1 = pml2(d1, sx, s.mx[2], mx, s.ax.a, s.ax.b, s.ax.ik, i);
      d2 = pml2(d2, sy, s.my[2], my, s.ay.a, s.ay.b, s.ay.ik, j);
      const float f = HET ? __fdiv_rn(s.dt, s.rho[c]) : s.dt_over_rho;
      vx = fmaf(__fadd_rn(d1, d2), f, vx);
    }
    // v_y: j = 1..NY-1, i = 1..NX-1 (2D4:623-641)
    if (j <= a.ny - 2 && i <= a.nx - 2) {
      float d1 = d4(g.at(s.sxy, i + 1, j), sxy, g.at(s.sxy, i + 2, j), g.at(s.sxy, i - 1, j), ox);
      float d2 = d4(g.at(s.syy, i, j + 1), syy, g.at(s.syy, i, j + 2), g.at(s.syy, i, j - 1), oy);
      d1 = pml2(d1, sx, s.mx[3], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
      d2 = pml2(d2, sy, s.my[3], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
      float f = s.dt_over_rho;
      if (HET) {
        const float* r = s.rho;
        const float r4 = __fadd_rn(__fadd_rn(__fadd_rn(r[c], r[c + 1]), r[c + 1 + px]), r[c + px]);
        f = __fdiv_rn(s.dt, __fmul_rn(0.25f, r4));
      }
      vy = fmaf(__fadd_rn(d1, d2), f, vy);
    }
    if (i == s.isrc && j == s.jsrc) {  // 2D4:672-680
      vx = __fadd_rn(vx, s.src_fx[it - 1]);
      vy = __fadd_rn(vy, s.src_fy[it - 1]);
    }
    if (i == 0 || i == a.nx - 1 || j == 0 || j == a.ny - 1) { vx = 0.f; vy = 0.f; }  // 2D4:683-693
    s.vx[c] = vx;
    s.vy[c] = vy;
    const float v2 = vx * vx + vy * vy;
    vm2 = v2;
    bad = not_finite(v2);
    // energy over Fortran [NPML, N-NPML+1], 0-based [npml-1, n-npml] (2D4:696-712)
    const int lo = a.npml - 1;
    if (i >= lo && i <= a.nx - a.npml && j >= lo && j <= a.ny - a.npml) {
      float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
      if (HET) {
        const float l = s.lam[c], m = s.mu[c];
        const float den = 1.0f / (4.0f * m * (l + m));
        hr = 0.5f * s.rho[c];
        c1 = (l + 2.0f * m) * den;
        c2 = l * den;
        i2m = 1.0f / (2.0f * m);
      }
      ek = hr * v2;
      const float exx = c1 * sxx - c2 * syy;
      const float eyy = c1 * syy - c2 * sxx;
      ep = 0.5f * (exx * sxx + eyy * syy) + i2m * (sxy * sxy);
    }
  }
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  block_partials<E2X * E2Y>(DF{ek, 0.f}, DF{ep, 0.f}, vm2, bad, a.partials + ((size_t)ls * a.nblocks + blin) * 4);
}

// --------------------------------------------------------------------------
// classical split-field PML
// --------------------------------------------------------------------------
// (old * A + rhs) / B with A = 1/dt - d, B = 1/dt + d (PML:352-362 and the like)
__device__ __forceinline__ float relax(float old, float A, float B, float rhs) {
  return __fdiv_rn(fmaf(old, A, rhs), B);
}

__global__ void __launch_bounds__(E2X* E2Y) stress_split(StepArgs a, int ls) {
  const int tid = threadIdx.x + threadIdx.y * E2X;
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  if (ls > 0)
    record_receivers2d_ext(a, *a.it_base + ls, blin * (E2X * E2Y) + tid,
                           (long long)gridDim.x * gridDim.y * (E2X * E2Y));
  const int i = blockIdx.x * E2X + threadIdx.x;
  const int j = blockIdx.y * E2Y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const long long px = a.px, c = (long long)j * px + i;
  const Fields& P = a.f;   // x parts (_1)
  const Fields& Q = a.g;   // y parts (_2)
  const float oh = a.odx;
  // sigma_xx, sigma_yy: j = 2..NY, i = 1..NX-1 (PML:344-364)
  if (j >= 1 && i <= a.nx - 2) {
    const float vdx = __fadd_rn(__fmul_rn(__fsub_rn(P.vx[c + 1], P.vx[c]), oh),
                                __fmul_rn(__fsub_rn(Q.vx[c + 1], Q.vx[c]), oh));
    const float vdy = __fadd_rn(__fmul_rn(__fsub_rn(P.vy[c], P.vy[c - px]), oh),
                                __fmul_rn(__fsub_rn(Q.vy[c], Q.vy[c - px]), oh));
    float A = __ldg(a.ax.ah + i), B = __ldg(a.ax.bh + i);
    P.sxx[c] = relax(P.sxx[c], A, B, __fmul_rn(a.l2m_split, vdx));
    P.syy[c] = relax(P.syy[c], A, B, __fmul_rn(a.lam_split, vdx));
    A = __ldg(a.ay.a + j); B = __ldg(a.ay.b + j);
    Q.sxx[c] = relax(Q.sxx[c], A, B, __fmul_rn(a.lam_split, vdy));
    Q.syy[c] = relax(Q.syy[c], A, B, __fmul_rn(a.l2m_split, vdy));
  }
  // sigma_xy: j = 1..NY-1, i = 2..NX (PML:366-383)
  if (j <= a.ny - 2 && i >= 1) {
    const float vdx = __fadd_rn(__fmul_rn(__fsub_rn(P.vy[c], P.vy[c - 1]), oh),
                                __fmul_rn(__fsub_rn(Q.vy[c], Q.vy[c - 1]), oh));
    const float vdy = __fadd_rn(__fmul_rn(__fsub_rn(P.vx[c + px], P.vx[c]), oh),
                                __fmul_rn(__fsub_rn(Q.vx[c + px], Q.vx[c]), oh));
    P.sxy[c] = relax(P.sxy[c], __ldg(a.ax.a + i), __ldg(a.ax.b + i), __fmul_rn(a.mu_split, vdx));
    Q.sxy[c] = relax(Q.sxy[c], __ldg(a.ay.ah + j), __ldg(a.ay.bh + j), __fmul_rn(a.mu_split, vdy));
  }
}

__global__ void __launch_bounds__(E2X* E2Y) velocity_split(StepArgs a, int ls) {
  const int it = *a.it_base + ls + 1;
  const int i = blockIdx.x * E2X + threadIdx.x;
  const int j = blockIdx.y * E2Y + threadIdx.y;
  float ek = 0.f, ep = 0.f, vm2 = 0.f;
  int bad = 0;
  if (i < a.nx && j < a.ny) {
    const long long px = a.px, c = (long long)j * px + i;
    const Fields& P = a.f;
    const Fields& Q = a.g;
    const float oh = a.odx, orho = a.orho_split;
    float vx1 = P.vx[c], vx2 = Q.vx[c], vy1 = P.vy[c], vy2 = Q.vy[c];
    // v_x: j = 2..NY, i = 2..NX (PML:389-406)
    if (j >= 1 && i >= 1) {
      const float sdx = __fadd_rn(__fmul_rn(__fsub_rn(P.sxx[c], P.sxx[c - 1]), oh),
                                  __fmul_rn(__fsub_rn(Q.sxx[c], Q.sxx[c - 1]), oh));
      const float sdy = __fadd_rn(__fmul_rn(__fsub_rn(P.sxy[c], P.sxy[c - px]), oh),
                                  __fmul_rn(__fsub_rn(Q.sxy[c], Q.sxy[c - px]), oh));
      vx1 = relax(vx1, __ldg(a.ax.a + i), __ldg(a.ax.b + i), __fmul_rn(sdx, orho));
      vx2 = relax(vx2, __ldg(a.ay.a + j), __ldg(a.ay.b + j), __fmul_rn(sdy, orho));
    }
    // v_y: j = 1..NY-1, i = 1..NX-1 (PML:408-425)
    if (j <= a.ny - 2 && i <= a.nx - 2) {
      const float sdx = __fadd_rn(__fmul_rn(__fsub_rn(P.sxy[c + 1], P.sxy[c]), oh),
                                  __fmul_rn(__fsub_rn(Q.sxy[c + 1], Q.sxy[c]), oh));
      const float sdy = __fadd_rn(__fmul_rn(__fsub_rn(P.syy[c + px], P.syy[c]), oh),
                                  __fmul_rn(__fsub_rn(Q.syy[c + px], Q.syy[c]), oh));
      vy1 = relax(vy1, __ldg(a.ax.ah + i), __ldg(a.ax.bh + i), __fmul_rn(sdx, orho));
      vy2 = relax(vy2, __ldg(a.ay.ah + j), __ldg(a.ay.bh + j), __fmul_rn(sdy, orho));
    }
    if (i == a.isrc && j == a.jsrc) {  // the x parts take the source (PML:449-451)
      vx1 = __fadd_rn(vx1, a.src_fx[it - 1]);
      vy1 = __fadd_rn(vy1, a.src_fy[it - 1]);
    }
    if (i == 0 || i == a.nx - 1 || j == 0 || j == a.ny - 1) { vx1 = vx2 = vy1 = vy2 = 0.f; }  // PML:453-478
    P.vx[c] = vx1; Q.vx[c] = vx2; P.vy[c] = vy1; Q.vy[c] = vy2;
    const float vx = __fadd_rn(vx1, vx2), vy = __fadd_rn(vy1, vy2);
    const float v2 = vx * vx + vy * vy;
    vm2 = v2;
    bad = not_finite(v2);
    const int n0 = a.npml;
    if (i >= n0 && i < a.nx - n0 && j >= n0 && j < a.ny - n0) {   // PML:486-515
      const float sxx = __fadd_rn(P.sxx[c], Q.sxx[c]), syy = __fadd_rn(P.syy[c], Q.syy[c]);
      const float sxy = __fadd_rn(P.sxy[c], Q.sxy[c]);
      ek = a.half_rho * v2;
      const float exx = a.e_c1 * sxx - a.e_c2 * syy;
      const float eyy = a.e_c1 * syy - a.e_c2 * sxx;
      ep = 0.5f * (exx * sxx + eyy * syy) + a.inv_2mu * (sxy * sxy);
    }
  }
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  block_partials<E2X * E2Y>(DF{ek, 0.f}, DF{ep, 0.f}, vm2, bad, a.partials + ((size_t)ls * a.nblocks + blin) * 4);
}

void launch_step2d_order4(const StepArgs& s, int ls, bool het, cudaStream_t st) {
  const dim3 g((s.nx + E2X - 1) / E2X, (s.ny + E2Y - 1) / E2Y), b(E2X, E2Y);
  if (het) {
    stress2d4<true><<<g, b, 0, st>>>(s, ls);
    velocity2d4<true><<<g, b, 0, st>>>(s, ls);
  } else {
    stress2d4<false><<<g, b, 0, st>>>(s, ls);
    velocity2d4<false><<<g, b, 0, st>>>(s, ls);
  }
}

void launch_step2d_split(const StepArgs& s, int ls, cudaStream_t st) {
  const dim3 g((s.nx + E2X - 1) / E2X, (s.ny + E2Y - 1) / E2Y), b(E2X, E2Y);
  stress_split<<<g, b, 0, st>>>(s, ls);
  velocity_split<<<g, b, 0, st>>>(s, ls);
}

}  // namespace cpml
