// kernels2d.cu -- 2D P-SV velocity-stress C-PML time step, two-sweep form.
//
// One time step of seismic_CPML_2D_isotropic_second_order.f90 (2D:556-713):
//   stress2d   -- sigma_xx/sigma_yy (2D:556-580) and sigma_xy (2D:582-600)
//                 with their C-PML memory variables, plus the receivers of
//                 the previous step (2D:683-686).
//   velocity2d -- v_x (2D:606-621), v_y (2D:623-641), source (2D:644-667),
//                 rigid edges (2D:670-680), energy partials (2D:694-713) and
//                 max|v|^2 (2D:718).
// HET selects per-cell lambda/mu/rho with the reference's staggered averages
// (2D:559-562, 586, 627); otherwise the homogeneous constants of 2D:468-474.
#include "cpml_internal.cuh"
#include "kutil.cuh"

namespace cpml {

constexpr int T2X = 32, T2Y = 8;

__device__ __forceinline__ void record_receivers2d(const StepArgs& s, int it, long long gtid,
                                                   long long gsize) {
  const size_t slab = (size_t)s.nrec * s.nstep;
  for (long long r = gtid; r < s.nrec; r += gsize) {
    const long long c = s.rec_cell[r];
    const size_t o = (size_t)r * s.nstep + (size_t)(it - 1);
    s.seis[o] = s.f.vx[c];
    s.seis[slab + o] = s.f.vy[c];
  }
}

template <bool HET>
__global__ void __launch_bounds__(T2X* T2Y) stress2d(StepArgs s, int ls) {
  const Fields F = s.f;
  const int tid = threadIdx.x + threadIdx.y * T2X;
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  if (ls > 0)
    record_receivers2d(s, *s.it_base + ls, blin * (T2X * T2Y) + tid,
                       (long long)gridDim.x * gridDim.y * (T2X * T2Y));
  const int i = blockIdx.x * T2X + threadIdx.x;
  const int j = blockIdx.y * T2Y + threadIdx.y;
  if (i >= s.nx || j >= s.ny) return;
  const int sx = s.ax.slab(i), sy = s.ay.slab(j);
  const long long px = s.px;
  const long long c = (long long)j * px + i;
  const long long mx = (long long)j * s.ax.width() + sx;
  const long long my = (long long)sy * px + i;
  const float vxc = F.vx[c], vyc = F.vy[c];
  // sigma_xx, sigma_yy: j = 2..NY, i = 1..NX-1
  if (j >= 1 && i <= s.nx - 2) {
    float d1 = (F.vx[c + 1] - vxc) * s.odx;
    float d2 = (vyc - F.vy[c - px]) * s.ody;
    d1 = pml(d1, sx, s.m.x[0], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml(d2, sy, s.m.y[1], my, s.ay.a, s.ay.b, s.ay.ik, j);
    float dl = s.dt_lam, dl2m = s.dt_l2m;
    if (HET) {
      const float lh = 0.5f * (s.mdl.lam[c + 1] + s.mdl.lam[c]);
      const float mh = 0.5f * (s.mdl.mu[c + 1] + s.mdl.mu[c]);
      dl = s.dt * lh;
      dl2m = s.dt * (lh + 2.0f * mh);
    }
    F.sxx[c] = F.sxx[c] + (dl2m * d1 + dl * d2);
    F.syy[c] = F.syy[c] + (dl * d1 + dl2m * d2);
  }
  // sigma_xy: j = 1..NY-1, i = 2..NX
  if (j <= s.ny - 2 && i >= 1) {
    float d1 = (vyc - F.vy[c - 1]) * s.odx;
    float d2 = (F.vx[c + px] - vxc) * s.ody;
    d1 = pml(d1, sx, s.m.x[1], mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml(d2, sy, s.m.y[0], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
    const float dm = HET ? s.dt * (0.5f * (s.mdl.mu[c + px] + s.mdl.mu[c])) : s.dt_mu;
    F.sxy[c] = F.sxy[c] + dm * (d1 + d2);
  }
}

template <bool HET>
__global__ void __launch_bounds__(T2X* T2Y) velocity2d(StepArgs s, int ls) {
  const Fields F = s.f;
  const int it = *s.it_base + ls + 1;
  const int i = blockIdx.x * T2X + threadIdx.x;
  const int j = blockIdx.y * T2Y + threadIdx.y;
  float ek = 0.f, ep = 0.f, vm2 = 0.f;
  int bad = 0;
  if (i < s.nx && j < s.ny) {
    const int sx = s.ax.slab(i), sy = s.ay.slab(j);
    const long long px = s.px;
    const long long c = (long long)j * px + i;
    const long long mx = (long long)j * s.ax.width() + sx;
    const long long my = (long long)sy * px + i;
    float vx = F.vx[c], vy = F.vy[c];
    const float sxx = F.sxx[c], syy = F.syy[c], sxy = F.sxy[c];
    // v_x: j = 2..NY, i = 2..NX
    if (j >= 1 && i >= 1) {
      float d1 = (sxx - F.sxx[c - 1]) * s.odx;
      float d2 = (sxy - F.sxy[c - px]) * s.ody;
      d1 = pml(d1, sx, s.m.x[2], mx, s.ax.a, s.ax.b, s.ax.ik, i);
      d2 = pml(d2, sy, s.m.y[2], my, s.ay.a, s.ay.b, s.ay.ik, j);
      const float f = HET ? s.dt / s.mdl.rho[c] : s.dt_over_rho;
      vx = vx + (d1 + d2) * f;
    }
    // v_y: j = 1..NY-1, i = 1..NX-1
    if (j <= s.ny - 2 && i <= s.nx - 2) {
      float d1 = (F.sxy[c + 1] - sxy) * s.odx;
      float d2 = (F.syy[c + px] - syy) * s.ody;
      d1 = pml(d1, sx, s.m.x[3], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
      d2 = pml(d2, sy, s.m.y[3], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
      float f = s.dt_over_rho;
      if (HET) {
        const float* r = s.mdl.rho;
        f = s.dt / (0.25f * (r[c] + r[c + 1] + r[c + 1 + px] + r[c + px]));
      }
      vy = vy + (d1 + d2) * f;
    }
    if (i == s.isrc && j == s.jsrc) {  // 2D:664-667
      vx += s.src_fx[it - 1];
      vy += s.src_fy[it - 1];
    }
    if (i == 0 || i == s.nx - 1 || j == 0 || j == s.ny - 1) { vx = 0.f; vy = 0.f; }  // 2D:670-680
    F.vx[c] = vx;
    F.vy[c] = vy;
    const float v2 = vx * vx + vy * vy;
    vm2 = v2;
    bad = not_finite(v2);
    const int n0 = s.npml;
    if (i >= n0 && i < s.nx - n0 && j >= n0 && j < s.ny - n0) {
      float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
      if (HET) {
        const float l = s.mdl.lam[c], m = s.mdl.mu[c];
        const float den = 1.0f / (4.0f * m * (l + m));
        hr = 0.5f * s.mdl.rho[c];
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
  block_partials<T2X * T2Y>((double)ek, (double)ep, vm2, bad,
                            s.partials + ((size_t)ls * s.nblocks + blin) * 4);
}

dim3 grid2d(const StepArgs& s) { return dim3((s.nx + T2X - 1) / T2X, (s.ny + T2Y - 1) / T2Y); }

int blocks2d(const StepArgs& s) {
  dim3 g = grid2d(s);
  return (int)(g.x * g.y);
}

void launch_step2d_two_sweep(const StepArgs& s, int ls, bool het, cudaStream_t st) {
  const dim3 g = grid2d(s), b(T2X, T2Y);
  if (het) {
    stress2d<true><<<g, b, 0, st>>>(s, ls);
    velocity2d<true><<<g, b, 0, st>>>(s, ls);
  } else {
    stress2d<false><<<g, b, 0, st>>>(s, ls);
    velocity2d<false><<<g, b, 0, st>>>(s, ls);
  }
}

}  // namespace cpml
