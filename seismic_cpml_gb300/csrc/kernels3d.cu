// kernels3d.cu -- 3D velocity-stress C-PML time step, two-sweep form.
//
// One time step of seismic_CPML_3D_isotropic_MPI_OpenMP.f90 (3D:825-1180) as
// two kernels on the whole single-GPU domain:
//   stress3d    -- sigma_xx/yy/zz (3D:836-863), sigma_xy (3D:877-894),
//                  sigma_xz (3D:908-925), sigma_yz (3D:927-942), with their
//                  C-PML memory variables; also records the receivers of the
//                  previous step (3D:1124-1129), whose velocities are final.
//   velocity3d  -- v_x, v_y (3D:976-1017), v_z (3D:1031-1052) with memory
//                  variables, then the source (3D:1055-1083), the Dirichlet
//                  faces (3D:1087-1121), the energy partials (3D:1131-1180)
//                  and max|v|^2 (3D:1185), written per block for a
//                  deterministic FP64 reduction.
// Index ranges are the reference's global ranges for one domain: the MPI
// halo exchange (3D:811-823, 951-963) only moves planes so that every slab
// sees its neighbours, and k2begin/kminus1end (3D:792-796) trim the global
// first/last plane.
//
// Block = 32 x 8 threads over (i, j), each thread sweeping KC planes in k:
// rows are coalesced 128-byte lines; x/y neighbours come through L1, z
// neighbours are the previous plane's loads in L1/L2.
#include "cpml_internal.cuh"
#include "kutil.cuh"

namespace cpml {

constexpr int T3X = 32, T3Y = 8, T3K = 8;

__device__ __forceinline__ void record_receivers(const StepArgs& s, const float* __restrict__ vx,
                                                 const float* __restrict__ vy,
                                                 const float* __restrict__ vz, int it,
                                                 long long gtid, long long gsize) {
  const size_t slab = (size_t)s.nrec * s.nstep;
  for (long long r = gtid; r < s.nrec; r += gsize) {
    const long long c = s.rec_cell[r];
    const size_t o = (size_t)r * s.nstep + (size_t)(it - 1);
    s.seis[o] = vx[c];
    s.seis[slab + o] = vy[c];
    if (vz) s.seis[2 * slab + o] = vz[c];
  }
}

template <bool HET>
__global__ void __launch_bounds__(T3X* T3Y) stress3d(StepArgs s, int ls) {
  const Fields F = s.f;
  const int tid = threadIdx.x + threadIdx.y * T3X;
  const long long blin = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
  if (ls > 0)  // receivers of the step that just ended (1-based base + ls)
    record_receivers(s, F.vx, F.vy, F.vz, *s.it_base + ls, blin * (T3X * T3Y) + tid,
                     (long long)gridDim.x * gridDim.y * gridDim.z * (T3X * T3Y));
  const int i = blockIdx.x * T3X + threadIdx.x;
  const int j = blockIdx.y * T3Y + threadIdx.y;
  if (i >= s.nx || j >= s.ny) return;
  const int k0 = blockIdx.z * T3K;
  const int k1 = min(k0 + T3K, s.nz);
  const int sx = s.ax.slab(i), sy = s.ay.slab(j);
  const int wx = s.ax.width(), wy = s.ay.width();
  const long long px = s.px, pl = s.plane;
  for (int k = k0; k < k1; ++k) {
    const long long c = cell3(s, i, j, k);
    const int sz = s.az.slab(k);
    const long long mx = ((long long)k * s.ny + j) * wx + sx;
    const long long my = ((long long)k * wy + sy) * px + i;
    const long long mz = ((long long)sz * s.ny + j) * px + i;
    const float vxc = F.vx[c], vyc = F.vy[c], vzc = F.vz[c];
    // sigma_xx, sigma_yy, sigma_zz: k = 2..NZ, j = 2..NY, i = 1..NX-1
    if (k >= 1 && j >= 1 && i <= s.nx - 2) {
      float dxx = (F.vx[c + 1] - vxc) * s.odx;
      float dyy = (vyc - F.vy[c - px]) * s.ody;
      float dzz = (vzc - F.vz[c - pl]) * s.odz;
      dxx = pml(dxx, sx, s.m.x[0], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
      dyy = pml(dyy, sy, s.m.y[1], my, s.ay.a, s.ay.b, s.ay.ik, j);
      dzz = pml(dzz, sz, s.m.z[2], mz, s.az.a, s.az.b, s.az.ik, k);
      float dl = s.dt_lam, dl2m = s.dt_l2m;
      if (HET) {
        const float lh = 0.5f * (s.mdl.lam[c + 1] + s.mdl.lam[c]);
        const float mh = 0.5f * (s.mdl.mu[c + 1] + s.mdl.mu[c]);
        dl = s.dt * lh;
        dl2m = s.dt * (lh + 2.0f * mh);
      }
      F.sxx[c] = F.sxx[c] + (dl2m * dxx + dl * (dyy + dzz));
      F.syy[c] = F.syy[c] + (dl * (dxx + dzz) + dl2m * dyy);
      F.szz[c] = F.szz[c] + (dl * (dxx + dyy) + dl2m * dzz);
    }
    // sigma_xy: k = 1..NZ, j = 1..NY-1, i = 2..NX
    if (j <= s.ny - 2 && i >= 1) {
      float d1 = (vyc - F.vy[c - 1]) * s.odx;
      float d2 = (F.vx[c + px] - vxc) * s.ody;
      d1 = pml(d1, sx, s.m.x[1], mx, s.ax.a, s.ax.b, s.ax.ik, i);
      d2 = pml(d2, sy, s.m.y[0], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
      const float dm = HET ? s.dt * (0.5f * (s.mdl.mu[c + px] + s.mdl.mu[c])) : s.dt_mu;
      F.sxy[c] = F.sxy[c] + dm * (d1 + d2);
    }
    if (k <= s.nz - 2) {
      // sigma_xz: k = 1..NZ-1, j = 1..NY, i = 2..NX
      if (i >= 1) {
        float d1 = (vzc - F.vz[c - 1]) * s.odx;
        float d2 = (F.vx[c + pl] - vxc) * s.odz;
        d1 = pml(d1, sx, s.m.x[2], mx, s.ax.a, s.ax.b, s.ax.ik, i);
        d2 = pml(d2, sz, s.m.z[0], mz, s.az.ah, s.az.bh, s.az.ikh, k);
        const float dm = HET ? s.dt * (0.5f * (s.mdl.mu[c + pl] + s.mdl.mu[c])) : s.dt_mu;
        F.sxz[c] = F.sxz[c] + dm * (d1 + d2);
      }
      // sigma_yz: k = 1..NZ-1, j = 1..NY-1, i = 1..NX
      if (j <= s.ny - 2) {
        float d1 = (F.vz[c + px] - vzc) * s.ody;
        float d2 = (F.vy[c + pl] - vyc) * s.odz;
        d1 = pml(d1, sy, s.m.y[2], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
        d2 = pml(d2, sz, s.m.z[1], mz, s.az.ah, s.az.bh, s.az.ikh, k);
        float dm = s.dt_mu;
        if (HET) {  // 8-point average at (i+1/2, j+1/2, k+1/2); i+1 clamped on the last column
          const float* mu = s.mdl.mu;
          const long long di = (i < s.nx - 1) ? 1 : 0;
          const float sm = ((((((mu[c] + mu[c + di]) + mu[c + px]) + mu[c + px + di]) + mu[c + pl]) +
                             mu[c + pl + di]) + mu[c + pl + px]) + mu[c + pl + px + di];
          dm = s.dt * (0.125f * sm);
        }
        F.syz[c] = F.syz[c] + dm * (d1 + d2);
      }
    }
  }
}

template <bool HET>
__global__ void __launch_bounds__(T3X* T3Y) velocity3d(StepArgs s, int ls) {
  const Fields F = s.f;
  const int it = *s.it_base + ls + 1;  // 1-based current step
  const int i = blockIdx.x * T3X + threadIdx.x;
  const int j = blockIdx.y * T3Y + threadIdx.y;
  const bool valid = i < s.nx && j < s.ny;
  const int k0 = blockIdx.z * T3K;
  const int k1 = min(k0 + T3K, s.nz);
  Kahan ek, ep;
  float vm2 = 0.f;
  int bad = 0;
  if (valid) {
    const int sx = s.ax.slab(i), sy = s.ay.slab(j);
    const int wx = s.ax.width(), wy = s.ay.width();
    const long long px = s.px, pl = s.plane;
    const int n0 = s.npml;
    const bool in_ij = i >= n0 && i < s.nx - n0 && j >= n0 && j < s.ny - n0;
    for (int k = k0; k < k1; ++k) {
      const long long c = cell3(s, i, j, k);
      const int sz = s.az.slab(k);
      const long long mx = ((long long)k * s.ny + j) * wx + sx;
      const long long my = ((long long)k * wy + sy) * px + i;
      const long long mz = ((long long)sz * s.ny + j) * px + i;
      float vx = F.vx[c], vy = F.vy[c], vz = F.vz[c];
      const float sxx = F.sxx[c], syy = F.syy[c], szz = F.szz[c];
      const float sxy = F.sxy[c], sxz = F.sxz[c], syz = F.syz[c];
      // v_x: k = 2..NZ, j = 2..NY, i = 2..NX
      if (k >= 1 && j >= 1 && i >= 1) {
        float d1 = (sxx - F.sxx[c - 1]) * s.odx;
        float d2 = (sxy - F.sxy[c - px]) * s.ody;
        float d3 = (sxz - F.sxz[c - pl]) * s.odz;
        d1 = pml(d1, sx, s.m.x[3], mx, s.ax.a, s.ax.b, s.ax.ik, i);
        d2 = pml(d2, sy, s.m.y[3], my, s.ay.a, s.ay.b, s.ay.ik, j);
        d3 = pml(d3, sz, s.m.z[3], mz, s.az.a, s.az.b, s.az.ik, k);
        const float f = HET ? s.dt / s.mdl.rho[c] : s.dt_over_rho;
        vx = vx + f * (d1 + d2 + d3);
      }
      // v_y: k = 2..NZ, j = 1..NY-1, i = 1..NX-1
      if (k >= 1 && j <= s.ny - 2 && i <= s.nx - 2) {
        float d1 = (F.sxy[c + 1] - sxy) * s.odx;
        float d2 = (F.syy[c + px] - syy) * s.ody;
        float d3 = (syz - F.syz[c - pl]) * s.odz;
        d1 = pml(d1, sx, s.m.x[4], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
        d2 = pml(d2, sy, s.m.y[4], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
        d3 = pml(d3, sz, s.m.z[4], mz, s.az.a, s.az.b, s.az.ik, k);
        float f = s.dt_over_rho;
        if (HET) {
          const float* r = s.mdl.rho;
          f = s.dt / (0.25f * (r[c] + r[c + 1] + r[c + 1 + px] + r[c + px]));
        }
        vy = vy + f * (d1 + d2 + d3);
      }
      // v_z: k = 1..NZ-1, j = 2..NY, i = 1..NX-1
      if (k <= s.nz - 2 && j >= 1 && i <= s.nx - 2) {
        float d1 = (F.sxz[c + 1] - sxz) * s.odx;
        float d2 = (syz - F.syz[c - px]) * s.ody;
        float d3 = (F.szz[c + pl] - szz) * s.odz;
        d1 = pml(d1, sx, s.m.x[5], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
        d2 = pml(d2, sy, s.m.y[5], my, s.ay.a, s.ay.b, s.ay.ik, j);
        d3 = pml(d3, sz, s.m.z[5], mz, s.az.ah, s.az.bh, s.az.ikh, k);
        float f = s.dt_over_rho;
        if (HET) {
          const float* r = s.mdl.rho;
          f = s.dt / (0.25f * (r[c] + r[c + 1] + r[c + 1 + pl] + r[c + pl]));
        }
        vz = vz + f * (d1 + d2 + d3);
      }
      if (i == s.isrc && j == s.jsrc && k == s.ksrc) {  // 3D:1080-1081
        vx += s.src_fx[it - 1];
        vy += s.src_fy[it - 1];
      }
      if (i == 0 || i == s.nx - 1 || j == 0 || j == s.ny - 1 || k == 0 || k == s.nz - 1) {
        vx = 0.f; vy = 0.f; vz = 0.f;  // rigid faces (3D:1087-1121)
      }
      F.vx[c] = vx; F.vy[c] = vy; F.vz[c] = vz;
      const float v2 = vx * vx + vy * vy + vz * vz;
      vm2 = fmaxf(vm2, v2);
      bad |= not_finite(v2);
      if (in_ij && k >= n0 && k < s.nz - n0) {  // energy interior (3D:1136-1143)
        float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
        if (HET) {
          const float l = s.mdl.lam[c], m = s.mdl.mu[c];
          const float den = 1.0f / (2.0f * m * (3.0f * l + 2.0f * m));
          hr = 0.5f * s.mdl.rho[c];
          c1 = 2.0f * (l + m) * den;
          c2 = l * den;
          i2m = 1.0f / (2.0f * m);
        }
        ek.add(hr * v2);
        const float exx = c1 * sxx - c2 * (syy + szz);
        const float eyy = c1 * syy - c2 * (sxx + szz);
        float third;
        if (s.ep_physical) {
          third = (c1 * szz - c2 * (sxx + syy)) * szz;
        } else {
          third = eyy * syy;  // the reference adds eps_yy*sigma_yy twice (3D:1170-1171)
        }
        ep.add(0.5f * (exx * sxx + eyy * syy + third) +
               i2m * (sxy * sxy + sxz * sxz + syz * syz));
      }
    }
  }
  const long long blin = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
  block_partials<T3X * T3Y>(ek.df(), ep.df(), vm2, bad,
                            s.partials + ((size_t)ls * s.nblocks + blin) * 4);
}

dim3 grid3d(const StepArgs& s) {
  return dim3((s.nx + T3X - 1) / T3X, (s.ny + T3Y - 1) / T3Y, (s.nz + T3K - 1) / T3K);
}

int blocks3d(const StepArgs& s) {
  dim3 g = grid3d(s);
  return (int)(g.x * g.y * g.z);
}

void launch_step3d_two_sweep(const StepArgs& s, int ls, bool het, cudaStream_t st) {
  const dim3 g = grid3d(s), b(T3X, T3Y);
  if (het) {
    stress3d<true><<<g, b, 0, st>>>(s, ls);
    velocity3d<true><<<g, b, 0, st>>>(s, ls);
  } else {
    stress3d<false><<<g, b, 0, st>>>(s, ls);
    velocity3d<false><<<g, b, 0, st>>>(s, ls);
  }
}

}  // namespace cpml
