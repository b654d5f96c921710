// fused3d.cu -- one-sweep 3D velocity-stress C-PML time step for sm_103a.
//
// One launch advances every field one full time step of
// seismic_CPML_3D_isotropic_MPI_OpenMP.f90 (stress 3D:836-943, velocity
// 3D:976-1052, source 3D:1055-1083, rigid faces 3D:1087-1121, energy
// 3D:1131-1180), reading time level n from buffer set A and writing time
// level n+1 to buffer set B. With separate read and write sets no CTA can
// see another CTA's half-updated cells, so the sweep needs no grid-wide
// synchronisation and every field crosses HBM exactly once per step
// (9 reads + 9 writes = 72 B/cell, the compulsory minimum).
//
// CTA work: a 32 x TY tile of (i, j) columns over a chunk [kb, ke) of planes.
// The CTA streams planes in z (2.5D): at iteration m it
//   1. waits for load group g(m): TMA boxes of v_x(m+1), v_y(m+1), v_z(m)
//      and the six old stresses at plane m, each a (32+8) x (TY+2) box with
//      a one-cell halo in y and an x window rounded out to 16-byte TMA
//      alignment (x starts at i0-4);
//   2. computes the new stresses at plane m on the tile plus the halo cells
//      the velocity update reads (left column: sigma_xx, top row: sigma_yy,
//      right column: sigma_xy/sigma_xz, bottom row: sigma_xy/sigma_yz) into a
//      shared-memory ring of planes, storing only its own cells to B;
//   3. computes the new velocities one plane behind (plane m-1), which needs
//      new stresses at planes m-2..m, all in the ring, then source, rigid
//      faces, receivers-free store to B and the energy partials;
//   4. issues load group g(m+2) into the slots freed by this iteration.
// Old velocities live in a 4-slot (v_x, v_y) / 3-slot (v_z) ring, old
// stresses in 2 slots, so each TMA box is loaded two iterations ahead.
// Stress-side C-PML memory variables are ping-ponged like the fields (halo
// cells read time-n values that the owner is overwriting); velocity-side
// ones are updated in place (only the owner touches them).
//
// Waits on the TMA barriers are bounded (clock64); on timeout the CTA sets
// the device error word, drains its outstanding copies with a second bounded
// wait and leaves the sweep. The host reports CPML_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>
#include "cpml_internal.cuh"
#include "kutil.cuh"

namespace cpml {

struct TmapSet {
  CUtensorMap f[9];    // vx vy vz sxx syy szz sxy sxz syz of the read set
  CUtensorMap lam, mu, rho;
};

constexpr int FTX = 32;            // tile width in i (one warp)
constexpr int FNT = 256;           // threads per CTA: 32 x 8
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kWaitCycles) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ int mod3(int m) { return (m + 6) % 3; }

// Memory-variable update with ping-pong: reads the time-n value from mA,
// writes time n+1 to mB when this CTA owns the cell. `upd` false leaves the
// variable unchanged (cells outside the reference's loop range).
__device__ __forceinline__ float pml_pp(float d, bool upd, bool own, int sidx,
                                        const float* __restrict__ mA, float* __restrict__ mB,
                                        long long midx, const float* __restrict__ a,
                                        const float* __restrict__ b, const float* __restrict__ ik,
                                        int idx) {
  if (sidx < 0) return d;
  const float old = mA[midx];
  const float m = upd ? __ldg(b + idx) * old + __ldg(a + idx) * d : old;
  if (own) mB[midx] = m;
  return d * __ldg(ik + idx) + m;
}

template <int TY, bool HET>
struct Geo {
  static constexpr int BX = FTX + 8;                 // TMA box width (x from i0-4)
  static constexpr int BY = TY + 2;                  // box height (y from j0-1)
  static constexpr int BOX = BX * BY;                // floats per box
  static constexpr int SLOT = (BOX * 4 + 127) / 128 * 32;  // slot stride, 128-byte aligned
  static constexpr int RX = FTX + 2, RY = TY + 2, REG = RX * RY;  // stress ring plane
  static constexpr int NBOX = 4 + 4 + 3 + 12 + (HET ? 8 : 0);
  static constexpr int RING = 14 * REG;
  static constexpr size_t SMEM = (size_t)NBOX * SLOT * 4 + (size_t)RING * 4 + 64;
  static constexpr int NH = 2 * FTX + 2 * TY;        // halo stress cells
};

template <int TY, bool HET>
__global__ void __launch_bounds__(FNT, 2)
    fused3d_kernel(const __grid_constant__ TmapSet tm, StepArgs s, int ls, int Lz) {
  using G = Geo<TY, HET>;
  constexpr int BX = G::BX, SLOT = G::SLOT, RX = G::RX, REG = G::REG;
  extern __shared__ __align__(128) float sm[];
  float* vxs = sm;                       // [4] slots
  float* vys = vxs + 4 * SLOT;           // [4]
  float* vzs = vys + 4 * SLOT;           // [3]
  float* sos = vzs + 3 * SLOT;           // [2][6]
  float* lms = sos + 12 * SLOT;          // HET: lam[2], mu[3], rho[3]
  float* mus = lms + 2 * SLOT;
  float* rhs = mus + 3 * SLOT;
  float* ring = sm + G::NBOX * SLOT;
  float* r_sxx = ring;                   // [2]
  float* r_syy = r_sxx + 2 * REG;        // [2]
  float* r_sxy = r_syy + 2 * REG;        // [2]
  float* r_szz = r_sxy + 2 * REG;        // [2]
  float* r_sxz = r_szz + 2 * REG;        // [3]
  float* r_syz = r_sxz + 3 * REG;        // [3]
  uint64_t* bar = reinterpret_cast<uint64_t*>(r_syz + 3 * REG);

  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int nty = (s.ny + TY - 1) / TY;
  const int i0 = blockIdx.x * FTX;
  const int j0 = (blockIdx.y % nty) * TY;
  const int kb = (blockIdx.y / nty) * Lz;
  const int ke = min(kb + Lz, s.nz);
  const int kk0 = kb - 1;
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  const int it = *s.it_base + ls + 1;

  // receivers of the step that just ended, from the read set
  if (ls > 0) {
    const size_t slab = (size_t)s.nrec * s.nstep;
    for (long long r = blin * FNT + tid; r < s.nrec; r += (long long)gridDim.x * gridDim.y * FNT) {
      const long long c = s.rec_cell[r];
      const size_t o = (size_t)r * s.nstep + (size_t)(it - 2);
      s.seis[o] = s.f.vx[c];
      s.seis[slab + o] = s.f.vy[c];
      s.seis[2 * slab + o] = s.f.vz[c];
    }
  }

  constexpr uint32_t kBoxBytes = (uint32_t)G::BOX * 4;
  auto issue_group = [&](int m, uint64_t* b, bool prologue) {
    // g(m): vx(m+1), vy(m+1), vz(m), six old stresses at m (+ lam(m), mu(m+1), rho(m))
    const int x = i0 - 4, y = j0 - 1;
    uint32_t nb = 9 + (HET ? 3 : 0) + (prologue ? (3 + (HET ? 1 : 0)) : 0);
    mbar_expect_tx(b, nb * kBoxBytes);
    tma_load_3d(vxs + ((m + 1) & 3) * SLOT, &tm.f[0], x, y, m + 1, b);
    tma_load_3d(vys + ((m + 1) & 3) * SLOT, &tm.f[1], x, y, m + 1, b);
    tma_load_3d(vzs + mod3(m) * SLOT, &tm.f[2], x, y, m, b);
#pragma unroll
    for (int c = 0; c < 6; ++c) tma_load_3d(sos + ((m & 1) * 6 + c) * SLOT, &tm.f[3 + c], x, y, m, b);
    if (HET) {
      tma_load_3d(lms + (m & 1) * SLOT, &tm.lam, x, y, m, b);
      tma_load_3d(mus + mod3(m + 1) * SLOT, &tm.mu, x, y, m + 1, b);
      tma_load_3d(rhs + mod3(m) * SLOT, &tm.rho, x, y, m, b);
    }
    if (prologue) {
      tma_load_3d(vxs + (m & 3) * SLOT, &tm.f[0], x, y, m, b);
      tma_load_3d(vys + (m & 3) * SLOT, &tm.f[1], x, y, m, b);
      tma_load_3d(vzs + mod3(m - 1) * SLOT, &tm.f[2], x, y, m - 1, b);
      if (HET) tma_load_3d(mus + mod3(m) * SLOT, &tm.mu, x, y, m, b);
    }
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    issue_group(kk0, &bar[0], true);
    if (kk0 + 1 <= ke) issue_group(kk0 + 1, &bar[1], false);
  }

  const int wx = s.ax.width(), wy = s.ay.width();
  const long long px = s.px, pl = s.plane;
  Kahan ek, ep;
  float vm2 = 0.f;
  int bad = 0;
  bool ok_all = true;

  // Stress at cell (i, j) of plane m. comps: 1 normal, 2 xy, 4 xz, 8 yz.
  // bxi/byj: box coordinates of the cell; rxi/ryj: ring coordinates.
  auto stress_cell = [&](int i, int j, int m, int comps, bool own) {
    const int bxi = i - i0 + 4, byj = j - j0 + 1;
    const int ridx = (j - j0 + 1) * RX + (i - i0 + 1);
    const bool inside = i >= 0 && i < s.nx && j >= 0 && j < s.ny && m >= 0 && m < s.nz;
    if (!inside) return;
    const float* VX0 = vxs + (m & 3) * SLOT;
    const float* VX1 = vxs + ((m + 1) & 3) * SLOT;
    const float* VY0 = vys + (m & 3) * SLOT;
    const float* VY1 = vys + ((m + 1) & 3) * SLOT;
    const float* VZ0 = vzs + mod3(m) * SLOT;
    const float* VZm = vzs + mod3(m - 1) * SLOT;
    const float* SO = sos + (m & 1) * 6 * SLOT;
    const int b0 = byj * BX + bxi;
    const float vxc = VX0[b0], vyc = VY0[b0], vzc = VZ0[b0];
    const int sx = s.ax.slab(i), sy = s.ay.slab(j), sz = s.az.slab(m);
    const long long mx = ((long long)m * s.ny + j) * wx + sx;
    const long long my = ((long long)m * wy + sy) * px + i;
    const long long mz = ((long long)sz * s.ny + j) * px + i;
    const bool st = own && m >= kb && m < ke;  // this CTA stores the cell
    const long long c = (long long)m * pl + (long long)j * px + i;
    if (comps & 1) {
      const bool upd = m >= 1 && j >= 1 && i <= s.nx - 2;
      float dxx = (VX0[b0 + 1] - vxc) * s.odx;
      float dyy = (vyc - VY0[b0 - BX]) * s.ody;
      float dzz = (vzc - VZm[b0]) * s.odz;
      dxx = pml_pp(dxx, upd, st, sx, s.m.x[0], s.mb.x[0], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
      dyy = pml_pp(dyy, upd, st, sy, s.m.y[1], s.mb.y[1], my, s.ay.a, s.ay.b, s.ay.ik, j);
      dzz = pml_pp(dzz, upd, st, sz, s.m.z[2], s.mb.z[2], mz, s.az.a, s.az.b, s.az.ik, m);
      float dl = s.dt_lam, dl2m = s.dt_l2m;
      if (HET) {
        const float* L = lms + (m & 1) * SLOT;
        const float* M = mus + mod3(m) * SLOT;
        const float lh = 0.5f * (L[b0 + 1] + L[b0]);
        const float mh = 0.5f * (M[b0 + 1] + M[b0]);
        dl = s.dt * lh;
        dl2m = s.dt * (lh + 2.0f * mh);
      }
      float nxx = SO[0 * SLOT + b0], nyy = SO[1 * SLOT + b0], nzz = SO[2 * SLOT + b0];
      if (upd) {
        nxx = nxx + (dl2m * dxx + dl * (dyy + dzz));
        nyy = nyy + (dl * (dxx + dzz) + dl2m * dyy);
        nzz = nzz + (dl * (dxx + dyy) + dl2m * dzz);
      }
      r_sxx[(m & 1) * REG + ridx] = nxx;
      r_syy[(m & 1) * REG + ridx] = nyy;
      r_szz[(m & 1) * REG + ridx] = nzz;
      if (st) { s.g.sxx[c] = nxx; s.g.syy[c] = nyy; s.g.szz[c] = nzz; }
    }
    if (comps & 2) {
      const bool upd = j <= s.ny - 2 && i >= 1;
      float d1 = (vyc - VY0[b0 - 1]) * s.odx;
      float d2 = (VX0[b0 + BX] - vxc) * s.ody;
      d1 = pml_pp(d1, upd, st, sx, s.m.x[1], s.mb.x[1], mx, s.ax.a, s.ax.b, s.ax.ik, i);
      d2 = pml_pp(d2, upd, st, sy, s.m.y[0], s.mb.y[0], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
      float dm = s.dt_mu;
      if (HET) {
        const float* M = mus + mod3(m) * SLOT;
        dm = s.dt * (0.5f * (M[b0 + BX] + M[b0]));
      }
      float n = SO[3 * SLOT + b0];
      if (upd) n = n + dm * (d1 + d2);
      r_sxy[(m & 1) * REG + ridx] = n;
      if (st) s.g.sxy[c] = n;
    }
    if (comps & 4) {
      const bool upd = m <= s.nz - 2 && i >= 1;
      float d1 = (vzc - VZ0[b0 - 1]) * s.odx;
      float d2 = (VX1[b0] - vxc) * s.odz;
      d1 = pml_pp(d1, upd, st, sx, s.m.x[2], s.mb.x[2], mx, s.ax.a, s.ax.b, s.ax.ik, i);
      d2 = pml_pp(d2, upd, st, sz, s.m.z[0], s.mb.z[0], mz, s.az.ah, s.az.bh, s.az.ikh, m);
      float dm = s.dt_mu;
      if (HET) {
        const float* M0 = mus + mod3(m) * SLOT;
        const float* M1 = mus + mod3(m + 1) * SLOT;
        dm = s.dt * (0.5f * (M1[b0] + M0[b0]));
      }
      float n = SO[4 * SLOT + b0];
      if (upd) n = n + dm * (d1 + d2);
      r_sxz[mod3(m) * REG + ridx] = n;
      if (st) s.g.sxz[c] = n;
    }
    if (comps & 8) {
      const bool upd = m <= s.nz - 2 && j <= s.ny - 2;
      float d1 = (VZ0[b0 + BX] - vzc) * s.ody;
      float d2 = (VY1[b0] - vyc) * s.odz;
      d1 = pml_pp(d1, upd, st, sy, s.m.y[2], s.mb.y[2], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
      d2 = pml_pp(d2, upd, st, sz, s.m.z[1], s.mb.z[1], mz, s.az.ah, s.az.bh, s.az.ikh, m);
      float dm = s.dt_mu;
      if (HET) {
        const float* M0 = mus + mod3(m) * SLOT;
        const float* M1 = mus + mod3(m + 1) * SLOT;
        const int di = (i < s.nx - 1) ? 1 : 0;
        const float sm8 = ((((((M0[b0] + M0[b0 + di]) + M0[b0 + BX]) + M0[b0 + BX + di]) + M1[b0]) +
                            M1[b0 + di]) + M1[b0 + BX]) + M1[b0 + BX + di];
        dm = s.dt * (0.125f * sm8);
      }
      float n = SO[5 * SLOT + b0];
      if (upd) n = n + dm * (d1 + d2);
      r_syz[mod3(m) * REG + ridx] = n;
      if (st) s.g.syz[c] = n;
    }
  };

  for (int m = kk0; m <= ke; ++m) {
    const int use = m - kk0;
    const bool ok = mbar_wait_bounded(&bar[use & 1], (uint32_t)((use >> 1) & 1));
    // ---- stress at plane m: own cells, then halo cells --------------------
#pragma unroll
    for (int q = 0; q < TY / 8; ++q) stress_cell(i0 + tx, j0 + ty + 8 * q, m, 15, true);
    if (tid < G::NH) {
      int i, j, comps;
      if (tid < FTX) { i = i0 + tid; j = j0 + TY; comps = 1; }                 // top row: sigma_yy
      else if (tid < 2 * FTX) { i = i0 + tid - FTX; j = j0 - 1; comps = 2 | 8; }  // bottom: xy, yz
      else if (tid < 2 * FTX + TY) { i = i0 - 1; j = j0 + tid - 2 * FTX; comps = 1; }  // left: sigma_xx
      else { i = i0 + FTX; j = j0 + tid - 2 * FTX - TY; comps = 2 | 4; }       // right: xy, xz
      stress_cell(i, j, m, comps, false);
    }
    if (!__syncthreads_and(ok ? 1 : 0)) { ok_all = false; break; }
    // ---- velocity at plane p = m - 1 --------------------------------------
    const int p = m - 1;
    if (p >= kb && p < ke) {
      const float* VXp = vxs + (p & 3) * SLOT;
      const float* VYp = vys + (p & 3) * SLOT;
      const float* VZp = vzs + mod3(p) * SLOT;
      const float* Sxx = r_sxx + (p & 1) * REG;
      const float* Syy = r_syy + (p & 1) * REG;
      const float* Sxy = r_sxy + (p & 1) * REG;
      const float* Szz0 = r_szz + (p & 1) * REG;
      const float* Szz1 = r_szz + ((p + 1) & 1) * REG;
      const float* Sxz0 = r_sxz + mod3(p) * REG;
      const float* Sxzm = r_sxz + mod3(p - 1) * REG;
      const float* Syz0 = r_syz + mod3(p) * REG;
      const float* Syzm = r_syz + mod3(p - 1) * REG;
      const int sz = s.az.slab(p);
#pragma unroll
      for (int q = 0; q < TY / 8; ++q) {
        const int i = i0 + tx, j = j0 + ty + 8 * q;
        if (i >= s.nx || j >= s.ny) continue;
        const int b0 = (j - j0 + 1) * BX + (i - i0 + 4);
        const int r0 = (j - j0 + 1) * RX + (i - i0 + 1);
        const int sx = s.ax.slab(i), sy = s.ay.slab(j);
        const long long mx = ((long long)p * s.ny + j) * wx + sx;
        const long long my = ((long long)p * wy + sy) * px + i;
        const long long mz = ((long long)sz * s.ny + j) * px + i;
        const long long c = (long long)p * pl + (long long)j * px + i;
        float vx = VXp[b0], vy = VYp[b0], vz = VZp[b0];
        const float sxx = Sxx[r0], syy = Syy[r0], szz = Szz0[r0];
        const float sxy = Sxy[r0], sxz = Sxz0[r0], syz = Syz0[r0];
        if (p >= 1 && j >= 1 && i >= 1) {  // v_x (3D:976-993)
          float d1 = (sxx - Sxx[r0 - 1]) * s.odx;
          float d2 = (sxy - Sxy[r0 - RX]) * s.ody;
          float d3 = (sxz - Sxzm[r0]) * s.odz;
          d1 = pml(d1, sx, s.m.x[3], mx, s.ax.a, s.ax.b, s.ax.ik, i);
          d2 = pml(d2, sy, s.m.y[3], my, s.ay.a, s.ay.b, s.ay.ik, j);
          d3 = pml(d3, sz, s.m.z[3], mz, s.az.a, s.az.b, s.az.ik, p);
          float f = s.dt_over_rho;
          if (HET) f = s.dt / (rhs + mod3(p) * SLOT)[b0];
          vx = vx + f * (d1 + d2 + d3);
        }
        if (p >= 1 && j <= s.ny - 2 && i <= s.nx - 2) {  // v_y (3D:995-1014)
          float d1 = (Sxy[r0 + 1] - sxy) * s.odx;
          float d2 = (Syy[r0 + RX] - syy) * s.ody;
          float d3 = (syz - Syzm[r0]) * s.odz;
          d1 = pml(d1, sx, s.m.x[4], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
          d2 = pml(d2, sy, s.m.y[4], my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
          d3 = pml(d3, sz, s.m.z[4], mz, s.az.a, s.az.b, s.az.ik, p);
          float f = s.dt_over_rho;
          if (HET) {
            const float* R = rhs + mod3(p) * SLOT;
            f = s.dt / (0.25f * (R[b0] + R[b0 + 1] + R[b0 + 1 + BX] + R[b0 + BX]));
          }
          vy = vy + f * (d1 + d2 + d3);
        }
        if (p <= s.nz - 2 && j >= 1 && i <= s.nx - 2) {  // v_z (3D:1031-1052)
          float d1 = (Sxz0[r0 + 1] - sxz) * s.odx;
          float d2 = (syz - Syz0[r0 - RX]) * s.ody;
          float d3 = (Szz1[r0] - szz) * s.odz;
          d1 = pml(d1, sx, s.m.x[5], mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
          d2 = pml(d2, sy, s.m.y[5], my, s.ay.a, s.ay.b, s.ay.ik, j);
          d3 = pml(d3, sz, s.m.z[5], mz, s.az.ah, s.az.bh, s.az.ikh, p);
          float f = s.dt_over_rho;
          if (HET) {
            const float* R0 = rhs + mod3(p) * SLOT;
            const float* R1 = rhs + mod3(p + 1) * SLOT;
            f = s.dt / (0.25f * (R0[b0] + R0[b0 + 1] + R1[b0 + 1] + R1[b0]));
          }
          vz = vz + f * (d1 + d2 + d3);
        }
        if (i == s.isrc && j == s.jsrc && p == s.ksrc) {
          vx += s.src_fx[it - 1];
          vy += s.src_fy[it - 1];
        }
        if (i == 0 || i == s.nx - 1 || j == 0 || j == s.ny - 1 || p == 0 || p == s.nz - 1) {
          vx = 0.f; vy = 0.f; vz = 0.f;
        }
        s.g.vx[c] = vx; s.g.vy[c] = vy; s.g.vz[c] = vz;
        const float v2 = vx * vx + vy * vy + vz * vz;
        vm2 = fmaxf(vm2, v2);
        bad |= not_finite(v2);
        const int n0 = s.npml;
        if (i >= n0 && i < s.nx - n0 && j >= n0 && j < s.ny - n0 && p >= n0 && p < s.nz - n0) {
          float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
          if (HET) {
            const float l = __ldg(s.mdl.lam + c), mu = __ldg(s.mdl.mu + c);
            const float den = 1.0f / (2.0f * mu * (3.0f * l + 2.0f * mu));
            hr = 0.5f * (rhs + mod3(p) * SLOT)[b0];
            c1 = 2.0f * (l + mu) * den;
            c2 = l * den;
            i2m = 1.0f / (2.0f * mu);
          }
          ek.add(hr * v2);
          const float exx = c1 * sxx - c2 * (syy + szz);
          const float eyy = c1 * syy - c2 * (sxx + szz);
          const float third = s.ep_physical ? (c1 * szz - c2 * (sxx + syy)) * szz : eyy * syy;
          ep.add(0.5f * (exx * sxx + eyy * syy + third) + i2m * (sxy * sxy + sxz * sxz + syz * syz));
        }
      }
    }
    __syncthreads();
    if (tid == 0 && m + 2 <= ke) issue_group(m + 2, &bar[use & 1], false);
  }
  if (!ok_all) {
    if (tid == 0) {
      atomicOr(s.err, 1);
      // drain copies that may still be in flight into this CTA's shared memory
      mbar_wait_bounded(&bar[0], 0);
      mbar_wait_bounded(&bar[0], 1);
      mbar_wait_bounded(&bar[1], 0);
      mbar_wait_bounded(&bar[1], 1);
    }
    __syncthreads();
  }
  block_partials<FNT>(ek.value(), ep.value(), vm2, bad, s.partials + ((size_t)ls * s.nblocks + blin) * 4);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3D map over one padded FP32 field: dims (nx, ny, nz), row pitch px floats;
// box (32 + 8) x (TY + 2) x 1; out-of-range elements read as zero.
static bool make_map(CUtensorMap* m, const float* base, int nx, int ny, int nz, int px, int ty) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base) return false;
  cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  cuuint64_t strides[2] = {(cuuint64_t)px * 4, (cuuint64_t)px * ny * 4};
  cuuint32_t box[3] = {FTX + 8, (cuuint32_t)(ty + 2), 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int TY, bool HET>
static cudaError_t set_smem_attr() {
  return cudaFuncSetAttribute(fused3d_kernel<TY, HET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)Geo<TY, HET>::SMEM);
}

struct FusedPlan {
  TmapSet maps[2];  // maps[q] reads buffer set q
  int ty, lz;
  bool het;
};

bool fused3d_supported() { return encode_fn() != nullptr; }

size_t fused3d_smem(int ty, bool het) {
  if (ty == 8) return het ? Geo<8, true>::SMEM : Geo<8, false>::SMEM;
  return het ? Geo<16, true>::SMEM : Geo<16, false>::SMEM;
}

// Build the tensor maps of both buffer sets. fields[q][f] = field f of set q.
bool fused3d_make_maps(void* plan_mem, float* const fields[2][9], const float* lam, const float* mu,
                       const float* rho, int nx, int ny, int nz, int px, int ty, int lz, bool het) {
  FusedPlan* P = static_cast<FusedPlan*>(plan_mem);
  P->ty = ty; P->lz = lz; P->het = het;
  // opt in to the dynamic shared memory once per configuration, outside any
  // stream capture
  cudaError_t e = ty == 8 ? (het ? set_smem_attr<8, true>() : set_smem_attr<8, false>())
                          : (het ? set_smem_attr<16, true>() : set_smem_attr<16, false>());
  if (e != cudaSuccess) return false;
  for (int q = 0; q < 2; ++q) {
    for (int f = 0; f < 9; ++f)
      if (!make_map(&P->maps[q].f[f], fields[q][f], nx, ny, nz, px, ty)) return false;
    if (het) {
      if (!make_map(&P->maps[q].lam, lam, nx, ny, nz, px, ty)) return false;
      if (!make_map(&P->maps[q].mu, mu, nx, ny, nz, px, ty)) return false;
      if (!make_map(&P->maps[q].rho, rho, nx, ny, nz, px, ty)) return false;
    } else {
      P->maps[q].lam = P->maps[q].f[0];
      P->maps[q].mu = P->maps[q].f[0];
      P->maps[q].rho = P->maps[q].f[0];
    }
  }
  return true;
}

size_t fused3d_plan_bytes() { return sizeof(FusedPlan); }

dim3 fused3d_grid(int nx, int ny, int nz, int ty, int lz) {
  const int ntx = (nx + FTX - 1) / FTX, nty = (ny + ty - 1) / ty, nkz = (nz + lz - 1) / lz;
  return dim3(ntx, nty * nkz, 1);
}

template <int TY, bool HET>
static cudaError_t launch_t(const FusedPlan* P, const StepArgs& s, int ls, int parity, cudaStream_t st) {
  using G = Geo<TY, HET>;
  const dim3 g = fused3d_grid(s.nx, s.ny, s.nz, TY, P->lz);
  fused3d_kernel<TY, HET><<<g, FNT, G::SMEM, st>>>(P->maps[parity], s, ls, P->lz);
  return cudaGetLastError();
}

cudaError_t fused3d_launch(const void* plan_mem, const StepArgs& s, int ls, int parity, cudaStream_t st) {
  const FusedPlan* P = static_cast<const FusedPlan*>(plan_mem);
  if (P->ty == 8) return P->het ? launch_t<8, true>(P, s, ls, parity, st) : launch_t<8, false>(P, s, ls, parity, st);
  return P->het ? launch_t<16, true>(P, s, ls, parity, st) : launch_t<16, false>(P, s, ls, parity, st);
}

}  // namespace cpml
