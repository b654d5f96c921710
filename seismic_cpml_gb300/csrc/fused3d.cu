// fused3d.cu -- one-sweep 3D velocity-stress C-PML time step for sm_103a.
//
// One step advances every field one full time step of
// seismic_CPML_3D_isotropic_MPI_OpenMP.f90 (stress 3D:836-943, velocity
// 3D:976-1052, source 3D:1055-1083, rigid faces 3D:1087-1121, energy
// 3D:1131-1180), reading time level n from buffer set A and writing time
// level n+1 to buffer set B. With separate read and write sets no CTA can
// see another CTA's half-updated cells, so the sweep needs no grid-wide
// synchronisation and every field crosses HBM once per step (9 reads + 9
// writes = 72 B/cell, the compulsory minimum).
//
// Work items: a 32 x TY tile of (i, j) columns over a chunk [kb, ke) of
// planes. Items are split into two lists launched as two kernels that run
// concurrently (they share no cells and only read set A):
//   interior items -- the tile, its one-cell halo and all planes kb-1..ke lie
//       outside every C-PML slab and every rigid face: no memory variables,
//       no loop-range masks; compiled lean for high occupancy (a per-cell
//       model adds lambda/mu/rho boxes to the same TMA pipeline);
//   general items  -- everything else (PML slabs, faces, partial tiles),
//       with every memory-variable load of a cell issued together before
//       its arithmetic.
// A CTA streams its planes in z (2.5D); at iteration m it
//   1. computes the new stresses at plane m on the tile plus the halo cells
//      the velocity update reads (left column: sigma_xx, top row: sigma_yy,
//      right column: sigma_xy/sigma_xz, bottom row: sigma_xy/sigma_yz) into a
//      shared-memory ring of planes, storing its own cells to B; the old
//      velocities and stresses come from TMA boxes (32+8) x (TY+2) loaded two
//      planes ahead (x window from i0-4 for 16-byte TMA alignment, one-cell
//      halo in y, zero fill outside the grid);
//   2. requests load group g(m+2) into the slots stress(m) was the last to
//      read (each thread carries its own cells' old velocities in registers);
//   3. computes the new velocities one plane behind (plane m-1) from the
//      stress ring (planes m-2..m), then source, rigid faces, store to B and
//      the energy partials;
//   4. (next iteration) every thread waits for g(m+1) on its mbarrier; the
//      one CTA barrier of an iteration sits between its stress and velocity
//      sweeps, and 4-plane stress rings let a warp's stress sweep of plane
//      m+1 overlap other warps' velocity sweep of plane m-1.
// Stress-side C-PML memory variables are ping-ponged like the fields (halo
// cells read time-n values that their owner is overwriting); velocity-side
// ones are updated in place (only the owner touches them).
//
// Waits on the TMA barriers are bounded (clock64); on timeout the CTA sets
// the device error word, drains its outstanding copies with a second bounded
// wait and leaves the sweep. The host reports CPML_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>
#include <vector>
#include "cpml_internal.cuh"
#include "kutil.cuh"
#include "tma.cuh"

namespace cpml {

struct TmapSet {
  CUtensorMap f[9];    // vx vy vz sxx syy szz sxy sxz syz of the read set
  CUtensorMap lam, mu, rho;
};

constexpr int FTX = 32;            // tile width in i (one warp)
constexpr int FNT = 256;           // threads per CTA: 32 x 8
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

// Which updates of a cell apply as far as its (i, j) go, for the general
// path's face handling (the plane conditions are added per plane):
//   bit 0 sigma_xx/yy/zz  j >= 1, i <= NX-2     bit 4 v_x   j >= 1, i >= 1
//   bit 1 sigma_xy        j <= NY-2, i >= 1     bit 5 v_y   j <= NY-2, i <= NX-2
//   bit 2 sigma_xz        i >= 1                bit 6 v_z   j >= 1, i <= NX-2
//   bit 3 sigma_yz        j <= NY-2             bit 7 on an x or y face (rigid)
__device__ __forceinline__ int cell_bits(int i, int j, int nx, int ny) {
  const bool jl = j >= 1, jh = j <= ny - 2, il = i >= 1, ih = i <= nx - 2;
  return (jl && ih ? 1 : 0) | (jh && il ? 2 : 0) | (il ? 4 : 0) | (jh ? 8 : 0) | (jl && il ? 16 : 0) |
         (jh && ih ? 32 : 0) | (jl && ih ? 64 : 0) | (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 ? 128 : 0);
}
// position of the n-th (0-based) set bit of m
__device__ __forceinline__ int nth_set(unsigned m, int n) {
  for (int k = 0; k < n; ++k) m &= m - 1;
  return __ffs(m) - 1;
}

template <int TY, bool HET>
struct Geo {
  static constexpr int BX = FTX + 8;                 // TMA box width (x from i0-4)
  static constexpr int BY = TY + 2;                  // box height (y from j0-1)
  static constexpr int BOX = BX * BY;                // floats per box
  static constexpr int SLOT = (BOX * 4 + 127) / 128 * 32;  // slot stride, 128-byte aligned
  static constexpr int RX = FTX + 2, RY = TY + 2, REG = RX * RY;  // stress ring plane
  // Power-of-two rings, a plane's slot is (m & (S-1)). Loads run two planes
  // ahead: v_x/v_y/v_z and rho need at most 4 live planes, old stresses 2.
  // lambda (4) and mu (8: plane m+3 is requested while the velocity sweep of
  // plane m-1 still reads plane m-1) also serve the energy of the velocity
  // sweep's plane. The six stress rings hold 4 planes each, so the stress
  // sweep of plane m+1 never overwrites a plane the velocity sweep of plane
  // m-1 still reads (they may overlap in time: one CTA barrier per plane).
  static constexpr int NBOX = 4 + 4 + 4 + 12 + (HET ? 4 + 8 + 4 : 0);
  static constexpr int RING = 24 * REG;
  // the tile's C-PML coefficients: a, b, 1/K at grid and half points, for
  // x = i0-4 .. i0+FTX+3 and y = j0-1 .. j0+TY
  static constexpr int NCOF = 6 * (BX + RY);
  static constexpr size_t SMEM = (size_t)NBOX * SLOT * 4 + (size_t)RING * 4 + (size_t)NCOF * 4 + 16 + 64;
  static constexpr int NH = 2 * FTX + 2 * TY;        // halo stress cells
};

// Item classes. Interior items take the lean path; the other four take the
// general path, compiled per class so that a class whose items can touch
// only one C-PML slab (and that axis's rigid faces) carries no code or
// registers for the other two, and requests all of a plane's memory
// variables at the top of the iteration (see below).
enum : int { CLS_INTERIOR = 0, CLS_X = 1, CLS_Y = 2, CLS_Z = 3, CLS_GEN = 4 };

template <int TY, int CLS, bool HET>
__global__ void __launch_bounds__(FNT, HET ? 2 : ((CLS == CLS_INTERIOR || TY == 8) ? 3 : 2))
    fused3d_kernel(const __grid_constant__ TmapSet tm, StepArgs s, int ls,
                   const int4* __restrict__ items, int item_base, int record) {
  constexpr bool FAST = CLS == CLS_INTERIOR;
  constexpr bool UX = CLS == CLS_X || CLS == CLS_GEN;   // x slab / x faces possible
  constexpr bool UY = CLS == CLS_Y || CLS == CLS_GEN;
  constexpr bool UZ = CLS == CLS_Z || CLS == CLS_GEN;
  constexpr bool EARLY = CLS == CLS_X || CLS == CLS_Y || CLS == CLS_Z;
  // Z-class items away from the z faces take a lean copy of the interior
  // code with only the z-axis memory variables added
  constexpr bool LEANZ = CLS == CLS_Z;
  using G = Geo<TY, HET>;
  constexpr int BX = G::BX, SLOT = G::SLOT, RX = G::RX, REG = G::REG;
  constexpr int NQ = TY / 8;             // own rows per thread
  extern __shared__ __align__(128) float sm[];
  float* vxs = sm;                       // [4] slots
  float* vys = vxs + 4 * SLOT;           // [4]
  float* vzs = vys + 4 * SLOT;           // [4]
  float* sos = vzs + 4 * SLOT;           // [2][6]
  float* lms = sos + 12 * SLOT;          // per-cell model: lam[4], mu[8], rho[4]
  float* mus = lms + 4 * SLOT;
  float* rhs = mus + 8 * SLOT;
  float* ring = sm + G::NBOX * SLOT;
  float* r_sxx = ring;                   // [4] each
  float* r_syy = r_sxx + 4 * REG;
  float* r_sxy = r_syy + 4 * REG;
  float* r_szz = r_sxy + 4 * REG;
  float* r_sxz = r_szz + 4 * REG;
  float* r_syz = r_sxz + 4 * REG;
  float* cfx = r_syz + 4 * REG;          // [6][BX]: a b ik ah bh ikh along x
  float* cfy = cfx + 6 * BX;             // [6][RY] along y
  uint64_t* bar = reinterpret_cast<uint64_t*>(cfy + 6 * G::RY);

  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  const int4 item = items[blockIdx.x];
  const int i0 = item.x, j0 = item.y, kb = item.z, ke = item.w;
  const int kk0 = kb - 1;
  const long long blin = item_base + blockIdx.x;   // slot of this item's energy partials
  const int it = *s.it_base + ls + 1;

  // receivers of the step that just ended, from the read set
  if (record && ls > 0) {
    const size_t slab = (size_t)s.nrec * s.nstep;
    for (long long r = (long long)blockIdx.x * FNT + tid; r < s.nrec; r += (long long)gridDim.x * FNT) {
      const long long c = s.rec_cell[r];
      const size_t o = (size_t)r * s.nstep + (size_t)(it - 2);
      s.seis[o] = s.f.vx[c];
      s.seis[slab + o] = s.f.vy[c];
      s.seis[2 * slab + o] = s.f.vz[c];
    }
  }

  constexpr uint32_t kBoxBytes = (uint32_t)G::BOX * 4;
  // load group g(m): vx(m+1), vy(m+1), vz(m), six old stresses at m
  // (+ lam(m), mu(m+1), rho(m)); the first group also brings vx(m), vy(m),
  // vz(m-1) (+ mu(m)).
  auto issue_group = [&](int m, uint64_t* b, bool prologue) {
    const int x = i0 - 4, y = j0 - 1;
    const uint32_t nb = 9 + (HET ? 3 : 0) + (prologue ? (3 + (HET ? 1 : 0)) : 0);
    mbar_expect_tx(b, nb * kBoxBytes);
    tma_load_3d(vxs + ((m + 1) & 3) * SLOT, &tm.f[0], x, y, m + 1, b);
    tma_load_3d(vys + ((m + 1) & 3) * SLOT, &tm.f[1], x, y, m + 1, b);
    tma_load_3d(vzs + (m & 3) * SLOT, &tm.f[2], x, y, m, b);
#pragma unroll
    for (int c = 0; c < 6; ++c) tma_load_3d(sos + ((m & 1) * 6 + c) * SLOT, &tm.f[3 + c], x, y, m, b);
    if (HET) {
      tma_load_3d(lms + (m & 3) * SLOT, &tm.lam, x, y, m, b);
      tma_load_3d(mus + ((m + 1) & 7) * SLOT, &tm.mu, x, y, m + 1, b);
      tma_load_3d(rhs + (m & 3) * SLOT, &tm.rho, x, y, m, b);
    }
    if (prologue) {
      tma_load_3d(vxs + (m & 3) * SLOT, &tm.f[0], x, y, m, b);
      tma_load_3d(vys + (m & 3) * SLOT, &tm.f[1], x, y, m, b);
      tma_load_3d(vzs + ((m - 1) & 3) * SLOT, &tm.f[2], x, y, m - 1, b);
      if (HET) tma_load_3d(mus + (m & 7) * SLOT, &tm.mu, x, y, m, b);
    }
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // The coefficients depend on one coordinate only: staged once per item,
  // they cost the plane loop shared-memory reads instead of an L2 round
  // trip per sweep. Points off the axis get the neutral a = b = 0, 1/K = 1.
  if (UX) {
    for (int t = tid; t < 6 * BX; t += FNT) {
      const int c = t / BX, i = i0 - 4 + (t - c * BX);
      const float* arr = c == 0 ? s.ax.a : c == 1 ? s.ax.b : c == 2 ? s.ax.ik
                       : c == 3 ? s.ax.ah : c == 4 ? s.ax.bh : s.ax.ikh;
      cfx[t] = (i >= 0 && i < s.ax.n) ? __ldg(arr + i) : (c == 2 || c == 5 ? 1.f : 0.f);
    }
  }
  if (UY) {
    for (int t = tid; t < 6 * G::RY; t += FNT) {
      const int c = t / G::RY, j = j0 - 1 + (t - c * G::RY);
      const float* arr = c == 0 ? s.ay.a : c == 1 ? s.ay.b : c == 2 ? s.ay.ik
                       : c == 3 ? s.ay.ah : c == 4 ? s.ay.bh : s.ay.ikh;
      cfy[t] = (j >= 0 && j < s.ay.n) ? __ldg(arr + j) : (c == 2 || c == 5 ? 1.f : 0.f);
    }
  }
  __syncthreads();
  if (tid == 0) {
    issue_group(kk0, &bar[0], true);
    if (kk0 + 1 <= ke) issue_group(kk0 + 1, &bar[1], false);
  }
  bool ok_all = true;

  // ---- tile classification (uniform over the CTA) ---------------------------
  const int wx = s.ax.width(), wy = s.ay.width();
  const long long px = s.px, pl = s.plane;
  const bool xs_tile = UX && wx > 0 && (i0 - 1 < s.ax.lo || i0 + FTX >= nx - s.ax.hi);
  const bool ys_tile = UY && wy > 0 && (j0 - 1 < s.ay.lo || j0 + TY >= ny - s.ay.hi);
  const bool edge_tile = i0 - 1 < 1 || i0 + FTX > nx - 2 || j0 - 1 < 1 || j0 + TY > ny - 2;
  const int n0 = s.npml;
  const bool e_full_xy = i0 >= n0 && i0 + FTX <= nx - n0 && j0 >= n0 && j0 + TY <= ny - n0;
  const bool has_src = s.isrc >= i0 && s.isrc < i0 + FTX && s.jsrc >= j0 && s.jsrc < j0 + TY &&
                       s.ksrc >= kb && s.ksrc < ke;
  const float src_x = has_src ? s.src_fx[it - 1] : 0.f;
  const float src_y = has_src ? s.src_fy[it - 1] : 0.f;

  // ---- per-thread constants ---------------------------------------------------
  // In-plane offsets, fixed for the whole item: fo = j * px + i of a cell's
  // fields, and of its memory variables on each slab axis (-1 outside the
  // slab): x slab [k][j][sx], y slab [k][sy][i], z slab [sz][j][i] (= fo).
  // A plane's base is added per plane, so every access is one 32-bit offset
  // from a plane pointer.
  const int pxi = (int)px;
  // The thread's own cell (cx, cy) in the tile: lanes are columns, except in
  // X-class items, where the tile's x-slab columns are packed into the lowest
  // warps (then its other columns inside the grid, then those past it) so
  // that only those warps run the C-PML code -- a warp pays for a branch
  // whether 10 or 32 of its lanes take it. Halo cells go to the highest
  // warps (hid counts down from the last thread).
  static_assert(CLS != CLS_X || TY * FTX == FNT, "X-class items are one cell per thread");
  int cx = tx, cy = ty;
  if (CLS == CLS_X) {
    const int ci = i0 + tx;
    const unsigned vmask = __ballot_sync(0xffffffffu, ci < nx);
    const unsigned smask = __ballot_sync(0xffffffffu, ci < nx && s.ax.slab(ci) >= 0);
    const unsigned grp[3] = {smask, vmask & ~smask, ~vmask};
    int u = tid;
#pragma unroll
    for (int g = 0; g < 3; ++g) {
      const int w = __popc(grp[g]);
      if (u >= 0 && u < w * TY) { cy = u / w; cx = nth_set(grp[g], u % w); }
      u -= w * TY;
    }
  }
  const int oi = i0 + cx;
  const int osx = (oi < nx) ? s.ax.slab(oi) : -1;
  int oj[NQ], ofo[NQ], omx[NQ], omy[NQ], ocb[NQ];
  bool ov[NQ], oe[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    oj[q] = j0 + cy + 8 * q;
    ov[q] = oi < nx && oj[q] < ny;
    const int osy = ov[q] ? s.ay.slab(oj[q]) : -1;
    ofo[q] = oj[q] * pxi + oi;
    omx[q] = (UX && xs_tile && ov[q] && osx >= 0) ? oj[q] * wx + osx : -1;
    omy[q] = (UY && ys_tile && osy >= 0) ? osy * pxi + oi : -1;
    oe[q] = e_full_xy || (oi >= n0 && oi < nx - n0 && oj[q] >= n0 && oj[q] < ny - n0);
    ocb[q] = cell_bits(oi, oj[q], nx, ny);
  }
  const int b_own = (cy + 1) * BX + cx + 4;
  const int r_own = (cy + 1) * RX + cx + 1;
  const int hid = FNT - 1 - tid;
  int hi = 0, hj = 0, hcomps = 0;
  if (hid < G::NH) {
    if (hid < FTX) { hi = i0 + hid; hj = j0 + TY; hcomps = 1; }                        // top: yy
    else if (hid < 2 * FTX) { hi = i0 + hid - FTX; hj = j0 - 1; hcomps = 2 | 8; }       // bottom: xy, yz
    else if (hid < 2 * FTX + TY) { hi = i0 - 1; hj = j0 + hid - 2 * FTX; hcomps = 1; }  // left: xx
    else { hi = i0 + FTX; hj = j0 + hid - 2 * FTX - TY; hcomps = 2 | 4; }               // right: xy, xz
  }
  const bool hv = hid < G::NH && hi >= 0 && hi < nx && hj >= 0 && hj < ny;
  const int hfo = hj * pxi + hi;
  const int hmx = (UX && xs_tile && hv && s.ax.slab(hi) >= 0) ? hj * wx + s.ax.slab(hi) : -1;
  const int hmy = (UY && ys_tile && hv && s.ay.slab(hj) >= 0) ? s.ay.slab(hj) * pxi + hi : -1;
  const int hcb = cell_bits(hi, hj, nx, ny);
  const int hb = (hj - j0 + 1) * BX + (hi - i0 + 4);
  const int hr = (hj - j0 + 1) * RX + (hi - i0 + 1);

  Kahan ek, ep;
  float vm2 = 0.f;
  int bad = 0;
  // own cells' time-n velocities of plane m, carried from the stress sweep
  // of iteration m to the velocity sweep of iteration m+1
  float cvx[NQ], cvy[NQ], cvz[NQ], nvx[NQ], nvy[NQ], nvz[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) { cvx[q] = cvy[q] = cvz[q] = nvx[q] = nvy[q] = nvz[q] = 0.f; }

  for (int m = kk0; m <= ke; ++m) {
    const int use = m - kk0;
    // Single-axis classes: every memory variable this iteration reads (own
    // and halo stress cells at plane m, own velocity cells at plane m-1) is
    // requested here, before the TMA wait, so one HBM round trip per plane
    // overlaps all the work instead of three following one another.
    float e_own[NQ][3], e_vel[NQ][3], e_halo[3];
    if (EARLY) {
      const int p = m - 1;
      const bool sm_ok = m >= 0 && m < nz, vp_ok = p >= kb && p < ke;
      const int szm = (CLS == CLS_Z && sm_ok) ? s.az.slab(m) : -1;
      const int szp = (CLS == CLS_Z && vp_ok) ? s.az.slab(p) : -1;
      // plane base of the class axis's memory variables (Z: the slab plane)
      auto mbase = [&](int k, int sz_) -> long long {
        if (CLS == CLS_X) return (long long)k * ny * wx;
        if (CLS == CLS_Y) return (long long)k * wy * px;
        return (long long)sz_ * ny * px;
      };
      const float* const* A = CLS == CLS_X ? s.m.x : (CLS == CLS_Y ? s.m.y : s.m.z);
      const bool m_in = sm_ok && (CLS != CLS_Z || szm >= 0);
      const bool p_in = vp_ok && (CLS != CLS_Z || szp >= 0);
      const long long bm = m_in ? mbase(m, szm) : 0, bp = p_in ? mbase(p, szp) : 0;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        e_own[q][0] = e_own[q][1] = e_own[q][2] = 0.f;
        e_vel[q][0] = e_vel[q][1] = e_vel[q][2] = 0.f;
        const int mo = CLS == CLS_X ? omx[q] : (CLS == CLS_Y ? omy[q] : (ov[q] ? ofo[q] : -1));
        if (m_in && mo >= 0) {
          e_own[q][0] = (A[0] + bm)[mo]; e_own[q][1] = (A[1] + bm)[mo]; e_own[q][2] = (A[2] + bm)[mo];
        }
        if (p_in && mo >= 0) {
          e_vel[q][0] = (A[3] + bp)[mo]; e_vel[q][1] = (A[4] + bp)[mo]; e_vel[q][2] = (A[5] + bp)[mo];
        }
      }
      e_halo[0] = e_halo[1] = e_halo[2] = 0.f;
      const int hmo = CLS == CLS_X ? hmx : (CLS == CLS_Y ? hmy : (hv ? hfo : -1));
      if (m_in && hmo >= 0) {
        e_halo[0] = (A[0] + bm)[hmo]; e_halo[1] = (A[1] + bm)[hmo]; e_halo[2] = (A[2] + bm)[hmo];
      }
    }
    // every thread waits for load group g(m) itself (try_wait suspends the
    // thread in hardware), so there is one CTA barrier per plane
    const bool landed = mbar_wait_bounded(&bar[use & 1], (uint32_t)((use >> 1) & 1), kWaitCycles);
    // ======================= stress at plane m ==============================
    const float* VX0 = vxs + (m & 3) * SLOT;
    const float* VX1 = vxs + ((m + 1) & 3) * SLOT;
    const float* VY0 = vys + (m & 3) * SLOT;
    const float* VY1 = vys + ((m + 1) & 3) * SLOT;
    const float* VZ0 = vzs + (m & 3) * SLOT;
    const float* VZm = vzs + ((m - 1) & 3) * SLOT;
    const float* SO = sos + (m & 1) * 6 * SLOT;
    float* Rxx = r_sxx + (m & 3) * REG;
    float* Ryy = r_syy + (m & 3) * REG;
    float* Rzz = r_szz + (m & 3) * REG;
    float* Rxy = r_sxy + (m & 3) * REG;
    float* Rxz = r_sxz + (m & 3) * REG;
    float* Ryz = r_syz + (m & 3) * REG;
    const bool st_plane = m >= kb && m < ke;
    if (!landed) {
      // nothing to compute on boxes that did not arrive
    } else if (FAST) {
      const long long cpl = (long long)m * pl + (long long)j0 * px + i0;
      const float* Lm = lms + (m & 3) * SLOT;
      const float* M0 = mus + (m & 7) * SLOT;
      const float* M1 = mus + ((m + 1) & 7) * SLOT;
      // interior tiles never touch the last column, so the 8-point mu
      // average of sigma_yz always takes i+1 (the general path clamps it)
      auto cell = [&](int b, int r, int comps, bool store, long long c, float& ox, float& oy, float& oz) {
        const float vxc = VX0[b], vyc = VY0[b], vzc = VZ0[b];
        ox = vxc; oy = vyc; oz = vzc;
        if (comps & 1) {
          const float dxx = (VX0[b + 1] - vxc) * s.odx;
          const float dyy = (vyc - VY0[b - BX]) * s.ody;
          const float dzz = (vzc - VZm[b]) * s.odz;
          float dl = s.dt_lam, dl2m = s.dt_l2m;
          if (HET) {
            const float lh = 0.5f * (Lm[b + 1] + Lm[b]);
            const float mh = 0.5f * (M0[b + 1] + M0[b]);
            dl = s.dt * lh;
            dl2m = s.dt * (lh + 2.0f * mh);
          }
          const float nxx = SO[b] + (dl2m * dxx + dl * (dyy + dzz));
          const float nyy = SO[SLOT + b] + (dl * (dxx + dzz) + dl2m * dyy);
          const float nzz = SO[2 * SLOT + b] + (dl * (dxx + dyy) + dl2m * dzz);
          Rxx[r] = nxx; Ryy[r] = nyy; Rzz[r] = nzz;
          if (store) { s.g.sxx[c] = nxx; s.g.syy[c] = nyy; s.g.szz[c] = nzz; }
        }
        if (comps & 2) {
          const float dm = HET ? s.dt * (0.5f * (M0[b + BX] + M0[b])) : s.dt_mu;
          const float n = SO[3 * SLOT + b] + dm * ((vyc - VY0[b - 1]) * s.odx + (VX0[b + BX] - vxc) * s.ody);
          Rxy[r] = n;
          if (store) s.g.sxy[c] = n;
        }
        if (comps & 4) {
          const float dm = HET ? s.dt * (0.5f * (M1[b] + M0[b])) : s.dt_mu;
          const float n = SO[4 * SLOT + b] + dm * ((vzc - VZ0[b - 1]) * s.odx + (VX1[b] - vxc) * s.odz);
          Rxz[r] = n;
          if (store) s.g.sxz[c] = n;
        }
        if (comps & 8) {
          float dm = s.dt_mu;
          if (HET) {
            const float sm8 = ((((((M0[b] + M0[b + 1]) + M0[b + BX]) + M0[b + BX + 1]) + M1[b]) + M1[b + 1]) +
                               M1[b + BX]) + M1[b + BX + 1];
            dm = s.dt * (0.125f * sm8);
          }
          const float n = SO[5 * SLOT + b] + dm * ((VZ0[b + BX] - vzc) * s.ody + (VY1[b] - vyc) * s.odz);
          Ryz[r] = n;
          if (store) s.g.syz[c] = n;
        }
      };
#pragma unroll
      for (int q = 0; q < NQ; ++q)
        cell(b_own + q * 8 * BX, r_own + q * 8 * RX, 15, st_plane, cpl + (long long)(ty + 8 * q) * px + tx,
             nvx[q], nvy[q], nvz[q]);
      if (hid < G::NH) {
        float dx, dy, dz;
        cell(hb, hr, hcomps, false, 0, dx, dy, dz);
      }
    } else if (LEANZ && m >= 1 && m <= nz - 2 && !edge_tile) {
      // Z-class items away from the z faces: the interior path's code with
      // only the z-derivative terms through the C-PML memory variables (the
      // same arithmetic as the general path, whose face handling and x/y
      // slab code these items never need)
      const long long cpl = (long long)m * pl;
      const float* Lm = lms + (m & 3) * SLOT;
      const float* M0 = mus + (m & 7) * SLOT;
      const float* M1 = mus + ((m + 1) & 7) * SLOT;
      const int sz = s.az.slab(m);
      const bool zs = sz >= 0;
      float za = 0.f, zb = 0.f, zk = 1.f, zah = 0.f, zbh = 0.f, zkh = 1.f;
      if (zs) {
        za = __ldg(s.az.a + m); zb = __ldg(s.az.b + m); zk = __ldg(s.az.ik + m);
        zah = __ldg(s.az.ah + m); zbh = __ldg(s.az.bh + m); zkh = __ldg(s.az.ikh + m);
      }
      const long long mzp = (long long)sz * ny * px;
      auto cellz = [&](int b, int r, int fo, int comps, bool store, const float* pre) {
        const long long c = cpl + fo;
        auto psi = [&](float d, float old, int k, float a_, float b_, float k_) {
          const float nw = b_ * old + a_ * d;
          if (store) (s.mb.z[k] + mzp)[fo] = nw;
          return d * k_ + nw;
        };
        const float vxc = VX0[b], vyc = VY0[b], vzc = VZ0[b];
        if (comps & 1) {
          const float dxx = (VX0[b + 1] - vxc) * s.odx;
          const float dyy = (vyc - VY0[b - BX]) * s.ody;
          float dzz = (vzc - VZm[b]) * s.odz;
          if (zs) dzz = psi(dzz, pre[2], 2, za, zb, zk);
          float dl = s.dt_lam, dl2m = s.dt_l2m;
          if (HET) {
            const float lh = 0.5f * (Lm[b + 1] + Lm[b]);
            const float mh = 0.5f * (M0[b + 1] + M0[b]);
            dl = s.dt * lh;
            dl2m = s.dt * (lh + 2.0f * mh);
          }
          const float nxx = SO[b] + (dl2m * dxx + dl * (dyy + dzz));
          const float nyy = SO[SLOT + b] + (dl * (dxx + dzz) + dl2m * dyy);
          const float nzz = SO[2 * SLOT + b] + (dl * (dxx + dyy) + dl2m * dzz);
          Rxx[r] = nxx; Ryy[r] = nyy; Rzz[r] = nzz;
          if (store) { s.g.sxx[c] = nxx; s.g.syy[c] = nyy; s.g.szz[c] = nzz; }
        }
        if (comps & 2) {
          const float dm = HET ? s.dt * (0.5f * (M0[b + BX] + M0[b])) : s.dt_mu;
          const float d1 = (vyc - VY0[b - 1]) * s.odx;
          const float d2 = (VX0[b + BX] - vxc) * s.ody;
          const float n = SO[3 * SLOT + b] + dm * (d1 + d2);
          Rxy[r] = n;
          if (store) s.g.sxy[c] = n;
        }
        if (comps & 4) {
          const float dm = HET ? s.dt * (0.5f * (M1[b] + M0[b])) : s.dt_mu;
          const float d1 = (vzc - VZ0[b - 1]) * s.odx;
          float d2 = (VX1[b] - vxc) * s.odz;
          if (zs) d2 = psi(d2, pre[0], 0, zah, zbh, zkh);
          const float n = SO[4 * SLOT + b] + dm * (d1 + d2);
          Rxz[r] = n;
          if (store) s.g.sxz[c] = n;
        }
        if (comps & 8) {
          float dm = s.dt_mu;
          if (HET) {
            const float sm8 = ((((((M0[b] + M0[b + 1]) + M0[b + BX]) + M0[b + BX + 1]) + M1[b]) + M1[b + 1]) +
                               M1[b + BX]) + M1[b + BX + 1];
            dm = s.dt * (0.125f * sm8);
          }
          const float d1 = (VZ0[b + BX] - vzc) * s.ody;
          float d2 = (VY1[b] - vyc) * s.odz;
          if (zs) d2 = psi(d2, pre[1], 1, zah, zbh, zkh);
          const float n = SO[5 * SLOT + b] + dm * (d1 + d2);
          Ryz[r] = n;
          if (store) s.g.syz[c] = n;
        }
      };
#pragma unroll
      for (int q = 0; q < NQ; ++q)
        if (ov[q]) {
          const int b = b_own + q * 8 * BX;
          nvx[q] = VX0[b]; nvy[q] = VY0[b]; nvz[q] = VZ0[b];
          cellz(b, r_own + q * 8 * RX, ofo[q], 15, st_plane, e_own[q]);
        }
      if (hv) cellz(hb, hr, hfo, hcomps, false, e_halo);
    } else if (m >= 0 && m < nz) {
      const float* Lm = lms + (m & 3) * SLOT;
      const float* M0 = mus + (m & 7) * SLOT;
      const float* M1 = mus + ((m + 1) & 7) * SLOT;
      const bool edge = edge_tile || m < 1 || m > nz - 2;
      const int sz = UZ ? s.az.slab(m) : -1;
      const bool zs = UZ && sz >= 0;
      float za = 0.f, zb = 0.f, zk = 1.f, zah = 0.f, zbh = 0.f, zkh = 1.f;
      if (zs) {
        za = __ldg(s.az.a + m); zb = __ldg(s.az.b + m); zk = __ldg(s.az.ik + m);
        zah = __ldg(s.az.ah + m); zbh = __ldg(s.az.bh + m); zkh = __ldg(s.az.ikh + m);
      }
      const long long mxp = (long long)m * ny * wx;
      const long long myp = (long long)m * wy * px;
      const long long mzp = (long long)sz * ny * px;
      const long long cpl = (long long)m * pl;

      // one stress cell: box/ring offsets, grid (i, j), in-plane offsets of
      // its fields (fo) and x/y memory variables (-1 outside the slab),
      // components (1 normal, 2 xy, 4 xz, 8 yz); own = this CTA stores it
      // updates that apply at plane m (bits 0-3 of cell_bits): all of them
      // away from the faces
      const int sbits = edge ? (m >= 1 ? 1 : 0) | 2 | (m <= nz - 2 ? 12 : 0) : 15;
      auto stress = [&](int b, int r, int i, int j, int fo, int mx_, int my_, int cb, int comps, bool own,
                        const float* pre) {
        const bool st = own && st_plane;
        const int ok = edge ? (cb & sbits) : 15;
        const long long c = cpl + fo;
        const bool hx = UX && mx_ >= 0, hy = UY && my_ >= 0;
        const int mxi = mx_, myi = my_, mzi = fo;
        // every time-n memory variable and coefficient of the cell, issued
        // together so their latencies overlap
        float qx0 = 0.f, qx1 = 0.f, qx2 = 0.f, qy0 = 0.f, qy1 = 0.f, qy2 = 0.f;
        float qz0 = 0.f, qz1 = 0.f, qz2 = 0.f;
        float xa = 0.f, xb = 0.f, xk = 1.f, xah = 0.f, xbh = 0.f, xkh = 1.f;
        float ya = 0.f, yb = 0.f, yk = 1.f, yah = 0.f, ybh = 0.f, ykh = 1.f;
        if (hx) {
          if (EARLY) { qx0 = pre[0]; qx1 = pre[1]; qx2 = pre[2]; }
          else { qx0 = (s.m.x[0] + mxp)[mxi]; qx1 = (s.m.x[1] + mxp)[mxi]; qx2 = (s.m.x[2] + mxp)[mxi]; }
          const float* cx = cfx + (i - i0 + 4);
          xa = cx[0]; xb = cx[BX]; xk = cx[2 * BX]; xah = cx[3 * BX]; xbh = cx[4 * BX]; xkh = cx[5 * BX];
        }
        if (hy) {
          if (EARLY) { qy0 = pre[0]; qy1 = pre[1]; qy2 = pre[2]; }
          else { qy0 = (s.m.y[0] + myp)[myi]; qy1 = (s.m.y[1] + myp)[myi]; qy2 = (s.m.y[2] + myp)[myi]; }
          const float* cy = cfy + (j - j0 + 1);
          ya = cy[0]; yb = cy[G::RY]; yk = cy[2 * G::RY]; yah = cy[3 * G::RY]; ybh = cy[4 * G::RY];
          ykh = cy[5 * G::RY];
        }
        if (zs) {
          if (EARLY) { qz0 = pre[0]; qz1 = pre[1]; qz2 = pre[2]; }
          else { qz0 = (s.m.z[0] + mzp)[mzi]; qz1 = (s.m.z[1] + mzp)[mzi]; qz2 = (s.m.z[2] + mzp)[mzi]; }
        }
        // psi(n+1) = b psi(n) + a d ; d' = d / K + psi(n+1) (3D:846-852 and
        // the other sweeps); unchanged where the component is not updated
        auto psi = [&](float d, bool upd, float old, float* mB, int mi, float a_, float b_, float k_) {
          const float nw = upd ? b_ * old + a_ * d : old;
          if (st) mB[mi] = nw;
          return d * k_ + nw;
        };
        const float vxc = VX0[b], vyc = VY0[b], vzc = VZ0[b];
        if (comps & 1) {  // sigma_xx, yy, zz: k = 2..NZ, j = 2..NY, i = 1..NX-1 (3D:836-863)
          float d1 = (VX0[b + 1] - vxc) * s.odx;
          float d2 = (vyc - VY0[b - BX]) * s.ody;
          float d3 = (vzc - VZm[b]) * s.odz;
          const bool upd = ok & 1;
          if (hx) d1 = psi(d1, upd, qx0, s.mb.x[0] + mxp, mxi, xah, xbh, xkh);
          if (hy) d2 = psi(d2, upd, qy1, s.mb.y[1] + myp, myi, ya, yb, yk);
          if (zs) d3 = psi(d3, upd, qz2, s.mb.z[2] + mzp, mzi, za, zb, zk);
          float dl = s.dt_lam, dl2m = s.dt_l2m;
          if (HET) {
            const float lh = 0.5f * (Lm[b + 1] + Lm[b]);
            const float mh = 0.5f * (M0[b + 1] + M0[b]);
            dl = s.dt * lh;
            dl2m = s.dt * (lh + 2.0f * mh);
          }
          const float o1 = SO[b], o2 = SO[SLOT + b], o3 = SO[2 * SLOT + b];
          float nxx = o1 + (dl2m * d1 + dl * (d2 + d3));
          float nyy = o2 + (dl * (d1 + d3) + dl2m * d2);
          float nzz = o3 + (dl * (d1 + d2) + dl2m * d3);
          if (!upd) { nxx = o1; nyy = o2; nzz = o3; }
          Rxx[r] = nxx; Ryy[r] = nyy; Rzz[r] = nzz;
          if (st) { s.g.sxx[c] = nxx; s.g.syy[c] = nyy; s.g.szz[c] = nzz; }
        }
        if (comps & 2) {  // sigma_xy: k = 1..NZ, j = 1..NY-1, i = 2..NX (3D:877-894)
          float d1 = (vyc - VY0[b - 1]) * s.odx;
          float d2 = (VX0[b + BX] - vxc) * s.ody;
          const bool upd = ok & 2;
          if (hx) d1 = psi(d1, upd, qx1, s.mb.x[1] + mxp, mxi, xa, xb, xk);
          if (hy) d2 = psi(d2, upd, qy0, s.mb.y[0] + myp, myi, yah, ybh, ykh);
          const float dm = HET ? s.dt * (0.5f * (M0[b + BX] + M0[b])) : s.dt_mu;
          const float o = SO[3 * SLOT + b];
          const float n = upd ? o + dm * (d1 + d2) : o;
          Rxy[r] = n;
          if (st) s.g.sxy[c] = n;
        }
        if (comps & 4) {  // sigma_xz: k = 1..NZ-1, j = 1..NY, i = 2..NX (3D:908-925)
          float d1 = (vzc - VZ0[b - 1]) * s.odx;
          float d2 = (VX1[b] - vxc) * s.odz;
          const bool upd = ok & 4;
          if (hx) d1 = psi(d1, upd, qx2, s.mb.x[2] + mxp, mxi, xa, xb, xk);
          if (zs) d2 = psi(d2, upd, qz0, s.mb.z[0] + mzp, mzi, zah, zbh, zkh);
          const float dm = HET ? s.dt * (0.5f * (M1[b] + M0[b])) : s.dt_mu;
          const float o = SO[4 * SLOT + b];
          const float n = upd ? o + dm * (d1 + d2) : o;
          Rxz[r] = n;
          if (st) s.g.sxz[c] = n;
        }
        if (comps & 8) {  // sigma_yz: k = 1..NZ-1, j = 1..NY-1, i = 1..NX (3D:927-942)
          float d1 = (VZ0[b + BX] - vzc) * s.ody;
          float d2 = (VY1[b] - vyc) * s.odz;
          const bool upd = ok & 8;
          if (hy) d1 = psi(d1, upd, qy2, s.mb.y[2] + myp, myi, yah, ybh, ykh);
          if (zs) d2 = psi(d2, upd, qz1, s.mb.z[1] + mzp, mzi, zah, zbh, zkh);
          float dm = s.dt_mu;
          if (HET) {  // 8-point average at (i+1/2, j+1/2, k+1/2); i+1 clamped on the last column
            const int di = (i < nx - 1) ? 1 : 0;
            const float sm8 = ((((((M0[b] + M0[b + di]) + M0[b + BX]) + M0[b + BX + di]) + M1[b]) +
                                M1[b + di]) + M1[b + BX]) + M1[b + BX + di];
            dm = s.dt * (0.125f * sm8);
          }
          const float o = SO[5 * SLOT + b];
          const float n = upd ? o + dm * (d1 + d2) : o;
          Ryz[r] = n;
          if (st) s.g.syz[c] = n;
        }
      };

#pragma unroll
      for (int q = 0; q < NQ; ++q)
        if (ov[q]) {
          const int b = b_own + q * 8 * BX;
          nvx[q] = VX0[b]; nvy[q] = VY0[b]; nvz[q] = VZ0[b];
          stress(b, r_own + q * 8 * RX, oi, oj[q], ofo[q], omx[q], omy[q], ocb[q], 15, true, e_own[q]);
        }
      if (hv) stress(hb, hr, hi, hj, hfo, hmx, hmy, hcb, hcomps, false, e_halo);
    }
    if (!__syncthreads_and(landed ? 1 : 0)) { ok_all = false; break; }
    // g(m+2) goes into slots whose last reader was stress(m) (own-cell
    // velocities travel in registers; the velocity sweep reads only the
    // stress rings and rho planes m-1, m), so it is requested before velocity.
    if (tid == 0 && m + 2 <= ke) issue_group(m + 2, &bar[use & 1], false);

    // ======================= velocity at plane p = m - 1 ====================
    const int p = m - 1;
    if (p >= kb && p < ke) {
      const float* Sxx = r_sxx + (p & 3) * REG;
      const float* Syy = r_syy + (p & 3) * REG;
      const float* Sxy = r_sxy + (p & 3) * REG;
      const float* Szz0 = r_szz + (p & 3) * REG;
      const float* Szz1 = r_szz + ((p + 1) & 3) * REG;
      const float* Sxz0 = r_sxz + (p & 3) * REG;
      const float* Sxzm = r_sxz + ((p - 1) & 3) * REG;
      const float* Syz0 = r_syz + (p & 3) * REG;
      const float* Syzm = r_syz + ((p - 1) & 3) * REG;
      const bool e_z = p >= n0 && p < nz - n0;
      if (FAST) {
        const long long cpl = (long long)p * pl + (long long)j0 * px + i0;
        const float* R0 = rhs + (p & 3) * SLOT;
        const float* R1 = rhs + ((p + 1) & 3) * SLOT;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int r = r_own + q * 8 * RX;
          const int b = b_own + q * 8 * BX;
          const long long c = cpl + (long long)(ty + 8 * q) * px + tx;
          const float sxx = Sxx[r], syy = Syy[r], szz = Szz0[r];
          const float sxy = Sxy[r], sxz = Sxz0[r], syz = Syz0[r];
          float fx = s.dt_over_rho, fy = s.dt_over_rho, fz = s.dt_over_rho;
          if (HET) {
            fx = s.dt / R0[b];
            fy = s.dt / (0.25f * (R0[b] + R0[b + 1] + R0[b + 1 + BX] + R0[b + BX]));
            fz = s.dt / (0.25f * (R0[b] + R0[b + 1] + R1[b + 1] + R1[b]));
          }
          float vx = cvx[q] + fx * (((sxx - Sxx[r - 1]) * s.odx + (sxy - Sxy[r - RX]) * s.ody) +
                                    (sxz - Sxzm[r]) * s.odz);
          float vy = cvy[q] + fy * (((Sxy[r + 1] - sxy) * s.odx + (Syy[r + RX] - syy) * s.ody) +
                                    (syz - Syzm[r]) * s.odz);
          const float vz = cvz[q] + fz * (((Sxz0[r + 1] - sxz) * s.odx + (syz - Syz0[r - RX]) * s.ody) +
                                          (Szz1[r] - szz) * s.odz);
          if (has_src && p == s.ksrc && oi == s.isrc && oj[q] == s.jsrc) {
            vx += src_x;
            vy += src_y;
          }
          s.g.vx[c] = vx; s.g.vy[c] = vy; s.g.vz[c] = vz;
          const float v2 = vx * vx + vy * vy + vz * vz;
          vm2 = fmaxf(vm2, v2);
          bad |= not_finite(v2);
          if (e_z) {
            float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
            if (HET) {  // per-cell model of plane p
              const float l = lms[(p & 3) * SLOT + b], mu = mus[(p & 7) * SLOT + b];
              const float den = 1.0f / (2.0f * mu * (3.0f * l + 2.0f * mu));
              hr = 0.5f * R0[b];
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
      } else if (LEANZ && p >= 1 && p <= nz - 2 && !edge_tile) {
        // Z-class items away from the z faces (see the stress sweep)
        const long long cpl = (long long)p * pl;
        const float* R0 = rhs + (p & 3) * SLOT;
        const float* R1 = rhs + ((p + 1) & 3) * SLOT;
        const int sz = s.az.slab(p);
        const bool zs = sz >= 0;
        float za = 0.f, zb = 0.f, zk = 1.f, zah = 0.f, zbh = 0.f, zkh = 1.f;
        if (zs) {
          za = __ldg(s.az.a + p); zb = __ldg(s.az.b + p); zk = __ldg(s.az.ik + p);
          zah = __ldg(s.az.ah + p); zbh = __ldg(s.az.bh + p); zkh = __ldg(s.az.ikh + p);
        }
        const long long mzp = (long long)sz * ny * px;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          if (!ov[q]) continue;
          const int r = r_own + q * 8 * RX;
          const int b = b_own + q * 8 * BX;
          const long long c = cpl + ofo[q];
          const float sxx = Sxx[r], syy = Syy[r], szz = Szz0[r];
          const float sxy = Sxy[r], sxz = Sxz0[r], syz = Syz0[r];
          float d1 = (sxx - Sxx[r - 1]) * s.odx;   // v_x (3D:976-993)
          float d2 = (sxy - Sxy[r - RX]) * s.ody;
          float d3 = (sxz - Sxzm[r]) * s.odz;
          float e1 = (Sxy[r + 1] - sxy) * s.odx;   // v_y (3D:995-1014)
          float e2 = (Syy[r + RX] - syy) * s.ody;
          float e3 = (syz - Syzm[r]) * s.odz;
          float f1 = (Sxz0[r + 1] - sxz) * s.odx;  // v_z (3D:1031-1052)
          float f2 = (syz - Syz0[r - RX]) * s.ody;
          float f3 = (Szz1[r] - szz) * s.odz;
          if (zs) {   // in place (3D:979-985 and the like)
            auto psi = [&](float d, float old, int k, float a_, float b_, float k_) {
              const float nw = b_ * old + a_ * d;
              (s.m.z[k] + mzp)[ofo[q]] = nw;
              return d * k_ + nw;
            };
            d3 = psi(d3, e_vel[q][0], 3, za, zb, zk);
            e3 = psi(e3, e_vel[q][1], 4, za, zb, zk);
            f3 = psi(f3, e_vel[q][2], 5, zah, zbh, zkh);
          }
          float fx = s.dt_over_rho, fy = s.dt_over_rho, fz = s.dt_over_rho;
          if (HET) {
            fx = s.dt / R0[b];
            fy = s.dt / (0.25f * (R0[b] + R0[b + 1] + R0[b + 1 + BX] + R0[b + BX]));
            fz = s.dt / (0.25f * (R0[b] + R0[b + 1] + R1[b + 1] + R1[b]));
          }
          float vx = cvx[q] + fx * (d1 + d2 + d3);
          float vy = cvy[q] + fy * (e1 + e2 + e3);
          const float vz = cvz[q] + fz * (f1 + f2 + f3);
          if (has_src && p == s.ksrc && oi == s.isrc && oj[q] == s.jsrc) {  // 3D:1080-1081
            vx += src_x;
            vy += src_y;
          }
          s.g.vx[c] = vx; s.g.vy[c] = vy; s.g.vz[c] = vz;
          const float v2 = vx * vx + vy * vy + vz * vz;
          vm2 = fmaxf(vm2, v2);
          bad |= not_finite(v2);
          if (e_z && oe[q]) {  // energy interior (3D:1136-1143)
            float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
            if (HET) {
              const float l = lms[(p & 3) * SLOT + b], mu = mus[(p & 7) * SLOT + b];
              const float den = 1.0f / (2.0f * mu * (3.0f * l + 2.0f * mu));
              hr = 0.5f * R0[b];
              c1 = 2.0f * (l + mu) * den;
              c2 = l * den;
              i2m = 1.0f / (2.0f * mu);
            }
            ek.add(hr * v2);
            const float exx = c1 * sxx - c2 * (syy + szz);
            const float eyy = c1 * syy - c2 * (sxx + szz);
            // the reference adds eps_yy*sigma_yy twice and no zz term (3D:1170-1171)
            const float third = s.ep_physical ? (c1 * szz - c2 * (sxx + syy)) * szz : eyy * syy;
            ep.add(0.5f * (exx * sxx + eyy * syy + third) + i2m * (sxy * sxy + sxz * sxz + syz * syz));
          }
        }
      } else {
        const float* R0 = rhs + (p & 3) * SLOT;
        const float* R1 = rhs + ((p + 1) & 3) * SLOT;
        const bool edge = edge_tile || p < 1 || p > nz - 2;
        // updates that apply at plane p (bits 4-7 of cell_bits)
        const int vbits = (p >= 1 ? 48 : 0) | (p <= nz - 2 ? 64 : 0) | 128;
        const bool pface = p == 0 || p == nz - 1;
        const int sz = UZ ? s.az.slab(p) : -1;
        const bool zs = UZ && sz >= 0;
        float za = 0.f, zb = 0.f, zk = 1.f, zah = 0.f, zbh = 0.f, zkh = 1.f;
        if (zs) {
          za = __ldg(s.az.a + p); zb = __ldg(s.az.b + p); zk = __ldg(s.az.ik + p);
          zah = __ldg(s.az.ah + p); zbh = __ldg(s.az.bh + p); zkh = __ldg(s.az.ikh + p);
        }
        const long long mxp = (long long)p * ny * wx;
        const long long myp = (long long)p * wy * px;
        const long long mzp = (long long)sz * ny * px;
        const long long cpl = (long long)p * pl;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          if (!ov[q]) continue;
          const int i = oi, j = oj[q];
          const int b = b_own + q * 8 * BX, r = r_own + q * 8 * RX;
          const long long c = cpl + ofo[q];
          const bool hx = UX && omx[q] >= 0, hy = UY && omy[q] >= 0;
          const int mxi = omx[q], myi = omy[q], mzi = ofo[q];
          // the velocity sweep's memory variables and coefficients, issued together
          float qx3 = 0.f, qx4 = 0.f, qx5 = 0.f, qy3 = 0.f, qy4 = 0.f, qy5 = 0.f;
          float qz3 = 0.f, qz4 = 0.f, qz5 = 0.f;
          float xa = 0.f, xb = 0.f, xk = 1.f, xah = 0.f, xbh = 0.f, xkh = 1.f;
          float ya = 0.f, yb = 0.f, yk = 1.f, yah = 0.f, ybh = 0.f, ykh = 1.f;
          if (hx) {
            if (EARLY) { qx3 = e_vel[q][0]; qx4 = e_vel[q][1]; qx5 = e_vel[q][2]; }
            else { qx3 = (s.m.x[3] + mxp)[mxi]; qx4 = (s.m.x[4] + mxp)[mxi]; qx5 = (s.m.x[5] + mxp)[mxi]; }
            const float* cx = cfx + (i - i0 + 4);
            xa = cx[0]; xb = cx[BX]; xk = cx[2 * BX]; xah = cx[3 * BX]; xbh = cx[4 * BX]; xkh = cx[5 * BX];
          }
          if (hy) {
            if (EARLY) { qy3 = e_vel[q][0]; qy4 = e_vel[q][1]; qy5 = e_vel[q][2]; }
            else { qy3 = (s.m.y[3] + myp)[myi]; qy4 = (s.m.y[4] + myp)[myi]; qy5 = (s.m.y[5] + myp)[myi]; }
            const float* cy = cfy + (j - j0 + 1);
            ya = cy[0]; yb = cy[G::RY]; yk = cy[2 * G::RY]; yah = cy[3 * G::RY]; ybh = cy[4 * G::RY];
            ykh = cy[5 * G::RY];
          }
          if (zs) {
            if (EARLY) { qz3 = e_vel[q][0]; qz4 = e_vel[q][1]; qz5 = e_vel[q][2]; }
            else { qz3 = (s.m.z[3] + mzp)[mzi]; qz4 = (s.m.z[4] + mzp)[mzi]; qz5 = (s.m.z[5] + mzp)[mzi]; }
          }
          const float sxx = Sxx[r], syy = Syy[r], szz = Szz0[r];
          const float sxy = Sxy[r], sxz = Sxz0[r], syz = Syz0[r];
          float d1 = (sxx - Sxx[r - 1]) * s.odx;   // v_x (3D:976-993)
          float d2 = (sxy - Sxy[r - RX]) * s.ody;
          float d3 = (sxz - Sxzm[r]) * s.odz;
          float e1 = (Sxy[r + 1] - sxy) * s.odx;   // v_y (3D:995-1014)
          float e2 = (Syy[r + RX] - syy) * s.ody;
          float e3 = (syz - Syzm[r]) * s.odz;
          float f1 = (Sxz0[r + 1] - sxz) * s.odx;  // v_z (3D:1031-1052)
          float f2 = (syz - Syz0[r - RX]) * s.ody;
          float f3 = (Szz1[r] - szz) * s.odz;
          const int ok = edge ? (ocb[q] & vbits) : 112;
          const bool ux = ok & 16, uy = ok & 32, uz = ok & 64;
          // in place: updated where the component is (3D:979-985 and the like)
          auto psi = [&](float d, bool upd, float old, float* mm, int mi, float a_, float b_, float k_) {
            float nw = old;
            if (upd) { nw = b_ * old + a_ * d; mm[mi] = nw; }
            return d * k_ + nw;
          };
          if (hx) {
            d1 = psi(d1, ux, qx3, s.m.x[3] + mxp, mxi, xa, xb, xk);
            e1 = psi(e1, uy, qx4, s.m.x[4] + mxp, mxi, xah, xbh, xkh);
            f1 = psi(f1, uz, qx5, s.m.x[5] + mxp, mxi, xah, xbh, xkh);
          }
          if (hy) {
            d2 = psi(d2, ux, qy3, s.m.y[3] + myp, myi, ya, yb, yk);
            e2 = psi(e2, uy, qy4, s.m.y[4] + myp, myi, yah, ybh, ykh);
            f2 = psi(f2, uz, qy5, s.m.y[5] + myp, myi, ya, yb, yk);
          }
          if (zs) {
            d3 = psi(d3, ux, qz3, s.m.z[3] + mzp, mzi, za, zb, zk);
            e3 = psi(e3, uy, qz4, s.m.z[4] + mzp, mzi, za, zb, zk);
            f3 = psi(f3, uz, qz5, s.m.z[5] + mzp, mzi, zah, zbh, zkh);
          }
          float fx = s.dt_over_rho, fy = s.dt_over_rho, fz = s.dt_over_rho;
          if (HET) {
            fx = s.dt / R0[b];
            fy = s.dt / (0.25f * (R0[b] + R0[b + 1] + R0[b + 1 + BX] + R0[b + BX]));
            fz = s.dt / (0.25f * (R0[b] + R0[b + 1] + R1[b + 1] + R1[b]));
          }
          const float ox = cvx[q], oy = cvy[q], oz = cvz[q];
          float vx = ox + fx * (d1 + d2 + d3);
          float vy = oy + fy * (e1 + e2 + e3);
          float vz = oz + fz * (f1 + f2 + f3);
          if (edge) {
            if (!ux) vx = ox;
            if (!uy) vy = oy;
            if (!uz) vz = oz;
          }
          if (has_src && p == s.ksrc && i == s.isrc && j == s.jsrc) {  // 3D:1080-1081
            vx += src_x;
            vy += src_y;
          }
          if (edge && ((ok & 128) || pface)) {
            vx = 0.f; vy = 0.f; vz = 0.f;  // rigid faces (3D:1087-1121)
          }
          s.g.vx[c] = vx; s.g.vy[c] = vy; s.g.vz[c] = vz;
          const float v2 = vx * vx + vy * vy + vz * vz;
          vm2 = fmaxf(vm2, v2);
          bad |= not_finite(v2);
          if (e_z && oe[q]) {  // energy interior (3D:1136-1143)
            float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
            if (HET) {
              const float l = lms[(p & 3) * SLOT + b], mu = mus[(p & 7) * SLOT + b];
              const float den = 1.0f / (2.0f * mu * (3.0f * l + 2.0f * mu));
              hr = 0.5f * R0[b];
              c1 = 2.0f * (l + mu) * den;
              c2 = l * den;
              i2m = 1.0f / (2.0f * mu);
            }
            ek.add(hr * v2);
            const float exx = c1 * sxx - c2 * (syy + szz);
            const float eyy = c1 * syy - c2 * (sxx + szz);
            // the reference adds eps_yy*sigma_yy twice and no zz term (3D:1170-1171)
            const float third = s.ep_physical ? (c1 * szz - c2 * (sxx + syy)) * szz : eyy * syy;
            ep.add(0.5f * (exx * sxx + eyy * syy + third) + i2m * (sxy * sxy + sxz * sxz + syz * syz));
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) { cvx[q] = nvx[q]; cvy[q] = nvy[q]; cvz[q] = nvz[q]; }
  }
  if (!ok_all) {
    if (tid == 0) {
      atomicOr(s.err, 1);
      // let copies still in flight into this CTA's shared memory land
      for (int q = 0; q < 2; ++q) {
        mbar_wait_bounded(&bar[q], 0, kWaitCycles);
        mbar_wait_bounded(&bar[q], 1, kWaitCycles);
      }
    }
    __syncthreads();
  }
  block_partials<FNT>(ek.df(), ep.df(), vm2, bad, s.partials + ((size_t)ls * s.nblocks + blin) * 4);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// 3D map over one padded FP32 field: dims (nx, ny, nz), row pitch px floats;
// box (32 + 8) x (TY + 2) x 1; out-of-range elements read as zero.
static bool make_map(CUtensorMap* m, const float* base, int nx, int ny, int nz, int px, int ty,
                     CUtensorMapL2promotion promo) {
  EncodeTiledFn fn = encode_fn();
  if (!fn || !base) return false;
  cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  cuuint64_t strides[2] = {(cuuint64_t)px * 4, (cuuint64_t)px * ny * 4};
  cuuint32_t box[3] = {FTX + 8, (cuuint32_t)(ty + 2), 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, promo,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <int TY, int CLS, bool HET>
static cudaError_t set_smem_attr() {
  return cudaFuncSetAttribute(fused3d_kernel<TY, CLS, HET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)Geo<TY, HET>::SMEM);
}

struct FusedPlan {
  TmapSet maps[2];  // maps[q] reads buffer set q (interior kernel, ty-row boxes)
  TmapSet gmaps[2]; // the same for the general kernels' 8-row boxes
  int ty, lz, depth;
  bool het;
  const int4* items_fast;  // device item lists
  const int4* items_gen;   // general items, grouped by class X, Y, Z, GEN
  int n_fast, n_gen;
  int n_cls[4];            // general items of class X, Y, Z, GEN
  cudaStream_t aux[4];     // one stream per general class, forked from the step stream
  cudaEvent_t fork, join[4];
};

template <bool HET>
static cudaError_t set_attr_het(int ty) {
  cudaError_t e;
  if (ty == 8) {
    if ((e = set_smem_attr<8, CLS_INTERIOR, HET>()) != cudaSuccess) return e;
  } else if (ty == 16) {
    if ((e = set_smem_attr<16, CLS_INTERIOR, HET>()) != cudaSuccess) return e;
  } else {
    return cudaErrorInvalidValue;
  }
  if ((e = set_smem_attr<8, CLS_X, HET>()) != cudaSuccess) return e;
  if ((e = set_smem_attr<8, CLS_Y, HET>()) != cudaSuccess) return e;
  if ((e = set_smem_attr<8, CLS_Z, HET>()) != cudaSuccess) return e;
  return set_smem_attr<8, CLS_GEN, HET>();
}

static cudaError_t set_attr_for(int ty, bool het) { return het ? set_attr_het<true>(ty) : set_attr_het<false>(ty); }

bool fused3d_shape_ok(int ty, int d) { return (ty == 8 || ty == 16) && d == 2; }

bool fused3d_supported() { return encode_fn() != nullptr; }

size_t fused3d_smem(int ty, int d, bool het) {
  (void)d;
  if (ty == 8) return het ? Geo<8, true>::SMEM : Geo<8, false>::SMEM;
  return het ? Geo<16, true>::SMEM : Geo<16, false>::SMEM;
}

// Work items of one step: every (tile, z-chunk). A chunk is interior when its
// tile plus halo avoids every x/y slab, face and the energy boundary, and all
// its stress planes kb-1..ke avoid the z slabs and the z faces. Interior
// chunks are cut from the planes [zi0 + 1, zi1 - 1); the rest of each
// column, and every other tile, is general, cut at the same plane bounds so
// that a general chunk lies either inside or outside the z slabs. General
// items are grouped by class: X, Y or Z when the only C-PML slab they can
// touch is that axis's, GEN otherwise (n_cls gets the four counts). The
// z-chunk is the outermost loop so concurrently resident CTAs share their
// halos in L2.
void fused3d_items(int nx, int ny, int nz, const Axis& ax, const Axis& ay, const Axis& az, int npml,
                   int ty, int lz, bool het, std::vector<int4>& fast, std::vector<int4>& gen, int n_cls[4]) {
  (void)het;
  fast.clear();
  gen.clear();
  const int ntx = (nx + FTX - 1) / FTX, nty = (ny + ty - 1) / ty;
  const int zi0 = az.lo > 1 ? az.lo : 1;                              // first interior plane
  const int zi1 = (nz - az.hi) < (nz - 1) ? (nz - az.hi) : (nz - 1);  // one past the last
  const int f0 = zi0 + 1, f1 = zi1 - 1;
  // chunks of lz planes from the bottom of each range, the shorter
  // remainder last: the items that start last in the launch order finish
  // soonest, which shortens the step's tail (276^3: 0.4287 ms at lz = 40
  // against 0.4331 for the best even split)
  auto chunks = [&](int a, int b, std::vector<int2>& out) {
    for (int k0 = a; k0 < b; k0 += lz) out.push_back(make_int2(k0, k0 + lz < b ? k0 + lz : b));
  };
  auto interior_tile = [&](int i0, int j0) {
    const bool xs = ax.width() > 0 && (i0 - 1 < ax.lo || i0 + FTX >= nx - ax.hi);
    const bool ys = ay.width() > 0 && (j0 - 1 < ay.lo || j0 + ty >= ny - ay.hi);
    const bool edge = i0 - 1 < 1 || i0 + FTX > nx - 2 || j0 - 1 < 1 || j0 + ty > ny - 2;
    const bool efull = i0 >= npml && i0 + FTX <= nx - npml && j0 >= npml && j0 + ty <= ny - npml;
    return !xs && !ys && !edge && efull;
  };
  const bool has_inner = f1 > f0;
  std::vector<int2> all, inner, outer;
  if (has_inner) {
    chunks(0, f0, all);
    chunks(f0, f1, all);
    chunks(f1, nz, all);
    chunks(f0, f1, inner);
    chunks(0, f0, outer);
    chunks(f1, nz, outer);
  } else {
    chunks(0, nz, all);
  }
  // Interior tiles have ty rows; the general kernels always use 8-row tiles
  // (a smaller footprint gives them three CTAs per SM), which split every
  // ty-row tile exactly.
  for (const int2& z : inner)
    for (int tyi = 0; tyi < nty; ++tyi)
      for (int txi = 0; txi < ntx; ++txi)
        if (interior_tile(txi * FTX, tyi * ty)) fast.push_back(make_int4(txi * FTX, tyi * ty, z.x, z.y));
  std::vector<int4> cls[4];
  // the slab tests of the general kernel (xs_tile, ys_tile, z slab of planes kb-1..ke)
  auto add_gen = [&](int i0, int j0, const int2& z) {
    for (int jj = j0; jj < j0 + ty && jj < ny; jj += 8) {
      const bool xsl = ax.width() > 0 && (i0 - 1 < ax.lo || i0 + FTX >= nx - ax.hi);
      const bool ysl = ay.width() > 0 && (jj - 1 < ay.lo || jj + 8 >= ny - ay.hi);
      const int mlo = z.x - 1 > 0 ? z.x - 1 : 0, mhi = z.y < nz - 1 ? z.y : nz - 1;
      const bool zsl = az.width() > 0 && (mlo < az.lo || mhi >= nz - az.hi);
      const int k = (xsl ? 1 : 0) + (ysl ? 1 : 0) + (zsl ? 1 : 0);
      const int c = k != 1 ? 3 : (xsl ? 0 : (ysl ? 1 : 2));
      cls[c].push_back(make_int4(i0, jj, z.x, z.y));
    }
  };
  for (const int2& z : all)
    for (int tyi = 0; tyi < nty; ++tyi)
      for (int txi = 0; txi < ntx; ++txi)
        if (!has_inner || !interior_tile(txi * FTX, tyi * ty)) add_gen(txi * FTX, tyi * ty, z);
  for (const int2& z : outer)
    for (int tyi = 0; tyi < nty; ++tyi)
      for (int txi = 0; txi < ntx; ++txi)
        if (interior_tile(txi * FTX, tyi * ty)) add_gen(txi * FTX, tyi * ty, z);
  for (int c = 0; c < 4; ++c) {
    n_cls[c] = (int)cls[c].size();
    gen.insert(gen.end(), cls[c].begin(), cls[c].end());
  }
}

// Build the tensor maps of both buffer sets. fields[q][f] = field f of set q.
bool fused3d_make_maps(void* plan_mem, float* const fields[2][9], const float* lam, const float* mu,
                       const float* rho, int nx, int ny, int nz, int px, int ty, int lz, int depth,
                       bool het) {
  FusedPlan* P = static_cast<FusedPlan*>(plan_mem);
  P->ty = ty; P->lz = lz; P->depth = depth; P->het = het;
  // opt in to the dynamic shared memory once per configuration, outside any
  // stream capture
  if (set_attr_for(ty, het) != cudaSuccess || set_attr_for(8, het) != cudaSuccess) return false;
  for (int q = 0; q < 2; ++q)
    for (int pass = 0; pass < 2; ++pass) {
      TmapSet& M = pass == 0 ? P->maps[q] : P->gmaps[q];
      const int rows = pass == 0 ? ty : 8;
      // Interior boxes promote their L2 fills to whole 128-byte lines (the
      // neighbouring tiles read the rest of those lines at about the same
      // time); the general classes' neighbours are mostly interior tiles of
      // another kernel, so their halo columns fetch 64-byte pieces only.
      const CUtensorMapL2promotion promo =
          pass == 0 ? CU_TENSOR_MAP_L2_PROMOTION_L2_128B : CU_TENSOR_MAP_L2_PROMOTION_L2_64B;
      for (int f = 0; f < 9; ++f)
        if (!make_map(&M.f[f], fields[q][f], nx, ny, nz, px, rows, promo)) return false;
      if (het) {
        if (!make_map(&M.lam, lam, nx, ny, nz, px, rows, promo)) return false;
        if (!make_map(&M.mu, mu, nx, ny, nz, px, rows, promo)) return false;
        if (!make_map(&M.rho, rho, nx, ny, nz, px, rows, promo)) return false;
      } else {
        M.lam = M.f[0];
        M.mu = M.f[0];
        M.rho = M.f[0];
      }
    }
  return true;
}

void fused3d_set_items(void* plan_mem, const int4* fast, int n_fast, const int4* gen, const int n_cls[4],
                       const cudaStream_t aux[4], cudaEvent_t fork, const cudaEvent_t join[4]) {
  FusedPlan* P = static_cast<FusedPlan*>(plan_mem);
  P->items_fast = fast; P->n_fast = n_fast;
  P->items_gen = gen;
  P->n_gen = 0;
  for (int c = 0; c < 4; ++c) {
    P->n_cls[c] = n_cls[c];
    P->n_gen += n_cls[c];
    P->aux[c] = aux[c];
    P->join[c] = join[c];
  }
  P->fork = fork;
}

size_t fused3d_plan_bytes() { return sizeof(FusedPlan); }

int fused3d_kernels_per_step(const void* plan_mem) {
  const FusedPlan* P = static_cast<const FusedPlan*>(plan_mem);
  int n = P->n_fast > 0 ? 1 : 0;
  for (int c = 0; c < 4; ++c) n += P->n_cls[c] > 0 ? 1 : 0;
  return n;
}

template <int TY, bool HET>
static void launch_classes(const FusedPlan* P, const StepArgs& s, int ls, int parity, cudaStream_t st) {
  const size_t smf = Geo<TY, HET>::SMEM, smg = Geo<8, HET>::SMEM;
  // Every general class runs on its own auxiliary stream, concurrently with
  // the interior items on the step stream (forked and joined with events, so
  // a captured graph holds the same fan-out). Exactly one kernel records the
  // receivers: the first class with items, or the interior kernel.
  int recorder = -1;
  for (int c = 0; c < 4 && recorder < 0; ++c)
    if (P->n_cls[c] > 0) recorder = c;
  if (P->n_gen > 0) {
    cudaEventRecord(P->fork, st);
    int off = 0;
    for (int c = 0; c < 4; ++c) {
      const int n = P->n_cls[c];
      if (n > 0) {
        cudaStreamWaitEvent(P->aux[c], P->fork, 0);
        const int4* it = P->items_gen + off;
        const int base = P->n_fast + off, rec = c == recorder ? 1 : 0;
        cudaStream_t sc = P->aux[c];
        if (c == 0) fused3d_kernel<8, CLS_X, HET><<<n, FNT, smg, sc>>>(P->gmaps[parity], s, ls, it, base, rec);
        if (c == 1) fused3d_kernel<8, CLS_Y, HET><<<n, FNT, smg, sc>>>(P->gmaps[parity], s, ls, it, base, rec);
        if (c == 2) fused3d_kernel<8, CLS_Z, HET><<<n, FNT, smg, sc>>>(P->gmaps[parity], s, ls, it, base, rec);
        if (c == 3) fused3d_kernel<8, CLS_GEN, HET><<<n, FNT, smg, sc>>>(P->gmaps[parity], s, ls, it, base, rec);
      }
      off += n;
    }
  }
  if (P->n_fast > 0)
    fused3d_kernel<TY, CLS_INTERIOR, HET><<<P->n_fast, FNT, smf, st>>>(P->maps[parity], s, ls, P->items_fast, 0,
                                                                       recorder < 0 ? 1 : 0);
  for (int c = 0; c < 4; ++c)
    if (P->n_cls[c] > 0) {
      cudaEventRecord(P->join[c], P->aux[c]);
      cudaStreamWaitEvent(st, P->join[c], 0);
    }
}

template <int TY>
static cudaError_t launch_t(const FusedPlan* P, const StepArgs& s, int ls, int parity, cudaStream_t st) {
  if (P->het)
    launch_classes<TY, true>(P, s, ls, parity, st);
  else
    launch_classes<TY, false>(P, s, ls, parity, st);
  return cudaGetLastError();
}

cudaError_t fused3d_launch(const void* plan_mem, const StepArgs& s, int ls, int parity, cudaStream_t st) {
  const FusedPlan* P = static_cast<const FusedPlan*>(plan_mem);
  if (P->ty == 8) return launch_t<8>(P, s, ls, parity, st);
  if (P->ty == 16) return launch_t<16>(P, s, ls, parity, st);
  return cudaErrorInvalidValue;
}

}  // namespace cpml
