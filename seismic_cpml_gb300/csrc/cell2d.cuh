// cell2d.cuh -- the per-cell 2D velocity-stress C-PML update, shared by the
// single-shot kernels (kernels2d.cu) and the batched multi-shot engine
// (batch2d.cu) so both compute bit-identical results.
//
// Follows seismic_CPML_2D_isotropic_second_order.f90: sigma_xx/sigma_yy
// (2D:556-580), sigma_xy (2D:582-600), v_x (2D:606-621), v_y (2D:623-641),
// source (2D:644-667), rigid edges (2D:670-680), energy (2D:694-713).
#pragma once
#include "cpml_internal.cuh"
#include "kutil.cuh"

namespace cpml {

// Every rounding step is spelled out (fmaf, __fmul_rn, __fadd_rn are never
// re-associated or contracted by the compiler), so the single-shot and the
// batched kernels produce the same bits whatever code surrounds the inlined
// cell update.
__device__ __forceinline__ float pml2(float d, int sidx, float* __restrict__ mem, long long midx,
                                      const float* __restrict__ a, const float* __restrict__ b,
                                      const float* __restrict__ ik, int idx) {
  if (sidx < 0) return d;
  const float m = fmaf(__ldg(b + idx), mem[midx], __fmul_rn(__ldg(a + idx), d));  // 2D:574-575
  mem[midx] = m;
  return fmaf(d, __ldg(ik + idx), m);                                            // 2D:577-578
}

// pml2 with the memory variable's old value already loaded (old); the same
// arithmetic.
__device__ __forceinline__ float pml2v(float d, int sidx, float old, float* __restrict__ mem, long long midx,
                                       const float* __restrict__ a, const float* __restrict__ b,
                                       const float* __restrict__ ik, int idx) {
  if (sidx < 0) return d;
  const float m = fmaf(__ldg(b + idx), old, __fmul_rn(__ldg(a + idx), d));  // 2D:574-575
  mem[midx] = m;
  return fmaf(d, __ldg(ik + idx), m);                                      // 2D:577-578
}

// Everything one 2D shot's cell updates read or write.
struct Shot2D {
  int nx, ny, px;              // grid and row pitch (floats)
  int npml;                    // energy interior [npml, n - npml)
  int het;                     // per-cell model present
  float odx, ody, dt;
  float dt_lam, dt_mu, dt_l2m, dt_over_rho;   // homogeneous model (het == 0)
  float half_rho, inv_2mu, e_c1, e_c2;        // homogeneous energy constants
  const float* lam;
  const float* mu;
  const float* rho;
  float* vx; float* vy; float* sxx; float* syy; float* sxy;
  Axis ax, ay;
  float* mx[4];                // x slab: dvx_dx dvy_dx | dsxx_dx dsxy_dx, [j][sx]
  float* my[4];                // y slab: dvx_dy dvy_dy | dsxy_dy dsyy_dy, [sy][i]
  int isrc, jsrc;              // 0-based source cell
  const float* src_fx;         // per-step velocity increments at the source
  const float* src_fy;
};

// Where a cell update finds the fields, the per-cell model and the memory
// variables it touches. GlobalView is a shot's own arrays in HBM; a kernel
// that stages a region in shared memory supplies its own view. The update
// functions below are the same source for every view, so the arithmetic
// (and every rounding) is identical wherever the state lives.
struct GlobalView {
  const Shot2D& s;
  __device__ __forceinline__ float* vx() const { return s.vx; }
  __device__ __forceinline__ float* vy() const { return s.vy; }
  __device__ __forceinline__ float* sxx() const { return s.sxx; }
  __device__ __forceinline__ float* syy() const { return s.syy; }
  __device__ __forceinline__ float* sxy() const { return s.sxy; }
  __device__ __forceinline__ const float* lam() const { return s.lam; }
  __device__ __forceinline__ const float* mu() const { return s.mu; }
  __device__ __forceinline__ const float* rho() const { return s.rho; }
  __device__ __forceinline__ float* mx(int q) const { return s.mx[q]; }
  __device__ __forceinline__ float* my(int q) const { return s.my[q]; }
  __device__ __forceinline__ long long pitch() const { return s.px; }
  __device__ __forceinline__ long long at(int i, int j) const { return (long long)j * s.px + i; }
  __device__ __forceinline__ long long mxi(int i, int j, int sx) const {
    (void)i;
    return (long long)j * s.ax.width() + sx;
  }
  __device__ __forceinline__ long long myi(int i, int j, int sy) const {
    (void)j;
    return (long long)sy * s.px + i;
  }
};

// Stress update of cell (i, j), 0-based, in two halves: stress2d_load
// issues every load of the cell (fields, memory variables, per-cell model),
// stress2d_store computes and stores. The arrays never overlap, but the
// compiler cannot know that and would hold each load behind the stores
// before it; with the loads first, one memory latency covers the cell (or,
// in a kernel that loads two cells before storing either, both cells). The
// arithmetic does not depend on the order.
struct StressIn {
  int sx, sy;
  long long c, mx, my;
  bool un, us;   // sigma_xx/yy and sigma_xy updated
  float vxc, vyc, vxe, vys, oxx, oyy, vyw, vxn, oxy;
  float qx0, qy1, qx1, qy0;
  float l0, l1, m0, m1, mn;
};
template <bool HET, class V>
__device__ __forceinline__ StressIn stress2d_load(const Shot2D& s, const V& v, int i, int j) {
  StressIn r;
  r.sx = s.ax.slab(i); r.sy = s.ay.slab(j);
  const long long px = v.pitch();
  r.c = v.at(i, j);
  r.mx = v.mxi(i, j, r.sx);
  r.my = v.myi(i, j, r.sy);
  const long long c = r.c;
  const float* const VX = v.vx();
  const float* const VY = v.vy();
  r.un = j >= 1 && i <= s.nx - 2;  // sigma_xx, sigma_yy: j = 2..NY, i = 1..NX-1
  r.us = j <= s.ny - 2 && i >= 1;  // sigma_xy: j = 1..NY-1, i = 2..NX
  r.vxc = VX[c]; r.vyc = VY[c];
  r.vxe = r.vys = r.oxx = r.oyy = r.vyw = r.vxn = r.oxy = 0.f;
  r.qx0 = r.qy1 = r.qx1 = r.qy0 = 0.f;
  r.l0 = r.l1 = r.m0 = r.m1 = r.mn = 0.f;
  if (r.un) {
    r.vxe = VX[c + 1]; r.vys = VY[c - px]; r.oxx = v.sxx()[c]; r.oyy = v.syy()[c];
    if (r.sx >= 0) r.qx0 = v.mx(0)[r.mx];
    if (r.sy >= 0) r.qy1 = v.my(1)[r.my];
    if (HET) { r.l1 = v.lam()[c + 1]; r.l0 = v.lam()[c]; r.m1 = v.mu()[c + 1]; }
  }
  if (r.us) {
    r.vyw = VY[c - 1]; r.vxn = VX[c + px]; r.oxy = v.sxy()[c];
    if (r.sx >= 0) r.qx1 = v.mx(1)[r.mx];
    if (r.sy >= 0) r.qy0 = v.my(0)[r.my];
    if (HET) r.mn = v.mu()[c + px];
  }
  if (HET && (r.un || r.us)) r.m0 = v.mu()[c];
  return r;
}
template <bool HET, class V>
__device__ __forceinline__ void stress2d_store(const Shot2D& s, const V& v, int i, int j, const StressIn& r) {
  const long long c = r.c;
  if (r.un) {
    float d1 = __fmul_rn(__fsub_rn(r.vxe, r.vxc), s.odx);
    float d2 = __fmul_rn(__fsub_rn(r.vyc, r.vys), s.ody);
    d1 = pml2v(d1, r.sx, r.qx0, v.mx(0), r.mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml2v(d2, r.sy, r.qy1, v.my(1), r.my, s.ay.a, s.ay.b, s.ay.ik, j);
    float dl = s.dt_lam, dl2m = s.dt_l2m;
    if (HET) {
      const float lh = __fmul_rn(0.5f, __fadd_rn(r.l1, r.l0));
      const float mh = __fmul_rn(0.5f, __fadd_rn(r.m1, r.m0));
      dl = __fmul_rn(s.dt, lh);
      dl2m = __fmul_rn(s.dt, fmaf(2.0f, mh, lh));
    }
    v.sxx()[c] = __fadd_rn(r.oxx, fmaf(dl2m, d1, __fmul_rn(dl, d2)));
    v.syy()[c] = __fadd_rn(r.oyy, fmaf(dl, d1, __fmul_rn(dl2m, d2)));
  }
  if (r.us) {
    float d1 = __fmul_rn(__fsub_rn(r.vyc, r.vyw), s.odx);
    float d2 = __fmul_rn(__fsub_rn(r.vxn, r.vxc), s.ody);
    d1 = pml2v(d1, r.sx, r.qx1, v.mx(1), r.mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml2v(d2, r.sy, r.qy0, v.my(0), r.my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
    const float dm = HET ? __fmul_rn(s.dt, __fmul_rn(0.5f, __fadd_rn(r.mn, r.m0))) : s.dt_mu;
    v.sxy()[c] = fmaf(dm, __fadd_rn(d1, d2), r.oxy);
  }
}
template <bool HET, class V>
__device__ __forceinline__ void stress2d_cell(const Shot2D& s, const V& v, int i, int j) {
  stress2d_store<HET>(s, v, i, j, stress2d_load<HET>(s, v, i, j));
}

template <bool HET>
__device__ __forceinline__ void stress2d_cell(const Shot2D& s, int i, int j) {
  stress2d_cell<HET>(s, GlobalView{s}, i, j);
}

// Velocity update of cell (i, j) at 1-based step it, with source, rigid
// edges, and the cell's energy and |v|^2 contributions; split into loads
// and the rest as the stress update is.
struct VelocityIn {
  int sx, sy;
  long long c, mx, my;
  bool ux, uy, en;   // v_x, v_y updated; cell inside the energy interior
  float vx, vy, sxx, syy, sxy, sxw, sys, sye, syn;
  float qx2, qy2, qx3, qy3;
  float r0, r1, r1n, rn, lc, mc;
};
template <bool HET, class V>
__device__ __forceinline__ VelocityIn velocity2d_load(const Shot2D& s, const V& v, int i, int j) {
  VelocityIn r;
  r.sx = s.ax.slab(i); r.sy = s.ay.slab(j);
  const long long px = v.pitch();
  r.c = v.at(i, j);
  r.mx = v.mxi(i, j, r.sx);
  r.my = v.myi(i, j, r.sy);
  const long long c = r.c;
  const float* const SXX = v.sxx();
  const float* const SYY = v.syy();
  const float* const SXY = v.sxy();
  r.ux = j >= 1 && i >= 1;                  // v_x: j = 2..NY, i = 2..NX
  r.uy = j <= s.ny - 2 && i <= s.nx - 2;    // v_y: j = 1..NY-1, i = 1..NX-1
  const int n0 = s.npml;
  r.en = i >= n0 && i < s.nx - n0 && j >= n0 && j < s.ny - n0;
  r.vx = v.vx()[c]; r.vy = v.vy()[c];
  r.sxx = SXX[c]; r.syy = SYY[c]; r.sxy = SXY[c];
  r.sxw = r.sys = r.sye = r.syn = 0.f;
  r.qx2 = r.qy2 = r.qx3 = r.qy3 = 0.f;
  r.r0 = r.r1 = r.r1n = r.rn = r.lc = r.mc = 0.f;
  if (r.ux) {
    r.sxw = SXX[c - 1]; r.sys = SXY[c - px];
    if (r.sx >= 0) r.qx2 = v.mx(2)[r.mx];
    if (r.sy >= 0) r.qy2 = v.my(2)[r.my];
  }
  if (r.uy) {
    r.sye = SXY[c + 1]; r.syn = SYY[c + px];
    if (r.sx >= 0) r.qx3 = v.mx(3)[r.mx];
    if (r.sy >= 0) r.qy3 = v.my(3)[r.my];
    if (HET) { r.r1 = v.rho()[c + 1]; r.r1n = v.rho()[c + 1 + px]; r.rn = v.rho()[c + px]; }
  }
  if (HET) {
    if (r.ux || r.uy || r.en) r.r0 = v.rho()[c];
    if (r.en) { r.lc = v.lam()[c]; r.mc = v.mu()[c]; }
  }
  return r;
}
template <bool HET, class V>
__device__ __forceinline__ void velocity2d_store(const Shot2D& s, const V& v, int i, int j, int it,
                                                 const VelocityIn& r, float& ek, float& ep, float& vm2, int& bad) {
  const long long c = r.c;
  float vx = r.vx, vy = r.vy;
  if (r.ux) {
    float d1 = __fmul_rn(__fsub_rn(r.sxx, r.sxw), s.odx);
    float d2 = __fmul_rn(__fsub_rn(r.sxy, r.sys), s.ody);
    d1 = pml2v(d1, r.sx, r.qx2, v.mx(2), r.mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml2v(d2, r.sy, r.qy2, v.my(2), r.my, s.ay.a, s.ay.b, s.ay.ik, j);
    const float f = HET ? __fdiv_rn(s.dt, r.r0) : s.dt_over_rho;
    vx = fmaf(__fadd_rn(d1, d2), f, vx);
  }
  if (r.uy) {
    float d1 = __fmul_rn(__fsub_rn(r.sye, r.sxy), s.odx);
    float d2 = __fmul_rn(__fsub_rn(r.syn, r.syy), s.ody);
    d1 = pml2v(d1, r.sx, r.qx3, v.mx(3), r.mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml2v(d2, r.sy, r.qy3, v.my(3), r.my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
    float f = s.dt_over_rho;
    if (HET) {
      const float r4 = __fadd_rn(__fadd_rn(__fadd_rn(r.r0, r.r1), r.r1n), r.rn);
      f = __fdiv_rn(s.dt, __fmul_rn(0.25f, r4));
    }
    vy = fmaf(__fadd_rn(d1, d2), f, vy);
  }
  if (i == s.isrc && j == s.jsrc) {  // 2D:664-667
    vx = __fadd_rn(vx, s.src_fx[it - 1]);
    vy = __fadd_rn(vy, s.src_fy[it - 1]);
  }
  if (i == 0 || i == s.nx - 1 || j == 0 || j == s.ny - 1) { vx = 0.f; vy = 0.f; }  // 2D:670-680
  v.vx()[c] = vx;
  v.vy()[c] = vy;
  const float v2 = vx * vx + vy * vy;
  vm2 = fmaxf(vm2, v2);
  bad |= not_finite(v2);
  if (r.en) {
    float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
    if (HET) {
      const float l = r.lc, m = r.mc;
      const float den = 1.0f / (4.0f * m * (l + m));
      hr = 0.5f * r.r0;
      c1 = (l + 2.0f * m) * den;
      c2 = l * den;
      i2m = 1.0f / (2.0f * m);
    }
    ek += hr * v2;
    const float sxx = r.sxx, syy = r.syy, sxy = r.sxy;
    const float exx = c1 * sxx - c2 * syy;
    const float eyy = c1 * syy - c2 * sxx;
    ep += 0.5f * (exx * sxx + eyy * syy) + i2m * (sxy * sxy);
  }
}
template <bool HET, class V>
__device__ __forceinline__ void velocity2d_cell(const Shot2D& s, const V& v, int i, int j, int it, float& ek,
                                                float& ep, float& vm2, int& bad) {
  velocity2d_store<HET>(s, v, i, j, it, velocity2d_load<HET>(s, v, i, j), ek, ep, vm2, bad);
}

template <bool HET>
__device__ __forceinline__ void velocity2d_cell(const Shot2D& s, int i, int j, int it, float& ek, float& ep,
                                                float& vm2, int& bad) {
  velocity2d_cell<HET>(s, GlobalView{s}, i, j, it, ek, ep, vm2, bad);
}

// View of a single-shot handle's state as a Shot2D.
__device__ __forceinline__ Shot2D shot_from_args(const StepArgs& a) {
  Shot2D s;
  s.nx = a.nx; s.ny = a.ny; s.px = a.px; s.npml = a.npml; s.het = a.mdl.rho != nullptr;
  s.odx = a.odx; s.ody = a.ody; s.dt = a.dt;
  s.dt_lam = a.dt_lam; s.dt_mu = a.dt_mu; s.dt_l2m = a.dt_l2m; s.dt_over_rho = a.dt_over_rho;
  s.half_rho = a.half_rho; s.inv_2mu = a.inv_2mu; s.e_c1 = a.e_c1; s.e_c2 = a.e_c2;
  s.lam = a.mdl.lam; s.mu = a.mdl.mu; s.rho = a.mdl.rho;
  s.vx = a.f.vx; s.vy = a.f.vy; s.sxx = a.f.sxx; s.syy = a.f.syy; s.sxy = a.f.sxy;
  s.ax = a.ax; s.ay = a.ay;
  for (int q = 0; q < 4; ++q) { s.mx[q] = a.m.x[q]; s.my[q] = a.m.y[q]; }
  s.isrc = a.isrc; s.jsrc = a.jsrc; s.src_fx = a.src_fx; s.src_fy = a.src_fy;
  return s;
}

}  // namespace cpml
