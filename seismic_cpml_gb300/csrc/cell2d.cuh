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

// Stress update of cell (i, j), 0-based.
template <bool HET, class V>
__device__ __forceinline__ void stress2d_cell(const Shot2D& s, const V& v, int i, int j) {
  const int sx = s.ax.slab(i), sy = s.ay.slab(j);
  const long long px = v.pitch();
  const long long c = v.at(i, j);
  const long long mx = v.mxi(i, j, sx);
  const long long my = v.myi(i, j, sy);
  float* const VX = v.vx();
  float* const VY = v.vy();
  const float vxc = VX[c], vyc = VY[c];
  // sigma_xx, sigma_yy: j = 2..NY, i = 1..NX-1
  if (j >= 1 && i <= s.nx - 2) {
    float d1 = __fmul_rn(__fsub_rn(VX[c + 1], vxc), s.odx);
    float d2 = __fmul_rn(__fsub_rn(vyc, VY[c - px]), s.ody);
    d1 = pml2(d1, sx, v.mx(0), mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml2(d2, sy, v.my(1), my, s.ay.a, s.ay.b, s.ay.ik, j);
    float dl = s.dt_lam, dl2m = s.dt_l2m;
    if (HET) {
      const float lh = __fmul_rn(0.5f, __fadd_rn(v.lam()[c + 1], v.lam()[c]));
      const float mh = __fmul_rn(0.5f, __fadd_rn(v.mu()[c + 1], v.mu()[c]));
      dl = __fmul_rn(s.dt, lh);
      dl2m = __fmul_rn(s.dt, fmaf(2.0f, mh, lh));
    }
    float* const SXX = v.sxx();
    float* const SYY = v.syy();
    SXX[c] = __fadd_rn(SXX[c], fmaf(dl2m, d1, __fmul_rn(dl, d2)));
    SYY[c] = __fadd_rn(SYY[c], fmaf(dl, d1, __fmul_rn(dl2m, d2)));
  }
  // sigma_xy: j = 1..NY-1, i = 2..NX
  if (j <= s.ny - 2 && i >= 1) {
    float d1 = __fmul_rn(__fsub_rn(vyc, VY[c - 1]), s.odx);
    float d2 = __fmul_rn(__fsub_rn(VX[c + px], vxc), s.ody);
    d1 = pml2(d1, sx, v.mx(1), mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml2(d2, sy, v.my(0), my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
    const float dm = HET ? __fmul_rn(s.dt, __fmul_rn(0.5f, __fadd_rn(v.mu()[c + px], v.mu()[c]))) : s.dt_mu;
    float* const SXY = v.sxy();
    SXY[c] = fmaf(dm, __fadd_rn(d1, d2), SXY[c]);
  }
}

template <bool HET>
__device__ __forceinline__ void stress2d_cell(const Shot2D& s, int i, int j) {
  stress2d_cell<HET>(s, GlobalView{s}, i, j);
}

// Velocity update of cell (i, j) at 1-based step it, with source, rigid
// edges, and the cell's energy and |v|^2 contributions.
template <bool HET, class V>
__device__ __forceinline__ void velocity2d_cell(const Shot2D& s, const V& v, int i, int j, int it, float& ek,
                                                float& ep, float& vm2, int& bad) {
  const int sx = s.ax.slab(i), sy = s.ay.slab(j);
  const long long px = v.pitch();
  const long long c = v.at(i, j);
  const long long mx = v.mxi(i, j, sx);
  const long long my = v.myi(i, j, sy);
  float* const VX = v.vx();
  float* const VY = v.vy();
  const float* const SXX = v.sxx();
  const float* const SYY = v.syy();
  const float* const SXY = v.sxy();
  float vx = VX[c], vy = VY[c];
  const float sxx = SXX[c], syy = SYY[c], sxy = SXY[c];
  // v_x: j = 2..NY, i = 2..NX
  if (j >= 1 && i >= 1) {
    float d1 = __fmul_rn(__fsub_rn(sxx, SXX[c - 1]), s.odx);
    float d2 = __fmul_rn(__fsub_rn(sxy, SXY[c - px]), s.ody);
    d1 = pml2(d1, sx, v.mx(2), mx, s.ax.a, s.ax.b, s.ax.ik, i);
    d2 = pml2(d2, sy, v.my(2), my, s.ay.a, s.ay.b, s.ay.ik, j);
    const float f = HET ? __fdiv_rn(s.dt, v.rho()[c]) : s.dt_over_rho;
    vx = fmaf(__fadd_rn(d1, d2), f, vx);
  }
  // v_y: j = 1..NY-1, i = 1..NX-1
  if (j <= s.ny - 2 && i <= s.nx - 2) {
    float d1 = __fmul_rn(__fsub_rn(SXY[c + 1], sxy), s.odx);
    float d2 = __fmul_rn(__fsub_rn(SYY[c + px], syy), s.ody);
    d1 = pml2(d1, sx, v.mx(3), mx, s.ax.ah, s.ax.bh, s.ax.ikh, i);
    d2 = pml2(d2, sy, v.my(3), my, s.ay.ah, s.ay.bh, s.ay.ikh, j);
    float f = s.dt_over_rho;
    if (HET) {
      const float* r = v.rho();
      const float r4 = __fadd_rn(__fadd_rn(__fadd_rn(r[c], r[c + 1]), r[c + 1 + px]), r[c + px]);
      f = __fdiv_rn(s.dt, __fmul_rn(0.25f, r4));
    }
    vy = fmaf(__fadd_rn(d1, d2), f, vy);
  }
  if (i == s.isrc && j == s.jsrc) {  // 2D:664-667
    vx = __fadd_rn(vx, s.src_fx[it - 1]);
    vy = __fadd_rn(vy, s.src_fy[it - 1]);
  }
  if (i == 0 || i == s.nx - 1 || j == 0 || j == s.ny - 1) { vx = 0.f; vy = 0.f; }  // 2D:670-680
  VX[c] = vx;
  VY[c] = vy;
  const float v2 = vx * vx + vy * vy;
  vm2 = fmaxf(vm2, v2);
  bad |= not_finite(v2);
  const int n0 = s.npml;
  if (i >= n0 && i < s.nx - n0 && j >= n0 && j < s.ny - n0) {
    float hr = s.half_rho, c1 = s.e_c1, c2 = s.e_c2, i2m = s.inv_2mu;
    if (HET) {
      const float l = v.lam()[c], m = v.mu()[c];
      const float den = 1.0f / (4.0f * m * (l + m));
      hr = 0.5f * v.rho()[c];
      c1 = (l + 2.0f * m) * den;
      c2 = l * den;
      i2m = 1.0f / (2.0f * m);
    }
    ek += hr * v2;
    const float exx = c1 * sxx - c2 * syy;
    const float eyy = c1 * syy - c2 * sxx;
    ep += 0.5f * (exx * sxx + eyy * syy) + i2m * (sxy * sxy);
  }
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
