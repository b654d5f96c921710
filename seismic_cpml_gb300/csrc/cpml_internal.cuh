// cpml_internal.cuh -- device-side state layout shared by the kernels and the
// host runtime of libcpml.
//
// HBM layout
//   - Wavefields and per-cell model: one FP32 array per quantity, C order
//     [k][j][i], row pitch px = nx rounded up to 32 floats so every row starts
//     on a 128-byte line (coalesced rows, TMA-legal strides).
//   - C-PML memory variables: stored only where their coefficient a is
//     nonzero, i.e. in the PML slab of the axis they belong to. Outside its
//     slab a memory variable is identically zero (a = 0 keeps psi = b*0 = 0,
//     2D:327-394), so the slab store is exact.
//       x slab: [k][j][sx], sx < wx   (wx = slab points on x, both sides)
//       y slab: [k][sy][i], row pitch px
//       z slab: [sz][j][i], row pitch px
//   - 1-D profile tables a, b, 1/K at grid and half points, FP32, built in
//     FP64 on the GPU and rounded once.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cpml {

// One axis of C-PML coefficients (device pointers).
struct Axis {
  const float* a;    // a at grid points
  const float* b;    // b at grid points
  const float* ik;   // 1/K at grid points
  const float* ah;   // a at half points (i + 1/2)
  const float* bh;
  const float* ikh;
  int n;             // points on the axis
  int lo;            // slab points on the low side   [0, lo)
  int hi;            // slab points on the high side  [n - hi, n)
  __host__ __device__ int width() const { return lo + hi; }
  // slab index of grid index i, or -1 outside the slab
  __host__ __device__ int slab(int i) const {
    return i < lo ? i : (i >= n - hi ? lo + (i - (n - hi)) : -1);
  }
};

// Memory variables of one axis: 6 in 3D (3 for the stress sweep, 3 for the
// velocity sweep), 4 in 2D.
//   x: dvx_dx dvy_dx dvz_dx | dsxx_dx dsxy_dx dsxz_dx
//   y: dvx_dy dvy_dy dvz_dy | dsxy_dy dsyy_dy dsyz_dy
//   z: dvx_dz dvy_dz dvz_dz | dsxz_dz dsyz_dz dszz_dz
//   2D x: dvx_dx dvy_dx | dsxx_dx dsxy_dx ; 2D y: dvx_dy dvy_dy | dsxy_dy dsyy_dy
struct Slabs {
  float* x[6];
  float* y[6];
  float* z[6];
};

struct Fields {
  float* vx; float* vy; float* vz;
  float* sxx; float* syy; float* szz;
  float* sxy; float* sxz; float* syz;
};

struct Model {        // per-cell model (nullptr = homogeneous scalars)
  const float* lam;
  const float* mu;
  const float* rho;
};

// Everything a time-step kernel needs; passed by value.
struct StepArgs {
  int nx, ny, nz;          // grid (nz = 1 in 2D)
  int px;                  // row pitch in floats
  long long plane;         // px * ny
  float odx, ody, odz;     // 1/DELTA (3D) ...
  float dx, dy;            // ... and DELTA (2D divides, 2D:573-574)
  float dt;
  // homogeneous model, pre-multiplied by dt (3D:296-300)
  float dt_lam, dt_mu, dt_l2m, dt_over_rho;
  // energy constants (homogeneous)
  float half_rho, inv_2mu, e_c1, e_c2;   // see kernels
  Axis ax, ay, az;
  Slabs m;                 // memory variables (stress-side: time-n copy when ping-ponged)
  Slabs mb;                // stress-side memory variables, time n+1 copy (fused path)
  Fields f;                // wavefields read this step (time n)
  Fields g;                // wavefields written this step (fused path; == f in place)
  Model mdl;
  int npml;                // energy interior: [npml, n-npml) on every axis
  int isrc, jsrc, ksrc;    // 0-based source cell
  const float* src_fx;     // per-step velocity increments at the source, [nstep]
  const float* src_fy;
  int nrec;
  const int* rec_cell;     // [nrec] linear padded cell index
  float* seis;             // [3][nrec][nstep] FP32 samples
  int nstep;
  const int* it_base;      // device counter: steps completed before this chunk
  double* partials;        // [chunk][nblocks][4]: ek, ep, vmax^2, nan
  int nblocks;             // blocks of the velocity kernel
  int ep_physical;         // 3D: textbook Ep instead of the reference's
  int* err;                // device error word (bounded waits that gave up)
  float o24dx, o24dy;      // 2D fourth order: 1 / (24 DELTA) (2D4:565-566)
  int split;               // 2D split-field PML: f holds the x parts, g the y parts
  float lam_split, mu_split, l2m_split, orho_split;  // its homogeneous model (PML:106-111)
};

// Inputs of the FP64 C-PML profile builder of one axis (support.cu).
struct ProfileArgs {
  int n, npml, use_min, use_max;
  int high_cells;  // high-side origin = high_cells * delta - thickness (n - 1; n on the
                   // y axis of the fourth-order program, 2D4:401)
  double delta, cp, f0, dt, npower, kmax, amax, rcoef;
};

// On-chip layout of a small 2D grid held by one thread-block cluster
// (cluster2d.cu); ncl = 0 when the grid does not fit.
struct ClusterLayout {
  int ncl;        // CTAs in the cluster (rows split into ncl bands)
  int rows;       // own rows per CTA (the last one may have fewer)
  int pitch;      // shared-memory row pitch (floats)
  int ysl;        // y-slab rows a CTA can own
  int het;
  size_t smem;    // dynamic shared memory per CTA
};

// Linear index helpers
__host__ __device__ inline long long cell3(const StepArgs& s, int i, int j, int k) {
  return (long long)k * s.plane + (long long)j * s.px + i;
}

}  // namespace cpml
