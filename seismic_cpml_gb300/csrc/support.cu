// support.cu -- set-up and bookkeeping kernels of libcpml.
//
//   build_profile_kernel  FP64 C-PML profile of one axis on the GPU
//                         (2D:283-465, 3D:399-667), rounded once to the FP32
//                         tables a, b, 1/K the stencil kernels read.
//   reduce_chunk_kernel   second stage of the deterministic FP64 reductions:
//                         per-block partials of each step of a chunk summed in
//                         a fixed order into Ek, Ep (2D:694-713, 3D:1131-1180)
//                         and max|v| (2D:718, 3D:1185); also records the
//                         receivers of the chunk's last step.
//   advance_kernel        moves the device step counter on by one chunk.
#include <cuda_runtime.h>
#include "cpml_internal.cuh"
#include "kutil.cuh"

namespace cpml {


// One thread per grid index: full point and half point.
__global__ void build_profile_kernel(ProfileArgs P, double* __restrict__ out64,
                                     float* __restrict__ out32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double th = P.npml * P.delta;
  const double d0 = -(P.npower + 1) * P.cp * log(P.rcoef) / (2.0 * th);
  const double ol = th, orr = P.high_cells * P.delta - th;
  const double val = P.delta * double(i);
  double d = 0, K = 1, al = 0, dh = 0, Kh = 1, alh = 0;
  if (P.use_min) {
    double ab = ol - val;
    if (ab >= 0.0) { double nr = ab / th; d = d0 * pow(nr, P.npower); K = 1.0 + (P.kmax - 1.0) * pow(nr, P.npower); al = P.amax * (1.0 - nr); }
    ab = ol - (val + P.delta / 2.0);
    if (ab >= 0.0) { double nr = ab / th; dh = d0 * pow(nr, P.npower); Kh = 1.0 + (P.kmax - 1.0) * pow(nr, P.npower); alh = P.amax * (1.0 - nr); }
  }
  if (P.use_max) {
    double ab = val - orr;
    if (ab >= 0.0) { double nr = ab / th; d = d0 * pow(nr, P.npower); K = 1.0 + (P.kmax - 1.0) * pow(nr, P.npower); al = P.amax * (1.0 - nr); }
    ab = val + P.delta / 2.0 - orr;
    if (ab >= 0.0) { double nr = ab / th; dh = d0 * pow(nr, P.npower); Kh = 1.0 + (P.kmax - 1.0) * pow(nr, P.npower); alh = P.amax * (1.0 - nr); }
  }
  if (al < 0.0) al = 0.0;
  if (alh < 0.0) alh = 0.0;
  const double b = exp(-(d / K + al) * P.dt);
  const double bh = exp(-(dh / Kh + alh) * P.dt);
  const double a = fabs(d) > 1e-6 ? d * (b - 1.0) / (K * (d + K * al)) : 0.0;
  const double ah = fabs(dh) > 1e-6 ? dh * (bh - 1.0) / (Kh * (dh + Kh * alh)) : 0.0;
  const int n = P.n;
  double* o = out64;
  o[0 * n + i] = d; o[1 * n + i] = K; o[2 * n + i] = al; o[3 * n + i] = a; o[4 * n + i] = b;
  o[5 * n + i] = dh; o[6 * n + i] = Kh; o[7 * n + i] = alh; o[8 * n + i] = ah; o[9 * n + i] = bh;
  float* f = out32;  // a, b, 1/K, a_half, b_half, 1/K_half
  f[0 * n + i] = (float)a; f[1 * n + i] = (float)b; f[2 * n + i] = (float)(1.0 / K);
  f[3 * n + i] = (float)ah; f[4 * n + i] = (float)bh; f[5 * n + i] = (float)(1.0 / Kh);
}

void launch_build_profile(const ProfileArgs& P, double* out64, float* out32, cudaStream_t st) {
  build_profile_kernel<<<(P.n + 127) / 128, 128, 0, st>>>(P, out64, out32);
}

constexpr int kRedThreads = 256;

// Blocks 0..C-1 reduce local step b of the chunk; block C records receivers
// of the chunk's last step from the final velocities.
__global__ void __launch_bounds__(kRedThreads)
reduce_chunk_kernel(StepArgs s, int C, double* __restrict__ ek_out, double* __restrict__ ep_out,
                    double* __restrict__ vmax_out, int* __restrict__ bad_out) {
  const int base = *s.it_base;
  if ((int)blockIdx.x == C) {
    const size_t slab = (size_t)s.nrec * s.nstep;
    const int it = base + C;
    for (int r = threadIdx.x; r < s.nrec; r += blockDim.x) {
      const long long c = s.rec_cell[r];
      const size_t o = (size_t)r * s.nstep + (size_t)(it - 1);
      s.seis[o] = s.split ? __fadd_rn(s.f.vx[c], s.g.vx[c]) : s.f.vx[c];
      s.seis[slab + o] = s.split ? __fadd_rn(s.f.vy[c], s.g.vy[c]) : s.f.vy[c];
      if (s.f.vz) s.seis[2 * slab + o] = s.f.vz[c];
    }
    return;
  }
  const double* P = s.partials + (size_t)blockIdx.x * s.nblocks * 4;
  double ek = 0.0, ep = 0.0;
  float vm = 0.f;
  int bad = 0;
  for (int q = threadIdx.x; q < s.nblocks; q += blockDim.x) {
    ek += P[4 * (size_t)q + 0];
    ep += P[4 * (size_t)q + 1];
    vm = fmaxf(vm, (float)P[4 * (size_t)q + 2]);
    bad |= P[4 * (size_t)q + 3] != 0.0;
  }
  __shared__ double out[4];
  block_partials<kRedThreads>(ek, ep, vm, bad, out);
  if (threadIdx.x == 0) {
    const int it = base + blockIdx.x + 1;
    ek_out[it - 1] = out[0];
    ep_out[it - 1] = out[1];
    vmax_out[it - 1] = sqrt(out[2]);
    bad_out[it - 1] = out[3] != 0.0;
  }
}

__global__ void advance_kernel(int* it_base, int C) { *it_base += C; }

void launch_reduce_chunk(const StepArgs& s, int C, double* ek, double* ep, double* vmax, int* bad,
                         cudaStream_t st) {
  reduce_chunk_kernel<<<C + 1, kRedThreads, 0, st>>>(s, C, ek, ep, vmax, bad);
  advance_kernel<<<1, 1, 0, st>>>(const_cast<int*>(s.it_base), C);
}

}  // namespace cpml
