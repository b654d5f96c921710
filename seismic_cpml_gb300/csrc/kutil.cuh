// kutil.cuh -- small device helpers shared by the stencil kernels.
#pragma once
#include <cuda_runtime.h>
#include "cpml_internal.cuh"

namespace cpml {

// C-PML memory-variable recursion and derivative correction
// (2D:574-578 and every sweep of 3D:836-1052):
//   psi <- b*psi + a*d ;  d' = d/K + psi
// Outside the slab (sidx < 0) a = 0, psi = 0 and K = 1, so d' = d.
__device__ __forceinline__ float pml(float d, int sidx, float* __restrict__ mem, long long midx,
                                     const float* __restrict__ a, const float* __restrict__ b,
                                     const float* __restrict__ ik, int idx) {
  if (sidx < 0) return d;
  const float m = __ldg(b + idx) * mem[midx] + __ldg(a + idx) * d;
  mem[midx] = m;
  return d * __ldg(ik + idx) + m;
}

// A double-float value hi + lo (about 48 significant bits) built from FP32
// arithmetic alone: the energy reductions sum per-thread partials this way,
// because FP64 adds run at a small fraction of the FP32 rate on this part.
struct DF {
  float hi, lo;
};
// Knuth's two-sum of the leading parts plus the trailing parts, renormalised.
// The _rn intrinsics keep the compiler from contracting or re-associating.
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  const float t = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
  const float h = __fadd_rn(s, t);
  return DF{h, __fsub_rn(t, __fsub_rn(h, s))};
}

// Compensated (Kahan) FP32 accumulator: per-thread energy partials stay at
// FP64-like accuracy without FP64 arithmetic per cell (FP64 throughput on
// this part is a small fraction of FP32).
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ DF df() const { return DF{s, -c}; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_or(int v) {
  return __any_sync(0xffffffffu, v) ? 1 : 0;
}

// Deterministic block reduction of (ek, ep, vmax^2, bad) to thread 0, written
// to out[0..3]. Fixed tree order => bitwise reproducible.
template <int NT>
__device__ __forceinline__ void block_partials(double ek, double ep, float vm2, int bad,
                                               double* __restrict__ out) {
  constexpr int NW = NT / 32;
  __shared__ double s_ek[NW], s_ep[NW];
  __shared__ float s_vm[NW];
  __shared__ int s_bad[NW];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y;
  const int lane = tid & 31, w = tid >> 5;
  ek = warp_sum(ek);
  ep = warp_sum(ep);
  vm2 = warp_max(vm2);
  bad = warp_or(bad);
  if (lane == 0) { s_ek[w] = ek; s_ep[w] = ep; s_vm[w] = vm2; s_bad[w] = bad; }
  __syncthreads();
  if (w == 0) {
    ek = lane < NW ? s_ek[lane] : 0.0;
    ep = lane < NW ? s_ep[lane] : 0.0;
    vm2 = lane < NW ? s_vm[lane] : 0.f;
    bad = lane < NW ? s_bad[lane] : 0;
    ek = warp_sum(ek);
    ep = warp_sum(ep);
    vm2 = warp_max(vm2);
    bad = warp_or(bad);
    if (lane == 0) { out[0] = ek; out[1] = ep; out[2] = (double)vm2; out[3] = (double)bad; }
  }
}

// Bounded grid barrier of a cooperative launch (every CTA resident) on one
// monotonically increasing arrival counter: the n-th barrier of a launch
// (n = 1, 2, ...) is passed once *count reaches target = n * CTAs. Thread 0
// of each CTA arrives with a release add (ordering the CTA's earlier writes,
// gathered by the __syncthreads) and polls with acquire loads; there is no
// reset and no generation word, so the critical path is one arrival and the
// poll that sees the last one. *count must be zero at launch. A wait longer
// than wait_cycles SM cycles sets err_bit in *err and returns false; the CTA
// then leaves the kernel, and every other CTA gives up at its next barrier
// within the same bound. Wrap-safe: the counter never runs more than one
// barrier's arrivals ahead of a waiting CTA's target.
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned target, int* err, int err_bit,
                                             long long wait_cycles) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
    ok = 1;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
    const long long t0 = clock64();
    for (;;) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(count) : "memory");
      if ((int)(v - target) >= 0) break;
      if (clock64() - t0 > wait_cycles) {
        atomicOr(err, err_bit);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
  }
  __syncthreads();
  return ok != 0;
}

// The same reduction with double-float partials: a fixed shuffle tree per
// warp, then warp 0 over the warps' results, all in FP32 two-sum arithmetic;
// only the block's two totals are converted to FP64 (out[0..3] as above).
template <int NT>
__device__ __forceinline__ void block_partials(DF ek, DF ep, float vm2, int bad, double* __restrict__ out) {
  constexpr int NW = NT / 32;
  __shared__ float s_e[4][NW];
  __shared__ float s_vm[NW];
  __shared__ int s_bad[NW];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y;
  const int lane = tid & 31, w = tid >> 5;
  auto wsum = [](DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v = df_add(v, DF{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
    return v;
  };
  ek = wsum(ek);
  ep = wsum(ep);
  vm2 = warp_max(vm2);
  bad = warp_or(bad);
  if (lane == 0) {
    s_e[0][w] = ek.hi; s_e[1][w] = ek.lo; s_e[2][w] = ep.hi; s_e[3][w] = ep.lo;
    s_vm[w] = vm2; s_bad[w] = bad;
  }
  __syncthreads();
  if (w == 0) {
    const bool in = lane < NW;
    ek = DF{in ? s_e[0][lane] : 0.f, in ? s_e[1][lane] : 0.f};
    ep = DF{in ? s_e[2][lane] : 0.f, in ? s_e[3][lane] : 0.f};
    vm2 = in ? s_vm[lane] : 0.f;
    bad = in ? s_bad[lane] : 0;
    ek = wsum(ek);
    ep = wsum(ep);
    vm2 = warp_max(vm2);
    bad = warp_or(bad);
    if (lane == 0) {
      out[0] = (double)ek.hi + (double)ek.lo;
      out[1] = (double)ep.hi + (double)ep.lo;
      out[2] = (double)vm2;
      out[3] = (double)bad;
    }
  }
}

// v^2 check that also catches NaN / Inf (the reference's maxval would skip
// NaN; flagging it is an extension).
__device__ __forceinline__ int not_finite(float v2) { return !(v2 <= 3.0e38f); }

}  // namespace cpml
