// surrogate.cu -- kernels of the learned seismogram surrogate.
//
// A small convolutional network maps a velocity model and a source position
// to receiver seismograms; shots it predicts poorly are re-run by the FD
// solver. Every layer of its training and inference runs on these kernels:
//   cpml_nn_gemm      C = alpha op(A) op(B) on BF16 tensor cores (mma.sync
//                     m16n8k16, FP32 accumulation), optional split-K with a
//                     fixed-order reduction, fused bias + ReLU epilogue,
//                     FP32 and/or BF16 output, optional accumulate
//   cpml_nn_gemm_tc   the same contract on tcgen05.mma with a TMEM accumulator
//   cpml_nn_im2col    3x3 stride-2 pad-1 patches of an NHWC BF16 activation
//   cpml_nn_col2im    its adjoint, as a gather (fixed order, no atomics)
//   cpml_nn_relu_bwd  dX = dY * (Y > 0), FP32 in, BF16 and/or FP32 out
//   cpml_nn_shift_rows per-shot row shift (offset axis <-> receiver axis)
//   cpml_nn_colsum    bias gradients: column sums in a fixed two-stage order
//   cpml_nn_rel_l2    per-shot squared relative L2 misfit and its gradient
//   cpml_nn_head_grad gradient of the misfit-prediction head
//   cpml_nn_adam      FP32 Adam on master weights, refreshed BF16 copies
//   cpml_nn_cast      FP32 -> BF16
// No counterpart in the reference, which has no learned component.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <mutex>

#include "../../include/cpml.h"

namespace {

constexpr int GBM = 64, GBN = 64, GBK = 32, GKP = GBK + 8;  // tile; padded smem row
constexpr int GT = 128;                                      // 4 warps, 2 x 2, 32 x 32 each

__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct Epilogue {
  float* Cf;
  __nv_bfloat16* Cb;
  int ldc;
  const float* bias;
  int relu, accum;
  float alpha;
};

__device__ __forceinline__ void epilogue_store(const Epilogue& e, int row, int col, float acc) {
  float v = e.alpha * acc;
  if (e.bias) v += e.bias[col];
  const size_t o = (size_t)row * e.ldc + col;
  if (e.accum && e.Cf) v += e.Cf[o];
  if (e.relu) v = fmaxf(v, 0.f);
  if (e.Cf) e.Cf[o] = v;
  if (e.Cb) e.Cb[o] = __float2bfloat16(v);
}

// C[M,N] = op(A)[M,K] * op(B)[K,N].
//   ta == 0: A is [M][lda] (k contiguous); ta == 1: A is [K][lda] (m contiguous)
//   tb == 0: B is [K][ldb] (n contiguous); tb == 1: B is [N][ldb] (k contiguous)
// blockIdx.z selects a K range of kchunk (a multiple of GBK). With one split
// the epilogue is applied here; otherwise the raw partial sums go to
// work[z][M][N] and gemm_reduce_kernel finishes.
__global__ void __launch_bounds__(GT) gemm_bf16_kernel(int M, int N, int K, int kchunk,
                                                       const __nv_bfloat16* __restrict__ A, int lda, int ta,
                                                       const __nv_bfloat16* __restrict__ B, int ldb, int tb,
                                                       Epilogue ep, float* __restrict__ work) {
  __shared__ __align__(16) __nv_bfloat16 As[GBM][GKP];   // [m][k]
  __shared__ __align__(16) __nv_bfloat16 Bs[GBN][GKP];   // [n][k]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.x * GBM, n0 = blockIdx.y * GBN;   // M tiles on x (up to 2^31 - 1)
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  const int g = lane >> 2, t4 = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = kb; k0 < ke; k0 += GBK) {
    // stage 64 x 32 tiles of A and B, coalesced along the contiguous index
    for (int e = tid; e < GBM * GBK; e += GT) {
      int mm, kk;
      if (ta) { mm = e % GBM; kk = e / GBM; } else { kk = e % GBK; mm = e / GBK; }
      const int gm = m0 + mm, gk = k0 + kk;
      __nv_bfloat16 v = zero;
      if (gm < M && gk < ke) v = ta ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      As[mm][kk] = v;
    }
    for (int e = tid; e < GBN * GBK; e += GT) {
      int nn, kk;
      if (tb) { kk = e % GBK; nn = e / GBK; } else { nn = e % GBN; kk = e / GBN; }
      const int gn = n0 + nn, gk = k0 + kk;
      __nv_bfloat16 v = zero;
      if (gn < N && gk < ke) v = tb ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      Bs[nn][kk] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < GBK; ks += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int r = wm + a * 16 + g;
        af[a][0] = pack2(&As[r][ks + t4 * 2]);
        af[a][1] = pack2(&As[r + 8][ks + t4 * 2]);
        af[a][2] = pack2(&As[r][ks + t4 * 2 + 8]);
        af[a][3] = pack2(&As[r + 8][ks + t4 * 2 + 8]);
      }
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int c = wn + b * 8 + g;
        bf[b][0] = pack2(&Bs[c][ks + t4 * 2]);
        bf[b][1] = pack2(&Bs[c][ks + t4 * 2 + 8]);
      }
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) mma_bf16(acc[a][b], af[a], bf[b]);
    }
    __syncthreads();
  }
  // accumulator fragment layout of m16n8: rows g and g + 8, columns 2 t4 + {0,1}
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int row = m0 + wm + a * 16 + g + h * 8;
          const int col = n0 + wn + b * 8 + t4 * 2 + q;
          if (row >= M || col >= N) continue;
          const float v = acc[a][b][h * 2 + q];
          if (work)
            work[((size_t)blockIdx.z * M + row) * N + col] = v;
          else
            epilogue_store(ep, row, col, v);
        }
}

__global__ void gemm_reduce_kernel(int M, int N, int splits, const float* __restrict__ work, Epilogue ep) {
  const long long total = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += work[(size_t)z * total + e];
    epilogue_store(ep, (int)(e / N), (int)(e % N), s);
  }
}

// 3x3, stride 2, pad 1 patches. in: NHWC [B][H][W][C]; out row m = (b, y, x)
// of the Ho x Wo output grid, column k = (ky*3 + kx)*C + c. One thread per
// (row m, tap, group of V channels): V = 8 moves 16 bytes per load and store
// (C a multiple of 8), V = 1 otherwise.
template <int V>
__global__ void im2col_kernel(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out, int B,
                              int H, int W, int C, int Ho, int Wo) {
  const int CG = C / V;                                   // channel groups per tap
  const long long total = (long long)B * Ho * Wo * 9 * CG;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int cg = (int)(e % CG);
    const long long mt = e / CG;                          // (row, tap)
    const int tap = (int)(mt % 9);
    const long long m = mt / 9;
    const int x = (int)(m % Wo);
    const long long by = m / Wo;
    const int y = (int)(by % Ho), b = (int)(by / Ho);
    const int iy = 2 * y + tap / 3 - 1, ix = 2 * x + tap % 3 - 1;
    const bool inside = iy >= 0 && iy < H && ix >= 0 && ix < W;
    const long long src = (((long long)b * H + iy) * W + ix) * C + (long long)cg * V;
    const long long dst = m * 9 * C + (long long)tap * C + (long long)cg * V;
    if (V == 8) {
      uint4 v = make_uint4(0, 0, 0, 0);
      if (inside) v = *reinterpret_cast<const uint4*>(in + src);
      *reinterpret_cast<uint4*>(out + dst) = v;
    } else {
      out[dst] = inside ? in[src] : __float2bfloat16(0.f);
    }
  }
}

// Adjoint of im2col as a gather: each input element sums, in a fixed order,
// the (at most 2 x 2) patch entries that read it. One thread per (pixel,
// group of V channels); V = 4 moves 16 bytes per access (C a multiple of 4).
template <int V>
__global__ void col2im_kernel(const float* __restrict__ col, float* __restrict__ out, int B, int H, int W, int C,
                              int Ho, int Wo) {
  const int CG = C / V;
  const long long total = (long long)B * H * W * CG;
  const long long K = 9LL * C;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int cg = (int)(e % CG);
    const long long pix = e / CG;
    const int ix = (int)(pix % W);
    const long long bi = pix / W;
    const int iy = (int)(bi % H), b = (int)(bi / H);
    float s[V];
#pragma unroll
    for (int q = 0; q < V; ++q) s[q] = 0.f;
    for (int ky = 0; ky < 3; ++ky) {
      const int ty = iy + 1 - ky;
      if (ty < 0 || (ty & 1) || (ty >> 1) >= Ho) continue;
      const int y = ty >> 1;
      for (int kx = 0; kx < 3; ++kx) {
        const int tx = ix + 1 - kx;
        if (tx < 0 || (tx & 1) || (tx >> 1) >= Wo) continue;
        const int x = tx >> 1;
        const long long m = ((long long)b * Ho + y) * Wo + x;
        const float* p = col + m * K + (ky * 3 + kx) * C + cg * V;
        if (V == 4) {
          const float4 v = *reinterpret_cast<const float4*>(p);
          s[0] += v.x; s[1] += v.y; s[2 % V] += v.z; s[3 % V] += v.w;
        } else {
#pragma unroll
          for (int q = 0; q < V; ++q) s[q] += p[q];
        }
      }
    }
    float* o = out + pix * C + cg * V;
    if (V == 4)
      *reinterpret_cast<float4*>(o) = make_float4(s[0], s[1 % V], s[2 % V], s[3 % V]);
    else
#pragma unroll
      for (int q = 0; q < V; ++q) o[q] = s[q];
  }
}

__global__ void relu_bwd_kernel(const float* __restrict__ dy, const float* __restrict__ y,
                                __nv_bfloat16* __restrict__ dx_b, float* __restrict__ dx_f, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float v = y[e] > 0.f ? dy[e] : 0.f;
    if (dx_b) dx_b[e] = __float2bfloat16(v);
    if (dx_f) dx_f[e] = v;
  }
}

// dst[b][r][:] = src[b][r + shift[b]][:] where 0 <= r + shift[b] < rows_src,
// else 0: moves traces between the source-centred offset axis and the
// receiver axis (a gather in both directions, so its adjoint is one too).
__global__ void shift_rows_kernel(const float* __restrict__ src, const int* __restrict__ shift,
                                  float* __restrict__ dst_f, __nv_bfloat16* __restrict__ dst_b, int B, int rows_src,
                                  int rows_dst, int L) {
  const long long total = (long long)B * rows_dst * L;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % L);
    const long long br = e / L;
    const int r = (int)(br % rows_dst), b = (int)(br / rows_dst);
    const int q = r + shift[b];
    const float v = (q >= 0 && q < rows_src) ? src[((long long)b * rows_src + q) * L + i] : 0.f;
    if (dst_f) dst_f[e] = v;
    if (dst_b) dst_b[e] = __float2bfloat16(v);
  }
}

__global__ void cast_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    y[e] = __float2bfloat16(x[e]);
}

constexpr int COLSUM_ROWS = 256;

// Stage 1: part[c][n] = sum of rows [c R, (c+1) R) of column n, rows in order.
__global__ void colsum_part_kernel(const float* __restrict__ x, float* __restrict__ part, int M, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int r0 = blockIdx.y * COLSUM_ROWS, r1 = min(M, r0 + COLSUM_ROWS);
  float s = 0.f;
  for (int m = r0; m < r1; ++m) s += x[(size_t)m * N + n];
  part[(size_t)blockIdx.y * N + n] = s;
}

// Stage 2: out[n] (+)= sum over chunks in order.
__global__ void colsum_final_kernel(const float* __restrict__ part, float* __restrict__ out, int chunks, int N,
                                    int accum) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int c = 0; c < chunks; ++c) s += part[(size_t)c * N + n];
  out[n] = accum ? out[n] + s : s;
}

// Per shot b: loss_b = ||p - t||^2 / (||t||^2 + tiny); grad = 2 (p - t) / (||t||^2 + tiny) / B.
// Sums in FP64 within the block, fixed tree order.
__global__ void rel_l2_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                              float* __restrict__ grad, float* __restrict__ loss, int B, int L) {
  const int b = blockIdx.x;
  __shared__ double sn[256], se[256];
  double n2 = 0.0, e2 = 0.0;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const double t = target[(size_t)b * L + i], d = (double)pred[(size_t)b * L + i] - t;
    n2 += t * t;
    e2 += d * d;
  }
  sn[threadIdx.x] = n2;
  se[threadIdx.x] = e2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { sn[threadIdx.x] += sn[threadIdx.x + o]; se[threadIdx.x] += se[threadIdx.x + o]; }
    __syncthreads();
  }
  const double den = sn[0] + 1e-30;
  if (threadIdx.x == 0) loss[b] = (float)(se[0] / den);
  if (grad) {
    const float s = (float)(2.0 / den / B);
    for (int i = threadIdx.x; i < L; i += blockDim.x)
      grad[(size_t)b * L + i] = s * (pred[(size_t)b * L + i] - target[(size_t)b * L + i]);
  }
}

// Misfit head: h_b predicts log(loss_b); gradient of w * mean_b (h_b - log loss_b)^2.
__global__ void head_grad_kernel(const float* __restrict__ h, int ldh, const float* __restrict__ loss,
                                 float* __restrict__ dh, int B, float w) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float t = logf(fmaxf(loss[b], 1e-12f));
  dh[b] = 2.f * w * (h[(size_t)b * ldh] - t) / (float)B;
}

__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, long long n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gr = g[e] + wd * w[e];
    const float mm = b1 * m[e] + (1.f - b1) * gr;
    const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
    m[e] = mm;
    v[e] = vv;
    const float nw = w[e] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    w[e] = nw;
    if (wb) wb[e] = __float2bfloat16(nw);
  }
}

// ---------------------------------------------------------------------------
// The same GEMM on the 5th-generation tensor cores: tcgen05.mma with the
// accumulator in tensor memory. A CTA of 4 warps owns a 128 x 128 output
// tile; operand tiles of 64 k-values are staged into shared memory in the
// canonical K-major, non-swizzled core-matrix layout (8 rows x 16 bytes per
// core matrix, core matrices 128 B apart along k and 1 KB apart along m/n),
// two stages deep: while the tensor core works on one stage, the threads
// fill the other. One thread issues the MMAs (4 x K=16 per stage) and
// commits them to the stage's mbarrier; the 128 fp32 accumulator columns are
// read back with tcgen05.ld (warp w reads TMEM lanes 32w..32w+31 = rows).
// ---------------------------------------------------------------------------
namespace tc {

constexpr int BM = 128, BK = 64, NT = 128, STAGES = 3;
constexpr int A_BYTES = BM * BK * 2;                       // 16 KB A tile
constexpr uint32_t LBO = 128, SBO = 1024;                  // k- and m/n-direction core-matrix strides
constexpr long long kWait = 2000000000LL;                  // ~1 s at 2 GHz

// Output tile width BN (32, 64 or 128: the narrowest that holds N, so thin
// layers do not multiply zeros); BN fp32 TMEM columns hold the accumulator.
template <int BN>
struct Cfg {
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 64;
  // Instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
  // (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at
  // bit 17, M >> 4 at bit 24.
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                    ((uint32_t)(BM >> 4) << 24);
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start >> 4, LBO >> 4 at bit 16, SBO >> 4
// at bit 32, descriptor version 1 at bit 46, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((LBO >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((SBO >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// byte offset of element (r, k) of a staged tile
__device__ __forceinline__ int core_off(int r, int k) {
  return ((r >> 3) * (BK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Stage rows [r0, r0 + ROWS) x k-values [k0, k0 + 64) of a bf16 operand
// into `tile`; trans == 0: element (r, k) at src[r * ld + k], else at
// src[k * ld + r]. Out-of-range elements are zero.
template <int ROWS>
__device__ __forceinline__ void stage(unsigned char* tile, const __nv_bfloat16* __restrict__ src, int ld, int trans,
                                      int r0, int R, int k0, int ke) {
  const int tid = threadIdx.x;
  if (!trans) {
    const bool vec = (ld & 7) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    // ROWS rows x 8 groups of 8 k-values; consecutive threads take consecutive groups
    for (int e = tid; e < ROWS * (BK / 8); e += NT) {
      const int r = e >> 3, g = e & 7;
      const int gr = r0 + r, gk = k0 + g * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gr < R) {
        if (vec && gk + 8 <= ke) {
          v = *reinterpret_cast<const uint4*>(src + (size_t)gr * ld + gk);
        } else {
          __nv_bfloat16 t[8];
#pragma unroll
          for (int q = 0; q < 8; ++q)
            t[q] = (gk + q < ke) ? src[(size_t)gr * ld + gk + q] : __float2bfloat16(0.f);
          v = *reinterpret_cast<const uint4*>(t);
        }
      }
      *reinterpret_cast<uint4*>(tile + core_off(r, g * 8)) = v;
    }
  } else {
    // consecutive threads take consecutive rows (contiguous in memory)
    for (int e = tid; e < ROWS * BK; e += NT) {
      const int r = e % ROWS, k = e / ROWS;
      const int gr = r0 + r, gk = k0 + k;
      const __nv_bfloat16 v = (gr < R && gk < ke) ? src[(size_t)gk * ld + gr] : __float2bfloat16(0.f);
      *reinterpret_cast<__nv_bfloat16*>(tile + core_off(r, k)) = v;
    }
  }
}

// Asynchronous form of stage() for a k-contiguous operand whose rows start
// on 16-byte boundaries (ld a multiple of 8, src 16-byte aligned): every
// 8-value group is one 16-byte cp.async straight into its core-matrix row,
// zero-filled past the end of the row or of the matrix.
template <int ROWS>
__device__ __forceinline__ void stage_async(unsigned char* tile, const __nv_bfloat16* __restrict__ src, int ld,
                                            int r0, int R, int k0, int ke) {
  for (int e = threadIdx.x; e < ROWS * (BK / 8); e += NT) {
    const int r = e >> 3, g = e & 7;
    const int gr = r0 + r, gk = k0 + g * 8;
    int bytes = 0;
    const __nv_bfloat16* p = src;  // a valid address even when nothing is read
    if (gr < R && gk < ke) {
      bytes = (ke - gk >= 8 ? 8 : ke - gk) * 2;
      p = src + (size_t)gr * ld + gk;
    }
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(tile + core_off(r, g * 8))),
                 "l"(p), "r"(bytes)
                 : "memory");
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kWait) return false;
  }
}

}  // namespace tc

__device__ int g_nn_err;  // set when a bounded tensor-core wait gives up

template <int BN>
__global__ void __launch_bounds__(tc::NT) gemm_tc_kernel(int M, int N, int K, int kchunk,
                                                        const __nv_bfloat16* __restrict__ A, int lda, int ta,
                                                        const __nv_bfloat16* __restrict__ B, int ldb, int tb,
                                                        Epilogue ep, float* __restrict__ work) {
  using namespace tc;
  using C = Cfg<BN>;
  constexpr int STAGE_BYTES = C::STAGE_BYTES;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + STAGES * STAGE_BYTES + 32);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  const int nk = ke > kb ? (ke - kb + BK - 1) / BK : 0;

  if (warp == 0) {  // BN fp32 accumulator columns for the 128 x BN tile
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&bar[s])), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  // k-contiguous, 16-byte-aligned operands are staged with cp.async (several
  // stages in flight); the others with plain loads and stores
  const bool avec = !ta && (lda & 7) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
  const bool bvec = tb && (ldb & 7) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
  auto load_stage = [&](int kt) {
    unsigned char* sa = smem + (kt % STAGES) * STAGE_BYTES;
    unsigned char* sb = sa + A_BYTES;
    const int k0 = kb + kt * BK;
    if (avec) stage_async<BM>(sa, A, lda, m0, M, k0, ke); else stage<BM>(sa, A, lda, ta, m0, M, k0, ke);
    if (bvec) stage_async<BN>(sb, B, ldb, n0, N, k0, ke); else stage<BN>(sb, B, ldb, tb ? 0 : 1, n0, N, k0, ke);
  };
  // prologue: k-tiles 0 .. STAGES-2, one cp.async group each (empty if absent)
  for (int q = 0; q < STAGES - 1; ++q) {
    if (q < nk) load_stage(q);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  bool ok = true;
  for (int kt = 0; kt < nk && ok; ++kt) {
    const int s = kt % STAGES;
    unsigned char* sa = smem + s * STAGE_BYTES;
    unsigned char* sb = sa + A_BYTES;
    // this thread's copies of k-tile kt have landed (later groups may not)
    asm volatile("cp.async.wait_group %0;" ::"n"(STAGES - 2) : "memory");
    // make the stores of this stage visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < BK / 16; ++ks) {
        const uint64_t da = desc(smem_addr(sa) + ks * 2 * LBO);
        const uint64_t db = desc(smem_addr(sb) + ks * 2 * LBO);
        const uint32_t acc = (kt > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(C::IDESC), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(&bar[s]))
                   : "memory");
    }
    // refill the stage that k-tile kt - 1 used with k-tile kt + STAGES - 1,
    // once its MMAs have finished (the j-th commit to a stage's barrier
    // completes its phase j)
    const int kn = kt + STAGES - 1;
    if (kn < nk) {
      if (kt >= 1) ok = mbar_wait(&bar[(kt - 1) % STAGES], (uint32_t)(((kt - 1) / STAGES) & 1));
      if (!__syncthreads_and(ok ? 1 : 0)) { ok = false; break; }
      load_stage(kn);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // all MMAs done: the last commit covers every earlier one of this thread
  if (ok && nk > 0) ok = mbar_wait(&bar[(nk - 1) % STAGES], (uint32_t)(((nk - 1) / STAGES) & 1));
  ok = __syncthreads_and(ok ? 1 : 0) != 0;   // uniform: tcgen05.ld below is warp-collective
  if (!ok && tid == 0) atomicOr(&g_nn_err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: warp w reads TMEM lanes 32w..32w+31 (tile rows, one per
  // thread) into a padded fp32 tile in the now idle stage buffers, then the
  // CTA writes the tile out row by row, consecutive threads on consecutive
  // columns (coalesced)
  float* cs = reinterpret_cast<float*>(smem);   // [BM][BN + 1]
  constexpr int CP = BN + 1;
  static_assert(BM * CP * 4 <= STAGES * STAGE_BYTES, "epilogue tile fits in the stage buffers");
  const int rloc = warp * 32 + lane;
#pragma unroll 1
  for (int c = 0; c < BN; c += 16) {
    uint32_t r[16];
    if (ok && nk > 0) {
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) r[q] = 0u;  // empty K range (or a failed wait): zero
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) cs[rloc * CP + c + q] = __uint_as_float(r[q]);
  }
  __syncthreads();
  for (int e = tid; e < BM * BN; e += NT) {
    const int rr = e / BN, cc = e % BN;
    const int row = m0 + rr, col = n0 + cc;
    if (row >= M || col >= N) continue;
    const float v = cs[rr * CP + cc];
    if (work)
      work[((size_t)blockIdx.z * M + row) * N + col] = v;
    else
      epilogue_store(ep, row, col, v);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

int status() { return cudaGetLastError() == cudaSuccess ? CPML_OK : CPML_ERR_CUDA; }

}  // namespace

extern "C" {

int cpml_nn_gemm(int M, int N, int K, const void* A, int lda, int ta, const void* B, int ldb, int tb, float* Cf,
                 void* Cb, int ldc, const float* bias, int relu, int accum, float alpha, int splits, float* work,
                 long long work_elems, void* stream) {
  if (M < 0 || N < 0 || K < 0 || !A || !B || (!Cf && !Cb) || splits < 1) return CPML_ERR_INVALID;
  if (accum && !Cf) return CPML_ERR_INVALID;
  if (M == 0 || N == 0) return CPML_OK;
  if ((N + GBN - 1) / GBN > 65535) return CPML_ERR_RANGE;
  int kchunk = (K + splits - 1) / splits;
  kchunk = ((kchunk + GBK - 1) / GBK) * GBK;
  if (kchunk < GBK) kchunk = GBK;
  splits = K > 0 ? (K + kchunk - 1) / kchunk : 1;
  if (splits > 65535) return CPML_ERR_RANGE;
  if (splits > 1 && (!work || work_elems < (long long)splits * M * N)) return CPML_ERR_INVALID;
  const Epilogue ep{Cf, (__nv_bfloat16*)Cb, ldc, bias, relu, accum, alpha};
  const dim3 grid((M + GBM - 1) / GBM, (N + GBN - 1) / GBN, splits);
  cudaStream_t st = (cudaStream_t)stream;
  gemm_bf16_kernel<<<grid, GT, 0, st>>>(M, N, K, kchunk, (const __nv_bfloat16*)A, lda, ta,
                                        (const __nv_bfloat16*)B, ldb, tb, ep, splits > 1 ? work : nullptr);
  if (splits > 1) gemm_reduce_kernel<<<grid_for((long long)M * N), 256, 0, st>>>(M, N, splits, work, ep);
  return status();
}

int cpml_nn_gemm_tc(int M, int N, int K, const void* A, int lda, int ta, const void* B, int ldb, int tb, float* Cf,
                    void* Cb, int ldc, const float* bias, int relu, int accum, float alpha, int splits, float* work,
                    long long work_elems, void* stream) {
  if (M < 0 || N < 0 || K < 0 || !A || !B || (!Cf && !Cb) || splits < 1) return CPML_ERR_INVALID;
  if (accum && !Cf) return CPML_ERR_INVALID;
  if (M == 0 || N == 0) return CPML_OK;
  const int bn = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
  if ((N + bn - 1) / bn > 65535) return CPML_ERR_RANGE;
  {
    // the dynamic shared-memory limit is a per-device function attribute:
    // set it once for every device this process launches the GEMM on
    static std::mutex mu;
    static unsigned long long done = 0;  // bit d: set on device d
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CPML_ERR_CUDA;
    std::lock_guard<std::mutex> lock(mu);
    if (!((done >> dev) & 1ull)) {
      if (cudaFuncSetAttribute(gemm_tc_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               tc::Cfg<32>::SMEM) != cudaSuccess ||
          cudaFuncSetAttribute(gemm_tc_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               tc::Cfg<64>::SMEM) != cudaSuccess ||
          cudaFuncSetAttribute(gemm_tc_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               tc::Cfg<128>::SMEM) != cudaSuccess)
        return CPML_ERR_CUDA;
      done |= 1ull << dev;
    }
  }
  int kchunk = (K + splits - 1) / splits;
  kchunk = ((kchunk + tc::BK - 1) / tc::BK) * tc::BK;
  if (kchunk < tc::BK) kchunk = tc::BK;
  splits = K > 0 ? (K + kchunk - 1) / kchunk : 1;
  if (splits > 65535) return CPML_ERR_RANGE;
  if (splits > 1 && (!work || work_elems < (long long)splits * M * N)) return CPML_ERR_INVALID;
  const Epilogue ep{Cf, (__nv_bfloat16*)Cb, ldc, bias, relu, accum, alpha};
  const dim3 grid((M + tc::BM - 1) / tc::BM, (N + bn - 1) / bn, splits);
  cudaStream_t st = (cudaStream_t)stream;
  const __nv_bfloat16 *a = (const __nv_bfloat16*)A, *b = (const __nv_bfloat16*)B;
  float* w = splits > 1 ? work : nullptr;
  if (bn == 32)
    gemm_tc_kernel<32><<<grid, tc::NT, tc::Cfg<32>::SMEM, st>>>(M, N, K, kchunk, a, lda, ta, b, ldb, tb, ep, w);
  else if (bn == 64)
    gemm_tc_kernel<64><<<grid, tc::NT, tc::Cfg<64>::SMEM, st>>>(M, N, K, kchunk, a, lda, ta, b, ldb, tb, ep, w);
  else
    gemm_tc_kernel<128><<<grid, tc::NT, tc::Cfg<128>::SMEM, st>>>(M, N, K, kchunk, a, lda, ta, b, ldb, tb, ep, w);
  if (splits > 1) gemm_reduce_kernel<<<grid_for((long long)M * N), 256, 0, st>>>(M, N, splits, work, ep);
  return status();
}

int cpml_nn_error(int* err) {
  if (!err) return CPML_ERR_INVALID;
  int zero = 0;
  if (cudaMemcpyFromSymbol(err, g_nn_err, sizeof(int)) != cudaSuccess) return CPML_ERR_CUDA;
  if (cudaMemcpyToSymbol(g_nn_err, &zero, sizeof(int)) != cudaSuccess) return CPML_ERR_CUDA;
  return CPML_OK;
}

int cpml_nn_im2col(const void* in, void* out, int B, int H, int W, int C, void* stream) {
  if (!in || !out || B < 1 || H < 2 || W < 2 || C < 1) return CPML_ERR_INVALID;
  const int Ho = (H + 1) / 2, Wo = (W + 1) / 2;
  const bool vec = C % 8 == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(out) & 15) == 0;
  const long long n = (long long)B * Ho * Wo * 9 * (vec ? C / 8 : C);
  if (vec)
    im2col_kernel<8><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, (__nv_bfloat16*)out, B,
                                                                      H, W, C, Ho, Wo);
  else
    im2col_kernel<1><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, (__nv_bfloat16*)out, B,
                                                                      H, W, C, Ho, Wo);
  return status();
}

int cpml_nn_col2im(const float* col, float* out, int B, int H, int W, int C, void* stream) {
  if (!col || !out || B < 1 || H < 2 || W < 2 || C < 1) return CPML_ERR_INVALID;
  const int Ho = (H + 1) / 2, Wo = (W + 1) / 2;
  const bool vec = C % 4 == 0 && (reinterpret_cast<uintptr_t>(col) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(out) & 15) == 0;
  const long long n = (long long)B * H * W * (vec ? C / 4 : C);
  if (vec)
    col2im_kernel<4><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(col, out, B, H, W, C, Ho, Wo);
  else
    col2im_kernel<1><<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(col, out, B, H, W, C, Ho, Wo);
  return status();
}

int cpml_nn_relu_bwd(const float* dy, const float* y, void* dx_bf16, float* dx_f32, long long n, void* stream) {
  if (!dy || !y || n < 0 || (!dx_bf16 && !dx_f32)) return CPML_ERR_INVALID;
  if (n == 0) return CPML_OK;
  relu_bwd_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(dy, y, (__nv_bfloat16*)dx_bf16, dx_f32, n);
  return status();
}

int cpml_nn_shift_rows(const float* src, const int* shift, float* dst_f32, void* dst_bf16, int B, int rows_src,
                       int rows_dst, int L, void* stream) {
  if (!src || !shift || (!dst_f32 && !dst_bf16) || B < 1 || rows_src < 1 || rows_dst < 1 || L < 1)
    return CPML_ERR_INVALID;
  const long long n = (long long)B * rows_dst * L;
  shift_rows_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(src, shift, dst_f32, (__nv_bfloat16*)dst_bf16, B,
                                                                    rows_src, rows_dst, L);
  return status();
}

int cpml_nn_cast(const float* x, void* y, long long n, void* stream) {
  if (!x || !y || n < 0) return CPML_ERR_INVALID;
  if (n == 0) return CPML_OK;
  cast_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, (__nv_bfloat16*)y, n);
  return status();
}

int cpml_nn_colsum(const float* x, float* out, int M, int N, int accum, float* work, long long work_elems,
                   void* stream) {
  if (!x || !out || M < 1 || N < 1 || !work) return CPML_ERR_INVALID;
  const int chunks = (M + COLSUM_ROWS - 1) / COLSUM_ROWS;
  if (chunks > 65535) return CPML_ERR_RANGE;
  if (work_elems < (long long)chunks * N) return CPML_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  colsum_part_kernel<<<dim3((N + 127) / 128, chunks), 128, 0, st>>>(x, work, M, N);
  colsum_final_kernel<<<(N + 127) / 128, 128, 0, st>>>(work, out, chunks, N, accum);
  return status();
}

int cpml_nn_rel_l2(const float* pred, const float* target, float* grad, float* loss, int B, int L, void* stream) {
  if (!pred || !target || !loss || B < 1 || L < 1) return CPML_ERR_INVALID;
  rel_l2_kernel<<<B, 256, 0, (cudaStream_t)stream>>>(pred, target, grad, loss, B, L);
  return status();
}

int cpml_nn_head_grad(const float* h, int ldh, const float* loss, float* dh, int B, float weight, void* stream) {
  if (!h || !loss || !dh || B < 1 || ldh < 1) return CPML_ERR_INVALID;
  head_grad_kernel<<<(B + 127) / 128, 128, 0, (cudaStream_t)stream>>>(h, ldh, loss, dh, B, weight);
  return status();
}

int cpml_nn_adam(float* w, void* wb, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                 float eps, int step, float wd, void* stream) {
  if (!w || !g || !m || !v || n < 0 || step < 1) return CPML_ERR_INVALID;
  if (n == 0) return CPML_OK;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)wb, g, m, v, n, lr, b1, b2, eps,
                                                              c1, c2, wd);
  return status();
}

}  // extern "C"
