// batch2d.cu -- many 2D shots in one persistent launch.
//
// Each shot is a complete run of seismic_CPML_2D_isotropic_second_order.f90
// (its own grid size, model, source, receivers, DELTAT and NSTEP). All shots
// advance together in ONE cooperative kernel launch (captured in a CUDA
// graph): per time step a stress phase over every (shot, tile) item of the
// shots still running, a grid barrier, a velocity phase, a grid barrier. The
// per-cell arithmetic is the single-shot path's (cell2d.cuh), so a shot's
// seismograms and fields are bit-identical to running it alone.
//
// Shots are scheduled in decreasing NSTEP, so the items active at step t are
// a prefix of the item table and a finished shot costs nothing. Items are
// 32 x 8 tiles handed out round-robin over the resident CTAs, so uneven grid
// sizes balance without a queue. Grid barriers spin with a bound (~2 s) and
// report CPML_ERR_TIMEOUT instead of hanging.
//
// Temporal blocking (depth D = 2 or 3, batch2d_tb_kernel): each item, a
// 32 x TH tile, is staged in shared memory with a halo of 2D cells (fields,
// per-cell model and, on C-PML tiles, memory variables) and advanced D time
// steps there: stress on the tile grown by 2(D-u)-1 cells, then velocity on
// it grown by 2(D-u)-2, for u = 0..D-1, so each update only reads cells the
// previous one produced. Only the tile's own cells go back to HBM, into the
// other of two buffer sets (neighbouring items still read the old set), and
// one grid barrier ends the phase: D time steps per HBM round trip and per
// barrier instead of one step and two barriers. The cell updates are the
// same functions (cell2d.cuh) on a shared-memory view, so the results are
// bit-identical to depth 1.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cpml.h"
#include "cpml_internal.cuh"
#include "kutil.cuh"
#include "cell2d.cuh"

namespace cpml {

void launch_build_profile(const ProfileArgs& P, double* out64, float* out32, cudaStream_t st);

constexpr int BTX = 32, BTY = 8, BNT = BTX * BTY;
constexpr long long kBarrierCycles = 4000000000LL;

struct BatchArgs {
  const Shot2D* shots;      // by shot id
  const Shot2D* shots_alt;  // the same shots on their second buffer set (temporal blocking)
  const int* item_rb;       // temporal blocking: receivers of item q are [item_rb[q], item_rb[q+1])
  const int* shot_nstep;    // NSTEP by shot id
  const int4* items;        // (shot, i0, j0, -) in schedule order
  const int* items_at;      // [max_nstep] items of the shots running at step t
  const int* recs_at;       // [max_nstep] receivers of the shots running at step t
  const int2* rec;          // (shot, padded cell) in schedule order
  const long long* rec_off; // sample 0 of the receiver's v_x trace in seis
  const long long* rec_offy;// sample 0 of its v_y trace
  float* seis;
  int max_nstep;
  unsigned* bar;            // [0] grid-barrier arrivals (zeroed before each launch)
  int* err;                 // 2 = barrier gave up, 4 = non-finite velocity
  long long wait_cycles;    // bound of one grid-barrier wait
};

// nbar counts the launch's barriers so far (the arrival counter's target)
__device__ __forceinline__ bool grid_sync(const BatchArgs& a, unsigned& nbar) {
  return grid_barrier(a.bar, ++nbar * gridDim.x, a.err, 2, a.wait_cycles);
}

__device__ __forceinline__ void record_batch(const BatchArgs& a, int t) {
  const int n = a.recs_at[t];
  for (long long r = (long long)blockIdx.x * BNT + threadIdx.x; r < n; r += (long long)gridDim.x * BNT) {
    const int2 rc = a.rec[r];
    const Shot2D& S = a.shots[rc.x];
    a.seis[a.rec_off[r] + t] = S.vx[rc.y];
    a.seis[a.rec_offy[r] + t] = S.vy[rc.y];
  }
}

// The current item's shot descriptor, staged in shared memory when the item
// belongs to another shot than the warp's previous one. Read through a
// reference into global memory, every field would be a global load in front
// of the data load it addresses, repeated after each store, since a store
// through one of the descriptor's pointers could, for all the compiler
// knows, change the descriptor itself. Each warp (one tile row) keeps its own
// copy, so staging needs warp synchronisation only.
__device__ __forceinline__ void stage_shot(const Shot2D* shots, int id, Shot2D& sh, int& cur) {
  static_assert(sizeof(Shot2D) % 8 == 0, "descriptor copied in 8-byte words");
  if (id == cur) return;
  __syncwarp();  // every lane is done with the previous descriptor
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(shots + id);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sh);
  for (int w = threadIdx.x & 31; w < (int)(sizeof(Shot2D) / 8); w += 32) dst[w] = src[w];
  __syncwarp();
  cur = id;
}

// 5 resident CTAs per SM (48 registers, 24 bytes spilled): the kernel is bound by
// memory latency. The cell updates issue all of a cell's loads before its
// stores, which takes more registers than 6 CTAs per SM leave (40) but
// covers a cell's reads with one latency instead of two or three (36.6 ->
// 39.6 Gcell-updates/s on a 32-shot batch). Taking two items per loop
// iteration with both cells' loads first needs ~90 registers per thread and
// spilled at every occupancy. Each CTA also requests its next item one
// iteration ahead (40.2 -> 41.0 Gcell-updates/s on the 32-shot batch).
__global__ void __launch_bounds__(BNT, 5) batch2d_kernel(BatchArgs a) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __shared__ Shot2D shw[BNT / 32];  // one descriptor copy per warp
  Shot2D& sh = shw[ty];
  int cur = -1;
  unsigned nbar = 0;
  for (int t = 0; t < a.max_nstep; ++t) {
    if (t > 0) record_batch(a, t - 1);
    const int n = a.items_at[t];
    // the next item is requested one iteration ahead (its index load would
    // otherwise be a second memory latency in front of every cell's loads)
    int4 nxt = blockIdx.x < n ? a.items[blockIdx.x] : make_int4(0, 0, 0, 0);
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
      const int4 itm = nxt;
      if (q + (int)gridDim.x < n) nxt = a.items[q + gridDim.x];
      stage_shot(a.shots, itm.x, sh, cur);
      const Shot2D& S = sh;
      const int i = itm.y + tx, j = itm.z + ty;
      if (i < S.nx && j < S.ny) {
        if (S.het) stress2d_cell<true>(S, i, j);
        else stress2d_cell<false>(S, i, j);
      }
    }
    if (!grid_sync(a, nbar)) return;
    nxt = blockIdx.x < n ? a.items[blockIdx.x] : make_int4(0, 0, 0, 0);
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
      const int4 itm = nxt;
      if (q + (int)gridDim.x < n) nxt = a.items[q + gridDim.x];
      stage_shot(a.shots, itm.x, sh, cur);
      const Shot2D& S = sh;
      const int i = itm.y + tx, j = itm.z + ty;
      if (i < S.nx && j < S.ny) {
        float ek = 0.f, ep = 0.f, vm2 = 0.f;
        int bad = 0;
        if (S.het) velocity2d_cell<true>(S, i, j, t + 1, ek, ep, vm2, bad);
        else velocity2d_cell<false>(S, i, j, t + 1, ek, ep, vm2, bad);
        if (bad) atomicOr(a.err, 4);
      }
    }
    if (!grid_sync(a, nbar)) return;
  }
  if (a.max_nstep > 0) record_batch(a, a.max_nstep - 1);
}

// The staged region of one item: 16 arrays of RW x RH cells in shared
// memory (vx vy sxx syy sxy | lambda mu rho | four x-slab and four y-slab
// memory variables, all indexed like the fields); grid cell (i, j) is
// element (j - oy) * RW + (i - ox).
template <int RW, int RC>
struct RegionView {
  float* f;
  int ox, oy;
  __device__ __forceinline__ float* vx() const { return f; }
  __device__ __forceinline__ float* vy() const { return f + RC; }
  __device__ __forceinline__ float* sxx() const { return f + 2 * RC; }
  __device__ __forceinline__ float* syy() const { return f + 3 * RC; }
  __device__ __forceinline__ float* sxy() const { return f + 4 * RC; }
  __device__ __forceinline__ const float* lam() const { return f + 5 * RC; }
  __device__ __forceinline__ const float* mu() const { return f + 6 * RC; }
  __device__ __forceinline__ const float* rho() const { return f + 7 * RC; }
  __device__ __forceinline__ float* mx(int q) const { return f + (8 + q) * RC; }
  __device__ __forceinline__ float* my(int q) const { return f + (12 + q) * RC; }
  __device__ __forceinline__ long long pitch() const { return RW; }
  __device__ __forceinline__ long long at(int i, int j) const { return (long long)(j - oy) * RW + (i - ox); }
  __device__ __forceinline__ long long mxi(int i, int j, int sx) const { (void)sx; return at(i, j); }
  __device__ __forceinline__ long long myi(int i, int j, int sy) const { (void)sy; return at(i, j); }
};

template <int TH, int D>
struct TbGeo {
  static constexpr int R = 2 * D;              // halo: 2 cells per time step
  static constexpr int RW = BTX + 2 * R, RH = TH + 2 * R, RC = RW * RH;
  static constexpr size_t SMEM = size_t(16) * RC * sizeof(float);
};

// Temporal blocking: D time steps of every running shot per grid-barrier
// phase (see the file comment). Items are (shot, i0, j0, -) tiles of 32 x TH.
template <int TH, int D>
__global__ void __launch_bounds__(BNT, TH == 8 ? 4 : (D == 2 ? 3 : 2)) batch2d_tb_kernel(BatchArgs a) {
  using G = TbGeo<TH, D>;
  constexpr int R = G::R, RW = G::RW, RC = G::RC;
  extern __shared__ __align__(16) float reg[];
  __shared__ Shot2D shd;
  static_assert(sizeof(Shot2D) % 8 == 0, "descriptor copied in 8-byte words");
  const int tid = threadIdx.x;
  unsigned nbar = 0;
  int phase = 0;
  for (int t = 0; t < a.max_nstep; t += D, ++phase) {
    const int n = a.items_at[t];
    const Shot2D* SA = (phase & 1) ? a.shots_alt : a.shots;   // holds time step t
    const Shot2D* SB = (phase & 1) ? a.shots : a.shots_alt;   // receives step t + k
    for (int q = blockIdx.x; q < n; q += gridDim.x) {
      const int4 itm = a.items[q];
      __syncthreads();   // the previous item is done with shd and the region
      {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(SA + itm.x);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(&shd);
        for (int w = tid; w < (int)(sizeof(Shot2D) / 8); w += BNT) dst[w] = src[w];
      }
      __syncthreads();
      const Shot2D& S = shd;
      const int k = min(D, a.shot_nstep[itm.x] - t);  // steps of this shot in this phase
      const int i0 = itm.y, j0 = itm.z, ox = i0 - R, oy = j0 - R;
      const RegionView<RW, RC> V{reg, ox, oy};
      const int wx = S.ax.width(), wy = S.ay.width();
      const bool xs = wx > 0 && (ox < S.ax.lo || ox + RW > S.nx - S.ax.hi);
      const bool ys = wy > 0 && (oy < S.ay.lo || oy + G::RH > S.ny - S.ay.hi);
      // stage the region (zero outside the grid; the updates never read there)
      for (int c = tid; c < RC; c += BNT) {
        const int gi = ox + c % RW, gj = oy + c / RW;
        const bool in = gi >= 0 && gi < S.nx && gj >= 0 && gj < S.ny;
        const long long g = (long long)gj * S.px + gi;
        reg[c] = in ? S.vx[g] : 0.f;
        reg[RC + c] = in ? S.vy[g] : 0.f;
        reg[2 * RC + c] = in ? S.sxx[g] : 0.f;
        reg[3 * RC + c] = in ? S.syy[g] : 0.f;
        reg[4 * RC + c] = in ? S.sxy[g] : 0.f;
        if (S.het) {
          reg[5 * RC + c] = in ? S.lam[g] : 0.f;
          reg[6 * RC + c] = in ? S.mu[g] : 0.f;
          reg[7 * RC + c] = in ? S.rho[g] : 0.f;
        }
        if (xs) {
          const int sx = in ? S.ax.slab(gi) : -1;
          const long long m = (long long)gj * wx + sx;
#pragma unroll
          for (int v = 0; v < 4; ++v) reg[(8 + v) * RC + c] = sx >= 0 ? S.mx[v][m] : 0.f;
        }
        if (ys) {
          const int sy = in ? S.ay.slab(gj) : -1;
          const long long m = (long long)sy * S.px + gi;
#pragma unroll
          for (int v = 0; v < 4; ++v) reg[(12 + v) * RC + c] = sy >= 0 ? S.my[v][m] : 0.f;
        }
      }
      __syncthreads();
      // the tile grown by e cells, inside the grid (e is a compile-time
      // constant on full phases, so the cell index splits without a division)
      auto sweep = [&](int e, auto&& fn) {
        const int w = BTX + 2 * e, h = TH + 2 * e;
        for (int c = tid; c < w * h; c += BNT) {
          const int gi = i0 - e + c % w, gj = j0 - e + c / w;
          if (gi >= 0 && gi < S.nx && gj >= 0 && gj < S.ny) fn(gi, gj);
        }
      };
      auto substep = [&](int u, int es) {
        sweep(es, [&](int gi, int gj) {
          if (S.het) stress2d_cell<true>(S, V, gi, gj);
          else stress2d_cell<false>(S, V, gi, gj);
        });
        __syncthreads();
        sweep(es - 1, [&](int gi, int gj) {
          float ek = 0.f, ep = 0.f, vm2 = 0.f;
          int bad = 0;
          if (S.het) velocity2d_cell<true>(S, V, gi, gj, t + u + 1, ek, ep, vm2, bad);
          else velocity2d_cell<false>(S, V, gi, gj, t + u + 1, ek, ep, vm2, bad);
          if (bad && gi >= i0 && gi < i0 + BTX && gj >= j0 && gj < j0 + TH) atomicOr(a.err, 4);
        });
        __syncthreads();
        // receivers in this tile, sample of step t + u + 1
        for (int r = a.item_rb[q] + tid; r < a.item_rb[q + 1]; r += BNT) {
          const int cell = a.rec[r].y;
          const long long rc = V.at(cell % S.px, cell / S.px);
          a.seis[a.rec_off[r] + t + u] = reg[rc];
          a.seis[a.rec_offy[r] + t + u] = reg[RC + rc];
        }
      };
      if (k == D) {
#pragma unroll
        for (int u = 0; u < D; ++u) substep(u, 2 * (D - u) - 1);
      } else {   // the last phase of a shot whose NSTEP is not a multiple of D
        for (int u = 0; u < k; ++u) substep(u, 2 * (k - u) - 1);
      }
      // own cells to the other buffer set
      const Shot2D& W = SB[itm.x];
      float* const wf[5] = {W.vx, W.vy, W.sxx, W.syy, W.sxy};
      for (int c = tid; c < BTX * TH; c += BNT) {
        const int gi = i0 + c % BTX, gj = j0 + c / BTX;
        if (gi >= S.nx || gj >= S.ny) continue;
        const long long g = (long long)gj * S.px + gi;
        const long long rc = V.at(gi, gj);
#pragma unroll
        for (int f = 0; f < 5; ++f) wf[f][g] = reg[f * RC + rc];
        if (xs) {
          const int sx = S.ax.slab(gi);
          if (sx >= 0)
#pragma unroll
            for (int v = 0; v < 4; ++v) W.mx[v][(long long)gj * wx + sx] = reg[(8 + v) * RC + rc];
        }
        if (ys) {
          const int sy = S.ay.slab(gj);
          if (sy >= 0)
#pragma unroll
            for (int v = 0; v < 4; ++v) W.my[v][(long long)sy * S.px + gi] = reg[(12 + v) * RC + rc];
        }
      }
    }
    if (!grid_sync(a, nbar)) return;
  }
}

}  // namespace cpml

using namespace cpml;

namespace {
const double kPi = 3.141592653589793238462643;

double stf(const cpml_params& p, int it) {  // 2D:644-654
  const double a = kPi * kPi * p.f0 * p.f0;
  const double tt = double(it - 1) * p.deltat - p.t0;
  const double tt2 = tt * tt;
  if (p.stf == CPML_STF_GAUSSIAN) return p.factor * std::exp(-(a * tt2));
  if (p.stf == CPML_STF_RICKER) return p.factor * (1.0 - 2.0 * a * tt2) * std::exp(-(a * tt2));
  return -(p.factor * 2.0 * a * tt * std::exp(-(a * tt2)));
}

struct HostShot {
  cpml_params p;
  int px = 0;
  Shot2D s{};
  Shot2D alt{};            // s on the second buffer set (temporal blocking)
  std::vector<int> rec;    // padded cells
  std::vector<int> recij;  // 1-based pairs
  double rho_src[2];
  float* seis = nullptr;   // [2][nrec][nstep]
  float* model = nullptr;  // [3][px*ny]
};
}  // namespace

struct cpml_batch {
  std::vector<HostShot> shots;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  Shot2D* d_shots = nullptr;
  Shot2D* d_shots_alt = nullptr;
  int* d_item_rb = nullptr;
  int* d_shot_nstep = nullptr;
  int depth = 1, tile_y = 8;   // time steps per phase, tile rows (1: the two-barrier kernel)
  bool alt_ready = false;      // second buffer sets allocated
  int trial_steps = 0;         // >0: runs stop after this many steps (autotuning trials)
  int4* d_items = nullptr;
  int* d_items_at = nullptr;
  int* d_recs_at = nullptr;
  int2* d_rec = nullptr;
  long long* d_rec_off = nullptr;
  long long* d_rec_offy = nullptr;
  float* d_seis = nullptr;
  unsigned* d_bar = nullptr;
  int* d_err = nullptr;
  size_t seis_floats = 0;
  int max_nstep = 0;
  int grid = 0;
  bool dirty = true;
  long long wait_cycles = 0;  // 0: the default bound of a grid-barrier wait
  cudaGraphExec_t graph = nullptr;
  bool graph_ok = false;
  BatchArgs args{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  std::vector<size_t> field_bytes;  // per shot, for reset
};

namespace {
#define BCK(x)                                                              \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) {                                                \
      cudaGetLastError();                                                   \
      return e_ == cudaErrorMemoryAllocation ? CPML_ERR_OOM : CPML_ERR_CUDA; \
    }                                                                       \
  } while (0)

template <typename T>
int balloc(cpml_batch* b, T** out, size_t n) {
  *out = nullptr;
  if (n == 0) return CPML_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) { cudaGetLastError(); return e == cudaErrorMemoryAllocation ? CPML_ERR_OOM : CPML_ERR_CUDA; }
  b->allocs.push_back(p);
  *out = (T*)p;
  return CPML_OK;
}

// Replaces *slot by a fresh buffer of n elements and releases the old one
// (cudaFree waits for the device, so no launch still reads it); on failure
// *slot is left as it was.
template <typename T>
int brealloc(cpml_batch* b, T** slot, size_t n) {
  T* fresh = nullptr;
  int st = balloc(b, &fresh, n);
  if (st) return st;
  if (*slot) {
    for (size_t i = 0; i < b->allocs.size(); ++i)
      if (b->allocs[i] == (void*)*slot) {
        b->allocs[i] = b->allocs.back();
        b->allocs.pop_back();
        cudaFree((void*)*slot);
        break;
      }
  }
  *slot = fresh;
  return CPML_OK;
}

// FP64 profile of one axis on the GPU, slab extents from its a / a_half.
int shot_axis(cpml_batch* b, const cpml_params& p, int axis, int n, double delta, Axis* A) {
  ProfileArgs P{};
  P.n = n; P.npml = p.npoints_pml; P.use_min = p.use_pml[2 * axis]; P.use_max = p.use_pml[2 * axis + 1];
  P.high_cells = n - 1;
  P.delta = delta; P.cp = p.cp; P.f0 = p.f0; P.dt = p.deltat; P.npower = p.npower; P.kmax = p.k_max_pml;
  P.amax = p.alpha_max_pml < 0 ? 2.0 * kPi * (p.f0 / 2.0) : p.alpha_max_pml;
  P.rcoef = p.rcoef;
  double* d64 = nullptr;
  float* d32 = nullptr;
  int st;
  if ((st = balloc(b, &d64, size_t(10) * n))) return st;
  if ((st = balloc(b, &d32, size_t(6) * n))) return st;
  launch_build_profile(P, d64, d32, b->stream);
  std::vector<double> hp(size_t(10) * n);
  BCK(cudaMemcpyAsync(hp.data(), d64, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  auto nzero = [&](int i) { return hp[3 * size_t(n) + i] != 0.0 || hp[8 * size_t(n) + i] != 0.0; };
  int lo = 0, hi = 0;
  for (int i = 0; i < n / 2; ++i) if (nzero(i)) lo = i + 1;
  for (int i = n - 1; i >= n / 2; --i) if (nzero(i)) hi = n - i;
  for (int i = lo; i < n - hi; ++i)
    if (nzero(i)) { lo = n; hi = 0; break; }
  A->a = d32; A->b = d32 + n; A->ik = d32 + 2 * n; A->ah = d32 + 3 * n; A->bh = d32 + 4 * n;
  A->ikh = d32 + 5 * n; A->n = n; A->lo = lo; A->hi = hi;
  return CPML_OK;
}

int upload_source(cpml_batch* b, HostShot& H, float** fx, float** fy) {
  const cpml_params& p = H.p;
  const double ang = p.angle_force * (kPi / 180.0);
  std::vector<float> x(p.nstep), y(p.nstep);
  for (int it = 1; it <= p.nstep; ++it) {
    const double st = stf(p, it);
    x[it - 1] = float(std::sin(ang) * st * p.deltat / H.rho_src[0]);
    y[it - 1] = float(std::cos(ang) * st * p.deltat / H.rho_src[1]);
  }
  int st;
  if (!*fx && (st = balloc(b, fx, p.nstep))) return st;
  if (!*fy && (st = balloc(b, fy, p.nstep))) return st;
  BCK(cudaMemcpyAsync(*fx, x.data(), sizeof(float) * p.nstep, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(*fy, y.data(), sizeof(float) * p.nstep, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return CPML_OK;
}

// The kernel of a (depth, tile rows) choice and its dynamic shared memory;
// *fn = nullptr for an unsupported pair.
void kernel_for(int depth, int tile_y, const void** fn, size_t* smem) {
  *fn = nullptr;
  *smem = 0;
  if (depth == 1 && tile_y == 8) { *fn = (const void*)batch2d_kernel; return; }
  if (depth == 2 && tile_y == 8) { *fn = (const void*)batch2d_tb_kernel<8, 2>; *smem = TbGeo<8, 2>::SMEM; }
  if (depth == 2 && tile_y == 16) { *fn = (const void*)batch2d_tb_kernel<16, 2>; *smem = TbGeo<16, 2>::SMEM; }
  if (depth == 3 && tile_y == 16) { *fn = (const void*)batch2d_tb_kernel<16, 3>; *smem = TbGeo<16, 3>::SMEM; }
}

// The second buffer set of every shot (fields and memory variables) that
// temporal blocking alternates with the first.
int alloc_alt(cpml_batch* b) {
  if (b->alt_ready) return CPML_OK;
  for (HostShot& H : b->shots) {
    const size_t n = size_t(H.px) * H.p.ny;
    Shot2D A = H.s;
    float* f = nullptr;
    int st;
    if ((st = balloc(b, &f, 5 * n))) return st;
    A.vx = f; A.vy = f + n; A.sxx = f + 2 * n; A.syy = f + 3 * n; A.sxy = f + 4 * n;
    const size_t wx = H.s.ax.width(), wy = H.s.ay.width();
    for (int v = 0; v < 4; ++v) {
      if ((st = balloc(b, &A.mx[v], wx * H.p.ny))) return st;
      if ((st = balloc(b, &A.my[v], wy * size_t(H.px)))) return st;
    }
    H.alt = A;
  }
  b->alt_ready = true;
  return CPML_OK;
}

int build_schedule(cpml_batch* b) {
  const int ns = (int)b->shots.size();
  std::vector<int> order(ns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->shots[x].p.nstep > b->shots[y].p.nstep; });
  b->max_nstep = ns ? b->shots[order[0]].p.nstep : 0;
  std::vector<int4> items;
  std::vector<int> items_end(ns), recs_end(ns);
  std::vector<int2> rec;
  std::vector<long long> off, offy;
  size_t seis_total = 0;
  std::vector<size_t> seis_base(ns);
  for (int s = 0; s < ns; ++s) {
    HostShot& H = b->shots[s];
    seis_base[s] = seis_total;
    seis_total += size_t(2) * H.rec.size() * H.p.nstep;
  }
  // depth 1: 32 x 8 tiles, receivers grouped by shot (recorded from HBM after
  // each step); temporal blocking: 32 x tile_y tiles, receivers grouped by the
  // tile that holds them (recorded from the staged region)
  const bool tb = b->depth > 1;
  const int th = tb ? b->tile_y : BTY;
  std::vector<int> item_rb(1, 0);
  for (int k = 0; k < ns; ++k) {
    const int s = order[k];
    const HostShot& H = b->shots[s];
    const size_t nr = H.rec.size();
    for (int j0 = 0; j0 < H.p.ny; j0 += th)
      for (int i0 = 0; i0 < H.p.nx; i0 += BTX) {
        items.push_back(make_int4(s, i0, j0, 0));
        if (!tb) continue;
        for (size_t r = 0; r < nr; ++r) {
          const int i = H.rec[r] % H.px, j = H.rec[r] / H.px;
          if (i < i0 || i >= i0 + BTX || j < j0 || j >= j0 + th) continue;
          rec.push_back(make_int2(s, H.rec[r]));
          off.push_back((long long)(seis_base[s] + r * H.p.nstep));
          offy.push_back((long long)(seis_base[s] + (nr + r) * H.p.nstep));
        }
        item_rb.push_back((int)rec.size());
      }
    items_end[k] = (int)items.size();
    if (!tb)
      for (size_t r = 0; r < nr; ++r) {
        rec.push_back(make_int2(s, H.rec[r]));
        off.push_back((long long)(seis_base[s] + r * H.p.nstep));
        offy.push_back((long long)(seis_base[s] + (nr + r) * H.p.nstep));
      }
    recs_end[k] = (int)rec.size();
  }
  std::vector<int> items_at(b->max_nstep), recs_at(b->max_nstep);
  for (int t = 0; t < b->max_nstep; ++t) {
    int k = 0;
    while (k < ns && b->shots[order[k]].p.nstep > t) ++k;   // shots running at step t
    items_at[t] = k ? items_end[k - 1] : 0;
    recs_at[t] = k ? recs_end[k - 1] : 0;
  }
  int st;
  if ((st = brealloc(b, &b->d_items, std::max<size_t>(items.size(), 1)))) return st;
  if ((st = brealloc(b, &b->d_items_at, std::max(b->max_nstep, 1)))) return st;
  if ((st = brealloc(b, &b->d_recs_at, std::max(b->max_nstep, 1)))) return st;
  if ((st = brealloc(b, &b->d_rec, std::max<size_t>(rec.size(), 1)))) return st;
  if ((st = brealloc(b, &b->d_rec_off, std::max<size_t>(off.size(), 1)))) return st;
  if ((st = brealloc(b, &b->d_rec_offy, std::max<size_t>(offy.size(), 1)))) return st;
  if ((st = brealloc(b, &b->d_seis, std::max<size_t>(seis_total, 1)))) return st;
  if ((st = brealloc(b, &b->d_item_rb, item_rb.size()))) return st;
  BCK(cudaMemcpy(b->d_item_rb, item_rb.data(), sizeof(int) * item_rb.size(), cudaMemcpyHostToDevice));
  std::vector<int> nsteps(ns);
  for (int s = 0; s < ns; ++s) nsteps[s] = b->shots[s].p.nstep;
  if ((st = brealloc(b, &b->d_shot_nstep, std::max(ns, 1)))) return st;
  BCK(cudaMemcpy(b->d_shot_nstep, nsteps.data(), sizeof(int) * ns, cudaMemcpyHostToDevice));
  b->seis_floats = seis_total;
  if (!items.empty()) BCK(cudaMemcpy(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
  if (b->max_nstep) {
    BCK(cudaMemcpy(b->d_items_at, items_at.data(), sizeof(int) * b->max_nstep, cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->d_recs_at, recs_at.data(), sizeof(int) * b->max_nstep, cudaMemcpyHostToDevice));
  }
  if (!rec.empty()) {
    BCK(cudaMemcpy(b->d_rec, rec.data(), sizeof(int2) * rec.size(), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->d_rec_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->d_rec_offy, offy.data(), sizeof(long long) * offy.size(), cudaMemcpyHostToDevice));
  }
  for (int s = 0; s < ns; ++s) b->shots[s].seis = b->d_seis + seis_base[s];
  // shot descriptors, on both buffer sets
  std::vector<Shot2D> ds(ns), da(ns);
  for (int s = 0; s < ns; ++s) { ds[s] = b->shots[s].s; da[s] = b->alt_ready ? b->shots[s].alt : b->shots[s].s; }
  if (!b->d_shots && (st = balloc(b, &b->d_shots, std::max(ns, 1)))) return st;
  if (!b->d_shots_alt && (st = balloc(b, &b->d_shots_alt, std::max(ns, 1)))) return st;
  BCK(cudaMemcpy(b->d_shots, ds.data(), sizeof(Shot2D) * ns, cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_shots_alt, da.data(), sizeof(Shot2D) * ns, cudaMemcpyHostToDevice));
  // resident grid: every CTA must be co-resident for the grid barrier
  int dev = 0, nsm = 0, per_sm = 0;
  BCK(cudaGetDevice(&dev));
  BCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const void* fn = nullptr;
  size_t smem = 0;
  kernel_for(b->depth, b->tile_y, &fn, &smem);
  if (!fn) return CPML_ERR_INVALID;
  if (smem > 48 * 1024) BCK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BNT, smem));
  const int first = b->max_nstep ? items_at[0] : 1;
  b->grid = std::max(1, std::min(nsm * std::max(per_sm, 1), first));
  BatchArgs& A = b->args;
  A.shots = b->d_shots; A.shots_alt = b->d_shots_alt; A.item_rb = b->d_item_rb;
  A.shot_nstep = b->d_shot_nstep;
  A.items = b->d_items; A.items_at = b->d_items_at; A.recs_at = b->d_recs_at;
  A.rec = b->d_rec; A.rec_off = b->d_rec_off; A.rec_offy = b->d_rec_offy; A.seis = b->d_seis;
  A.max_nstep = b->trial_steps > 0 ? std::min(b->max_nstep, b->trial_steps) : b->max_nstep;
  A.bar = b->d_bar; A.err = b->d_err;
  A.wait_cycles = b->wait_cycles > 0 ? b->wait_cycles : kBarrierCycles;
  b->dirty = false;
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  b->graph_ok = false;
  return CPML_OK;
}

cudaError_t launch_batch(cpml_batch* b) {
  const void* fn = nullptr;
  size_t smem = 0;
  kernel_for(b->depth, b->tile_y, &fn, &smem);
  if (!fn) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(b->grid);
  cfg.blockDim = dim3(BNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = b->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {&b->args};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

int zero_batch(cpml_batch* b) {
  for (HostShot& H : b->shots) {
    const size_t n = size_t(H.px) * H.p.ny;
    for (const Shot2D* S : {&H.s, &H.alt}) {
      if (S == &H.alt && !b->alt_ready) continue;
      for (float* f : {S->vx, S->vy, S->sxx, S->syy, S->sxy}) BCK(cudaMemsetAsync(f, 0, 4 * n, b->stream));
      const size_t wx = S->ax.width(), wy = S->ay.width();
      for (int v = 0; v < 4; ++v) {
        if (S->mx[v]) BCK(cudaMemsetAsync(S->mx[v], 0, 4 * wx * H.p.ny, b->stream));
        if (S->my[v]) BCK(cudaMemsetAsync(S->my[v], 0, 4 * wy * size_t(H.px), b->stream));
      }
    }
  }
  if (b->d_seis) BCK(cudaMemsetAsync(b->d_seis, 0, 4 * std::max<size_t>(b->seis_floats, 1), b->stream));
  BCK(cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned), b->stream));
  BCK(cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream));
  return CPML_OK;
}

int validate2d(const cpml_params& p) {
  if (p.ndim != 2 || p.nx < 3 || p.ny < 3 || p.nstep < 1 || p.npoints_pml < 1) return CPML_ERR_INVALID;
  if (!(p.deltax > 0) || !(p.deltay > 0) || !(p.deltat > 0) || !(p.cp > 0) || !(p.cs > 0) || !(p.rho > 0))
    return CPML_ERR_INVALID;
  if (!(p.rcoef > 0 && p.rcoef < 1) || p.npower < 1) return CPML_ERR_INVALID;
  if (p.stf < CPML_STF_DGAUSSIAN || p.stf > CPML_STF_RICKER) return CPML_ERR_INVALID;
  // the batched engine runs the second-order C-PML program only: a
  // fourth-order or split-field shot would otherwise run the wrong program
  if ((p.order != 0 && p.order != 2) || p.scheme != CPML_SCHEME_CPML) return CPML_ERR_INVALID;
  if (p.isource < 1 || p.isource > p.nx - 1 || p.jsource < 1 || p.jsource > p.ny - 1) return CPML_ERR_INVALID;
  if (cpml_courant(&p, p.cp) > 1.0) return CPML_ERR_CFL;
  return CPML_OK;
}
}  // namespace

extern "C" {

int cpml_batch_create(int nshots, const cpml_params* params, cpml_batch** out) {
  if (!out || nshots < 1 || !params) return CPML_ERR_INVALID;
  *out = nullptr;
  for (int s = 0; s < nshots; ++s) {
    int st = validate2d(params[s]);
    if (st) return st;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) { cudaGetLastError(); return CPML_ERR_CUDA; }
  cpml_batch* b = new cpml_batch();
  auto fail = [&](int code) { cpml_batch_destroy(b); return code; };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(CPML_ERR_CUDA);
  if (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) return fail(CPML_ERR_CUDA);
  int st;
  if ((st = balloc(b, &b->d_bar, 2))) return fail(st);
  if ((st = balloc(b, &b->d_err, 1))) return fail(st);
  b->shots.resize(nshots);
  for (int s = 0; s < nshots; ++s) {
    HostShot& H = b->shots[s];
    H.p = params[s];
    const cpml_params& p = H.p;
    H.px = (p.nx + 31) / 32 * 32;
    Shot2D& S = H.s;
    S.nx = p.nx; S.ny = p.ny; S.px = H.px; S.npml = p.npoints_pml; S.het = 0;
    S.odx = float(1.0 / p.deltax); S.ody = float(1.0 / p.deltay); S.dt = float(p.deltat);
    const double lam = p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs), mu = p.rho * p.cs * p.cs;
    S.dt_lam = float(p.deltat * lam); S.dt_mu = float(p.deltat * mu); S.dt_l2m = float(p.deltat * (lam + 2.0 * mu));
    S.dt_over_rho = float(p.deltat / p.rho);
    S.half_rho = float(0.5 * p.rho); S.inv_2mu = float(1.0 / (2.0 * mu));
    const double den = 4.0 * mu * (lam + mu);
    S.e_c1 = float((lam + 2.0 * mu) / den); S.e_c2 = float(lam / den);
    if ((st = shot_axis(b, p, 0, p.nx, p.deltax, &S.ax))) return fail(st);
    if ((st = shot_axis(b, p, 1, p.ny, p.deltay, &S.ay))) return fail(st);
    const size_t n = size_t(H.px) * p.ny;
    float* f = nullptr;
    if ((st = balloc(b, &f, 5 * n))) return fail(st);
    S.vx = f; S.vy = f + n; S.sxx = f + 2 * n; S.syy = f + 3 * n; S.sxy = f + 4 * n;
    const size_t wx = S.ax.width(), wy = S.ay.width();
    for (int v = 0; v < 4; ++v) {
      if ((st = balloc(b, &S.mx[v], wx * p.ny))) return fail(st);
      if ((st = balloc(b, &S.my[v], wy * size_t(H.px)))) return fail(st);
    }
    S.isrc = p.isource - 1; S.jsrc = p.jsource - 1;
    H.rho_src[0] = H.rho_src[1] = p.rho;
    float *fx = nullptr, *fy = nullptr;
    if ((st = upload_source(b, H, &fx, &fy))) return fail(st);
    S.src_fx = fx; S.src_fy = fy;
  }
  *out = b;
  return CPML_OK;
}

int cpml_batch_set_model(cpml_batch* b, int shot, const float* lam, const float* mu, const float* rho) {
  if (!b || shot < 0 || shot >= (int)b->shots.size() || !lam || !mu || !rho) return CPML_ERR_INVALID;
  HostShot& H = b->shots[shot];
  const cpml_params& p = H.p;
  const size_t n = size_t(p.nx) * p.ny, np = size_t(H.px) * p.ny;
  double cpm = 0.0;
  for (size_t c = 0; c < n; ++c) {
    if (!(rho[c] > 0) || !(mu[c] > 0) || !(lam[c] + 2 * mu[c] > 0)) return CPML_ERR_INVALID;
    cpm = std::max(cpm, std::sqrt((double(lam[c]) + 2.0 * mu[c]) / rho[c]));
  }
  if (cpml_courant(&p, cpm) > 1.0) return CPML_ERR_CFL;
  int st;
  if (!H.model && (st = balloc(b, &H.model, 3 * np))) return st;
  const float* src[3] = {lam, mu, rho};
  for (int q = 0; q < 3; ++q) {
    BCK(cudaMemset2DAsync(H.model + q * np, 4 * H.px, 0, 4 * H.px, p.ny, b->stream));
    BCK(cudaMemcpy2DAsync(H.model + q * np, 4 * H.px, src[q], 4 * size_t(p.nx), 4 * size_t(p.nx), p.ny,
                          cudaMemcpyHostToDevice, b->stream));
  }
  H.s.lam = H.model; H.s.mu = H.model + np; H.s.rho = H.model + 2 * np; H.s.het = 1;
  if (b->alt_ready) { H.alt.lam = H.s.lam; H.alt.mu = H.s.mu; H.alt.rho = H.s.rho; H.alt.het = 1; }
  const int i = p.isource, j = p.jsource;
  auto R = [&](int i1, int j1) { return double(rho[size_t(j1 - 1) * p.nx + (i1 - 1)]); };
  H.rho_src[0] = R(i, j);
  H.rho_src[1] = 0.25 * (R(i, j) + R(i + 1, j) + R(i + 1, j + 1) + R(i, j + 1));  // 2D:661
  float* fx = const_cast<float*>(H.s.src_fx);
  float* fy = const_cast<float*>(H.s.src_fy);
  if ((st = upload_source(b, H, &fx, &fy))) return st;
  b->dirty = true;
  return CPML_OK;
}

int cpml_batch_set_receivers(cpml_batch* b, int shot, int nrec, const int* ix, const int* iy) {
  if (!b || shot < 0 || shot >= (int)b->shots.size() || nrec < 0 || (nrec > 0 && (!ix || !iy)))
    return CPML_ERR_INVALID;
  HostShot& H = b->shots[shot];
  std::vector<int> cells(nrec), ij(2 * size_t(nrec));
  for (int r = 0; r < nrec; ++r) {
    if (ix[r] < 1 || ix[r] > H.p.nx || iy[r] < 1 || iy[r] > H.p.ny) return CPML_ERR_INVALID;
    cells[r] = (iy[r] - 1) * H.px + (ix[r] - 1);
    ij[2 * r] = ix[r]; ij[2 * r + 1] = iy[r];
  }
  H.rec = cells;
  H.recij = ij;
  b->dirty = true;
  return CPML_OK;
}

int cpml_batch_run(cpml_batch* b) {
  if (!b) return CPML_ERR_INVALID;
  int st;
  if (b->dirty && (st = build_schedule(b))) return st;
  if ((st = zero_batch(b))) return st;
  BCK(cudaEventRecord(b->ev0, b->stream));
  if (!b->graph && !b->graph_ok) {
    // one cooperative launch, captured once and replayed on later runs
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const cudaError_t le = launch_batch(b);
      const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      ok = le == cudaSuccess && ce == cudaSuccess && g &&
           cudaGraphInstantiate(&b->graph, g, 0) == cudaSuccess;
      if (g) cudaGraphDestroy(g);
    }
    if (!ok) { cudaGetLastError(); b->graph = nullptr; }
    b->graph_ok = true;
  }
  if (b->graph) BCK(cudaGraphLaunch(b->graph, b->stream));
  else BCK(launch_batch(b));
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaEventSynchronize(b->ev1));
  float ms = 0;
  BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->last_ms = ms;
  int err = 0;
  BCK(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err & 2) return CPML_ERR_TIMEOUT;
  if (err & 4) return CPML_ERR_UNSTABLE;
  return CPML_OK;
}

int cpml_batch_get_seismograms(cpml_batch* b, int shot, double* vx, double* vy) {
  if (!b || shot < 0 || shot >= (int)b->shots.size()) return CPML_ERR_INVALID;
  HostShot& H = b->shots[shot];
  if (b->dirty || !H.seis) return CPML_ERR_NOT_READY;
  const size_t nr = H.rec.size(), ns = H.p.nstep;
  if (nr == 0) return CPML_OK;
  std::vector<float> buf(2 * nr * ns);
  BCK(cudaMemcpy(buf.data(), H.seis, sizeof(float) * buf.size(), cudaMemcpyDeviceToHost));
  for (size_t q = 0; q < nr * ns; ++q) {
    if (vx) vx[q] = buf[q];
    if (vy) vy[q] = buf[nr * ns + q];
  }
  return CPML_OK;
}

int cpml_batch_get_field(cpml_batch* b, int shot, int field, float* out) {
  if (!b || shot < 0 || shot >= (int)b->shots.size() || !out) return CPML_ERR_INVALID;
  HostShot& H = b->shots[shot];
  // temporal blocking alternates the buffer sets once per phase of `depth`
  // steps: a shot that ran an odd number of phases ends on its second set
  const int phases = (H.p.nstep + b->depth - 1) / b->depth;
  const Shot2D& S = (b->depth > 1 && (phases & 1)) ? H.alt : H.s;
  const float* f = nullptr;
  switch (field) {
    case CPML_FIELD_VX: f = S.vx; break;
    case CPML_FIELD_VY: f = S.vy; break;
    case CPML_FIELD_SXX: f = S.sxx; break;
    case CPML_FIELD_SYY: f = S.syy; break;
    case CPML_FIELD_SXY: f = S.sxy; break;
    default: return CPML_ERR_INVALID;
  }
  BCK(cudaMemcpy2D(out, 4 * size_t(H.p.nx), f, 4 * size_t(H.px), 4 * size_t(H.p.nx), H.p.ny,
                   cudaMemcpyDeviceToHost));
  return CPML_OK;
}

int cpml_batch_set_wait_limit(cpml_batch* b, long long cycles) {
  if (!b || cycles < 0) return CPML_ERR_INVALID;
  b->wait_cycles = cycles;
  b->dirty = true;   // the bound travels in the captured launch arguments
  return CPML_OK;
}

int cpml_batch_set_tuning(cpml_batch* b, int depth, int tile_y) {
  if (!b) return CPML_ERR_INVALID;
  const void* fn = nullptr;
  size_t smem = 0;
  kernel_for(depth, tile_y, &fn, &smem);
  if (!fn) return CPML_ERR_INVALID;
  int st;
  if (depth > 1 && (st = alloc_alt(b))) return st;
  b->depth = depth;
  b->tile_y = tile_y;
  b->dirty = true;
  return CPML_OK;
}

int cpml_batch_get_tuning(cpml_batch* b, int* depth, int* tile_y) {
  if (!b) return CPML_ERR_INVALID;
  if (depth) *depth = b->depth;
  if (tile_y) *tile_y = b->tile_y;
  return CPML_OK;
}

int cpml_batch_autotune(cpml_batch* b, int trial_steps, int* depth, int* tile_y, double* ms_per_step) {
  if (!b || trial_steps < 1) return CPML_ERR_INVALID;
  const int cand[4][2] = {{1, 8}, {2, 8}, {2, 16}, {3, 16}};
  int bd = 1, bt = 8, st;
  double best = 1e300;
  for (const auto& c : cand) {
    if ((st = cpml_batch_set_tuning(b, c[0], c[1]))) { b->trial_steps = 0; return st; }
    b->trial_steps = trial_steps;
    if ((st = cpml_batch_run(b)) || (st = cpml_batch_run(b))) {   // the first run builds the graph
      b->trial_steps = 0;
      b->dirty = true;
      return st;
    }
    const int steps = std::min(trial_steps, b->max_nstep);
    const double ms = b->last_ms / std::max(steps, 1);
    if (ms < best) { best = ms; bd = c[0]; bt = c[1]; }
  }
  b->trial_steps = 0;
  if ((st = cpml_batch_set_tuning(b, bd, bt))) return st;
  if (depth) *depth = bd;
  if (tile_y) *tile_y = bt;
  if (ms_per_step) *ms_per_step = best;
  return CPML_OK;
}

int cpml_batch_last_run_ms(cpml_batch* b, double* ms) {
  if (!b || !ms) return CPML_ERR_INVALID;
  *ms = b->last_ms;
  return CPML_OK;
}

void cpml_batch_destroy(cpml_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void* p : b->allocs) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
