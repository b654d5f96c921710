// kernels2d.cu -- 2D P-SV velocity-stress C-PML time step, two-sweep form.
//
// One time step of seismic_CPML_2D_isotropic_second_order.f90 (2D:556-713):
//   stress2d   -- sigma_xx/sigma_yy (2D:556-580) and sigma_xy (2D:582-600)
//                 with their C-PML memory variables, plus the receivers of
//                 the previous step (2D:683-686).
//   velocity2d -- v_x (2D:606-621), v_y (2D:623-641), source (2D:644-667),
//                 rigid edges (2D:670-680), energy partials (2D:694-713) and
//                 max|v|^2 (2D:718).
// persist2d runs the same two sweeps for a chunk of steps in one cooperative
// launch (grid barriers between the sweeps).
// The per-cell arithmetic lives in cell2d.cuh and is shared with the batched
// multi-shot engine, so a shot gives bit-identical results on either path.
// HET selects per-cell lambda/mu/rho with the reference's staggered averages
// (2D:559-562, 586, 627); otherwise the homogeneous constants of 2D:468-474.
#include <algorithm>

#include "cpml_internal.cuh"
#include "kutil.cuh"
#include "cell2d.cuh"

namespace cpml {

constexpr int T2X = 32, T2Y = 8;

__device__ __forceinline__ void record_receivers2d(const StepArgs& s, int it, long long gtid,
                                                   long long gsize) {
  const size_t slab = (size_t)s.nrec * s.nstep;
  for (long long r = gtid; r < s.nrec; r += gsize) {
    const long long c = s.rec_cell[r];
    const size_t o = (size_t)r * s.nstep + (size_t)(it - 1);
    s.seis[o] = s.f.vx[c];
    s.seis[slab + o] = s.f.vy[c];
  }
}

template <bool HET>
__global__ void __launch_bounds__(T2X* T2Y) stress2d(StepArgs a, int ls) {
  const int tid = threadIdx.x + threadIdx.y * T2X;
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  if (ls > 0)
    record_receivers2d(a, *a.it_base + ls, blin * (T2X * T2Y) + tid,
                       (long long)gridDim.x * gridDim.y * (T2X * T2Y));
  const int i = blockIdx.x * T2X + threadIdx.x;
  const int j = blockIdx.y * T2Y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const Shot2D s = shot_from_args(a);
  stress2d_cell<HET>(s, i, j);
}

template <bool HET>
__global__ void __launch_bounds__(T2X* T2Y) velocity2d(StepArgs a, int ls) {
  const int it = *a.it_base + ls + 1;
  const int i = blockIdx.x * T2X + threadIdx.x;
  const int j = blockIdx.y * T2Y + threadIdx.y;
  float ek = 0.f, ep = 0.f, vm2 = 0.f;
  int bad = 0;
  if (i < a.nx && j < a.ny) {
    const Shot2D s = shot_from_args(a);
    velocity2d_cell<HET>(s, i, j, it, ek, ep, vm2, bad);
  }
  const long long blin = blockIdx.x + (long long)gridDim.x * blockIdx.y;
  block_partials<T2X * T2Y>(DF{ek, 0.f}, DF{ep, 0.f}, vm2, bad,
                            a.partials + ((size_t)ls * a.nblocks + blin) * 4);
}

// Persistent form: C time steps of one shot in ONE cooperative launch, the
// same two sweeps separated by grid barriers instead of kernel boundaries.
// Tile q of the two-sweep grid (q = bx + gx * by) is handed to CTA
// q mod gridDim.x, each warp is one tile row as in the two-sweep kernels,
// and its energy partials go to the same slot, so the chunk reduction and
// every result are bit-identical to the two-sweep path. For grids too small
// to fill the GPU the step time is set by launch latency, which this form
// pays once per chunk instead of twice per step.
constexpr long long kGridWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

// Five CTAs per SM (at most 51 registers, a few bytes of spill): the kernel is
// latency-bound, and resident warps matter more than the last registers.

template <bool HET>
__global__ void __launch_bounds__(T2X* T2Y, 5) persist2d(StepArgs a, int C, unsigned* bar) {
  const int tid = threadIdx.x, tx = tid & (T2X - 1), ty = tid / T2X;
  const int gx = (a.nx + T2X - 1) / T2X;
  const int ntiles = a.nblocks;
  const int base = *a.it_base;
  const long long gtid = (long long)blockIdx.x * (T2X * T2Y) + tid;
  const long long gsize = (long long)gridDim.x * (T2X * T2Y);
  const Shot2D s = shot_from_args(a);
  unsigned nbar = 0;   // barriers passed; the arrival counter's target is nbar * CTAs
  for (int ls = 0; ls < C; ++ls) {
    if (ls > 0) record_receivers2d(a, base + ls, gtid, gsize);
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
      const int i = (q % gx) * T2X + tx, j = (q / gx) * T2Y + ty;
      if (i < a.nx && j < a.ny) stress2d_cell<HET>(s, i, j);
    }
    if (!grid_barrier(bar, ++nbar * gridDim.x, a.err, 1, kGridWaitCycles)) return;
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
      const int i = (q % gx) * T2X + tx, j = (q / gx) * T2Y + ty;
      float ek = 0.f, ep = 0.f, vm2 = 0.f;
      int bad = 0;
      if (i < a.nx && j < a.ny) velocity2d_cell<HET>(s, i, j, base + ls + 1, ek, ep, vm2, bad);
      block_partials<T2X * T2Y>(DF{ek, 0.f}, DF{ep, 0.f}, vm2, bad, a.partials + ((size_t)ls * ntiles + q) * 4);
      __syncthreads();   // block_partials' shared scratch is reused by the next tile
    }
    if (ls + 1 < C && !grid_barrier(bar, ++nbar * gridDim.x, a.err, 1, kGridWaitCycles)) return;
  }
}

// CTAs the persistent form launches: every tile's CTA if they can all be
// resident at once, else as many as can (each then takes several tiles);
// 0 if the device has no cooperative launch.
int persist2d_grid(const StepArgs& s, bool het) {
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const cudaError_t e = het ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persist2d<true>, T2X * T2Y, 0)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persist2d<false>, T2X * T2Y, 0);
  if (e != cudaSuccess || per_sm < 1) { cudaGetLastError(); return 0; }
  return std::min(s.nblocks, nsm * per_sm);
}

cudaError_t launch_chunk2d_persistent(const StepArgs& s, int C, bool het, unsigned* bar, int grid,
                                      cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(T2X * T2Y);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return het ? cudaLaunchKernelEx(&cfg, persist2d<true>, s, C, bar)
             : cudaLaunchKernelEx(&cfg, persist2d<false>, s, C, bar);
}

dim3 grid2d(const StepArgs& s) { return dim3((s.nx + T2X - 1) / T2X, (s.ny + T2Y - 1) / T2Y); }

int blocks2d(const StepArgs& s) {
  dim3 g = grid2d(s);
  return (int)(g.x * g.y);
}

void launch_step2d_two_sweep(const StepArgs& s, int ls, bool het, cudaStream_t st) {
  const dim3 g = grid2d(s), b(T2X, T2Y);
  if (het) {
    stress2d<true><<<g, b, 0, st>>>(s, ls);
    velocity2d<true><<<g, b, 0, st>>>(s, ls);
  } else {
    stress2d<false><<<g, b, 0, st>>>(s, ls);
    velocity2d<false><<<g, b, 0, st>>>(s, ls);
  }
}

}  // namespace cpml
