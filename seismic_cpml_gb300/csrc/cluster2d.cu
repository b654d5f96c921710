// cluster2d.cu -- a whole small 2D grid held on chip by one thread-block
// cluster for a chunk of time steps.
//
// The 2D program's grids are small (the reference's 101 x 641 is 65 k cells,
// under 4 MB of state), so a time step is two short sweeps whose cost is set
// by launch latency and HBM round trips, not by bandwidth. Here one cluster of
// NCL CTAs (16 on GB300: the non-portable maximum) runs every step of a chunk
// in ONE launch with the fields, the per-cell model and the C-PML memory
// variables resident in shared memory: CTA r owns the grid rows
// [r R, r R + R) plus one halo row below and above. Per step (2D:556-735):
//   stress sweep over the own rows (sigma_xx/yy, sigma_xy + their memory
//   variables), then each CTA writes the boundary rows its neighbours need
//   (sigma_yy of its first row down, sigma_xy of its last row up) straight
//   into their halo rows through distributed shared memory, then a cluster
//   barrier; velocity sweep (v_x, v_y, source, rigid edges, receivers,
//   energy), the same exchange for v_x (down) and v_y (up), a cluster
//   barrier. The cell updates are the functions of cell2d.cuh on a
//   shared-memory view, so fields and seismograms are bit-identical to the
//   two-sweep kernels; the energy partials are summed per CTA instead of per
//   32 x 8 tile (the same values to rounding).
// State is read from HBM at the start of a chunk and written back at its end,
// so chunk boundaries, readbacks and restarts see the usual layout. Every CTA
// runs the same number of cluster barriers (uniform control flow), and no
// CTA reads or writes another's shared memory after the last one.
#include <algorithm>

#include <cuda_runtime.h>

#include "cpml_internal.cuh"
#include "kutil.cuh"
#include "cell2d.cuh"

namespace cpml {

constexpr int CL_THREADS = 1024;
constexpr int CL_MAX = 16;
constexpr int CL_CHUNK = 128;     // longest chunk of steps the runtime launches
constexpr int CL_REC = 64;        // receivers a CTA buffers on chip ...
constexpr int CL_RECBUF = 4096;   // ... in at most this many samples

// Shared-memory view of a CTA's band: fields and model on rows jb-1 .. je
// (own rows plus one halo row each side), x-slab memory variables on the own
// rows, y-slab ones on the own rows that lie in the y slab (from row yb).
struct BandView {
  float* f;        // 5 fields then 3 model arrays, each (rows + 2) x pp
  float* xm;       // 4 x-slab arrays, rows x wx
  float* ym;       // 4 y-slab arrays, ysl x pp
  int pp, band, jb, yb, wx, ym_stride, xm_stride;
  __device__ __forceinline__ float* vx() const { return f; }
  __device__ __forceinline__ float* vy() const { return f + band; }
  __device__ __forceinline__ float* sxx() const { return f + 2 * band; }
  __device__ __forceinline__ float* syy() const { return f + 3 * band; }
  __device__ __forceinline__ float* sxy() const { return f + 4 * band; }
  __device__ __forceinline__ const float* lam() const { return f + 5 * band; }
  __device__ __forceinline__ const float* mu() const { return f + 6 * band; }
  __device__ __forceinline__ const float* rho() const { return f + 7 * band; }
  __device__ __forceinline__ float* mx(int q) const { return xm + q * xm_stride; }
  __device__ __forceinline__ float* my(int q) const { return ym + q * ym_stride; }
  __device__ __forceinline__ long long pitch() const { return pp; }
  __device__ __forceinline__ long long at(int i, int j) const { return (long long)(j - jb + 1) * pp + i; }
  __device__ __forceinline__ long long mxi(int i, int j, int sx) const {
    (void)i;
    return (long long)(j - jb) * wx + sx;
  }
  __device__ __forceinline__ long long myi(int i, int j, int sy) const {
    (void)sy;
    return (long long)(j - yb) * pp + i;
  }
};

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// store v at the shared-memory offset of `local` in CTA `rank` of the cluster
__device__ __forceinline__ void st_peer(const float* local, unsigned rank, float v) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(r), "f"(v) : "memory");
}

template <bool HET>
__global__ void __launch_bounds__(CL_THREADS, 1)
    cluster2d_kernel(StepArgs a, int C, ClusterLayout L) {
  extern __shared__ __align__(16) float smem[];
  const int tid = threadIdx.x;
  const unsigned rank = cluster_rank();
  const int nx = a.nx, ny = a.ny;
  const int jb = min(ny, (int)rank * L.rows), je = min(ny, jb + L.rows);
  const int nrow = je - jb;
  const int band = (L.rows + 2) * L.pitch;
  const Shot2D s = shot_from_args(a);
  const int wx = s.ax.width();
  BandView V;
  V.f = smem;
  V.xm = smem + 8 * band;
  V.ym = V.xm + 4 * L.rows * wx;
  V.pp = L.pitch; V.band = band; V.jb = jb; V.wx = wx;
  V.xm_stride = L.rows * wx; V.ym_stride = L.ysl * L.pitch;
  // own rows [yb, ye) lie in the y slab (one side only: a band never holds
  // rows of both slabs)
  int yb = je;
  for (int j = jb; j < je; ++j)
    if (s.ay.slab(j) >= 0) { yb = j; break; }
  int ye = yb;
  while (ye < je && s.ay.slab(ye) >= 0) ++ye;
  V.yb = yb;

  // ---- load the band (fields and model with halo rows) from HBM ------------
  const float* const gf[8] = {a.f.vx, a.f.vy, a.f.sxx, a.f.syy, a.f.sxy, a.mdl.lam, a.mdl.mu, a.mdl.rho};
  const int nload = HET ? 8 : 5;
  const int brows = nrow + 2;
  for (int q = 0; q < nload; ++q)
    for (int c = tid; c < brows * nx; c += CL_THREADS) {
      const int r = c / nx, i = c - r * nx, j = jb - 1 + r;
      smem[q * band + r * L.pitch + i] = (j >= 0 && j < ny) ? gf[q][(long long)j * a.px + i] : 0.f;
    }
  for (int v = 0; v < 4; ++v) {
    for (int c = tid; c < nrow * wx; c += CL_THREADS) {
      const int r = c / wx, x = c - r * wx;
      V.mx(v)[r * wx + x] = a.m.x[v][(long long)(jb + r) * wx + x];
    }
    for (int c = tid; c < (ye - yb) * nx; c += CL_THREADS) {
      const int r = c / nx, i = c - r * nx, j = yb + r;
      V.my(v)[r * L.pitch + i] = a.m.y[v][(long long)s.ay.slab(j) * a.px + i];
    }
  }
  // The step loop writes nothing to HBM (a cluster barrier with release
  // semantics would wait for such writes every half step): the energy
  // partials and, when they fit, this CTA's receiver samples are kept in
  // shared memory and written out after the last step of the chunk.
  __shared__ double part_buf[CL_CHUNK][4];
  __shared__ float rec_buf[CL_RECBUF];
  __shared__ int rec_id[CL_REC];
  __shared__ int n_own;
  if (tid == 0) n_own = 0;
  __syncthreads();
  for (int r = tid; r < a.nrec; r += CL_THREADS) {
    const int j = a.rec_cell[r] / a.px;
    if (j >= jb && j < je) {
      const int q = atomicAdd(&n_own, 1);
      if (q < CL_REC) rec_id[q] = r;
    }
  }
  __syncthreads();
  const bool rec_on_chip = n_own <= CL_REC && 2 * n_own * C <= CL_RECBUF && C <= CL_CHUNK;
  __syncthreads();
  cluster_sync();

  // own cells are walked in row-major order, CL_THREADS apart
  const int ncell = nrow * nx;
  const int dj = CL_THREADS / nx, di = CL_THREADS - dj * nx;
  const int j0 = tid / nx, i0 = tid - j0 * nx;
  const int base = *a.it_base;
  for (int ls = 0; ls < C; ++ls) {
    const int it = base + ls + 1;
    // ---- stress (2D:556-600) -------------------------------------------------
    {
      int i = i0, j = jb + j0;
      for (int c = tid; c < ncell; c += CL_THREADS) {
        stress2d_cell<HET>(s, V, i, j);
        i += di; j += dj;
        if (i >= nx) { i -= nx; ++j; }
      }
    }
    __syncthreads();
    // sigma_yy of the first own row -> halo row above of the CTA below;
    // sigma_xy of the last own row -> halo row below of the CTA above
    for (int i = tid; i < nx; i += CL_THREADS) {
      if (rank > 0) st_peer(V.syy() + (long long)(L.rows + 1) * L.pitch + i, rank - 1, V.syy()[V.at(i, jb)]);
      if ((int)rank + 1 < L.ncl) st_peer(V.sxy() + i, rank + 1, V.sxy()[V.at(i, je - 1)]);
    }
    cluster_sync();
    // ---- velocity, source, rigid edges, energy (2D:606-713) ----------------
    Kahan ek, ep;
    float vm2 = 0.f;
    int bad = 0;
    {
      int i = i0, j = jb + j0;
      for (int c = tid; c < ncell; c += CL_THREADS) {
        float e1 = 0.f, e2 = 0.f;
        velocity2d_cell<HET>(s, V, i, j, it, e1, e2, vm2, bad);
        ek.add(e1);
        ep.add(e2);
        i += di; j += dj;
        if (i >= nx) { i -= nx; ++j; }
      }
    }
    __syncthreads();
    // v_x of the first own row -> the CTA below; v_y of the last -> the CTA above
    for (int i = tid; i < nx; i += CL_THREADS) {
      if (rank > 0) st_peer(V.vx() + (long long)(L.rows + 1) * L.pitch + i, rank - 1, V.vx()[V.at(i, jb)]);
      if ((int)rank + 1 < L.ncl) st_peer(V.vy() + i, rank + 1, V.vy()[V.at(i, je - 1)]);
    }
    // receivers on the own rows, sample of step it (2D:683-686)
    if (rec_on_chip) {
      for (int q = tid; q < n_own; q += CL_THREADS) {
        const int cell = a.rec_cell[rec_id[q]], j = cell / a.px, i = cell - j * a.px;
        rec_buf[2 * (q * C + ls)] = V.vx()[V.at(i, j)];
        rec_buf[2 * (q * C + ls) + 1] = V.vy()[V.at(i, j)];
      }
    } else {
      for (int r = tid; r < a.nrec; r += CL_THREADS) {
        const int cell = a.rec_cell[r], j = cell / a.px, i = cell - j * a.px;
        if (j >= jb && j < je) {
          const size_t o = (size_t)r * a.nstep + (size_t)(it - 1);
          a.seis[o] = V.vx()[V.at(i, j)];
          a.seis[(size_t)a.nrec * a.nstep + o] = V.vy()[V.at(i, j)];
        }
      }
    }
    if (C <= CL_CHUNK)
      block_partials<CL_THREADS>(ek.df(), ep.df(), vm2, bad, part_buf[ls]);
    else
      block_partials<CL_THREADS>(ek.df(), ep.df(), vm2, bad, a.partials + ((size_t)ls * a.nblocks + rank) * 4);
    cluster_sync();
  }

  // ---- the chunk's energy partials and receiver samples ---------------------
  if (C <= CL_CHUNK)
    for (int q = tid; q < 4 * C; q += CL_THREADS)
      a.partials[((size_t)(q >> 2) * a.nblocks + rank) * 4 + (q & 3)] = part_buf[q >> 2][q & 3];
  if (rec_on_chip)
    for (int q = tid; q < n_own * C; q += CL_THREADS) {
      const int k = q / C, ls = q - k * C, r = rec_id[k];
      const size_t o = (size_t)r * a.nstep + (size_t)(base + ls);
      a.seis[o] = rec_buf[2 * q];
      a.seis[(size_t)a.nrec * a.nstep + o] = rec_buf[2 * q + 1];
    }

  // ---- write the band's own rows and memory variables back -----------------
  float* const go[5] = {a.f.vx, a.f.vy, a.f.sxx, a.f.syy, a.f.sxy};
  for (int q = 0; q < 5; ++q)
    for (int c = tid; c < nrow * nx; c += CL_THREADS) {
      const int r = c / nx, i = c - r * nx, j = jb + r;
      go[q][(long long)j * a.px + i] = smem[q * band + (r + 1) * L.pitch + i];
    }
  for (int v = 0; v < 4; ++v) {
    for (int c = tid; c < nrow * wx; c += CL_THREADS) {
      const int r = c / wx, x = c - r * wx;
      a.m.x[v][(long long)(jb + r) * wx + x] = V.mx(v)[r * wx + x];
    }
    for (int c = tid; c < (ye - yb) * nx; c += CL_THREADS) {
      const int r = c / nx, i = c - r * nx, j = yb + r;
      a.m.y[v][(long long)s.ay.slab(j) * a.px + i] = V.my(v)[r * L.pitch + i];
    }
  }
}

// A cluster layout for this grid, or ncl = 0 when the grid does not fit on
// chip (or the device cannot schedule such a cluster). Every CTA must own at
// least two rows, and no CTA may own rows of both y slabs.
ClusterLayout cluster2d_layout(const StepArgs& s, bool het) {
  ClusterLayout L{};
  int dev = 0, optin = 0, cl = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return L;
  if (cudaDeviceGetAttribute(&cl, cudaDevAttrClusterLaunch, dev) != cudaSuccess || !cl) { cudaGetLastError(); return L; }
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return L;
  const int wx = s.ax.width();
  const int interior = s.ny - s.ay.lo - s.ay.hi;
  for (int ncl : {CL_MAX, 8}) {
    ClusterLayout T{};
    T.ncl = ncl;
    T.rows = (s.ny + ncl - 1) / ncl;
    if ((long long)T.rows * (ncl - 1) >= s.ny) continue;     // the last CTA would own nothing
    if (T.rows < 2 || (s.ay.lo > 0 && s.ay.hi > 0 && T.rows >= interior)) continue;
    T.pitch = (s.nx + 3) / 4 * 4;
    T.ysl = std::min(T.rows, std::max(s.ay.lo, s.ay.hi));
    T.het = het ? 1 : 0;
    T.smem = sizeof(float) * ((size_t)8 * (T.rows + 2) * T.pitch + (size_t)4 * T.rows * wx +
                              (size_t)4 * T.ysl * T.pitch);
    const void* fn = het ? (const void*)cluster2d_kernel<true> : (const void*)cluster2d_kernel<false>;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) { cudaGetLastError(); return L; }
    if (T.smem + fa.sharedSizeBytes > (size_t)optin) continue;   // static buffers count too
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T.smem) != cudaSuccess ||
        (ncl > 8 && cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ncl);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = T.smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ncl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    return T;
  }
  return L;
}

cudaError_t launch_chunk2d_cluster(const StepArgs& s, int C, bool het, const ClusterLayout& L, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(L.ncl);
  cfg.blockDim = dim3(CL_THREADS);
  cfg.dynamicSmemBytes = L.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = L.ncl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return het ? cudaLaunchKernelEx(&cfg, cluster2d_kernel<true>, s, C, L)
             : cudaLaunchKernelEx(&cfg, cluster2d_kernel<false>, s, C, L);
}

}  // namespace cpml
