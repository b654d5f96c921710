// kernels2d.cu -- 2D P-SV velocity-stress C-PML time step, two-sweep form.
//
// One time step of seismic_CPML_2D_isotropic_second_order.f90 (2D:556-713):
//   stress2d   -- sigma_xx/sigma_yy (2D:556-580) and sigma_xy (2D:582-600)
//                 with their C-PML memory variables, plus the receivers of
//                 the previous step (2D:683-686).
//   velocity2d -- v_x (2D:606-621), v_y (2D:623-641), source (2D:644-667),
//                 rigid edges (2D:670-680), energy partials (2D:694-713) and
//                 max|v|^2 (2D:718).
// The per-cell arithmetic lives in cell2d.cuh and is shared with the batched
// multi-shot engine, so a shot gives bit-identical results on either path.
// HET selects per-cell lambda/mu/rho with the reference's staggered averages
// (2D:559-562, 586, 627); otherwise the homogeneous constants of 2D:468-474.
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
  block_partials<T2X * T2Y>((double)ek, (double)ep, vm2, bad,
                            a.partials + ((size_t)ls * a.nblocks + blin) * 4);
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
