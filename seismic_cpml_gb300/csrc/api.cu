// api.cu -- the libcpml runtime behind include/cpml.h.
//
// A handle owns one CUDA stream and all device state of one simulation. The
// time loop of the reference (2D:550-735, 3D:802-1245) runs as chunks of
// steps; each chunk is one CUDA graph (its step kernels, then the chunk
// reduction) replayed from a per-length cache. Kernels read the step counter
// from device memory, so one graph serves every chunk of the same length.
// Chunks end on the reference's display steps (it = 5 and multiples of
// IT_DISPLAY, 2D:716), where the host checks max|v| against the 1e25 blow-up
// threshold, exactly where the reference checks it.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>
#include <algorithm>
#include <tuple>

#include <cuda_runtime.h>

#include "../../include/cpml.h"
#include "cpml_internal.cuh"

namespace cpml {
void launch_build_profile(const ProfileArgs& P, double* out64, float* out32, cudaStream_t st);
void launch_reduce_chunk(const StepArgs& s, int C, double* ek, double* ep, double* vmax, int* bad,
                         cudaStream_t st);
void launch_step3d_two_sweep(const StepArgs& s, int ls, bool het, cudaStream_t st);
void launch_step2d_two_sweep(const StepArgs& s, int ls, bool het, cudaStream_t st);
void launch_step2d_order4(const StepArgs& s, int ls, bool het, cudaStream_t st);
void launch_step2d_split(const StepArgs& s, int ls, cudaStream_t st);
int persist2d_grid(const StepArgs& s, bool het);
ClusterLayout cluster2d_layout(const StepArgs& s, bool het);
cudaError_t launch_chunk2d_cluster(const StepArgs& s, int C, bool het, const ClusterLayout& L, cudaStream_t st);
cudaError_t launch_chunk2d_persistent(const StepArgs& s, int C, bool het, unsigned* bar, int grid,
                                      cudaStream_t st);
int blocks3d(const StepArgs& s);
int blocks2d(const StepArgs& s);
bool fused3d_supported();
size_t fused3d_plan_bytes();
bool fused3d_make_maps(void* plan_mem, float* const fields[2][9], const float* lam, const float* mu,
                       const float* rho, int nx, int ny, int nz, int px, int ty, int lz, int depth,
                       bool het);
bool fused3d_shape_ok(int ty, int depth);
void fused3d_items(int nx, int ny, int nz, const Axis& ax, const Axis& ay, const Axis& az, int npml,
                   int ty, int lz, bool het, std::vector<int4>& fast, std::vector<int4>& gen, int n_cls[4]);
void fused3d_set_items(void* plan_mem, const int4* fast, int n_fast, const int4* gen, const int n_cls[4],
                       const cudaStream_t aux[4], cudaEvent_t fork, const cudaEvent_t join[4]);
cudaError_t fused3d_launch(const void* plan_mem, const StepArgs& s, int ls, int parity, cudaStream_t st);
int fused3d_kernels_per_step(const void* plan_mem);
}  // namespace cpml

using namespace cpml;

namespace {
const double kPi = 3.141592653589793238462643;
const double kStability = 1.0e25;  // STABILITY_THRESHOLD (2D:201)
const int kMaxChunk = 128;

// FNV-1a, 64-bit: fingerprints of the parameter block, model and receivers
// that a state snapshot must match before it is loaded
const uint64_t kFnvBasis = 1469598103934665603ULL;
uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ULL; }
  return h;
}

double source_term(const cpml_params* p, int it) {  // 2D:644-654
  const double a = kPi * kPi * p->f0 * p->f0;
  const double tt = double(it - 1) * p->deltat - p->t0;
  const double tt2 = tt * tt;
  if (p->stf == CPML_STF_GAUSSIAN) return p->factor * std::exp(-(a * tt2));
  if (p->stf == CPML_STF_RICKER) return p->factor * (1.0 - 2.0 * a * tt2) * std::exp(-(a * tt2));
  return -(p->factor * 2.0 * a * tt * std::exp(-(a * tt2)));
}
}  // namespace

struct cpml_handle {
  cpml_params p{};
  int ndim = 0, nx = 0, ny = 0, nz = 1, px = 0;
  long long plane = 0;
  size_t ncellp = 0;  // padded cells
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  float* fld[9] = {};      // buffer set 0
  float* fld1[9] = {};     // buffer set 1 (fused 3D path: time n+1 while set 0 holds n)
  bool pingpong = false;   // fields alternate between the sets every step
  bool plan_ok = false;    // the last re-plan (configure_path) completed; cpml_run needs it
  bool cluster = false;    // 2D: the whole grid on chip in one cluster launch per chunk
  ClusterLayout clay{};    // its layout
  bool persist = false;    // 2D: one cooperative launch per chunk of steps
  int persist_grid = 0;    // its CTAs
  unsigned* bar = nullptr; // its grid-barrier words
  int kernel = 0;          // CPML_KERNEL_*
  int tile_y = 8, zchunk = 24, depth = 2;
  std::vector<unsigned char> plan;  // fused-path tensor maps and item lists
  cudaStream_t aux[4] = {};         // streams of the fused step's fork/join (one per general class)
  cudaEvent_t fork = nullptr, join[4] = {};
  int* err = nullptr;      // device error word
  float* prof32[3] = {};
  double* prof64[3] = {};
  Axis axes[3] = {};
  float* model[3] = {};  // lam, mu, rho (per-cell, optional)
  bool het = false;
  uint64_t model_hash = 0; // FNV-1a of the per-cell model's host arrays (0: homogeneous)
  double cp_max = 0;
  double rho_src[2] = {0, 0};  // rho used for the x / y source increments
  float* src_fx = nullptr;
  float* src_fy = nullptr;
  int nrec = 0;
  std::vector<int> rec_ijk;    // 1-based triples
  int* rec_cell = nullptr;
  float* seis = nullptr;
  double* partials = nullptr;
  int4* items_fast = nullptr;  // fused-path item lists (device copies of the plan's tables)
  int4* items_gen = nullptr;
  int nblocks = 0;
  double *ek = nullptr, *ep = nullptr, *vmax = nullptr;
  int* bad = nullptr;
  int* it_base = nullptr;
  int it = 0;
  double last_vmax = 0;
  std::map<int, cudaGraphExec_t> graphs;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  Slabs slabs{};
  Slabs slabs1{};          // stress-side memory variables of buffer set 1
  size_t partials_cap = 0;
};

namespace {

bool is_split(const cpml_handle* h) { return h->ndim == 2 && h->p.scheme == CPML_SCHEME_SPLIT; }
bool is_order4(const cpml_handle* h) { return h->ndim == 2 && h->p.order == 4; }
// the second-order 2D C-PML program: the only 2D form with a persistent kernel
bool is_standard2d(const cpml_handle* h) { return h->ndim == 2 && !is_split(h) && !is_order4(h); }

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return CPML_OK;
  if (e == cudaErrorMemoryAllocation) return CPML_ERR_OOM;
  return CPML_ERR_CUDA;
}
#define CK(x)                                   \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

template <typename T>
int dalloc(cpml_handle* h, T** out, size_t count) {
  *out = nullptr;
  if (count == 0) return CPML_OK;
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, count * sizeof(T));
  if (e != cudaSuccess) { cudaGetLastError(); return cuda_status(e); }
  h->allocs.push_back(ptr);
  *out = (T*)ptr;
  return CPML_OK;
}

// Releases one buffer that dalloc made (no-op for nullptr). cudaFree waits for
// the device, so no launch still reads it.
void dfree(cpml_handle* h, void* ptr) {
  if (!ptr) return;
  for (size_t i = 0; i < h->allocs.size(); ++i)
    if (h->allocs[i] == ptr) {
      h->allocs[i] = h->allocs.back();
      h->allocs.pop_back();
      cudaFree(ptr);
      return;
    }
}

// Replaces *slot by a fresh buffer of count elements; the old buffer is
// released only once the new one exists, so a failed call leaves *slot as it was.
template <typename T>
int drealloc(cpml_handle* h, T** slot, size_t count) {
  T* fresh = nullptr;
  int st = dalloc(h, &fresh, count);
  if (st) return st;
  dfree(h, *slot);
  *slot = fresh;
  return CPML_OK;
}

void drop_graphs(cpml_handle* h) {
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
  h->graphs.clear();
}

int validate(const cpml_params* p) {
  if (!p) return CPML_ERR_INVALID;
  if (p->ndim != 2 && p->ndim != 3) return CPML_ERR_INVALID;
  const int nz = p->ndim == 3 ? p->nz : 1;
  if (p->nx < 3 || p->ny < 3 || (p->ndim == 3 && p->nz < 3)) return CPML_ERR_INVALID;
  if (p->nstep < 1 || p->npoints_pml < 1) return CPML_ERR_INVALID;
  if (!(p->deltax > 0) || !(p->deltay > 0) || (p->ndim == 3 && !(p->deltaz > 0)) ||
      !(p->deltat > 0))
    return CPML_ERR_INVALID;
  if (!(p->cp > 0) || !(p->cs > 0) || !(p->rho > 0) || !(p->rcoef > 0 && p->rcoef < 1))
    return CPML_ERR_INVALID;
  if (p->npower < 1) return CPML_ERR_INVALID;  // 2D:293
  if (p->stf < CPML_STF_DGAUSSIAN || p->stf > CPML_STF_RICKER) return CPML_ERR_INVALID;
  if (p->isource < 1 || p->isource > p->nx - 1 || p->jsource < 1 || p->jsource > p->ny - 1)
    return CPML_ERR_INVALID;
  if (p->ndim == 3 && (p->ksource < 1 || p->ksource > nz)) return CPML_ERR_INVALID;
  if (p->it_display < 1) return CPML_ERR_INVALID;
  if (p->order != 0 && p->order != 2 && p->order != 4) return CPML_ERR_INVALID;
  if (p->scheme != CPML_SCHEME_CPML && p->scheme != CPML_SCHEME_SPLIT) return CPML_ERR_INVALID;
  if (p->order == 4 && (p->ndim != 2 || p->scheme != CPML_SCHEME_CPML)) return CPML_ERR_INVALID;
  // the split-field program has one grid spacing h (PML:100)
  if (p->scheme == CPML_SCHEME_SPLIT && (p->ndim != 2 || p->deltax != p->deltay)) return CPML_ERR_INVALID;
  const double cells = double(p->nx) * p->ny * nz;
  if (cells > 4.0e9) return CPML_ERR_RANGE;
  return CPML_OK;
}

// Arguments of a step that reads buffer set `q` (and, ping-ponged, writes 1-q).
StepArgs make_args(cpml_handle* h, int q = 0) {
  StepArgs s{};
  const cpml_params& p = h->p;
  s.nx = h->nx; s.ny = h->ny; s.nz = h->nz; s.px = h->px; s.plane = h->plane;
  s.odx = float(1.0 / p.deltax); s.ody = float(1.0 / p.deltay);
  s.odz = float(1.0 / (h->ndim == 3 ? p.deltaz : 1.0));
  s.dx = float(p.deltax); s.dy = float(p.deltay);
  s.dt = float(p.deltat);
  const double lam = p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs);
  const double mu = p.rho * p.cs * p.cs;
  const double l2m = h->ndim == 3 ? p.rho * p.cp * p.cp : lam + 2.0 * mu;  // 3D:144 / 2D:562
  s.dt_lam = float(p.deltat * lam);
  s.dt_mu = float(p.deltat * mu);
  s.dt_l2m = float(p.deltat * l2m);
  s.dt_over_rho = float(p.deltat / p.rho);
  s.half_rho = float(0.5 * p.rho);
  s.inv_2mu = float(1.0 / (2.0 * mu));
  if (h->ndim == 3) {
    const double den = 2.0 * mu * (3.0 * lam + 2.0 * mu);  // 3D:1160-1165
    s.e_c1 = float(2.0 * (lam + mu) / den);
    s.e_c2 = float(lam / den);
  } else {
    const double den = 4.0 * mu * (lam + mu);              // 2D:704-707
    s.e_c1 = float((lam + 2.0 * mu) / den);
    s.e_c2 = float(lam / den);
  }
  s.ax = h->axes[0]; s.ay = h->axes[1]; s.az = h->axes[2];
  float* const* F = (q == 0 || !h->pingpong) ? h->fld : h->fld1;
  float* const* Gd = (!h->pingpong) ? F : (q == 0 ? h->fld1 : h->fld);
  s.f.vx = F[0]; s.f.vy = F[1]; s.f.vz = F[2];
  s.f.sxx = F[3]; s.f.syy = F[4]; s.f.szz = F[5];
  s.f.sxy = F[6]; s.f.sxz = F[7]; s.f.syz = F[8];
  s.g.vx = Gd[0]; s.g.vy = Gd[1]; s.g.vz = Gd[2];
  s.g.sxx = Gd[3]; s.g.syy = Gd[4]; s.g.szz = Gd[5];
  s.g.sxy = Gd[6]; s.g.sxz = Gd[7]; s.g.syz = Gd[8];
  s.m = h->slabs;
  s.mb = h->slabs;
  if (h->pingpong) {  // stress-side memory variables (indices 0..2) alternate too
    const Slabs& A = q == 0 ? h->slabs : h->slabs1;
    const Slabs& B = q == 0 ? h->slabs1 : h->slabs;
    for (int v = 0; v < 3; ++v) {
      s.m.x[v] = A.x[v]; s.m.y[v] = A.y[v]; s.m.z[v] = A.z[v];
      s.mb.x[v] = B.x[v]; s.mb.y[v] = B.y[v]; s.mb.z[v] = B.z[v];
    }
  }
  s.err = h->err;
  s.mdl.lam = h->model[0]; s.mdl.mu = h->model[1]; s.mdl.rho = h->model[2];
  s.npml = p.npoints_pml;
  s.isrc = p.isource - 1; s.jsrc = p.jsource - 1; s.ksrc = h->ndim == 3 ? p.ksource - 1 : 0;
  s.src_fx = h->src_fx; s.src_fy = h->src_fy;
  s.nrec = h->nrec; s.rec_cell = h->rec_cell; s.seis = h->seis;
  s.nstep = p.nstep;
  s.it_base = h->it_base;
  s.partials = h->partials;
  s.nblocks = h->nblocks;
  s.ep_physical = (p.flags & CPML_FLAG_EP_PHYSICAL) ? 1 : 0;
  s.o24dx = float(1.0 / (24.0 * p.deltax));
  s.o24dy = float(1.0 / (24.0 * p.deltay));
  if (is_split(h)) {  // x parts in set 0, y parts in set 1 (PML:163-165)
    s.split = 1;
    s.g.vx = h->fld1[0]; s.g.vy = h->fld1[1];
    s.g.sxx = h->fld1[3]; s.g.syy = h->fld1[4]; s.g.sxy = h->fld1[6];
    s.lam_split = float(lam);
    s.mu_split = float(mu);
    s.l2m_split = float(p.rho * p.cp * p.cp);   // lambda_plus_two_mu = rho cp^2 (PML:111)
    s.orho_split = float(1.0 / p.rho);
  }
  return s;
}

// Per-step source increments: force * DELTAT / rho (2D:664-667, 3D:1080-1081)
int upload_source(cpml_handle* h) {
  const cpml_params& p = h->p;
  const double ang = p.angle_force * (kPi / 180.0);
  const double sa = std::sin(ang), ca = std::cos(ang);
  std::vector<float> fx(p.nstep), fy(p.nstep);
  for (int it = 1; it <= p.nstep; ++it) {
    const double st = source_term(&p, it);
    fx[it - 1] = float(sa * st * p.deltat / h->rho_src[0]);
    fy[it - 1] = float(ca * st * p.deltat / h->rho_src[1]);
  }
  CK(cudaMemcpyAsync(h->src_fx, fx.data(), sizeof(float) * p.nstep, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->src_fy, fy.data(), sizeof(float) * p.nstep, cudaMemcpyHostToDevice, h->stream));
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? CPML_OK : CPML_ERR_CUDA;
}

// Split-field PML tables of one axis (PML:180-250), built on the host in
// FP64: the damping profile divided by two at grid and half points, d and dh,
// and the relaxation factors a = 1/dt - d, b = 1/dt + d (ah, bh at half
// points) the kernels read. No memory variables: slab width 0.
int build_axis_split(cpml_handle* h, int axis, int n, double h_) {
  const cpml_params& p = h->p;
  const double delta = p.npoints_pml * h_;
  const double d0 = 3.0 * p.cp * std::log(1.0 / p.rcoef) / (2.0 * delta);
  const double ol = delta, orr = (n - 1) * h_ - delta, odt = 1.0 / p.deltat;
  std::vector<double> hp(size_t(10) * n, 0.0);
  std::vector<float> f32(size_t(6) * n, 0.0f);
  for (int i = 0; i < n; ++i) {
    const double x = h_ * double(i);
    double f = 0.0, g = 0.0;
    if (x < ol) {
      f = d0 * std::pow((ol - x) / delta, 2);
      g = d0 * std::pow((ol - x - h_ / 2.0) / delta, 2);
    } else if (x >= 0.9999 * orr) {   // the reference's edge fix (PML:213)
      f = d0 * std::pow((x - orr) / delta, 2);
      g = d0 * std::pow((x + h_ / 2.0 - orr) / delta, 2);
    }
    f /= 2.0;
    g /= 2.0;
    hp[0 * size_t(n) + i] = f; hp[1 * size_t(n) + i] = 1.0; hp[4 * size_t(n) + i] = 1.0;
    hp[5 * size_t(n) + i] = g; hp[6 * size_t(n) + i] = 1.0; hp[9 * size_t(n) + i] = 1.0;
    f32[0 * size_t(n) + i] = float(odt - f); f32[1 * size_t(n) + i] = float(odt + f);
    f32[2 * size_t(n) + i] = 1.0f;
    f32[3 * size_t(n) + i] = float(odt - g); f32[4 * size_t(n) + i] = float(odt + g);
    f32[5 * size_t(n) + i] = 1.0f;
  }
  int st;
  if ((st = dalloc(h, &h->prof64[axis], size_t(10) * n))) return st;
  if ((st = dalloc(h, &h->prof32[axis], size_t(6) * n))) return st;
  CK(cudaMemcpy(h->prof64[axis], hp.data(), sizeof(double) * hp.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->prof32[axis], f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice));
  Axis& A = h->axes[axis];
  const float* t = h->prof32[axis];
  A.a = t; A.b = t + n; A.ik = t + 2 * n; A.ah = t + 3 * n; A.bh = t + 4 * n; A.ikh = t + 5 * n;
  A.n = n; A.lo = 0; A.hi = 0;
  return CPML_OK;
}

int build_axis(cpml_handle* h, int axis, int n, double delta) {
  if (is_split(h)) return build_axis_split(h, axis, n, delta);
  const cpml_params& p = h->p;
  ProfileArgs P{};
  P.n = n; P.npml = p.npoints_pml;
  P.high_cells = (is_order4(h) && axis == 1) ? n : n - 1;
  P.use_min = p.use_pml[2 * axis]; P.use_max = p.use_pml[2 * axis + 1];
  P.delta = delta; P.cp = p.cp; P.f0 = p.f0; P.dt = p.deltat; P.npower = p.npower;
  P.kmax = p.k_max_pml; P.amax = p.alpha_max_pml < 0 ? 2.0 * kPi * (p.f0 / 2.0) : p.alpha_max_pml;
  P.rcoef = p.rcoef;
  int st;
  if ((st = dalloc(h, &h->prof64[axis], size_t(10) * n))) return st;
  if ((st = dalloc(h, &h->prof32[axis], size_t(6) * n))) return st;
  launch_build_profile(P, h->prof64[axis], h->prof32[axis], h->stream);
  CK(cudaGetLastError());
  std::vector<double> hp(size_t(10) * n);
  CK(cudaMemcpyAsync(hp.data(), h->prof64[axis], sizeof(double) * hp.size(), cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  // slab extents: every index whose a or a_half is nonzero must be inside
  auto nzero = [&](int i) { return hp[3 * size_t(n) + i] != 0.0 || hp[8 * size_t(n) + i] != 0.0; };
  int lo = 0, hi = 0;
  for (int i = 0; i < n / 2; ++i) if (nzero(i)) lo = i + 1;
  for (int i = n - 1; i >= n / 2; --i) if (nzero(i)) hi = n - i;
  for (int i = lo; i < n - hi; ++i)
    if (nzero(i)) { lo = n; hi = 0; break; }
  // 3D x slab, stored [k][j][sx]: each side widened to whole 32-byte
  // sectors, so that the two sides of a row never share a sector and a
  // row's memory variables are read and written as full sectors. The added
  // points lie outside the layer (a = 0, b = 1, 1/K = 1): their memory
  // variables stay zero and leave the derivatives unchanged.
  if (h->ndim == 3 && axis == 0 && lo < n) {
    const int lo8 = (lo + 7) / 8 * 8, hi8 = (hi + 7) / 8 * 8;
    if (lo8 + hi8 < n) { lo = lo8; hi = hi8; }
  }
  Axis& A = h->axes[axis];
  const float* f = h->prof32[axis];
  A.a = f; A.b = f + n; A.ik = f + 2 * n; A.ah = f + 3 * n; A.bh = f + 4 * n; A.ikh = f + 5 * n;
  A.n = n; A.lo = lo; A.hi = hi;
  return CPML_OK;
}

int alloc_slabs(cpml_handle* h) {
  const size_t nx = h->nx, ny = h->ny, nz = h->nz, px = h->px;
  const int nvar = h->ndim == 3 ? 6 : 4;
  const size_t wx = h->axes[0].width(), wy = h->axes[1].width();
  const size_t wz = h->ndim == 3 ? h->axes[2].width() : 0;
  (void)nx;
  for (int v = 0; v < nvar; ++v) {
    int st;
    if ((st = dalloc(h, &h->slabs.x[v], nz * ny * wx))) return st;
    if ((st = dalloc(h, &h->slabs.y[v], nz * wy * px))) return st;
    if (h->ndim == 3 && (st = dalloc(h, &h->slabs.z[v], wz * ny * px))) return st;
  }
  if (h->ndim == 3)
    for (int v = 0; v < 3; ++v) {
      int st;
      if ((st = dalloc(h, &h->slabs1.x[v], nz * ny * wx))) return st;
      if ((st = dalloc(h, &h->slabs1.y[v], nz * wy * px))) return st;
      if ((st = dalloc(h, &h->slabs1.z[v], wz * ny * px))) return st;
    }
  return CPML_OK;
}

size_t slab_floats(const cpml_handle* h, int axis) {
  const size_t ny = h->ny, nz = h->nz, px = h->px;
  if (axis == 0) return nz * ny * h->axes[0].width();
  if (axis == 1) return nz * h->axes[1].width() * px;
  return h->axes[2].width() * ny * px;
}

int zero_state(cpml_handle* h) {
  const int nf = h->ndim == 3 ? 9 : 5;
  const int map2d[5] = {0, 1, 3, 4, 6};
  for (int q = 0; q < nf; ++q) {
    const int f = h->ndim == 3 ? q : map2d[q];
    CK(cudaMemsetAsync(h->fld[f], 0, sizeof(float) * h->ncellp, h->stream));
    if (h->fld1[f]) CK(cudaMemsetAsync(h->fld1[f], 0, sizeof(float) * h->ncellp, h->stream));
  }
  const int nvar = h->ndim == 3 ? 6 : 4;
  for (const Slabs* S : {&h->slabs, &h->slabs1})
    for (int v = 0; v < nvar; ++v) {
      if (S->x[v]) CK(cudaMemsetAsync(S->x[v], 0, sizeof(float) * slab_floats(h, 0), h->stream));
      if (S->y[v]) CK(cudaMemsetAsync(S->y[v], 0, sizeof(float) * slab_floats(h, 1), h->stream));
      if (S->z[v]) CK(cudaMemsetAsync(S->z[v], 0, sizeof(float) * slab_floats(h, 2), h->stream));
    }
  CK(cudaMemsetAsync(h->err, 0, sizeof(int), h->stream));
  const size_t ns = h->p.nstep;
  if (h->seis) CK(cudaMemsetAsync(h->seis, 0, sizeof(float) * 3 * size_t(std::max(h->nrec, 1)) * ns, h->stream));
  CK(cudaMemsetAsync(h->ek, 0, sizeof(double) * ns, h->stream));
  CK(cudaMemsetAsync(h->ep, 0, sizeof(double) * ns, h->stream));
  CK(cudaMemsetAsync(h->vmax, 0, sizeof(double) * ns, h->stream));
  CK(cudaMemsetAsync(h->bad, 0, sizeof(int) * ns, h->stream));
  CK(cudaMemsetAsync(h->it_base, 0, sizeof(int), h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->it = 0;
  h->last_vmax = 0;
  return CPML_OK;
}

// One time step that reads buffer set q.
void launch_step(cpml_handle* h, int q, int ls) {
  const StepArgs s = make_args(h, q);
  if (h->ndim == 3) {
    if (h->pingpong) fused3d_launch(h->plan.data(), s, ls, q, h->stream);
    else launch_step3d_two_sweep(s, ls, h->het, h->stream);
  } else if (is_split(h)) {
    launch_step2d_split(s, ls, h->stream);
  } else if (is_order4(h)) {
    launch_step2d_order4(s, ls, h->het, h->stream);
  } else {
    launch_step2d_two_sweep(s, ls, h->het, h->stream);
  }
}

// Graph of one chunk of C steps starting from buffer set q0; cached by (C, q0).
int get_graph(cpml_handle* h, int C, cudaGraphExec_t* out) {
  const int q0 = h->pingpong ? (h->it & 1) : 0;
  const int key = 2 * C + q0;
  auto it = h->graphs.find(key);
  if (it != h->graphs.end()) { *out = it->second; return CPML_OK; }
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  if (h->cluster || h->persist) {
    const cudaError_t le = h->cluster ? launch_chunk2d_cluster(make_args(h), C, h->het, h->clay, h->stream)
                                      : launch_chunk2d_persistent(make_args(h), C, h->het, h->bar, h->persist_grid,
                                                                  h->stream);
    if (le != cudaSuccess) {
      cudaStreamEndCapture(h->stream, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return cuda_status(le);
    }
  } else {
    for (int ls = 0; ls < C; ++ls) launch_step(h, h->pingpong ? ((q0 + ls) & 1) : 0, ls);
  }
  const StepArgs s = make_args(h, h->pingpong ? ((q0 + C) & 1) : 0);  // set holding the chunk's result
  launch_reduce_chunk(s, C, h->ek, h->ep, h->vmax, h->bad, h->stream);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) { cudaGetLastError(); return CPML_ERR_CUDA; }
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { cudaGetLastError(); return CPML_ERR_CUDA; }
  h->graphs[key] = ex;
  *out = ex;
  return CPML_OK;
}

size_t padded_index(const cpml_handle* h, int i1, int j1, int k1) {
  return size_t(k1 - 1) * h->plane + size_t(j1 - 1) * h->px + size_t(i1 - 1);
}

int upload_receivers(cpml_handle* h) {
  std::vector<int> cells(std::max(h->nrec, 1), 0);
  for (int r = 0; r < h->nrec; ++r)
    cells[r] = (int)padded_index(h, h->rec_ijk[3 * r], h->rec_ijk[3 * r + 1], h->rec_ijk[3 * r + 2]);
  CK(cudaMemcpyAsync(h->rec_cell, cells.data(), sizeof(int) * cells.size(), cudaMemcpyHostToDevice,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

// Choose the step kernel and (re)build what it needs: the fused one-sweep 3D
// kernel ping-pongs two buffer sets and reads them through TMA tensor maps;
// the two-sweep kernels update one set in place.
int configure_path_impl(cpml_handle* h) {
  const bool fused = h->ndim == 3 && h->kernel != CPML_KERNEL_TWO_SWEEP && fused3d_supported();
  if (h->ndim == 3 && h->kernel == CPML_KERNEL_FUSED && !fused) return CPML_ERR_CUDA;
  int st;
  if (fused) {
    for (int f = 0; f < 9; ++f)
      if (!h->fld1[f] && (st = dalloc(h, &h->fld1[f], h->ncellp))) return st;
    h->plan.assign(fused3d_plan_bytes(), 0);
    float* sets[2][9];
    for (int f = 0; f < 9; ++f) { sets[0][f] = h->fld[f]; sets[1][f] = h->fld1[f]; }
    if (!fused3d_make_maps(h->plan.data(), sets, h->model[0], h->model[1], h->model[2], h->nx, h->ny, h->nz,
                           h->px, h->tile_y, h->zchunk, h->depth, h->het))
      return CPML_ERR_CUDA;
    std::vector<int4> fast, gen;
    int n_cls[4] = {0, 0, 0, 0};
    fused3d_items(h->nx, h->ny, h->nz, h->axes[0], h->axes[1], h->axes[2], h->p.npoints_pml, h->tile_y,
                  h->zchunk, h->het, fast, gen, n_cls);
    // both new lists exist before either old one is released
    int4 *dfast = nullptr, *dgen = nullptr;
    if ((st = dalloc(h, &dfast, fast.size()))) return st;
    if ((st = dalloc(h, &dgen, gen.size()))) { dfree(h, dfast); return st; }
    drop_graphs(h);  // cached graphs launch with the item lists about to be replaced
    dfree(h, h->items_fast);
    dfree(h, h->items_gen);
    h->items_fast = dfast;
    h->items_gen = dgen;
    if (!fast.empty())
      CK(cudaMemcpy(dfast, fast.data(), sizeof(int4) * fast.size(), cudaMemcpyHostToDevice));
    if (!gen.empty())
      CK(cudaMemcpy(dgen, gen.data(), sizeof(int4) * gen.size(), cudaMemcpyHostToDevice));
    if (!h->fork) {
      CK(cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming));
      for (int c = 0; c < 4; ++c) {
        CK(cudaStreamCreateWithFlags(&h->aux[c], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->join[c], cudaEventDisableTiming));
      }
    }
    fused3d_set_items(h->plan.data(), dfast, (int)fast.size(), dgen, n_cls, h->aux, h->fork, h->join);
    h->nblocks = int(fast.size() + gen.size());
  } else {
    StepArgs s = make_args(h);
    h->nblocks = h->ndim == 3 ? blocks3d(s) : blocks2d(s);
  }
  h->persist = false;
  h->cluster = false;
  if (is_standard2d(h) && h->kernel == CPML_KERNEL_CLUSTER) {
    // the grid on chip in one cluster (only on request: on the 101 x 641
    // reference grid it measured 13.3 against 9.0 us per step two-sweep)
    h->clay = cluster2d_layout(make_args(h), h->het);
    if (h->clay.ncl <= 0) return CPML_ERR_INVALID;
    h->cluster = true;
    h->nblocks = h->clay.ncl;
  }
  if (!h->cluster && is_standard2d(h) && h->kernel != CPML_KERNEL_TWO_SWEEP) {
    const StepArgs s = make_args(h);
    h->persist_grid = persist2d_grid(s, h->het);
    // persistent only on request (or when the autotuner picks it): the two
    // kernels per step replayed from a CUDA graph measured faster on every
    // grid above 280 x 280 (440^2: 20.4 against 15.3 Gcell-updates/s,
    // 1280^2: 36.7 against 30.9) and on the 101 x 641 reference grid
    if (h->persist_grid < 1) {
      if (h->kernel == CPML_KERNEL_PERSISTENT) return CPML_ERR_CUDA;
    } else if (h->kernel == CPML_KERNEL_PERSISTENT) {
      if (!h->bar && (st = dalloc(h, &h->bar, 2))) return st;
      h->persist = true;
    }
  }
  h->pingpong = fused;
  const size_t need = size_t(kMaxChunk) * h->nblocks * 4;
  if (need > h->partials_cap) {
    drop_graphs(h);
    if ((st = drealloc(h, &h->partials, need))) return st;
    h->partials_cap = need;
  }
  drop_graphs(h);
  return CPML_OK;
}

// A re-plan that fails part-way leaves the handle's plan, item lists and
// partials out of step with one another: cpml_run refuses such a handle
// (CPML_ERR_NOT_READY) until a later re-plan succeeds.
int configure_path(cpml_handle* h) {
  const int st = configure_path_impl(h);
  h->plan_ok = st == CPML_OK;
  return st;
}

// Buffer set that holds the current time level.
float* const* cur_fields(cpml_handle* h) { return (h->pingpong && (h->it & 1)) ? h->fld1 : h->fld; }

}  // namespace

extern "C" {

int cpml_create(const cpml_params* pin, cpml_handle** out) {
  if (!out) return CPML_ERR_INVALID;
  *out = nullptr;
  int st = validate(pin);
  if (st) return st;
  if (cpml_courant(pin, pin->cp) > 1.0) return CPML_ERR_CFL;  // 2D:516, 3D:717
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) { cudaGetLastError(); return CPML_ERR_CUDA; }
  cpml_handle* h = new cpml_handle();
  h->p = *pin;
  h->ndim = pin->ndim;
  h->nx = pin->nx; h->ny = pin->ny; h->nz = pin->ndim == 3 ? pin->nz : 1;
  if (h->ndim == 2) h->p.nz = 1;
  h->px = (h->nx + 31) / 32 * 32;
  h->plane = (long long)h->px * h->ny;
  h->ncellp = size_t(h->plane) * h->nz;
  h->cp_max = pin->cp;
  h->rho_src[0] = h->rho_src[1] = pin->rho;
  auto fail = [&](int code) { cpml_destroy(h); return code; };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(CPML_ERR_CUDA);
  if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) return fail(CPML_ERR_CUDA);
  const int used3[9] = {1, 1, 1, 1, 1, 1, 1, 1, 1};
  const int used2[9] = {1, 1, 0, 1, 1, 0, 1, 0, 0};
  for (int f = 0; f < 9; ++f)
    if ((h->ndim == 3 ? used3 : used2)[f] && (st = dalloc(h, &h->fld[f], h->ncellp))) return fail(st);
  if (is_split(h))   // the y parts of the split fields (vx_2 ... sigmaxy_2, PML:163-165)
    for (int f = 0; f < 9; ++f)
      if (used2[f] && (st = dalloc(h, &h->fld1[f], h->ncellp))) return fail(st);
  if ((st = build_axis(h, 0, h->nx, pin->deltax))) return fail(st);
  if ((st = build_axis(h, 1, h->ny, pin->deltay))) return fail(st);
  if (h->ndim == 3) {
    if ((st = build_axis(h, 2, h->nz, pin->deltaz))) return fail(st);
  } else {
    h->axes[2] = Axis{};
    h->axes[2].n = 1;
  }
  if ((st = alloc_slabs(h))) return fail(st);
  if ((st = dalloc(h, &h->src_fx, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->src_fy, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->ek, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->ep, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->vmax, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->bad, pin->nstep))) return fail(st);
  if ((st = dalloc(h, &h->it_base, 1))) return fail(st);
  if ((st = dalloc(h, &h->err, 1))) return fail(st);
  if ((st = configure_path(h))) return fail(st);
  // default receivers: none; seismogram buffer sized for one dummy receiver
  h->nrec = 0;
  if ((st = dalloc(h, &h->rec_cell, 1))) return fail(st);
  if ((st = dalloc(h, &h->seis, size_t(3) * pin->nstep))) return fail(st);
  if ((st = upload_source(h))) return fail(st);
  if ((st = zero_state(h))) return fail(st);
  *out = h;
  return CPML_OK;
}

int cpml_set_model(cpml_handle* h, const float* lam, const float* mu, const float* rho) {
  if (!h) return CPML_ERR_INVALID;
  if (!lam && !mu && !rho) return CPML_OK;
  if (is_split(h)) return CPML_ERR_INVALID;   // the split-field program is homogeneous
  const cpml_params& p = h->p;
  const size_t n = size_t(h->nx) * h->ny * h->nz;
  const float def[3] = {float(p.rho * (p.cp * p.cp - 2.0 * p.cs * p.cs)), float(p.rho * p.cs * p.cs),
                        float(p.rho)};
  const float* src[3] = {lam, mu, rho};
  // Courant number with the model's largest P velocity
  double cpm = 0.0;
  for (size_t c = 0; c < n; ++c) {
    const double l = lam ? lam[c] : def[0], m = mu ? mu[c] : def[1], r = rho ? rho[c] : def[2];
    if (!(r > 0) || !(m > 0) || !(l + 2 * m > 0)) return CPML_ERR_INVALID;
    cpm = std::max(cpm, std::sqrt((l + 2.0 * m) / r));
  }
  if (cpml_courant(&p, cpm) > 1.0) return CPML_ERR_CFL;
  uint64_t hash = kFnvBasis;
  for (int q = 0; q < 3; ++q) {
    if (src[q]) hash = fnv1a(hash, src[q], sizeof(float) * n);
    else hash = fnv1a(hash, &def[q], sizeof(float));
  }
  int st;
  std::vector<float> tmp;
  for (int q = 0; q < 3; ++q) {
    if (!h->model[q] && (st = dalloc(h, &h->model[q], h->ncellp))) return st;
    const float* s = src[q];
    if (!s) { tmp.assign(n, def[q]); s = tmp.data(); }
    CK(cudaMemset2DAsync(h->model[q], sizeof(float) * h->px, 0, sizeof(float) * h->px,
                         size_t(h->ny) * h->nz, h->stream));
    CK(cudaMemcpy2DAsync(h->model[q], sizeof(float) * h->px, s, sizeof(float) * h->nx,
                         sizeof(float) * h->nx, size_t(h->ny) * h->nz, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  h->het = true;
  h->model_hash = hash;
  h->cp_max = cpm;
  if ((st = configure_path(h))) return st;
  // rho at the source (2D:661-667 uses rho(i,j) and the 4-point average for
  // v_y; 3D:1080-1081 uses rho for both)
  auto R = [&](int i1, int j1, int k1) {
    const size_t c = size_t(k1 - 1) * h->nx * h->ny + size_t(j1 - 1) * h->nx + (i1 - 1);
    return rho ? double(rho[c]) : double(def[2]);
  };
  const int i = p.isource, j = p.jsource, k = h->ndim == 3 ? p.ksource : 1;
  h->rho_src[0] = R(i, j, k);
  h->rho_src[1] = h->ndim == 2 ? 0.25 * (R(i, j, 1) + R(i + 1, j, 1) + R(i + 1, j + 1, 1) + R(i, j + 1, 1))
                               : R(i, j, k);
  drop_graphs(h);
  return upload_source(h);
}

int cpml_set_receivers(cpml_handle* h, int nrec, const int* ix, const int* iy, const int* iz) {
  if (!h || nrec < 0 || (nrec > 0 && (!ix || !iy))) return CPML_ERR_INVALID;
  std::vector<int> ijk(size_t(3) * nrec);
  for (int r = 0; r < nrec; ++r) {
    const int k = h->ndim == 3 ? (iz ? iz[r] : h->p.ksource) : 1;
    if (ix[r] < 1 || ix[r] > h->nx || iy[r] < 1 || iy[r] > h->ny || k < 1 || k > h->nz)
      return CPML_ERR_INVALID;
    ijk[3 * r] = ix[r]; ijk[3 * r + 1] = iy[r]; ijk[3 * r + 2] = k;
  }
  if (h->it != 0) return CPML_ERR_INVALID;  // set receivers before running (or after reset)
  int st;
  if (nrec > std::max(h->nrec, 1)) {
    // both new buffers exist before either old one is released, so a failed
    // call leaves the previous receivers intact
    int* cells = nullptr;
    float* seis = nullptr;
    if ((st = dalloc(h, &cells, size_t(nrec)))) return st;
    if ((st = dalloc(h, &seis, size_t(3) * nrec * h->p.nstep))) { dfree(h, cells); return st; }
    drop_graphs(h);
    dfree(h, h->rec_cell);
    dfree(h, h->seis);
    h->rec_cell = cells;
    h->seis = seis;
  }
  h->nrec = nrec;
  h->rec_ijk = ijk;
  drop_graphs(h);
  if ((st = upload_receivers(h))) {  // never leave indices on the device that were not uploaded
    h->nrec = 0;
    h->rec_ijk.clear();
    return st;
  }
  CK(cudaMemsetAsync(h->seis, 0, sizeof(float) * 3 * size_t(std::max(nrec, 1)) * h->p.nstep, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

int cpml_reset(cpml_handle* h) {
  if (!h) return CPML_ERR_INVALID;
  return zero_state(h);
}

int cpml_run(cpml_handle* h, int nsteps) {
  if (!h || nsteps < 0) return CPML_ERR_INVALID;
  if (!h->plan_ok) return CPML_ERR_NOT_READY;
  if (h->it + nsteps > h->p.nstep) return CPML_ERR_RANGE;
  const bool check = !(h->p.flags & CPML_FLAG_NO_STABILITY);
  const int d = h->p.it_display;
  int st;
  int done = 0;
  CK(cudaEventRecord(h->ev0, h->stream));
  while (done < nsteps) {
    int end = h->it + (nsteps - done);
    if (check) {
      int nd = (h->it / d + 1) * d;
      if (h->it < 5) nd = std::min(nd, 5);
      end = std::min(end, nd);
    }
    end = std::min(end, h->it + kMaxChunk);
    const int C = end - h->it;
    cudaGraphExec_t g;
    if ((st = get_graph(h, C, &g))) return st;
    CK(cudaGraphLaunch(g, h->stream));
    done += C;
    const int it_end = end;
    h->it = end;
    if (check && (it_end % d == 0 || it_end == 5)) {
      double vm = 0;
      CK(cudaMemcpyAsync(&vm, h->vmax + (it_end - 1), sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      std::vector<int> bad(C);
      CK(cudaMemcpyAsync(bad.data(), h->bad + (it_end - C), sizeof(int) * C, cudaMemcpyDeviceToHost, h->stream));
      CK(cudaStreamSynchronize(h->stream));
      h->last_vmax = vm;
      bool nonfinite = false;
      for (int b : bad) nonfinite |= b != 0;
      if (vm > kStability || nonfinite || !(vm == vm)) {  // 2D:724, 3D:1193
        cudaEventRecord(h->ev1, h->stream);
        cudaEventSynchronize(h->ev1);
        return CPML_ERR_UNSTABLE;
      }
    }
  }
  CK(cudaEventRecord(h->ev1, h->stream));
  CK(cudaEventSynchronize(h->ev1));
  int err = 0;
  CK(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return CPML_ERR_TIMEOUT;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->last_ms = ms;
  CK(cudaGetLastError());
  return CPML_OK;
}

int cpml_status(cpml_handle* h, int* it, double* vmax) {
  if (!h) return CPML_ERR_INVALID;
  if (it) *it = h->it;
  if (vmax) *vmax = h->last_vmax;
  return CPML_OK;
}

int cpml_get_seismograms(cpml_handle* h, double* vx, double* vy, double* vz) {
  if (!h) return CPML_ERR_INVALID;
  const size_t ns = h->p.nstep, nr = h->nrec;
  if (nr == 0) return CPML_OK;
  std::vector<float> buf(3 * nr * ns);
  CK(cudaMemcpyAsync(buf.data(), h->seis, sizeof(float) * buf.size(), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  double* out[3] = {vx, vy, h->ndim == 3 ? vz : nullptr};
  for (int c = 0; c < 3; ++c) {
    if (!out[c]) continue;
    for (size_t r = 0; r < nr; ++r)
      for (size_t t = 0; t < ns; ++t)
        out[c][r * ns + t] = t < size_t(h->it) ? double(buf[c * nr * ns + r * ns + t]) : 0.0;
  }
  return CPML_OK;
}

int cpml_get_energy(cpml_handle* h, double* ek, double* ep) {
  if (!h) return CPML_ERR_INVALID;
  const size_t ns = h->p.nstep;
  if (ek) CK(cudaMemcpyAsync(ek, h->ek, sizeof(double) * ns, cudaMemcpyDeviceToHost, h->stream));
  if (ep) CK(cudaMemcpyAsync(ep, h->ep, sizeof(double) * ns, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

static float* field_ptr(cpml_handle* h, int field) {
  if (field < 0 || field > 8) return nullptr;
  return cur_fields(h)[field];
}

}  // extern "C"
namespace {
// The split-field program's total field is the sum of its x and y parts
// (PML:153-159); this adds the y part, copied the same way, into out.
template <typename Copy>
int add_split_part(cpml_handle* h, int field, size_t n, float* out, Copy copy) {
  if (!is_split(h)) return CPML_OK;
  std::vector<float> part(n);
  CK(copy(part.data(), h->fld1[field]));
  CK(cudaStreamSynchronize(h->stream));
  for (size_t c = 0; c < n; ++c) out[c] = out[c] + part[c];
  return CPML_OK;
}
}  // namespace
extern "C" {

int cpml_get_field(cpml_handle* h, int field, float* out) {
  if (!h || !out) return CPML_ERR_INVALID;
  float* f = field_ptr(h, field);
  if (!f) return CPML_ERR_INVALID;
  auto copy = [&](float* dst, const float* src) {
    return cudaMemcpy2DAsync(dst, sizeof(float) * h->nx, src, sizeof(float) * h->px, sizeof(float) * h->nx,
                             size_t(h->ny) * h->nz, cudaMemcpyDeviceToHost, h->stream);
  };
  CK(copy(out, f));
  CK(cudaStreamSynchronize(h->stream));
  return add_split_part(h, field, size_t(h->nx) * h->ny * h->nz, out, copy);
}

// Split-field handles: the total goes to the x part, the y part is zeroed.
int cpml_set_field(cpml_handle* h, int field, const float* in) {
  if (!h || !in) return CPML_ERR_INVALID;
  float* f = field_ptr(h, field);
  if (!f) return CPML_ERR_INVALID;
  CK(cudaMemcpy2DAsync(f, sizeof(float) * h->px, in, sizeof(float) * h->nx, sizeof(float) * h->nx,
                       size_t(h->ny) * h->nz, cudaMemcpyHostToDevice, h->stream));
  if (is_split(h)) CK(cudaMemsetAsync(h->fld1[field], 0, sizeof(float) * h->ncellp, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

// ---- checkpoint / restart ---------------------------------------------------
// Snapshot layout (host memory, native byte order): StateHeader, then the
// current time level's wavefields ([k][j][i] FP32, 9 in 3D, vx vy sxx syy sxy
// in 2D), every C-PML memory variable in its slab layout (axis by axis,
// variable by variable, the stress-side ones at the current time level),
// the seismogram samples so far ([3][nrec][it] FP32), then ek, ep, max|v|
// (FP64) and the non-finite flags (int32) of steps 1..it.
}  // extern "C"
namespace {
struct StateHeader {
  char magic[8];
  int32_t version, ndim, nx, ny, nz, npml, nstep, nrec, it, het, nfield, nvar;
  int32_t slab_w[3];
  int32_t unused;
  uint64_t param_hash, model_hash, rec_hash;
  double last_vmax;
  uint64_t bytes;
};
const char kStateMagic[8] = {'C', 'P', 'M', 'L', 'S', 'T', 'A', 'T'};
const int32_t kStateVersion = 1;

uint64_t param_hash(const cpml_handle* h) {
  cpml_params q = h->p;
  std::memset(q.reserved_i, 0, sizeof(q.reserved_i));
  std::memset(q.reserved_d, 0, sizeof(q.reserved_d));
  return fnv1a(kFnvBasis, &q, sizeof(q));
}
uint64_t rec_hash(const cpml_handle* h) {
  return fnv1a(kFnvBasis, h->rec_ijk.data(), sizeof(int) * h->rec_ijk.size());
}
// Device arrays of the time level held in buffer set `set` (set 1 only
// exists on the fused 3D path); a split-field handle adds its y parts.
int state_fields(const cpml_handle* h, int set, float** out) {
  static const int f2[5] = {0, 1, 3, 4, 6};
  const int n = h->ndim == 3 ? 9 : 5;
  float* const* F = set == 0 ? h->fld : h->fld1;
  for (int q = 0; q < n; ++q) out[q] = F[h->ndim == 3 ? q : f2[q]];
  if (!is_split(h)) return n;
  for (int q = 0; q < 5; ++q) out[5 + q] = h->fld1[f2[q]];
  return 10;
}
int state_nfield(const cpml_handle* h) { return h->ndim == 3 ? 9 : (is_split(h) ? 10 : 5); }
size_t state_bytes(const cpml_handle* h, int it) {
  const size_t ncell = size_t(h->nx) * h->ny * h->nz;
  const int nf = state_nfield(h), nvar = h->ndim == 3 ? 6 : 4;
  size_t b = sizeof(StateHeader) + size_t(nf) * ncell * sizeof(float);
  for (int a = 0; a < h->ndim; ++a) b += size_t(nvar) * slab_floats(h, a) * sizeof(float);
  b += size_t(3) * h->nrec * it * sizeof(float);
  b += size_t(it) * (3 * sizeof(double) + sizeof(int));
  return b;
}
float* slab_ptr(const Slabs& S, int axis, int v) { return axis == 0 ? S.x[v] : (axis == 1 ? S.y[v] : S.z[v]); }
}  // namespace
extern "C" {

int cpml_state_size(cpml_handle* h, size_t* bytes) {
  if (!h || !bytes) return CPML_ERR_INVALID;
  *bytes = state_bytes(h, h->it);
  return CPML_OK;
}

int cpml_save_state(cpml_handle* h, void* buf, size_t bytes) {
  if (!h || !buf) return CPML_ERR_INVALID;
  const size_t need = state_bytes(h, h->it);
  if (bytes < need) return CPML_ERR_RANGE;
  StateHeader H{};
  std::memcpy(H.magic, kStateMagic, 8);
  H.version = kStateVersion;
  H.ndim = h->ndim; H.nx = h->nx; H.ny = h->ny; H.nz = h->nz; H.npml = h->p.npoints_pml;
  H.nstep = h->p.nstep; H.nrec = h->nrec; H.it = h->it; H.het = h->het ? 1 : 0;
  float* F[10];
  H.nfield = state_fields(h, (h->pingpong && (h->it & 1)) ? 1 : 0, F);
  H.nvar = h->ndim == 3 ? 6 : 4;
  for (int a = 0; a < 3; ++a) H.slab_w[a] = a < h->ndim ? h->axes[a].width() : 0;
  H.param_hash = param_hash(h); H.model_hash = h->model_hash; H.rec_hash = rec_hash(h);
  H.last_vmax = h->last_vmax;
  H.bytes = need;
  char* out = static_cast<char*>(buf);
  std::memcpy(out, &H, sizeof(H));
  out += sizeof(H);
  const size_t fs = sizeof(float), ncell = size_t(h->nx) * h->ny * h->nz;
  for (int q = 0; q < H.nfield; ++q) {
    CK(cudaMemcpy2DAsync(out, fs * h->nx, F[q], fs * h->px, fs * h->nx, size_t(h->ny) * h->nz,
                         cudaMemcpyDeviceToHost, h->stream));
    out += ncell * fs;
  }
  // stress-side memory variables (0..2) alternate with the fields on the fused path
  const bool odd = h->pingpong && (h->it & 1);
  for (int a = 0; a < h->ndim; ++a)
    for (int v = 0; v < H.nvar; ++v) {
      const size_t n = slab_floats(h, a);
      const float* src = slab_ptr((v < 3 && odd) ? h->slabs1 : h->slabs, a, v);
      if (n) CK(cudaMemcpyAsync(out, src, n * fs, cudaMemcpyDeviceToHost, h->stream));
      out += n * fs;
    }
  const size_t it = h->it, ns = h->p.nstep;
  if (h->nrec > 0 && it > 0)
    CK(cudaMemcpy2DAsync(out, fs * it, h->seis, fs * ns, fs * it, size_t(3) * h->nrec, cudaMemcpyDeviceToHost,
                         h->stream));
  out += size_t(3) * h->nrec * it * fs;
  if (it > 0) {
    for (double* src : {h->ek, h->ep, h->vmax}) {
      CK(cudaMemcpyAsync(out, src, it * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      out += it * sizeof(double);
    }
    CK(cudaMemcpyAsync(out, h->bad, it * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

int cpml_load_state(cpml_handle* h, const void* buf, size_t bytes) {
  if (!h || !buf || bytes < sizeof(StateHeader)) return CPML_ERR_INVALID;
  StateHeader H;
  std::memcpy(&H, buf, sizeof(H));
  const int nf = state_nfield(h);
  bool ok = std::memcmp(H.magic, kStateMagic, 8) == 0 && H.version == kStateVersion && H.ndim == h->ndim &&
            H.nx == h->nx && H.ny == h->ny && H.nz == h->nz && H.npml == h->p.npoints_pml &&
            H.nstep == h->p.nstep && H.nrec == h->nrec && H.het == (h->het ? 1 : 0) && H.nfield == nf &&
            H.nvar == (h->ndim == 3 ? 6 : 4) && H.it >= 0 && H.it <= h->p.nstep &&
            H.param_hash == param_hash(h) && H.model_hash == h->model_hash && H.rec_hash == rec_hash(h);
  for (int a = 0; a < 3 && ok; ++a) ok = H.slab_w[a] == (a < h->ndim ? h->axes[a].width() : 0);
  if (!ok) return CPML_ERR_INVALID;
  if (H.bytes != state_bytes(h, H.it) || bytes < H.bytes) return CPML_ERR_INVALID;
  int st;
  if ((st = zero_state(h))) return st;   // clears records beyond it, the step counter and the error word
  h->it = H.it;
  h->last_vmax = H.last_vmax;
  const char* in = static_cast<const char*>(buf) + sizeof(H);
  const size_t fs = sizeof(float), ncell = size_t(h->nx) * h->ny * h->nz;
  // both buffer sets of the fused path get the snapshot (the write set is
  // overwritten by the next step anyway)
  float* F[2][10];
  state_fields(h, 0, F[0]);
  const bool two = h->pingpong;
  if (two) state_fields(h, 1, F[1]);
  for (int q = 0; q < nf; ++q) {
    for (int set = 0; set < (two ? 2 : 1); ++set)
      CK(cudaMemcpy2DAsync(F[set][q], fs * h->px, in, fs * h->nx, fs * h->nx, size_t(h->ny) * h->nz,
                           cudaMemcpyHostToDevice, h->stream));
    in += ncell * fs;
  }
  for (int a = 0; a < h->ndim; ++a)
    for (int v = 0; v < H.nvar; ++v) {
      const size_t n = slab_floats(h, a);
      for (const Slabs* S : {&h->slabs, &h->slabs1}) {
        float* dst = slab_ptr(*S, a, v);
        if (n && dst) CK(cudaMemcpyAsync(dst, in, n * fs, cudaMemcpyHostToDevice, h->stream));
      }
      in += n * fs;
    }
  const size_t it = H.it, ns = h->p.nstep;
  if (h->nrec > 0 && it > 0)
    CK(cudaMemcpy2DAsync(h->seis, fs * ns, in, fs * it, fs * it, size_t(3) * h->nrec, cudaMemcpyHostToDevice,
                         h->stream));
  in += size_t(3) * h->nrec * it * fs;
  if (it > 0) {
    for (double* dst : {h->ek, h->ep, h->vmax}) {
      CK(cudaMemcpyAsync(dst, in, it * sizeof(double), cudaMemcpyHostToDevice, h->stream));
      in += it * sizeof(double);
    }
    CK(cudaMemcpyAsync(h->bad, in, it * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  }
  const int itv = H.it;
  CK(cudaMemcpyAsync(h->it_base, &itv, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CPML_OK;
}

int cpml_get_plane(cpml_handle* h, int field, int axis, int index, float* out) {
  if (!h || !out || axis < 0 || axis > 2) return CPML_ERR_INVALID;
  float* f = field_ptr(h, field);
  if (!f) return CPML_ERR_INVALID;
  const int n[3] = {h->nx, h->ny, h->nz};
  if (index < 1 || index > n[axis]) return CPML_ERR_INVALID;
  const size_t fs = sizeof(float);
  auto copy = [&](float* dst, const float* src) {
    if (axis == 2)         // [j][i]
      return cudaMemcpy2DAsync(dst, fs * h->nx, src + size_t(index - 1) * h->plane, fs * h->px, fs * h->nx,
                               h->ny, cudaMemcpyDeviceToHost, h->stream);
    if (axis == 1)         // [k][i]
      return cudaMemcpy2DAsync(dst, fs * h->nx, src + size_t(index - 1) * h->px, fs * h->plane, fs * h->nx,
                               h->nz, cudaMemcpyDeviceToHost, h->stream);
    return cudaMemcpy2DAsync(dst, fs, src + (index - 1), fs * h->px, fs, size_t(h->ny) * h->nz,  // [k][j]
                             cudaMemcpyDeviceToHost, h->stream);
  };
  CK(copy(out, f));
  CK(cudaStreamSynchronize(h->stream));
  const size_t np = axis == 2 ? size_t(h->nx) * h->ny : (axis == 1 ? size_t(h->nx) * h->nz : size_t(h->ny) * h->nz);
  return add_split_part(h, field, np, out, copy);
}

double cpml_algorithmic_bytes_per_step(cpml_handle* h) {
  if (!h) return 0.0;
  const double ncell = double(h->nx) * h->ny * h->nz;
  if (is_split(h)) return 8.0 * 10 * ncell;   // ten split fields read and written once
  const int nfield = h->ndim == 3 ? 9 : 5;
  double bytes = 8.0 * nfield * ncell + (h->het ? 12.0 * ncell : 0.0);
  const int nax = h->ndim;
  const int per = h->ndim == 3 ? 3 : 2;  // memory variables per (axis, full|half)
  for (int a = 0; a < nax; ++a) {
    const int n = h->axes[a].n;
    std::vector<double> hp(size_t(10) * n);
    if (cudaMemcpy(hp.data(), h->prof64[a], sizeof(double) * hp.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
      return 0.0;
    double nf = 0, nh = 0;
    for (int i = 0; i < n; ++i) { nf += hp[3 * size_t(n) + i] != 0.0; nh += hp[8 * size_t(n) + i] != 0.0; }
    const double other = ncell / n;
    bytes += 8.0 * per * (nf + nh) * other;
  }
  return bytes;
}

int cpml_get_stream(cpml_handle* h, void** stream) {
  if (!h || !stream) return CPML_ERR_INVALID;
  *stream = (void*)h->stream;
  return CPML_OK;
}

int cpml_last_run_ms(cpml_handle* h, double* ms) {
  if (!h || !ms) return CPML_ERR_INVALID;
  *ms = h->last_ms;
  return CPML_OK;
}

int cpml_set_tuning(cpml_handle* h, int kernel, int tile_y, int zchunk, int depth) {
  if (!h || kernel < 0 || kernel > 4) return CPML_ERR_INVALID;
  if ((kernel == CPML_KERNEL_FUSED && h->ndim != 3) ||
      ((kernel == CPML_KERNEL_PERSISTENT || kernel == CPML_KERNEL_CLUSTER) && !is_standard2d(h)))
    return CPML_ERR_INVALID;
  if (zchunk < 2 || !fused3d_shape_ok(tile_y, depth)) return CPML_ERR_INVALID;
  if (h->it != 0) return CPML_ERR_INVALID;  // only on a fresh or reset handle
  h->kernel = kernel;
  h->tile_y = tile_y;
  h->zchunk = zchunk;
  h->depth = depth;
  return configure_path(h);
}

int cpml_get_tuning(cpml_handle* h, int* kernel, int* tile_y, int* zchunk, int* depth) {
  if (!h) return CPML_ERR_INVALID;
  if (kernel)
    *kernel = h->pingpong ? CPML_KERNEL_FUSED
                          : (h->cluster ? CPML_KERNEL_CLUSTER
                                        : (h->persist ? CPML_KERNEL_PERSISTENT : CPML_KERNEL_TWO_SWEEP));
  if (tile_y) *tile_y = h->tile_y;
  if (zchunk) *zchunk = h->zchunk;
  if (depth) *depth = h->depth;
  return CPML_OK;
}

int cpml_launches_per_step(cpml_handle* h, int* step_kernels, int* chunk_kernels) {
  if (!h) return CPML_ERR_INVALID;
  const bool chunked = h->persist || h->cluster;   // one launch runs the chunk's steps
  if (step_kernels) *step_kernels = h->pingpong ? fused3d_kernels_per_step(h->plan.data()) : (chunked ? 0 : 2);
  // chunk reduction + step counter (+ the chunk's persistent or cluster launch)
  if (chunk_kernels) *chunk_kernels = chunked ? 3 : 2;
  return CPML_OK;
}

// ---- autotuner -------------------------------------------------------------
namespace {
struct TuneKey {
  int ndim, nx, ny, nz, het, npml, pml_mask;
  bool operator<(const TuneKey& o) const {
    return std::tie(ndim, nx, ny, nz, het, npml, pml_mask) <
           std::tie(o.ndim, o.nx, o.ny, o.nz, o.het, o.npml, o.pml_mask);
  }
};
struct TuneVal { int kernel, tile_y, zchunk, depth; double ms; };
// Shape-class cache shared by every handle of the process; handles are
// independent and may autotune from different threads, so every access to
// the map and to the cache file holds tune_mutex (never the trials).
std::map<TuneKey, TuneVal>& tune_cache() {
  static std::map<TuneKey, TuneVal> c;
  return c;
}
std::mutex& tune_mutex() {
  static std::mutex m;
  return m;
}
TuneKey tune_key(const cpml_handle* h) {
  int mask = 0;
  for (int q = 0; q < 6; ++q) mask |= (h->p.use_pml[q] ? 1 : 0) << q;
  return TuneKey{h->ndim, h->nx, h->ny, h->nz, h->het ? 1 : 0, h->p.npoints_pml, mask};
}
bool read_cache_file(const char* path, const TuneKey& k, TuneVal* v) {
  FILE* f = path ? std::fopen(path, "r") : nullptr;
  if (!f) return false;
  TuneKey r{};
  TuneVal x{};
  bool found = false;
  while (std::fscanf(f, "%d %d %d %d %d %d %d %d %d %d %d %lf", &r.ndim, &r.nx, &r.ny, &r.nz, &r.het, &r.npml,
                     &r.pml_mask, &x.kernel, &x.tile_y, &x.zchunk, &x.depth, &x.ms) == 12)
    if (!(r < k) && !(k < r)) { *v = x; found = true; }
  std::fclose(f);
  return found;
}
}  // namespace

int cpml_autotune(cpml_handle* h, int trial_steps, const char* cache_path, int* kernel, int* tile_y,
                  int* zchunk, double* ms_per_step) {
  if (!h || trial_steps < 1) return CPML_ERR_INVALID;
  if (trial_steps + 2 > h->p.nstep) trial_steps = h->p.nstep - 2;
  if (trial_steps < 1) return CPML_ERR_RANGE;
  const TuneKey key = tune_key(h);
  TuneVal best{};
  bool have = false;
  {
    std::lock_guard<std::mutex> lock(tune_mutex());
    auto it = tune_cache().find(key);
    if (it != tune_cache().end()) { best = it->second; have = true; }
    if (!have && read_cache_file(cache_path, key, &best)) { tune_cache()[key] = best; have = true; }
  }
  int st;
  if (!have) {
    // candidates: launch shapes of the one-sweep 3D kernel, and the two-sweep form
    std::vector<TuneVal> cand;
    if (h->ndim == 3 && fused3d_supported())
      for (int ty : {8, 16})
        for (int lz : {16, 24, 32, 40, 48, 64}) cand.push_back(TuneVal{CPML_KERNEL_FUSED, ty, lz, 2, 0.0});
    cand.push_back(TuneVal{CPML_KERNEL_TWO_SWEEP, 8, 32, 2, 0.0});
    if (is_standard2d(h)) {
      if (persist2d_grid(make_args(h), h->het) > 0) cand.push_back(TuneVal{CPML_KERNEL_PERSISTENT, 8, 32, 2, 0.0});
      if (cluster2d_layout(make_args(h), h->het).ncl > 0) cand.push_back(TuneVal{CPML_KERNEL_CLUSTER, 8, 32, 2, 0.0});
    }
    const int flags = h->p.flags;
    h->p.flags |= CPML_FLAG_NO_STABILITY;  // time the kernels, not the host checks
    best.ms = 1e300;
    for (TuneVal& c : cand) {
      if ((st = cpml_reset(h)) || (st = cpml_set_tuning(h, c.kernel, c.tile_y, c.zchunk, c.depth))) {
        h->p.flags = flags;
        return st;
      }
      if ((st = cpml_run(h, 2))) { h->p.flags = flags; return st; }       // warm-up, graphs built
      if ((st = cpml_run(h, trial_steps))) { h->p.flags = flags; return st; }
      c.ms = h->last_ms / trial_steps;
      if (c.ms < best.ms) best = c;
    }
    h->p.flags = flags;
    std::lock_guard<std::mutex> lock(tune_mutex());
    tune_cache()[key] = best;
    if (cache_path) {
      if (FILE* f = std::fopen(cache_path, "a")) {
        std::fprintf(f, "%d %d %d %d %d %d %d %d %d %d %d %.6f\n", key.ndim, key.nx, key.ny, key.nz, key.het,
                     key.npml, key.pml_mask, best.kernel, best.tile_y, best.zchunk, best.depth, best.ms);
        std::fclose(f);
      }
    }
  }
  if ((st = cpml_reset(h))) return st;
  if ((st = cpml_set_tuning(h, best.kernel, best.tile_y, best.zchunk, best.depth))) return st;
  if ((st = cpml_reset(h))) return st;
  if (kernel) *kernel = best.kernel;
  if (tile_y) *tile_y = best.tile_y;
  if (zchunk) *zchunk = best.zchunk;
  if (ms_per_step) *ms_per_step = best.ms;
  return CPML_OK;
}

void cpml_destroy(cpml_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int c = 0; c < 4; ++c)
    if (h->aux[c]) cudaStreamSynchronize(h->aux[c]);
  drop_graphs(h);
  for (void* p : h->allocs) cudaFree(p);
  if (h->fork) cudaEventDestroy(h->fork);
  for (int c = 0; c < 4; ++c) {
    if (h->join[c]) cudaEventDestroy(h->join[c]);
    if (h->aux[c]) cudaStreamDestroy(h->aux[c]);
  }
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

}  // extern "C"
