// noalloc.cu -- energy of caller-owned 3D wavefields without any device
// allocation.
//
// Why it exists: a host program that already owns its wavefields on the GPU
// (for example a Fortran driver whose device arrays come from its own pool
// allocator, or an application that reserves a fixed device-memory budget at
// start-up) may be unable to call cudaMalloc in the middle of its time loop:
// cudaMalloc can synchronise the whole device, and inside a fixed budget it
// can fail. This entry point computes the kinetic and potential energy of
// such fields with a scratch area that lives in the library image itself.
//
// The scratch is one file-scope __device__ array of per-plane partial sums
// (kMaxPlanes planes, 128 KiB). Every GPU that loads the library holds it
// until the process exits. Host code cannot use the array's name as a device
// address, so the address is fetched once per device with
// cudaGetSymbolAddress (on that device's first call, with the device
// current) and passed to the kernels. The first call on each device should
// therefore come before any stream capture. Every call on a device uses the
// same array: calls whose kernels overlap on the GPU race on it, so callers
// must order them (one stream, or events). Each call writes every plane
// slot it later reads, so nothing has to be cleared between calls. The
// cached address belongs to the device's current context: a device or
// context reset (cudaDeviceReset) between calls is not supported.
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/cpml.h"
#include "kutil.cuh"

namespace {

constexpr int kMaxPlanes = 8192;  // largest nz accepted
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

__device__ __align__(256) double g_plane_partials[2 * kMaxPlanes];

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

// Stage 1: block k sums the energy of plane k over the interior
// [npml, n - npml) in x and y (3D:1136-1143); planes outside the interior
// write zeros so stage 2 never reads a stale slot.
__global__ void __launch_bounds__(kThreads)
plane_energy_kernel(const float* __restrict__ vx, const float* __restrict__ vy,
                    const float* __restrict__ vz, const float* __restrict__ sxx,
                    const float* __restrict__ syy, const float* __restrict__ szz,
                    const float* __restrict__ sxy, const float* __restrict__ sxz,
                    const float* __restrict__ syz, int nx, int ny, int nz, long long pitch,
                    int npml, float half_rho, float c1, float c2, float inv_2mu,
                    const float* __restrict__ lam_c, const float* __restrict__ mu_c,
                    const float* __restrict__ rho_c, int ep_physical, double* __restrict__ part) {
  const int k = blockIdx.x;
  cpml::Kahan ek, ep;
  const int w = nx - 2 * npml, h = ny - 2 * npml;
  if (k >= npml && k < nz - npml && w > 0 && h > 0) {
    for (int q = threadIdx.x; q < w * h; q += blockDim.x) {
      const int i = npml + q % w, j = npml + q / w;
      const long long c = ((long long)k * ny + j) * pitch + i;
      float hr = half_rho, e1 = c1, e2 = c2, i2m = inv_2mu;
      if (lam_c) {
        const float l = lam_c[c], m = mu_c[c];
        const float den = 1.0f / (2.0f * m * (3.0f * l + 2.0f * m));
        hr = 0.5f * rho_c[c];
        e1 = 2.0f * (l + m) * den;
        e2 = l * den;
        i2m = 1.0f / (2.0f * m);
      }
      const float a = vx[c], b = vy[c], d = vz[c];
      ek.add(hr * (a * a + b * b + d * d));
      const float s1 = sxx[c], s2 = syy[c], s3 = szz[c], s4 = sxy[c], s5 = sxz[c], s6 = syz[c];
      const float exx = e1 * s1 - e2 * (s2 + s3);
      const float eyy = e1 * s2 - e2 * (s1 + s3);
      // the reference counts eps_yy*sigma_yy twice and has no zz term (3D:1170-1171)
      const float third = ep_physical ? (e1 * s3 - e2 * (s1 + s2)) * s3 : eyy * s2;
      ep.add(0.5f * (exx * s1 + eyy * s2 + third) + i2m * (s4 * s4 + s5 * s5 + s6 * s6));
    }
  }
  __shared__ double out[4];
  cpml::block_partials<kThreads>(ek.value(), ep.value(), 0.f, 0, out);
  if (threadIdx.x == 0) {
    part[2 * k] = out[0];
    part[2 * k + 1] = out[1];
  }
}

// Stage 2: the plane sums in k order, like the per-plane partials of the
// reference's OpenMP reduction summed by one thread.
__global__ void sum_planes_kernel(const double* __restrict__ part, int nz, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double ek = 0.0, ep = 0.0;
  for (int k = 0; k < nz; ++k) {
    ek += part[2 * k];
    ep += part[2 * k + 1];
  }
  out[0] = ek;
  out[1] = ep;
}

// Device address of g_plane_partials on the current device, looked up once.
int scratch_for_current_device(double** ptr) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return CPML_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return CPML_ERR_RANGE;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_plane_partials) != cudaSuccess || !p) {
      cudaGetLastError();
      return CPML_ERR_CUDA;
    }
    g_scratch[dev] = static_cast<double*>(p);
  }
  *ptr = g_scratch[dev];
  return CPML_OK;
}

}  // namespace

extern "C" int cpml_energy3d_noalloc(const float* const* fields, int nx, int ny, int nz,
                                     int pitch, int npml, double lam, double mu, double rho,
                                     const float* lam_cell, const float* mu_cell,
                                     const float* rho_cell, int flags, double* out,
                                     void* stream) {
  if (!fields || !out || nx < 1 || ny < 1 || nz < 1 || pitch < nx || npml < 0) return CPML_ERR_INVALID;
  // the energy interior [npml, n - npml) must hold at least one cell on every axis
  if (2 * npml >= nx || 2 * npml >= ny || 2 * npml >= nz) return CPML_ERR_INVALID;
  for (int f = 0; f < 9; ++f)
    if (!fields[f]) return CPML_ERR_INVALID;
  if ((lam_cell || mu_cell || rho_cell) && !(lam_cell && mu_cell && rho_cell)) return CPML_ERR_INVALID;
  if (!lam_cell && !(mu > 0 && rho > 0 && 3.0 * lam + 2.0 * mu != 0.0)) return CPML_ERR_INVALID;
  if (nz > kMaxPlanes) return CPML_ERR_RANGE;  // the static scratch holds kMaxPlanes planes
  double* part = nullptr;
  int st = scratch_for_current_device(&part);
  if (st != CPML_OK) return st;
  const double den = 2.0 * mu * (3.0 * lam + 2.0 * mu);
  const float c1 = lam_cell ? 0.f : float(2.0 * (lam + mu) / den);
  const float c2 = lam_cell ? 0.f : float(lam / den);
  const float i2m = lam_cell ? 0.f : float(1.0 / (2.0 * mu));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  plane_energy_kernel<<<nz, kThreads, 0, s>>>(fields[0], fields[1], fields[2], fields[3], fields[4],
                                               fields[5], fields[6], fields[7], fields[8], nx, ny, nz,
                                               (long long)pitch, npml, float(0.5 * rho), c1, c2, i2m,
                                               lam_cell, mu_cell, rho_cell,
                                               (flags & CPML_FLAG_EP_PHYSICAL) ? 1 : 0, part);
  sum_planes_kernel<<<1, 32, 0, s>>>(part, nz, out);
  return cudaGetLastError() == cudaSuccess ? CPML_OK : CPML_ERR_CUDA;
}
