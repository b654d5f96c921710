// host.cpp -- host-only entry points of libcpml: reference parameter blocks,
// Courant number, receiver placement, FP64 C-PML profiles, and the
// reference's output files (seismograms, energy.dat, PNM snapshots).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cpml.h"

namespace {
const double kPi = 3.141592653589793238462643;

std::string join(const char* dir, const char* name) {
  std::string s = (dir && dir[0]) ? std::string(dir) : std::string(".");
  if (s.back() != '/') s += '/';
  return s + name;
}

// A REAL(4) item of a list-directed WRITE, modelled on gfortran: 9
// significant digits, fixed notation for 0.1 <= |x| < 1e8 (and for zero),
// scientific otherwise; every item starts with one separating blank. Not
// checked against a Fortran build: none exists in this environment.
void put_real4(FILE* f, float xf) {
  const double x = xf;
  const double ax = std::fabs(x);
  if (x == 0.0) {
    std::fprintf(f, "   0.00000000    ");
  } else if (ax >= 0.1 && ax < 1.0e8) {
    const int e = (int)std::floor(std::log10(ax));
    int dec = 8 - e;
    if (dec < 0) dec = 0;
    std::fprintf(f, " %15.*f    ", dec, x);
  } else {
    std::fprintf(f, " %15.8E", x);
  }
}

// A REAL(8) item: 17 significant digits, same rules.
void put_real8(FILE* f, double x) {
  const double ax = std::fabs(x);
  if (x == 0.0) {
    std::fprintf(f, "   0.0000000000000000     ");
  } else if (ax >= 0.1 && ax < 1.0e16) {
    const int e = (int)std::floor(std::log10(ax));
    int dec = 16 - e;
    if (dec < 0) dec = 0;
    std::fprintf(f, " %24.*f    ", dec, x);
  } else {
    std::fprintf(f, " %24.16E", x);
  }
}
}  // namespace

extern "C" {

int cpml_params_default_2d(cpml_params* p) {
  if (!p) return CPML_ERR_INVALID;
  std::memset(p, 0, sizeof(*p));
  p->ndim = 2;
  p->nx = 101; p->ny = 641; p->nz = 1;                  // 2D:141-142
  p->deltax = p->deltay = p->deltaz = 10.0;              // 2D:145-146
  p->use_pml[0] = p->use_pml[1] = p->use_pml[2] = p->use_pml[3] = 1;  // 2D:149-152
  p->npoints_pml = 10;                                   // 2D:155
  p->cp = 3300.0; p->cs = 3300.0 / 1.732; p->rho = 2800.0;  // 2D:158-160
  p->nstep = 2000;                                       // 2D:163
  p->deltat = 2.0e-3;                                    // 2D:166
  p->f0 = 7.0; p->t0 = 1.20 / 7.0; p->factor = 1.0e7;    // 2D:169-171
  p->isource = p->nx - 2 * p->npoints_pml - 1;           // 2D:174
  p->jsource = 2 * p->ny / 3 + 1;                        // 2D:175
  p->ksource = 1;
  p->angle_force = 135.0;                                // 2D:179
  p->stf = CPML_STF_DGAUSSIAN;                           // 2D:651
  p->it_display = 100;                                   // 2D:189
  p->flags = CPML_FLAG_ENERGY;
  p->npower = 2.0;                                       // 2D:213
  p->k_max_pml = 1.0;                                    // 2D:216
  p->alpha_max_pml = -1.0;                               // 2*pi*(f0/2), 2D:217
  p->rcoef = 0.001;                                      // 2D:290
  return CPML_OK;
}

int cpml_params_default_3d(cpml_params* p) {
  if (!p) return CPML_ERR_INVALID;
  cpml_params_default_2d(p);
  p->ndim = 3;
  p->nx = 101; p->ny = 641; p->nz = 640;                 // 3D:124-126
  for (int q = 0; q < 6; ++q) p->use_pml[q] = 1;         // 3D:158-163
  p->nstep = 2500;                                       // 3D:147
  p->deltat = 1.6e-3;                                    // 3D:150
  p->isource = p->nx - 2 * p->npoints_pml - 1;           // 3D:181
  p->jsource = 2 * p->ny / 3 + 1;                        // 3D:182
  p->ksource = p->nz / 2;                                // global plane of 3D:1080
  return CPML_OK;
}

int cpml_params_default_2d_fourth(cpml_params* p) {
  if (!p) return CPML_ERR_INVALID;
  cpml_params_default_2d(p);
  p->order = 4;
  p->nstep = 2000 * 2;                                   // 2D4:156
  p->deltat = 2.0e-3 / 2;                                // 2D4:162
  p->it_display = 100 * 2;                               // 2D4:187
  return CPML_OK;
}

int cpml_params_default_2d_split(cpml_params* p) {
  if (!p) return CPML_ERR_INVALID;
  cpml_params_default_2d(p);                             // PML:96-141 share the 2D block
  p->scheme = CPML_SCHEME_SPLIT;
  return CPML_OK;
}

double cpml_courant(const cpml_params* p, double cp_max) {
  if (!p) return NAN;
  // the split-field program checks a one-dimensional number (PML:304)
  if (p->scheme == CPML_SCHEME_SPLIT) return cp_max * p->deltat / p->deltax;
  double s = 1.0 / (p->deltax * p->deltax) + 1.0 / (p->deltay * p->deltay);
  if (p->ndim == 3) s += 1.0 / (p->deltaz * p->deltaz);
  return cp_max * p->deltat * std::sqrt(s);
}

int cpml_nearest_gridpoint(int nx, int ny, double deltax, double deltay, double x, double y,
                           int* i_out, int* j_out) {
  if (nx < 1 || ny < 1 || !i_out || !j_out) return CPML_ERR_INVALID;
  double dist = 1.0e30;  // HUGEVAL (2D:198)
  int bi = 1, bj = 1;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const double dx = deltax * double(i - 1) - x, dy = deltay * double(j - 1) - y;
      const double d = std::sqrt(dx * dx + dy * dy);
      if (d < dist) { dist = d; bi = i; bj = j; }
    }
  *i_out = bi;
  *j_out = bj;
  return CPML_OK;
}

int cpml_pml_profile(const cpml_params* p, int axis, int n, double* d, double* K, double* alpha,
                     double* a, double* b, double* dh, double* Kh, double* alphah, double* ah,
                     double* bh) {
  if (!p || axis < 0 || axis > 2 || n < 1 || p->npoints_pml < 1) return CPML_ERR_INVALID;
  const double delta = axis == 0 ? p->deltax : (axis == 1 ? p->deltay : p->deltaz);
  if (p->scheme == CPML_SCHEME_SPLIT) {
    // split-field damping divided by two (PML:180-250); K = 1, alpha = a = 0, b = 1
    const double th = p->npoints_pml * delta;
    const double d0 = 3.0 * p->cp * std::log(1.0 / p->rcoef) / (2.0 * th);
    const double ol = th, orr = (n - 1) * delta - th;
    for (int i = 0; i < n; ++i) {
      const double x = delta * double(i);
      double f = 0.0, g = 0.0;
      if (x < ol) {
        f = d0 * std::pow((ol - x) / th, 2);
        g = d0 * std::pow((ol - x - delta / 2.0) / th, 2);
      } else if (x >= 0.9999 * orr) {
        f = d0 * std::pow((x - orr) / th, 2);
        g = d0 * std::pow((x + delta / 2.0 - orr) / th, 2);
      }
      if (d) d[i] = f / 2.0;
      if (dh) dh[i] = g / 2.0;
      if (K) K[i] = 1.0;
      if (Kh) Kh[i] = 1.0;
      if (alpha) alpha[i] = 0.0;
      if (alphah) alphah[i] = 0.0;
      if (a) a[i] = 0.0;
      if (ah) ah[i] = 0.0;
      if (b) b[i] = 1.0;
      if (bh) bh[i] = 1.0;
    }
    return CPML_OK;
  }
  const bool umin = p->use_pml[2 * axis] != 0, umax = p->use_pml[2 * axis + 1] != 0;
  const double amax = p->alpha_max_pml < 0 ? 2.0 * kPi * (p->f0 / 2.0) : p->alpha_max_pml;
  const double th = p->npoints_pml * delta;
  const double d0 = -(p->npower + 1) * p->cp * std::log(p->rcoef) / (2.0 * th);
  // the fourth-order program's y origin is one cell further out (2D4:401)
  const int high = (p->ndim == 2 && p->order == 4 && axis == 1) ? n : n - 1;
  const double ol = th, orr = high * delta - th;
  for (int i = 0; i < n; ++i) {
    double vd = 0, vK = 1, va = 0, vdh = 0, vKh = 1, vah = 0;
    const double val = delta * double(i);
    auto set = [&](double ab, double& dd, double& kk, double& aa) {
      if (ab >= 0.0) {
        const double nr = ab / th;
        dd = d0 * std::pow(nr, p->npower);
        kk = 1.0 + (p->k_max_pml - 1.0) * std::pow(nr, p->npower);
        aa = amax * (1.0 - nr);
      }
    };
    if (umin) { set(ol - val, vd, vK, va); set(ol - (val + delta / 2.0), vdh, vKh, vah); }
    if (umax) { set(val - orr, vd, vK, va); set(val + delta / 2.0 - orr, vdh, vKh, vah); }
    if (va < 0) va = 0;
    if (vah < 0) vah = 0;
    const double vb = std::exp(-(vd / vK + va) * p->deltat);
    const double vbh = std::exp(-(vdh / vKh + vah) * p->deltat);
    const double vA = std::fabs(vd) > 1e-6 ? vd * (vb - 1.0) / (vK * (vd + vK * va)) : 0.0;
    const double vAh = std::fabs(vdh) > 1e-6 ? vdh * (vbh - 1.0) / (vKh * (vdh + vKh * vah)) : 0.0;
    if (d) d[i] = vd;
    if (K) K[i] = vK;
    if (alpha) alpha[i] = va;
    if (a) a[i] = vA;
    if (b) b[i] = vb;
    if (dh) dh[i] = vdh;
    if (Kh) Kh[i] = vKh;
    if (alphah) alphah[i] = vah;
    if (ah) ah[i] = vAh;
    if (bh) bh[i] = vbh;
  }
  return CPML_OK;
}

const char* cpml_strerror(int s) {
  switch (s) {
    case CPML_OK: return "ok";
    case CPML_ERR_INVALID: return "invalid parameter or argument";
    case CPML_ERR_CFL: return "time step is too large, simulation will be unstable (Courant number > 1)";
    case CPML_ERR_OOM: return "device allocation failed";
    case CPML_ERR_UNSTABLE: return "code became unstable and blew up (max |v| > 1e25 or not finite)";
    case CPML_ERR_TIMEOUT: return "a bounded device-side wait gave up";
    case CPML_ERR_CUDA: return "CUDA runtime error (no device, or a failed call)";
    case CPML_ERR_NOT_READY: return "results requested before they exist";
    case CPML_ERR_IO: return "file output failed";
    case CPML_ERR_RANGE: return "size beyond the documented maximum";
    default: return "unknown status";
  }
}

int cpml_write_seismograms(const char* dir, const double* vx, const double* vy, const double* vz,
                           int nt, int nrec, double deltat) {
  if (nt < 0 || nrec < 0 || !vx || !vy) return CPML_ERR_INVALID;
  const double* comp[3] = {vx, vy, vz};
  const char* tag[3] = {"Vx", "Vy", "Vz"};
  for (int c = 0; c < 3; ++c) {
    if (!comp[c]) continue;
    for (int r = 0; r < nrec; ++r) {
      char name[64];
      std::snprintf(name, sizeof name, "%s_file_%03d.dat", tag[c], r + 1);  // 2D:833
      FILE* f = std::fopen(join(dir, name).c_str(), "w");
      if (!f) return CPML_ERR_IO;
      for (int it = 1; it <= nt; ++it) {  // write(11,*) sngl(t),' ',sngl(v)  (2D:839)
        put_real4(f, (float)(double(it - 1) * deltat));
        std::fputs(" ", f);
        put_real4(f, (float)comp[c][size_t(r) * nt + (it - 1)]);
        std::fputc('\n', f);
      }
      if (std::fclose(f) != 0) return CPML_ERR_IO;
    }
  }
  return CPML_OK;
}

int cpml_write_seismograms_su(const char* dir, const double* vx, const double* vy, const double* vz,
                              int nt, int nrec, double deltat) {
  if (nt < 1 || nrec < 0 || !vx || !vy || !(deltat > 0)) return CPML_ERR_INVALID;
  // the header's sample count and interval are 16-bit integers
  // (integer(2) head(1:120), head(58) = nstep, head(59) = deltat*1e6)
  const double dt_us = std::trunc(deltat * 1.0e6);
  if (nt > 32767 || dt_us > 32767.0 || dt_us < 1.0) return CPML_ERR_RANGE;
  int16_t head[120];
  std::memset(head, 0, sizeof head);
  head[57] = (int16_t)nt;
  head[58] = (int16_t)dt_us;
  const double* comp[3] = {vx, vy, vz};
  const char* name[3] = {"seisVx.su", "seisVy.su", "seisVz.su"};
  std::vector<float> trace(nt);
  for (int c = 0; c < 3; ++c) {
    if (!comp[c]) continue;
    FILE* f = std::fopen(join(dir, name[c]).c_str(), "wb");
    if (!f) return CPML_ERR_IO;
    bool ok = true;
    for (int r = 0; r < nrec && ok; ++r) {   // one header + nt REAL(4) samples per receiver
      for (int it = 0; it < nt; ++it) trace[it] = (float)comp[c][size_t(r) * nt + it];
      ok = std::fwrite(head, sizeof head, 1, f) == 1 &&
           std::fwrite(trace.data(), sizeof(float), size_t(nt), f) == size_t(nt);
    }
    if (std::fclose(f) != 0 || !ok) return CPML_ERR_IO;
  }
  return CPML_OK;
}

int cpml_write_energy(const char* dir, const double* ek, const double* ep, int nt, double deltat,
                      int ncol) {
  if (!ek || !ep || nt < 0 || (ncol != 2 && ncol != 4)) return CPML_ERR_INVALID;
  FILE* f = std::fopen(join(dir, "energy.dat").c_str(), "w");
  if (!f) return CPML_ERR_IO;
  for (int it = 1; it <= nt; ++it) {
    put_real4(f, (float)(double(it - 1) * deltat));
    if (ncol == 4) {  // 2D:743: t, Ek, Ep, Ek+Ep as REAL(4)
      put_real4(f, (float)ek[it - 1]);
      put_real4(f, (float)ep[it - 1]);
      put_real4(f, (float)(ek[it - 1] + ep[it - 1]));
    } else {          // 3D:1255: t as REAL(4), total energy as REAL(8)
      put_real8(f, ek[it - 1] + ep[it - 1]);
    }
    std::fputc('\n', f);
  }
  return std::fclose(f) == 0 ? CPML_OK : CPML_ERR_IO;
}

int cpml_write_pnm(const char* dir, const float* data, int nx, int ny, int it, int isource,
                   int jsource, const int* ix_rec, const int* iy_rec, int nrec, int npml,
                   const int* use_pml4, int field_number) {
  if (!data || nx < 1 || ny < 1 || (nrec > 0 && (!ix_rec || !iy_rec))) return CPML_ERR_INVALID;
  const double POWER_DISPLAY = 0.30, cutvect = 0.01;        // 2D:868-871
  const int width_cross = 5, thickness_cross = 1, size_square = 3;  // 2D:877
  char name[64];
  std::snprintf(name, sizeof name, "image%06d_%s.pnm", it, field_number == 1 ? "Vx" : "Vy");
  FILE* f = std::fopen(join(dir, name).c_str(), "w");
  if (!f) return CPML_ERR_IO;
  std::fprintf(f, "P3\n%12d%12d\n 255\n", nx, ny);
  double amax = 0.0;
  for (size_t c = 0; c < size_t(nx) * ny; ++c) amax = std::fmax(amax, std::fabs((double)data[c]));
  const bool ux0 = use_pml4 && use_pml4[0], ux1 = use_pml4 && use_pml4[1];
  const bool uy0 = use_pml4 && use_pml4[2], uy1 = use_pml4 && use_pml4[3];
  for (int iy = ny; iy >= 1; --iy)       // image starts in the upper-left corner (2D:916)
    for (int ix = 1; ix <= nx; ++ix) {
      const double v = data[size_t(iy - 1) * nx + (ix - 1)];
      double nv = v / amax;
      if (nv < -1.0) nv = -1.0;
      if (nv > 1.0) nv = 1.0;
      int R, G, B;
      if ((ix >= isource - width_cross && ix <= isource + width_cross &&
           iy >= jsource - thickness_cross && iy <= jsource + thickness_cross) ||
          (ix >= isource - thickness_cross && ix <= isource + thickness_cross &&
           iy >= jsource - width_cross && iy <= jsource + width_cross)) {
        R = 255; G = 157; B = 0;          // orange source cross
      } else if (ix <= 2 || ix >= nx - 1 || iy <= 2 || iy >= ny - 1) {
        R = 0; G = 0; B = 0;              // black frame
      } else if ((ux0 && ix == npml) || (ux1 && ix == nx - npml) || (uy0 && iy == npml) ||
                 (uy1 && iy == ny - npml)) {
        R = 255; G = 150; B = 0;          // PML edges
      } else if (std::fabs(v) <= amax * cutvect) {
        R = 255; G = 255; B = 255;        // white background
      } else if (nv >= 0.0) {
        R = (int)std::lround(255.0 * std::pow(nv, POWER_DISPLAY)); G = 0; B = 0;
      } else {
        R = 0; G = 0; B = (int)std::lround(255.0 * std::pow(std::fabs(nv), POWER_DISPLAY));
      }
      for (int r = 0; r < nrec; ++r)
        if (ix >= ix_rec[r] - size_square && ix <= ix_rec[r] + size_square &&
            iy >= iy_rec[r] - size_square && iy <= iy_rec[r] + size_square) {
          R = 30; G = 180; B = 60;        // green receiver squares
        }
      std::fprintf(f, "%3d %3d %3d\n", R, G, B);
    }
  return std::fclose(f) == 0 ? CPML_OK : CPML_ERR_IO;
}

}  // extern "C"
