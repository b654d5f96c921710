// driver.cpp -- cpml_program: the two reference programs as one C++ host
// program over the C ABI.
//
// Usage:  cpml_program [2d|3d] [params.par] [output_dir]
//
// It replaces the main program units of
//   seismic_CPML_2D_isotropic_second_order.f90  (program seismic_CPML_2D_iso_second)
//   seismic_CPML_3D_isotropic_MPI_OpenMP.f90    (program seismic_CPML_3D_iso_MPI_OpenMP)
// with the same flow: the parameter block (defaults = the reference's
// constants, 2D:138-218 / 3D:124-218, overridable by "NAME = value" lines
// using the Fortran names), receivers placed by the nearest-point rule
// (2D:483-509), the Courant check (2D:513-516), the time loop in
// IT_DISPLAY pieces with the progress print-out and PNM snapshots at the
// display steps (2D:716-733), and the final seismogram files, energy.dat and
// gnuplot scripts (2D:738-808, 3D:1247-1319). The reference's stop messages
// are printed and the program exits non-zero where the reference stops.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cpml.h"

namespace {

std::string upper(std::string s) {
  for (char& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

struct Setup {
  cpml_params p{};
  // receivers as the reference defines them (metres), 2D:180-183 / 3D:175-178
  int nrec = 2;
  double xdeb = 0, ydeb = 2300.0, xfin = 0, yfin = 300.0;
  bool rec_given = false;
  std::map<std::string, bool> given;
};

// "NAME = value" lines, Fortran names, '!' or '#' comments; logicals as
// .true./.false./1/0.
int read_params(const char* path, Setup& S) {
  std::ifstream f(path);
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path); return 1; }
  std::string line;
  int ln = 0;
  while (std::getline(f, line)) {
    ++ln;
    for (char c : {'!', '#'}) {
      const size_t q = line.find(c);
      if (q != std::string::npos) line = line.substr(0, q);
    }
    const size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    std::string k = upper(line.substr(0, eq)), v = line.substr(eq + 1);
    k.erase(0, k.find_first_not_of(" \t"));
    k.erase(k.find_last_not_of(" \t") + 1);
    v.erase(0, v.find_first_not_of(" \t"));
    v.erase(v.find_last_not_of(" \t\r") + 1);
    const std::string vu = upper(v);
    std::string num = v;                       // Fortran double literals: 2.d-3
    for (char& c : num)
      if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    const double d = std::strtod(num.c_str(), &end);
    const bool logical = vu == ".TRUE." || vu == "T" || vu == ".FALSE." || vu == "F";
    const bool numeric = end != num.c_str() && *end == '\0';
    if (k != "SOURCE_TIME_FUNCTION" && !logical && !numeric) {   // a number or a logical, nothing else
      std::fprintf(stderr, "%s:%d: bad value for %s: '%s'\n", path, ln, k.c_str(), v.c_str());
      return 1;
    }
    S.given[k] = true;
    const int iv = (vu == ".TRUE." || vu == "T") ? 1 : (vu == ".FALSE." || vu == "F") ? 0 : (int)std::lround(d);
    cpml_params& p = S.p;
    if (k == "NX") p.nx = iv;
    else if (k == "NY") p.ny = iv;
    else if (k == "NZ") p.nz = iv;
    else if (k == "NSTEP") p.nstep = iv;
    else if (k == "NPOINTS_PML") p.npoints_pml = iv;
    else if (k == "DELTAX") { p.deltax = d; }
    else if (k == "DELTAY") p.deltay = d;
    else if (k == "DELTAZ") p.deltaz = d;
    else if (k == "DELTAT") p.deltat = d;
    else if (k == "CP") p.cp = d;
    else if (k == "CS") p.cs = d;
    else if (k == "RHO" || k == "DENSITY") p.rho = d;
    else if (k == "F0") p.f0 = d;
    else if (k == "T0") p.t0 = d;
    else if (k == "FACTOR") p.factor = d;
    else if (k == "ANGLE_FORCE") p.angle_force = d;
    else if (k == "ISOURCE") p.isource = iv;
    else if (k == "JSOURCE") p.jsource = iv;
    else if (k == "KSOURCE") p.ksource = iv;
    else if (k == "IT_DISPLAY") p.it_display = iv;
    else if (k == "NPOWER") p.npower = d;
    else if (k == "K_MAX_PML") p.k_max_pml = d;
    else if (k == "ALPHA_MAX_PML") p.alpha_max_pml = d;
    else if (k == "RCOEF") p.rcoef = d;
    else if (k == "USE_PML_XMIN") p.use_pml[0] = iv;
    else if (k == "USE_PML_XMAX") p.use_pml[1] = iv;
    else if (k == "USE_PML_YMIN") p.use_pml[2] = iv;
    else if (k == "USE_PML_YMAX") p.use_pml[3] = iv;
    else if (k == "USE_PML_ZMIN") p.use_pml[4] = iv;
    else if (k == "USE_PML_ZMAX") p.use_pml[5] = iv;
    else if (k == "SOURCE_TIME_FUNCTION") {
      p.stf = vu.find("RICKER") != std::string::npos ? CPML_STF_RICKER
            : vu.find("DERIV") != std::string::npos ? CPML_STF_DGAUSSIAN : CPML_STF_GAUSSIAN;
    } else if (k == "NREC") { S.nrec = iv; S.rec_given = true; }
    else if (k == "XDEB") { S.xdeb = d; S.rec_given = true; }
    else if (k == "YDEB") { S.ydeb = d; S.rec_given = true; }
    else if (k == "XFIN") { S.xfin = d; S.rec_given = true; }
    else if (k == "YFIN") { S.yfin = d; S.rec_given = true; }
    else if (k == "EP_PHYSICAL") { if (iv) p.flags |= CPML_FLAG_EP_PHYSICAL; }
    else { std::fprintf(stderr, "%s:%d: unknown parameter %s\n", path, ln, k.c_str()); return 1; }
  }
  return 0;
}

void write_gnuplot(const std::string& dir, bool three_d, int nrec) {
  FILE* f = std::fopen((dir + "/plot_energy").c_str(), "w");
  if (f) {
    std::fprintf(f, " # set term x11\n set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                    " set xlabel \"Time (s)\"\n set ylabel \"Total energy\"\n\n set output \"%s\"\n set logscale y\n",
                 three_d ? "CPML3D_total_energy_semilog.eps" : "cpml_total_energy_semilog.eps");
    if (three_d)
      std::fprintf(f, " plot \"energy.dat\" t 'Total energy' w l lc 1\n");
    else
      std::fprintf(f, " plot \"energy.dat\" us 1:2 t 'Ec' w l lc 1, \"energy.dat\" us 1:3 t 'Ep' w l lc 3, "
                      "\"energy.dat\" us 1:4 t 'Total energy' w l lc 4\n");
    std::fprintf(f, " pause -1 \"Hit any key...\"\n\n");
    std::fclose(f);
  }
  if (!three_d) {
    // energy of this run against the classical split-field PML run of the
    // Collino program in ../collino (2D:764-777)
    f = std::fopen((dir + "/plot_comparison").c_str(), "w");
    if (f) {
      std::fprintf(f, " # set term x11\n set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                      " set xlabel \"Time (s)\"\n set ylabel \"Total energy\"\n\n"
                      " set output \"compare_total_energy_semilog.eps\"\n set logscale y\n"
                      " plot \"energy.dat\" us 1:4 t 'Total energy CPML' w l lc 1, "
                      "\"../collino/energy.dat\" us 1:4 t 'Total energy Collino' w l lc 2\n"
                      " pause -1 \"Hit any key...\"\n\n");
      std::fclose(f);
    }
  }
  f = std::fopen((dir + "/plotgnu").c_str(), "w");
  if (f) {
    std::fprintf(f, " set term x11\n # set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                    " set xlabel \"Time (s)\"\n set ylabel \"Amplitude (m / s)\"\n\n");
    const char* comps[3] = {"Vx", "Vy", "Vz"};
    for (int r = 1; r <= nrec; ++r)
      for (int c = 0; c < (three_d ? 3 : 2); ++c)
        std::fprintf(f, " set output \"v_sigma_%s_receiver_%03d.eps\"\n plot \"%s_file_%03d.dat\" t '%s C-PML' w l lc 1\n"
                        " pause -1 \"Hit any key...\"\n\n", comps[c], r, comps[c], r, comps[c]);
    std::fclose(f);
  }
}

}  // namespace

int main(int argc, char** argv) {
  const bool three_d = argc > 1 && std::strcmp(argv[1], "3d") == 0;
  Setup S;
  if (three_d) cpml_params_default_3d(&S.p); else cpml_params_default_2d(&S.p);
  if (argc > 2 && std::strcmp(argv[2], "-") != 0 && read_params(argv[2], S)) return 2;
  const std::string dir = argc > 3 ? argv[3] : ".";
  cpml_params& p = S.p;
  // derived constants of the parameter block follow the grid unless given
  if (!S.given["ISOURCE"]) p.isource = p.nx - 2 * p.npoints_pml - 1;   // 2D:174
  if (!S.given["JSOURCE"]) p.jsource = 2 * p.ny / 3 + 1;               // 2D:175
  if (!S.given["KSOURCE"] && three_d) p.ksource = p.nz / 2;            // cut plane NZ/2
  if (!S.given["T0"]) p.t0 = 1.20 / p.f0;                               // 2D:170
  if (!S.given["DELTAY"]) p.deltay = p.deltax;                          // 2D:146
  if (!S.given["DELTAZ"]) p.deltaz = p.deltax;
  if (!S.rec_given || S.xfin == 0) {
    const double xsource = (p.isource - 1) * p.deltax;   // 2D:178, 180-183
    if (!S.rec_given || S.xdeb == 0) S.xdeb = xsource - 100.0;
    if (S.xfin == 0) S.xfin = xsource;
  }

  std::printf("\n %dD elastic finite-difference code in velocity and stress formulation with C-PML\n\n",
              three_d ? 3 : 2);
  std::printf(" NX = %d\n NY = %d\n", p.nx, p.ny);
  if (three_d) std::printf(" NZ = %d\n", p.nz);
  std::printf(" Total number of grid points = %lld\n\n", (long long)p.nx * p.ny * (three_d ? p.nz : 1));

  // receivers on the segment (xdeb, ydeb) - (xfin, yfin) (2D:487-509)
  std::vector<int> ix(S.nrec), iy(S.nrec), iz(S.nrec, p.ksource);
  const double xs = S.nrec > 1 ? (S.xfin - S.xdeb) / (S.nrec - 1) : 0.0;
  const double ys = S.nrec > 1 ? (S.yfin - S.ydeb) / (S.nrec - 1) : 0.0;
  for (int r = 0; r < S.nrec; ++r) {
    const double xr = S.xdeb + r * xs, yr = S.ydeb + r * ys;
    cpml_nearest_gridpoint(p.nx, p.ny, p.deltax, p.deltay, xr, yr, &ix[r], &iy[r]);
    std::printf(" receiver %d x_target,y_target = %g %g\n closest grid point found in i,j = %d %d\n\n", r + 1,
                xr, yr, ix[r], iy[r]);
  }
  std::printf(" Courant number is %.15g\n\n", cpml_courant(&p, p.cp));

  cpml_handle* h = nullptr;
  int st = cpml_create(&p, &h);
  if (st == CPML_ERR_CFL) { std::printf(" time step is too large, simulation will be unstable\n"); return 3; }
  if (st != CPML_OK) { std::printf(" cpml_create: %s\n", cpml_strerror(st)); return 4; }
  if ((st = cpml_set_receivers(h, S.nrec, ix.data(), iy.data(), iz.data())) != CPML_OK) {
    std::printf(" cpml_set_receivers: %s\n", cpml_strerror(st));
    cpml_destroy(h);
    return 4;
  }
  std::vector<float> plane(size_t(p.nx) * p.ny);
  int it = 0;
  const int use4[4] = {p.use_pml[0], p.use_pml[1], p.use_pml[2], p.use_pml[3]};
  std::vector<double> ek(p.nstep), ep(p.nstep);
  while (it < p.nstep) {
    int next = (it / p.it_display + 1) * p.it_display;
    if (it < 5) next = std::min(next, 5);
    next = std::min(next, p.nstep);
    st = cpml_run(h, next - it);
    double vmax = 0;
    cpml_status(h, &it, &vmax);
    if (st == CPML_ERR_UNSTABLE) {
      std::printf(" code became unstable and blew up\n");
      cpml_destroy(h);
      return 5;
    }
    if (st != CPML_OK) { std::printf(" cpml_run: %s\n", cpml_strerror(st)); cpml_destroy(h); return 4; }
    if (it % p.it_display == 0 || it == 5) {             // 2D:716-733
      cpml_get_energy(h, ek.data(), ep.data());
      std::printf(" Time step # %d out of %d\n Time: %g seconds\n Max norm velocity vector V (m/s) = %.15g\n"
                  " total energy = %.15g\n\n", it, p.nstep, (float)((it - 1) * p.deltat), vmax,
                  ek[it - 1] + ep[it - 1]);
      const int k = three_d ? p.ksource : 1;
      for (int fld = 0; fld < 2; ++fld) {
        cpml_get_plane(h, fld == 0 ? CPML_FIELD_VX : CPML_FIELD_VY, 2, k, plane.data());
        cpml_write_pnm(dir.c_str(), plane.data(), p.nx, p.ny, it, p.isource, p.jsource, ix.data(), iy.data(),
                       S.nrec, p.npoints_pml, use4, fld + 1);
      }
    }
  }
  std::vector<double> sx(size_t(S.nrec) * p.nstep), sy(sx.size()), sz(sx.size());
  cpml_get_seismograms(h, sx.data(), sy.data(), three_d ? sz.data() : nullptr);
  cpml_get_energy(h, ek.data(), ep.data());
  // the 3D reference writes no Vz files (its gnuplot script names them, 3D:1293-1296)
  if ((st = cpml_write_seismograms(dir.c_str(), sx.data(), sy.data(), nullptr, p.nstep, S.nrec, p.deltat)) ||
      (st = cpml_write_energy(dir.c_str(), ek.data(), ep.data(), p.nstep, p.deltat, three_d ? 2 : 4))) {
    std::printf(" writing outputs: %s\n", cpml_strerror(st));
    cpml_destroy(h);
    return 6;
  }
  write_gnuplot(dir, three_d, S.nrec);
  cpml_destroy(h);
  std::printf("\n End of the simulation\n\n");
  return 0;
}
