// driver.cpp -- cpml_program: the two reference programs as one C++ host
// program over the C ABI.
//
// Usage:  cpml_program [2d|2d4|2dpml|3d] [params.par | program.f90] [output_dir]
//                      [--print-params | --scripts-only]
//
// 2d4 and 2dpml run the fourth-order program and the classical split-field
// PML program (seismic_CPML_2D_isotropic_fourth_order.f90,
// seismic_PML_Collino_2D_isotropic.f90) with the same flow and outputs.
//
// The parameters come from a params.par file of "NAME = value" lines, or
// from a reference program's own source file (.f90): its parameter block,
// evaluated as Fortran evaluates it (read_fortran_params).
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
#include <chrono>
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

// ---- the reference program's own source as the parameter file -------------
// A reference program is configured by editing its `parameter` lines
// (2D:138-218, 3D:124-218). Given that .f90 file, the driver evaluates those
// declarations as Fortran does: integer arithmetic truncates, literals
// without a D exponent are single precision, ** with an integer exponent is
// repeated multiplication. It also reads Rcoef from its assignment (2D:289)
// and the wavelet from whichever source_term line is not commented out
// (2D:648-654). Names the solver has no use for (PI, HUGEVAL, NPROC, ...)
// are evaluated and ignored.
struct FVal {
  double v = 0;
  int kind = 2;   // 0 integer/logical, 1 single precision, 2 double precision
};

FVal fnorm(FVal x) {
  if (x.kind == 1) x.v = double(float(x.v));
  return x;
}

class FExpr {
 public:
  FExpr(const std::string& s, const std::map<std::string, FVal>& sym) : s_(s), sym_(sym) {}
  bool eval(FVal* out, std::string* err) {
    FVal v = add();
    skip();
    if (!err_.empty() || i_ != s_.size()) {
      *err = err_.empty() ? "unexpected '" + s_.substr(i_) + "'" : err_;
      return false;
    }
    *out = v;
    return true;
  }

 private:
  const std::string& s_;
  const std::map<std::string, FVal>& sym_;
  size_t i_ = 0;
  std::string err_;
  void skip() { while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_; }
  bool eat(const char* t) {
    skip();
    const size_t n = std::strlen(t);
    if (s_.compare(i_, n, t) == 0) { i_ += n; return true; }
    return false;
  }
  static FVal arith(char op, FVal a, FVal b) {
    FVal r;
    r.kind = std::max(a.kind, b.kind);
    if (r.kind == 0) {
      const long long x = (long long)a.v, y = (long long)b.v;
      r.v = double(op == '+' ? x + y : op == '-' ? x - y : op == '*' ? x * y : (y ? x / y : 0));
      return r;
    }
    r.v = op == '+' ? a.v + b.v : op == '-' ? a.v - b.v : op == '*' ? a.v * b.v : a.v / b.v;
    return fnorm(r);
  }
  FVal add() {
    FVal v;
    if (eat("-")) { v = mul(); v.v = -v.v; }
    else { eat("+"); v = mul(); }
    for (;;) {
      if (eat("+")) v = arith('+', v, mul());
      else if (eat("-")) v = arith('-', v, mul());
      else return v;
    }
  }
  FVal mul() {
    FVal v = pw();
    for (;;) {
      skip();
      if (s_.compare(i_, 2, "**") == 0) return v;
      if (eat("*")) v = arith('*', v, pw());
      else if (eat("/")) v = arith('/', v, pw());
      else return v;
    }
  }
  FVal pw() {
    FVal b = prim();
    if (!eat("**")) return b;
    FVal e = pw();
    FVal r;
    if (e.kind == 0) {   // by multiplication, squaring (gfortran's lowering of x**n)
      const long long n = (long long)e.v;
      unsigned long long m = n < 0 ? 0ull - (unsigned long long)n : (unsigned long long)n;
      r.kind = b.kind;
      auto mul = [&](double x, double y) { return r.kind == 1 ? double(float(x * y)) : x * y; };
      double x = b.v, acc = (m & 1) ? x : 1.0;
      while (m >>= 1) {
        x = mul(x, x);
        if (m & 1) acc = mul(acc, x);
      }
      r.v = n < 0 ? 1.0 / acc : acc;
      return fnorm(r);
    }
    r.kind = (b.kind == 2 || e.kind == 2) ? 2 : 1;   // a real power of reals
    r.v = std::pow(b.v, e.v);
    return fnorm(r);
  }
  FVal prim() {
    skip();
    FVal v;
    if (eat("(")) {
      v = add();
      if (!eat(")")) err_ = "missing ')'";
      return v;
    }
    if (eat(".true.")) { v.v = 1; v.kind = 0; return v; }
    if (eat(".false.")) { v.v = 0; v.kind = 0; return v; }
    if (i_ < s_.size() && (std::isdigit((unsigned char)s_[i_]) || s_[i_] == '.')) {
      const size_t b = i_;
      while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
      bool real = false;
      if (i_ < s_.size() && s_[i_] == '.' && !(i_ + 1 < s_.size() && std::isalpha((unsigned char)s_[i_ + 1]) &&
                                                 s_[i_ + 1] != 'd' && s_[i_ + 1] != 'e')) {
        real = true;
        ++i_;
        while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
      }
      int kind = real ? 1 : 0;
      if (i_ < s_.size() && (s_[i_] == 'd' || s_[i_] == 'e')) {
        kind = s_[i_] == 'd' ? 2 : 1;
        ++i_;
        if (i_ < s_.size() && (s_[i_] == '+' || s_[i_] == '-')) ++i_;
        while (i_ < s_.size() && std::isdigit((unsigned char)s_[i_])) ++i_;
      }
      std::string t = s_.substr(b, i_ - b);
      for (char& c : t) if (c == 'd') c = 'e';
      v.kind = kind;
      v.v = kind == 0 ? double(std::strtoll(t.c_str(), nullptr, 10))
                      : kind == 1 ? double(std::strtof(t.c_str(), nullptr)) : std::strtod(t.c_str(), nullptr);
      return v;
    }
    size_t b = i_;
    while (i_ < s_.size() && (std::isalnum((unsigned char)s_[i_]) || s_[i_] == '_')) ++i_;
    const std::string name = s_.substr(b, i_ - b);
    auto it = sym_.find(name);
    if (name.empty() || it == sym_.end()) {
      if (err_.empty()) err_ = name.empty() ? "expected a value" : "unknown name " + name;
      return v;
    }
    return it->second;
  }
};

// statements of a free-form Fortran file: comments removed, continuation
// lines joined, lower case outside string literals
std::vector<std::string> fortran_statements(std::istream& in) {
  std::vector<std::string> out;
  std::string line, buf;
  char quote = 0;
  while (std::getline(in, line)) {
    if (!buf.empty()) {
      const size_t b = line.find_first_not_of(" \t");
      line = b == std::string::npos ? "" : line.substr(b);
      if (!line.empty() && line[0] == '&') line = line.substr(1);
    }
    std::string t;
    for (char c : line) {
      if (quote) { t += c; if (c == quote) quote = 0; continue; }
      if (c == '\'' || c == '"') { quote = c; t += c; continue; }
      if (c == '!') break;
      t += (char)std::tolower((unsigned char)c);
    }
    t.erase(t.find_last_not_of(" \t\r") + 1);
    if (t.empty()) continue;
    if (t.back() == '&') { t.pop_back(); buf += t; continue; }
    buf += t;
    const size_t b = buf.find_first_not_of(" \t");
    out.push_back(buf.substr(b));
    buf.clear();
    quote = 0;
  }
  return out;
}

std::vector<std::string> split_top(const std::string& s) {
  std::vector<std::string> out;
  int depth = 0;
  std::string cur;
  for (char c : s) {
    if (c == '(') ++depth;
    if (c == ')') --depth;
    if (c == ',' && depth == 0) { out.push_back(cur); cur.clear(); continue; }
    cur += c;
  }
  out.push_back(cur);
  return out;
}

std::string trim(const std::string& s) {
  const size_t b = s.find_first_not_of(" \t"), e = s.find_last_not_of(" \t");
  return b == std::string::npos ? "" : s.substr(b, e - b + 1);
}

int read_fortran_params(const char* path, Setup& S, bool three_d) {
  std::ifstream f(path);
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path); return 1; }
  std::map<std::string, FVal> sym;
  int n_source_lines = 0;
  for (const std::string& st : fortran_statements(f)) {
    const bool decl = st.rfind("integer", 0) == 0 || st.rfind("double precision", 0) == 0 ||
                      st.rfind("logical", 0) == 0 || st.rfind("real", 0) == 0;
    const size_t dc = st.find("::");
    if (decl && dc != std::string::npos && st.substr(0, dc).find("parameter") != std::string::npos) {
      const int kind = st.rfind("integer", 0) == 0 || st.rfind("logical", 0) == 0 ? 0
                       : st.rfind("real", 0) == 0 ? 1 : 2;
      for (const std::string& ent : split_top(st.substr(dc + 2))) {
        const size_t eq = ent.find('=');
        if (eq == std::string::npos) continue;
        const std::string name = trim(ent.substr(0, eq)), ex = trim(ent.substr(eq + 1));
        FVal v;
        std::string err;
        if (!FExpr(ex, sym).eval(&v, &err)) {
          std::fprintf(stderr, "%s: parameter %s = %s: %s\n", path, name.c_str(), ex.c_str(), err.c_str());
          return 1;
        }
        if (kind == 0) v.v = double((long long)v.v);   // integer parameters truncate
        v.kind = kind;
        sym[name] = fnorm(v);
      }
      continue;
    }
    // Rcoef is assigned, not declared a parameter (2D:289, 3D:408)
    if (st.rfind("rcoef", 0) == 0 && st.find('=') != std::string::npos) {
      FVal v;
      std::string err;
      if (FExpr(trim(st.substr(st.find('=') + 1)), sym).eval(&v, &err)) sym["rcoef"] = v;
      continue;
    }
    // the active source-time function (2D:648-654): its source_term line
    if (st.rfind("source_term", 0) == 0 && st.find('=') != std::string::npos) {
      ++n_source_lines;
      const std::string r = st.substr(st.find('=') + 1);
      S.p.stf = r.find("(1.d0 - 2.d0") != std::string::npos ? CPML_STF_RICKER
              : r.find("2.d0*a*(t-t0)") != std::string::npos ? CPML_STF_DGAUSSIAN : CPML_STF_GAUSSIAN;
    }
  }
  if (n_source_lines != 1) {
    std::fprintf(stderr, "%s: expected one active source_term line, found %d\n", path, n_source_lines);
    return 1;
  }
  auto get = [&](const char* k, double* dst) {
    auto it = sym.find(k);
    if (it != sym.end()) { *dst = it->second.v; S.given[upper(k)] = true; }
    return it != sym.end();
  };
  auto geti = [&](const char* k, int* dst) {
    double v;
    if (get(k, &v)) *dst = (int)v;
  };
  cpml_params& p = S.p;
  const char* need[] = {"nx", "ny", "deltat", "nstep", "npoints_pml", "cp", "cs", "f0",
                        "factor", "isource", "jsource", "angle_force"};
  for (const char* k : need)
    if (!sym.count(k)) { std::fprintf(stderr, "%s: no parameter %s\n", path, k); return 1; }
  if (!sym.count("deltax") && !sym.count("h")) { std::fprintf(stderr, "%s: no parameter DELTAX or h\n", path); return 1; }
  geti("nx", &p.nx); geti("ny", &p.ny); geti("nstep", &p.nstep); geti("npoints_pml", &p.npoints_pml);
  if (get("h", &p.deltax)) {     // the split-field program's one grid spacing (PML:100)
    p.deltay = p.deltax;
    S.given["DELTAX"] = S.given["DELTAY"] = true;
  }
  get("deltax", &p.deltax); get("deltay", &p.deltay); get("deltat", &p.deltat);
  get("cp", &p.cp); get("cs", &p.cs); get("f0", &p.f0); get("t0", &p.t0); get("factor", &p.factor);
  if (!get("density", &p.rho)) get("rho", &p.rho);
  geti("isource", &p.isource); geti("jsource", &p.jsource); get("angle_force", &p.angle_force);
  geti("it_display", &p.it_display);
  get("npower", &p.npower); get("k_max_pml", &p.k_max_pml); get("alpha_max_pml", &p.alpha_max_pml);
  get("rcoef", &p.rcoef);
  const char* faces[6] = {"use_pml_xmin", "use_pml_xmax", "use_pml_ymin", "use_pml_ymax",
                          "use_pml_zmin", "use_pml_zmax"};
  for (int q = 0; q < (three_d ? 6 : 4); ++q) geti(faces[q], &p.use_pml[q]);
  if (three_d) {
    geti("nz", &p.nz);
    get("deltaz", &p.deltaz);
    p.ksource = p.nz / 2;      // the cut plane of rank nb_procs/2 - 1 (3D:346, 1080)
    S.given["KSOURCE"] = true;
  }
  int nrec = S.nrec;
  geti("nrec", &nrec);
  S.nrec = nrec;
  get("xdeb", &S.xdeb); get("ydeb", &S.ydeb); get("xfin", &S.xfin); get("yfin", &S.yfin);
  S.rec_given = true;
  return 0;
}

void print_params(const Setup& S, bool three_d) {
  const cpml_params& p = S.p;
  std::printf("NX = %d\nNY = %d\n", p.nx, p.ny);
  if (three_d) std::printf("NZ = %d\n", p.nz);
  std::printf("NSTEP = %d\nNPOINTS_PML = %d\nIT_DISPLAY = %d\n", p.nstep, p.npoints_pml, p.it_display);
  std::printf("DELTAX = %.17g\nDELTAY = %.17g\n", p.deltax, p.deltay);
  if (three_d) std::printf("DELTAZ = %.17g\n", p.deltaz);
  std::printf("DELTAT = %.17g\ncp = %.17g\ncs = %.17g\nrho = %.17g\n", p.deltat, p.cp, p.cs, p.rho);
  std::printf("f0 = %.17g\nt0 = %.17g\nfactor = %.17g\nANGLE_FORCE = %.17g\n", p.f0, p.t0, p.factor,
              p.angle_force);
  std::printf("ISOURCE = %d\nJSOURCE = %d\n", p.isource, p.jsource);
  if (three_d) std::printf("KSOURCE = %d\n", p.ksource);
  std::printf("NPOWER = %.17g\nK_MAX_PML = %.17g\nALPHA_MAX_PML = %.17g\nRCOEF = %.17g\n", p.npower,
              p.k_max_pml, p.alpha_max_pml, p.rcoef);
  const char* faces[6] = {"USE_PML_XMIN", "USE_PML_XMAX", "USE_PML_YMIN", "USE_PML_YMAX",
                          "USE_PML_ZMIN", "USE_PML_ZMAX"};
  for (int q = 0; q < (three_d ? 6 : 4); ++q) std::printf("%s = %s\n", faces[q], p.use_pml[q] ? ".true." : ".false.");
  std::printf("! program: %s\n", p.scheme == CPML_SCHEME_SPLIT ? "split-field PML (PML)"
                                 : p.order == 4 ? "fourth order (2D4)" : three_d ? "3D" : "2D");
  std::printf("SOURCE_TIME_FUNCTION = %s\n", p.stf == CPML_STF_RICKER ? "ricker"
                                            : p.stf == CPML_STF_DGAUSSIAN ? "derivative_of_gaussian" : "gaussian");
  std::printf("NREC = %d\nXDEB = %.17g\nYDEB = %.17g\nXFIN = %.17g\nYFIN = %.17g\n", S.nrec, S.xdeb, S.ydeb,
              S.xfin, S.yfin);
}

// split: the Collino program's scripts (PML:562-606), which name the energy
// plot collino_total_energy_semilog.eps and write no plot_comparison
void write_gnuplot(const std::string& dir, bool three_d, bool split, int nrec) {
  FILE* f = std::fopen((dir + "/plot_energy").c_str(), "w");
  if (f) {
    std::fprintf(f, " # set term x11\n set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                    " set xlabel \"Time (s)\"\n set ylabel \"Total energy\"\n\n set output \"%s\"\n set logscale y\n",
                 three_d ? "CPML3D_total_energy_semilog.eps"
                 : split ? "collino_total_energy_semilog.eps" : "cpml_total_energy_semilog.eps");
    if (three_d)
      std::fprintf(f, " plot \"energy.dat\" t 'Total energy' w l lc 1\n");
    else
      // two blanks where the programs continue the string literal (2D:759-760)
      std::fprintf(f, " plot \"energy.dat\" us 1:2 t 'Ec' w l lc 1, \"energy.dat\" us 1:3  t 'Ep' w l lc 3, "
                      "\"energy.dat\" us 1:4 t 'Total energy' w l lc 4\n");
    std::fprintf(f, " pause -1 \"Hit any key...\"\n\n");
    std::fclose(f);
  }
  if (!three_d && !split) {
    // energy of this run against the classical split-field PML run of the
    // Collino program in ../collino (2D:764-777)
    f = std::fopen((dir + "/plot_comparison").c_str(), "w");
    if (f) {
      std::fprintf(f, " # set term x11\n set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                      " set xlabel \"Time (s)\"\n set ylabel \"Total energy\"\n\n"
                      " set output \"compare_total_energy_semilog.eps\"\n set logscale y\n"
                      " plot \"energy.dat\" us 1:4 t 'Total energy CPML' w l lc 1,  "
                      "\"../collino/energy.dat\" us 1:4 t 'Total energy Collino' w l lc 2\n"
                      " pause -1 \"Hit any key...\"\n\n");
      std::fclose(f);
    }
  }
  f = std::fopen((dir + "/plotgnu").c_str(), "w");
  if (f) {
    std::fprintf(f, " set term x11\n # set term postscript landscape monochrome dashed \"Helvetica\" 22\n\n"
                    " set xlabel \"Time (s)\"\n set ylabel \"Amplitude (m / s)\"\n\n");
    // the programs plot receivers 1 and 2, written out, whatever NREC is
    // (2D:784-806, 3D:1273-1310); 3D adds Vz files it never writes (3D:1293-1296)
    (void)nrec;
    const char* comps[3] = {"Vx", "Vy", "Vz"};
    for (int r = 1; r <= 2; ++r)
      for (int c = 0; c < (three_d ? 3 : 2); ++c)
        std::fprintf(f, " set output \"v_sigma_%s_receiver_%03d.eps\"\n plot \"%s_file_%03d.dat\" t '%s C-PML' w l lc 1\n"
                        " pause -1 \"Hit any key...\"\n\n", comps[c], r, comps[c], r, comps[c]);
    std::fclose(f);
  }
}

}  // namespace

int main(int argc_in, char** argv_in) {
  // --print-params: print the resolved parameter block (params.par format)
  // and the receiver points, then stop before any device call
  // --scripts-only: write the gnuplot scripts of the resolved run and stop
  bool print_only = false, scripts_only = false;
  std::vector<char*> args;
  for (int a = 0; a < argc_in; ++a) {
    if (std::strcmp(argv_in[a], "--print-params") == 0) print_only = true;
    else if (std::strcmp(argv_in[a], "--scripts-only") == 0) scripts_only = true;
    else args.push_back(argv_in[a]);
  }
  const int argc = (int)args.size();
  char** argv = args.data();
  // 2d: seismic_CPML_2D_isotropic_second_order; 2d4: the fourth-order
  // program; 2dpml: seismic_PML_Collino_2D_isotropic; 3d: the MPI program
  const std::string mode = argc > 1 ? argv[1] : "2d";
  if (mode != "2d" && mode != "3d" && mode != "2d4" && mode != "2dpml") {
    std::fprintf(stderr, "usage: cpml_program [2d|2d4|2dpml|3d] [params.par | program.f90 | -] [output_dir] "
                         "[--print-params]\n");
    return 2;
  }
  const bool three_d = mode == "3d";
  Setup S;
  if (three_d) cpml_params_default_3d(&S.p);
  else if (mode == "2d4") cpml_params_default_2d_fourth(&S.p);
  else if (mode == "2dpml") cpml_params_default_2d_split(&S.p);
  else cpml_params_default_2d(&S.p);
  if (argc > 2 && std::strcmp(argv[2], "-") != 0) {
    const std::string path = argv[2];
    const bool f90 = path.size() > 4 && upper(path.substr(path.size() - 4)) == ".F90";
    if ((f90 ? read_fortran_params(argv[2], S, three_d) : read_params(argv[2], S))) return 2;
  }
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
  if (print_only) {
    print_params(S, three_d);
    return 0;
  }
  if (scripts_only) {
    write_gnuplot(dir, three_d, mode == "2dpml", S.nrec);
    return 0;
  }

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
  const auto t_start = std::chrono::steady_clock::now();
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
      if (three_d) {   // elapsed time, and its timestamp file (3D:1197-1228)
        const double tcpu =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        const int itc = (int)tcpu, hh = itc / 3600, mm = (itc - 3600 * hh) / 60, ss = itc - 3600 * hh - 60 * mm;
        char lines[512];
        std::snprintf(lines, sizeof lines,
                      " Elapsed time in seconds = %.15g\n Elapsed time in hh:mm:ss = %4d h %02d m %02d s\n"
                      " Mean elapsed time per time step in seconds = %.15g\n", tcpu, hh, mm, ss, tcpu / it);
        std::printf("%s\n", lines);
        char name[64];
        std::snprintf(name, sizeof name, "/timestamp%06d", it);
        FILE* ts = std::fopen((dir + name).c_str(), "w");
        if (ts) {
          std::fprintf(ts, " Time step # %d\n Time: %g seconds\n Max norm velocity vector V (m/s) = %.15g\n"
                           " Total energy = %.15g\n%s", it, (float)((it - 1) * p.deltat), vmax,
                       ek[it - 1] + ep[it - 1], lines);
          std::fclose(ts);
        }
      }
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
  write_gnuplot(dir, three_d, mode == "2dpml", S.nrec);
  cpml_destroy(h);
  std::printf("\n End of the simulation\n\n");
  return 0;
}
