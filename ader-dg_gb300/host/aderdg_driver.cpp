// aderdg_driver.cpp -- the reference's driver (program ADERDG,
// Euler/main.f90:1-111, Baer-Nunziato/main.f90:1-111,
// Advection-Diffusion/main.f90:1-88) restated in C++ over the C ABI of
// include/aderdg_gpu.h.  It reads the reference's params.ini files
// unchanged (Euler/initialize.f90:21-38, Baer-Nunziato/initialize.f90:21-41,
// Advection-Diffusion/initialize.f90:19-37), projects the initial field,
// runs the initial limiter, and advances `do while (time < tend)` calling one
// C-ABI function per reference phase (--phases) or the fused step (default).
//
//   aderdg_driver euler|bn|ad params.ini [--phases] [--N n] [--max-steps k] [--quiet] [--dump file]
//
// --dump writes the final uh (Fortran layout, raw FP64) and the step count.
//
// An optional extension block after the reference fields sets what the
// reference fixes at compile time or hard-wires (lines `key = value`):
//   N = 4            polynomial degree (reference: Euler/AD N=1, BN N=4)
//   cfl = 0.9        CFL number
//   precision = fp32 FP32-mixed predictor (default fp64)
//   limiter = 0|1    a posteriori subcell limiter
//   ad_flux = fused  advection-diffusion predictor flux (default: viscous only)
//   ic = vortex|rp2d|dmr|cylinder|sine|zero|rp1d
//   icparams = p1 p2 ...  parameters of the initial field (see aderdg_gpu.h)
//   bc_mode = 0|1    Euler: 1 = double Mach reflection boundaries (default when ic = dmr)
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/aderdg_gpu.h"

namespace {

struct Params {
  aderdg_config cfg{};
  int ic = ADERDG_IC_EULER_DMR;
  std::vector<double> icp;
  double tend = 0.0;
  int write_interval = 0;
};

// positional `read(1,*)` of the first value on each line, then the extension block
bool read_params(const char* sys, const char* path, Params& p, std::string& err) {
  std::ifstream f(path);
  if (!f) return err = std::string("cannot open ") + path, false;
  std::vector<double> vals;
  std::vector<std::pair<std::string, std::string>> ext;
  std::string line;
  while (std::getline(f, line)) {
    const size_t eq = line.find('=');
    const size_t bang = line.find('!');
    if (eq != std::string::npos && (bang == std::string::npos || eq < bang)) {
      std::string k = line.substr(0, eq), v = line.substr(eq + 1, bang == std::string::npos ? std::string::npos : bang - eq - 1);
      auto trim = [](std::string s) {
        size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
        return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
      };
      ext.emplace_back(trim(k), trim(v));
      continue;
    }
    std::istringstream is(line);
    double v;
    if (is >> v) vals.push_back(v);
  }
  aderdg_config& c = p.cfg;
  std::memset(&c, 0, sizeof(c));
  c.cfl = 0.9;
  c.limiter = 1;
  c.gamma = 1.4;
  c.gamma_s = c.gamma_g = 1.4;
  size_t k = 0;
  auto next = [&](double& out) {
    if (k >= vals.size()) return false;
    out = vals[k++];
    return true;
  };
  double d;
  bool ok = true;
  if (!std::strcmp(sys, "euler")) {
    c.system = ADERDG_SYS_EULER;
    c.N = 1;
    ok &= next(c.gamma);
    ok &= next(d); c.imax = (int)d;
    ok &= next(d); c.jmax = (int)d;
    ok &= next(c.xl[0]) && next(c.xl[1]) && next(c.xr[0]) && next(c.xr[1]);
    for (int s = 0; s < 4; ++s) { ok &= next(d); c.bc[s] = (int)d; }
    ok &= next(d);  // ICType: InitialField is the double Mach reflection for every value
    ok &= next(p.tend);
    ok &= next(d); p.write_interval = (int)d;
    p.ic = ADERDG_IC_EULER_DMR;
    c.bc_mode = 1;
  } else if (!std::strcmp(sys, "bn")) {
    c.system = ADERDG_SYS_BN;
    c.N = 4;
    ok &= next(c.gamma_s) && next(c.gamma_g) && next(c.pi_s) && next(c.pi_g);
    ok &= next(d); c.imax = (int)d;
    ok &= next(d); c.jmax = (int)d;
    ok &= next(c.xl[0]) && next(c.xl[1]) && next(c.xr[0]) && next(c.xr[1]);
    for (int s = 0; s < 4; ++s) { ok &= next(d); c.bc[s] = (int)d; }
    ok &= next(d);
    p.ic = ADERDG_IC_BN_RP1D;
    p.icp = {d, 0.0};
    ok &= next(p.tend);
    ok &= next(d); p.write_interval = (int)d;
  } else if (!std::strcmp(sys, "ad")) {
    c.system = ADERDG_SYS_ADVDIFF;
    c.N = 1;
    c.limiter = 0;
    ok &= next(c.cx) && next(c.cy) && next(c.a);
    ok &= next(d); c.imax = (int)d;
    ok &= next(d); c.jmax = (int)d;
    ok &= next(c.xl[0]) && next(c.xl[1]) && next(c.xr[0]) && next(c.xr[1]);
    ok &= next(p.tend);
    for (int s = 0; s < 4; ++s) { ok &= next(d); c.bc[s] = (int)d; }
    ok &= next(d); p.write_interval = (int)d;
    p.ic = ADERDG_IC_AD_ZERO;
  } else {
    return err = "system must be euler, bn or ad", false;
  }
  if (!ok) return err = "params.ini has too few fields", false;
  for (auto& kv : ext) {
    const std::string& key = kv.first;
    const std::string& v = kv.second;
    if (key == "N") c.N = std::atoi(v.c_str());
    else if (key == "cfl") c.cfl = std::atof(v.c_str());
    else if (key == "precision") c.precision = (v == "fp32") ? ADERDG_FP32_MIXED : ADERDG_FP64;
    else if (key == "limiter") c.limiter = std::atoi(v.c_str());
    else if (key == "ad_flux") c.ad_flux_mode = (v == "fused") ? 1 : 0;
    else if (key == "bc_mode") c.bc_mode = std::atoi(v.c_str());
    else if (key == "icparams") {
      std::istringstream is(v);
      p.icp.clear();
      while (is >> d) p.icp.push_back(d);
    } else if (key == "ic") {
      if (v == "vortex") p.ic = ADERDG_IC_EULER_VORTEX, c.bc_mode = 0;
      else if (v == "rp2d") p.ic = ADERDG_IC_EULER_RP2D, c.bc_mode = 0;
      else if (v == "dmr") p.ic = ADERDG_IC_EULER_DMR, c.bc_mode = 1;
      else if (v == "cylinder") p.ic = ADERDG_IC_BN_CYLINDER;
      else if (v == "rp1d") p.ic = ADERDG_IC_BN_RP1D;
      else if (v == "sine") p.ic = ADERDG_IC_AD_SINE;
      else if (v == "zero") p.ic = ADERDG_IC_AD_ZERO;
      else return err = "unknown ic " + v, false;
    } else {
      return err = "unknown extension key " + key, false;
    }
  }
  if (p.ic == ADERDG_IC_AD_SINE && p.icp.empty()) p.icp = {1.0};
  return true;
}

// Fortran Ew.d edit descriptor: 0.ddd...E+xx right-aligned in w columns
std::string fortran_e(double x, int w, int d) {
  char buf[64];
  if (!std::isfinite(x)) {
    std::snprintf(buf, sizeof(buf), "%*s", w, x != x ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
    return buf;
  }
  std::string s;
  if (x == 0.0) {
    s = "0." + std::string(d, '0') + "E+00";
  } else {
    std::snprintf(buf, sizeof(buf), "%.*E", d - 1, std::fabs(x));  // correctly rounded d significant digits
    std::string m(buf);
    const size_t epos = m.find('E');
    std::string digits = m.substr(0, 1) + (epos > 2 ? m.substr(2, epos - 2) : std::string());
    const int e = std::atoi(m.c_str() + epos + 1) + 1;
    std::snprintf(buf, sizeof(buf), "%s0.%sE%c%02d", x < 0 ? "-" : "", digits.c_str(), e < 0 ? '-' : '+', std::abs(e));
    s = buf;
  }
  if ((int)s.size() < w) s = std::string(w - s.size(), ' ') + s;
  return s;
}

// write_data (Euler/write_data.f90:8-95 and the BN / AD copies): cell-average
// primitive variables on the cell centres, legacy ASCII VTK
bool write_vtk(const std::string& path, const aderdg_config& c, const std::vector<double>& wh, double time) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  const int I = c.imax, J = c.jmax;
  const int V = c.system == ADERDG_SYS_ADVDIFF ? 1 : c.system == ADERDG_SYS_EULER ? 4 : 9;
  const double dx = (c.xr[0] - c.xl[0]) / I, dy = (c.xr[1] - c.xl[1]) / J;
  std::fprintf(f, "# vtk DataFile Version 2.0\n2D Euler\nASCII\nDATASET STRUCTURED_GRID\nFIELD FieldData 1\n");
  std::fprintf(f, "TIME 1 1 double\n%s\n", fortran_e(time, 15, 9).c_str());
  std::fprintf(f, "DIMENSIONS %5d%5d%5d\nPOINTS %10d double\n", I, J, 1, I * J);
  for (int j = 0; j < J; ++j)
    for (int i = 0; i < I; ++i)
      std::fprintf(f, "%s%s%s\n", fortran_e(c.xl[0] + ((double)(i + 1) - 0.5) * dx, 15, 7).c_str(),
                   fortran_e(c.xl[1] + ((double)(j + 1) - 0.5) * dy, 15, 7).c_str(), fortran_e(0.0, 15, 7).c_str());
  std::fprintf(f, "POINT_DATA%10d\n", I * J);
  struct Field { bool vec; const char* name; int a, b; };
  static const Field euler[] = {{false, "Density", 0, 0}, {true, "Velocity", 1, 2}, {false, "Pressure", 3, 0}};
  static const Field bn[] = {{false, "RHO_S", 0, 0}, {true, "V_S", 1, 2}, {false, "P_S", 3, 0}, {false, "RHO_G", 4, 0},
                             {true, "V_G", 5, 6},     {false, "P_G", 7, 0}, {false, "PHI_S", 8, 0}};
  static const Field ad[] = {{false, "U", 0, 0}};
  const Field* fields = c.system == ADERDG_SYS_EULER ? euler : c.system == ADERDG_SYS_BN ? bn : ad;
  const int nf = c.system == ADERDG_SYS_EULER ? 3 : c.system == ADERDG_SYS_BN ? 7 : 1;
  for (int k = 0; k < nf; ++k) {
    if (fields[k].vec) std::fprintf(f, "VECTORS %s double\n", fields[k].name);
    else std::fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", fields[k].name);
    for (long q = 0; q < (long)I * J; ++q) {
      if (fields[k].vec)
        std::fprintf(f, "%s%s%s\n", fortran_e(wh[q * V + fields[k].a], 15, 7).c_str(),
                     fortran_e(wh[q * V + fields[k].b], 15, 7).c_str(), fortran_e(0.0, 15, 7).c_str());
      else
        std::fprintf(f, "%s\n", fortran_e(wh[q * V + fields[k].a], 15, 7).c_str());
    }
  }
  std::fclose(f);
  return true;
}

// plot_troubled_cells (Euler/write_data.f90:101-192): the recompute map on the mesh
bool write_troubled_vtk(const std::string& path, const aderdg_config& c, const std::vector<int>& rec, double time) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  const int I = c.imax, J = c.jmax;
  const long nn = (long)(I + 1) * (J + 1), ne = (long)I * J;
  const double dx = (c.xr[0] - c.xl[0]) / I, dy = (c.xr[1] - c.xl[1]) / J;
  std::fprintf(f, "# vtk DataFile Version 2.0\n2D Euler\nASCII\nDATASET UNSTRUCTURED_GRID\nFIELD FieldData 1\n");
  std::fprintf(f, "TIME 1 1 double\n%s\nPOINTS %10ld double\n", fortran_e(time, 15, 9).c_str(), nn);
  for (int j = 0; j <= J; ++j)
    for (int i = 0; i <= I; ++i)
      std::fprintf(f, "%s%s%s\n", fortran_e(c.xl[0] + i * dx, 15, 7).c_str(), fortran_e(c.xl[1] + j * dy, 15, 7).c_str(),
                   fortran_e(0.0, 15, 7).c_str());
  std::fprintf(f, "CELLS %10ld%10ld\n", ne, ne * 5);
  auto idxn = [&](int i, int j) { return (long)i + (long)(I + 1) * j; };
  for (int j = 0; j < J; ++j)
    for (int i = 0; i < I; ++i)
      std::fprintf(f, "%10d%10ld%10ld%10ld%10ld\n", 4, idxn(i, j), idxn(i + 1, j), idxn(i + 1, j + 1), idxn(i, j + 1));
  std::fprintf(f, "CELL_TYPES %10ld\n", ne);
  for (long q = 0; q < ne; ++q) std::fprintf(f, "%5d\n", 9);
  std::fprintf(f, "CELL_DATA%10ld\nSCALARS TCells double 1\nLOOKUP_TABLE default\n", ne);
  for (long q = 0; q < ne; ++q)
    std::fprintf(f, "%s\n", fortran_e(rec[q] == 1 ? 2.0 : rec[q] == 2 ? 1.0 : 0.0, 15, 7).c_str());
  std::fclose(f);
  return true;
}

int die(aderdg_ctx* ctx, int code, const char* what) {
  std::fprintf(stderr, "%s failed (%d): %s\n", what, code, aderdg_last_error(ctx));
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr,
                 "usage: %s euler|bn|ad params.ini [--phases] [--N n] [--max-steps k] [--quiet] [--dump file]\n"
                 "       [--vtk basename] [--analyze]\n",
                 argv[0]);
    return 2;
  }
  Params p;
  std::string err;
  if (!read_params(argv[1], argv[2], p, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return 2;
  }
  bool phases = false, quiet = false;
  long max_steps = -1;
  const char* dump = nullptr;
  const char* vtk = nullptr;  // write_data every WriteInterval steps: <basename>-<timestep>.vtk
  bool analyze = false;       // analyze_soln at the end
  for (int a = 3; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--phases")) phases = true;
    else if (!std::strcmp(argv[a], "--quiet")) quiet = true;
    else if (!std::strcmp(argv[a], "--N") && a + 1 < argc) p.cfg.N = std::atoi(argv[++a]);
    else if (!std::strcmp(argv[a], "--max-steps") && a + 1 < argc) max_steps = std::atol(argv[++a]);
    else if (!std::strcmp(argv[a], "--dump") && a + 1 < argc) dump = argv[++a];
    else if (!std::strcmp(argv[a], "--vtk") && a + 1 < argc) vtk = argv[++a];
    else if (!std::strcmp(argv[a], "--analyze")) analyze = true;
  }
  const aderdg_config& c = p.cfg;
  const int V = c.system == ADERDG_SYS_ADVDIFF ? 1 : c.system == ADERDG_SYS_EULER ? 4 : 9;
  const long P = c.N + 1, S = 2 * c.N + 1, cells = (long)c.imax * c.jmax;
  std::vector<double> uh(V * P * P * cells), lh(V * S * S * cells);
  std::vector<double> icp(32, 0.0);
  for (size_t k = 0; k < p.icp.size() && k < icp.size(); ++k) icp[k] = p.icp[k];
  int r = aderdg_project_initial_condition(&c, p.ic, icp.data(), uh.data(), lh.data());
  if (r) return die(nullptr, r, "aderdg_project_initial_condition");
  aderdg_ctx* ctx = nullptr;
  r = aderdg_create(&c, &ctx);
  if (r) return die(nullptr, r, "aderdg_create");
  if ((r = aderdg_upload(ctx, uh.data()))) return die(ctx, r, "aderdg_upload");
  int nlim = 0;
  if ((r = aderdg_init_limiter(ctx, lh.data(), &nlim))) return die(ctx, r, "aderdg_init_limiter");
  double time = 0.0, dt = 0.0;
  int nrec = 0;
  long steps = 0;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<double> wh(vtk ? (size_t)V * cells : 0);
  auto write_out = [&](long timestep) -> int {
    if (!vtk) return 0;
    int rr = aderdg_cell_averages(ctx, 1, wh.data());
    if (rr) return rr;
    char name[64];
    std::snprintf(name, sizeof(name), "-%08ld.vtk", timestep);
    if (!write_vtk(std::string(vtk) + name, c, wh, time)) return ADERDG_EINVAL;
    if (c.limiter && c.system != ADERDG_SYS_ADVDIFF) {
      std::vector<int> rec((size_t)cells);
      rr = aderdg_get_array(ctx, ADERDG_A_RECOMPUTE, rec.data());
      if (rr) return rr;
      const std::string base(vtk);
      const size_t slash = base.find_last_of('/');
      const std::string dir = slash == std::string::npos ? std::string() : base.substr(0, slash + 1);
      std::snprintf(name, sizeof(name), "Tcells-%08ld.vtk", timestep);
      if (!write_troubled_vtk(dir + name, c, rec, time)) return ADERDG_EINVAL;
    }
    return 0;
  };
  while (time < p.tend && (max_steps < 0 || steps < max_steps)) {
    // Euler/main.f90:25-28: write_data every WriteInterval steps
    if (vtk && p.write_interval > 0 && steps % p.write_interval == 0)
      if ((r = write_out(steps))) return die(ctx, r, "write_data");
    if (phases) {
      // the loop body of Euler/main.f90:24-100, one call per phase
      if ((r = aderdg_calc_time_step(ctx, time, p.tend, &dt))) return die(ctx, r, "calc_time_step");
      if (!quiet) std::printf(" nRecomp = %d t = %.15g dt = %.15g\n", nrec, time, dt);
      if ((r = aderdg_limiter_prepare(ctx))) return die(ctx, r, "limiter_prepare");
      if ((r = aderdg_space_time_predictor(ctx))) return die(ctx, r, "space_time_predictor");
      if ((r = aderdg_volume_integral(ctx))) return die(ctx, r, "volume_integral");
      if ((r = aderdg_riemann_problem(ctx))) return die(ctx, r, "riemann_problem");
      if ((r = aderdg_surface_integral(ctx))) return die(ctx, r, "surface_integral");
      if ((r = aderdg_element_update(ctx, &nrec))) return die(ctx, r, "element_update");
      if ((r = aderdg_limiter(ctx))) return die(ctx, r, "limiter");
      time = time + dt;
    } else {
      const double t_before = time;
      if ((r = aderdg_step(ctx, &time, p.tend, &dt, &nrec))) return die(ctx, r, "aderdg_step");
      if (!quiet) std::printf(" nRecomp = %d t = %.15g dt = %.15g\n", nrec, t_before, dt);
    }
    ++steps;
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf(" nRecomp = %d t = %.15g dt = %.15g\n", nrec, time, dt);
  std::printf(" steps = %ld  initially limited = %d  wall time = %.6f s  DOF-updates/s = %.4e\n", steps, nlim, secs,
              (double)V * P * P * cells * steps / (secs > 0 ? secs : 1));
  if (vtk && (r = write_out(steps))) return die(ctx, r, "write_data");
  if (analyze) {
    // analyze_soln (Euler/analyze_soln.f90:10-56): max over cells of the cell-average error of variable 1
    double norms[3];
    if ((r = aderdg_error_norms(ctx, p.ic, icp.data(), 0, norms))) return die(ctx, r, "aderdg_error_norms");
    std::printf(" %.15g\n", norms[2]);
  }
  if ((r = aderdg_download(ctx, uh.data(), nullptr))) return die(ctx, r, "aderdg_download");
  if (dump) {
    FILE* f = std::fopen(dump, "wb");
    if (!f) return std::fprintf(stderr, "cannot write %s\n", dump), 1;
    std::fwrite(&steps, sizeof(long), 1, f);
    std::fwrite(&time, sizeof(double), 1, f);
    std::fwrite(uh.data(), sizeof(double), uh.size(), f);
    std::fclose(f);
  }
  aderdg_destroy(ctx);
  return 0;
}
