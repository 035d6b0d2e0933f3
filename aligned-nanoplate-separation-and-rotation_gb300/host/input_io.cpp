// input_io.cpp -- bcp.input parser and the .res / .bin formats of the
// reference (code/read_input.cpp:7-242, code/io_utils.cpp:138-240,375-397).
//
// bcp.input is positional: each value group sits at the start of its line and
// the rest of the line is a comment; sections are separated by a blank line
// and a header line.  The parser reads the groups in the reference's order.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "driver.h"

namespace scftrun {

namespace {

struct Reader {
  FILE *f;
  char line[512];
  bool ok = true;
  // skips the rest of the current line
  void rest() {
    if (!fgets(line, sizeof line, f)) ok = false;
  }
  void skip_lines(int n) {
    for (int i = 0; i < n; i++) rest();
  }
  template <class... T> void scan(const char *fmt, T *...p) {
    const int want = (int)sizeof...(T);
    if (fscanf(f, fmt, p...) != want) ok = false;
    rest();
  }
};

}  // namespace

std::string read_input(const std::string &path, Input &in) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return "failed to open " + path;
  Reader r{f};
  r.skip_lines(1);  // # Main parameters
  r.scan("%d %d", &in.Nda, &in.Ndb);
  r.scan("%lf %d", &in.phiH, &in.Nah);
  r.scan("%lf", &in.a_smear);
  r.scan("%lf", &in.rho0);
  r.skip_lines(2);
  r.scan("%lf", &in.chi_ab);
  r.scan("%lf", &in.chi_bc);
  r.scan("%lf", &in.chi_ac);
  r.scan("%lf", &in.kappa);
  r.skip_lines(2);
  r.scan("%d %lf %lf %lf", &in.ic_flag[0], &in.ic_pre[0], &in.ic_dir[0], &in.ic_period[0]);
  r.scan("%d %lf %lf %lf", &in.ic_flag[1], &in.ic_pre[1], &in.ic_dir[1], &in.ic_period[1]);
  r.skip_lines(2);
  r.scan("%d %d %d", &in.Nx[0], &in.Nx[1], &in.Nx[2]);
  r.scan("%lf %lf %lf", &in.L[0], &in.L[1], &in.L[2]);
  r.scan("%lf", &in.lam_pl);
  r.scan("%lf", &in.lam_mi);
  r.scan("%d", &in.itermax);
  r.scan("%d", &in.print_freq);
  r.scan("%d %d", &in.sample_freq, &in.sample_wait);
  r.scan("%le", &in.error_tol);
  r.scan("%d", &in.update_scheme);
  r.scan("%d", &in.do_CL);
  r.skip_lines(2);
  r.scan("%d", &in.do_film);
  r.scan("%lf %lf", &in.wallT, &in.wallXi);
  r.scan("%lf %lf", &in.lamA_top, &in.lamB_top);
  r.scan("%lf %lf", &in.lamA_bot, &in.lamB_bot);
  r.skip_lines(2);
  r.scan("%d %d %d", &in.do_channel, &in.hor_dir, &in.vert_dir);
  r.scan("%lf %lf %lf", &in.wall_width, &in.channel_width, &in.channel_xi);
  r.skip_lines(2);
  r.scan("%d", &in.n_exp_nr);
  r.scan("%d", &in.do_fld_np);
  r.scan("%d", &in.np_type);
  r.scan("%d", &in.np_chem);
  r.scan("%lf", &in.sigma);
  r.scan("%d", &in.Ng);
  r.scan("%d", &in.Nu);
  r.scan("%lf", &in.np_frac);
  r.scan("%lf %lf %lf", &in.L_nr, &in.R_nr, &in.xi_nr);
  for (int j = 0; j < 2; j++) {
    r.scan("%lf %lf %lf", &in.center[j][0], &in.center[j][1], &in.center[j][2]);
    r.scan("%lf %lf %lf", &in.orient[j][0], &in.orient[j][1], &in.orient[j][2]);
  }
  fclose(f);
  if (!r.ok) return path + ": truncated or malformed";
  // the reference's own rejections and what this library does not cover
  if (in.phiH > 0) return "No homopolymer allowed unless it's a diblock homopolymer (code/read_input.cpp:40-45)";
  if (in.do_fld_np) return "No field-based nanoparticles (code/read_input.cpp:184-189)";
  if (in.do_film && in.do_channel) return "Can't do film and channel in same simulation";
  if (in.do_film || in.do_channel) return "films and channels are not built here";
  if (in.n_exp_nr > 0 && in.np_type != 2) return "explicit particles must be nanorods/plates (np_type = 2)";
  for (int j = 0; j < in.n_exp_nr; j++)
    for (int d = 0; d < 3; d++)
      if (in.center[j][d] < 0.0 || in.center[j][d] > 1.0)
        return "Nanorod center isn't valid. Must be between 0 and 1";
  for (int d = 0; d < 3; d++)
    if (in.Nx[d] < 1 || !(in.L[d] > 0.0)) return "grid sizes and box lengths must be positive";
  if (in.Ng == 0) in.sigma = 0;  // code/read_input.cpp:200
  if (in.print_freq < 1) return "print_freq must be >= 1";
  return "";
}

scft_params to_params(const Input &in, int precision) {
  scft_params p;
  memset(&p, 0, sizeof p);
  p.Nda = in.Nda;
  p.Ndb = in.Ndb;
  p.a_smear = in.a_smear;
  p.rho0 = in.rho0;
  p.chi_ab = in.chi_ab;
  p.chi_bc = in.chi_bc;
  p.chi_ac = in.chi_ac;
  p.kappa = in.kappa;
  for (int d = 0; d < 3; d++) {
    p.Nx[d] = in.Nx[d];
    p.L[d] = in.L[d];
  }
  p.lam_pl = in.lam_pl;
  p.lam_mi = in.lam_mi;
  p.n_exp_nr = in.n_exp_nr;
  p.np_chem = in.np_chem;
  p.sigma = in.sigma;
  p.Ng = in.Ng;
  p.L_nr = in.L_nr;
  p.R_nr = in.R_nr;
  p.xi_nr = in.xi_nr;
  for (int j = 0; j < 2; j++)
    for (int d = 0; d < 3; d++) {
      p.center[j][d] = in.center[j][d];
      p.orient[j][d] = in.orient[j][d];
    }
  p.precision = precision;
  // code/simulate.cpp:86-89: update_scheme 0 runs update_Euler, anything else update_1s
  p.update_scheme = in.update_scheme == 0 ? SCFT_UPDATE_EULER : SCFT_UPDATE_1S;
  p.do_cl = in.do_CL != 0;
  p.cl_seed = 1;  // the driver sets the run's seed
  p.plate_shape = SCFT_PLATE_REFERENCE;
  return p;
}

bool read_res(const std::string &path, long M, std::vector<cd> &w, std::string &err) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return false;
  w.assign(M, cd(0.0, 0.0));
  for (long i = 0; i < M; i++) {
    double x, y, z, re, im;
    if (fscanf(f, "%lf %lf %lf %lf %lf", &x, &y, &z, &re, &im) != 5) {
      err = path + ": fewer than Nx*Ny*Nz lines";
      fclose(f);
      return false;
    }
    w[i] = cd(re, im);
  }
  fclose(f);
  return true;
}

bool write_bin(const std::string &path, const int Nx[3], const double L[3], const cd *a, long M) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const int dim = 3, nprocs = 1, ml = (int)M;
  bool ok = fwrite(&dim, sizeof(int), 1, f) == 1;
  ok = ok && fwrite(Nx, sizeof(int), 3, f) == 3;
  ok = ok && fwrite(L, sizeof(double), 3, f) == 3;
  ok = ok && fwrite(&nprocs, sizeof(int), 1, f) == 1;
  ok = ok && fwrite(&ml, sizeof(int), 1, f) == 1;
  ok = ok && fwrite(a, sizeof(cd), M, f) == (size_t)M;
  fclose(f);
  return ok;
}

}  // namespace scftrun
