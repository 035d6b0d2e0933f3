// driver.h -- host side of scft_run: the reference driver's input, output and
// loop surface (read_input / initialize / simulate) on top of libscft.
#pragma once

#include <complex>
#include <string>
#include <vector>

#include "scft.h"

namespace scftrun {

// Everything bcp.input holds (code/read_input.cpp:30-236).
struct Input {
  int Nda = 0, Ndb = 0;
  double phiH = 0.0;
  int Nah = 0;
  double a_smear = 0.0, rho0 = 0.0;
  double chi_ab = 0.0, chi_bc = 0.0, chi_ac = 0.0;  // signed, as read
  double kappa = 0.0;
  int ic_flag[2] = {0, 0};
  double ic_pre[2] = {0, 0}, ic_dir[2] = {0, 0}, ic_period[2] = {0, 0};
  int Nx[3] = {0, 0, 0};
  double L[3] = {0, 0, 0};
  double lam_pl = 0.0, lam_mi = 0.0;
  int itermax = 0, print_freq = 1, sample_freq = 0, sample_wait = 0;
  double error_tol = 0.0;
  int update_scheme = 1, do_CL = 0;
  int do_film = 0;
  double wallT = 0, wallXi = 0, lamA_top = 0, lamB_top = 0, lamA_bot = 0, lamB_bot = 0;
  int do_channel = 0, hor_dir = 0, vert_dir = 0;
  double wall_width = 0, channel_width = 0, channel_xi = 0;
  int n_exp_nr = 0, do_fld_np = 0, np_type = 0, np_chem = 0;
  double sigma = 0.0;
  int Ng = 0, Nu = 0;
  double np_frac = 0.0, L_nr = 0.0, R_nr = 0.0, xi_nr = 0.0;
  double center[2][3] = {}, orient[2][3] = {};
};

// Parses `path`; returns an empty string on success, else the reason
// (the reference prints it and exits, code/read_input.cpp:12-19,40-45,184-189).
std::string read_input(const std::string &path, Input &in);

// Input -> libscft parameters (precision chosen by the caller).
scft_params to_params(const Input &in, int precision);

typedef std::complex<double> cd;

// Reads one resume file (code/io_utils.cpp:138-177, Dim = 3: x y z re im per
// line, stack order).  Returns false if the file does not exist.
bool read_res(const std::string &path, long M, std::vector<cd> &w, std::string &err);

// write_data_bin (code/io_utils.cpp:375-397): header int Dim, int Nx[3],
// double L[3], int nprocs, then int ML and ML complex values.
bool write_bin(const std::string &path, const int Nx[3], const double L[3], const cd *a, long M);

}  // namespace scftrun
