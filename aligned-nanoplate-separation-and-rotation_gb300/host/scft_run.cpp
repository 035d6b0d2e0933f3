// scft_run.cpp -- drop-in driver for the reference executable: reads bcp.input
// and w*.res in each run directory, runs the 1S iteration on the GPU through
// libscft and writes data.dat and the *.p0.bin outputs in the reference's
// formats (code/main.cpp:7-64, code/simulate.cpp:16-167, code/io_utils.cpp:11-104).
//
//   scft_run [--mixed] [--quiet] [dir ...]      (default: the current directory)
//
// All directories form one batch: one context, every kernel launch covers all
// of them.  Each run keeps its own convergence state; once a run meets the
// reference's stop rule its outputs are final (later iterations of the batch
// do not touch its files).
#include <cmath>
#include <complex>
#include <cstdio>
#include <ctime>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "driver.h"

using namespace scftrun;

namespace {

const double kPI = 3.14159265358979323846263383;  // code/globals.h:31
const char *kFieldNames[7] = {"wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm"};

struct Run {
  std::string dir;
  Input in;
  long M = 0;
  double V = 0.0;
  std::complex<double> Ho{0.0, 0.0}, Hcur{0.0, 0.0};
  double error = 0.0;
  int close_to_tol = 0;
  bool done = false;
  FILE *dat = nullptr;
  // complex-Langevin averages (code/array_utils.cpp:13-45)
  std::vector<std::complex<double>> avg_a, avg_b, avg_g;
  double n_samples = 0.0;
  // resume fields read (and checked) before the GPU is touched; empty: absent
  std::vector<std::complex<double>> res[7];
};

int check(int st, const char *what) {
  if (st != SCFT_OK) {
    fprintf(stderr, "%s failed (%d): %s\n", what, st, scft_last_error());
    exit(1);
  }
  return st;
}

// Initial fields (code/initialize.cpp:419-565): the cosine/sine pattern on
// w_AB^-, zero inside walls and plates, or uniform random fields; then the
// resume files override what they provide.
std::vector<std::complex<double>> initial_fields(scft_ctx *ctx, int k, const Run &r) {
  typedef std::complex<double> cd;
  const Input &in = r.in;
  const long M = r.M;
  std::vector<cd> w(7 * M, cd(0.0, 0.0));
  const cd I(0.0, 1.0);
  const int neg_ab = in.chi_ab < 0, neg_bc = in.chi_bc < 0, neg_ac = in.chi_ac < 0;
  if (in.ic_flag[0] < -1) {
    std::vector<double> rho_np(M, 0.0);
    check(scft_get_plate_density(ctx, k, rho_np.data()), "scft_get_plate_density");
    for (long i = 0; i < M; i++) {
      const int n[3] = {(int)(i % in.Nx[0]), (int)((i / in.Nx[0]) % in.Nx[1]),
                        (int)(i / ((long)in.Nx[0] * in.Nx[1]))};
      double x[3];
      for (int d = 0; d < 3; d++) {  // get_r, code/array_utils.cpp:159-179
        x[d] = in.L[d] / in.Nx[d] * double(n[d]);
        if (x[d] > in.L[d] / 2.0) x[d] -= in.L[d];
        else if (x[d] <= -in.L[d] / 2.0) x[d] += in.L[d];
      }
      cd v = 0.0;
      if (!(rho_np[i] > 0.5)) {
        v = 1.0;
        for (int j = 0; j < 2; j++) {
          const int dir = (int)in.ic_dir[j];
          const cd ph = (in.chi_ab != 0 ? (neg_ab ? I : cd(1.0)) : cd(1.0));
          if (in.ic_flag[j] == -2)
            v *= in.ic_pre[j] * std::tanh(std::cos(2.0 * kPI * in.ic_period[j] * x[dir] / in.L[dir]) / 0.2) * ph;
          else if (in.ic_flag[j] == -3)
            v *= in.ic_pre[j] * std::tanh(std::sin(2.0 * kPI * in.ic_period[j] * x[dir] / in.L[dir]) / 0.2) * ph;
          else if (in.ic_flag[j] < -4) {
            fprintf(stderr, "Initial condition flags smaller than -4 not supported\n");
            exit(1);
          }
        }
      }
      w[2 * M + i] = v;
    }
  } else if (in.ic_flag[0] == -1) {
    // the reference draws from ran2 seeded by the clock; a seeded generator here
    std::mt19937_64 gen(12345 + k);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (long i = 0; i < M; i++) {
      const double pre = in.ic_pre[0];
      if (in.chi_ab != 0) {
        w[1 * M + i] = pre * (u(gen) - 0.5) * (neg_ab ? cd(1.0) : I);
        w[2 * M + i] = pre * (u(gen) - 0.5) * (neg_ab ? I : cd(1.0));
      }
      if (in.chi_bc != 0) {
        w[3 * M + i] = pre * (u(gen) - 0.5) * (neg_bc ? cd(1.0) : I);
        w[4 * M + i] = pre * (u(gen) - 0.5) * (neg_bc ? I : cd(1.0));
      }
      if (in.chi_ac != 0) {
        w[5 * M + i] = pre * (u(gen) - 0.5) * (neg_ac ? cd(1.0) : I);
        w[6 * M + i] = pre * (u(gen) - 0.5) * (neg_ac ? I : cd(1.0));
      }
      w[i] = pre * (u(gen) - 0.5) * I;
    }
  }
  for (int f = 0; f < 7; f++)
    if ((long)r.res[f].size() == M) {
      for (long i = 0; i < M; i++) w[f * M + i] = r.res[f][i];
      printf("Read %s.res\n", kFieldNames[f]);
    }
  return w;
}

// write_outputs (code/io_utils.cpp:11-104): smeared and raw densities, fields,
// and with complex Langevin the running averages divided by the sample count
// once iter >= sample_wait (avg_rhog of free grafted particles stays zero).
void write_outputs(scft_ctx *ctx, int k, const Run &r, int iter) {
  typedef std::complex<double> cd;
  const Input &in = r.in;
  const long M = r.M;
  std::vector<cd> ra(M), rb(M), rg(M);
  check(scft_get_density(ctx, k, reinterpret_cast<double *>(ra.data()), reinterpret_cast<double *>(rb.data()),
                         reinterpret_cast<double *>(rg.data())),
        "scft_get_density");
  // hhat from get_k (code/initialize.cpp:97-102)
  std::vector<double> hh(M);
  for (long i = 0; i < M; i++) {
    const int n[3] = {(int)(i % in.Nx[0]), (int)((i / in.Nx[0]) % in.Nx[1]), (int)(i / ((long)in.Nx[0] * in.Nx[1]))};
    double k2 = 0.0;
    for (int d = 0; d < 3; d++) {
      const double kk = (double(n[d]) < double(in.Nx[d]) / 2.) ? 2 * kPI * double(n[d]) / in.L[d]
                                                              : 2 * kPI * double(n[d] - in.Nx[d]) / in.L[d];
      k2 += kk * kk;
    }
    hh[i] = std::exp(-k2 * in.a_smear * in.a_smear / 2.0);
  }
  auto smeared = [&](const std::vector<cd> &a) {
    std::vector<cd> t(a);
    check(scft_fft3d(ctx, k, reinterpret_cast<double *>(t.data()), 1, -1), "scft_fft3d");
    for (long i = 0; i < M; i++) t[i] *= hh[i];
    check(scft_fft3d(ctx, k, reinterpret_cast<double *>(t.data()), 1, +1), "scft_fft3d");
    return t;
  };
  const std::string d = r.dir + "/";
  const bool graft = in.sigma > 0.0;
  std::vector<cd> t = smeared(ra);
  write_bin(d + "rhoda.p0.bin", in.Nx, in.L, t.data(), M);
  write_bin(d + "rhoda_c.p0.bin", in.Nx, in.L, ra.data(), M);
  t = smeared(rb);
  write_bin(d + "rhodb.p0.bin", in.Nx, in.L, t.data(), M);
  write_bin(d + "rhodb_c.p0.bin", in.Nx, in.L, rb.data(), M);
  if (graft) {
    t = smeared(rg);
    write_bin(d + "rhog_exp.p0.bin", in.Nx, in.L, t.data(), M);
    write_bin(d + "rhog_exp_c.p0.bin", in.Nx, in.L, rg.data(), M);
  }
  if (in.do_CL && iter >= in.sample_wait) {
    auto write_avg = [&](const char *name, const std::vector<cd> &acc) {
      std::vector<cd> a(M);
      for (long i = 0; i < M; i++) a[i] = (acc.empty() ? cd(0.0) : acc[i]) / r.n_samples;
      write_bin(d + name + ".p0.bin", in.Nx, in.L, a.data(), M);
    };
    write_avg("avg_rhoda", r.avg_a);
    write_avg("avg_rhodb", r.avg_b);
    write_avg("avg_rhog", std::vector<cd>());
    write_avg("avg_rhog_exp", r.avg_g);
  }
  std::vector<cd> w(7 * M);
  check(scft_get_fields(ctx, k, reinterpret_cast<double *>(w.data())), "scft_get_fields");
  write_bin(d + "wpl.p0.bin", in.Nx, in.L, w.data(), M);
  const double chis[3] = {in.chi_ab, in.chi_ac, in.chi_bc};
  const int idx[3] = {1, 5, 3};
  for (int j = 0; j < 3; j++)
    if (chis[j] != 0) {
      write_bin(d + kFieldNames[idx[j]] + ".p0.bin", in.Nx, in.L, w.data() + idx[j] * M, M);
      write_bin(d + kFieldNames[idx[j] + 1] + ".p0.bin", in.Nx, in.L, w.data() + (idx[j] + 1) * M, M);
    }
}

}  // namespace

int main(int argc, char **argv) {
  int precision = SCFT_PREC_FP64;
  // complex-Langevin seed: the reference seeds ran2 with idum = -time(0)
  // (code/main.cpp:20); --seed S reproduces a run seeded with idum = -S
  long long seed = (long long)time(nullptr);
  bool quiet = false;
  std::vector<std::string> dirs;
  for (int a = 1; a < argc; a++) {
    const std::string s = argv[a];
    if (s == "--mixed") precision = SCFT_PREC_MIXED;
    else if (s == "--quiet") quiet = true;
    else if (s == "--seed" && a + 1 < argc) seed = atoll(argv[++a]);
    else dirs.push_back(s);
  }
  if (dirs.empty()) dirs.push_back(".");
  std::vector<Run> runs(dirs.size());
  std::vector<scft_params> params;
  for (size_t k = 0; k < dirs.size(); k++) {
    runs[k].dir = dirs[k];
    const std::string err = read_input(dirs[k] + "/bcp.input", runs[k].in);
    if (!err.empty()) {
      fprintf(stderr, "%s: %s\n", dirs[k].c_str(), err.c_str());
      return 1;
    }
    params.push_back(to_params(runs[k].in, precision));
    params.back().cl_seed = seed;
    // resume files (code/io_utils.cpp:138-177): read and checked here, before
    // any GPU work, so that a short or malformed file ends the run cleanly
    const long M = (long)runs[k].in.Nx[0] * runs[k].in.Nx[1] * runs[k].in.Nx[2];
    for (int f = 0; f < 7; f++) {
      std::string rerr;
      const std::string path = dirs[k] + "/" + kFieldNames[f] + ".res";
      if (!read_res(path, M, runs[k].res[f], rerr)) {
        runs[k].res[f].clear();
        if (!rerr.empty()) {
          fprintf(stderr, "%s\n", rerr.c_str());
          return 1;
        }
      }
    }
  }
  scft_ctx *ctx = nullptr;
  check(scft_create(params.data(), (int)params.size(), &ctx), "scft_create");
  const int n = (int)runs.size();
  for (int k = 0; k < n; k++) {
    scft_info info;
    check(scft_get_info(ctx, k, &info), "scft_get_info");
    runs[k].M = info.M;
    runs[k].V = info.V;
    std::vector<std::complex<double>> w = initial_fields(ctx, k, runs[k]);
    check(scft_set_fields(ctx, k, reinterpret_cast<double *>(w.data())), "scft_set_fields");
    runs[k].dat = fopen((runs[k].dir + "/data.dat").c_str(), "w");
    if (!runs[k].dat) {
      fprintf(stderr, "Failed to open data.dat!\n");
      return 1;
    }
    if (!quiet)
      printf("%s: V = %lf, N = %d, nD = %lf, np_frac = %lf\n", runs[k].dir.c_str(), info.V, info.N, info.nD,
             info.np_frac);
  }
  std::vector<double> h(5 * n);
  check(scft_calc_poly_density(ctx), "scft_calc_poly_density");
  int st = scft_calc_H(ctx, h.data());
  for (int k = 0; k < n; k++) {
    if (!quiet) printf("%s: Starting H: %lf\n", runs[k].dir.c_str(), h[5 * k]);
    write_outputs(ctx, k, runs[k], 0);
  }
  int itermax = 0;
  for (auto &r : runs) itermax = std::max(itermax, r.in.itermax);
  // main loop (code/simulate.cpp:85-157); `Ho = Hcur` uses the loop's own
  // Hcur, which starts at zero, as in the reference (code/simulate.cpp:17,98)
  for (int iter = 0; iter <= itermax; iter++) {
    bool all_done = true;
    for (auto &r : runs) all_done = all_done && (r.done || iter > r.in.itermax);
    if (all_done) break;
    check(scft_update_1s(ctx, 1), "scft_update_1s");
    // complex-Langevin sampling (code/simulate.cpp:91-92)
    for (int k = 0; k < n; k++) {
      Run &r = runs[k];
      if (r.done || iter > r.in.itermax || !r.in.do_CL || iter < r.in.sample_wait || r.in.sample_freq <= 0 ||
          iter % r.in.sample_freq != 0)
        continue;
      std::vector<std::complex<double>> ra(r.M), rb(r.M), rg(r.M);
      check(scft_get_density(ctx, k, reinterpret_cast<double *>(ra.data()), reinterpret_cast<double *>(rb.data()),
                             reinterpret_cast<double *>(rg.data())),
            "scft_get_density");
      if (r.avg_a.empty()) {
        r.avg_a.assign(r.M, 0.0);
        r.avg_b.assign(r.M, 0.0);
        r.avg_g.assign(r.M, 0.0);
      }
      for (long i = 0; i < r.M; i++) {
        r.avg_a[i] += ra[i];
        r.avg_b[i] += rb[i];
        r.avg_g[i] += rg[i];
      }
      r.n_samples += 1.0;
    }
    bool need_h = false;
    for (auto &r : runs)
      if (!r.done && iter <= r.in.itermax && iter % r.in.print_freq == 0) need_h = true;
    if (need_h) {
      st = scft_calc_H(ctx, h.data());
      if (st == SCFT_ERR_NAN) {
        fprintf(stderr, "Crashed! iteration %d (H is NaN)\n", iter);
        return 1;
      }
      if (st == SCFT_ERR_QNONPOS) {
        fprintf(stderr, "%s\n", scft_last_error());
        return 4;
      }
      check(st, "scft_calc_H");
    }
    for (int k = 0; k < n; k++) {
      Run &r = runs[k];
      if (r.done || iter > r.in.itermax) continue;
      if (iter % r.in.print_freq == 0) {
        const std::complex<double> H(h[5 * k], h[5 * k + 1]), Qd(h[5 * k + 2], h[5 * k + 3]);
        r.Ho = r.Hcur;
        r.Hcur = H;
        r.error = std::abs(H - r.Ho) / r.V / double(r.in.print_freq);
        if (r.error < r.in.error_tol * 10) r.close_to_tol++;
        const std::complex<double> mlq = -std::log(Qd);
        const std::complex<double> mlqh = -std::log(std::complex<double>(1.0, 0.0));
        const std::complex<double> mlqp = -std::log(std::complex<double>(1.0, 0.0)) + 0.0;
        if (!quiet) printf("%s Iter: %d, H=%lf, -log(Qd)=%lf, err=%1.1e\n", r.dir.c_str(), iter, H.real(), mlq.real(),
                           r.error);
        fprintf(r.dat, "%d %5.6lf %1.3e %5.6lf %1.3e %5.6lf %1.3e %5.6lf %1.3e %1.3e\n", iter, H.real(), H.imag(),
                mlq.real(), mlq.imag(), mlqh.real(), mlqh.imag(), mlqp.real(), mlqp.imag(), r.error);
        fflush(r.dat);
        write_outputs(ctx, k, r, iter);
      }
      if (!r.in.do_CL && iter > 25 && r.error < r.in.error_tol && r.close_to_tol > 10) {
        r.done = true;
        if (!quiet) printf("%s: Tolerance reached. Error = %.4e\n", r.dir.c_str(), r.error);
      }
    }
  }
  for (auto &r : runs) fclose(r.dat);
  scft_destroy(ctx);
  return 0;
}
