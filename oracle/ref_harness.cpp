/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE: a replacement main() that drives the
 * reference SCFT code's own functions (compiled from its sources with Dim=3
 * and the oracle FFT shim, see oracle/Makefile) and dumps its state at full
 * precision, because the reference itself prints H with only six decimals
 * (code/simulate.cpp:132-135).
 *
 * The call sequence mirrors the reference driver:
 *   code/main.cpp:7-22      read_input(); initialize_1(); allocate();
 *   code/simulate.cpp:30-36 initialize_1(); initialize_2(); calc_poly_density();
 *   code/simulate.cpp:74    Ho = calc_H();
 *   code/simulate.cpp:85-99 loop { update_1s(); calc_H(); }
 * calc_H() is called after every update here; it has no side effects on the
 * fields (it writes only tmp, tmp2 and Hcur).
 *
 * Usage (run inside a directory holding bcp.input and optional w*.res):
 *   scft_ref dump  <iters> [hist]   writes scalars.txt, trace.txt, *.f64
 *   scft_ref time  <iters>          prints "seconds_per_iter <t>"
 *   scft_ref homopoly <Nh> <nK>     homopolymer_discrete(smwa, q, Nh) and
 *                                   integrate_homopoly_discrete(q, Q, nK, rho,
 *                                   smwa, Nh) on the smeared w_A after set-up
 *                                   (code/homopolymer_discrete.cpp:3-55,
 *                                   code/calc_poly_density.cpp:193-212; dead
 *                                   in the shipped inputs, read_input.cpp:40-45):
 *                                   writes homo_W.f64, homo_rho.f64, homo.txt
 *   scft_ref simulate 0             the reference's own main(): read_input,
 *                                   initialize_1, allocate, simulate
 *                                   (writes data.dat and *.p0.bin)
 * Arrays are written as raw little-endian complex<double> (2*ML doubles).
 */
#include <chrono>
#include <csignal>
#include <unistd.h>

#define MAIN
#include "main.hpp"

void update_1s(void);
double simulate(void);
complex<double> homopolymer_discrete(complex<double> *, complex<double> **, int);
void integrate_homopoly_discrete(complex<double> **, complex<double>, complex<double>, complex<double> *,
                                 complex<double> *, int);

// simulate() has no return statement (code/simulate.cpp:16-167).  Built at
// -O0 (oracle/Makefile), GCC ends it with a trap instruction, which runs only
// after the loop has finished and data.dat is closed: that trap is the end of
// a completed run.
static void simulate_fell_off_end(int) { _exit(0); }

static void dump(const char *name, const complex<double> *a) {
  char fn[256];
  snprintf(fn, sizeof fn, "%s.f64", name);
  FILE *f = fopen(fn, "wb");
  if (!f) { perror(fn); exit(2); }
  fwrite(a, sizeof(complex<double>), ML, f);
  fclose(f);
}

static void dump_hist(const char *name, complex<double> **q, int n) {
  char fn[256];
  snprintf(fn, sizeof fn, "%s.f64", name);
  FILE *f = fopen(fn, "wb");
  if (!f) { perror(fn); exit(2); }
  for (int s = 0; s < n; s++) fwrite(q[s], sizeof(complex<double>), ML, f);
  fclose(f);
}

static void setup() {
  myrank = 0;
  nprocs = 1;
  idum = -12345;
  read_input();
  initialize_1();
  allocate();
  initialize_1();
  initialize_2();
  calc_poly_density();
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s dump|time <iters> [hist]\n", argv[0]);
    return 2;
  }
  const int iters = atoi(argv[2]);
  if (!strcmp(argv[1], "simulate")) {
    signal(SIGILL, simulate_fell_off_end);
    myrank = 0;
    nprocs = 1;
    idum = -12345;
    read_input();
    initialize_1();
    allocate();
    simulate();
    return 0;
  }
  if (!strcmp(argv[1], "homopoly")) {
    if (argc < 4) return 2;
    const int Nh = atoi(argv[2]);
    const double nK = atof(argv[3]);
    setup();
    complex<double> **qh = new complex<double> *[Nh];
    for (int s = 0; s < Nh; s++) qh[s] = new complex<double>[ML];
    complex<double> *rh = new complex<double>[ML];
    const complex<double> Qh = homopolymer_discrete(smwa, qh, Nh);
    integrate_homopoly_discrete(qh, Qh, complex<double>(nK, 0.0), rh, smwa, Nh);
    dump("homo_W", smwa);
    dump("homo_rho", rh);
    FILE *f = fopen("homo.txt", "w");
    fprintf(f, "Q_re %.17g\nQ_im %.17g\n", real(Qh), imag(Qh));
    fclose(f);
    return 0;
  }
  if (!strcmp(argv[1], "time")) {
    setup();
    calc_H();
    auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; it < iters; it++) update_1s();
    auto t1 = std::chrono::steady_clock::now();
    complex<double> H = calc_H();
    double s = std::chrono::duration<double>(t1 - t0).count();
    printf("seconds_per_iter %.6f\nH %.17g\n", s / (iters > 0 ? iters : 1), real(H));
    return 0;
  }
  if (strcmp(argv[1], "dump")) return 2;
  const int want_hist = argc > 3 && !strcmp(argv[3], "hist");

  setup();
  FILE *sc = fopen("scalars.txt", "w");
  fprintf(sc, "M %d\nV %.17g\nVf %.17g\nnD %.17g\nphiD %.17g\nnp_frac %.17g\n", M, V, Vf, nD, phiD,
          np_frac);
  fprintf(sc, "nP %.17g\nng_per_np %.17g\nphiG %.17g\nrho0 %.17g\nN %d\nNda %d\nNg %d\n", nP,
          ng_per_np, phiG, rho0, N, Nda, Ng);
  fprintf(sc, "Qd_re %.17g\nQd_im %.17g\nQga_re %.17g\nQga_im %.17g\n", real(Qd), imag(Qd),
          real(Qga_exp), imag(Qga_exp));

  dump("hhat", hhat);
  dump("poly_bond_fft", poly_bond_fft);
  dump("gaa", gaa);
  dump("gab", gab);
  dump("gbb", gbb);
  if (sigma > 0) dump("gc", gc);
  dump("rho_exp_nr", rho_exp_nr);
  dump("exp_nrH", exp_nrH);
  dump("expl_grafts", expl_grafts);
  dump("smwa0", smwa);
  dump("smwb0", smwb);
  dump("smwg0", smwg);
  dump("rhoda0", rhoda);
  dump("rhodb0", rhodb);
  if (sigma > 0 && n_exp_nr > 0) dump("rhog_exp0", rhog_exp);
  if (want_hist) {
    dump_hist("qd0", qd, N);
    dump_hist("qddag0", qddag, N);
    if (sigma > 0 && n_exp_nr > 0) {
      dump_hist("qg0", qg, Ng);
      dump_hist("qgdag0", qgdag_exp, Ng);
    }
  }

  complex<double> H = calc_H();
  fprintf(sc, "H0_re %.17g\nH0_im %.17g\n", real(H), imag(H));
  fclose(sc);

  FILE *tr = fopen("trace.txt", "w");
  fprintf(tr, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", 0, real(H), imag(H), real(Qd), imag(Qd),
          real(Qga_exp), imag(Qga_exp));
  for (int it = 1; it <= iters; it++) {
    update_1s();
    H = calc_H();
    fprintf(tr, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", it, real(H), imag(H), real(Qd),
            imag(Qd), real(Qga_exp), imag(Qga_exp));
  }
  fclose(tr);

  dump("wpl", wpl);
  dump("wabp", wabp);
  dump("wabm", wabm);
  dump("wbcp", wbcp);
  dump("wbcm", wbcm);
  dump("wacp", wacp);
  dump("wacm", wacm);
  dump("smwa", smwa);
  dump("smwb", smwb);
  dump("rhoda", rhoda);
  dump("rhodb", rhodb);
  if (sigma > 0 && n_exp_nr > 0) dump("rhog_exp", rhog_exp);
  return 0;
}
