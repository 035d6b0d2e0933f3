/*
 * fftw_shim.cpp -- project-written mixed-radix FP64 FFT behind the FFTW 3
 * API subset declared in fftw3.h.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the reference SCFT sources be compiled
 * into the CPU oracle (oracle/_ref/).  The reference pins nothing at the FFT
 * boundary (it links FFTW 3.3.4, README.md:16-19, not vendored), so this
 * transform is itself pinned by known-answer tests against a direct DFT
 * (tests/test_oracle_fft.py).
 *
 * Algorithm: Stockham autosort, decimation in time, mixed radix 4/2/3/5 and
 * direct DFTs for any other prime factor.  Each stage with radix R turns
 * sub-transforms of length Ns into length Ns*R:
 *     v[r]  = src[j + r*n/R] * w^(r*k*n/(Ns*R)),   k = j mod Ns
 *     v     = DFT_R(v)
 *     dst[(j/Ns)*Ns*R + k + r*Ns] = v[r]
 * Twiddles w^t = exp(sign*2*pi*i*t/n) are tabulated once per length in long
 * double.  Multi-dimensional transforms apply the 1-D transform along every
 * axis (row-major, last axis fastest), gathering strided lines in blocks.
 */
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef std::complex<double> cd;

namespace {

struct Line1D {
  int n = 1;
  std::vector<int> radix;
  std::vector<cd> tw;  // tw[t] = exp(-2*pi*i*t/n)
};

void make_line(Line1D &p, int n) {
  p.n = n;
  p.radix.clear();
  int m = n;
  while (m % 4 == 0) { p.radix.push_back(4); m /= 4; }
  while (m % 2 == 0) { p.radix.push_back(2); m /= 2; }
  while (m % 3 == 0) { p.radix.push_back(3); m /= 3; }
  while (m % 5 == 0) { p.radix.push_back(5); m /= 5; }
  for (int f = 7; m > 1; f += 2)
    while (m % f == 0) { p.radix.push_back(f); m /= f; }
  p.tw.resize(n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int t = 0; t < n; t++) {
    long double a = two_pi * (long double)t / (long double)n;
    p.tw[t] = cd((double)cosl(a), (double)-sinl(a));
  }
}

inline cd twiddle(const Line1D &p, long t, int sign) {
  cd w = p.tw[t % p.n];
  return sign < 0 ? w : std::conj(w);
}

// In-place small DFT of length R with exponent sign `sign`.
void small_dft(cd *v, int R, int sign, const Line1D &p) {
  if (R == 2) {
    cd a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if (R == 4) {
    cd a0 = v[0] + v[2], a1 = v[0] - v[2];
    cd b0 = v[1] + v[3], b1 = v[1] - v[3];
    // multiply b1 by exp(sign*i*pi/2) = sign*i
    cd jb1 = sign < 0 ? cd(b1.imag(), -b1.real()) : cd(-b1.imag(), b1.real());
    v[0] = a0 + b0;
    v[2] = a0 - b0;
    v[1] = a1 + jb1;
    v[3] = a1 - jb1;
  } else if (R == 3) {
    const double c = -0.5;
    const double s = (sign < 0 ? -1.0 : 1.0) * 0.86602540378443864676372317075294;
    cd t1 = v[1] + v[2];
    cd t2 = v[0] + c * t1;
    cd t3 = s * (v[1] - v[2]);
    cd jt3(-t3.imag(), t3.real());
    v[0] = v[0] + t1;
    v[1] = t2 + jt3;
    v[2] = t2 - jt3;
  } else {
    // direct DFT; exponents taken from the length-n table (R divides n)
    cd out[64];
    std::vector<cd> big;
    cd *o = out;
    if (R > 64) { big.resize(R); o = big.data(); }
    const long step = p.n / R;
    for (int m = 0; m < R; m++) {
      cd s = 0.0;
      for (int r = 0; r < R; r++) s += v[r] * twiddle(p, (long)r * m % R * step, sign);
      o[m] = s;
    }
    for (int m = 0; m < R; m++) v[m] = o[m];
  }
}

// Transforms one contiguous line x (length p.n) in place using work buffer w.
void fft_line(const Line1D &p, cd *x, cd *w, int sign) {
  const int n = p.n;
  if (n == 1) return;
  cd *src = x, *dst = w;
  long Ns = 1;
  std::vector<cd> vbuf;
  for (size_t s = 0; s < p.radix.size(); s++) {
    const int R = p.radix[s];
    const int nR = n / R;
    const long tstep = n / (Ns * R);
    cd vs[64];
    cd *v = vs;
    if (R > 64) { vbuf.resize(R); v = vbuf.data(); }
    for (int j = 0; j < nR; j++) {
      const long k = j % Ns;
      v[0] = src[j];
      for (int r = 1; r < R; r++) v[r] = src[j + r * nR] * twiddle(p, r * k * tstep, sign);
      small_dft(v, R, sign, p);
      const long idxD = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; r++) dst[idxD + r * Ns] = v[r];
    }
    cd *t = src; src = dst; dst = t;
    Ns *= R;
  }
  if (src != x) std::memcpy(x, src, sizeof(cd) * n);
}

}  // namespace

struct oracle_fft_plan_s {
  int rank;
  std::vector<int> n;
  long total;
  int sign;
  fftw_complex *in, *out;
  std::vector<Line1D> lines;
};

extern "C" {

void *fftw_malloc(size_t n) { return calloc(n ? n : 1, 1); }

void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_dft(int rank, const int *n, fftw_complex *in, fftw_complex *out, int sign,
                        unsigned flags) {
  (void)flags;
  oracle_fft_plan_s *p = new oracle_fft_plan_s;
  p->rank = rank;
  p->n.assign(n, n + rank);
  p->total = 1;
  for (int d = 0; d < rank; d++) p->total *= n[d];
  p->sign = sign;
  p->in = in;
  p->out = out;
  p->lines.resize(rank);
  for (int d = 0; d < rank; d++) make_line(p->lines[d], n[d]);
  return p;
}

void fftw_execute(const fftw_plan p) {
  cd *data = reinterpret_cast<cd *>(p->out);
  if (p->out != p->in) std::memcpy(p->out, p->in, sizeof(fftw_complex) * p->total);
  const int B = 16;  // strided lines gathered per block
  std::vector<cd> buf, work;
  long stride = 1;
  for (int d = p->rank - 1; d >= 0; d--) {
    const int nd = p->n[d];
    const Line1D &L = p->lines[d];
    work.resize(nd);
    const long outer = p->total / (stride * nd);
    if (stride == 1) {
      for (long o = 0; o < outer; o++) fft_line(L, data + o * nd, work.data(), p->sign);
    } else {
      buf.resize((size_t)B * nd);
      for (long o = 0; o < outer; o++) {
        cd *base = data + o * stride * nd;
        for (long i0 = 0; i0 < stride; i0 += B) {
          const int nb = (int)((stride - i0) < B ? (stride - i0) : B);
          for (int j = 0; j < nd; j++)
            for (int b = 0; b < nb; b++) buf[(size_t)b * nd + j] = base[(long)j * stride + i0 + b];
          for (int b = 0; b < nb; b++) fft_line(L, buf.data() + (size_t)b * nd, work.data(), p->sign);
          for (int j = 0; j < nd; j++)
            for (int b = 0; b < nb; b++) base[(long)j * stride + i0 + b] = buf[(size_t)b * nd + j];
        }
      }
    }
    stride *= nd;
  }
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

}  // extern "C"
