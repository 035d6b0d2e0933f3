// refrng.h -- the reference's random stream, for complex-Langevin noise that
// is bit-identical to a reference run with the same seed.
//
// The reference draws uniform deviates from L'Ecuyer's combined generator
// with a Bays-Durham shuffle (the published "ran2" of Numerical Recipes,
// code/ran2.cpp:32-67, seeded by a negative idum) and Gaussian deviates with
// the polar Box-Muller method that returns the second deviate of each pair on
// the next call (code/ran2.cpp:69-90).  This is a restatement of those two
// published algorithms with their published constants; the state lives in
// one object per instance instead of function statics.
#pragma once

#include <cmath>
#include <cstdint>

namespace scft {

class RefRng {
 public:
  explicit RefRng(int64_t seed = 1) { reseed(seed); }
  // the reference's `idum = -seed` before the first draw
  void reseed(int64_t seed) {
    idum_ = -(seed < 0 ? -seed : seed);
    idum2_ = 123456789;
    iy_ = 0;
    for (auto &v : iv_) v = 0;
    have_ = false;
    spare_ = 0.0;
  }

  double uniform() {
    constexpr int64_t m1 = 2147483563, m2 = 2147483399, a1 = 40014, a2 = 40692, q1 = 53668, q2 = 52774,
                      r1 = 12211, r2 = 3791, ntab = 32, mm1 = m1 - 1, ndiv = 1 + mm1 / ntab;
    constexpr double am = 1.0 / m1, rnmx = 1.0 - 1.2e-7;
    if (idum_ <= 0) {
      idum_ = (-idum_ < 1) ? 1 : -idum_;
      idum2_ = idum_;
      for (int j = ntab + 7; j >= 0; j--) {
        const int64_t k = idum_ / q1;
        idum_ = a1 * (idum_ - k * q1) - k * r1;
        if (idum_ < 0) idum_ += m1;
        if (j < ntab) iv_[j] = idum_;
      }
      iy_ = iv_[0];
    }
    int64_t k = idum_ / q1;
    idum_ = a1 * (idum_ - k * q1) - k * r1;
    if (idum_ < 0) idum_ += m1;
    k = idum2_ / q2;
    idum2_ = a2 * (idum2_ - k * q2) - k * r2;
    if (idum2_ < 0) idum2_ += m2;
    const int64_t j = iy_ / ndiv;
    iy_ = iv_[j] - idum2_;
    iv_[j] = idum_;
    if (iy_ < 1) iy_ += mm1;
    const double t = am * (double)iy_;
    return t > rnmx ? rnmx : t;
  }

  double gauss() {
    if (have_) {
      have_ = false;
      return spare_;
    }
    double v1, v2, rsq;
    do {
      v1 = 2.0 * uniform() - 1.0;
      v2 = 2.0 * uniform() - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = std::sqrt(-2.0 * std::log(rsq) / rsq);
    spare_ = v1 * fac;
    have_ = true;
    return v2 * fac;
  }

 private:
  int64_t idum_, idum2_, iy_, iv_[32];
  bool have_;
  double spare_;
};

}  // namespace scft
