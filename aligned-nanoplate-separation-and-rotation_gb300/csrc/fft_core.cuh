// fft_core.cuh -- device building blocks for the batched 3-D FFTs of libscft.
//
// A line FFT of length n is a sequence of Stockham stages (decimation in
// time, mixed radix 8/4/2/3/5).  Stage s with radix R turns sub-transforms of
// length Ns into length Ns*R:
//     v[r] = src[j + r*n/R] * w^(r*k*n/(Ns*R)),  k = j mod Ns,  r = 0..R-1
//     v    = DFT_R(v)
//     dst[(j/Ns)*Ns*R + k + r*Ns] = v[r]
// with w = exp(sign*2*pi*i/n).  Stages run in place on shared memory: every
// thread first gathers, twiddles and transforms all butterflies it owns into
// registers, the block synchronises, then every thread scatters its results.
// This halves the shared memory of a ping-pong Stockham and keeps the whole
// xy plane (or z-column tile) resident for the fused pointwise work around it.
#pragma once

#include "common.h"

namespace scft {

template <typename T> struct CxT;
template <> struct CxT<double> { typedef double2 type; };
template <> struct CxT<float> { typedef float2 type; };
template <typename T> using cx = typename CxT<T>::type;

__device__ __forceinline__ double2 mkc(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mkc(float a, float b) { return make_float2(a, b); }

template <class C> __device__ __forceinline__ C cadd(C a, C b) { return mkc(a.x + b.x, a.y + b.y); }
template <class C> __device__ __forceinline__ C csub(C a, C b) { return mkc(a.x - b.x, a.y - b.y); }
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
  return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class C, typename S> __device__ __forceinline__ C cscale(C a, S s) { return mkc(a.x * s, a.y * s); }
// principal square root of a complex FP64 number (the branch of std::sqrt)
__device__ __forceinline__ double2 csqrt_d(double2 z) {
  const double x = z.x, y = z.y;
  if (x == 0.0 && y == 0.0) return make_double2(0.0, y);
  const double r = hypot(x, y);
  if (x >= 0.0) {
    const double t = sqrt(0.5 * (r + x));
    return make_double2(t, y / (2.0 * t));
  }
  const double t = sqrt(0.5 * (r - x));
  return make_double2(fabs(y) / (2.0 * t), copysign(t, y));
}

// a * w (SIGN < 0) or a * conj(w) (SIGN > 0); tables hold exp(-2*pi*i*t/n).
template <int SIGN, class C> __device__ __forceinline__ C ctw(C a, C w) {
  if (SIGN < 0) return mkc(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
  return mkc(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}

// a * (SIGN * i)
template <int SIGN, class C> __device__ __forceinline__ C mul_si(C a) {
  if (SIGN < 0) return mkc(a.y, -a.x);
  return mkc(-a.y, a.x);
}

template <int R, int SIGN, class C> struct Dft;

template <int SIGN, class C> struct Dft<2, SIGN, C> {
  static __device__ __forceinline__ void run(C *v) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int SIGN, class C> struct Dft<4, SIGN, C> {
  static __device__ __forceinline__ void run(C *v) {
    C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    C b0 = cadd(v[1], v[3]), b1 = mul_si<SIGN>(csub(v[1], v[3]));
    v[0] = cadd(a0, b0);
    v[2] = csub(a0, b0);
    v[1] = cadd(a1, b1);
    v[3] = csub(a1, b1);
  }
};

template <int SIGN, class C> struct Dft<3, SIGN, C> {
  static __device__ __forceinline__ void run(C *v) {
    typedef decltype(v[0].x) T;
    const T s3 = (T)(SIGN < 0 ? -0.86602540378443864676372317075294 : 0.86602540378443864676372317075294);
    C t1 = cadd(v[1], v[2]);
    C t2 = mkc(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
    C d = csub(v[1], v[2]);
    C jt3 = mkc(-s3 * d.y, s3 * d.x);  // i * s3 * (v1 - v2)
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, jt3);
    v[2] = csub(t2, jt3);
  }
};

template <int SIGN, class C> struct Dft<5, SIGN, C> {
  static __device__ __forceinline__ void run(C *v) {
    typedef decltype(v[0].x) T;
    const T c1 = (T)0.30901699437494742410229341718281906;   // cos(2 pi/5)
    const T c2 = (T)-0.80901699437494742410229341718281906;  // cos(4 pi/5)
    const T s1 = (T)(SIGN < 0 ? -0.95105651629515357211643933337938214 : 0.95105651629515357211643933337938214);
    const T s2 = (T)(SIGN < 0 ? -0.58778525229247312916870595463907277 : 0.58778525229247312916870595463907277);
    const C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    const C a1 = mkc(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    const C a2 = mkc(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    const C b1 = mkc(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    const C b2 = mkc(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    v[0] = cadd(v[0], cadd(t1, t2));
    // X1 = a1 + i b1, X4 = a1 - i b1, X2 = a2 + i b2, X3 = a2 - i b2
    v[1] = mkc(a1.x - b1.y, a1.y + b1.x);
    v[4] = mkc(a1.x + b1.y, a1.y - b1.x);
    v[2] = mkc(a2.x - b2.y, a2.y + b2.x);
    v[3] = mkc(a2.x + b2.y, a2.y - b2.x);
  }
};

template <int SIGN, class C> struct Dft<8, SIGN, C> {
  static __device__ __forceinline__ void run(C *v) {
    typedef decltype(v[0].x) T;
    const T h = (T)0.70710678118654752440084436210485;
    // even / odd DFT4s
    C e[4] = {v[0], v[2], v[4], v[6]};
    C o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, SIGN, C>::run(e);
    Dft<4, SIGN, C>::run(o);
    // o[k] *= W8^k, W8 = exp(SIGN*i*pi/4)
    C o1 = o[1], o3 = o[3];
    // W8^1 = h*(1 + SIGN*i):  (x + iy)(1 + s i) = (x - s y) + i (y + s x)
    o[1] = SIGN < 0 ? mkc(h * (o1.x + o1.y), h * (o1.y - o1.x)) : mkc(h * (o1.x - o1.y), h * (o1.y + o1.x));
    o[2] = mul_si<SIGN>(o[2]);
    // W8^3 = h*(-1 + SIGN*i): (x + iy)(-1 + s i) = (-x - s y) + i (s x - y)
    o[3] = SIGN < 0 ? mkc(h * (o3.y - o3.x), -h * (o3.x + o3.y)) : mkc(-h * (o3.x + o3.y), h * (o3.x - o3.y));
#pragma unroll
    for (int k = 0; k < 4; k++) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

// One in-place stage over `nlines` lines stored in shared memory: element e
// of line l lives at data[l*ls + e*es].  `lines_fast` maps consecutive
// threads to consecutive lines (for interleaved lines, ls == 1), otherwise to
// consecutive butterflies of one line.  MAXV bounds the complex values a
// thread holds: the caller guarantees nlines*n <= MAXV*blockDim.x.
template <typename T, int R, int SIGN, int MAXV>
__device__ __forceinline__ void fft_stage(cx<T> *data, int n, int nlines, int ls, int es, int Ns,
                                          const cx<T> *tw, bool lines_fast) {
  typedef cx<T> C;
  constexpr int MAXB = (MAXV + R - 1) / R;
  const int nb = n / R;
  const int total = nb * nlines;
  const int tstep = n / (Ns * R);
  C v[MAXB][R];
#pragma unroll
  for (int i = 0; i < MAXB; i++) {
    const int b = threadIdx.x + i * blockDim.x;
    if (b < total) {
      int l, j;
      if (lines_fast) { l = b % nlines; j = b / nlines; } else { j = b % nb; l = b / nb; }
      const int k = j % Ns;
      const C *src = data + l * ls + j * es;
      v[i][0] = src[0];
#pragma unroll
      for (int r = 1; r < R; r++) v[i][r] = ctw<SIGN>(src[r * nb * es], tw[r * k * tstep]);
      Dft<R, SIGN, C>::run(v[i]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < MAXB; i++) {
    const int b = threadIdx.x + i * blockDim.x;
    if (b < total) {
      int l, j;
      if (lines_fast) { l = b % nlines; j = b / nlines; } else { j = b % nb; l = b / nb; }
      const int k = j % Ns;
      C *dst = data + l * ls + ((j / Ns) * Ns * R + k) * es;
#pragma unroll
      for (int r = 0; r < R; r++) dst[r * Ns * es] = v[i][r];
    }
  }
  __syncthreads();
}

// Full line FFT (all stages of plan `ap`) on shared-memory lines.
template <typename T, int SIGN, int MAXV>
__device__ __forceinline__ void fft_lines(cx<T> *data, const AxisPlan &ap, int nlines, int ls, int es,
                                          const cx<T> *tw) {
  const bool lf = (ls == 1 && es != 1);
  int Ns = 1;
  for (int s = 0; s < ap.nst; s++) {
    const int R = ap.radix[s];
    if (R == 8) fft_stage<T, 8, SIGN, MAXV>(data, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 4) fft_stage<T, 4, SIGN, MAXV>(data, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 3) fft_stage<T, 3, SIGN, MAXV>(data, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 5) fft_stage<T, 5, SIGN, MAXV>(data, ap.n, nlines, ls, es, Ns, tw, lf);
    else fft_stage<T, 2, SIGN, MAXV>(data, ap.n, nlines, ls, es, Ns, tw, lf);
    Ns *= R;
  }
}

// 2-D FFT of an nx-by-ny plane (x fastest) resident in shared memory.
template <typename T, int SIGN, int MAXV>
__device__ __forceinline__ void fft_plane(cx<T> *plane, const DevGeom &g, const cx<T> *twx,
                                          const cx<T> *twy) {
  fft_lines<T, SIGN, MAXV>(plane, g.ax[0], g.ny, g.nx, 1, twx);  // rows along x
  fft_lines<T, SIGN, MAXV>(plane, g.ax[1], g.nx, 1, g.nx, twy);  // columns along y
}

// Out-of-place ("ping-pong") Stockham stage, src -> dst: each thread reads,
// transforms and writes one butterfly at a time, so it holds only R values
// and the stage needs a single barrier (after the writes).  For the FP32
// kernels of the mixed form, whose planes leave room for a second buffer: the
// in-place form above keeps all MAXV values of a thread in registers across
// its barrier, which spills for MAXV >= 16.
template <typename T, int R, int SIGN>
__device__ __forceinline__ void fft_stage_pp(const cx<T> *__restrict__ src, cx<T> *__restrict__ dst, int n,
                                             int nlines, int ls, int es, int Ns, const cx<T> *tw, bool lines_fast) {
  typedef cx<T> C;
  const int nb = n / R;
  const int total = nb * nlines;
  const int tstep = n / (Ns * R);
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    int l, j;
    if (lines_fast) { l = b % nlines; j = b / nlines; } else { j = b % nb; l = b / nb; }
    const int k = j % Ns;
    const C *sp = src + l * ls + j * es;
    C v[R];
    v[0] = sp[0];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = ctw<SIGN>(sp[r * nb * es], tw[r * k * tstep]);
    Dft<R, SIGN, C>::run(v);
    C *dp = dst + l * ls + ((j - k) * R + k) * es;
#pragma unroll
    for (int r = 0; r < R; r++) dp[r * Ns * es] = v[r];
  }
  __syncthreads();
}

// All stages of plan `ap` alternating between buffers a and b (the data
// starts in a and must be visible to the whole block); returns the buffer
// holding the result.
template <typename T, int SIGN>
__device__ __forceinline__ cx<T> *fft_lines_pp(cx<T> *a, cx<T> *b, const AxisPlan &ap, int nlines, int ls, int es,
                                               const cx<T> *tw) {
  const bool lf = (ls == 1 && es != 1);
  int Ns = 1;
  for (int s = 0; s < ap.nst; s++) {
    const int R = ap.radix[s];
    if (R == 8) fft_stage_pp<T, 8, SIGN>(a, b, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 4) fft_stage_pp<T, 4, SIGN>(a, b, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 3) fft_stage_pp<T, 3, SIGN>(a, b, ap.n, nlines, ls, es, Ns, tw, lf);
    else if (R == 5) fft_stage_pp<T, 5, SIGN>(a, b, ap.n, nlines, ls, es, Ns, tw, lf);
    else fft_stage_pp<T, 2, SIGN>(a, b, ap.n, nlines, ls, es, Ns, tw, lf);
    cx<T> *t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// 2-D FFT of an nx-by-ny plane held in buffer a (other: a second buffer of
// the same size); returns the buffer holding the result.
template <typename T, int SIGN>
__device__ __forceinline__ cx<T> *fft_plane_pp(cx<T> *a, cx<T> *other, const DevGeom &g, const cx<T> *twx,
                                               const cx<T> *twy) {
  cx<T> *r = fft_lines_pp<T, SIGN>(a, other, g.ax[0], g.ny, g.nx, 1, twx);
  return fft_lines_pp<T, SIGN>(r, r == a ? other : a, g.ax[1], g.nx, 1, g.nx, twy);
}

// Copies a twiddle table (n entries) from global to shared memory.
template <typename T>
__device__ __forceinline__ void load_tw(cx<T> *dst, const cx<T> *twbuf, const AxisPlan &ap) {
  for (int t = threadIdx.x; t < ap.n; t += blockDim.x) dst[t] = twbuf[ap.tw + t];
}

}  // namespace scft
