// common.h -- types shared by the host side and the CUDA kernels of libscft.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace scft {

constexpr int kMaxStages = 8;

// Polls of a bounded mbarrier wait before the kernel records a timeout in the
// context's error word (each poll is one mbarrier.try_wait, which itself
// suspends the thread for a hardware-chosen interval).
constexpr int kWaitPolls = 1 << 22;
// Polls (each followed by a ~64 ns sleep) of a dependency wait of the
// persistent sweep before it gives up.
constexpr int kSpinPolls = 1 << 24;

// Stage plan of a 1-D FFT of length n along one grid axis: radices applied in
// order (Stockham autosort, decimation in time) and the offset of this
// length's twiddle table exp(-2*pi*i*t/n), t = 0..n-1, in the context's
// twiddle buffer.
struct AxisPlan {
  int n;
  int nst;
  int radix[kMaxStages];
  int tw;
};

// Geometry of one instance's grid, as the kernels see it.
struct DevGeom {
  int nx, ny, nz;
  int tx;  // x-columns per z-pass tile (divides nx)
  long long M;
  AxisPlan ax[3];
  // 1/M in FP64 and as an FP32 two-float pair, formed once on the host: the
  // transform kernels scale by it and GB300 runs FP64 division (and FP64 in
  // general) at a small fraction of the FP32 rate
  double inv_m;
  float inv_m_hi, inv_m_lo;
};

inline void set_inv_m(DevGeom &g) {
  g.inv_m = 1.0 / (double)g.M;
  g.inv_m_hi = (float)g.inv_m;
  g.inv_m_lo = (float)(g.inv_m - (double)g.inv_m_hi);
}

// One CTA of an xy-plane pass: array base pointer (complex, M entries),
// geometry index, z plane.
struct PlaneJob {
  void *ptr;
  int geom;
  int z;
};

// One CTA of a z-column pass: tile of `tx` consecutive x columns at row y.
// kern: optional real k-space multiplier table (M entries) for a fused
// forward-multiply-inverse pass; NULL means plain transform.
struct ColJob {
  void *ptr;
  const void *kern;
  int geom;
  int x0, y;
};

}  // namespace scft
