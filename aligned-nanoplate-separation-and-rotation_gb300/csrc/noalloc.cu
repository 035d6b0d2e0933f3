// noalloc.cu -- scft_diblock_density_noalloc: the FP64 diblock propagator and
// density (the same kernels as scft_diblock_density) for callers that must not
// allocate device memory, with all scratch in one file-scope device array.
//
// Who needs it: code whose GPU memory is owned by another framework's pool
// allocator (allocating behind its back fragments or oversubscribes that
// pool), services with a fixed memory budget set at start-up, and code that
// cannot accept the device-wide wait of cudaFree (it waits for all work
// queued on the device, other streams included).  They pass device buffers for the inputs and
// outputs; everything else lives in g_noalloc_scratch.
//
// The array is g_noalloc_scratch (kNoAllocScratchBytes = 64 MiB); every GPU
// that loads libscft holds it until the process exits.  Host code cannot use
// the symbol's name as a device address, so on the first call on each device
// (with that device current) the address is fetched once with
// cudaGetSymbolAddress and cached; that first call should come before any
// stream capture.  The cache is keyed by device ordinal and does not survive
// cudaDeviceReset (or any teardown of the device's primary context): the
// module is loaded again there, possibly at another address.  All calls
// share the array and it keeps the last call's contents: the density
// accumulators are cleared on every call, the tables and job lists
// rewritten; calls that overlap on the GPU (different streams, or different
// host threads) race on it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/scft.h"
#include "fft_core.cuh"
#include "prop_launch.h"

namespace scft {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void *g_addr[kMaxDevices] = {};

constexpr double kPI_na = 3.14159265358979323846263383;  // code/globals.h:31

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

bool plan_axis(int n, AxisPlan &ap) {
  ap.n = n;
  ap.nst = 0;
  int m = n;
  const int rs[5] = {8, 4, 2, 3, 5};
  for (int r : rs)
    while (m % r == 0 && ap.nst < kMaxStages) {
      ap.radix[ap.nst++] = r;
      m /= r;
    }
  return m == 1;
}

LaunchShape shape_for(int E, size_t extra) {
  LaunchShape s;
  int maxv = 8, t = 0;
  for (maxv = 8; maxv <= 32; maxv *= 2) {
    t = ((E + maxv - 1) / maxv + 31) / 32 * 32;
    if (t <= 512) break;
  }
  if (maxv > 32) maxv = 32;
  if (t < 64) t = 64;
  s.threads = t;
  s.maxv = maxv;
  s.smem = (int)(E * sizeof(double2) + extra);
  s.gm = 0;  // larger planes are rejected below
  return s;
}

// Fills the scratch: twiddle tables, the bond kernel exp(-k^2/6) with the
// reference's get_k (code/array_utils.cpp:239-272, code/initialize.cpp:401-404),
// the geometry and instance views, and the job lists of the sweep.
__global__ void k_noalloc_prepare(DevGeom g, double L0, double L1, double L2, double2 *tw, double *pbond,
                                  DevGeom *dgeom, PropInst pi, PropInst *dpi, FieldInst fi, FieldInst *dfi,
                                  PropJob *pj, int npj_per_p, ColJob *cj, int ncj_per_p, int nprop) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (tid == 0) {
    *dgeom = g;
    *dpi = pi;
    *dfi = fi;
  }
  const int n3[3] = {g.nx, g.ny, g.nz};
  for (int d = 0; d < 3; d++)
    for (long long t = tid; t < n3[d]; t += stride) {
      double s, c;
      sincospi(2.0 * (double)t / (double)n3[d], &s, &c);
      tw[g.ax[d].tw + t] = make_double2(c, -s);
    }
  const double Ls[3] = {L0, L1, L2};
  for (long long i = tid; i < g.M; i += stride) {
    const int n[3] = {(int)(i % g.nx), (int)((i / g.nx) % g.ny), (int)(i / ((long long)g.nx * g.ny))};
    double kmag = 0.0;
    for (int d = 0; d < 3; d++) {
      const double k = (double(n[d]) < double(n3[d]) / 2.) ? 2 * kPI_na * double(n[d]) / Ls[d]
                                                         : 2 * kPI_na * double(n[d] - n3[d]) / Ls[d];
      kmag += k * k;
    }
    pbond[i] = exp(-kmag / 6.0);
  }
  for (long long j = tid; j < (long long)nprop * npj_per_p; j += stride) {
    const int p = (int)(j / npj_per_p), z = (int)(j % npj_per_p);
    pj[j] = PropJob{0, p, z};
  }
  const int tiles_x = g.nx / g.tx;
  for (long long j = tid; j < (long long)nprop * ncj_per_p; j += stride) {
    const int p = (int)(j / ncj_per_p), r = (int)(j % ncj_per_p);
    const int y = r / tiles_x, x0 = (r % tiles_x) * g.tx;
    cj[j] = ColJob{pi.work[p], pbond, 0, x0, y};
  }
}

}  // namespace

// Device address of g_noalloc_scratch on the current device (fetched once).
static int noalloc_base(void **out, std::string &msg) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    msg = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return SCFT_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    msg = "device ordinal beyond the no-allocation table";
    return SCFT_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      msg = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return SCFT_ERR_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return SCFT_OK;
}

int noalloc_diblock(const int *Nx, const double *L, int Nda, int Ndb, double nD, const double *smwa,
                    const double *smwb, double *rhoda, double *rhodb, double *Q, void *stream, std::string &msg) {
  if (!Nx || !L || !smwa || !smwb || !rhoda || !rhodb || !Q) {
    msg = "null argument";
    return SCFT_ERR_ARG;
  }
  const int N = Nda + Ndb;
  if (Nda < 0 || Ndb < 0 || N < 1) {
    msg = "Nda + Ndb must be >= 1";
    return SCFT_ERR_ARG;
  }
  DevGeom g;
  g.nx = Nx[0];
  g.ny = Nx[1];
  g.nz = Nx[2];
  for (int d = 0; d < 3; d++) {
    if (Nx[d] < 2 || !(L[d] > 0)) {
      msg = "grid sizes must be >= 2 and box lengths positive";
      return SCFT_ERR_ARG;
    }
    if (!plan_axis(Nx[d], g.ax[d])) {
      msg = "grid sizes must be 2^a 3^b 5^c";
      return SCFT_ERR_UNSUPPORTED;
    }
  }
  g.M = (long long)g.nx * g.ny * g.nz;
  set_inv_m(g);
  g.tx = 16;
  while (g.nx % g.tx) g.tx /= 2;
  g.ax[0].tw = 0;
  g.ax[1].tw = g.nx;
  g.ax[2].tw = g.nx + g.ny;
  const long long M = g.M;
  const int single = (Nda == 0 || Nda == N);
  const int nprop = single ? 1 : 2;
  const int hmax = (N - 1) / 2;
  const int npj = g.nz;
  const int ncj = g.ny * (g.nx / g.tx);
  // scratch layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  const size_t o_geom = take(sizeof(DevGeom));
  const size_t o_pi = take(sizeof(PropInst));
  const size_t o_fi = take(sizeof(FieldInst));
  const size_t o_tw = take(sizeof(double2) * (size_t)(g.nx + g.ny + g.nz));
  const size_t o_pb = take(sizeof(double) * (size_t)M);
  const size_t o_E = take(sizeof(double2) * (size_t)M * 2);
  const size_t o_work = take(sizeof(double2) * (size_t)M * nprop);
  const size_t o_hist = take(sizeof(double2) * (size_t)M * (hmax + 1) * nprop);
  const size_t o_acc = take(sizeof(double2) * (size_t)M * 4);
  const size_t o_qp = take(sizeof(double2) * (size_t)g.nz);
  const size_t o_sc = take(sizeof(double2) * kNumScalars);
  const size_t o_pj = take(sizeof(PropJob) * (size_t)npj * nprop);
  const size_t o_cj = take(sizeof(ColJob) * (size_t)ncj * nprop);
  if (off > kNoAllocScratchBytes) {
    msg = "grid x chain length needs " + std::to_string(off >> 20) +
          " MiB of scratch; scft_diblock_density_noalloc is limited to 64 MiB "
          "(about M * (136 + 32 * ((N - 1) / 2 + 1)) bytes for a diblock)";
    return SCFT_ERR_ARG;
  }
  const LaunchShape sp = shape_for(g.nx * g.ny, (g.nx + g.ny + 32) * sizeof(double2));
  const LaunchShape sc = shape_for(g.tx * g.nz, (g.nz + 32) * sizeof(double2));
  if (sp.smem > 227 * 1024) {
    msg = "xy plane too large for the FP64 plane pass";
    return SCFT_ERR_UNSUPPORTED;
  }
  if (sc.smem > 227 * 1024) {
    msg = "z columns too long for the FP64 column pass";
    return SCFT_ERR_UNSUPPORTED;
  }
  void *basev = nullptr;
  if (int st = noalloc_base(&basev, msg)) return st;
  unsigned char *base = static_cast<unsigned char *>(basev);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto at = [&](size_t o) { return static_cast<void *>(base + o); };

  double2 *E = static_cast<double2 *>(at(o_E));
  double2 *work = static_cast<double2 *>(at(o_work));
  double2 *hist = static_cast<double2 *>(at(o_hist));
  double2 *acc = static_cast<double2 *>(at(o_acc));
  PropInst pi;
  memset(&pi, 0, sizeof pi);
  pi.geom = 0;
  pi.N = N;
  pi.Na = Nda;
  pi.single = single;
  pi.hmax = hmax;
  for (int q = 0; q < 2; q++) {
    const int qq = single ? 0 : q;
    pi.work[q] = work + (size_t)M * qq;
    pi.hist[q] = hist + (size_t)M * (hmax + 1) * qq;
    pi.expw[q] = E + (size_t)M * q;
    for (int s = 0; s < 2; s++) pi.acc[q][s] = acc + (size_t)M * (2 * q + s);
  }
  pi.qpart = static_cast<double2 *>(at(o_qp));
  FieldInst fi;
  memset(&fi, 0, sizeof fi);
  fi.M = M;
  fi.geom = 0;
  double V = 1.0;
  for (int d = 0; d < 3; d++) {
    fi.dx[d] = L[d] / double(Nx[d]);
    V *= L[d];
  }
  fi.V = V;
  fi.nD = nD;
  fi.N = N;
  fi.single = single;
  fi.sm[0] = const_cast<double2 *>(reinterpret_cast<const double2 *>(smwa));
  fi.sm[1] = const_cast<double2 *>(reinterpret_cast<const double2 *>(smwb));
  fi.expw[0] = E;
  fi.expw[1] = E + M;
  fi.rho[0] = reinterpret_cast<double2 *>(rhoda);
  fi.rho[1] = reinterpret_cast<double2 *>(rhodb);
  for (int q = 0; q < 2; q++)
    for (int s = 0; s < 2; s++) fi.acc[q][s] = acc + (size_t)M * (2 * q + s);
  fi.qpart = pi.qpart;
  fi.nz = g.nz;
  fi.scal = static_cast<double2 *>(at(o_sc));

  const DevGeom *dgeom = static_cast<const DevGeom *>(at(o_geom));
  const PropInst *dpi = static_cast<const PropInst *>(at(o_pi));
  const FieldInst *dfi = static_cast<const FieldInst *>(at(o_fi));
  PropJob *pj = static_cast<PropJob *>(at(o_pj));
  ColJob *cj = static_cast<ColJob *>(at(o_cj));
  const int blocks = (int)std::min<long long>(1024, (M + 255) / 256);
  cudaError_t e = cudaSuccess;
  k_noalloc_prepare<<<blocks, 256, 0, st>>>(g, L[0], L[1], L[2], static_cast<double2 *>(at(o_tw)),
                                            static_cast<double *>(at(o_pb)), const_cast<DevGeom *>(dgeom), pi,
                                            const_cast<PropInst *>(dpi), fi, const_cast<FieldInst *>(dfi), pj, npj,
                                            cj, ncj, nprop);
  e = cudaGetLastError();
  // the accumulators must start at zero on every call
  if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, sizeof(double2) * (size_t)M * 4, st);
  if (e == cudaSuccess) e = launch_boltzmann(dfi, 1, blocks, st);
  if (e == cudaSuccess) e = launch_prop_plane_f64(sp, pj, nprop * npj, dpi, dgeom, at(o_tw), 0, st);
  for (int s = 1; s < N && e == cudaSuccess; s++) {
    e = launch_col_fft<double>(sc, cj, nprop * ncj, dgeom, at(o_tw), 2, 1, st);
    if (e == cudaSuccess) e = launch_prop_plane_f64(sp, pj, nprop * npj, dpi, dgeom, at(o_tw), s, st);
  }
  if (e == cudaSuccess) e = launch_q_finalize(dfi, 1, st);
  if (e == cudaSuccess) e = launch_density(dfi, 1, blocks, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(Q, static_cast<double2 *>(at(o_sc)) + kQd, sizeof(double2), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) {
    msg = std::string("CUDA: ") + cudaGetErrorString(e);
    return SCFT_ERR_CUDA;
  }
  return SCFT_OK;
}

}  // namespace scft
