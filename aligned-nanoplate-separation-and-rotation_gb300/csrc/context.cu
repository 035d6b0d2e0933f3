// context.cu -- scft_ctx: instance set-up and the per-iteration sequences.
//
// Set-up follows code/initialize.cpp:45-412 (grid, smearing kernel hhat, plate
// density and graft map, volumes and chain counts, Debye functions, bond
// kernel).  Every per-point table is built on the device: the tables that the
// reference computes point by point from get_k() (hhat, poly_bond_fft, gaa,
// gab, gbb, gc) and the mixed form's update coefficients in
// kernels_setup.cu, with the same FP64 expressions; the plate profile and its
// spectral gradient with the library's FFTs.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <stdexcept>

#include "context.h"
#include "kernels_setup.h"
#include "fft_core.cuh"
#include "prop_launch.h"
#include "grad.h"
#include "plate_profile.cuh"

namespace scft {

constexpr double kPI = 3.14159265358979323846263383;  // code/globals.h:31
// Realness check of the mixed form's fields: blocks per instance and the
// per-instance stride of its per-block maxima (9 per block)
constexpr int kCheckBlocks = 112;
constexpr int kCheckStride = 1024;
static_assert(9 * kCheckBlocks <= kCheckStride, "check maxima overlap");

struct ScftError : std::runtime_error {
  int code;
  ScftError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess)                                                                      \
      throw ScftError(SCFT_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));          \
  } while (0)

// ---------------------------------------------------------------------------
// FFT plans
// ---------------------------------------------------------------------------
static bool make_axis_plan(int n, AxisPlan &ap) {
  ap.n = n;
  ap.nst = 0;
  int m = n;
  while (m % 8 == 0 && ap.nst < kMaxStages) { ap.radix[ap.nst++] = 8; m /= 8; }
  while (m % 4 == 0 && ap.nst < kMaxStages) { ap.radix[ap.nst++] = 4; m /= 4; }
  while (m % 2 == 0 && ap.nst < kMaxStages) { ap.radix[ap.nst++] = 2; m /= 2; }
  while (m % 3 == 0 && ap.nst < kMaxStages) { ap.radix[ap.nst++] = 3; m /= 3; }
  while (m % 5 == 0 && ap.nst < kMaxStages) { ap.radix[ap.nst++] = 5; m /= 5; }
  return m == 1;
}

// Stage orders an n-point axis can run with: radices 8, 4, 2, 3, 5 whose
// product is n, at most one radix-2 stage and kMaxStages stages, every
// distinct order of each such multiset; the greedy plan (make_axis_plan)
// first, then by number of stages, at most `cap` plans.  The Stockham stages
// (fft_core.cuh) take the radices in any order, so each is a valid plan.
static std::vector<AxisPlan> axis_plan_candidates(int n, int cap) {
  std::vector<std::vector<int>> sets;
  std::vector<int> cur;
  const int rs[5] = {8, 4, 2, 3, 5};
  // multisets as non-increasing index sequences into rs
  std::function<void(int, int, int)> rec = [&](int m, int from, int twos) {
    if (m == 1) {
      sets.push_back(cur);
      return;
    }
    if ((int)cur.size() >= kMaxStages) return;
    for (int k = from; k < 5; k++) {
      const int r = rs[k];
      if (m % r || (r == 2 && twos >= 1)) continue;
      cur.push_back(r);
      rec(m / r, k, twos + (r == 2));
      cur.pop_back();
    }
  };
  rec(n, 0, 0);
  std::sort(sets.begin(), sets.end(), [](const std::vector<int> &a, const std::vector<int> &b) {
    return a.size() < b.size();
  });
  std::vector<AxisPlan> out;
  AxisPlan greedy;
  if (make_axis_plan(n, greedy)) out.push_back(greedy);
  for (auto &st : sets) {
    std::vector<int> perm = st;
    std::sort(perm.begin(), perm.end());
    do {
      AxisPlan ap;
      ap.n = n;
      ap.nst = (int)perm.size();
      for (int i = 0; i < ap.nst; i++) ap.radix[i] = perm[i];
      bool dup = false;
      for (auto &o : out)
        dup = dup || (o.nst == ap.nst && std::equal(o.radix, o.radix + o.nst, ap.radix));
      if (!dup) out.push_back(ap);
    } while (std::next_permutation(perm.begin(), perm.end()) && (int)out.size() < cap);
    if ((int)out.size() >= cap) break;
  }
  return out;
}

static LaunchShape choose_shape(int E, size_t elem, size_t extra) {
  LaunchShape s;
  int maxv = 8;
  int t = 0;
  for (maxv = 8; maxv <= 32; maxv *= 2) {
    t = ((E + maxv - 1) / maxv + 31) / 32 * 32;
    if (t <= 512) break;
  }
  if (maxv > 32) {
    maxv = 32;
    t = ((E + maxv - 1) / maxv + 31) / 32 * 32;
  }
  if (t < 64) t = 64;
  s.threads = t;
  s.maxv = maxv;
  s.smem = (int)(E * elem + extra);
  s.gm = 0;
  if (s.smem > 227 * 1024) {  // plane worked on in place in global memory
    s.gm = 1;
    s.smem = (int)extra;
  }
  return s;
}

template <class T> static T *dalloc(scft_ctx *c, size_t n) {
  void *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw ScftError(SCFT_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  c->allocs.push_back(p);
  CK(cudaMemsetAsync(p, 0, n * sizeof(T), c->st));
  return reinterpret_cast<T *>(p);
}

template <class T> static T *dupload(scft_ctx *c, const std::vector<T> &v) {
  T *p = dalloc<T>(c, v.size());
  CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->st));
  return p;
}

// ---------------------------------------------------------------------------
// device set-up kernels: plate profile and graft map
// ---------------------------------------------------------------------------
struct PlateArgs {
  int nx, ny, nz;
  double dx[3], L[3], c[3], u[3];
  double len, rad, xi;
  int shape;
};

// code/initialize.cpp:578-612 (explicit_nanorod), code/array_utils.cpp:588-646;
// the profile of either shape is plate_value (plate_profile.cuh)
__global__ void k_plate(double2 *out, PlateArgs a, int accumulate) {
  const long long M = (long long)a.nx * a.ny * a.nz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % a.nx);
    const int iy = (int)((i / a.nx) % a.ny);
    const int iz = (int)(i / ((long long)a.nx * a.ny));
    const int nn[3] = {ix, iy, iz};
    double dr[3];
    for (int d = 0; d < 3; d++) {
      const double x = double(nn[d]) * a.dx[d];
      double r = x - a.c[d];
      if (r >= 0.5 * a.L[d]) r -= a.L[d];
      else if (r < -0.5 * a.L[d]) r += a.L[d];
      dr[d] = r;
    }
    const double v = plate_value(a.shape, dr, a.u, a.len, a.rad, a.xi);
    if (accumulate) out[i] = make_double2(out[i].x + v, out[i].y);
    else out[i] = make_double2(v, 0.0);
  }
}

// multiply k-space array by I*k_alias[dir] (code/array_utils.cpp:181-235, :565-579)
__global__ void k_mul_ik_alias(double2 *a, int nx, int ny, int nz, double Lx, double Ly, double Lz, int dir) {
  const long long M = (long long)nx * ny * nz;
  const int Nn[3] = {nx, ny, nz};
  const double L[3] = {Lx, Ly, Lz};
  const int has_nyq = (nx % 2 == 0) || (ny % 2 == 0) || (nz % 2 == 0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const int n[3] = {(int)(i % nx), (int)((i / nx) % ny), (int)(i / ((long long)nx * ny))};
    double k[3];
    for (int d = 0; d < 3; d++) {
      if (Nn[d] % 2 == 0 && n[d] == Nn[d] / 2) k[d] = 0.0;
      else if (double(n[d]) < double(Nn[d]) / 2.) k[d] = 2 * kPI * double(n[d]) / L[d];
      else k[d] = 2 * kPI * double(n[d] - Nn[d]) / L[d];
    }
    if (i != 0 && has_nyq) {
      for (int d = 0; d < 3; d++)
        if (k[d] == 0.0) { k[0] = k[1] = k[2] = 0.0; break; }
    }
    const double kv = k[dir];
    const double2 v = a[i];
    // v * (I*kv) with (I*kv) = (0, kv)
    a[i] = make_double2(v.x * 0.0 - v.y * kv, v.x * kv + v.y * 0.0);
  }
}

// graft map += sqrt(gx^2 + gy^2 + gz^2) (complex), code/initialize.cpp:175-186
__global__ void k_grad_mag_acc(double2 *acc, const double2 *gx, const double2 *gy, const double2 *gz, long long M) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    double2 t = make_double2(0.0, 0.0);
    const double2 *g[3] = {gx, gy, gz};
    for (int d = 0; d < 3; d++) t = cadd(t, cmul(g[d][i], g[d][i]));
    acc[i] = cadd(acc[i], csqrt_d(t));
  }
}

__global__ void k_scale_c(double2 *a, double2 s, long long M, int divide) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    if (divide) {
      // a / s (Smith)
      const double2 b = s, x = a[i];
      double2 r;
      if (fabs(b.x) < fabs(b.y)) {
        const double q = b.x / b.y, d = b.x * q + b.y;
        r = make_double2((x.x * q + x.y) / d, (x.y * q - x.x) / d);
      } else {
        const double q = b.y / b.x, d = b.y * q + b.x;
        r = make_double2((x.y * q + x.x) / d, (x.y - x.x * q) / d);
      }
      a[i] = r;
    } else {
      a[i] = cmul(a[i], s);
    }
  }
}

// U = lam * (Re big - Re core): the shell between the enlarged and the core plate.
__global__ void k_shell_potential(double *out, const double2 *big, const double2 *core, double lam, long long M) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    out[i] = lam * (big[i].x - core[i].x);
}

__global__ void k_real_part(double *out, const double2 *in, long long M) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i].x;
}

// plain block partial sums of a complex array (set-up only)
__global__ void k_sum_partials(const double2 *a, long long M, double2 *out) {
  __shared__ double2 red[32];
  double2 s = make_double2(0.0, 0.0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    s = cadd(s, a[i]);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, o);
    s.y += __shfl_down_sync(0xffffffffu, s.y, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = s;
  __syncthreads();
  if (w == 0) {
    s = l < (int)(blockDim.x >> 5) ? red[l] : make_double2(0.0, 0.0);
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o);
    }
    if (l == 0) out[blockIdx.x] = s;
  }
}

}  // namespace scft

using namespace scft;

// ---------------------------------------------------------------------------
// internal helpers (host)
// ---------------------------------------------------------------------------
namespace {

const int kSumBlocks = 128;

cd integ(scft_ctx *c, const Instance &I, const double2 *a, double2 *scratch) {
  k_sum_partials<<<kSumBlocks, 256, 0, c->st>>>(a, I.M, scratch);
  CK(cudaGetLastError());
  std::vector<double2> h(kSumBlocks);
  CK(cudaMemcpyAsync(h.data(), scratch, sizeof(double2) * kSumBlocks, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  cd s(0.0, 0.0);
  for (int b = 0; b < kSumBlocks; b++) s += cd(h[b].x, h[b].y);
  for (int d = 0; d < 3; d++) s *= I.info.dx[d];
  return s;
}

// Runs plane + column passes over a list of arrays of one instance.
void fft3d_arrays(scft_ctx *c, const Instance &I, const std::vector<double2 *> &arrs, int sign) {
  const DevGeom &g = c->geoms[I.geom];
  std::vector<PlaneJob> pj;
  std::vector<ColJob> cj;
  for (double2 *a : arrs) {
    for (int z = 0; z < g.nz; z++) pj.push_back(PlaneJob{a, I.geom, z});
    for (int y = 0; y < g.ny; y++)
      for (int x0 = 0; x0 < g.nx; x0 += g.tx) cj.push_back(ColJob{a, nullptr, I.geom, x0, y});
  }
  PlaneJob *dpj = nullptr;
  ColJob *dcj = nullptr;
  CK(cudaMalloc(&dpj, sizeof(PlaneJob) * pj.size()));
  CK(cudaMalloc(&dcj, sizeof(ColJob) * cj.size()));
  CK(cudaMemcpyAsync(dpj, pj.data(), sizeof(PlaneJob) * pj.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(dcj, cj.data(), sizeof(ColJob) * cj.size(), cudaMemcpyHostToDevice, c->st));
  LaunchShape sp = choose_shape(g.nx * g.ny, sizeof(double2), (g.nx + g.ny + 32) * sizeof(double2));
  LaunchShape sc = choose_shape(g.tx * g.nz, sizeof(double2), (g.nz + 32) * sizeof(double2));
  if (sign < 0) {
    CK(launch_plane_fft<double>(sp, dpj, (int)pj.size(), c->d_geoms, c->d_tw64, -1, 0, c->st));
    CK(launch_col_fft<double>(sc, dcj, (int)cj.size(), c->d_geoms, c->d_tw64, 0, 1, c->st));
  } else {
    CK(launch_col_fft<double>(sc, dcj, (int)cj.size(), c->d_geoms, c->d_tw64, 1, 0, c->st));
    CK(launch_plane_fft<double>(sp, dpj, (int)pj.size(), c->d_geoms, c->d_tw64, +1, 0, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  cudaFree(dpj);
  cudaFree(dcj);
}

void validate(const scft_params &p) {
  auto bad = [](const std::string &m) { throw ScftError(SCFT_ERR_ARG, m); };
  if (p.Nda < 0 || p.Ndb < 0 || p.Nda + p.Ndb < 1) bad("Nda + Ndb must be >= 1");
  for (int d = 0; d < 3; d++) {
    if (p.Nx[d] < 2) bad("Nx must be >= 2 in every direction");
    if (!(p.L[d] > 0)) bad("L must be positive");
    AxisPlan ap;
    if (!make_axis_plan(p.Nx[d], ap)) throw ScftError(SCFT_ERR_UNSUPPORTED, "grid sizes must be 2^a 3^b 5^c");
  }
  if (p.update_scheme != SCFT_UPDATE_1S && p.update_scheme != SCFT_UPDATE_EULER) bad("unknown update_scheme");
  if (p.do_cl && p.precision == SCFT_PREC_MIXED)
    throw ScftError(SCFT_ERR_UNSUPPORTED, "complex-Langevin noise makes the fields complex: FP64 method only");
  if (p.update_scheme == SCFT_UPDATE_1S && !(p.kappa > 0))
    bad("kappa must be > 0 with the 1S update (code/1s_update.cpp:72-78 leaves B unset otherwise)");
  if (!(p.rho0 > 0)) bad("rho0 must be positive");
  if (p.n_exp_nr < 0 || p.n_exp_nr > 2) bad("n_exp_nr must be 0, 1 or 2 (code/globals.h:57-58)");
  if (p.n_exp_nr > 0) {
    for (int j = 0; j < p.n_exp_nr; j++)
      for (int d = 0; d < 3; d++)
        if (p.center[j][d] < 0.0 || p.center[j][d] > 1.0) bad("plate centres are fractions of L in [0,1]");
    if (!(p.xi_nr > 0)) bad("xi_nr must be positive");
  }
  if (p.precision != SCFT_PREC_FP64 && p.precision != SCFT_PREC_MIXED) bad("unknown precision");
  if (p.shell_lambda != 0.0) {
    if (p.n_exp_nr == 0) bad("the shell potential needs at least one plate");
    if (!(p.shell_width > 0)) bad("shell_width must be positive when shell_lambda != 0");
  }
  if (p.sigma > 0 && p.Ng < 1) bad("grafted chains need Ng >= 1");
  // the z pass holds 16 columns of nz complex FP64 values in shared memory
  if (p.Nx[2] > 768) throw ScftError(SCFT_ERR_UNSUPPORTED, "Nx[2] above 768 is not supported by the z pass");
}

// Per-axis h_d = 1 - exp(-k_d^2/6) with get_k's branch
// (code/array_utils.cpp:248-265), g(k) = prod_d (1 - h_d), as [hx | hy | hz]
// for the specialised z passes.  order 2: x and y in the parity-major order
// of the 128 x 128 plane pass (wavenumber k at position (k % 2) n/2 + k / 2);
// order 3: x in the residue-major order of the 96 x 64 plane pass (k at
// (k % 3) n/3 + k / 3); 0: natural order.
std::vector<float> axis_h_table(const scft_params &p, int order) {
  std::vector<float> ht;
  for (int d = 0; d < 3; d++)
    for (int pos = 0; pos < p.Nx[d]; pos++) {
      const int r = (order == 2 && d < 2) ? 2 : ((order == 3 && d == 0) ? 3 : 1);
      const int h = p.Nx[d] / r;
      const int nn = r * (pos % h) + pos / h;
      const double k = (double(nn) < double(p.Nx[d]) / 2.) ? 2 * kPI * double(nn) / p.L[d]
                                                          : 2 * kPI * double(nn - p.Nx[d]) / p.L[d];
      ht.push_back((float)(-std::expm1(-k * k / 6.0)));
    }
  return ht;
}

void setup_instance(scft_ctx *c, Instance &I, int idx) {
  const scft_params &p = I.p;
  I.N = p.Nda + p.Ndb;
  I.Na = p.Nda;
  I.Ng = p.Ng;
  I.fD = I.N > 0 ? double(p.Nda) / double(I.N) : 0.0;
  I.Rg2 = double(I.N - 1) / 6.0;
  // code/read_input.cpp:53-85
  I.neg_ab = p.chi_ab < 0.0; I.cab = fabs(p.chi_ab);
  I.neg_bc = p.chi_bc < 0.0; I.cbc = fabs(p.chi_bc);
  I.neg_ac = p.chi_ac < 0.0; I.cac = fabs(p.chi_ac);
  const double sigma = (p.Ng == 0) ? 0.0 : p.sigma;  // code/read_input.cpp:200
  I.single = (I.Na == 0 || I.Na == I.N);
  I.hmax = (I.N - 1) / 2;
  // code/initialize.cpp:60-67
  I.M = 1;
  double V = 1.0;
  for (int d = 0; d < 3; d++) {
    I.M *= p.Nx[d];
    V *= p.L[d];
    I.info.dx[d] = p.L[d] / double(p.Nx[d]);
  }
  I.info.M = I.M;
  I.info.V = V;
  I.info.N = I.N;
  const long long M = I.M;

  // geometry record
  DevGeom g;
  g.nx = p.Nx[0];
  g.ny = p.Nx[1];
  g.nz = p.Nx[2];
  g.M = M;
  set_inv_m(g);
  g.tx = 16;
  while (g.nx % g.tx) g.tx /= 2;
  for (int d = 0; d < 3; d++) make_axis_plan(p.Nx[d], g.ax[d]);
  I.geom = (int)c->geoms.size();
  c->geoms.push_back(g);

  // k-space tables from get_k, built on the device (kernels_setup.cu)
  I.mixed = (p.precision == SCFT_PREC_MIXED);
  {
    SetupTableArgs ta;
    ta.nx = p.Nx[0];
    ta.ny = p.Nx[1];
    ta.nz = p.Nx[2];
    for (int d = 0; d < 3; d++) ta.L[d] = p.L[d];
    ta.a2 = p.a_smear * p.a_smear;
    ta.fD = I.fD;
    ta.Rg2 = I.Rg2;
    ta.alpha_c = (I.N > 1) ? double(p.Ng - 1) / double(I.N - 1) : 0.0;
    ta.graft = sigma > 0;
    I.hhat = dalloc<double>(c, M);
    I.pbond = dalloc<double>(c, M);
    I.gaa = dalloc<double>(c, M);
    I.gab = dalloc<double>(c, M);
    I.gbb = dalloc<double>(c, M);
    I.gc = dalloc<double>(c, M);
    if (I.mixed) I.h32 = dalloc<float>(c, M);
    CK(launch_setup_tables(ta, I.hhat, I.pbond, I.gaa, I.gab, I.gbb, I.gc, I.mixed ? I.h32 : nullptr, c->st));
  }

  // device arrays
  // the seven fields in one allocation, in scft_set_fields' order: one copy per instance
  I.w[0] = dalloc<double2>(c, 7 * (size_t)M);
  for (int f = 1; f < 7; f++) I.w[f] = I.w[0] + (size_t)f * M;
  for (int f = 0; f < 3; f++) I.rho[f] = dalloc<double2>(c, M);
  if (p.do_cl) {
    // noise arrays of code/1s_update.cpp:54-319: w+, then (+, -) of each pair with chi != 0
    I.eta[0] = dalloc<double2>(c, M);
    const double chis[3] = {p.chi_ab, p.chi_bc, p.chi_ac};
    for (int k = 0; k < 3; k++)
      if (chis[k] != 0.0) {
        I.eta[1 + 2 * k] = dalloc<double2>(c, M);
        I.eta[2 + 2 * k] = dalloc<double2>(c, M);
      }
    CK(cudaMallocHost(&I.eta_host, sizeof(double2) * 7 * (size_t)M));
    I.rng.reseed(p.cl_seed);
  }
  if (!I.mixed) {
    for (int f = 0; f < 3; f++) {
      I.sm[f] = dalloc<double2>(c, M);
      I.expw[f] = dalloc<double2>(c, M);
    }
    for (int q = 0; q < 2; q++)
      for (int s2 = 0; s2 < 2; s2++) I.acc[q][s2] = dalloc<double2>(c, M);
    for (int q = 0; q < 2; q++) {
      if (q == 1 && I.single) {
        I.work[1] = I.work[0];
        I.hist[1] = I.hist[0];
        continue;
      }
      I.work[q] = dalloc<double2>(c, M);
      I.hist[q] = dalloc<double2>(c, (size_t)M * (I.hmax + 1));
    }
  } else {
    I.z32 = dalloc<float2>(c, M);
    I.E32 = dalloc<float2>(c, M);
    I.work32 = dalloc<float2>(c, M);
    I.hist32 = dalloc<float2>(c, (size_t)M * (I.hmax + 1));
    I.acc32[0] = dalloc<float>(c, M);
    I.acc32[1] = dalloc<float>(c, M);
    I.part = dalloc<double>(c, (size_t)2 * I.N * g.nz);
    I.K = dalloc<int>(c, (size_t)2 * I.N + 1);
    I.htab32 = dupload(c, axis_h_table(p, 0));  // alpha, beta: mix_coefficients_final, once the plates fix phiD, phiG
  }
  I.qpart = dalloc<double2>(c, g.nz);
  I.scal = dalloc<double2>(c, kNumScalars);
  I.exp_nrH = dalloc<double2>(c, M);
  I.grafts = dalloc<double2>(c, M);
  I.rho_exp_nr = dalloc<double>(c, M);
  (void)idx;
}

// alpha, beta of w <- alpha w - beta F for each field and sign branch of
// code/1s_update.cpp:58-329 (kernels_setup.cu): semi-implicit fields (lam_pl
// with A and B) alpha = (1 + lam B)/(1 + lam A), beta = lam/(1 + lam A);
// explicit fields (lam_mi) alpha = 1/(1 + lam 2 rho0/chi), beta = lam/(1 +
// lam 2 rho0/chi); with the Euler scheme (code/Euler_update.cpp:54-179)
// alpha = 1 - lam c, beta = lam.  Runs once the plates have fixed phiD, phiG.
void mix_coefficients_final(scft_ctx *c, Instance &I) {
  const scft_params &p = I.p;
  const double rho0 = p.rho0;
  const double li = p.lam_pl, lr = p.lam_mi;
  MixCoeffArgs a;
  memset(&a, 0, sizeof a);
  a.rho0 = rho0;
  a.kappa = p.kappa;
  a.N = I.N;
  a.Ng = I.Ng;
  a.phiD = I.info.phiD;
  a.phiG = I.info.phiG;
  auto semi = [&](int f, int formula, double cc, double boff) {
    a.f[f].kind = kCoeffSemi;
    a.f[f].formula = formula;
    a.f[f].lam = li;
    a.f[f].c = cc;
    a.f[f].boff = boff;
  };
  auto expl = [&](int f, double cc) {
    a.f[f].kind = kCoeffExplicit;
    a.f[f].lam = lr;
    a.f[f].c = cc;
  };
  auto eul = [&](int f, double lam, double cc) {
    a.f[f].kind = kCoeffEuler;
    a.f[f].lam = lam;
    a.f[f].c = cc;
  };
  const double chis[3] = {I.cab, I.cbc, I.cac};
  const int negs[3] = {I.neg_ab, I.neg_bc, I.neg_ac};
  if (p.update_scheme == SCFT_UPDATE_EULER) {
    eul(0, li, p.kappa > 0.0 ? rho0 / p.kappa : 0.0);
    for (int k = 0; k < 3; k++)
      if (chis[k] != 0.0) {
        eul(1 + 2 * k, li, 2.0 * rho0 / chis[k]);
        eul(2 + 2 * k, lr, 2.0 * rho0 / chis[k]);
      }
  } else {
    semi(0, kAPlus, 0.0, rho0 / p.kappa);
    const int pos[3] = {kAB, kBC, kAC}, neg[3] = {kABNeg, kBCNeg, kACNeg};
    for (int k = 0; k < 3; k++) {
      if (chis[k] == 0.0) continue;
      const double cc = chis[k];
      if (!negs[k]) {
        semi(1 + 2 * k, pos[k], cc, 2.0 * rho0 / cc);
        expl(2 + 2 * k, cc);
      } else {
        expl(1 + 2 * k, cc);
        semi(2 + 2 * k, neg[k], cc, 2.0 * rho0 / cc);
      }
    }
  }
  // tables for the active fields only (a field whose chi is zero has none;
  // the update skips it)
  for (int f = 0; f < 7; f++)
    if (a.f[f].kind != kCoeffNone) {
      if (!I.alpha[f]) I.alpha[f] = dalloc<double>(c, I.M);
      if (!I.beta[f]) I.beta[f] = dalloc<double>(c, I.M);
      a.f[f].alpha = I.alpha[f];
      a.f[f].beta = I.beta[f];
    }
  CK(launch_mix_coeff(a, I.M, I.hhat, I.gaa, I.gab, I.gbb, I.gc, c->st));
}

// Plate profile, graft map and chain counts (code/initialize.cpp:139-386).
// Plate j of instance I with thickness len and radius rad, as k_plate takes it.
PlateArgs plate_args_of(const Instance &I, int j, double len, double rad) {
  const scft_params &p = I.p;
  PlateArgs a;
  a.nx = p.Nx[0]; a.ny = p.Nx[1]; a.nz = p.Nx[2];
  double un = 0.0;
  for (int d = 0; d < 3; d++) un += p.orient[j][d] * p.orient[j][d];
  un = sqrt(un);
  for (int d = 0; d < 3; d++) {
    a.dx[d] = I.info.dx[d];
    a.L[d] = p.L[d];
    a.c[d] = p.center[j][d] * p.L[d];
    a.u[d] = p.orient[j][d] / un;  // code/read_input.cpp:220-235
  }
  a.len = len; a.rad = rad; a.xi = p.xi_nr;
  a.shape = p.plate_shape;
  return a;
}

// Spectral gradient component d of a real-space FP64 array (in place):
// forward transform, times i k_alias[d] (Nyquist killed), inverse transform
// (code/array_utils.cpp:181-235, :565-579).
void spectral_gradient(scft_ctx *c, const Instance &I, double2 *a, int d) {
  const scft_params &p = I.p;
  fft3d_arrays(c, I, {a}, -1);
  k_mul_ik_alias<<<1024, 256, 0, c->st>>>(a, p.Nx[0], p.Nx[1], p.Nx[2], p.L[0], p.L[1], p.L[2], d);
  CK(cudaGetLastError());
  fft3d_arrays(c, I, {a}, +1);
}

void setup_plates(scft_ctx *c, Instance &I) {
  const scft_params &p = I.p;
  const long long M = I.M;
  const double sigma = (p.Ng == 0) ? 0.0 : p.sigma;
  double2 *rho_np = dalloc<double2>(c, M);
  double2 *pd = dalloc<double2>(c, M);
  double2 *gr[3] = {dalloc<double2>(c, M), dalloc<double2>(c, M), dalloc<double2>(c, M)};
  double2 *scratch = dalloc<double2>(c, kSumBlocks);
  const int blocks = 1024;
  auto plate_args = [&](int j, double len, double rad) { return plate_args_of(I, j, len, rad); };
  // graft map from the 1.05x-enlarged plates (code/initialize.cpp:160-200)
  for (int j = 0; j < p.n_exp_nr; j++) {
    k_plate<<<blocks, 256, 0, c->st>>>(pd, plate_args(j, p.L_nr * 1.05, p.R_nr * 1.05), 0);
    CK(cudaGetLastError());
    for (int d = 0; d < 3; d++) {
      CK(cudaMemcpyAsync(gr[d], pd, sizeof(double2) * M, cudaMemcpyDeviceToDevice, c->st));
      spectral_gradient(c, I, gr[d], d);
    }
    k_grad_mag_acc<<<blocks, 256, 0, c->st>>>(I.grafts, gr[0], gr[1], gr[2], M);
    CK(cudaGetLastError());
    if (j == p.n_exp_nr - 1) {
      const cd tot = integ(c, I, I.grafts, scratch);
      k_scale_c<<<blocks, 256, 0, c->st>>>(I.grafts, make_double2(tot.real(), tot.imag()), M, 1);
      CK(cudaGetLastError());
    }
  }
  // core density (code/initialize.cpp:210-239)
  for (int j = 0; j < p.n_exp_nr; j++) {
    k_plate<<<blocks, 256, 0, c->st>>>(rho_np, plate_args(j, p.L_nr, p.R_nr), 1);
    CK(cudaGetLastError());
  }
  k_real_part<<<blocks, 256, 0, c->st>>>(I.rho_exp_nr, rho_np, M);
  CK(cudaGetLastError());
  // A-attractive shell (extension, no reference counterpart): U_A = Lambda *
  // sum_j [rho_p(L + 2w, R + w) - rho_p(L, R)], acting on A segments like an
  // external field added to the smeared w_A
  if (p.shell_lambda != 0.0 && p.n_exp_nr > 0) {
    double2 *big = dalloc<double2>(c, M);
    for (int j = 0; j < p.n_exp_nr; j++) {
      k_plate<<<blocks, 256, 0, c->st>>>(big, plate_args(j, p.L_nr + 2.0 * p.shell_width, p.R_nr + p.shell_width),
                                         1);
      CK(cudaGetLastError());
    }
    I.shellU = dalloc<double>(c, M);
    k_shell_potential<<<blocks, 256, 0, c->st>>>(I.shellU, big, rho_np, p.shell_lambda, M);
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(I.exp_nrH, rho_np, sizeof(double2) * M, cudaMemcpyDeviceToDevice, c->st));
  fft3d_arrays(c, I, {I.exp_nrH}, -1);
  // volumes and counts (code/initialize.cpp:249-386), no film, no field NPs
  const double V = I.info.V;
  const double V_exp = integ(c, I, rho_np, scratch).real();
  const double Vf = V - 0.0;
  const double np_frac = V_exp / Vf;
  const double V1 = p.n_exp_nr > 0 ? V_exp / double(p.n_exp_nr) : 0.0;
  if (sigma > 0.0 && p.n_exp_nr > 0) {
    const cd en = integ(c, I, I.grafts, scratch);
    const cd inv = 1.0 / en;
    k_scale_c<<<blocks, 256, 0, c->st>>>(I.grafts, make_double2(inv.real(), inv.imag()), M, 0);
    CK(cudaGetLastError());
  }
  const double nP = (p.n_exp_nr == 0) ? 0.0 : V_exp / V1;
  double ng_per_np = 0.0, phiG = 0.0;
  if (sigma > 0.0) {
    ng_per_np = sigma * 4.0 * kPI * p.R_nr * p.R_nr;
    phiG = ng_per_np * nP * p.Ng / p.rho0 / Vf;
  }
  const double phiD = 1.0 - 0.0 - np_frac - phiG;
  I.info.Vf = Vf;
  I.info.np_frac = np_frac;
  I.info.nP = nP;
  I.info.ng_per_np = ng_per_np;
  I.info.phiG = phiG;
  I.info.phiD = phiD;
  I.info.nD = phiD * p.rho0 * Vf / I.N;
  I.graft = (sigma > 0.0 && p.n_exp_nr > 0 && nP > 0.0) ? 1 : 0;
  if (I.graft && !I.mixed) {
    I.gwork = dalloc<double2>(c, M);
    I.ghist = dalloc<double2>(c, (size_t)M * p.Ng);
    I.gacc = dalloc<double2>(c, M);
  } else if (I.graft) {
    I.zg = dalloc<double2>(c, M);
    I.Eg32 = dalloc<float>(c, M);
    I.ghist32 = dalloc<float>(c, (size_t)M * p.Ng);
    I.gacc32 = dalloc<float>(c, M);
    I.gwork32 = dalloc<float2>(c, M);
    I.gK = dalloc<int>(c, (size_t)2 * p.Ng);
    I.gpart = dalloc<double>(c, (size_t)2 * p.Ng * p.Nx[2]);
    I.sm[2] = dalloc<double2>(c, M);
  }
  if (I.mixed) mix_coefficients_final(c, I);
  CK(cudaStreamSynchronize(c->st));
}

// TMA descriptor of a float2 array seen as `rows` rows of 64 float2 (128
// floats), boxes of 64 rows x 32 floats with the 128-byte swizzle; the entry
// point comes from the driver (cuTensorMapEncodeTiled) through the runtime.
CUtensorMap tensor_map_rows(const float2 *base, unsigned long long rows, unsigned row_floats, unsigned box_rows = 64) {
  typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                               const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeFn encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn)
      throw ScftError(SCFT_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    encode = reinterpret_cast<EncodeFn>(fn);
  }
  CUtensorMap m;
  const cuuint64_t dims[2] = {row_floats, rows};
  const cuuint64_t strides[1] = {row_floats * sizeof(float)};
  const cuuint32_t box[2] = {32, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2 *>(base), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw ScftError(SCFT_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

// The plane passes' error word and first-wait poll limit (see context.h).
void ensure_err(scft_ctx *c) {
  if (c->d_err) return;
  c->d_err = dalloc<int>(c, 3);
  const int init[3] = {0, kWaitPolls, kSpinPolls};
  CK(cudaMemcpyAsync(c->d_err, init, sizeof init, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
}

// Raises the plane pass's error word (an mbarrier wait that ran out) as an error.
void check_device_error(scft_ctx *c) {
  if (!c->d_err) return;
  int h = 0;
  CK(cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (h) {
    CK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    if (h == 2)
      throw ScftError(SCFT_ERR_CUDA,
                      "a dependency wait of the persistent sweep ran out: the sweep stopped (results of that call "
                      "are invalid; set the fields again)");
    throw ScftError(SCFT_ERR_CUDA, "a TMA wait of the plane pass ran out (results of that call are invalid)");
  }
}

ColJob *col64_jobs(scft_ctx *c) { return c->d_mix64_cj_tx[c->col64_tx == 8 ? 0 : (c->col64_tx == 16 ? 1 : 2)]; }
ColJob *col128_jobs(scft_ctx *c) { return c->d_mix128_cj_tx[c->col64_tx == 8 ? 0 : (c->col64_tx == 16 ? 1 : 2)]; }
ColJob *col96_jobs(scft_ctx *c) { return c->d_mix96_cj_tx[c->col64_tx == 8 ? 0 : (c->col64_tx == 16 ? 1 : 2)]; }

// Sweep groups: the job order is cut into `sweep_phases` contiguous phases and
// each phase into `sweep_streams` contiguous groups, all of about equal N * M.
void build_groups(scft_ctx *c) {
  const int n = (int)c->inst.size();
  const std::vector<int> &order = c->job_order;
  const int P = std::max(1, std::min(c->sweep_phases, n));
  auto work = [&](int oi) { return (double)c->inst[order[oi]].N * (double)c->inst[order[oi]].M; };
  // cuts [lo, hi) into k contiguous pieces of about equal work, none empty
  auto cut = [&](int lo, int hi, int k) {
    std::vector<int> ends;
    double total = 0.0;
    for (int oi = lo; oi < hi; oi++) total += work(oi);
    double acc = 0.0;
    int i = lo;
    for (int g = 0; g < k && i < hi; g++) {
      const double target = total * (g + 1) / k;
      int j = i;
      const int left = k - g - 1;  // pieces still to fill after this one
      while (j < hi && (g == k - 1 || acc + 0.5 * work(j) < target) && hi - j > left) {
        acc += work(j);
        j++;
      }
      if (j == i) {
        acc += work(j);
        j++;
      }
      ends.push_back(j);
      i = j;
    }
    return ends;
  };
  c->groups.clear();
  int p0 = 0, ph = 0;
  for (int pe : cut(0, n, P)) {
    const int G = std::max(1, std::min(c->sweep_streams, pe - p0));
    int i0 = p0;
    for (int i1 : cut(p0, pe, G)) {
      // a group never straddles the kernel classes of a batch of mixed grids
      // (64^3, 96 x 64 x 64, 48^3, the rest): split at those boundaries
      for (int a = i0; a < i1;) {
        int b = a + 1;
        while (b < i1 && (c->fast64.empty() || (c->fast64[b] == c->fast64[a] && c->fast96[b] == c->fast96[a] &&
                                                c->fast48[b] == c->fast48[a])))
          b++;
        scft_ctx::SweepGroup gr;
        gr.inst_begin = a;
        gr.inst_end = b;
        gr.pj_begin = a ? c->inst_pj_end[a - 1] : 0;
        gr.pj_end = c->inst_pj_end[b - 1];
        gr.cj_begin = a ? c->inst_cj_end[a - 1] : 0;
        gr.cj_end = c->inst_cj_end[b - 1];
        gr.phase = ph;
        gr.fast = c->fast64.empty() ? 0 : c->fast64[a];
        gr.fast96 = c->fast96.empty() ? 0 : c->fast96[a];
        gr.fast48 = c->fast48.empty() ? 0 : c->fast48[a];
        c->groups.push_back(gr);
        a = b;
      }
      i0 = i1;
    }
    p0 = pe;
    ph++;
  }
  const int ng = (int)c->groups.size();
  while ((int)c->side.size() < ng) {
    cudaStream_t sst;
    CK(cudaStreamCreateWithFlags(&sst, cudaStreamNonBlocking));
    c->side.push_back(sst);
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    c->ev_join.push_back(ev);
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    c->ev_up.push_back(ev);
  }
  if (!c->ev_fork) CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
  if (c->sweep_persistent && c->sweep_ctr_groups < ng) {
    // counters are cleared by each launch; old arrays stay in c->allocs
    c->d_sweep_ctr = dalloc<unsigned>(c, (size_t)ng * sweep64_counters(kMix64MaxInst));
    c->sweep_ctr_groups = ng;
  }
}

// Builds the device views and job lists once all instances exist.
void build_jobs(scft_ctx *c) {
  const int n = (int)c->inst.size();
  std::vector<FieldInst> fi(n);
  std::vector<PropInst> pi(n);
  for (int k = 0; k < n; k++) {
    Instance &I = c->inst[k];
    FieldInst &F = fi[k];
    memset(&F, 0, sizeof F);
    F.M = I.M;
    F.geom = I.geom;
    F.rho0 = I.p.rho0;
    F.kappa = I.p.kappa;
    F.ikappa = I.p.kappa > 0.0 ? 1.0 / I.p.kappa : 0.0;
    F.euler = I.p.update_scheme == SCFT_UPDATE_EULER;
    F.cab = I.cab; F.cbc = I.cbc; F.cac = I.cac;
    F.neg_ab = I.neg_ab; F.neg_bc = I.neg_bc; F.neg_ac = I.neg_ac;
    F.phiD = I.info.phiD; F.phiG = I.info.phiG;
    F.lam_pl = I.p.lam_pl; F.lam_mi = I.p.lam_mi;
    F.nD = I.info.nD; F.V = I.info.V;
    for (int d = 0; d < 3; d++) F.dx[d] = I.info.dx[d];
    F.N = I.N; F.Ng = I.Ng; F.np_chem = I.p.np_chem; F.graft = I.graft; F.single = I.single;
    F.ng_per_np = I.info.ng_per_np;
    F.n_exp_nr = I.p.n_exp_nr;
    for (int f = 0; f < 7; f++) F.w[f] = I.w[f];
    for (int f = 0; f < 3; f++) { F.sm[f] = I.sm[f]; F.rho[f] = I.rho[f]; F.expw[f] = I.expw[f]; }
    F.hhat = I.hhat; F.gaa = I.gaa; F.gab = I.gab; F.gbb = I.gbb; F.gc = I.gc;
    F.rho_exp_nr = I.rho_exp_nr;
    F.exp_nrH = I.exp_nrH;
    F.shellU = I.shellU;
    for (int q = 0; q < 2; q++)
      for (int s = 0; s < 2; s++) F.acc[q][s] = I.acc[q][s];
    F.qpart = I.qpart;
    F.nz = I.p.Nx[2];
    F.scal = I.scal;
    F.gacc = I.gacc;
    F.ghist_last = (I.graft && !I.mixed) ? I.ghist + (size_t)I.M * (I.Ng - 1) : nullptr;
    F.grafts = I.grafts;
    F.nx = I.p.Nx[0];
    F.ny = I.p.Nx[1];
    for (int f = 0; f < 7; f++) F.eta[f] = nullptr;
    if (I.p.do_cl) {
      // which noise array enters which field's update (code/1s_update.cpp:81-319,
      // code/Euler_update.cpp:65-172): with the 1S scheme and a negative chi the
      // + field of AB gets none and both BC (AC) fields get the + array
      const bool eul = I.p.update_scheme == SCFT_UPDATE_EULER;
      F.eta[0] = I.eta[0];
      const int negs[3] = {I.neg_ab, I.neg_bc, I.neg_ac};
      for (int k = 0; k < 3; k++) {
        double2 *ep = I.eta[1 + 2 * k], *em = I.eta[2 + 2 * k];
        if (!ep) continue;
        if (eul || !negs[k]) {
          F.eta[1 + 2 * k] = ep;
          F.eta[2 + 2 * k] = em;
        } else {
          F.eta[1 + 2 * k] = (k == 0) ? nullptr : ep;
          F.eta[2 + 2 * k] = ep;
        }
      }
    }
    F.z32 = I.z32;
    F.zg = I.zg;
    F.Eg32 = I.Eg32;
    F.gacc32 = I.gacc32;
    F.ghist32_last = (I.graft && I.mixed) ? I.ghist32 + (size_t)I.M * (I.Ng - 1) : nullptr;
    F.gK = I.gK;
    F.E32 = I.E32;
    F.acc32[0] = I.acc32[0];
    F.acc32[1] = I.acc32[1];
    F.K = I.K;
    F.part64 = I.part;
    for (int f = 0; f < 7; f++) {
      F.alpha[f] = I.alpha[f];
      F.beta[f] = I.beta[f];
    }

    PropInst &P = pi[k];
    memset(&P, 0, sizeof P);
    P.geom = I.geom;
    P.N = I.N;
    P.Na = I.Na;
    P.single = I.single;
    P.hmax = I.hmax;
    for (int q = 0; q < 2; q++) {
      P.work[q] = I.work[q];
      P.hist[q] = I.hist[q];
      P.expw[q] = I.expw[q];
      for (int s = 0; s < 2; s++) P.acc[q][s] = I.acc[q][s];
    }
    P.qpart = I.qpart;
    P.graft = I.graft;
    P.Ng = I.Ng;
    P.gwork = I.gwork;
    P.ghist = I.ghist;
    P.gacc = I.gacc;
    P.gexpw = I.expw[2];
    P.grafts = I.grafts;
  }
  c->d_fi = dupload(c, fi);
  c->h_fi = fi;
  if (c->inst[0].mixed) {  // (c->mixed is set further down)
    // scft_set_fields: check results, instance mask, job staging for the
    // forward transforms of up to all seven fields of every instance
    c->d_realout = dalloc<double>(c, kCheckStride * (size_t)n);
    c->d_skip = dalloc<int>(c, n);
    size_t jobs = 0;
    for (auto &I : c->inst) {
      const DevGeom &g = c->geoms[I.geom];
      jobs += 7 * (size_t)std::max(g.nz, g.ny * (g.nx / g.tx));
    }
    c->jobs_cap = 2 * jobs * std::max(sizeof(PlaneJob), sizeof(ColJob));
    c->d_jobs = dalloc<char>(c, c->jobs_cap);
    CK(cudaMallocHost(&c->h_jobs, c->jobs_cap));
    CK(cudaMallocHost(&c->h_skip, sizeof(int) * (size_t)n));
  }
  if (!c->h_pin) CK(cudaMallocHost(&c->h_pin, kCheckStride * sizeof(double) * (size_t)std::max(1, n)));
  c->d_pi = dupload(c, pi);
  c->mixed = c->inst[0].mixed;
  for (auto &I : c->inst)
    if (I.mixed != c->mixed) throw ScftError(SCFT_ERR_ARG, "all instances of a context must use one precision");
  if (c->mixed) {
    std::vector<MixInst> mi(n);
    for (int k = 0; k < n; k++) {
      Instance &I = c->inst[k];
      MixInst &X = mi[k];
      memset(&X, 0, sizeof X);
      X.geom = I.geom;
      X.N = I.N;
      X.Na = I.Na;
      X.hmax = I.hmax;
      X.work = I.work32;
      X.hist = I.hist32;
      X.E = I.E32;
      X.acc[0] = I.acc32[0];
      X.acc[1] = I.acc32[1];
      X.part = I.part;
      X.K = I.K;
    }
    c->d_mi = dupload(c, mi);
    c->h_mi = mi;
    std::vector<GraftMixInst> gmi(n);
    for (int k = 0; k < n; k++) {
      Instance &I = c->inst[k];
      GraftMixInst &X = gmi[k];
      memset(&X, 0, sizeof X);
      if (!I.graft) continue;
      X.geom = I.geom;
      X.Ng = I.Ng;
      X.work = I.gwork32;
      X.hist = I.ghist32;
      X.Eg = I.Eg32;
      X.acc = I.gacc32;
      X.part = I.gpart;
      X.K = I.gK;
      X.grafts = I.grafts;
    }
    c->d_gmi = dupload(c, gmi);
    c->h_gmi = gmi;
  }

  // field transform job lists
  std::vector<PlaneJob> pj_upd, pj_fld, pj_sm;
  std::vector<ColJob> cj_upd, cj_fld, cj_sm;
  int emax_plane = 0, emax_col = 0, nxy_max = 0, nz_max = 0;
  for (int k = 0; k < n; k++) {
    Instance &I = c->inst[k];
    const DevGeom &g = c->geoms[I.geom];
    emax_plane = std::max(emax_plane, g.nx * g.ny);
    emax_col = std::max(emax_col, g.tx * g.nz);
    nxy_max = std::max(nxy_max, g.nx + g.ny);
    nz_max = std::max(nz_max, g.nz);
    std::vector<double2 *> upd = {I.rho[0], I.rho[1]};
    if (I.graft) upd.push_back(I.rho[2]);
    std::vector<double2 *> fld = {I.w[0]};
    if (I.cab != 0.0) { fld.push_back(I.w[2]); fld.push_back(I.w[1]); }
    if (I.cbc != 0.0) { fld.push_back(I.w[4]); fld.push_back(I.w[3]); }
    if (I.cac != 0.0) { fld.push_back(I.w[6]); fld.push_back(I.w[5]); }
    for (double2 *a : fld) upd.push_back(a);
    for (int g = 0; g < 7; g++)
      if (I.eta[g]) upd.push_back(I.eta[g]);  // complex-Langevin noise, forward with the densities
    std::vector<double2 *> smr = {I.sm[0], I.sm[1]};
    if (I.graft) smr.push_back(I.sm[2]);
    auto add = [&](std::vector<double2 *> &arrs, std::vector<PlaneJob> &pj, std::vector<ColJob> &cj,
                   const void *kern) {
      for (double2 *a : arrs) {
        for (int z = 0; z < g.nz; z++) pj.push_back(PlaneJob{a, I.geom, z});
        for (int y = 0; y < g.ny; y++)
          for (int x0 = 0; x0 < g.nx; x0 += g.tx) cj.push_back(ColJob{a, kern, I.geom, x0, y});
      }
    };
    if (!I.mixed) {  // the mixed form builds its field-transform lists in job order below
      add(upd, pj_upd, cj_upd, nullptr);
      add(fld, pj_fld, cj_fld, nullptr);
      add(smr, pj_sm, cj_sm, I.hhat);
    }
  }
  c->shp_plane = choose_shape(emax_plane, sizeof(double2), (nxy_max + 32) * sizeof(double2));
  c->shp_col = choose_shape(emax_col, sizeof(double2), (nz_max + 32) * sizeof(double2));
  c->shp_prop = c->shp_plane;
  if (c->shp_col.gm) throw ScftError(SCFT_ERR_UNSUPPORTED, "z columns too long for the z pass (16 nz tx B > 227 KB)");
  c->d_pj_upd = dupload(c, pj_upd); c->n_pj_upd = (int)pj_upd.size();
  c->d_pj_fld = dupload(c, pj_fld); c->n_pj_fld = (int)pj_fld.size();
  c->d_pj_sm = dupload(c, pj_sm); c->n_pj_sm = (int)pj_sm.size();
  c->d_cj_upd = dupload(c, cj_upd); c->n_cj_upd = (int)cj_upd.size();
  c->d_cj_fld = dupload(c, cj_fld); c->n_cj_fld = (int)cj_fld.size();
  c->d_cj_sm = dupload(c, cj_sm); c->n_cj_sm = (int)cj_sm.size();

  // propagator job lists, instances ordered by decreasing N so that the jobs
  // still active at step n form a prefix
  std::vector<int> order(n);
  for (int k = 0; k < n; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->inst[a].N > c->inst[b].N; });
  std::vector<PropJob> ppj;
  std::vector<ColJob> pcj;
  std::vector<int> inst_pj_end(n), inst_cj_end(n);
  c->nmax = 0;
  for (int oi = 0; oi < n; oi++) {
    const int k = order[oi];
    Instance &I = c->inst[k];
    const DevGeom &g = c->geoms[I.geom];
    c->nmax = std::max(c->nmax, I.N);
    const int np = I.single ? 1 : 2;
    for (int q = 0; q < np; q++) {
      for (int z = 0; z < g.nz; z++) ppj.push_back(PropJob{k, q, z});
      for (int y = 0; y < g.ny; y++)
        for (int x0 = 0; x0 < g.nx; x0 += g.tx) pcj.push_back(ColJob{I.work[q], I.pbond, I.geom, x0, y});
    }
    inst_pj_end[oi] = (int)ppj.size();
    inst_cj_end[oi] = (int)pcj.size();
  }
  c->prop_pj_count.assign(c->nmax, 0);
  c->prop_cj_count.assign(c->nmax, 0);
  for (int s = 0; s < c->nmax; s++) {
    for (int oi = 0; oi < n; oi++) {
      if (c->inst[order[oi]].N > s) {
        c->prop_pj_count[s] = inst_pj_end[oi];
        c->prop_cj_count[s] = inst_cj_end[oi];
      }
    }
  }
  if (c->mixed) {
    // Kernel classes: a batch of 64 x 64 planes with one nz runs the 64-point
    // plane kernel throughout (xy64; and the 64- or 128-point z kernel,
    // colfast).  In a batch of mixed grids the 64^3 instances run the 64-point
    // kernels and the rest the generic ones: the 64^3 instances come first in
    // job order (each class still by decreasing N, so the instances active at
    // a step are a prefix of every sweep group), and the sweep groups never
    // straddle the two classes.
    c->xy64 = 1;
    for (auto &I : c->inst)
      if (I.p.Nx[0] != 64 || I.p.Nx[1] != 64 || I.p.Nx[2] != c->inst[0].p.Nx[2]) c->xy64 = 0;
    c->colfast = c->xy64 && (c->inst[0].p.Nx[2] == 64 || c->inst[0].p.Nx[2] == 128);
    {
      const int nz0 = c->inst[0].p.Nx[2];
      c->xy128 = (nz0 == 64 || nz0 == 128 || nz0 == 256) && c->d_tw32_64 && c->d_tw32_128 && c->d_tw32_z;
      for (auto &I : c->inst)
        if (I.p.Nx[0] != 128 || I.p.Nx[1] != 128 || I.p.Nx[2] != nz0) c->xy128 = 0;
    }
    auto is64 = [&](int k) {
      const int *X = c->inst[k].p.Nx;
      return X[0] == 64 && X[1] == 64 && X[2] == 64;
    };
    auto is96 = [&](int k) {
      const int *X = c->inst[k].p.Nx;
      return X[0] == 96 && X[1] == 64 && X[2] == 64;
    };
    auto is48 = [&](int k) {
      const int *X = c->inst[k].p.Nx;
      return X[0] == 48 && X[1] == 48 && X[2] == 48;
    };
    c->fast64.assign(n, 0);
    c->fast96.assign(n, 0);
    c->fast48.assign(n, 0);
    c->anyfast = 0;
    c->any96 = 0;
    c->any48 = 0;
    if (!c->xy64) {
      // 64^3 instances first, then 96 x 64 x 64, then 48^3, then the rest
      auto cls = [&](int k) { return is64(k) ? 0 : (is96(k) ? 1 : (is48(k) ? 2 : 3)); };
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cls(a) < cls(b); });
      for (int oi = 0; oi < n; oi++) {
        c->fast64[oi] = is64(order[oi]) ? 1 : 0;
        c->fast96[oi] = is96(order[oi]) ? 1 : 0;
        c->fast48[oi] = is48(order[oi]) ? 1 : 0;
        c->anyfast = c->anyfast || c->fast64[oi];
        if (c->fast96[oi] && !c->any96) c->first96 = oi;
        c->any96 = c->any96 || c->fast96[oi];
        if (c->fast48[oi] && !c->any48) c->first48 = oi;
        c->any48 = c->any48 || c->fast48[oi];
      }
    }
    // one plane job per z (q and qdag packed), FP32 column jobs
    ppj.clear();
    pcj.clear();
    for (int oi = 0; oi < n; oi++) {
      const int k = order[oi];
      Instance &I = c->inst[k];
      const DevGeom &g = c->geoms[I.geom];
      for (int z = 0; z < g.nz; z++) ppj.push_back(PropJob{k, 0, z});
      for (int y = 0; y < g.ny; y++)
        for (int x0 = 0; x0 < g.nx; x0 += g.tx) pcj.push_back(ColJob{I.work32, I.h32, I.geom, x0, y});
      inst_pj_end[oi] = (int)ppj.size();
      inst_cj_end[oi] = (int)pcj.size();
    }
    for (int s2 = 0; s2 < c->nmax; s2++)
      for (int oi = 0; oi < n; oi++)
        if (c->inst[order[oi]].N > s2) {
          c->prop_pj_count[s2] = inst_pj_end[oi];
          c->prop_cj_count[s2] = inst_cj_end[oi];
        }
    c->job_order = order;
    c->inst_pj_end = inst_pj_end;
    c->inst_cj_end = inst_cj_end;
    // field-level data in job order, so that a sweep group's instances are a
    // contiguous range for the field kernels and the field transforms too:
    // FP32 jobs of z32 (every instance), FP64 jobs of zg (grafted instances)
    std::vector<FieldInst> fio;
    std::vector<PlaneJob> zpj, gpj;
    std::vector<ColJob> zcj, gcj;
    c->fld_end.assign(4 * n, 0);
    for (int oi = 0; oi < n; oi++) {
      Instance &I = c->inst[order[oi]];
      const DevGeom &g = c->geoms[I.geom];
      fio.push_back(c->h_fi[order[oi]]);
      auto add_ord = [&](void *a, std::vector<PlaneJob> &pj, std::vector<ColJob> &cj) {
        for (int z = 0; z < g.nz; z++) pj.push_back(PlaneJob{a, I.geom, z});
        for (int y = 0; y < g.ny; y++)
          for (int x0 = 0; x0 < g.nx; x0 += g.tx) cj.push_back(ColJob{a, nullptr, I.geom, x0, y});
      };
      add_ord(I.z32, zpj, zcj);
      if (I.graft) add_ord(I.zg, gpj, gcj);
      c->fld_end[4 * oi + 0] = (int)zpj.size();
      c->fld_end[4 * oi + 1] = (int)zcj.size();
      c->fld_end[4 * oi + 2] = (int)gpj.size();
      c->fld_end[4 * oi + 3] = (int)gcj.size();
    }
    c->d_fi_ord = dupload(c, fio);
    c->d_zpj_ord = dupload(c, zpj);
    c->d_zcj_ord = dupload(c, zcj);
    c->d_gpj_ord = dupload(c, gpj);
    c->d_gcj_ord = dupload(c, gcj);
    build_groups(c);
    c->shp_mix = choose_shape(emax_plane, sizeof(float2), (nxy_max + 32) * sizeof(float2));
    c->shp_plane32 = c->shp_mix;  // same plane and twiddle footprint
    if (!c->shp_mix.gm && c->shp_mix.smem + emax_plane * (int)sizeof(float2) <= 227 * 1024) {
      c->shp_plane32.pp = 1;  // FP32 field transforms out of place: second plane buffer
      c->shp_plane32.smem += emax_plane * (int)sizeof(float2);
    }
    // 64-point kernel tables, indexed by job-order position (64 x (64 / tx)
    // z-pass jobs per instance); entries of generic-class instances are
    // placeholders that no launch reads
    if (c->colfast || c->anyfast) {
      for (int t = 0; t < 3; t++) {
        const int tx = 8 << t;
        std::vector<ColJob> cj64;
        for (int oi = 0; oi < n; oi++) {
          Instance &I = c->inst[order[oi]];
          const bool use = c->colfast || c->fast64[oi];
          for (int y = 0; y < 64; y++)
            for (int x0 = 0; x0 < 64; x0 += tx)
              cj64.push_back(ColJob{I.work32, I.htab32, I.geom, use ? x0 : 0, use ? y : 0});
        }
        c->d_mix64_cj_tx[t] = dupload(c, cj64);
      }
    }
    if (c->xy128) {
      // parity-major factor tables, z-pass jobs (128 x (128 / tx) per instance),
      // instance views and tensor maps of rows of 128 float2
      c->mix64_tab.clear();
      c->tmE.clear();
      c->tmH.clear();
      for (int t = 0; t < 3; t++) {
        const int tx = 8 << t;
        std::vector<ColJob> cj;
        for (int oi = 0; oi < n; oi++) {
          Instance &I = c->inst[order[oi]];
          for (int y = 0; y < 128; y++)
            for (int x0 = 0; x0 < 128; x0 += tx) cj.push_back(ColJob{I.work32, I.htab32, I.geom, x0, y});
        }
        c->d_mix128_cj_tx[t] = dupload(c, cj);
      }
      for (int oi = 0; oi < n; oi++) {
        Instance &I = c->inst[order[oi]];
        const std::vector<float> ht = axis_h_table(I.p, 2);
        CK(cudaMemcpyAsync(I.htab32, ht.data(), sizeof(float) * ht.size(), cudaMemcpyHostToDevice, c->st));
        c->mix64_tab.push_back(c->h_mi[order[oi]]);
        const unsigned long long rows = 128ULL * (unsigned long long)I.p.Nx[2];
        c->tmE.push_back(tensor_map_rows(I.E32, rows, 256));
        c->tmH.push_back(tensor_map_rows(I.hist32, rows * (unsigned long long)(I.hmax + 1), 256));
      }
      CK(cudaStreamSynchronize(c->st));  // the host tables are released
      ensure_err(c);
    }
    if (c->any96) {
      // residue-major x factor tables and z-pass jobs (64 x (96 / tx) per
      // instance) of the 96 x 64 x 64 instances, contiguous in job order
      for (int t = 0; t < 3; t++) {
        const int tx = 8 << t;
        std::vector<ColJob> cj;
        for (int oi = 0; oi < n; oi++) {
          if (!c->fast96[oi]) continue;
          Instance &I = c->inst[order[oi]];
          for (int y = 0; y < 64; y++)
            for (int x0 = 0; x0 < 96; x0 += tx) cj.push_back(ColJob{I.work32, I.htab32, I.geom, x0, y});
        }
        c->d_mix96_cj_tx[t] = dupload(c, cj);
      }
      for (int oi = 0; oi < n; oi++) {
        if (!c->fast96[oi]) continue;
        Instance &I = c->inst[order[oi]];
        const std::vector<float> ht = axis_h_table(I.p, 3);
        CK(cudaMemcpyAsync(I.htab32, ht.data(), sizeof(float) * ht.size(), cudaMemcpyHostToDevice, c->st));
      }
      CK(cudaStreamSynchronize(c->st));  // the host tables are released
    }
    if (c->any48) {
      // z-pass jobs of the 48^3 instances (48 x 3 tiles of 16 columns each),
      // contiguous in job order
      std::vector<ColJob> cj;
      for (int oi = 0; oi < n; oi++) {
        if (!c->fast48[oi]) continue;
        Instance &I = c->inst[order[oi]];
        for (int y = 0; y < 48; y++)
          for (int x0 = 0; x0 < 48; x0 += 16) cj.push_back(ColJob{I.work32, I.htab32, I.geom, x0, y});
      }
      c->d_mix48_cj = dupload(c, cj);
    }
    if (c->xy64 || c->anyfast || c->any96 || c->any48) {
      c->mix64_tab.clear();
      c->tmE.clear();
      c->tmH.clear();
      for (int oi = 0; oi < n; oi++) {
        c->mix64_tab.push_back(c->h_mi[order[oi]]);
        Instance &I = c->inst[order[oi]];
        if (c->xy64 || c->fast64[oi]) {
          const unsigned long long rows = 64ULL * (unsigned long long)I.p.Nx[2];
          c->tmE.push_back(tensor_map_rows(I.E32, rows, 128));
          c->tmH.push_back(tensor_map_rows(I.hist32, rows * (unsigned long long)(I.hmax + 1), 128));
        } else if (c->fast96[oi]) {  // rows of 96 float2
          const unsigned long long rows = 64ULL * (unsigned long long)I.p.Nx[2];
          c->tmE.push_back(tensor_map_rows(I.E32, rows, 192));
          c->tmH.push_back(tensor_map_rows(I.hist32, rows * (unsigned long long)(I.hmax + 1), 192));
        } else if (c->fast48[oi]) {  // rows of 48 float2, boxes of 48 rows
          const unsigned long long rows = 48ULL * (unsigned long long)I.p.Nx[2];
          c->tmE.push_back(tensor_map_rows(I.E32, rows, 96, 48));
          c->tmH.push_back(tensor_map_rows(I.hist32, rows * (unsigned long long)(I.hmax + 1), 96, 48));
        } else {
          c->tmE.push_back(CUtensorMap{});
          c->tmH.push_back(CUtensorMap{});
        }
      }
      ensure_err(c);
    }
    // Mixed plane passes in place (graft sweeps; the diblock sweep when a
    // second buffer does not fit): planes above 8192 points (128 x 128) run
    // with 16 values per thread on up to 1024 threads -- one CTA per SM by
    // shared memory either way, and half the per-thread values (and spills)
    // of the 512-thread shape.
    c->shp_mixg = c->shp_mix;
    if (emax_plane > 8192 && (emax_plane + 15) / 16 <= 1024) {
      c->shp_mixg.maxv = 16;
      c->shp_mixg.threads = ((emax_plane + 15) / 16 + 31) / 32 * 32;
    }
    // Diblock plane pass: out-of-place transforms (at most 512 threads) when a
    // second plane buffer fits; then bulk-copy staging of the planes when
    // every plane is 16-byte aligned (nx ny even) and a third buffer still
    // leaves room for two CTAs per SM.
    c->shp_mixp = c->shp_mixg;
    {
      const int pbytes = emax_plane * (int)sizeof(float2) + 16;
      bool even = true;
      for (auto &I : c->inst) even = even && ((I.p.Nx[0] * I.p.Nx[1]) % 2 == 0);
      if (!c->shp_mix.gm && c->shp_mix.smem + pbytes <= 227 * 1024) {
        c->shp_mixp = c->shp_mix;
        c->shp_mixp.pp = 1;
        c->shp_mixp.smem += pbytes;
        if (even && c->shp_mixp.smem + pbytes <= 113 * 1024) {
          c->shp_mixp.stage = 1;
          c->shp_mixp.smem += pbytes;
        }
      }
    }
    ensure_err(c);
    c->shp_col32 = choose_shape(emax_col, sizeof(float2), (nz_max + 32) * sizeof(float2));
    if (!c->shp_col32.gm && c->shp_col32.smem + emax_col * (int)sizeof(float2) <= 227 * 1024) {
      c->shp_col32.pp = 1;  // out-of-place z transforms: second tile buffer
      c->shp_col32.smem += emax_col * (int)sizeof(float2);
    }
    if (c->shp_mix.gm)
      throw ScftError(SCFT_ERR_UNSUPPORTED, "xy plane too large for the mixed plane pass (nx*ny*8 B > 227 KB)");
    if (c->shp_col32.gm) throw ScftError(SCFT_ERR_UNSUPPORTED, "z columns too long for the mixed z pass");
  }
  c->d_prop_pj = dupload(c, ppj);
  c->d_prop_cj = dupload(c, pcj);

  // graft sweep job lists, graft instances ordered by decreasing Ng
  std::vector<int> gorder;
  for (int k = 0; k < n; k++)
    if (c->inst[k].graft) gorder.push_back(k);
  std::stable_sort(gorder.begin(), gorder.end(), [&](int a, int b) { return c->inst[a].Ng > c->inst[b].Ng; });
  std::vector<PropJob> gpj;
  std::vector<ColJob> gcj;
  std::vector<int> gp_end, gc_end;
  c->ngmax = 0;
  for (int k : gorder) {
    Instance &I = c->inst[k];
    const DevGeom &g = c->geoms[I.geom];
    c->ngmax = std::max(c->ngmax, I.Ng);
    for (int z = 0; z < g.nz; z++) gpj.push_back(PropJob{k, 0, z});
    for (int y = 0; y < g.ny; y++)
      for (int x0 = 0; x0 < g.nx; x0 += g.tx)
        gcj.push_back(I.mixed ? ColJob{I.gwork32, I.h32, I.geom, x0, y} : ColJob{I.gwork, I.pbond, I.geom, x0, y});
    gp_end.push_back((int)gpj.size());
    gc_end.push_back((int)gcj.size());
  }
  c->graft_pj_count.assign(c->ngmax, 0);
  c->graft_cj_count.assign(c->ngmax, 0);
  for (int s2 = 0; s2 < c->ngmax; s2++)
    for (size_t oi = 0; oi < gorder.size(); oi++)
      if (c->inst[gorder[oi]].Ng > s2) {
        c->graft_pj_count[s2] = gp_end[oi];
        c->graft_cj_count[s2] = gc_end[oi];
      }
  if (!gpj.empty()) {
    c->d_graft_pj = dupload(c, gpj);
    c->d_graft_cj = dupload(c, gcj);
  }
  if (c->mixed && c->xy128 && !gorder.empty()) {
    c->gmi128.clear();
    for (int k : gorder) c->gmi128.push_back(c->h_gmi[k]);
    for (int t = 0; t < 3; t++) {
      const int tx = 8 << t;
      std::vector<ColJob> cj;
      for (int k : gorder) {
        Instance &I = c->inst[k];
        for (int y = 0; y < 128; y++)
          for (int x0 = 0; x0 < 128; x0 += tx) cj.push_back(ColJob{I.gwork32, I.htab32, I.geom, x0, y});
      }
      c->d_mix128_gcj_tx[t] = dupload(c, cj);
    }
  }
  c->gblocks = 64;
  c->d_gpart = dalloc<double2>(c, (size_t)n * c->gblocks * 2);
  long long mmax = 0;
  for (auto &I : c->inst) mmax = std::max(mmax, I.M);
  c->eblocks = (int)std::min<long long>(2048, (mmax + 255) / 256);
  // calc_H's partial sums: 256 blocks per instance (its FP64 products and
  // the index arithmetic of -k need a full grid)
  c->hblocks = 256;
  c->d_hpart = dalloc<double2>(c, (size_t)n * 4 * c->hblocks);
}

// Largest |Im| and |Re| of w_A and w_B over the grid (mixed form input check).
// Realness check of the mixed form's fields of every instance (blockIdx.y),
// from its FieldInst (code/calc_poly_density.cpp:45-54): per block, out[9 b] =
// max |Im w_A|, |Im w_B| (and |Im w_G| with grafts), out[9 b + 1] = the
// largest real part, out[9 b + 2 + f] = max |w_f|; out advances by
// kCheckStride per instance.  Instances with skip[inst] = 0 are checked.
// kCheckBlocks blocks per instance (the check reads all seven fields, 112
// bytes per point, and needs a full grid to run at memory speed).
__global__ void k_real_check_all(const FieldInst *__restrict__ fi, const int *__restrict__ skip, double *out) {
  const FieldInst &F = fi[blockIdx.y];
  if (skip && skip[blockIdx.y]) return;
  __shared__ double red[9][32];
  double m[9];
  for (int k = 0; k < 9; k++) m[k] = 0.0;
  const int neg_ab = F.neg_ab, neg_bc = F.neg_bc, neg_ac = F.neg_ac;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < F.M; i += (long long)gridDim.x * blockDim.x) {
    const double2 pl = F.w[0][i], abp = F.w[1][i], abm = F.w[2][i], bcp = F.w[3][i], bcm = F.w[4][i],
                  acp = F.w[5][i], acm = F.w[6][i];
    const double ia = pl.x + (neg_ab ? abm.x - abp.y : abp.x - abm.y) + (neg_ac ? acm.x - acp.y : acp.x - acm.y);
    const double ib = pl.x + (neg_ab ? -abm.x - abp.y : abp.x + abm.y) + (neg_bc ? bcm.x - bcp.y : bcp.x - bcm.y);
    const double ra = -pl.y + (neg_ab ? -abm.y - abp.x : -abp.y - abm.x) + (neg_ac ? -acm.y - acp.x : -acp.y - acm.x);
    const double rb = -pl.y + (neg_ab ? abm.y - abp.x : -abp.y + abm.x) + (neg_bc ? -bcm.y - bcp.x : -bcp.y - bcm.x);
    m[0] = fmax(m[0], fmax(fabs(ia), fabs(ib)));
    m[1] = fmax(m[1], fmax(fabs(ra), fabs(rb)));
    if (F.graft) {  // w_G (code/calc_poly_density.cpp:51-54)
      const double ig = pl.x + (neg_ac ? -acm.x - acp.y : acp.x + acm.y) + (neg_bc ? -bcm.x - bcp.y : bcp.x + bcm.y);
      const double rg = -pl.y + (neg_ac ? acm.y - acp.x : -acp.y + acm.x) + (neg_bc ? bcm.y - bcp.x : -bcp.y + bcm.x);
      m[0] = fmax(m[0], fabs(ig));
      m[1] = fmax(m[1], fabs(rg));
    }
    const double2 all[7] = {pl, abp, abm, bcp, bcm, acp, acm};
    for (int f = 0; f < 7; f++) m[2 + f] = fmax(m[2 + f], fmax(fabs(all[f].x), fabs(all[f].y)));
  }
  const int wp = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int k = 0; k < 9; k++) {
    double v = m[k];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (l == 0) red[k][wp] = v;
  }
  __syncthreads();
  if (wp == 0) {
    for (int k = 0; k < 9; k++) {
      double v = l < (int)(blockDim.x >> 5) ? red[k][l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
      if (l == 0) out[kCheckStride * (size_t)blockIdx.y + 9 * blockIdx.x + k] = v;
    }
  }
}



// CK plus one kernel launch on the context's counter
#define LK(x)        \
  do {               \
    CK(x);           \
    c->launches++;   \
  } while (0)

// calc_poly_density for every instance (code/calc_poly_density.cpp:37-161)
void seq_poly_density(scft_ctx *c) {
  const int n = (int)c->inst.size();
  cudaStream_t st = c->st;
  LK(launch_assemble(c->d_fi, n, c->eblocks, st));
  // smearing: smw = IFFT[ hhat * FFT[w] / M ]  (code/calc_poly_density.cpp:93-104)
  LK(launch_plane_fft<double>(c->shp_plane, c->d_pj_sm, c->n_pj_sm, c->d_geoms, c->d_tw64, -1, 0, st));
  LK(launch_col_fft<double>(c->shp_col, c->d_cj_sm, c->n_cj_sm, c->d_geoms, c->d_tw64, 2, 1, st));
  LK(launch_plane_fft<double>(c->shp_plane, c->d_pj_sm, c->n_pj_sm, c->d_geoms, c->d_tw64, +1, 0, st));
  LK(launch_boltzmann(c->d_fi, n, c->eblocks, st));
  for (auto &I : c->inst)
    for (int q = 0; q < 2; q++)
      for (int s = 0; s < 2; s++) CK(cudaMemsetAsync(I.acc[q][s], 0, sizeof(double2) * I.M, st));
  // propagator sweep (code/diblock_discrete.cpp:18-85, code/calc_poly_density.cpp:178-190)
  LK(launch_prop_plane_f64(c->shp_prop, c->d_prop_pj, c->prop_pj_count[0], c->d_pi, c->d_geoms, c->d_tw64, 0, st));
  for (int s = 1; s < c->nmax; s++) {
    LK(launch_col_fft<double>(c->shp_col, c->d_prop_cj, c->prop_cj_count[s], c->d_geoms, c->d_tw64, 2, 1, st));
    LK(launch_prop_plane_f64(c->shp_prop, c->d_prop_pj, c->prop_pj_count[s], c->d_pi, c->d_geoms, c->d_tw64, s,
                             st));
  }
  LK(launch_q_finalize(c->d_fi, n, st));
  LK(launch_density(c->d_fi, n, c->eblocks, st));
  // grafted chains (code/calc_poly_density.cpp:131-133,155-159)
  if (c->ngmax > 0) {
    for (auto &I : c->inst)
      if (I.graft) CK(cudaMemsetAsync(I.gacc, 0, sizeof(double2) * I.M, st));
    for (int sweep = 0; sweep < 2; sweep++) {
      LK(launch_graft_plane_f64(c->shp_prop, c->d_graft_pj, c->graft_pj_count[0], c->d_pi, c->d_geoms, c->d_tw64,
                                sweep, 0, st));
      for (int s = 1; s < c->ngmax; s++) {
        LK(launch_col_fft<double>(c->shp_col, c->d_graft_cj, c->graft_cj_count[s], c->d_geoms, c->d_tw64, 2, 1,
                                  st));
        LK(launch_graft_plane_f64(c->shp_prop, c->d_graft_pj, c->graft_pj_count[s], c->d_pi, c->d_geoms,
                                  c->d_tw64, sweep, s, st));
      }
    }
    LK(launch_graft_finalize(c->d_fi, n, c->gblocks, c->d_gpart, st));
    LK(launch_qga_finalize(c->d_fi, n, c->gblocks, c->d_gpart, st));
  }
}

// update_1s for every instance (code/1s_update.cpp:7-352)
// Complex-Langevin noise of one update (code/1s_update.cpp:356-368,
// generate_1s_noise): per array, sqrt(2 lambda) / sqrt(dx) / sqrt(dy) / sqrt(dz)
// times one Gaussian deviate of the reference's stream per grid point (stack
// order), real; the arrays are drawn in the reference's order (w+, then + and
// - of AB, BC, AC for the pairs with chi != 0) and forward-transformed with
// the densities.  Step sizes: 1S draws w+ with lam_pl and every pair's + and
// - arrays with lam_mi and lam_pl; Euler draws BC's with lam_pl and lam_mi.
void cl_generate(scft_ctx *c) {
  bool any = false;
  for (auto &I : c->inst) any = any || I.p.do_cl;
  if (!any) return;
  CK(cudaStreamSynchronize(c->st));  // the staging buffers of the last step are free
  for (auto &I : c->inst) {
    if (!I.p.do_cl) continue;
    const bool eul = I.p.update_scheme == SCFT_UPDATE_EULER;
    const double li = I.p.lam_pl, lr = I.p.lam_mi;
    const double lam[7] = {li, lr, li, eul ? li : lr, eul ? lr : li, lr, li};
    for (int g = 0; g < 7; g++) {
      if (!I.eta[g]) continue;
      double scale = std::sqrt(2.0 * lam[g]);
      for (int d = 0; d < 3; d++) scale /= std::sqrt(I.info.dx[d]);
      double2 *h = I.eta_host + (size_t)g * I.M;
      for (long long i = 0; i < I.M; i++) h[i] = make_double2(scale * I.rng.gauss(), 0.0);
      CK(cudaMemcpyAsync(I.eta[g], h, sizeof(double2) * I.M, cudaMemcpyHostToDevice, c->st));
    }
  }
}

void seq_update_1s(scft_ctx *c) {
  const int n = (int)c->inst.size();
  cudaStream_t st = c->st;
  cl_generate(c);
  LK(launch_plane_fft<double>(c->shp_plane, c->d_pj_upd, c->n_pj_upd, c->d_geoms, c->d_tw64, -1, 0, st));
  LK(launch_col_fft<double>(c->shp_col, c->d_cj_upd, c->n_cj_upd, c->d_geoms, c->d_tw64, 0, 1, st));
  LK(launch_update_1s(c->d_fi, n, c->eblocks, st));
  LK(launch_col_fft<double>(c->shp_col, c->d_cj_fld, c->n_cj_fld, c->d_geoms, c->d_tw64, 1, 0, st));
  LK(launch_plane_fft<double>(c->shp_plane, c->d_pj_fld, c->n_pj_fld, c->d_geoms, c->d_tw64, +1, 0, st));
  seq_poly_density(c);
}

// The group's sweep runs as one persistent launch: the context asks for it,
// and the group's instances are 64 x 64 x 64 grids, at most kMix64MaxInst.
bool persistent_group(const scft_ctx *c, const scft_ctx::SweepGroup &gr) {
  if (!c->sweep_persistent || c->plane64_form == 2) return false;
  const bool p64 = c->xy64 || gr.fast, z64 = c->colfast || gr.fast;
  const int nzi = gr.fast ? 64 : c->inst[0].p.Nx[2];
  return p64 && z64 && nzi == 64 && gr.inst_end - gr.inst_begin <= kMix64MaxInst;
}

// One pass of propagator step s for the instances of sweep group gr as the
// sweep launches it, on stream sg: the z pass (z = true; steps s > 0) or the
// plane pass, by the group's kernel class.  Returns false when no instance
// of the group is active at step s.
bool mix_group_step_pass(scft_ctx *c, const scft_ctx::SweepGroup &gr, int s, bool z, cudaStream_t sg) {
  // plane form 2: the generic kernels for every group (the reference the
  // specialised classes are checked against)
  const bool spec = c->plane64_form != 2;
  const bool p64 = spec && (c->xy64 || gr.fast), z64 = spec && (c->colfast || gr.fast);
  const bool c96 = spec && gr.fast96, c128 = spec && c->xy128, c48 = spec && gr.fast48;
  const int nzi = gr.fast ? 64 : c->inst[0].p.Nx[2];
  const void *twz = gr.fast ? c->d_tw32_64 : c->d_tw32_z;
  const int per = 64 * (64 / c->col64_tx);       // z-pass jobs per instance of the 64-point kernels
  const int per128 = 128 * (128 / c->col64_tx);  // and of the 128 x 128 kernels
  const int per96 = 64 * (96 / c->col64_tx);     // and of the 96 x 64 x 64 instances
  // instances of the group still active at step s: a prefix (decreasing N)
  int act = 0;
  for (int oi = gr.inst_begin; oi < gr.inst_end; oi++)
    if (c->inst[c->job_order[oi]].N > s) act = oi + 1 - gr.inst_begin;
  if (act == 0) return false;
  const int last = gr.inst_begin + act - 1;
  const int cnt = c->inst_pj_end[last] - gr.pj_begin;
  const int cc = c->inst_cj_end[last] - gr.cj_begin;
  if (z) {
    if (s == 0) return true;
    if (c48)
      LK(launch_mix_col48(c->d_mix48_cj + (size_t)(gr.inst_begin - c->first48) * 144, act * 144, c->d_tw32_48, 48, 48,
                          sg));
    else if (c96)
      LK(launch_mix_col64(col96_jobs(c) + (size_t)(gr.inst_begin - c->first96) * per96, act * per96, c->d_tw32_64, 96,
                          64, 64, c->col64_tx, sg));
    else if (c128)
      LK(launch_mix_col64(col128_jobs(c) + (size_t)gr.inst_begin * per128, act * per128, c->d_tw32_z, 128, 128, nzi,
                          c->col64_tx, sg));
    else if (z64)
      LK(launch_mix_col64(col64_jobs(c) + (size_t)gr.inst_begin * per, act * per, twz, 64, 64, nzi, c->col64_tx, sg));
    else
      LK(launch_col_fft<float>(c->shp_col32, c->d_prop_cj + gr.cj_begin, cc, c->d_geoms, c->d_tw32, 3, 1, sg));
    return true;
  }
  if (c48)
    LK(launch_mix_plane48(c->mix64_tab.data() + gr.inst_begin, c->tmE.data() + gr.inst_begin,
                          c->tmH.data() + gr.inst_begin, act, 48, c->d_tw32_48, s, c->d_err, sg));
  else if (c96)
    LK(launch_mix_plane96(c->mix64_tab.data() + gr.inst_begin, c->tmE.data() + gr.inst_begin,
                          c->tmH.data() + gr.inst_begin, act, 64, c->d_tw32_64, c->d_tw32_32, c->d_tw32_96, s, c->d_err,
                          sg));
  else if (c128)
    LK(launch_mix_plane128(c->mix64_tab.data() + gr.inst_begin, c->tmE.data() + gr.inst_begin,
                           c->tmH.data() + gr.inst_begin, act, nzi, c->d_tw32_64, c->d_tw32_128, s, c->d_err, sg));
  else if (p64)
    LK((c->plane64_form ? launch_mix_plane64w : launch_mix_plane64)(
        c->mix64_tab.data() + gr.inst_begin, c->tmE.data() + gr.inst_begin, c->tmH.data() + gr.inst_begin, act, nzi,
        c->d_tw32_64, s, c->d_err, sg));
  else
    LK(launch_mix_prop_plane(c->shp_mixp, c->d_prop_pj + gr.pj_begin, cnt, c->d_mi, c->d_geoms, c->d_tw32, s, c->d_err,
                             sg));
  return true;
}

// The FP32 propagator sweep of group g on stream sg (accumulators cleared,
// then every step), from the Boltzmann factors to the plane sums and the
// density accumulators: one persistent launch (persistent_group) or a z pass
// and a plane pass per step.
void mix_group_sweep(scft_ctx *c, int g, cudaStream_t sg) {
  const scft_ctx::SweepGroup &gr = c->groups[g];
  const int cnt_i = gr.inst_end - gr.inst_begin;
  for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) {
    Instance &I = c->inst[c->job_order[oi]];
    CK(cudaMemsetAsync(I.acc32[0], 0, sizeof(float) * I.M, sg));
    CK(cudaMemsetAsync(I.acc32[1], 0, sizeof(float) * I.M, sg));
  }
  if (persistent_group(c, gr)) {
    // the whole sweep of the group in one launch; concurrent groups share the
    // GPU's resident CTAs in proportion to their instances
    std::vector<const float *> ht;
    for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) ht.push_back(c->inst[c->job_order[oi]].htab32);
    const int G = (int)c->groups.size();
    int cap = 0;
    if (G > 1) {
      int in_phase = 0;
      for (auto &o : c->groups)
        if (o.phase == gr.phase) in_phase += o.inst_end - o.inst_begin;
      cap = std::max(1, (int)((long long)c->sweep64_cap * cnt_i / std::max(1, in_phase)));
    }
    LK(launch_mix_sweep64(c->mix64_tab.data() + gr.inst_begin, c->tmE.data() + gr.inst_begin,
                          c->tmH.data() + gr.inst_begin, ht.data(), cnt_i, c->d_tw32_64,
                          c->d_sweep_ctr + (size_t)g * sweep64_counters(kMix64MaxInst), c->d_err, cap, sg));
    return;
  }
  for (int s = 0; s < c->nmax; s++) {
    if (!mix_group_step_pass(c, gr, s, true, sg)) break;
    mix_group_step_pass(c, gr, s, false, sg);
  }
}

// Job ranges of sweep group g in the per-kind transform job lists (job
// order): FP32 plane and z jobs of the packed pair, FP64 plane and z jobs of
// the graft field.
struct GroupJobs {
  int pb, pm, cb, cm, gpb, gpm, gcb, gcm;
};
static GroupJobs group_jobs(const scft_ctx *c, const scft_ctx::SweepGroup &gr) {
  GroupJobs j;
  const int i0 = gr.inst_begin;
  auto range = [&](int kind, int &b0, int &n0) {
    b0 = i0 ? c->fld_end[4 * (i0 - 1) + kind] : 0;
    n0 = c->fld_end[4 * (gr.inst_end - 1) + kind] - b0;
  };
  range(0, j.pb, j.pm);
  range(1, j.cb, j.cm);
  range(2, j.gpb, j.gpm);
  range(3, j.gcb, j.gcm);
  return j;
}

// The k-space half of an update_1s for group g on stream sg: density pack ->
// forward FP32 transform (FP64 for the graft density) -> k-space update
// (which also forms the smeared pair).  The fields are then new and the
// densities those of the old fields.
static void mix_group_kspace_update(scft_ctx *c, int g, cudaStream_t sg) {
  const scft_ctx::SweepGroup &gr = c->groups[g];
  const int cnt_i = gr.inst_end - gr.inst_begin;
  const FieldInst *fi = c->d_fi_ord + gr.inst_begin;
  const GroupJobs j = group_jobs(c, gr);
  LK(launch_mix_rho_pack(fi, cnt_i, c->eblocks, 0, sg));
  LK(launch_plane_fft<float>(c->shp_plane32, c->d_zpj_ord + j.pb, j.pm, c->d_geoms, c->d_tw32, -1, 0, sg));
  LK(launch_col_fft<float>(c->shp_col32, c->d_zcj_ord + j.cb, j.cm, c->d_geoms, c->d_tw32, 0, 1, sg));
  if (j.gpm > 0) {
    LK(launch_plane_fft<double>(c->shp_plane, c->d_gpj_ord + j.gpb, j.gpm, c->d_geoms, c->d_tw64, -1, 0, sg));
    LK(launch_col_fft<double>(c->shp_col, c->d_gcj_ord + j.gcb, j.gcm, c->d_geoms, c->d_tw64, 0, 1, sg));
  }
  LK(launch_mix_update(fi, cnt_i, c->eblocks, sg));
}

// Mixed form, one sweep group on stream sg: the work of one update_1s (or of
// calc_poly_density when `update` is false) for the group's instances, from
// the densities of the last sweep to the densities of this one:
//   update:  the k-space half above ->
//   density: (smeared pair from the fields) ->
//   both:    inverse FP32 transform (FP64 for the graft field) -> Boltzmann
//            factors -> FP32 sweep -> Q.
// The fields stay in FP64 in k-space; only the densities going in and the
// mean-free smeared fields coming out pass through FP32 transforms, whose
// error (~1e-7 of the fluctuation) is below that of the FP32 sweep.
// Each group is an independent chain, so one group's field work runs beside
// another group's bandwidth-bound sweep.
void mix_group_chain(scft_ctx *c, int g, cudaStream_t sg, bool update) {
  const scft_ctx::SweepGroup &gr = c->groups[g];
  const int cnt_i = gr.inst_end - gr.inst_begin;
  const FieldInst *fi = c->d_fi_ord + gr.inst_begin;
  const GroupJobs j = group_jobs(c, gr);
  if (update)
    mix_group_kspace_update(c, g, sg);
  else
    LK(launch_mix_smear(fi, cnt_i, c->eblocks, sg));
  LK(launch_col_fft<float>(c->shp_col32, c->d_zcj_ord + j.cb, j.cm, c->d_geoms, c->d_tw32, 1, 0, sg));
  LK(launch_plane_fft<float>(c->shp_plane32, c->d_zpj_ord + j.pb, j.pm, c->d_geoms, c->d_tw32, +1, 0, sg));
  if (j.gpm > 0) {
    LK(launch_col_fft<double>(c->shp_col, c->d_gcj_ord + j.gcb, j.gcm, c->d_geoms, c->d_tw64, 1, 0, sg));
    LK(launch_plane_fft<double>(c->shp_plane, c->d_gpj_ord + j.gpb, j.gpm, c->d_geoms, c->d_tw64, +1, 0, sg));
  }
  LK(launch_mix_boltzmann(fi, cnt_i, c->eblocks, sg));
  mix_group_sweep(c, g, sg);
  LK(launch_mix_q_finalize(fi, cnt_i, sg));
}

// The groups of each phase forked onto side streams and joined back; then
// the grafted chains of every instance (code/calc_poly_density.cpp:131-133,
// 155-159) on the context stream.
void seq_mix(scft_ctx *c, bool update) {
  const int n = (int)c->inst.size();
  cudaStream_t st = c->st;
  const int G = (int)c->groups.size();
  const bool fork = G > 1;
  for (int g0 = 0; g0 < G;) {
    int g1 = g0;
    while (g1 < G && c->groups[g1].phase == c->groups[g0].phase) g1++;
    if (fork) {
      CK(cudaEventRecord(c->ev_fork, st));
      for (int g = g0; g < g1; g++) CK(cudaStreamWaitEvent(c->side[g], c->ev_fork, 0));
    }
    for (int g = g0; g < g1; g++) mix_group_chain(c, g, fork ? c->side[g] : st, update);
    if (fork)
      for (int g = g0; g < g1; g++) {
        CK(cudaEventRecord(c->ev_join[g], c->side[g]));
        CK(cudaStreamWaitEvent(st, c->ev_join[g], 0));
      }
    g0 = g1;
  }
  if (c->ngmax > 0) {
    for (auto &I : c->inst)
      if (I.graft) CK(cudaMemsetAsync(I.gacc32, 0, sizeof(float) * I.M, st));
    if (c->xy128 && c->plane64_form != 2) {
      // the cluster plane pass and the specialised z pass (parity-major planes)
      const int nz0 = c->inst[0].p.Nx[2];
      const int per128 = 128 * (128 / c->col64_tx);
      ColJob *gcj = c->d_mix128_gcj_tx[c->col64_tx == 8 ? 0 : (c->col64_tx == 16 ? 1 : 2)];
      for (int sweep = 0; sweep < 2; sweep++)
        for (int s = 0; s < c->ngmax; s++) {
          const int act = c->graft_pj_count[s] / nz0;  // grafted instances with Ng > s (a prefix)
          if (s > 0)
            LK(launch_mix_col64(gcj, act * per128, c->d_tw32_z, 128, 128, nz0, c->col64_tx, st));
          LK(launch_mix_graft_plane128(c->gmi128.data(), act, nz0, c->d_tw32_64, c->d_tw32_128, sweep, s, st));
        }
    } else
    for (int sweep = 0; sweep < 2; sweep++) {
      LK(launch_mix_graft_plane(c->shp_mixg, c->d_graft_pj, c->graft_pj_count[0], c->d_gmi, c->d_geoms, c->d_tw32,
                                sweep, 0, st));
      for (int s = 1; s < c->ngmax; s++) {
        LK(launch_col_fft<float>(c->shp_col32, c->d_graft_cj, c->graft_cj_count[s], c->d_geoms, c->d_tw32, 3, 1,
                                 st));
        LK(launch_mix_graft_plane(c->shp_mixg, c->d_graft_pj, c->graft_pj_count[s], c->d_gmi, c->d_geoms, c->d_tw32,
                                  sweep, s, st));
      }
    }
    LK(launch_mix_graft_finalize(c->d_fi, n, c->gblocks, c->d_gpart, st));
    LK(launch_qga_finalize(c->d_fi, n, c->gblocks, c->d_gpart, st));
  }
}

// Mixed calc_poly_density from the k-space fields.
void seq_mix_density(scft_ctx *c) { seq_mix(c, false); }

// Mixed update_1s.
void seq_mix_update(scft_ctx *c) { seq_mix(c, true); }

}  // namespace

// ---------------------------------------------------------------------------
// entry points used by capi.cpp
// ---------------------------------------------------------------------------
namespace scft {

void ctx_create(scft_ctx *c, const scft_params *params, int n_inst) {
  NvtxRange nvtx_range("scft_create");
  CK(cudaGetDevice(&c->device));
  CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  c->inst.resize(n_inst);
  for (int k = 0; k < n_inst; k++) {
    validate(params[k]);
    c->inst[k].p = params[k];
    setup_instance(c, c->inst[k], k);
  }
  // twiddle tables for every distinct axis length
  std::map<int, int> off;
  std::vector<double2> tw;
  for (auto &g : c->geoms) {
    for (int d = 0; d < 3; d++) {
      const int nn = g.ax[d].n;
      if (!off.count(nn)) {
        off[nn] = (int)tw.size();
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int t = 0; t < nn; t++) {
          const long double a = two_pi * (long double)t / (long double)nn;
          tw.push_back(make_double2((double)cosl(a), (double)-sinl(a)));
        }
      }
      g.ax[d].tw = off[nn];
    }
  }
  // the 32-, 48-, 64-, 96- and 128-point tables of the specialised passes
  for (int nn : {32, 48, 64, 96, 128})
    if (!off.count(nn)) {
      off[nn] = (int)tw.size();
      const long double two_pi = 6.283185307179586476925286766559005768L;
      for (int t = 0; t < nn; t++) {
        const long double a = two_pi * (long double)t / (long double)nn;
        tw.push_back(make_double2((double)cosl(a), (double)-sinl(a)));
      }
    }
  c->d_tw64 = dupload(c, tw);
  std::vector<float2> tw32(tw.size());
  for (size_t t = 0; t < tw.size(); t++) tw32[t] = make_float2((float)tw[t].x, (float)tw[t].y);
  c->d_tw32 = dupload(c, tw32);
  c->d_tw32_64 = static_cast<float2 *>(c->d_tw32) + off[64];
  c->d_tw32_128 = static_cast<float2 *>(c->d_tw32) + off[128];
  c->d_tw32_32 = static_cast<float2 *>(c->d_tw32) + off[32];
  c->d_tw32_96 = static_cast<float2 *>(c->d_tw32) + off[96];
  c->d_tw32_48 = static_cast<float2 *>(c->d_tw32) + off[48];
  {
    const int nz0 = c->inst.empty() ? 0 : c->inst[0].p.Nx[2];
    if (off.count(nz0)) c->d_tw32_z = static_cast<float2 *>(c->d_tw32) + off[nz0];
  }
  c->d_geoms = dupload(c, c->geoms);
  for (auto &I : c->inst) setup_plates(c, I);
  build_jobs(c);
  CK(cudaStreamSynchronize(c->st));
}

// The captured graphs (update iteration, density build, host-field steps)
// hold launches of one schedule; any change of schedule or kernel form drops
// them, and the next call captures anew.
static void drop_graphs(scft_ctx *c) {
  cudaGraphExec_t *gs[3] = {&c->g_update, &c->g_density, &c->g_step};
  for (cudaGraphExec_t *g : gs)
    if (*g) {
      CK(cudaGraphExecDestroy(*g));
      *g = nullptr;
    }
}

void ctx_destroy(scft_ctx *c) {
  if (c->g_update) cudaGraphExecDestroy(c->g_update);
  if (c->g_density) cudaGraphExecDestroy(c->g_density);
  if (c->g_step) cudaGraphExecDestroy(c->g_step);
  for (void *p : c->allocs) cudaFree(p);
  for (cudaStream_t sst : c->side) cudaStreamDestroy(sst);
  for (auto &I : c->inst)
    if (I.eta_host) cudaFreeHost(I.eta_host);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->h_jobs) cudaFreeHost(c->h_jobs);
  if (c->h_skip) cudaFreeHost(c->h_skip);
  for (cudaEvent_t ev : c->ev_join) cudaEventDestroy(ev);
  for (cudaEvent_t ev : c->ev_up) cudaEventDestroy(ev);
  if (c->h_hsum) cudaFreeHost(c->h_hsum);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->st) cudaStreamDestroy(c->st);
}

// calc_poly_density of every instance.  The first build runs eagerly (kernel
// attributes get set); later builds replay a captured graph, as update_1s
// does: a batch's density build is over a thousand launches.
void ctx_poly_density(scft_ctx *c) {
  NvtxRange nvtx_range("scft_calc_poly_density");
  auto body = [c]() {
    if (c->mixed)
      seq_mix_density(c);
    else
      seq_poly_density(c);
  };
  if (c->g_density) {
    CK(cudaGraphLaunch(c->g_density, c->st));
    c->launches += c->launches_per_density;
  } else if (!c->density_runs) {
    body();
  } else {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    const long long before = c->launches;
    try {
      body();
      c->launches_per_density = c->launches - before;
      c->launches = before;
    } catch (...) {
      cudaGraph_t g2;
      cudaStreamEndCapture(c->st, &g2);
      throw;
    }
    CK(cudaStreamEndCapture(c->st, &graph));
    CK(cudaGraphInstantiate(&c->g_density, graph, 0));
    cudaGraphDestroy(graph);
    CK(cudaGraphLaunch(c->g_density, c->st));
    c->launches += c->launches_per_density;
  }
  c->density_runs++;
  CK(cudaStreamSynchronize(c->st));
  check_device_error(c);
  c->dirty_density = 0;
}

void ctx_update(scft_ctx *c, int n_iter) {
  NvtxRange nvtx_range("scft_update_1s");
  if (n_iter <= 0) return;
  if (c->dirty_density) ctx_poly_density(c);
  int k = 0;
  bool cl = false;
  for (auto &I : c->inst) cl = cl || I.p.do_cl;
  if (cl) {  // the noise is drawn on the host every step: no captured graph
    for (; k < n_iter; k++) seq_update_1s(c);
    CK(cudaStreamSynchronize(c->st));
    return;
  }
  if (!c->g_update) {
    // first iteration runs eagerly (kernel attributes get set), then capture
    (c->mixed ? seq_mix_update(c) : seq_update_1s(c));
    CK(cudaStreamSynchronize(c->st));
    k = 1;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    const long long before = c->launches;
    try {
      (c->mixed ? seq_mix_update(c) : seq_update_1s(c));
      c->launches_per_update = c->launches - before;
      c->launches = before;
    } catch (...) {
      cudaGraph_t g2;
      cudaStreamEndCapture(c->st, &g2);
      throw;
    }
    CK(cudaStreamEndCapture(c->st, &graph));
    CK(cudaGraphInstantiate(&c->g_update, graph, 0));
    cudaGraphDestroy(graph);
  }
  for (; k < n_iter; k++) {
    CK(cudaGraphLaunch(c->g_update, c->st));
    c->launches += c->launches_per_update;
  }
  CK(cudaStreamSynchronize(c->st));
  check_device_error(c);
}

// Poll limits of the first bounded mbarrier wait of every mixed plane-pass
// CTA (d_err[1]) and of the persistent sweep's dependency waits (d_err[2]),
// read by the kernels at run time, so captured graphs need no re-capture;
// polls < 0 restores the defaults.
void ctx_set_wait_limit(scft_ctx *c, int polls) {
  ensure_err(c);
  const int lim[2] = {polls < 0 ? kWaitPolls : polls, polls < 0 ? kSpinPolls : polls};
  CK(cudaMemcpyAsync(c->d_err + 1, lim, sizeof lim, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
}

// Form of the 64-point plane pass (0: block-barrier exchanges, 1: warp-local
// columns); results are bit-identical, the captured graphs hold the old form.
void ctx_set_plane_form(scft_ctx *c, int form) {
  if (form < 0 || form > 2) throw ScftError(SCFT_ERR_ARG, "plane form must be 0, 1 or 2");
  c->plane64_form = form;
  drop_graphs(c);
}

// Persistent sweep on or off (64 x 64 x 64 groups only; others keep the
// per-step launches).  The captured graphs hold the old launches.
void ctx_set_persistent(scft_ctx *c, int on) {
  if (on && (c->xy64 || c->anyfast) && !c->sweep64_cap) CK(sweep64_capacity(&c->sweep64_cap));
  c->sweep_persistent = on ? 1 : 0;
  if (!c->mixed) return;
  build_groups(c);
  drop_graphs(c);
}

// Number of independent launch chains of the mixed sweep (1 = one chain).
void ctx_set_sweep_groups(scft_ctx *c, int groups, int phases) {
  if (groups < 1 || phases < 1) throw ScftError(SCFT_ERR_ARG, "groups and phases must be >= 1");
  c->sweep_streams = groups;
  c->sweep_phases = phases;
  if (!c->mixed) return;
  build_groups(c);
  drop_graphs(c);  // the captured graphs hold the old launch chains
}

// Autotuner of the mixed form's launch schedule: for every candidate
// (sequential phases x concurrent groups x z-pass columns per CTA of the
// 64-point kernels) it times `reps` density builds of the batch (smeared
// pair, inverse FP64 transform, Boltzmann factors, FP32 sweep: the chain of
// an update without its k-space step) with CUDA events on the context
// stream, after one untimed build, and keeps the fastest.  The builds
// recompute the current densities from the current fields, so the state is
// unchanged.
void ctx_autotune(scft_ctx *c, int reps, int *groups_out, int *phases_out, int *tx_out, double *ms_out) {
  NvtxRange nvtx_range("scft_autotune");
  *groups_out = 1;
  *phases_out = 1;
  *tx_out = 0;
  *ms_out = 0.0;
  if (!c->mixed) return;  // the FP64 method has a single schedule
  if (c->dirty_density) ctx_poly_density(c);
  const int n = (int)c->inst.size();
  std::vector<int> gs, txs;
  for (int g : {1, 2, 3, 4, 5, 6, 8})
    if (g <= n) gs.push_back(g);
  if (c->xy128 && c->inst[0].p.Nx[2] == 256)
    txs = {8, 16};  // the 256-point z pass takes at most 16 columns per CTA
  else if (c->colfast || c->anyfast || c->xy128 || c->any96)
    txs = {8, 16, 32};
  else
    txs = {c->col64_tx};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  std::vector<int> ps;
  for (int ph : {1, 2, 3, 4})
    if (ph <= n) ps.push_back(ph);
  double best = 1e300;
  int bg = c->sweep_streams, bt = c->col64_tx, bp = c->sweep_phases, bpers = c->sweep_persistent;
  // the persistent sweep applies to 64 x 64 x 64 instances
  const bool can_persist = (c->xy64 && c->inst[0].p.Nx[2] == 64) || c->anyfast;
  if (can_persist && !c->sweep64_cap) CK(sweep64_capacity(&c->sweep64_cap));
  const bool has64 = c->xy64 || c->anyfast;
  int bform = c->plane64_form;
  for (int form = 0; form <= (has64 ? 1 : 0); form++)
  for (int pers = 0; pers <= (can_persist ? 1 : 0); pers++)
  for (int ph : ps)
  for (int g : gs)
    for (int tx : txs) {
      if (g * ph > n) continue;
      // persistent: the z tasks take whole rows (tx unused); few groups, phases;
      // its plane tasks use the first form
      if (pers && (tx != txs[0] || g > 3 || ph > 2 || form)) continue;
      c->plane64_form = form;
      c->sweep_persistent = pers;
      c->sweep_phases = ph;
      c->sweep_streams = g;
      c->col64_tx = tx;
      build_groups(c);
      seq_mix_density(c);
      CK(cudaEventRecord(e0, c->st));
      for (int r = 0; r < reps; r++) seq_mix_density(c);
      CK(cudaEventRecord(e1, c->st));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms / reps < best) {
        best = ms / reps;
        bg = g;
        bt = tx;
        bp = ph;
        bpers = pers;
        bform = form;
      }
    }
  c->col64_tx = bt;
  c->sweep_persistent = bpers;
  c->plane64_form = bform;
  ctx_set_sweep_groups(c, bg, bp);
  // FFT stage orders of the generic transforms (field transforms; plane and
  // z passes of the generic grids), one axis length at a time with the
  // others fixed, timed the same way with the chosen schedule
  std::map<int, int> lens;  // axis length -> points it is applied to
  for (auto &I : c->inst)
    for (int d = 0; d < 3; d++) lens[I.p.Nx[d]] += (int)std::min<long long>(I.M, 1 << 30);
  auto time_builds = [&]() {
    seq_mix_density(c);
    CK(cudaEventRecord(e0, c->st));
    for (int r = 0; r < reps; r++) seq_mix_density(c);
    CK(cudaEventRecord(e1, c->st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    return (double)ms / reps;
  };
  auto apply = [&](int n, const AxisPlan &ap) {
    for (auto &g : c->geoms)
      for (int d = 0; d < 3; d++)
        if (g.ax[d].n == n) {
          const int tw = g.ax[d].tw;
          g.ax[d] = ap;
          g.ax[d].tw = tw;
        }
    CK(cudaMemcpyAsync(c->d_geoms, c->geoms.data(), sizeof(DevGeom) * c->geoms.size(), cudaMemcpyHostToDevice,
                       c->st));
  };
  best = time_builds();
  for (auto &kv : lens) {
    const int n = kv.first;
    const std::vector<AxisPlan> cand = axis_plan_candidates(n, 12);
    if (cand.size() < 2) continue;
    AxisPlan keep = cand[0];
    for (auto &g : c->geoms)
      for (int d = 0; d < 3; d++)
        if (g.ax[d].n == n) keep = g.ax[d];
    for (const AxisPlan &ap : cand) {
      apply(n, ap);
      const double ms = time_builds();
      if (ms < best) {
        best = ms;
        keep = ap;
      }
    }
    apply(n, keep);
  }
  CK(cudaStreamSynchronize(c->st));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graphs(c);
  *groups_out = bg;
  *phases_out = bp;
  *tx_out = (c->colfast || c->anyfast || c->xy128 || c->any96) ? bt : 0;
  *ms_out = best;
}

// Algorithmic bytes of one FP32 propagator sweep of a mixed instance (per
// point: z pass 8 + 8 per step n >= 1; plane pass: working plane in (n >= 1)
// and out (n < N - 1), Boltzmann pair, history plane out (n <= hmax) or
// stored partner in (paired steps), FP32 accumulators read and written).
static double mix_sweep_bytes(const Instance &I) {
  const int N = I.N, Na = I.p.Nda;
  double b = 0.0;
  for (int n = 0; n < N; n++) {
    const int m2 = N - 1 - n;
    double pt = 8.0;  // Boltzmann pair
    if (n >= 1) pt += 16.0 + 8.0;  // z pass in and out, plane in
    if (n < N - 1) pt += 8.0;      // plane out
    if (n <= I.hmax) pt += 8.0;    // history out
    if (m2 < n) pt += 8.0 + ((n < Na) == (m2 < Na) ? 8.0 : 16.0);  // partner in, accumulators
    else if (m2 == n) pt += 8.0;
    b += pt;
  }
  return b * (double)I.M;
}

// Isolated timing of `reps` FP32 propagator sweeps of the whole batch with
// the current schedule (groups of a phase concurrent, phases in order), no
// field work, with their algorithmic bytes.  Leaves the densities invalid.
void ctx_profile_sweep(scft_ctx *c, int reps, double *ms, double *bytes) {
  if (!c->mixed) throw ScftError(SCFT_ERR_UNSUPPORTED, "the sweep profile is for the mixed form");
  if (c->dirty_density) ctx_poly_density(c);
  auto sweep = [c]() {
    const int G = (int)c->groups.size();
    for (int g0 = 0; g0 < G;) {
      int g1 = g0;
      while (g1 < G && c->groups[g1].phase == c->groups[g0].phase) g1++;
      CK(cudaEventRecord(c->ev_fork, c->st));
      for (int g = g0; g < g1; g++) {
        CK(cudaStreamWaitEvent(c->side[g], c->ev_fork, 0));
        mix_group_sweep(c, g, c->side[g]);
        CK(cudaEventRecord(c->ev_join[g], c->side[g]));
        CK(cudaStreamWaitEvent(c->st, c->ev_join[g], 0));
      }
      g0 = g1;
    }
  };
  sweep();  // untimed
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, c->st));
  for (int r = 0; r < reps; r++) sweep();
  CK(cudaEventRecord(e1, c->st));
  CK(cudaEventSynchronize(e1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  check_device_error(c);
  double b = 0.0;
  for (auto &I : c->inst) b += mix_sweep_bytes(I);
  *ms = t / reps;
  *bytes = b;
  c->dirty_density = 1;
}

// Isolated timing of the two kernels of one propagator step (step 3(N-1)/4,
// a paired step) with their algorithmic bytes.
void ctx_profile_step(scft_ctx *c, int reps, double *ms_plane, double *bytes_plane, double *ms_col,
                      double *bytes_col) {
  if (c->dirty_density) ctx_poly_density(c);
  const int s = std::max(1, 3 * (c->nmax - 1) / 4);
  cudaEvent_t e0, e1, e2;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreate(&e2));
  CK(cudaEventRecord(e0, c->st));
  // the mixed form's passes one launch per kernel class (a run of the job
  // order with one class), as a single sweep group would launch them
  std::vector<scft_ctx::SweepGroup> runs;
  if (c->mixed) {
    const int n = (int)c->inst.size();
    for (int a = 0; a < n;) {
      int b = a + 1;
      while (b < n && (c->fast64.empty() || (c->fast64[b] == c->fast64[a] && c->fast96[b] == c->fast96[a] &&
                                             c->fast48[b] == c->fast48[a])))
        b++;
      scft_ctx::SweepGroup gr;
      gr.inst_begin = a;
      gr.inst_end = b;
      gr.pj_begin = a ? c->inst_pj_end[a - 1] : 0;
      gr.pj_end = c->inst_pj_end[b - 1];
      gr.cj_begin = a ? c->inst_cj_end[a - 1] : 0;
      gr.cj_end = c->inst_cj_end[b - 1];
      gr.phase = 0;
      gr.fast = c->fast64.empty() ? 0 : c->fast64[a];
      gr.fast96 = c->fast96.empty() ? 0 : c->fast96[a];
      gr.fast48 = c->fast48.empty() ? 0 : c->fast48[a];
      runs.push_back(gr);
      a = b;
    }
  }
  for (int r = 0; r < reps; r++) {
    if (c->mixed)
      for (auto &gr : runs) mix_group_step_pass(c, gr, s, false, c->st);
    else
      LK(launch_prop_plane_f64(c->shp_prop, c->d_prop_pj, c->prop_pj_count[s], c->d_pi, c->d_geoms, c->d_tw64, s,
                               c->st));
  }
  CK(cudaEventRecord(e1, c->st));
  for (int r = 0; r < reps; r++) {
    if (c->mixed)
      for (auto &gr : runs) mix_group_step_pass(c, gr, s, true, c->st);
    else
      LK(launch_col_fft<double>(c->shp_col, c->d_prop_cj, c->prop_cj_count[s], c->d_geoms, c->d_tw64, 2, 1,
                                c->st));
  }
  CK(cudaEventRecord(e2, c->st));
  CK(cudaEventSynchronize(e2));
  float a = 0.f, b = 0.f;
  CK(cudaEventElapsedTime(&a, e0, e1));
  CK(cudaEventElapsedTime(&b, e1, e2));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  double bp = 0.0, bc = 0.0;
  for (auto &I : c->inst) {
    if (I.N <= s) continue;
    if (I.mixed) {
      // plane: read z, E (8 B each), stored pair (8 B), write z (8 B), RMW of
      // the FP32 accumulators A and B (2 x 8 B); column: read + write z, plus
      // the h table in the generic pass (the 64-point pass forms h on the fly)
      bp += I.M * (4.0 * sizeof(float2) + 4.0 * sizeof(float));
      bc += I.M * 2.0 * sizeof(float2);  // (the generic z pass also reads its h table, 4 B per point)
    } else {
      const double props = I.single ? 1.0 : 2.0;
      bp += props * I.M * 6.0 * sizeof(double2);
      bc += props * I.M * (2.0 * sizeof(double2) + sizeof(double));
    }
  }
  *ms_plane = a / reps;
  *ms_col = b / reps;
  *bytes_plane = bp;
  *bytes_col = bc;
  c->dirty_density = 1;
}

// calc_H (code/calc_h.cpp:9-64); out per instance: Re H, Im H, Re Qd, Im Qd, Re Qga
static int h_collect(scft_ctx *c, double *out);
static int h_reduce(scft_ctx *c, double *out, const double2 *hp, const double2 *sc, const std::vector<int> *rows);

int ctx_calc_H(scft_ctx *c, double *out) {
  NvtxRange nvtx_range("scft_calc_H");
  if (c->dirty_density) ctx_poly_density(c);
  const int n = (int)c->inst.size();
  if (c->mixed)
    CK(launch_mix_h_partials(c->d_fi, n, c->hblocks, c->d_hpart, c->st));
  else
    CK(launch_h_partials(c->d_fi, n, c->hblocks, c->d_hpart, c->st));
  return h_collect(c, out);
}

// calc_H's host part: the partial sums and scalars of every instance,
// copied after the work queued so far, reduced per instance into out.
static int h_collect(scft_ctx *c, double *out) {
  const int n = (int)c->inst.size();
  std::vector<double2> hp((size_t)n * 4 * c->hblocks);
  CK(cudaMemcpyAsync(hp.data(), c->d_hpart, sizeof(double2) * hp.size(), cudaMemcpyDeviceToHost, c->st));
  std::vector<double2> sc((size_t)n * kNumScalars);
  for (int k = 0; k < n; k++)
    CK(cudaMemcpyAsync(&sc[(size_t)k * kNumScalars], c->inst[k].scal, sizeof(double2) * kNumScalars,
                       cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return h_reduce(c, out, hp.data(), sc.data(), nullptr);
}

// calc_H's reduction: the partial sums hp (instance k's at row (*rows)[k],
// or row k) and the scalars sc (kNumScalars per instance, instance order)
// into out, 5 per instance.
static int h_reduce(scft_ctx *c, double *out, const double2 *hp, const double2 *sc, const std::vector<int> *rows) {
  const int n = (int)c->inst.size();
  int status = SCFT_OK;
  for (int k = 0; k < n; k++) {
    const Instance &I = c->inst[k];
    cd part[4];
    for (int j = 0; j < 4; j++) {
      cd s(0.0, 0.0);
      for (int b = 0; b < c->hblocks; b++) {
        const double2 v = hp[((size_t)(rows ? (*rows)[k] : k) * 4 + j) * c->hblocks + b];
        s += cd(v.x, v.y);
      }
      if (I.mixed)
        s *= I.info.V;  // Parseval: int f g = V sum_k f(k) g(-k)
      else
        for (int d = 0; d < 3; d++) s *= I.info.dx[d];
      part[j] = s;
    }
    if (I.cbc == 0.0) part[1] = 0.0;
    if (I.cac == 0.0) part[2] = 0.0;
    if (I.cab == 0.0) part[3] = 0.0;
    cd H = part[0] + part[1] + part[2] + part[3];
    const cd Qd(sc[(size_t)k * kNumScalars + kQd].x, sc[(size_t)k * kNumScalars + kQd].y);
    const cd Qga(sc[(size_t)k * kNumScalars + kQga].x, sc[(size_t)k * kNumScalars + kQga].y);
    if (I.info.nD > 0.0) H += -I.info.nD * std::log(Qd);
    if (I.p.n_exp_nr > 0 && I.graft) H += -double(I.p.n_exp_nr) * I.info.ng_per_np * Qga.real();
    out[5 * k + 0] = H.real();
    out[5 * k + 1] = H.imag();
    out[5 * k + 2] = Qd.real();
    out[5 * k + 3] = Qd.imag();
    out[5 * k + 4] = Qga.real();
    if (H != H) status = SCFT_ERR_NAN;
    // the reference exits once 5 points have Re q_g[Ng-1] <= 0 (code/grafted_nanoparticle.cpp:82-107)
    if (I.graft && sc[(size_t)k * kNumScalars + kQg].x >= 5.0 && status == SCFT_OK) status = SCFT_ERR_QNONPOS;
  }
  return status;
}

// The fields an update changes: w+ and the pair of every nonzero chi (ab:
// w[1], w[2]; bc: w[3], w[4]; ac: w[5], w[6]).  The reference updates a pair
// only for nonzero chi (code/1s_update.cpp:42,168,339) and initialises the
// others to zero (code/initialize.cpp:430-431); the mixed form holds them at
// zero (its update assembles w_A, w_B without them).
static void fields_in_use(const Instance &I, bool active[7]) {
  const bool on[7] = {true, I.cab != 0.0, I.cab != 0.0, I.cbc != 0.0, I.cbc != 0.0, I.cac != 0.0, I.cac != 0.0};
  for (int f = 0; f < 7; f++) active[f] = on[f];
}

// scft_set_fields of one instance or of all: one copy per instance (the seven
// fields are contiguous on both sides), one realness check launch over the
// instances, one synchronisation (the caller may reuse its buffers, the check
// result is on the host), then one batched forward transform of the nonzero
// fields (zero fields are transforms of themselves), left to run on the
// stream.  Mixed-form instances set the pairs whose chi is 0 to zero.
// SCFT_ERR_COMPLEX leaves the instance's fields undefined until its next
// successful call.

static void set_fields_ks(scft_ctx *c, const std::vector<int> &ks, const double *const *w) {
  const int n = (int)c->inst.size();
  c->dirty_density = 1;
  bool mixed = false;
  for (size_t q = 0; q < ks.size(); q++) {
    Instance &I = c->inst[ks[q]];
    CK(cudaMemcpyAsync(I.w[0], w[q], sizeof(double2) * 7 * (size_t)I.M, cudaMemcpyHostToDevice, c->st));
    if (I.mixed) {
      bool active[7];
      fields_in_use(I, active);
      for (int f = 1; f < 7; f += 2)
        if (!active[f]) CK(cudaMemsetAsync(I.w[f], 0, sizeof(double2) * 2 * (size_t)I.M, c->st));
    }
    mixed = mixed || I.mixed;
  }
  if (!mixed) {
    CK(cudaStreamSynchronize(c->st));
    return;
  }
  if (!c->h_skip || !c->h_jobs || !c->d_realout || !c->h_pin)
    throw ScftError(SCFT_ERR_CUDA, "scft_set_fields: staging buffers missing");
  // check only the instances in ks
  for (int k = 0; k < n; k++) c->h_skip[k] = 1;
  for (int k : ks) c->h_skip[k] = 0;
  CK(cudaMemcpyAsync(c->d_skip, c->h_skip, sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
  k_real_check_all<<<dim3(kCheckBlocks, n), 256, 0, c->st>>>(c->d_fi, c->d_skip, c->d_realout);
  CK(cudaGetLastError());
  for (int k : ks)
    CK(cudaMemcpyAsync(c->h_pin + kCheckStride * (size_t)k, c->d_realout + kCheckStride * (size_t)k,
                       sizeof(double) * 9 * kCheckBlocks,
                       cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  std::vector<PlaneJob> pj;
  std::vector<ColJob> cj;
  std::string bad;
  for (int k : ks) {
    Instance &I = c->inst[k];
    double m[9] = {};
    for (int b = 0; b < kCheckBlocks; b++)
      for (int q = 0; q < 9; q++) m[q] = std::max(m[q], c->h_pin[kCheckStride * (size_t)k + 9 * b + q]);
    if (m[0] > 1e-12 * std::max(1.0, m[1])) {
      if (bad.empty()) bad = std::to_string(k);
      continue;
    }
    const DevGeom &g = c->geoms[I.geom];
    for (int f = 0; f < 7; f++) {
      if (m[2 + f] == 0.0) continue;
      for (int z = 0; z < g.nz; z++) pj.push_back(PlaneJob{I.w[f], I.geom, z});
      for (int y = 0; y < g.ny; y++)
        for (int x0 = 0; x0 < g.nx; x0 += g.tx) cj.push_back(ColJob{I.w[f], nullptr, I.geom, x0, y});
    }
  }
  if (!pj.empty()) {
    // the job lists go through pinned staging (no synchronisation needed:
    // the next call's writes to the staging come after a synchronisation)
    memcpy(c->h_jobs, pj.data(), sizeof(PlaneJob) * pj.size());
    memcpy(reinterpret_cast<char *>(c->h_jobs) + c->jobs_cap / 2, cj.data(), sizeof(ColJob) * cj.size());
    CK(cudaMemcpyAsync(c->d_jobs, c->h_jobs, sizeof(PlaneJob) * pj.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(reinterpret_cast<char *>(c->d_jobs) + c->jobs_cap / 2,
                       reinterpret_cast<char *>(c->h_jobs) + c->jobs_cap / 2, sizeof(ColJob) * cj.size(),
                       cudaMemcpyHostToDevice, c->st));
    CK(launch_plane_fft<double>(c->shp_plane, reinterpret_cast<PlaneJob *>(c->d_jobs), (int)pj.size(), c->d_geoms,
                                c->d_tw64, -1, 0, c->st));
    CK(launch_col_fft<double>(c->shp_col,
                              reinterpret_cast<ColJob *>(reinterpret_cast<char *>(c->d_jobs) + c->jobs_cap / 2),
                              (int)cj.size(), c->d_geoms, c->d_tw64, 0, 1, c->st));
  }
  if (!bad.empty())
    throw ScftError(SCFT_ERR_COMPLEX, "instance " + bad +
                                          ": mixed precision needs real w_A, w_B (and w_G with grafts): the "
                                          "mean-field phase convention");
}

void ctx_set_fields(scft_ctx *c, int k, const double *w) { set_fields_ks(c, {k}, &w); }

int ctx_calc_H(scft_ctx *c, double *out);
void ctx_update(scft_ctx *c, int n_iter);
void ctx_set_fields_all(scft_ctx *c, const double *const *w);
void ctx_get_fields(scft_ctx *c, int k, double *w);

// Per-group FP64 transform jobs, in job order, rebuilt when the groups
// change: the forward transforms of the uploaded fields (those an update
// changes) and, per round of three such fields, the inverse transforms of
// the updated fields to download (the q-th field of an instance goes
// through rho[q % 3] in round q / 3).
static void build_step_jobs(scft_ctx *c) {
  std::vector<int> sig;
  for (auto &gr : c->groups) {
    sig.push_back(gr.inst_begin);
    sig.push_back(gr.inst_end);
    sig.push_back(gr.phase);
  }
  if (sig == c->step_groups_sig && c->step_pj.size() == c->groups.size()) return;
  c->step_pj.clear();
  c->step_cj.clear();
  c->step_npj.clear();
  c->step_ncj.clear();
  c->out_pj.clear();
  c->out_cj.clear();
  c->out_npj.clear();
  c->out_ncj.clear();
  auto add = [&](std::vector<PlaneJob> &pj, std::vector<ColJob> &cj, const Instance &I, double2 *a) {
    const DevGeom &g = c->geoms[I.geom];
    for (int z = 0; z < g.nz; z++) pj.push_back(PlaneJob{a, I.geom, z});
    for (int y = 0; y < g.ny; y++)
      for (int x0 = 0; x0 < g.nx; x0 += g.tx) cj.push_back(ColJob{a, nullptr, I.geom, x0, y});
  };
  for (auto &gr : c->groups) {
    std::vector<PlaneJob> pj;
    std::vector<ColJob> cj;
    std::vector<PlaneJob> opj[3];
    std::vector<ColJob> ocj[3];
    for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) {
      const Instance &I = c->inst[c->job_order[oi]];
      bool active[7];
      fields_in_use(I, active);
      for (int f = 0, q = 0; f < 7; f++) {
        if (!active[f]) continue;
        add(pj, cj, I, I.w[f]);
        add(opj[q / 3], ocj[q / 3], I, I.rho[q % 3]);
        q++;
      }
    }
    c->step_pj.push_back(dupload(c, pj));
    c->step_cj.push_back(dupload(c, cj));
    c->step_npj.push_back((int)pj.size());
    c->step_ncj.push_back((int)cj.size());
    for (int r = 0; r < 3; r++) {
      c->out_pj.push_back(opj[r].empty() ? nullptr : dupload(c, opj[r]));
      c->out_cj.push_back(ocj[r].empty() ? nullptr : dupload(c, ocj[r]));
      c->out_npj.push_back((int)opj[r].size());
      c->out_ncj.push_back((int)ocj[r].size());
    }
  }
  c->step_groups_sig = sig;
}

// The graph body of scft_step_fields and scft_iterate_fields (mixed form, no
// grafted chains): per sweep group on its side stream, the upload of its
// instances' fields (w+ and the pairs of nonzero chi; the others are set to
// zero), their realness check (results copied to pinned host memory, read
// after the call's synchronisation), their FP64 forward transform, then
//   step_fields (iterate false): the density build and n_iter updates;
//   iterate_fields: the density build, calc_H's partial sums of the uploaded
//     fields, the k-space half of one update (no density build after it)
//     and, with w_out, the download of the updated fields in use (inverse
//     FP64 transforms with the instances' rho[0..2] as scratch, three
//     fields a round).
// One group's copies run beside another group's compute.
static void step_body(scft_ctx *c, const double *const *w, int n_iter, bool iterate, double *const *w_out) {
  cudaStream_t st = c->st;
  const int G = (int)c->groups.size();
  CK(cudaEventRecord(c->ev_fork, st));
  for (int g = 0; g < G; g++) {
    const scft_ctx::SweepGroup &gr = c->groups[g];
    cudaStream_t sg = c->side[g];
    CK(cudaStreamWaitEvent(sg, c->ev_fork, 0));
    // the groups' uploads run one after another, so that the first group
    // computes while the others' fields are still coming in
    if (g > 0) CK(cudaStreamWaitEvent(sg, c->ev_up[g - 1], 0));
    const int cnt = gr.inst_end - gr.inst_begin;
    // the fields an update changes come from the host (one copy per run of
    // adjacent ones); the pairs whose chi is 0 are held at zero in the mixed
    // form (its update treats them as zero) and are not read
    for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) {
      const int k = c->job_order[oi];
      Instance &I = c->inst[k];
      bool active[7];
      fields_in_use(I, active);
      const size_t fb = sizeof(double2) * (size_t)I.M;  // bytes per field
      for (int f = 0; f < 7;) {
        int f1 = f + 1;
        while (f1 < 7 && active[f1] == active[f]) f1++;
        if (active[f])
          CK(cudaMemcpyAsync(I.w[f], w[k] + 2 * (size_t)I.M * f, fb * (f1 - f), cudaMemcpyHostToDevice, sg));
        else
          CK(cudaMemsetAsync(I.w[f], 0, fb * (f1 - f), sg));
        f = f1;
      }
    }
    CK(cudaEventRecord(c->ev_up[g], sg));
    k_real_check_all<<<dim3(kCheckBlocks, cnt), 256, 0, sg>>>(c->d_fi_ord + gr.inst_begin, nullptr,
                                                              c->d_realout + kCheckStride * (size_t)gr.inst_begin);
    CK(cudaGetLastError());
    c->launches++;
    CK(cudaMemcpyAsync(c->h_pin + kCheckStride * (size_t)gr.inst_begin, c->d_realout + kCheckStride * (size_t)gr.inst_begin,
                       sizeof(double) * kCheckStride * (size_t)cnt, cudaMemcpyDeviceToHost, sg));
    if (c->step_npj[g] > 0) {
      LK(launch_plane_fft<double>(c->shp_plane, c->step_pj[g], c->step_npj[g], c->d_geoms, c->d_tw64, -1, 0, sg));
      LK(launch_col_fft<double>(c->shp_col, c->step_cj[g], c->step_ncj[g], c->d_geoms, c->d_tw64, 0, 1, sg));
    }
    mix_group_chain(c, g, sg, false);
    if (!iterate) {
      for (int it = 0; it < n_iter; it++) mix_group_chain(c, g, sg, true);
    } else {
      // H needs the fields (Parseval sums) and Qd only: its partial sums are
      // taken before the update changes the fields
      const size_t hrow = (size_t)4 * c->hblocks;
      LK(launch_mix_h_partials(c->d_fi_ord + gr.inst_begin, cnt, c->hblocks, c->d_hpart + hrow * gr.inst_begin, sg));
      CK(cudaMemcpyAsync(c->h_hsum + hrow * gr.inst_begin, c->d_hpart + hrow * gr.inst_begin,
                         sizeof(double2) * hrow * cnt, cudaMemcpyDeviceToHost, sg));
      for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) {
        const int k = c->job_order[oi];
        CK(cudaMemcpyAsync(c->h_hsum + hrow * c->inst.size() + (size_t)k * kNumScalars, c->inst[k].scal,
                           sizeof(double2) * kNumScalars, cudaMemcpyDeviceToHost, sg));
      }
      mix_group_kspace_update(c, g, sg);
      for (int r = 0; w_out && r < 3; r++) {
        const int jr = 3 * g + r;
        if (!c->out_npj[jr]) continue;
        auto each = [&](bool to_host) {
          for (int oi = gr.inst_begin; oi < gr.inst_end; oi++) {
            const int k = c->job_order[oi];
            Instance &I = c->inst[k];
            bool active[7];
            fields_in_use(I, active);
            const size_t fb = sizeof(double2) * (size_t)I.M;
            for (int f = 0, q = 0; f < 7; f++) {
              if (!active[f]) continue;
              if (q / 3 == r) {
                if (to_host)
                  CK(cudaMemcpyAsync(w_out[k] + 2 * (size_t)I.M * f, I.rho[q % 3], fb, cudaMemcpyDeviceToHost, sg));
                else
                  CK(cudaMemcpyAsync(I.rho[q % 3], I.w[f], fb, cudaMemcpyDeviceToDevice, sg));
              }
              q++;
            }
          }
        };
        each(false);
        LK(launch_col_fft<double>(c->shp_col, c->out_cj[jr], c->out_ncj[jr], c->d_geoms, c->d_tw64, 1, 0, sg));
        LK(launch_plane_fft<double>(c->shp_plane, c->out_pj[jr], c->out_npj[jr], c->d_geoms, c->d_tw64, +1, 0, sg));
        each(true);
      }
    }
    CK(cudaEventRecord(c->ev_join[g], sg));
    CK(cudaStreamWaitEvent(st, c->ev_join[g], 0));
  }
}

// Whether a host-field call runs as a captured graph: mixed-form batches
// without grafted chains or complex Langevin, with page-locked (pinned or
// registered) host buffers; a captured copy needs page-locked memory.
static bool step_graph_ok(scft_ctx *c, const double *const *w, const double *const *w_out) {
  bool cl = false;
  for (auto &I : c->inst) cl = cl || I.p.do_cl;
  if (!c->mixed || c->ngmax > 0 || cl || c->groups.empty()) return false;
  auto locked = [](const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.type == cudaMemoryTypeHost;
  };
  const int n = (int)c->inst.size();
  for (int k = 0; k < n; k++)
    if (!locked(w[k]) || (w_out && !locked(w_out[k]))) return false;
  return true;
}

// Runs the host-field graph of (call, host pointers, n_iter), capturing it
// first when the key differs from the last one's.  A first run ever is eager
// (kernel attributes get set), without the download, so that w stays the
// input of the captured run even when w_out aliases it.
static void run_step_graph(scft_ctx *c, const double *const *w, int n_iter, bool iterate, double *const *w_out) {
  if (!c->h_pin || !c->d_realout) throw ScftError(SCFT_ERR_CUDA, "host-field step: staging buffers missing");
  const int n = (int)c->inst.size();
  build_step_jobs(c);
  // pinned memory for the H sums the graph copies out
  if (!c->h_hsum)
    CK(cudaMallocHost(&c->h_hsum, sizeof(double2) * (size_t)n * (4 * (size_t)c->hblocks + kNumScalars)));
  std::vector<const void *> key(w, w + n);
  key.push_back(iterate ? c : nullptr);
  for (int k = 0; k < n; k++) key.push_back(w_out ? w_out[k] : nullptr);
  if (c->g_step && (key != c->step_ptrs || n_iter != c->step_iters)) {
    CK(cudaGraphExecDestroy(c->g_step));
    c->g_step = nullptr;
  }
  if (!c->g_step) {
    if (!c->update_runs && !c->density_runs) {
      step_body(c, w, n_iter, iterate, nullptr);
      CK(cudaStreamSynchronize(c->st));
      c->density_runs++;
      c->update_runs++;
    }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    try {
      step_body(c, w, n_iter, iterate, w_out);
    } catch (...) {
      cudaGraph_t g2;
      cudaStreamEndCapture(c->st, &g2);
      throw;
    }
    CK(cudaStreamEndCapture(c->st, &graph));
    CK(cudaGraphInstantiate(&c->g_step, graph, 0));
    cudaGraphDestroy(graph);
    c->step_ptrs = key;
    c->step_iters = n_iter;
  }
  CK(cudaGraphLaunch(c->g_step, c->st));
}

// The realness check of the uploaded fields, read after the call's
// synchronisation (maxima per check block in h_pin, job order).
static void check_step_realness(scft_ctx *c) {
  const int n = (int)c->inst.size();
  std::string bad;
  for (int oi = 0; oi < n; oi++) {
    double m[9] = {};
    for (int b = 0; b < kCheckBlocks; b++)
      for (int q = 0; q < 9; q++) m[q] = std::max(m[q], c->h_pin[kCheckStride * (size_t)oi + 9 * b + q]);
    if (m[0] > 1e-12 * std::max(1.0, m[1]) && bad.empty()) bad = std::to_string(c->job_order[oi]);
  }
  if (!bad.empty()) {
    c->dirty_density = 1;
    throw ScftError(SCFT_ERR_COMPLEX, "instance " + bad +
                                          ": mixed precision needs real w_A, w_B: the mean-field phase convention "
                                          "(the results of this call are invalid)");
  }
}

// scft_step_fields: fields of every instance from host memory (w[inst], 7 x M
// complex, the scft_set_fields layout; pinned memory lets the uploads overlap
// compute), the density build of those fields, n_iter updates, H into out
// (5 per instance, as scft_calc_H) -- one call and one synchronisation.
// Mixed-form batches without grafted chains or complex Langevin run as one
// captured graph (re-captured when the host pointers or n_iter change);
// everything else runs scft_set_fields_all, scft_update_1s and scft_calc_H.
int ctx_step_fields(scft_ctx *c, const double *const *w, int n_iter, double *out) {
  NvtxRange nvtx_range("scft_step_fields");
  if (!step_graph_ok(c, w, nullptr)) {
    ctx_set_fields_all(c, w);
    ctx_update(c, n_iter);
    return ctx_calc_H(c, out);
  }
  run_step_graph(c, w, n_iter, false, nullptr);
  c->dirty_density = 0;
  int status = ctx_calc_H(c, out);  // queues H and synchronises
  check_device_error(c);
  check_step_realness(c);
  return status;
}

// scft_iterate_fields: one iteration of the reference's main loop per
// instance, from and to host memory, in the order calc_poly_density, calc_H,
// update: the fields of every instance from w[inst], their density build, H
// of those fields into out, one field update; with w_out, the updated fields
// into w_out[inst] (the mixed form writes the fields the update changes;
// w_out may be w).
// The densities are then those of the uploaded fields (stale: the next call
// that needs the updated fields' densities rebuilds them).  Mixed-form
// batches without grafted chains or complex Langevin, with page-locked
// buffers, run as one captured graph (one density build per iteration);
// everything else runs scft_set_fields_all, scft_calc_H, scft_update_1s and
// scft_get_fields.
int ctx_iterate_fields(scft_ctx *c, const double *const *w, double *const *w_out, double *out) {
  NvtxRange nvtx_range("scft_iterate_fields");
  const int n = (int)c->inst.size();
  if (!step_graph_ok(c, w, w_out)) {
    ctx_set_fields_all(c, w);
    const int status = ctx_calc_H(c, out);
    ctx_update(c, 1);
    if (w_out)
      for (int k = 0; k < n; k++) {
        const Instance &I = c->inst[k];
        const size_t per = 2 * (size_t)I.M;  // doubles per field
        std::vector<double> all(7 * per);
        ctx_get_fields(c, k, all.data());
        bool active[7];
        fields_in_use(I, active);
        for (int f = 0; f < 7; f++)
          if (active[f] || !I.mixed) std::copy(all.begin() + f * per, all.begin() + (f + 1) * per, w_out[k] + f * per);
      }
    return status;
  }
  run_step_graph(c, w, 1, true, w_out);
  c->dirty_density = 1;
  std::vector<int> rows(n);
  for (int oi = 0; oi < n; oi++) rows[c->job_order[oi]] = oi;
  CK(cudaStreamSynchronize(c->st));
  const double2 *hp = c->h_hsum;  // the graph copied the H sums here
  const int status = h_reduce(c, out, hp, hp + (size_t)4 * c->hblocks * n, &rows);
  check_device_error(c);
  check_step_realness(c);
  return status;
}

void ctx_set_fields_all(scft_ctx *c, const double *const *w) {
  NvtxRange nvtx_range("scft_set_fields_all");
  std::vector<int> ks(c->inst.size());
  for (size_t k = 0; k < ks.size(); k++) ks[k] = (int)k;
  set_fields_ks(c, ks, w);
}

void ctx_get_fields(scft_ctx *c, int k, double *w) {
  Instance &I = c->inst[k];
  if (I.mixed) {
    // fields are held as transforms; return them in real space
    double2 *tmp = I.rho[2];
    for (int f = 0; f < 7; f++) {
      CK(cudaMemcpyAsync(tmp, I.w[f], sizeof(double2) * I.M, cudaMemcpyDeviceToDevice, c->st));
      fft3d_arrays(c, I, {tmp}, +1);
      CK(cudaMemcpyAsync(w + (size_t)f * 2 * I.M, tmp, sizeof(double2) * I.M, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
    }
    return;
  }
  for (int f = 0; f < 7; f++)
    CK(cudaMemcpyAsync(w + (size_t)f * 2 * I.M, I.w[f], sizeof(double2) * I.M, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
}

void ctx_get_density(scft_ctx *c, int k, double *ra, double *rb, double *rg) {
  if (c->dirty_density) ctx_poly_density(c);
  Instance &I = c->inst[k];
  if (I.mixed) {
    // FP64 densities from the accumulators (the sweep state is not touched)
    CK(launch_mix_rho_pack(c->d_fi, (int)c->inst.size(), c->eblocks, 1, c->st));
    if (!I.graft) CK(cudaMemsetAsync(I.rho[2], 0, sizeof(double2) * I.M, c->st));
  }
  double *outs[3] = {ra, rb, rg};
  for (int f = 0; f < 3; f++)
    if (outs[f]) CK(cudaMemcpyAsync(outs[f], I.rho[f], sizeof(double2) * I.M, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
}

void ctx_get_smeared(scft_ctx *c, int k, double *a, double *b, double *g) {
  if (c->dirty_density) ctx_poly_density(c);
  Instance &I = c->inst[k];
  if (I.mixed) {
    // z32 holds smwa + i smwb minus their means (real space, FP32); the means
    // are in scal[kSmean]
    std::vector<float2> h(I.M);
    std::vector<double2> sc(kNumScalars);
    CK(cudaMemcpyAsync(h.data(), I.z32, sizeof(float2) * I.M, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(sc.data(), I.scal, sizeof(double2) * kNumScalars, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    const double2 m = sc[kSmean];
    for (long long i = 0; i < I.M; i++) {
      if (a) { a[2 * i] = m.x + h[i].x; a[2 * i + 1] = 0.0; }
      if (b) { b[2 * i] = m.y + h[i].y; b[2 * i + 1] = 0.0; }
      if (g) { g[2 * i] = 0.0; g[2 * i + 1] = 0.0; }
    }
    if (g && I.graft) CK(cudaMemcpy(g, I.sm[2], sizeof(double2) * I.M, cudaMemcpyDeviceToHost));
    return;
  }
  double *outs[3] = {a, b, g};
  for (int f = 0; f < 3; f++)
    if (outs[f]) CK(cudaMemcpyAsync(outs[f], I.sm[f], sizeof(double2) * I.M, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
}

void ctx_fft3d(scft_ctx *c, int k, double *data, int count, int sign) {
  Instance &I = c->inst[k];
  double2 *buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(double2) * I.M * count));
  std::vector<double2 *> arrs;
  try {
    CK(cudaMemcpyAsync(buf, data, sizeof(double2) * I.M * count, cudaMemcpyHostToDevice, c->st));
    for (int j = 0; j < count; j++) arrs.push_back(buf + (size_t)j * I.M);
    fft3d_arrays(c, I, arrs, sign);
    CK(cudaMemcpyAsync(data, buf, sizeof(double2) * I.M * count, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  } catch (...) {
    cudaFree(buf);
    throw;
  }
  cudaFree(buf);
}

// diblock_discrete + integrate_diblock_discrete on given smeared fields.
void ctx_diblock_density(scft_ctx *c, int k, const double *smwa, const double *smwb, double *ra, double *rb,
                         double *Q) {
  Instance &I = c->inst[k];
  if (I.mixed) throw ScftError(SCFT_ERR_UNSUPPORTED, "scft_diblock_density runs the FP64 method only");
  CK(cudaMemcpyAsync(I.sm[0], smwa, sizeof(double2) * I.M, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(I.sm[1], smwb, sizeof(double2) * I.M, cudaMemcpyHostToDevice, c->st));
  const int n = (int)c->inst.size();
  cudaStream_t st = c->st;
  CK(launch_boltzmann(c->d_fi, n, c->eblocks, st));
  for (auto &J : c->inst)
    for (int q = 0; q < 2; q++)
      for (int s = 0; s < 2; s++) CK(cudaMemsetAsync(J.acc[q][s], 0, sizeof(double2) * J.M, st));
  CK(launch_prop_plane_f64(c->shp_prop, c->d_prop_pj, c->prop_pj_count[0], c->d_pi, c->d_geoms, c->d_tw64, 0, st));
  for (int s = 1; s < c->nmax; s++) {
    CK(launch_col_fft<double>(c->shp_col, c->d_prop_cj, c->prop_cj_count[s], c->d_geoms, c->d_tw64, 2, 1, st));
    CK(launch_prop_plane_f64(c->shp_prop, c->d_prop_pj, c->prop_pj_count[s], c->d_pi, c->d_geoms, c->d_tw64, s,
                             st));
  }
  CK(launch_q_finalize(c->d_fi, n, st));
  CK(launch_density(c->d_fi, n, c->eblocks, st));
  if (ra) CK(cudaMemcpyAsync(ra, I.rho[0], sizeof(double2) * I.M, cudaMemcpyDeviceToHost, st));
  if (rb) CK(cudaMemcpyAsync(rb, I.rho[1], sizeof(double2) * I.M, cudaMemcpyDeviceToHost, st));
  if (Q) CK(cudaMemcpyAsync(Q, I.scal + kQd, sizeof(double2), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  c->dirty_density = 1;
}

int error_code(const std::exception &e) {
  const ScftError *se = dynamic_cast<const ScftError *>(&e);
  return se ? se->code : SCFT_ERR_CUDA;
}

}  // namespace scft

namespace scft {
// dH/d(plate rotation about z) and dH/d(plate centre) at the current fields
// (kernels_grad.cu): out[8*inst + 4*j + {0, 1, 2, 3}] for plate j.
// Grafted plates: adds d(-n_exp_nr ng_per_np Re Qga)/dg_k of every plate j to
// out[4 j + k] at the current fields (kernels_grad.cu gives the terms).
// Device temporaries (about 12 arrays of the grid) are allocated here and
// freed before returning.
static void graft_map_derivative(scft_ctx *c, Instance &I, const GradArgs &g, double *out) {
  const scft_params &p = I.p;
  const long long M = I.M;
  const int nb = 128;
  const double dV = I.info.dx[0] * I.info.dx[1] * I.info.dx[2];
  std::vector<void *> tmp;
  auto get = [&](size_t bytes) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw ScftError(SCFT_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    tmp.push_back(q);
    return q;
  };
  auto sums = [&](double *part) {
    std::vector<double> h(4 * nb);
    CK(cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    double s4[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nb; b++)
      for (int k = 0; k < 4; k++) s4[k] += h[4 * b + k];
    return std::array<cd, 2>{cd(s4[0], s4[1]) * dV, cd(s4[2], s4[3]) * dV};
  };
  try {
    const size_t ab = sizeof(double2) * (size_t)M;
    double2 *L = static_cast<double2 *>(get(ab));
    double *part = static_cast<double *>(get(sizeof(double) * 4 * nb));
    if (I.mixed) {
      int K = 0;
      CK(cudaMemcpyAsync(&K, I.gK + (p.Ng - 1), sizeof(int), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      CK(launch_graft_log(L, I.grafts, nullptr, I.ghist32 + (size_t)(p.Ng - 1) * M, K, M, c->st));
    } else {
      CK(launch_graft_log(L, I.grafts, static_cast<const double2 *>(I.ghist) + (size_t)(p.Ng - 1) * M, nullptr, 0,
                          M, c->st));
    }
    const double len = p.L_nr * 1.05, rad = p.R_nr * 1.05;  // the graft map's enlarged plates
    const int np = p.n_exp_nr;
    std::vector<std::array<double2 *, 3>> gr(np);
    cd S(0.0, 0.0);
    for (int j = 0; j < np; j++) {
      double2 *pd = static_cast<double2 *>(get(ab));
      k_plate<<<1024, 256, 0, c->st>>>(pd, plate_args_of(I, j, len, rad), 0);
      CK(cudaGetLastError());
      for (int d = 0; d < 3; d++) {
        gr[j][d] = static_cast<double2 *>(get(ab));
        CK(cudaMemcpyAsync(gr[j][d], pd, ab, cudaMemcpyDeviceToDevice, c->st));
        spectral_gradient(c, I, gr[j][d], d);
      }
      CK(launch_graft_dmap(gr[j].data(), nullptr, L, M, part, nb, c->st));
      S += sums(part)[1];
    }
    std::vector<double2> sc(kNumScalars);
    CK(cudaMemcpyAsync(sc.data(), I.scal, sizeof(double2) * kNumScalars, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    const cd Qga(sc[kQga].x, sc[kQga].y);
    double2 *D = static_cast<double2 *>(get(ab));
    double2 *gd[3] = {static_cast<double2 *>(get(ab)), static_cast<double2 *>(get(ab)), static_cast<double2 *>(get(ab))};
    for (int j = 0; j < np; j++)
      for (int q = 0; q < 4; q++) {
        CK(launch_plate_deriv(D, g, j, q, len, rad, c->st));
        for (int d = 0; d < 3; d++) {
          CK(cudaMemcpyAsync(gd[d], D, ab, cudaMemcpyDeviceToDevice, c->st));
          spectral_gradient(c, I, gd[d], d);
        }
        CK(launch_graft_dmap(gr[j].data(), gd, L, M, part, nb, c->st));
        const auto I12 = sums(part);
        const cd dQ = (I12[0] - I12[1] * Qga) / S;
        out[4 * j + q] += -double(np) * I.info.ng_per_np * dQ.real();
      }
  } catch (...) {
    for (void *q : tmp) cudaFree(q);
    throw;
  }
  for (void *q : tmp) cudaFree(q);
}

int ctx_grad_geom(scft_ctx *c, double *out) {
  NvtxRange nvtx_range("scft_grad_geom");
  if (c->dirty_density) ctx_poly_density(c);
  const int n = (int)c->inst.size();
  const int blocks = 128;
  double *part = nullptr;
  CK(cudaMalloc(&part, sizeof(double) * blocks * 2 * kGradPerPlate));
  std::vector<double> hp(blocks * 2 * kGradPerPlate);
  std::vector<double2> sc(kNumScalars);
  int status = SCFT_OK;
  try {
    bool any_shell = false;
    for (auto &I : c->inst) any_shell = any_shell || (I.shellU != nullptr);
    if (c->mixed && any_shell)  // real-space FP64 rho_A of every instance
      CK(launch_mix_rho_pack(c->d_fi, n, c->eblocks, 1, c->st));
    for (int k = 0; k < n; k++) {
      Instance &I = c->inst[k];
      for (int j = 0; j < 8; j++) out[8 * k + j] = 0.0;
      const scft_params &p = I.p;
      if (p.n_exp_nr == 0) continue;
      const double2 *wpl = I.w[0];
      if (I.mixed) {  // fields are held as transforms
        CK(cudaMemcpyAsync(I.rho[2], I.w[0], sizeof(double2) * I.M, cudaMemcpyDeviceToDevice, c->st));
        fft3d_arrays(c, I, {I.rho[2]}, +1);
        wpl = I.rho[2];
      }
      GradArgs g;
      g.nx = p.Nx[0];
      g.ny = p.Nx[1];
      g.nz = p.Nx[2];
      g.nplates = p.n_exp_nr;
      for (int d = 0; d < 3; d++) {
        g.dx[d] = I.info.dx[d];
        g.L[d] = p.L[d];
      }
      for (int j = 0; j < p.n_exp_nr; j++) {
        double un = 0.0;
        for (int d = 0; d < 3; d++) un += p.orient[j][d] * p.orient[j][d];
        un = sqrt(un);
        for (int d = 0; d < 3; d++) {
          g.c[j][d] = p.center[j][d] * p.L[d];
          g.u[j][d] = p.orient[j][d] / un;
        }
      }
      g.len = p.L_nr;
      g.rad = p.R_nr;
      g.xi = p.xi_nr;
      g.shape = p.plate_shape;
      g.shell = I.shellU != nullptr;
      g.len_big = p.L_nr + 2.0 * p.shell_width;
      g.rad_big = p.R_nr + p.shell_width;
      CK(launch_geom_grad(g, wpl, I.rho[0], part, blocks, c->st));
      const int nv = g.nplates * kGradPerPlate;
      CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * blocks * nv, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(sc.data(), I.scal, sizeof(double2) * kNumScalars, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      const cd logQ = std::log(cd(sc[kQd].x, sc[kQd].y));
      const double dV = I.info.dx[0] * I.info.dx[1] * I.info.dx[2];
      for (int j = 0; j < g.nplates; j++)
        for (int q = 0; q < 4; q++) {
          double sv[kGradTerms] = {};
          for (int b = 0; b < blocks; b++)
            for (int t = 0; t < kGradTerms; t++) sv[t] += hp[(size_t)b * nv + j * kGradPerPlate + kGradTerms * q + t];
          // Re[ i rho0 dV sum(drho w+) ] + (rho0/N) dV sum(drho) Re log Qd
          const cd t = cd(0.0, p.rho0) * cd(sv[0], sv[1]) * dV + (p.rho0 / I.N) * dV * sv[2] * logQ;
          // shell: Lambda dV sum(rho_A d(rho_big - rho_p))
          const double ts = g.shell ? p.shell_lambda * dV * (sv[3] - sv[4]) : 0.0;
          out[8 * k + 4 * j + q] = t.real() + ts;
        }
      if (I.graft) graft_map_derivative(c, I, g, out + 8 * k);
    }
  } catch (...) {
    cudaFree(part);
    throw;
  }
  cudaFree(part);
  return status;
}

// Replaces nD of instance k (used by the homopolymer entry point, where the
// chain count nK is an argument).
void ctx_override_nD(scft_ctx *c, int k, double nD) {
  c->inst[k].info.nD = nD;
  CK(cudaMemcpyAsync(reinterpret_cast<char *>(c->d_fi + k) + offsetof(FieldInst, nD), &nD, sizeof(double),
                     cudaMemcpyHostToDevice, c->st));
  for (size_t oi = 0; c->d_fi_ord && oi < c->job_order.size(); oi++)
    if (c->job_order[oi] == k)
      CK(cudaMemcpyAsync(reinterpret_cast<char *>(c->d_fi_ord + oi) + offsetof(FieldInst, nD), &nD, sizeof(double),
                         cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
}
}  // namespace scft
