// capi.cu -- extern "C" entry points of libscft (declared in include/scft.h).
// Every entry point catches exceptions and turns them into a status code; the
// message is kept per host thread for scft_last_error().
#include <cstring>
#include <new>
#include <string>

#include "context.h"

namespace scft {
void ctx_create(scft_ctx *c, const scft_params *params, int n_inst);
void ctx_destroy(scft_ctx *c);
void ctx_poly_density(scft_ctx *c);
void ctx_update(scft_ctx *c, int n_iter);
int ctx_calc_H(scft_ctx *c, double *out);
void ctx_set_fields(scft_ctx *c, int k, const double *w);
void ctx_get_fields(scft_ctx *c, int k, double *w);
void ctx_get_density(scft_ctx *c, int k, double *ra, double *rb, double *rg);
void ctx_get_smeared(scft_ctx *c, int k, double *a, double *b, double *g);
void ctx_fft3d(scft_ctx *c, int k, double *data, int count, int sign);
void ctx_diblock_density(scft_ctx *c, int k, const double *smwa, const double *smwb, double *ra, double *rb,
                         double *Q);
void ctx_override_nD(scft_ctx *c, int k, double nD);
int ctx_grad_geom(scft_ctx *c, double *out);
void ctx_set_sweep_groups(scft_ctx *c, int groups, int phases);
void ctx_set_wait_limit(scft_ctx *c, int polls);
void ctx_set_persistent(scft_ctx *c, int on);
void ctx_set_plane_form(scft_ctx *c, int form);
void ctx_profile_sweep(scft_ctx *c, int reps, double *ms, double *bytes);
int ctx_step_fields(scft_ctx *c, const double *const *w, int n_iter, double *out);
int ctx_iterate_fields(scft_ctx *c, const double *const *w, double *const *w_out, double *out);
void ctx_set_fields_all(scft_ctx *c, const double *const *w);
void ctx_autotune(scft_ctx *c, int reps, int *groups_out, int *phases_out, int *tx_out, double *ms_out);
void ctx_profile_step(scft_ctx *c, int reps, double *ms_plane, double *bytes_plane, double *ms_col,
                      double *bytes_col);
int error_code(const std::exception &e);
int fp64_fma_rate(int reps, double *gflops, std::string &msg);
int noalloc_diblock(const int *Nx, const double *L, int Nda, int Ndb, double nD, const double *smwa,
                    const double *smwb, double *rhoda, double *rhodb, double *Q, void *stream, std::string &msg);
}  // namespace scft

static thread_local std::string g_err;

static int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define API_BODY(stmt)                                       \
  try {                                                      \
    stmt;                                                    \
  } catch (const std::bad_alloc &) {                         \
    return fail(SCFT_ERR_NOMEM, "host allocation failed");  \
  } catch (const std::exception &e) {                        \
    return fail(scft::error_code(e), e.what());              \
  }

static int check_ctx(scft_ctx *c, int inst) {
  if (!c) return fail(SCFT_ERR_ARG, "null context");
  if (inst < 0 || inst >= (int)c->inst.size()) return fail(SCFT_ERR_ARG, "instance index out of range");
  return SCFT_OK;
}

extern "C" {

const char *scft_last_error(void) { return g_err.c_str(); }

int scft_version(void) { return 2; }

int scft_create(const scft_params *params, int n_inst, scft_ctx **out) {
  if (!out) return fail(SCFT_ERR_ARG, "null output pointer");
  *out = nullptr;
  if (!params || n_inst < 1) return fail(SCFT_ERR_ARG, "need at least one instance");
  scft_ctx *c = new (std::nothrow) scft_ctx();
  if (!c) return fail(SCFT_ERR_NOMEM, "host allocation failed");
  try {
    scft::ctx_create(c, params, n_inst);
  } catch (const std::exception &e) {
    const int code = scft::error_code(e);
    g_err = e.what();
    scft::ctx_destroy(c);
    delete c;
    return code;
  }
  *out = c;
  return SCFT_OK;
}

void scft_destroy(scft_ctx *c) {
  if (!c) return;
  scft::ctx_destroy(c);
  delete c;
}

int scft_get_info(scft_ctx *c, int inst, scft_info *info) {
  if (int s = check_ctx(c, inst)) return s;
  if (!info) return fail(SCFT_ERR_ARG, "null info");
  *info = c->inst[inst].info;
  return SCFT_OK;
}

int scft_set_fields(scft_ctx *c, int inst, const double *w) {
  if (int s = check_ctx(c, inst)) return s;
  if (!w) return fail(SCFT_ERR_ARG, "null field buffer");
  API_BODY(scft::ctx_set_fields(c, inst, w));
  return SCFT_OK;
}

int scft_set_fields_all(scft_ctx *c, const double *const *w) {
  if (int s = check_ctx(c, 0)) return s;
  if (!w) return fail(SCFT_ERR_ARG, "null field buffers");
  for (size_t k = 0; k < c->inst.size(); k++)
    if (!w[k]) return fail(SCFT_ERR_ARG, "null field buffer");
  API_BODY(scft::ctx_set_fields_all(c, w));
  return SCFT_OK;
}

int scft_get_fields(scft_ctx *c, int inst, double *w) {
  if (int s = check_ctx(c, inst)) return s;
  if (!w) return fail(SCFT_ERR_ARG, "null field buffer");
  API_BODY(scft::ctx_get_fields(c, inst, w));
  return SCFT_OK;
}

int scft_calc_poly_density(scft_ctx *c) {
  if (int s = check_ctx(c, 0)) return s;
  API_BODY(scft::ctx_poly_density(c));
  return SCFT_OK;
}

int scft_update_1s(scft_ctx *c, int n_iter) {
  if (int s = check_ctx(c, 0)) return s;
  if (n_iter < 0) return fail(SCFT_ERR_ARG, "n_iter must be >= 0");
  API_BODY(scft::ctx_update(c, n_iter));
  return SCFT_OK;
}

int scft_calc_H(scft_ctx *c, double *out) {
  if (int s = check_ctx(c, 0)) return s;
  if (!out) return fail(SCFT_ERR_ARG, "null output");
  int st = SCFT_OK;
  API_BODY(st = scft::ctx_calc_H(c, out));
  if (st == SCFT_ERR_NAN) return fail(st, "H is NaN");
  if (st == SCFT_ERR_QNONPOS) return fail(st, "graft propagator q_g[Ng-1] <= 0 at 5 or more points");
  return st;
}

int scft_get_density(scft_ctx *c, int inst, double *ra, double *rb, double *rg) {
  if (int s = check_ctx(c, inst)) return s;
  API_BODY(scft::ctx_get_density(c, inst, ra, rb, rg));
  return SCFT_OK;
}

int scft_get_plate_density(scft_ctx *c, int inst, double *rho) {
  if (int s = check_ctx(c, inst)) return s;
  if (!rho) return fail(SCFT_ERR_ARG, "null output");
  cudaError_t e = cudaMemcpy(rho, c->inst[inst].rho_exp_nr, sizeof(double) * c->inst[inst].M, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  return SCFT_OK;
}

int scft_get_smeared(scft_ctx *c, int inst, double *a, double *b, double *g) {
  if (int s = check_ctx(c, inst)) return s;
  API_BODY(scft::ctx_get_smeared(c, inst, a, b, g));
  return SCFT_OK;
}

int scft_diblock_density(scft_ctx *c, int inst, const double *smwa, const double *smwb, double *ra, double *rb,
                         double *Q) {
  if (int s = check_ctx(c, inst)) return s;
  if (!smwa || !smwb) return fail(SCFT_ERR_ARG, "null field");
  API_BODY(scft::ctx_diblock_density(c, inst, smwa, smwb, ra, rb, Q));
  return SCFT_OK;
}

int scft_homopolymer_density(scft_ctx *c, int inst, const double *W, int N, double nK, double *rho, double *Q) {
  if (int s = check_ctx(c, inst)) return s;
  if (!W || N < 1) return fail(SCFT_ERR_ARG, "need a field and N >= 1");
  // homopolymer_discrete is diblock_discrete with a single block (Na = N):
  // q-dagger equals q (code/diblock_discrete.cpp:60-83 vs
  // code/homopolymer_discrete.cpp:18-41) and every term goes to rho_A.
  scft_params p = c->inst[inst].p;
  p.Nda = N;
  p.Ndb = 0;
  p.n_exp_nr = 0;
  p.sigma = 0.0;
  p.Ng = 0;
  p.precision = SCFT_PREC_FP64;
  scft_ctx *h = nullptr;
  int st = scft_create(&p, 1, &h);
  if (st != SCFT_OK) return st;
  try {
    scft::ctx_override_nD(h, 0, nK);
    scft::ctx_diblock_density(h, 0, W, W, rho, nullptr, Q);
  } catch (const std::exception &e) {
    const int code = scft::error_code(e);
    g_err = e.what();
    scft_destroy(h);
    return code;
  }
  scft_destroy(h);
  return SCFT_OK;
}

int scft_fft3d(scft_ctx *c, int inst, double *data, int count, int sign) {
  if (int s = check_ctx(c, inst)) return s;
  if (!data || count < 1 || (sign != -1 && sign != 1)) return fail(SCFT_ERR_ARG, "bad fft arguments");
  API_BODY(scft::ctx_fft3d(c, inst, data, count, sign));
  return SCFT_OK;
}

int scft_sync(scft_ctx *c) {
  if (!c) return fail(SCFT_ERR_ARG, "null context");
  cudaError_t e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return fail(SCFT_ERR_CUDA, cudaGetErrorString(e));
  return SCFT_OK;
}

int scft_grad_geom(scft_ctx *c, double *out) {
  if (int s = check_ctx(c, 0)) return s;
  if (!out) return fail(SCFT_ERR_ARG, "null output");
  int st = SCFT_OK;
  API_BODY(st = scft::ctx_grad_geom(c, out));
  return st;
}

int scft_get_stream(scft_ctx *c, void **stream) {
  if (!c || !stream) return fail(SCFT_ERR_ARG, "null argument");
  *stream = (void *)c->st;
  return SCFT_OK;
}

int scft_launch_count(scft_ctx *c, long long *count) {
  if (!c || !count) return fail(SCFT_ERR_ARG, "null argument");
  *count = c->launches;
  return SCFT_OK;
}

int scft_profile_step(scft_ctx *c, int reps, double *ms_plane, double *bytes_plane, double *ms_col,
                      double *bytes_col) {
  if (int s = check_ctx(c, 0)) return s;
  if (reps < 1 || !ms_plane || !bytes_plane || !ms_col || !bytes_col) return fail(SCFT_ERR_ARG, "bad arguments");
  API_BODY(scft::ctx_profile_step(c, reps, ms_plane, bytes_plane, ms_col, bytes_col));
  return SCFT_OK;
}

int scft_set_sweep_groups(scft_ctx *c, int groups, int phases) {
  if (int s = check_ctx(c, 0)) return s;
  if (groups < 1 || phases < 1) return fail(SCFT_ERR_ARG, "groups and phases must be >= 1");
  API_BODY(scft::ctx_set_sweep_groups(c, groups, phases));
  return SCFT_OK;
}

int scft_fp64_fma_rate(int reps, double *gflops) {
  if (!gflops || reps < 1) return fail(SCFT_ERR_ARG, "need reps >= 1 and an output pointer");
  std::string msg;
  const int st = scft::fp64_fma_rate(reps, gflops, msg);
  if (st != SCFT_OK) return fail(st, msg);
  return SCFT_OK;
}

int scft_set_wait_limit(scft_ctx *c, int polls) {
  if (int s = check_ctx(c, 0)) return s;
  API_BODY(scft::ctx_set_wait_limit(c, polls));
  return SCFT_OK;
}

int scft_set_persistent(scft_ctx *c, int on) {
  if (int s = check_ctx(c, 0)) return s;
  API_BODY(scft::ctx_set_persistent(c, on));
  return SCFT_OK;
}

int scft_step_fields(scft_ctx *c, const double *const *w, int n_iter, double *H_out) {
  if (int s = check_ctx(c, 0)) return s;
  if (!w || !H_out || n_iter < 1) return fail(SCFT_ERR_ARG, "need field pointers, an output and n_iter >= 1");
  for (size_t k = 0; k < c->inst.size(); k++)
    if (!w[k]) return fail(SCFT_ERR_ARG, "null field pointer");
  int st = SCFT_OK;
  API_BODY(st = scft::ctx_step_fields(c, w, n_iter, H_out));
  if (st == SCFT_ERR_NAN) return fail(st, "H is NaN");
  if (st == SCFT_ERR_QNONPOS) return fail(st, "graft propagator q_g[Ng-1] <= 0 at 5 or more points");
  return st;
}

int scft_iterate_fields(scft_ctx *c, const double *const *w, double *const *w_out, double *H_out) {
  if (int s = check_ctx(c, 0)) return s;
  if (!w || !H_out) return fail(SCFT_ERR_ARG, "need field pointers and an output");
  for (size_t k = 0; k < c->inst.size(); k++)
    if (!w[k] || (w_out && !w_out[k])) return fail(SCFT_ERR_ARG, "null field pointer");
  int st = SCFT_OK;
  API_BODY(st = scft::ctx_iterate_fields(c, w, w_out, H_out));
  if (st == SCFT_ERR_NAN) return fail(st, "H is NaN");
  if (st == SCFT_ERR_QNONPOS) return fail(st, "graft propagator q_g[Ng-1] <= 0 at 5 or more points");
  return st;
}

int scft_profile_sweep(scft_ctx *c, int reps, double *ms, double *bytes) {
  if (int s = check_ctx(c, 0)) return s;
  if (reps < 1 || !ms || !bytes) return fail(SCFT_ERR_ARG, "need reps >= 1 and output pointers");
  API_BODY(scft::ctx_profile_sweep(c, reps, ms, bytes));
  return SCFT_OK;
}

int scft_get_fft_plan(scft_ctx *c, int inst, int axis, int *radix, int *nst) {
  if (int s = check_ctx(c, inst)) return s;
  if (axis < 0 || axis > 2 || !radix || !nst) return fail(SCFT_ERR_ARG, "axis 0..2 and output pointers needed");
  const scft::AxisPlan &ap = c->geoms[c->inst[inst].geom].ax[axis];
  *nst = ap.nst;
  for (int k = 0; k < scft::kMaxStages; k++) radix[k] = k < ap.nst ? ap.radix[k] : 0;
  return SCFT_OK;
}

int scft_get_schedule(scft_ctx *c, int *groups, int *phases, int *col_tile, int *persistent) {
  if (int s = check_ctx(c, 0)) return s;
  if (groups) *groups = c->sweep_streams;
  if (phases) *phases = c->sweep_phases;
  if (col_tile)
    *col_tile = ((c->colfast || c->anyfast || c->xy128 || c->any96) && c->plane64_form != 2) ? c->col64_tx : 0;
  if (persistent) *persistent = c->sweep_persistent;
  return SCFT_OK;
}

int scft_set_plane_form(scft_ctx *c, int form) {
  if (int s = check_ctx(c, 0)) return s;
  API_BODY(scft::ctx_set_plane_form(c, form));
  return SCFT_OK;
}

int scft_get_plane_form(scft_ctx *c, int *form) {
  if (int s = check_ctx(c, 0)) return s;
  if (!form) return fail(SCFT_ERR_ARG, "null output pointer");
  *form = c->plane64_form;
  return SCFT_OK;
}

int scft_autotune(scft_ctx *c, int reps, int *groups, int *phases, int *col_tile, double *ms_per_sweep) {
  if (int s = check_ctx(c, 0)) return s;
  if (reps < 1 || !groups || !phases || !col_tile || !ms_per_sweep) return fail(SCFT_ERR_ARG, "bad arguments");
  API_BODY(scft::ctx_autotune(c, reps, groups, phases, col_tile, ms_per_sweep));
  return SCFT_OK;
}

// No allocation: see csrc/noalloc.cu for the scratch array, its limit and the
// first-call set-up.
int scft_diblock_density_noalloc(const int Nx[3], const double L[3], int Nda, int Ndb, double nD,
                                 const double *smwa, const double *smwb, double *rhoda, double *rhodb, double *Q,
                                 void *stream) {
  std::string msg;
  const int st = scft::noalloc_diblock(Nx, L, Nda, Ndb, nD, smwa, smwb, rhoda, rhodb, Q, stream, msg);
  if (st != SCFT_OK) return fail(st, msg);
  return SCFT_OK;
}

}  // extern "C"
