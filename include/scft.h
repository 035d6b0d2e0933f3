/*
 * scft.h -- C ABI of libscft, the GB300 (sm_103a) implementation of the SCFT
 * hot path of the aligned-nanoplate code (AB diblock melt + explicit plates
 * with grafted chains, discrete Gaussian chains, semi-implicit "1S" update).
 *
 * The reference has no plugin or FFI layer: its hot path is a set of C++ free
 * functions on global state.  Each entry point below names the reference
 * function it replaces (file:line inside the reference project):
 *
 *   scft_create            read_input() + initialize_1() + allocate() +
 *                          initialize_2()   code/read_input.cpp:7-242,
 *                          code/initialize.cpp:45-412, code/array_utils.cpp:336-547
 *   scft_set_fields        read_resume_files() code/io_utils.cpp:183-240
 *   scft_calc_poly_density calc_poly_density() code/calc_poly_density.cpp:37-161
 *   scft_update_1s         update_1s()         code/1s_update.cpp:7-352
 *   scft_calc_H            calc_H()            code/calc_h.cpp:9-64
 *   scft_get_density       the rhoda/rhodb/rhog_exp globals after
 *                          calc_poly_density   code/calc_poly_density.cpp:167-191
 *   scft_diblock_density   diblock_discrete() + integrate_diblock_discrete()
 *                          code/diblock_discrete.cpp:4-95,
 *                          code/calc_poly_density.cpp:167-191
 *   scft_homopolymer_density homopolymer_discrete() +
 *                          integrate_homopoly_discrete()
 *                          code/homopolymer_discrete.cpp:3-55,
 *                          code/calc_poly_density.cpp:193-212
 *   scft_fft3d             fft_fwd_wrapper()/fft_bck_wrapper()
 *                          code/fft_wrappers.cpp:4-67
 *
 * Conventions (same as the reference):
 *  - grids are 3-D, stack order index = x + Nx*(y + Ny*z);
 *  - complex arrays are interleaved (re, im) doubles, M = Nx*Ny*Nz entries;
 *  - forward FFT is scaled by 1/M, backward is unscaled;
 *  - b-units (bond length 1), Rg^2 = (N-1)/6;
 *  - the seven fields are ordered wpl, wabp, wabm, wbcp, wbcm, wacp, wacm.
 *
 * Ownership: the context owns all device memory; host buffers passed in are
 * copied and may be reused on return.  Calls on one context must come from
 * one host thread.  Every call returns SCFT_OK (0) or a negative error code;
 * scft_last_error() gives a message for the calling thread.
 */
#ifndef SCFT_H
#define SCFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCFT_OK 0
#define SCFT_ERR_ARG (-1)         /* bad argument or configuration */
#define SCFT_ERR_CUDA (-2)        /* CUDA runtime error */
#define SCFT_ERR_NAN (-3)         /* H is NaN (code/calc_h.cpp:37-61 exits) */
#define SCFT_ERR_QNONPOS (-4)     /* graft q <= 0 (code/grafted_nanoparticle.cpp:87-107 exits) */
#define SCFT_ERR_UNSUPPORTED (-5) /* feature or grid size not built */
#define SCFT_ERR_NOMEM (-6)       /* device allocation failed */
#define SCFT_ERR_COMPLEX (-7)     /* mixed precision needs real-valued (mean-field) w_A, w_B */

/* Precision modes. */
#define SCFT_PREC_FP64 0  /* plain method: complex FP64 throughout, as the reference */
#define SCFT_PREC_MIXED 1 /* FP32 propagators/FFTs, FP64 fields, reductions, log Q, H */

/* Plate shapes. */
#define SCFT_PLATE_REFERENCE 0 /* 0.25 erfc((|u.r|-L/2)/xi) erfc((|u x r|-R)/xi), code/initialize.cpp:578-612 */
#define SCFT_PLATE_CUBOID 1    /* product of three erfc slabs (extension, no reference counterpart) */

/* Field update schemes (scft_params.update_scheme). */
#define SCFT_UPDATE_1S 0    /* semi-implicit, code/1s_update.cpp:7-352 */
#define SCFT_UPDATE_EULER 1 /* explicit, code/Euler_update.cpp:5-213 */

/* One SCFT instance.  Field names and meanings follow bcp.input
 * (code/read_input.cpp:30-236); negative chi selects the attractive branch. */
typedef struct scft_params {
  int Nda, Ndb;        /* beads in the A and B blocks */
  double a_smear;      /* Gaussian smearing length a */
  double rho0;         /* bulk segment density */
  double chi_ab, chi_bc, chi_ac; /* signed, per segment */
  double kappa;        /* compressibility; must be > 0 */
  int Nx[3];           /* grid points (each a product of 2s, 3s and 5s, >= 2) */
  double L[3];         /* box lengths */
  double lam_pl, lam_mi; /* 1S step sizes for the + and - fields */
  int n_exp_nr;        /* explicit plates: 0, 1 or 2 */
  int np_chem;         /* 0 neutral, 1 A-like (code/1s_update.cpp:103-104) */
  double sigma;        /* graft density (chains per b^2); 0 = bare */
  int Ng;              /* beads per grafted chain */
  double L_nr, R_nr, xi_nr; /* plate thickness, radius, interface width */
  double center[2][3]; /* plate centres, fractions of L */
  double orient[2][3]; /* plate axes (normalised on input, as the reference) */
  int precision;       /* SCFT_PREC_FP64 or SCFT_PREC_MIXED */
  int plate_shape;     /* SCFT_PLATE_REFERENCE or SCFT_PLATE_CUBOID */
  /* Extension (no counterpart in the reference): a potential on A segments
   * in a shell around the plates, U_A = shell_lambda * sum_j [rho_p(L_nr +
   * 2 w, R_nr + w) - rho_p(L_nr, R_nr)] with w = shell_width, added to the
   * smeared w_A wherever the propagators and densities use it (negative:
   * A-attractive).  Needs a plate and w > 0; 0 turns it off. */
  double shell_lambda;
  double shell_width;
  /* SCFT_UPDATE_1S (0) or SCFT_UPDATE_EULER (1): the reference's
   * update_scheme 1 (update_1s, code/1s_update.cpp) and 0 (update_Euler,
   * code/Euler_update.cpp).  kappa <= 0 (no w+^2 term) is allowed with Euler. */
  int update_scheme;
  /* Complex-Langevin noise in the field update (do_CL, code/1s_update.cpp:
   * 54-319, code/Euler_update.cpp:49-172), FP64 method only.  The noise is
   * the reference's own stream: its ran2/Gaussian deviates seeded like
   * idum = -cl_seed, so a run with the same seed adds the same noise. */
  int do_cl;
  long long cl_seed;
} scft_params;

/* Derived per-instance quantities (code/initialize.cpp:249-386). */
typedef struct scft_info {
  long M;
  double V, Vf, nD, phiD, phiG, np_frac, nP, ng_per_np;
  int N;
  double dx[3];
} scft_info;

typedef struct scft_ctx scft_ctx;

/* Message of the last failed call on this host thread, and the ABI version
 * (2: with the mixed form).  No counterpart in the reference, which prints
 * and exits on errors. */
const char *scft_last_error(void);
int scft_version(void);

/* Creates n_inst instances (sizes may differ) on the current CUDA device.
 * Fields start at zero.  scft_destroy frees everything the context holds (the
 * reference frees its globals only at process exit). */
int scft_create(const scft_params *params, int n_inst, scft_ctx **out);
void scft_destroy(scft_ctx *ctx);

/* The derived quantities of one instance (see scft_info above). */
int scft_get_info(scft_ctx *ctx, int inst, scft_info *info);

/* scft_set_fields for every instance of the context in one call: w[inst]
 * as for scft_set_fields.  The copies and checks of all instances are issued
 * back to back with one synchronisation (the per-instance call waits once
 * per instance).  No counterpart in the reference (one process per run). */
int scft_set_fields_all(scft_ctx *ctx, const double *const *w);

/* Sets/gets the seven fields of one instance: w[f*2*M + 2*i + {0,1}]
 * (read_resume_files(), code/io_utils.cpp:183-240; the get side feeds the
 * field files of write_outputs(), code/io_utils.cpp:11-105).  Mixed-form
 * instances hold the pairs whose chi is 0 at zero, as the reference
 * initialises them (code/initialize.cpp:430-431; its update never changes
 * them): values given there are not kept. */
int scft_set_fields(scft_ctx *ctx, int inst, const double *w);
int scft_get_fields(scft_ctx *ctx, int inst, double *w);

/* One call for "iterate from these fields": uploads the fields of every
 * instance from host memory (w[inst], each as for scft_set_fields; pinned
 * memory lets the uploads overlap compute), builds the densities of
 * those fields, runs n_iter field updates (as scft_update_1s) and writes H
 * into H_out (5 doubles per instance, as scft_calc_H), with one
 * synchronisation.  The sequence scft_set_fields_all, scft_update_1s,
 * scft_calc_H does the same; here, for mixed-form batches without grafted
 * chains or complex Langevin and with page-locked host buffers (pinned or
 * registered; others run the sequence), each sweep group's upload, realness check,
 * field transform, density build and updates run as one chain on its own
 * stream inside one captured graph (re-captured when the host pointers or
 * n_iter change), so one group's upload runs beside another group's
 * compute; only w+ and the pairs of nonzero chi are read (the others are held
 * at zero, as scft_set_fields does).  The realness check of the mixed form
 * is read after the work:
 * SCFT_ERR_COMPLEX then means this call's results are invalid.  Returns
 * SCFT_ERR_NAN / SCFT_ERR_QNONPOS like scft_calc_H.  No counterpart in the
 * reference (its driver keeps the fields in host memory throughout). */
int scft_step_fields(scft_ctx *ctx, const double *const *w, int n_iter, double *H_out);

/* One iteration of the reference's main loop per instance from and to host
 * memory, in the order calc_poly_density, calc_H, update_1s (the set-up
 * code/simulate.cpp:36,74 and the main loop :85-157, whose update_1s ends in
 * the next calc_poly_density, code/1s_update.cpp:351): uploads the fields of every
 * instance from w[inst] (as scft_set_fields), builds their densities, writes
 * H of those fields into H_out (5 doubles per instance, as scft_calc_H), runs
 * one field update (update_1s, or update_Euler per instance) and, when w_out
 * is not NULL, writes the updated fields into w_out[inst] (same layout; w_out
 * may be w, which makes repeated calls a host-driven iteration).  Mixed-form
 * instances write the fields an update changes (w+ and the pairs of nonzero
 * chi; a pair whose chi is 0 is never updated) and leave the others as they
 * are; FP64 instances write all seven.  The
 * densities are not rebuilt for the updated fields: a call that needs them
 * (scft_get_density, scft_calc_H, scft_update_1s) rebuilds them first.  For
 * mixed-form batches without grafted chains or complex Langevin and with
 * page-locked buffers (pinned or registered), the uploads, density builds,
 * H sums, k-space updates and downloads of each sweep group run as one chain
 * on its own stream inside one captured graph (re-captured when the host
 * pointers change), so an iteration costs one density build; the others run
 * scft_set_fields_all, scft_calc_H, scft_update_1s and scft_get_fields.
 * Returns and realness check as scft_step_fields (SCFT_ERR_COMPLEX: this
 * call's results, w_out included, are invalid). */
int scft_iterate_fields(scft_ctx *ctx, const double *const *w, double *const *w_out, double *H_out);

/* calc_poly_density() for every instance. */
int scft_calc_poly_density(scft_ctx *ctx);

/* n_iter field updates of every instance, each followed by
 * calc_poly_density: update_1s(), or update_Euler() for instances with
 * update_scheme = SCFT_UPDATE_EULER (code/simulate.cpp:86-89). */
int scft_update_1s(scft_ctx *ctx, int n_iter);

/* calc_H() per instance.  out[5*inst + {0..4}] = Re H, Im H, Re Qd, Im Qd,
 * Re Qga (Qga = 0 without grafted plates). */
int scft_calc_H(scft_ctx *ctx, double *out);

/* Densities of one instance after calc_poly_density (real space):
 * rhoda, rhodb, rhog_exp (any may be NULL). */
int scft_get_density(scft_ctx *ctx, int inst, double *rhoda, double *rhodb, double *rhog_exp);

/* Derivatives of H (real part) with respect to the plate geometry at the
 * current fields: out[8*inst + 4*j + {0,1,2,3}] = dH/dtheta, dH/dc_x,
 * dH/dc_y, dH/dc_z for plate j (0 or 1), theta a rotation of the plate axis
 * about z in radians, c the centre in b-units.  At a converged saddle point
 * (delta H / delta w = 0) these are the total derivatives of the converged
 * H; a separation d of two plates along an axis e gives
 * dH/dd = (dH/dc_2 - dH/dc_1).e / 2.  The reference has no derivative code;
 * this replaces finite differences over its sweeps (angle-rotation/,
 * particle-separation/).  With the shell potential the derivative includes
 * shell_lambda * int rho_A d(shell)/dg; with grafted plates it includes
 * -n_exp_nr ng_per_np Re int (dg_map/dg) log q_g[Ng-1], the graft map
 * g_map ~ |grad rho_p(1.05 L, 1.05 R)| differentiated through its spectral
 * gradient and normalisation (code/initialize.cpp:160-200,
 * code/grafted_nanoparticle.cpp:82-112).  Both plate shapes are covered;
 * for SCFT_PLATE_CUBOID the in-plane axes turn with u. */
int scft_grad_geom(scft_ctx *ctx, double *out);

/* The explicit plates' density rho_exp_nr of one instance (M real values),
 * as built at set-up (code/initialize.cpp:210-239). */
int scft_get_plate_density(scft_ctx *ctx, int inst, double *rho_exp_nr);

/* Smeared fields of one instance (smwa, smwb, smwg; any may be NULL): the
 * globals calc_poly_density() forms, code/calc_poly_density.cpp:92-104. */
int scft_get_smeared(scft_ctx *ctx, int inst, double *smwa, double *smwb, double *smwg);

/* diblock_discrete + integrate_diblock_discrete on given smeared fields of
 * instance `inst` (its grid, N, Nda, nD); writes rhoda, rhodb and Q[2]. */
int scft_diblock_density(scft_ctx *ctx, int inst, const double *smwa, const double *smwb,
                         double *rhoda, double *rhodb, double *Q);

/* homopolymer_discrete(W, N) + integrate_homopoly_discrete with nK. */
int scft_homopolymer_density(scft_ctx *ctx, int inst, const double *W, int N, double nK,
                             double *rho, double *Q);

/* The same computation as scft_diblock_density (FP64 method) for callers that
 * cannot allocate GPU memory: code whose device memory belongs to another
 * framework's pool allocator, services with a fixed memory budget, and code
 * that cannot accept the device-wide wait of cudaFree.  No counterpart in the
 * reference.
 *
 * All pointers except Nx and L are DEVICE pointers owned by the caller:
 * smwa, smwb (inputs) and rhoda, rhodb (outputs) hold M complex values each,
 * Q receives 2 doubles; nD is the number of chains (the reference's nD).
 * Work is queued on `stream` (a cudaStream_t, NULL for the default stream)
 * and the call returns without synchronising.  Nothing is allocated: the
 * scratch is one file-scope device array of 64 MiB that every GPU loading
 * libscft holds until exit; a diblock needs about
 * M * (136 + 32 * ((Nda + Ndb - 1)/2 + 1)) bytes of it (32^3 grid up to
 * N ~ 118); larger problems are rejected with SCFT_ERR_ARG.  The first call
 * on a device looks up the array's device address (make that call before any
 * stream capture); that cached address does not survive cudaDeviceReset.
 * Calls share the array and it keeps the last call's contents (what must
 * start at zero is cleared on every call): calls that overlap on the GPU
 * race. */
int scft_diblock_density_noalloc(const int Nx[3], const double L[3], int Nda, int Ndb, double nD,
                                 const double *smwa, const double *smwb, double *rhoda, double *rhodb,
                                 double *Q, void *stream);

/* 3-D FFT of `count` arrays of instance inst's grid (host buffers, in place):
 * sign -1 forward (scaled 1/M), +1 backward (unscaled). */
int scft_fft3d(scft_ctx *ctx, int inst, double *data, int count, int sign);

/* Synchronises the context's stream; returns the first asynchronous error.
 * This and the next four entry points have no counterpart in the reference:
 * they expose the GPU context (stream, launch count, schedule, timing). */
int scft_sync(scft_ctx *ctx);

/* The cudaStream_t on which every kernel of this context runs (for callers
 * that time or order work around it). */
int scft_get_stream(scft_ctx *ctx, void **stream);

/* Number of kernel launches this context has issued so far (kernels inside a
 * replayed CUDA graph count once per replay). */
int scft_launch_count(scft_ctx *ctx, long long *count);

/* Launch schedule of the mixed form's propagator sweep (no counterpart in
 * the reference).  The batch is cut into `phases` sub-batches that sweep one
 * after another (so that a sub-batch's working set can stay in L2), and each
 * sub-batch into `groups` independent chains of launches (contiguous instance
 * ranges, about equal work) on side streams inside the captured iteration, so
 * that one chain's z passes fill the last wave of another chain's plane pass.
 * Default 2 groups, 1 phase. */
int scft_set_sweep_groups(scft_ctx *ctx, int groups, int phases);

/* Measurement (no counterpart in the reference): the FP64 FMA throughput of
 * the current GPU in GFLOP/s (2 flops per FMA), from `reps` timed launches of
 * a register-only FMA kernel over every SM (CUDA events).  The plain FP64
 * method's kernels are placed against it as well as against HBM bandwidth. */
int scft_fp64_fma_rate(int reps, double *gflops);

/* Diagnostic (no counterpart in the reference, whose loops have no waits):
 * the number of polls a bounded wait makes before it records a timeout in
 * the context's error word: the first mbarrier wait of each mixed plane-pass
 * CTA (default 4194304) and each dependency wait of the persistent sweep
 * (default 16777216); polls < 0 restores the defaults.  A plane-pass CTA
 * whose mbarrier wait ran out still waits, bounded, for its copies to land,
 * so its results are complete and the context stays usable; the call returns
 * SCFT_ERR_CUDA ("a TMA wait ... ran out").  A dependency wait that runs out
 * stops the persistent sweep (every CTA leaves within its own bounded wait):
 * the call returns SCFT_ERR_CUDA ("a dependency wait ... ran out"), its
 * results are invalid, and the context is usable again once the fields are
 * set anew.  polls = 0 makes every such wait run out at once, which is how a
 * test sees both paths without a fault. */
int scft_set_wait_limit(scft_ctx *ctx, int polls);

/* Persistent sweep (no counterpart in the reference): on = 1 runs the whole
 * propagator sweep of each group of 64 x 64 x 64 instances as one persistent
 * launch, whose CTAs take plane and z-column tasks of every step from a
 * counter and wait (bounded) on per-instance task counts, instead of two
 * launches per step.  Other grids keep the per-step launches.  Results are
 * bit-identical either way. */
int scft_set_persistent(scft_ctx *ctx, int on);

/* The current launch schedule of the mixed sweep (any pointer may be NULL):
 * groups, phases, z-pass columns per CTA of the 64-point kernels (0 where it
 * does not apply) and whether the sweep is persistent. */
int scft_get_schedule(scft_ctx *ctx, int *groups, int *phases, int *col_tile, int *persistent);

/* Form of the mixed form's plane pass (no counterpart in the reference):
 * 0 (default) the specialised kernels of each grid class, with the 64-point
 * plane pass exchanging through a padded shared plane with block barriers
 * (k_mix_plane64); 1 the same with the 64-point pass loading the working
 * plane asynchronously into a swizzled shared plane and transforming
 * columns inside one warp (k_mix_plane64w; bit-identical, the autotuner
 * picks 0 or 1); 2 the generic plane and z passes for every instance, the
 * reference the specialised classes (64 x 64, 96 x 64 x 64 and 128 x 128
 * planes) are checked against. */
int scft_set_plane_form(scft_ctx *ctx, int form);
int scft_get_plane_form(scft_ctx *ctx, int *form);

/* The FFT stage plan of instance inst along axis 0 (x), 1 or 2: *nst radices
 * in application order in radix[0..7] (the rest 0).  Generic transforms
 * only; the 64-point kernels use a fixed 8 x 8 four-step transform. */
int scft_get_fft_plan(scft_ctx *ctx, int inst, int axis, int *radix, int *nst);

/* Autotuner: times reps full propagator sweeps of the batch for every
 * candidate schedule (1-4 phases x 1-6 or 8 groups; for 64-point grids also
 * 8, 16 or 32 z-pass columns per CTA, and the persistent sweep with 1-3
 * groups x 1-2 phases) with CUDA events and keeps the fastest
 * (scft_get_schedule reads the choice); then, with that schedule, the stage
 * order of the generic FFTs for each axis length of the batch (every order of
 * radices 8, 4, 2, 3, 5 with at most one radix-2 stage, up to 12 plans per
 * length, one length at a time; scft_get_fft_plan reads the choice).  Reports the choice (col_tile 0 where it does not apply) and its
 * time per sweep.  FP64 contexts have a single schedule (1 group, 1 phase). */
int scft_autotune(scft_ctx *ctx, int reps, int *groups, int *phases, int *col_tile, double *ms_per_sweep);

/* Times the two kernels of one propagator step in isolation on the context
 * stream (CUDA events, `reps` launches each, all instances): the xy-plane pass
 * at a step of the second half of the sweep and the z-column pass.  Writes
 * the mean milliseconds per launch and the algorithmic bytes one launch has
 * to move: per grid point of every propagator, the plane pass reads its input,
 * the Boltzmann factor and the stored partner propagator, writes its output
 * and read-modify-writes one density accumulator; the column pass reads and
 * writes the array and reads the bond-kernel table.  Leaves the propagator
 * buffers in an undefined state; call scft_calc_poly_density afterwards. */
int scft_profile_step(scft_ctx *ctx, int reps, double *ms_plane, double *bytes_plane, double *ms_col,
                      double *bytes_col);

/* Times `reps` FP32 propagator sweeps of the whole batch (mixed form) with
 * the current schedule, alone (no field work), on the context stream with
 * CUDA events; writes the mean milliseconds per sweep and the algorithmic
 * bytes of one sweep (per point and step: the z pass's 16 B, the plane
 * pass's working plane in and out, Boltzmann pair, history out or stored
 * partner in, FP32 accumulators read and written).  With the persistent
 * sweep this is one launch per group.  Leaves the densities invalid; call
 * scft_calc_poly_density afterwards. */
int scft_profile_sweep(scft_ctx *ctx, int reps, double *ms, double *bytes);

#ifdef __cplusplus
}
#endif

#endif /* SCFT_H */
