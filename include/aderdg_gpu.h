/*
 * aderdg_gpu.h -- C ABI of the GB300 (sm_103a) ADER-DG time step.
 *
 * Drop-in boundary for one time step of dasikasunder/ADER-DG (2D Cartesian
 * advection-diffusion, Euler and Baer-Nunziato solvers).  The reference calls
 * its phases as Fortran external subroutines, per cell, from main.f90, with
 * all data in the module ader_dg (Euler/ader_dg.f90:8-103).  Per-cell calls
 * are far too fine for a GPU, so this ABI is grid-level: one call per
 * reference phase over the whole grid, plus a fused step and a fused run.
 * Every array argument uses the reference's Fortran column-major layout
 * (first index fastest), so a Fortran caller passes its module arrays
 * unchanged through ISO_C_BINDING (see ader-dg_gb300/fortran/aderdg_gpu.f90).
 *
 * Conventions:
 *   - plain C types only; arrays are host pointers owned by the caller;
 *   - every call returns ADERDG_OK (0) or a negative ADERDG_E* code and never
 *     aborts or prints; aderdg_last_error() gives a one-line reason;
 *   - a context owns its device state and one CUDA stream; it is not
 *     re-entrant, distinct contexts may be used from distinct host threads.
 */
#ifndef ADERDG_GPU_H
#define ADERDG_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADERDG_ABI_VERSION 1

enum aderdg_status {
  ADERDG_OK = 0,
  ADERDG_EINVAL = -1,       /* bad argument or configuration */
  ADERDG_ENOMEM = -2,       /* device or host allocation failed */
  ADERDG_ECUDA = -3,        /* a CUDA runtime call failed */
  ADERDG_ETIMEOUT = -4,     /* a bounded device wait gave up */
  ADERDG_ENONFINITE = -5,   /* the state became non-finite (NaN/Inf time step) */
  ADERDG_ESTATE = -6,       /* call out of order (e.g. step before upload) */
  ADERDG_EUNSUPPORTED = -7, /* configuration not built (system, N) */
  ADERDG_ENOSPACE = -8      /* a fixed-capacity buffer is too small */
};

enum aderdg_system { ADERDG_SYS_ADVDIFF = 0, ADERDG_SYS_EULER = 1, ADERDG_SYS_BN = 2 };
/* ADERDG_FP64: every phase in FP64 (the reference's arithmetic).
 * ADERDG_FP32_MIXED: the predictor, volume and surface contractions and the
 *   Euler / advection-diffusion face fluxes in FP32 with FP32 accumulation;
 *   FP64 for the update of the state (conservation), the Baer-Nunziato
 *   path-conservative face flux with its Roe-matrix path integral, the
 *   subcell finite-volume re-solve, the CFL maximum and dt.  The DMP and
 *   positivity decisions are those of an FP64 evaluation of the same state:
 *   FP32 projections decide where their error bound settles the comparison,
 *   FP64 reference-order projections decide the rest.
 * ADERDG_FP32_WIDE: as ADERDG_FP32_MIXED, but the Baer-Nunziato face flux and
 *   the subcell re-solve in FP32 too, and DMP decisions from the FP32
 *   projections whenever their error bound is within the DMP's 1e-4 floor,
 *   without settling comparisons closer than that bound (faster; decisions
 *   near the thresholds may differ from FP64's). */
enum aderdg_precision { ADERDG_FP64 = 0, ADERDG_FP32_MIXED = 1, ADERDG_FP32_WIDE = 2 };

/* Configuration: what the reference reads from params.ini
 * (Euler/initialize.f90:21-38, Baer-Nunziato/initialize.f90:21-41,
 * Advection-Diffusion/initialize.f90:19-37) plus its compile-time parameters
 * N and CFL (Euler/ader_dg.f90:17-20), which are runtime choices here. */
typedef struct aderdg_config {
  int system;     /* aderdg_system */
  int N;          /* polynomial degree, 1..5 */
  int imax, jmax; /* cells in x and y */
  double xl[2], xr[2];
  int bc[4];      /* left, right, bottom, top: 1 transmissive (AD: Neumann),
                     2 AD Dirichlet (Advection-Diffusion/riemann_problem.f90:27-49),
                     3 periodic; bc_mode 1 overrides with the Euler double Mach
                     reflection boundaries hard-wired in Euler/riemann_problem.f90 */
  int bc_mode;    /* 0 per-side codes, 1 Euler double Mach reflection */
  double cfl;     /* CFL number (reference: 0.9) */
  double gamma;   /* Euler ratio of specific heats */
  double gamma_s, gamma_g, pi_s, pi_g; /* Baer-Nunziato stiffened-gas EOS */
  double cx, cy, a;  /* advection velocity and diffusion coefficient */
  int ad_flux_mode;  /* 0: predictor uses the viscous flux only, as
                        Advection-Diffusion/space_time_predictor.f90:78 does;
                        1: viscous + convective flux (PDEFusedViscConvFlux) */
  int limiter;       /* 1: a posteriori subcell limiter (Euler, BN) */
  int precision;     /* aderdg_precision */
} aderdg_config;

typedef struct aderdg_ctx aderdg_ctx;

/* Replaces the allocation and operator part of initialize
 * (Euler/initialize.f90:8-258): validates cfg, builds the 1D operators on the
 * host in FP64 and allocates the device state. */
int aderdg_create(const aderdg_config* cfg, aderdg_ctx** out);
int aderdg_destroy(aderdg_ctx* ctx);

/* Copies uh(nVar, N+1, N+1, IMAX, JMAX) to the device (the projected initial
 * field of Euler/initialize.f90:262-285, or any state).  Resets the limiter
 * status to 0 everywhere. */
int aderdg_upload(aderdg_ctx* ctx, const double* uh);

/* The initial limiter block of initialize (Euler/initialize.f90:287-307):
 * DMP with argmax 0.1 against each cell's own nodal min/max; cells that fail
 * get status 1 and Lh = lh_ic(nVar, 2N+1, 2N+1, IMAX, JMAX), the initial field
 * at the subcell barycentres.  *n_limited (nullable) receives the count. */
int aderdg_init_limiter(aderdg_ctx* ctx, const double* lh_ic, int* n_limited);

/* Restores / reads the limiter state: status(IMAX,JMAX) and
 * Lh(nVar,2N+1,2N+1,IMAX,JMAX) (only entries of cells with status != 0 matter). */
int aderdg_upload_limiter(aderdg_ctx* ctx, const int* status, const double* lh);
int aderdg_download_limiter(aderdg_ctx* ctx, int* status, double* lh);

/* Copies uh back; status (nullable) receives the limiter status per cell. */
int aderdg_download(aderdg_ctx* ctx, double* uh, int* status);

/* ---- phase API: one call per reference phase, in main.f90 order ---- */

/* calc_time_step.f90 (Euler :9-52, BN :9-52, AD :9-57): dt from the current
 * uh, clipped to tend - time.  Also records time and dt in the context for the
 * phases below. */
int aderdg_calc_time_step(aderdg_ctx* ctx, double time, double tend, double* dt);

/* Sets time and dt directly (a caller that computes dt itself). */
int aderdg_set_time_step(aderdg_ctx* ctx, double time, double dt);

/* get_min_max + recompute(:,:)=0 + save_olduh (Euler/main.f90:31-36,
 * Euler/limiter.f90:104-171, :251-265). No-op without the limiter. */
int aderdg_limiter_prepare(aderdg_ctx* ctx);

/* ader_space_time_predictor over all cells (Euler/main.f90:40-45,
 * Euler/space_time_predictor.f90:8-123, Baer-Nunziato/space_time_predictor.f90:8-143,
 * Advection-Diffusion/space_time_predictor.f90:10-155). */
int aderdg_space_time_predictor(aderdg_ctx* ctx);

/* volume_integral over all cells (Euler/volume_integral.f90:8-36,
 * Baer-Nunziato/volume_integral.f90:8-44). */
int aderdg_volume_integral(aderdg_ctx* ctx);

/* solve_riemann_problem with boundary conditions (Euler/riemann_problem.f90:10-116,
 * Baer-Nunziato/riemann_problem.f90:9-80, Advection-Diffusion/riemann_problem.f90:8-113). */
int aderdg_riemann_problem(aderdg_ctx* ctx);

/* surface_integral over all cells (Euler/surface_integral.f90:8-39, identical
 * in the three solvers). */
int aderdg_surface_integral(aderdg_ctx* ctx);

/* element_update over all cells (Euler/element_update.f90:8-30, identical in
 * the three solvers) followed, with the
 * limiter, by the DMP check of Euler/main.f90:74-88; *n_recompute (nullable)
 * receives the number of troubled cells (nRecompute). */
int aderdg_element_update(aderdg_ctx* ctx, int* n_recompute);

/* spread_recompute, allocate_limiter, subcell_recompute, update_limiter
 * (Euler/limiter.f90:272-647, Baer-Nunziato/limiter.f90:271-596). */
int aderdg_limiter(aderdg_ctx* ctx);

/* ---- fused API ---- */

/* One complete loop body of main.f90 (Euler :24-100, BN :24-101, AD :23-78):
 * calc_time_step, predictor with fused volume integral, Riemann problems,
 * fused surface integral + element update + DMP + CFL partials, limiter.
 * Time and dt stay on the device; on return *time has advanced by the step's
 * dt (nothing happens when *time >= tend).  Outputs are nullable. */
int aderdg_step(aderdg_ctx* ctx, double* time, double tend, double* dt, int* n_recompute);

/* Repeats fused steps until time >= tend or max_steps steps ran, as the
 * `do while (time < tend)` loop of main.f90; steps are replayed from a
 * captured CUDA graph and the host synchronises every `sync_every` steps
 * (<= 0: a default).  *steps_done (nullable) receives the count. */
int aderdg_run(aderdg_ctx* ctx, double* time, double tend, int max_steps, int sync_every, int* steps_done);

/* The drop-in for one reference step called with host arrays: copies
 * uh(nVar,P,P,IMAX,JMAX) to the device, recomputes the DMP min/max and the
 * CFL denominators of that state, runs one fused step and copies uh back. */
int aderdg_step_host(aderdg_ctx* ctx, double* uh, double* time, double tend, double* dt, int* n_recompute);

/* ---- measurement ---- */

/* Runs `steps` fused steps (graph replays) and returns the device time of
 * each in step_ms[steps], measured with CUDA events on the context's stream.
 * With flush_l2, a write over a buffer larger than L2 precedes every step,
 * outside the timed interval.  *time advances as in aderdg_run. */
int aderdg_time_steps(aderdg_ctx* ctx, double* time, double tend, int steps, int flush_l2, double* step_ms);

/* Runs one fused step eagerly with CUDA events between its launches and
 * returns each launch's device time in phase_ms[7]: begin, predictor, faces,
 * cells (surface + update + DMP), mark, subcell, end. */
int aderdg_profile_step(aderdg_ctx* ctx, double* time, double tend, double* phase_ms);

/* ---- introspection for parity checks ---- */
enum aderdg_array {
  ADERDG_A_UH = 0,       /* uh(nVar,P,P,I,J) */
  ADERDG_A_DUH,          /* duh(nVar,P,P,I,J) */
  ADERDG_A_QHI,          /* qhi(nVar,P,P,I,J)   (phase API only) */
  ADERDG_A_FHI,          /* Fhi(nVar,2,P,P,I,J) (phase API only) */
  ADERDG_A_SHI,          /* Shi(nVar,P,P,I,J)   (BN, phase API only) */
  ADERDG_A_QBND,         /* qbnd(nVar,4,P,I,J) */
  ADERDG_A_FBND,         /* Fbnd(nVar,4,P,I,J) (not AD) */
  ADERDG_A_GRADQBND,     /* gradQbnd(nVar,2,4,P,I,J) (AD) */
  ADERDG_A_FU,           /* Fu(nVar,P,I+1,J) (Euler, AD) / Fm for BN */
  ADERDG_A_GU,           /* Gu(nVar,P,I,J+1) (Euler, AD) / Gm for BN */
  ADERDG_A_FP,           /* Fp(nVar,P,I+1,J) (BN) */
  ADERDG_A_GP,           /* Gp(nVar,P,I,J+1) (BN) */
  ADERDG_A_LH,           /* Lh(nVar,S,S,I,J) */
  ADERDG_A_LMIN,         /* lmin(nVar,I,J): neighbourhood minimum used by the DMP */
  ADERDG_A_LMAX,
  ADERDG_A_RECOMPUTE,    /* int recompute(I,J) */
  ADERDG_A_STATUS        /* int status(I,J) */
};
/* Element count of an array (doubles or ints), or a negative error.  In the
 * FP32 modes DUH, QBND, FBND/GRADQBND and FU..GP are held in FP32 on the
 * device; get/set convert them to and from double. */
long aderdg_array_size(aderdg_ctx* ctx, int which);
int aderdg_get_array(aderdg_ctx* ctx, int which, void* out);
/* Overwrites a device array (same layouts; LMIN/LMAX are read-only).  Used
 * to restart from a checkpoint and to feed one phase the exact inputs of the
 * previous one when checking phases in isolation. */
int aderdg_set_array(aderdg_ctx* ctx, int which, const void* in);

/* Counters: cells, DOF per step, device bytes allocated, steps run. */
typedef struct aderdg_info {
  long cells;
  long dofs;            /* nVar * (N+1)^2 * cells: DOF-updates per step */
  long device_bytes;
  long steps;
  double time;
  double dt;
  int n_recompute;      /* last step */
  int n_limited;        /* cells with status != 0 after the last step */
  int n_settled;        /* FP32-mixed: DMP decisions of the last step that the FP32
                           error bounds left open and FP64 values settled */
  int n_listed;         /* cells the last step's limiter re-solved (recompute > 0) */
} aderdg_info;
int aderdg_get_info(aderdg_ctx* ctx, aderdg_info* info);

const char* aderdg_last_error(aderdg_ctx* ctx); /* ctx may be NULL: last global error */

/* ---- batched simulations ----
 * Many independent simulations of one (system, N, precision, limiter) stepped
 * by the same launches, each with its own grid, boundary conditions,
 * physical parameters, CFL time step and end time (the reference runs one
 * simulation per process; this is the GB300 form of running many).  The
 * batch owns a pool of units; a simulation with an IMAX x JMAX grid takes
 * (IMAX+1)(JMAX+1) consecutive units (first fit).  Simulations are admitted
 * and released between steps while the others keep running. */
typedef struct aderdg_batch aderdg_batch;

/* Device bytes per unit of a batch of this kind (admission by HBM footprint). */
long aderdg_batch_unit_bytes(int system, int N, int precision, int limiter);
int aderdg_batch_create(int system, int N, int precision, int limiter, long capacity_units, int max_instances,
                        aderdg_batch** out);
int aderdg_batch_destroy(aderdg_batch* b);
/* Admits one simulation (cfg must match the batch; uh and lh_ic as in
 * aderdg_upload / aderdg_init_limiter, lh_ic nullable) that runs until tend
 * or max_steps steps (<= 0: no limit).  *slot receives its id.
 * ADERDG_ENOSPACE when no free range or table entry is left.  The set-up is
 * queued on the batch's stream behind the steps already launched; the call
 * returns once uh and lh_ic have been copied (they may be reused), and
 * aderdg_batch_admit_ic returns without waiting for the GPU at all.
 * aderdg_batch_release frees the simulation's units and table entry, also
 * without waiting. */
int aderdg_batch_admit(aderdg_batch* b, const aderdg_config* cfg, const double* uh, const double* lh_ic, double tend,
                       long max_steps, int* slot);
int aderdg_batch_release(aderdg_batch* b, int slot);
/* Enqueues `steps` fused steps of every running simulation and returns
 * without waiting; aderdg_batch_sync waits, reads the per-simulation state
 * back and gives the number still running. */
int aderdg_batch_launch(aderdg_batch* b, int steps);
int aderdg_batch_sync(aderdg_batch* b, int* n_running);
/* Without waiting: *ready = 1 when everything queued on the batch's stream
 * (steps, admissions, releases) has completed, so that aderdg_batch_sync
 * returns at once; 0 otherwise.  Lets a host serve many batches in the order
 * their work completes. */
int aderdg_batch_ready(aderdg_batch* b, int* ready);
/* One simulation's state as read back by the last aderdg_batch_sync (read
 * back now, waiting for the batch's stream, when an admission or release came
 * after it). */
int aderdg_batch_query(aderdg_batch* b, int slot, double* time, double* dt, long* steps, int* done);
int aderdg_batch_download(aderdg_batch* b, int slot, double* uh);
/* Sums over the batch's simulations of the last step's counters: troubled
 * cells (nRecompute), cells the limiter re-solved (recompute > 0) and, in the
 * FP32-mixed mode, DMP decisions settled from FP64 values. */
int aderdg_batch_counters(aderdg_batch* b, int* n_recompute, int* n_listed, int* n_settled);
/* The simulation's limiter status(IMAX,JMAX) (as aderdg_download's status):
 * 1 for the cells its last step limited; zeros without the limiter. */
int aderdg_batch_download_status(aderdg_batch* b, int slot, int* status);
int aderdg_batch_info(aderdg_batch* b, long* used_units, long* capacity_units, long* device_bytes, int* n_instances);
/* One fused step of the batch, eager, with CUDA events between its launches:
 * device ms of each in phase_ms[7] (as aderdg_profile_step). */
int aderdg_batch_profile(aderdg_batch* b, double* phase_ms);
/* Measurement hook: `steps` fused steps of each of n batches, the batches on
 * their own streams concurrently, bracketed by CUDA events on a timing stream
 * that every batch stream waits for and that waits for all of them; *ms = the
 * device time between the two events.  Returns after the second event. */
int aderdg_batch_run_timed(aderdg_batch* const* batches, int n, int steps, double* ms);
const char* aderdg_batch_last_error(aderdg_batch* b);

/* ---- output and error analysis (not on the hot path) ---- */
/* Cell averages of uh, out[(i + IMAX*j)*nVar + v] (the reference's wh(nVar,IMAX,JMAX));
 * primitive != 0: converted with PDECons2Prim, i.e. exactly the field
 * write_data writes (Euler/write_data.f90:17-33). */
int aderdg_cell_averages(aderdg_ctx* ctx, int primitive, double* out);
int aderdg_batch_cell_averages(aderdg_batch* b, int slot, int primitive, double* out);
/* Error of the cell averages of variable `var` against an exact field at the
 * context's current time: norms = {mean |e|, root mean square of e, max |e|}.
 * max |e| at time 0 against the initial field is analyze_soln's number
 * (Euler/analyze_soln.f90:10-56); the isentropic vortex (translated with its
 * free stream) and the sine wave (translated with (cx, cy), damped by
 * exp(-8 pi^2 a t)) are compared with their exact solutions at that time,
 * other fields with the initial field. */
int aderdg_error_norms(aderdg_ctx* ctx, int ic, const double* params, int var, double* norms);

/* ---- host setup helpers (initial fields; not on the hot path) ---- */
enum aderdg_ic {
  ADERDG_IC_AD_ZERO = 0,      /* Advection-Diffusion/initialize.f90:148-164 */
  ADERDG_IC_AD_SINE = 1,      /* p = {A}: A sin(2 pi x) sin(2 pi y) */
  ADERDG_IC_EULER_DMR = 10,   /* Euler/initialize.f90:311-341 */
  ADERDG_IC_EULER_VORTEX = 11,/* p = {eps, xc, yc, rho, u, v, p} isentropic vortex */
  ADERDG_IC_EULER_RP2D = 12,  /* p = {xs, ys, (rho,u,v,p) x {UR, UL, LL, LR}} */
  ADERDG_IC_BN_RP1D = 20,     /* p = {ICType (1,2,3,7), x_interface}: Baer-Nunziato/initialize.f90:302-407 */
  ADERDG_IC_BN_CYLINDER = 21  /* p = {x0, y0, R, inside (a_s,rho_s,p_s,rho_g,p_g), outside (...)} */
};
/* Projects an initial field onto the Gauss-Legendre nodes (uh) and evaluates
 * it at the subcell barycentres (lh_ic, nullable) as initialize does
 * (Euler/initialize.f90:262-307), on the host.  params: up to 32 doubles. */
int aderdg_project_initial_condition(const aderdg_config* cfg, int ic, const double* params, double* uh, double* lh_ic);
/* The same on the device: the context's uh from the initial field, then the
 * initial limiter (aderdg_upload + aderdg_init_limiter without host arrays).
 * Values agree with the host set-up up to the rounding of transcendental
 * functions by the device math library. */
int aderdg_initial_condition(aderdg_ctx* ctx, int ic, const double* params, int* n_limited);
/* Batch admission with the initial field evaluated on the device (no host
 * projection, no host-to-device copy of uh / lh_ic); as aderdg_batch_admit. */
int aderdg_batch_admit_ic(aderdg_batch* b, const aderdg_config* cfg, int ic, const double* params, double tend,
                          long max_steps, int* slot);

/* One-dimensional operators of degree N as built on the host
 * (Euler/initialize.f90:88-213), column-major.  Returns the element count. */
enum aderdg_operator_id {
  ADERDG_OP_XI = 0, ADERDG_OP_W, ADERDG_OP_KXI, ADERDG_OP_DUDX, ADERDG_OP_IK1, ADERDG_OP_F0,
  ADERDG_OP_FL, ADERDG_OP_FR, ADERDG_OP_UH2LIM, ADERDG_OP_LIM2UH, ADERDG_OP_UH2LOB, ADERDG_OP_XILIMBARY
};
int aderdg_operator(int N, int which, double* out);

/* The time step of aderdg_calc_time_step for callers that cannot allocate
 * device memory (a host framework owns every device allocation, or an
 * allocation's implicit synchronisation is not allowed).  No counterpart in
 * the reference: it exists for such embedders.  uh is the caller's device
 * copy of uh(nVar,N+1,N+1,IMAX,JMAX), dt a caller-owned device double that
 * receives dt, stream a cudaStream_t (NULL: the legacy default stream).  It
 * allocates nothing: its scratch is a fixed device array inside the library
 * (8193 x 8 bytes, held by every GPU that loads the library until exit),
 * which limits grids to 2,097,152 cells; larger grids return ADERDG_ENOSPACE.
 * The first call on each device looks up that array's address (make it before
 * any stream capture).  Calls share the array: calls whose kernels overlap on
 * the GPU race, so serialise them. */
int aderdg_calc_time_step_noalloc(const aderdg_config* cfg, const double* uh, double time, double tend, double* dt,
                                  void* stream);

/* ---- tuning ----
 * Kernel shapes of the FP32 modes, per (system, N, precision), as picked by
 * the tuner (ader-dg_gb300/aderdg/tuner.py times every candidate on the GPU
 * and stores its table in a JSON file that the Python package applies when it
 * loads this library).  No counterpart in the reference, whose shapes are its
 * compile-time parameters (Euler/ader_dg.f90:17-20).  All zero selects the
 * hand-measured defaults.  The cell-kernel and subcell shapes change no
 * result; the predictor shapes change results by FP32 rounding (each is
 * compiled with fused multiply-adds, which the compiler may group
 * differently).  Contexts and batches read
 * the table when they launch; a CUDA graph captured earlier keeps the shapes
 * it was captured with, so set the table before the first step. */
typedef struct aderdg_tuning {
  int predictor;      /* FP32 predictor: 0 default, 1 twice the cells per CTA, 2 half,
                         3 one more CTA per SM for the register allocation,
                         4 middle Picard iterations unrolled, 5 per-node contractions */
  int cells;          /* FP32-mode cell kernel: 0 default CTA, 1 twice its size, 2 half */
  int subcell_per_sm; /* subcell re-solve CTAs per SM; 0: as many as fit */
} aderdg_tuning;
int aderdg_set_tuning(int system, int N, int precision, const aderdg_tuning* t);
int aderdg_get_tuning(int system, int N, int precision, aderdg_tuning* t);
/* Numbers of predictor and cell-kernel candidates. */
int aderdg_tuning_variants(int* n_predictor, int* n_cells);

/* Measured device peaks for roofline reporting: FP64 and FP32 FMA throughput
 * (GFLOP/s) from dependent-FMA microkernels on the current device. */
int aderdg_probe_peaks(double* fp64_gflops, double* fp32_gflops);
/* Accuracy check of the FP32-mixed mode's FP64 reciprocal and square root
 * (Newton-refined hardware approximations): for each of the n inputs x[i],
 * out[4i..4i+3] = refined 1/x, correctly rounded 1/x, refined sqrt(x),
 * correctly rounded sqrt(x), evaluated on the current device.  No reference
 * counterpart. */
int aderdg_probe_math(int n, const double* x, double* out);

/* Page-locked host memory for the host side of uploads and downloads
 * (aderdg_upload / aderdg_download / aderdg_batch_download and friends copy
 * at the interconnect's full rate from and into it; pageable buffers go
 * through a staging copy).  Not part of the reference's interface: its arrays
 * are Fortran allocatables, which a caller may keep using. */
int aderdg_host_alloc(size_t bytes, void** ptr);
int aderdg_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif
