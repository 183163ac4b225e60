/*
 * oracle.h -- C interface of the CPU oracle for the ADER-DG time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a line-by-line FP64 C++
 * restatement of the dasikasunder/ADER-DG Fortran solvers
 * (Advection-Diffusion/, Euler/, Baer-Nunziato/).  Only tests/, the smoke()
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py may load
 * it; the product library never links or calls it.
 *
 * PARITY UNPINNED: the reference ships no tests, golden vectors or fixtures,
 * and no Fortran compiler exists on either build machine, so this
 * restatement cannot be checked against the reference's own outputs.  It is
 * pinned instead by mathematical known-answer tests (operator identities,
 * free-stream preservation, conservation, exact solutions, convergence order).
 *
 * Layouts are the reference's Fortran column-major layouts, first index
 * fastest, zero-based here:
 *   uh(nVar, N+1, N+1, IMAX, JMAX), Lh(nVar, 2N+1, 2N+1, IMAX, JMAX), ...
 */
#ifndef ADERDG_ORACLE_H
#define ADERDG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_SYS_ADVDIFF = 0,
  ORC_SYS_EULER = 1,
  ORC_SYS_BN = 2
};

typedef struct oracle_config {
  int system;          /* ORC_SYS_* */
  int N;               /* polynomial degree 1..5 */
  int imax, jmax;
  double xl[2], xr[2];
  int bc[4];           /* left, right, bottom, top: 1 transmissive/Neumann, 2 AD Dirichlet, 3 periodic */
  int bc_mode;         /* 0 = per-side codes, 1 = Euler double Mach reflection (as shipped) */
  double cfl;          /* reference CFL parameter (0.9) */
  double gamma;        /* Euler */
  double gamma_s, gamma_g, pi_s, pi_g; /* Baer-Nunziato stiffened gas */
  double cx, cy, a;    /* advection-diffusion */
  int ad_flux_mode;    /* 0 = viscous flux only in the predictor (reference), 1 = fused */
  int limiter;         /* 1 = a-posteriori subcell limiter on (Euler/BN, N>0) */
} oracle_config;

/* which-codes for oracle_get_array */
enum {
  ORC_UH = 0, ORC_OLDUH, ORC_DUH, ORC_QHI, ORC_FHI, ORC_SHI, ORC_QBND, ORC_FBND,
  ORC_GRADQBND, ORC_FU, ORC_GU, ORC_FM, ORC_FP, ORC_GM, ORC_GP, ORC_LH, ORC_NEWLH,
  ORC_LMIN, ORC_LMAX, ORC_LMIN_OLD, ORC_LMAX_OLD
};
/* which-codes for oracle_get_int_array */
enum { ORC_RECOMPUTE = 0, ORC_STATUS, ORC_OLDSTATUS };
/* which-codes for oracle_get_operator */
enum {
  ORC_OP_XI = 0, ORC_OP_W, ORC_OP_MM, ORC_OP_IMM, ORC_OP_KXI, ORC_OP_DUDX, ORC_OP_F0,
  ORC_OP_K1, ORC_OP_IK1, ORC_OP_FL, ORC_OP_FR, ORC_OP_UH2LIM, ORC_OP_LIM2UH,
  ORC_OP_UH2LOB, ORC_OP_XILOB, ORC_OP_WLOB, ORC_OP_XILIMBARY
};

void* oracle_create(const oracle_config* cfg);
void oracle_destroy(void* h);
long oracle_array_size(void* h, int which);
int oracle_set_uh(void* h, const double* uh);
int oracle_get_array(void* h, int which, double* out);
int oracle_set_array(void* h, int which, const double* in);
int oracle_get_int_array(void* h, int which, int* out);
int oracle_set_int_array(void* h, int which, const int* in);
int oracle_get_operator(void* h, int which, double* out);

/* initialize.f90 limiter block: DMP with argmax 0.1 against the cell's own
 * nodal min/max; failing cells get status 1 and Lh = lh_ic (the initial
 * field at the subcell barycentres, NULL = leave Lh untouched). */
int oracle_init_limiter(void* h, const double* lh_ic);

/* phases of one loop body of main.f90 */
double oracle_calc_time_step(void* h, double time, double tend);
void oracle_set_dt(void* h, double dt);
void oracle_set_time(void* h, double time);
void oracle_get_min_max(void* h);
void oracle_save_olduh(void* h);
void oracle_predictor(void* h);
void oracle_volume_integral(void* h);
void oracle_riemann(void* h);
void oracle_surface_integral(void* h);
int oracle_element_update(void* h);   /* + DMP when the limiter is on; returns nRecompute */
void oracle_limiter(void* h);         /* spread_recompute, allocate_limiter, subcell_recompute, update_limiter */

/* one full loop body; returns nRecompute; advances *time by the step's dt */
int oracle_step(void* h, double* time, double tend, double* dt_out);

/* initial fields (setup patches, host only) -- evaluate at one point */
enum {
  ORC_IC_AD_ZERO = 0, ORC_IC_AD_SINE = 1,
  ORC_IC_EULER_DMR = 10, ORC_IC_EULER_VORTEX = 11, ORC_IC_EULER_RP2D = 12,
  ORC_IC_BN_RP1D = 20, ORC_IC_BN_CYLINDER = 21
};
int oracle_initial_field(const oracle_config* cfg, int ic, const double* p, double x, double y, double* u0);
/* fill uh at the Gauss-Legendre nodes and lh_ic at subcell barycentres (lh_ic may be NULL) */
int oracle_project_ic(void* h, int ic, const double* p, double* uh, double* lh_ic);

#ifdef __cplusplus
}
#endif
#endif
