// common.cuh -- device-side types shared by the ADER-DG kernels.
//
// Device layout (HBM), per batch of instances (one instance = one grid):
//   cells of all instances are numbered globally; instance k owns the cell
//   range [cell_base, cell_base + imax*jmax), cell = i + imax*j inside it.
//   uh      [cell][P*P nodes][V]   FP64, exactly the Fortran uh(v,i,j,I,J)
//   duh     [cell][P*P][V]         FP64 (FP32 in the FP32 modes)
//   qbnd    [cell][4][P][V]        face-major: a face's P points contiguous
//   fbnd    [cell][4][P][V]        (AD: gradQbnd [cell][4][P][2][V]); the API's
//                                  get/set give the reference's qbnd(v,face,l,I,J)
//   fu/gu   x faces [fx_base + i + (imax+1)*j][P][V], y faces [fy_base + i + imax*j][P][V]
//           (FP32 in the FP32 modes)
//   lh      [cell][S*S][V]         subcell state of limited cells
//   mm      [cell][2][V]           per-cell min/max for the DMP neighbourhood
//   mme     [cell][V]              FP32-mixed: a bound on the error of mm (0: exact FP64 value)
#pragma once

#include <cstdint>

namespace aderdg {

enum SysId { kSysAD = 0, kSysEuler = 1, kSysBN = 2 };

// Modes of the cell kernel K3 (cells.cuh).
enum CellMode { kCellFused = 0, kCellSurface = 1, kCellUpdate = 2, kCellPrime = 3, kCellInitDmp = 4, kCellCfl = 5,
                kCellPrimeLimited = 6 };

// Physical parameters of one instance.
struct Phys {
  double gamma;                // Euler
  double gs, gg, ps, pg;       // Baer-Nunziato
  double cx, cy, a;            // advection-diffusion
  int ad_fused;                // 1: convective + viscous flux in the AD predictor
  // the FP32-mixed mode's FP32 constants (Sys::FConst), rounded once on the
  // host: Euler (gamma - 1, gamma); Baer-Nunziato (gs, gg, gs - 1, gg - 1,
  // gs ps, gg pg, ps, pg)
  float f32c[8];
};

// Read-only description of one instance.
struct InstDesc {
  int imax, jmax;
  long long cell_base;
  long long fx_base, fy_base;  // first x face / y face
  double dx, dy;
  float idxf, idyf;            // 1/dx, 1/dy in FP32 (FP32-mixed CFL)
  double xl0, xl1;
  int bc[4];
  int bc_mode;
  double cfl_pnpm;             // CFL * PNPMTable(N)
  Phys ph;
  // advection-diffusion: constants of the instance formed once on the host in
  // the reference's FP64 operation order (equal to the per-point values bit for
  // bit): the face dissipation smax per direction (PDEViscLLFRiemannSolver,
  // Advection-Diffusion/pde.f90:121-152) and the CFL denominator of every node
  // (Advection-Diffusion/calc_time_step.f90:37-50)
  double ad_smax[2];
  double ad_denom;
};

// Mutable per-instance state, device resident.
struct InstState {
  double time, dt, tend;
  unsigned long long denom_bits;     // max over nodes of sum_d lambda_max/dx_d (positive double bits)
  unsigned long long denom_next;     // accumulator for the next step
  int active;                        // 1 while time < tend
  int n_recompute;                   // troubled cells of the last step (nRecompute)
  int n_settled;                     // FP32-mixed: DMP decisions of the last step settled from FP64 values
  int n_list;                        // cells the last step's limiter re-solved (recompute > 0)
  int nonfinite;                     // set when dt came out non-finite
  long long steps;
  long long max_steps;               // > 0: stop after this many steps
};

// Host-computed constants of the face kernel (transcendentals are evaluated
// once on the host so every device value matches the host's libm).
struct FaceConst {
  double Va[4], Vb[4];  // double Mach reflection inflow / ambient primitive states
  double xsw0, xsw1;    // shock position x_sw = xsw0 + xsw1 * t (Euler/riemann_problem.f90:1-8)
  double pi;            // 4 atan(1)
  double xi[10];        // Gauss-Legendre nodes (AD Dirichlet boundary)
};

// Operators for degree N in compute precision R (predictor) and FP64 (rest).
template <int N, class R>
struct DevOps {
  static constexpr int P = N + 1, S = 2 * N + 1;
  R w[P];
  R Kxi[P * P];      // Kxi(k,i) at [k + P*i]
  R dudx[P * P];     // dudx(a,b) at [a + P*b]
  R T[P * P];        // T(l',l) = iK1(l',l)*w(l) at [l' + P*l]
  R g[P];            // sum_l iK1(l',l)*F0(l)
  R ts[P];           // sum_l T(l',l)
  R tw[P];           // sum_l' w(l') T(l',l)
  R wg;              // sum_l' w(l') g(l')
  R FL[P], FR[P];
  double wd[P], FLd[P], FRd[P];
  float wf[P], FLf[P], FRf[P];  // FP32-mixed surface integral and update
  float iwwf[P * P];            // 1 / (w_i w_j) at [i + P*j]
  double xid[P];
  double uh2lim[S * P];  // (s,k) at [s + S*k]
  double lim2uh[P * S];  // (k,s) at [k + P*s]
  double uh2lob[P * P];  // (q,k) at [q + P*k]
  // FP32-mixed DMP: the projections in FP32, and a bound on their error:
  // |FP32 projection - exact projection| <= perr * max over the cell's nodes |uh|
  float uh2limf[S * P];
  float uh2lobf[P * P];
  float perr;
  // deviations d = fl(fl(uh) - ubar) formed in FP32 from the FP32-rounded
  // state: their rounding adds at most pdev * (|ubar| + 2 max|d|) to the projections
  float pdev;
};

// Arguments shared by all kernels of one (system, N) batch.  The state that
// lives across steps is double-buffered and selected per instance by the
// parity of its step counter: buffer [steps & 1] holds the state at the start
// of the step (the reference's olduh / Lh / oldstatus / lmin_old), buffer
// [(steps + 1) & 1] receives the new state.  A step therefore copies nothing,
// and a captured CUDA graph stays valid across replays.
struct BatchArgs {
  const InstDesc* inst;
  InstState* st;
  int ninst;
  long long ncells;
  long long nfx, nfy;                // total x / y faces
  double* uh[2];                     // uh [cell][P*P][V]
  double* duh;                       // FP32 storage in the FP32 modes
  void* qbnd;                        // R precision (predictor output)
  void* fbnd;                        // R precision; AD: gradQbnd
  double* fu;                        // BN: Fm; fu..gp FP32 storage in the FP32 modes
  double* gu;                        // BN: Gm
  double* fp;                        // BN only: Fp
  double* gp;                        // BN only: Gp
  // phase outputs (phase API only)
  double* qhi;
  double* fhi;
  double* shi;
  // limiter
  int* status[2];                    // limiter status per cell
  double* lh[2];                     // subcell data [cell][S*S][V]
  double* mm[2];                     // per-cell min/max [cell][2][V] (lmin_old/lmax_old)
  // FP32-mixed mode only (null otherwise): a bound on |mm - the FP64
  // reference-order min/max| per cell and variable [cell][V], 0 where mm holds
  // the FP64 value itself; double-buffered like mm.  The DMP decisions use it
  // to settle each comparison exactly (see k_cells / k_subcell).
  float* mme[2];
  double* lminmax;                   // neighbourhood lmin/lmax used by the DMP [cell][2][V]
  unsigned char* troubled;           // DMP failed after the update
  int* recompute;                    // 0, 1, 2
  int* list;                         // cells with recompute > 0
  int* list_count;                   // [0]: entries of list, [1]: entries of settle
  int* settle;                       // FP32-mixed only (null otherwise): cells whose DMP
                                     // decision k_settle takes from FP64 values
  double* denom;                     // per-cell CFL denominator
  const double* lh_ic;               // initial-limiter candidates
  int mode;                          // kernel mode switch
  long long cell0;                   // first cell of a launch over part of the cell range (K1, K3)
  int only_inst;                     // >= 0: the priming modes of K3 touch this instance only
};

__device__ __forceinline__ int parity(const InstState& s) { return (int)(s.steps & 1); }

// Locate the instance owning a global cell (binary search on cell_base, the
// table sorted by it); -1 when the cell lies in no instance (instances of a
// batch occupy ranges of a shared pool, with gaps between them).
__device__ __forceinline__ int find_inst_cell(const InstDesc* inst, int n, long long cell) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (inst[mid].cell_base <= cell) lo = mid; else hi = mid - 1;
  }
  const InstDesc& d = inst[lo];
  if (cell < d.cell_base || cell - d.cell_base >= (long long)d.imax * d.jmax) return -1;
  return lo;
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

}  // namespace aderdg
