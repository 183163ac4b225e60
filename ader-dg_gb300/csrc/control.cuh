// control.cuh -- per-instance step control on the device.
//
// The time step of the reference (calc_time_step.f90) is
//   dt = min over nodes of CFL*PNPM(N) / denom,  clipped to tend - time,
// starting from dt = 1e20.  Division by a positive number is monotone, so
// the minimum of the quotients equals CFL*PNPM(N) / max(denom) exactly; the
// kernels fold max(denom) with an atomic max on the bit pattern (positive
// doubles order like their bits) and this kernel forms the quotient.
#pragma once

#include "common.cuh"

namespace aderdg {

enum CtlMode {
  kCtlBegin = 0,        // start of a fused step: dt from denom_bits, reset accumulators
  kCtlEnd = 1,          // end of a step: time += dt, parity flip, denom_bits = denom_next
  kCtlPrimeReset = 2,   // before a priming pass: clear denom_next and counters
  kCtlPrimeCommit = 3,  // after a priming pass: denom_bits = denom_next
  kCtlCalcDt = 4        // phase API calc_time_step: dt from denom_next, time/tend from the state
};

__device__ __forceinline__ double dt_from_denom(double cfl_pnpm, double maxd) {
  double dt = 1.0e20;
  const double q = cfl_pnpm / maxd;  // +inf when maxd == 0, as CFL*PNPM/0 in the reference
  dt = fmin(dt, q);
  return dt;
}

// only >= 0: the priming modes (reset, commit) act on that instance alone
static __global__ void k_control(InstDesc* inst, InstState* st, int ninst, int* list_count, int mode, int only) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0 && list_count && (mode == kCtlBegin || (mode == kCtlPrimeReset && only < 0))) list_count[0] = 0;
  // the settle list serves one cell-kernel pass at a time: every pass that
  // fills it follows a begin or a priming reset on the same stream
  if (k == 0 && list_count && (mode == kCtlBegin || mode == kCtlPrimeReset)) list_count[1] = 0;
  if (k >= ninst) return;
  if (only >= 0 && k != only) return;
  InstState& s = st[k];
  switch (mode) {
    case kCtlBegin: {
      s.denom_next = 0ull;
      s.n_recompute = 0;
      s.n_settled = 0;
      s.n_list = 0;
      const double maxd = __longlong_as_double((long long)s.denom_bits);
      // a NaN denominator anywhere folds to the largest bit pattern
      if (isnan(maxd)) s.nonfinite = 1;
      const bool budget = s.max_steps <= 0 || s.steps < s.max_steps;
      if (s.time < s.tend && !s.nonfinite && budget) {
        double dt = dt_from_denom(inst[k].cfl_pnpm, maxd);
        if (s.time + dt > s.tend) dt = s.tend - s.time;
        if (!isfinite(dt) || !(dt > 0.0)) {
          s.nonfinite = 1;
          s.active = 0;
          s.dt = 0.0;
        } else {
          s.dt = dt;
          s.active = 1;
        }
      } else {
        s.active = 0;
        s.dt = 0.0;
      }
      break;
    }
    case kCtlEnd:
      if (s.active) {
        s.time = s.time + s.dt;
        s.steps += 1;
        s.denom_bits = s.denom_next;
      }
      s.active = 0;
      break;
    case kCtlPrimeReset:
      s.denom_next = 0ull;
      s.n_recompute = 0;
      s.n_settled = 0;
      break;
    case kCtlPrimeCommit:
      s.denom_bits = s.denom_next;
      break;
    case kCtlCalcDt: {
      double dt = dt_from_denom(inst[k].cfl_pnpm, __longlong_as_double((long long)s.denom_next));
      if (s.time + dt > s.tend) dt = s.tend - s.time;
      s.dt = dt;
      s.active = 1;
      break;
    }
  }
}

}  // namespace aderdg
