// cells.cuh -- K3: surface integral + element update + DMP / positivity
// detection + CFL partials, one thread per spatial node, CPB cells per CTA.
//
// Reference: surface_integral.f90:8-39, element_update.f90:8-30, the DMP of
// Euler/limiter.f90:179-245 (called from Euler/main.f90:74-88), the per-cell
// part of get_min_max (Euler/limiter.f90:115-143) for the next step, and the
// node loop of calc_time_step.f90.  Compiled with --fmad=false: all values
// follow the reference's FP64 operation order.
//
// Modes (BatchArgs::mode):
//   kCellFused   surface + update + [DMP, next min/max] + CFL partials
//   kCellSurface surface integral only (phase API)
//   kCellUpdate  update + [DMP, next min/max] + CFL partials (phase API)
//   kCellPrime   min/max of the current state for the DMP neighbourhood
//                (get_min_max step 1) + CFL denominators; no update
//   kCellInitDmp initial limiter: DMP with argmax 0.1 against the cell's own
//                nodal min/max; failing cells take the initial subcell data
//   kCellCfl     CFL denominators of the current state only
//   kCellPrimeLimited  kCellPrime for the limited cells only (their min/max
//                come from Lh), no CFL: after the initial limiter, where the
//                other cells' min/max and the CFL are those of kCellPrime
#pragma once

#include "common.cuh"
#include "physics.cuh"

namespace aderdg {

#define kInf __longlong_as_double(0x7ff0000000000000LL)

// Doubles mapped to integers of the same order (negative values have their
// magnitude bits flipped), so min/max run on the integer pipe instead of the
// FP64 pipe; the value returned is one of the inputs, as with fmin/fmax.
__device__ __forceinline__ long long okey(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double okey_inv(long long k) {
  return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffLL));
}

// Subcell / Gauss-Lobatto projections of one cell (get_subcell_data and
// get_lobatto_data, Euler/limiter.f90:12-68), sum-factorised y then x with
// the reference's summation order.  A "team" of nr threads with rank r works
// on one cell; the caller synchronises between the two passes.  The operators
// come from shared memory: lim = uh2lim (s,k) at [s + S*k], lob = uh2lob (q,k)
// at [q + P*k].  T = double: exact-order mul then add, or one fused
// multiply-add per term (kFast); T = float: fused multiply-adds (the FP32 modes).
template <int N, int V, class T>
struct Proj {
  static constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1;
  template <bool kFast>
  __device__ __forceinline__ static T madd(T acc, T a, T b) {
    if constexpr (kFast) return fma(a, b, acc);
    // reference order: a rounded product, then a rounded sum, also in the
    // translation units compiled with fused multiply-adds
    else if constexpr (sizeof(T) == 8) return __dadd_rn(acc, __dmul_rn(a, b));
    else return acc + a * b;
  }
  // y pass: LY[v][s][i] = sum_k U[v][i + P k] uh2lim(s,k); LB[v][s][i] likewise with uh2lob
  template <bool kFast = false>
  __device__ static void ypass(const T* U, T* LY, T* LB, const T* lim, const T* lob, int r, int nr) {
    for (int idx = r; idx < P * S; idx += nr) {
      const int ii = idx % P, s = idx / P;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        T acc = 0;
#pragma unroll
        for (int k = 0; k < P; ++k) acc = madd<kFast>(acc, U[v * P2 + ii + P * k], lim[s + S * k]);
        LY[(v * S + s) * P + ii] = acc;
      }
    }
    for (int idx = r; idx < P * P; idx += nr) {
      const int ii = idx % P, s = idx / P;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        T acc = 0;
#pragma unroll
        for (int k = 0; k < P; ++k) acc = madd<kFast>(acc, U[v * P2 + ii + P * k], lob[s + P * k]);
        LB[(v * P + s) * P + ii] = acc;
      }
    }
  }
  // subcell value (s1, s2) from the y pass
  template <bool kFast = false>
  __device__ static void subcell(const T* LY, const T* lim, int s1, int s2, T* out) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      T acc = 0;
#pragma unroll
      for (int k = 0; k < P; ++k) acc = madd<kFast>(acc, LY[(v * S + s2) * P + k], lim[s1 + S * k]);
      out[v] = acc;
    }
  }
  template <bool kFast = false>
  __device__ static void lobatto(const T* LB, const T* lob, int s1, int s2, T* out) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      T acc = 0;
#pragma unroll
      for (int k = 0; k < P; ++k) acc = madd<kFast>(acc, LB[(v * P + s2) * P + k], lob[s1 + P * k]);
      out[v] = acc;
    }
  }
  // x pass fused with min/max (integer keys) and the positivity test of every subcell (FP64)
  template <class Sys, bool kFast = false>
  __device__ static void xpass_minmax(const T* U, const T* LY, const T* LB, const T* lim, const T* lob,
                                      const Phys& ph, int r, int nr, T* mn, T* mx, bool& posfail) {
    T val[V];
    long long kmn[V], kmx[V];
#pragma unroll
    for (int v = 0; v < V; ++v) { kmn[v] = okey(mn[v]); kmx[v] = okey(mx[v]); }
    for (int idx = r; idx < S * S; idx += nr) {
      subcell<kFast>(LY, lim, idx % S, idx / S, val);
#pragma unroll
      for (int v = 0; v < V; ++v) { const long long k = okey(val[v]); kmn[v] = min(kmn[v], k); kmx[v] = max(kmx[v], k); }
      if constexpr (Sys::ID != kSysAD) {
        if (!Sys::positive_fast(ph, val)) posfail = true;
      }
    }
    for (int idx = r; idx < P * P; idx += nr) {
      lobatto<kFast>(LB, lob, idx % P, idx / P, val);
#pragma unroll
      for (int v = 0; v < V; ++v) { const long long k = okey(val[v]); kmn[v] = min(kmn[v], k); kmx[v] = max(kmx[v], k); }
    }
    for (int idx = r; idx < P2; idx += nr) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const long long k = okey(U[v * P2 + idx]);
        kmn[v] = min(kmn[v], k);
        kmx[v] = max(kmx[v], k);
      }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) { mn[v] = okey_inv(kmn[v]); mx[v] = okey_inv(kmx[v]); }
  }
  // FP32 x pass fused with min/max and the admissibility test.  The y pass
  // ran on the deviations d = uh - ubar from a reference state ubar of the
  // cell (the projections reproduce constants, so proj(uh) = ubar + proj(d));
  // min/max are of the projected deviations.  A subcell whose FP32 value
  // ubar + proj(d) is not clearly admissible (err = the error bound of
  // proj(d), plus the rounding of ubar to FP32) is projected again in FP64
  // from U64, in the reference's order (y pass, then x), and tested exactly:
  // the value and the decision are those of the FP64 path bit for bit.
  template <class Sys>
  __device__ static void xpass_minmax_f32(const float* LY, const float* LB, const float* lim, const float* lob,
                                          const double* U64, const double* lim64,
                                          const typename Sys::FConst& fc, const float* err, const float* ubf,
                                          const Phys& ph, int r, int nr, float* mn, float* mx, bool& posfail) {
    float val[V], q[V], e[V];
#pragma unroll
    for (int v = 0; v < V; ++v) e[v] = err[v] + 2.5e-7f * fabsf(ubf[v]);
    unsigned open = 0u;  // bit it: the it-th subcell of this thread needs the FP64 test
    int it = 0;
    for (int idx = r; idx < S * S; idx += nr, ++it) {
      subcell<true>(LY, lim, idx % S, idx / S, val);
#pragma unroll
      for (int v = 0; v < V; ++v) { mn[v] = fminf(mn[v], val[v]); mx[v] = fmaxf(mx[v], val[v]); }
      if constexpr (Sys::ID != kSysAD) {
#pragma unroll
        for (int v = 0; v < V; ++v) q[v] = ubf[v] + val[v];
        if (!Sys::admissible_box_f32(fc, q, e)) open |= 1u << it;
      }
    }
    for (int idx = r; idx < P * P; idx += nr) {
      lobatto<true>(LB, lob, idx % P, idx / P, val);
#pragma unroll
      for (int v = 0; v < V; ++v) { mn[v] = fminf(mn[v], val[v]); mx[v] = fmaxf(mx[v], val[v]); }
    }
    // the subcells left open, in FP64 in the reference's order (the y pass
    // of get_subcell_data, then x; lim64 = uh2lim (s,k) at [s + S*k]): the
    // FP64 path's value and decision bit for bit
    if constexpr (Sys::ID != kSysAD) while (open) {
      const int idx = r + (__ffs(open) - 1) * nr;
      open &= open - 1u;
      const int s1 = idx % S, s2 = idx / S;
      double qd[V];
#pragma unroll 1
      for (int v = 0; v < V; ++v) {
        double acc = 0.0;
#pragma unroll 1
        for (int k = 0; k < P; ++k) {
          double ly = 0.0;
          for (int m = 0; m < P; ++m) ly = ly + U64[v * P2 + k + P * m] * lim64[s2 + S * m];
          acc = acc + ly * lim64[s1 + S * k];
        }
        qd[v] = acc;
      }
      if (!Sys::positive(ph, qd)) posfail = true;
    }
  }
};

// Voronoi neighbour index along one axis (Euler/initialize.f90:219-258):
// periodic sides wrap, all others clamp.
__device__ __forceinline__ int nb_index(int x, int d, int n, int bc_lo, int bc_hi) {
  int y = x + d;
  if (y < 0) y = (bc_lo == 3) ? n - 1 : 0;
  if (y > n - 1) y = (bc_hi == 3) ? 0 : n - 1;
  return y;
}

// CFL denominator at one node (calc_time_step.f90: Euler/BN :31-45, AD :37-50)
template <class Sys, int N>
__device__ __forceinline__ double cfl_denom(const InstDesc& in, const double* Q) {
  if constexpr (Sys::ID == kSysAD) {
    // (|c_x| + 2 a (2N+1)/dx)/dx + (|c_y| + 2 a (2N+1)/dy)/dy, the same at every
    // node: formed on the host in this order
    return in.ad_denom;
  } else {
    double ex, ey;
    Sys::max_eig2(in.ph, Q, ex, ey);
    double denom = 0.0;
    denom = denom + ex / in.dx;
    denom = denom + ey / in.dy;
    return denom;
  }
}
// FP32-mixed: eigenvalues and the node's denominator in FP32 (the maximum
// over nodes, and dt, in FP64); states whose FP32 pressure is not settled
// take the FP64 evaluation on Qd
template <class Sys, int N>
__device__ __forceinline__ double cfl_denom_f32(const InstDesc& in, const typename Sys::FConst& fc, const float* q,
                                                const double* Qd) {
  if constexpr (Sys::ID == kSysAD) {
    return cfl_denom<Sys, N>(in, nullptr);
  } else {
    float ex, ey;
    if (Sys::max_eig2_f32(fc, q, ex, ey)) return (double)(ex * in.idxf + ey * in.idyf);
    return cfl_denom<Sys, N>(in, Qd);
  }
}

// Maximum over the P2 lanes of a cell when every cell is an aligned segment
// of a warp (P2 = 4 or 16): xor shuffles within the segment; every lane of the
// warp must call it.
template <int P2>
__device__ __forceinline__ unsigned seg_max(unsigned x) {
#pragma unroll
  for (int o = P2 / 2; o > 0; o >>= 1) {
    const unsigned y = __shfl_xor_sync(0xffffffffu, x, o, P2);
    x = x > y ? x : y;
  }
  return x;
}
template <int P2>
__device__ __forceinline__ unsigned long long seg_max(unsigned long long x) {
#pragma unroll
  for (int o = P2 / 2; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o, P2);
    x = x > y ? x : y;
  }
  return x;
}

// VAR: the CTA size the tuner (aderdg/tuner.py) picks for the FP32 modes: 0
// the default below, 1 twice, 2 half of it
constexpr int kCellVariants = 3;
template <class Sys, int N, int VAR = 0>
struct CellCfg {
  static constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V;
  // small CTAs (the kernel waits on latency and barriers: smaller CTAs, more
  // of them per SM, wait on fewer warps per barrier): 64 threads up to N = 3,
  // 128 at N = 4 and 256 at N = 5, where the 25- and 36-thread cells fill
  // smaller CTAs badly (measured: BN cylinder 0.559 -> 0.508 -> 0.487 ms,
  // Riemann problem 0.344 -> 0.330 -> 0.324 ms for 256 -> 128 -> 64 threads)
  static constexpr int CTA0 = N == 5 ? 256 : N == 4 ? 128 : 64;
  static constexpr int CTA = VAR == 1 ? 2 * CTA0 : VAR == 2 ? (CTA0 / 2 < 32 ? 32 : CTA0 / 2) : CTA0;
  static constexpr int CPB = (CTA / P2) < 1 ? 1 : (CTA / P2);
  static constexpr int THREADS = ((CPB * P2 + 31) / 32) * 32;
  // per cell: U [V][P2], LY [V][S][P], LB [V][P][P], red [2][V][P2] (FP64);
  // FP32-mixed: U64 [V][P2] then FP32 U [V][P2], LY, LB, red, |U| max [V]
  // in the same room
  static constexpr int CELL_DBL = V * P2 + V * S * P + V * P * P + 2 * V * P2;
  static_assert(8 * V * P2 + 4 * (3 * V * P2 + V * S * P + V * P * P) <= 8 * CELL_DBL, "FP32 cell layout");
  static constexpr int OPS_DBL = S * P + P * P;  // uh2lim, uh2lob (FP64, then FP32 in the FP32 modes)
  static constexpr int SMEM_BYTES = CPB * CELL_DBL * 8 + OPS_DBL * 12 + CPB * 8 /*cell max*/ + CPB * 4 /*flags*/ +
                                    CPB * V * 4 /*|U| max*/ + CPB * V * 4 /*FP32 reference state*/ + 16;
  // blocks per SM the register allocation aims at, in 256-thread units:
  // Euler's FP32-mixed cell kernel is latency-bound and gains from a fourth;
  // the other variants keep the allocation they reach unconstrained
  static constexpr int min_blocks(bool fast) {
    return (Sys::ID == kSysEuler ? (fast ? 4 : 3) : (Sys::ID == kSysBN ? 2 : 4)) * 256 / CTA < 1
               ? 1
               : (Sys::ID == kSysEuler ? (fast ? 4 : 3) : (Sys::ID == kSysBN ? 2 : 4)) * 256 / CTA;
  }
};

template <class Sys, int N, bool kFast, int VAR = 0>
__global__ void __launch_bounds__(CellCfg<Sys, N, VAR>::THREADS, CellCfg<Sys, N, VAR>::min_blocks(kFast))
    k_cells(BatchArgs a, DevOps<N, double> op) {
  using C = CellCfg<Sys, N, VAR>;
  constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V, CPB = C::CPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sm = reinterpret_cast<double*>(smem_raw);
  double* opsm = sm + CPB * C::CELL_DBL;
  float* opsf = reinterpret_cast<float*>(opsm + C::OPS_DBL);
  unsigned long long* cmax = reinterpret_cast<unsigned long long*>(opsf + C::OPS_DBL + (C::OPS_DBL & 1));
  int* cflag = reinterpret_cast<int*>(cmax + CPB);
  unsigned* amax_all = reinterpret_cast<unsigned*>(cflag + CPB);  // [CPB][V]
  float* ubs_all = reinterpret_cast<float*>(amax_all + CPB * V);  // [CPB][V]

  const int mode = a.mode;
  const int t = threadIdx.x;
  const int lc = t / P2;
  const int node = t - lc * P2;
  const int i = node % P, j = node / P;
  const long long cell = a.cell0 + (long long)blockIdx.x * CPB + lc;
  const bool in_cta = lc < CPB;
  const int k_found = (in_cta && cell < a.ncells) ? find_inst_cell(a.inst, a.ninst, cell) : -1;
  const bool valid = k_found >= 0;
  const int kc = valid ? k_found : 0;
  const InstDesc& in = a.inst[kc];
  const InstState& st = a.st[kc];
  const bool priming = mode == kCellPrime || mode == kCellInitDmp || mode == kCellCfl || mode == kCellPrimeLimited;
  const bool act = valid && (priming ? (a.only_inst < 0 || kc == a.only_inst) : st.active != 0) &&
                   (mode != kCellPrimeLimited || a.status[parity(st)][cell] != 0);
  if (!__syncthreads_or(act)) return;  // nothing to do in this CTA
  const int par = parity(st);
  const long long lcell = cell - in.cell_base;
  const int ci = valid ? (int)(lcell % in.imax) : 0, cj = valid ? (int)(lcell / in.imax) : 0;
  const bool limiter = Sys::ID != kSysAD && a.mm[0] != nullptr;
  double* U = sm + (size_t)(in_cta ? lc : 0) * C::CELL_DBL;
  double* LY = U + V * P2;
  double* LB = LY + V * S * P;
  double* RED = LB + V * P * P;
  // FP32-mixed views of the same room
  float* Uf = reinterpret_cast<float*>(U + V * P2);
  float* LYf = Uf + V * P2;
  float* LBf = LYf + V * S * P;
  float* REDf = LBf + V * P * P;
  unsigned* amax = amax_all + (in_cta ? lc : 0) * V;
  float* ubs = ubs_all + (in_cta ? lc : 0) * V;

  // DMP neighbourhood bounds (get_min_max step 2, Euler/limiter.f90:147-167):
  // thread v < V of a cell folds its 3x3 Voronoi neighbourhood now, so the
  // global loads overlap the update and the projections
  double nlmin = 0.0, nlmax = 0.0;
  float nen = 0.0f;  // FP32-mixed: largest error bound of the folded min/max
  if (limiter && act && node < V && (mode == kCellFused || mode == kCellUpdate)) {
    const int v = node;
    const double* mmi = a.mm[par];
    nlmin = mmi[(size_t)cell * 2 * V + v];
    nlmax = mmi[(size_t)cell * 2 * V + V + v];
    if constexpr (kFast) {
      // integer-key min/max (the integer pipe, not FP64)
      long long kmn = okey(nlmin), kmx = okey(nlmax);
      const float* mei = a.mme[par];
#pragma unroll
      for (int jj = -1; jj <= 1; ++jj)
#pragma unroll
        for (int ii = -1; ii <= 1; ++ii) {
          const int in_ = nb_index(ci, ii, in.imax, in.bc[0], in.bc[1]);
          const int jn_ = nb_index(cj, jj, in.jmax, in.bc[2], in.bc[3]);
          const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
          kmn = min(kmn, okey(mmi[(size_t)nc * 2 * V + v]));
          kmx = max(kmx, okey(mmi[(size_t)nc * 2 * V + V + v]));
          if (mei) nen = fmaxf(nen, mei[(size_t)nc * V + v]);
        }
      nlmin = okey_inv(kmn);
      nlmax = okey_inv(kmx);
    } else {
#pragma unroll
      for (int jj = -1; jj <= 1; ++jj)
#pragma unroll
        for (int ii = -1; ii <= 1; ++ii) {
          const int in_ = nb_index(ci, ii, in.imax, in.bc[0], in.bc[1]);
          const int jn_ = nb_index(cj, jj, in.jmax, in.bc[2], in.bc[3]);
          const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
          nlmin = fmin(nlmin, mmi[(size_t)nc * 2 * V + v]);
          nlmax = fmax(nlmax, mmi[(size_t)nc * 2 * V + V + v]);
        }
    }
  }

  // projection operators into shared memory (lanes index them by subcell)
  for (int k = t; k < C::OPS_DBL; k += blockDim.x) {
    opsm[k] = k < S * P ? op.uh2lim[k] : op.uh2lob[k - S * P];
    if constexpr (kFast) opsf[k] = k < S * P ? op.uh2limf[k] : op.uh2lobf[k - S * P];
  }
  if (in_cta && node == 0) {
    cmax[lc] = 0ull;
    cflag[lc] = 0;
  }
  if (kFast && in_cta && node < V) {
    // the cell's FP32 reference state ubar: its start-of-step state at node 0, rounded to FP32
    amax[node] = 0u;
    ubs[node] = act ? (float)a.uh[par][(size_t)cell * P2 * V + node] : 0.0f;
  }
  __syncthreads();

  // ---------------------------------------------------------------- update
  double u[V];
  const size_t off = ((size_t)(valid ? cell : 0) * P2 + node) * V;
  if (act) {
    if (mode == kCellFused || mode == kCellSurface || mode == kCellUpdate) {
      const long long fxl = in.fx_base + ci + (long long)(in.imax + 1) * cj;
      const long long fyb = in.fy_base + ci + (long long)in.imax * cj;
      const long long fyt = fyb + in.imax;
      if constexpr (kFast) {
        // FP32-mixed: duh and the face fluxes are stored in FP32; the surface
        // contraction and the scaling by 1/(w_i w_j) in FP32, the update of
        // the FP64 state in FP64
        const float* D32 = reinterpret_cast<const float*>(a.duh);
        const float* XL = reinterpret_cast<const float*>(a.fu);
        const float* XR = reinterpret_cast<const float*>((Sys::ID == kSysBN) ? a.fp : a.fu);
        const float* YB = reinterpret_cast<const float*>(a.gu);
        const float* YT = reinterpret_cast<const float*>((Sys::ID == kSysBN) ? a.gp : a.gu);
        float d[V];
#pragma unroll
        for (int v = 0; v < V; ++v) d[v] = D32[off + v];
        if (mode != kCellUpdate) {
          const float cxf = op.wf[j] * in.idxf, cyf = op.wf[i] * in.idyf;
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float fl = XL[((size_t)fxl * P + j) * V + v], fr = XR[((size_t)(fxl + 1) * P + j) * V + v];
            const float gb = YB[((size_t)fyb * P + i) * V + v], gt = YT[((size_t)fyt * P + i) * V + v];
            const float sx = fr * op.FRf[i] - fl * op.FLf[i];
            const float sy = gt * op.FRf[j] - gb * op.FLf[j];
            d[v] = d[v] - (cxf * sx + cyf * sy);
          }
        }
        if (mode == kCellSurface) {
          float* D32w = reinterpret_cast<float*>(a.duh);
#pragma unroll
          for (int v = 0; v < V; ++v) D32w[off + v] = d[v];
        } else {
          const double dt = st.dt;
          const double* uo = a.uh[par] + off;
          double* un = a.uh[par ^ 1] + off;
          const float iw = op.iwwf[i + P * j];
#pragma unroll
          for (int v = 0; v < V; ++v) {
            u[v] = fma(dt, (double)(d[v] * iw), uo[v]);
            un[v] = u[v];
          }
        }
      } else {
        double d[V];
#pragma unroll
        for (int v = 0; v < V; ++v) d[v] = a.duh[off + v];
        if (mode != kCellUpdate) {
          // surface_integral.f90:20-35: x faces then y faces
          const double* XL = a.fu;
          const double* XR = (Sys::ID == kSysBN) ? a.fp : a.fu;
          const double* YB = a.gu;
          const double* YT = (Sys::ID == kSysBN) ? a.gp : a.gu;
          const double cx = op.wd[j] / in.dx, cy = op.wd[i] / in.dy;
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const double fl = XL[((size_t)fxl * P + j) * V + v], fr = XR[((size_t)(fxl + 1) * P + j) * V + v];
            d[v] = d[v] - cx * (fr * op.FRd[i] - fl * op.FLd[i]);
          }
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const double gb = YB[((size_t)fyb * P + i) * V + v], gt = YT[((size_t)fyt * P + i) * V + v];
            d[v] = d[v] - cy * (gt * op.FRd[j] - gb * op.FLd[j]);
          }
        }
        if (mode == kCellSurface) {
#pragma unroll
          for (int v = 0; v < V; ++v) a.duh[off + v] = d[v];
        } else {
          // element_update.f90:18-26
          const double dt = st.dt;
          const double* uo = a.uh[par] + off;
          double* un = a.uh[par ^ 1] + off;
#pragma unroll
          for (int v = 0; v < V; ++v) {
            d[v] = d[v] / (op.wd[i] * op.wd[j]);
            u[v] = uo[v] + dt * d[v];
            un[v] = u[v];
          }
        }
      }
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) u[v] = a.uh[par][off + v];
    }
  }
  if (mode == kCellSurface) return;  // uniform per launch: no barrier follows

  // FP32-mixed: the node's state in FP32, and its deviation from the cell's
  // FP32 reference state ubar, formed in FP32 (one conversion per value)
  float uf[V], du[V], ubf[V];
  if constexpr (kFast) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      ubf[v] = ubs[v];
      uf[v] = act ? (float)u[v] : 0.0f;
      du[v] = act ? uf[v] - ubf[v] : 0.0f;
    }
  }

  // ------------------------------------------------------------- CFL part
  const bool want_cfl = mode != kCellInitDmp && mode != kCellPrimeLimited;
  // cells as aligned warp segments: per-cell maxima by shuffles, one store per
  // cell instead of P2 atomics on one shared address
  constexpr bool kSeg = (32 % P2) == 0 && (C::THREADS % 32) == 0 && C::CPB * P2 == C::THREADS;
  if constexpr (kSeg && Sys::ID != kSysAD) {
    if (want_cfl) {
      unsigned long long bits = 0ull;
      if (act) {
        double dn;
        if constexpr (kFast) dn = cfl_denom_f32<Sys, N>(in, typename Sys::FConst(in.ph), uf, u);
        else dn = cfl_denom<Sys, N>(in, u);
        bits = (unsigned long long)__double_as_longlong(dn);
      }
      bits = seg_max<P2>(bits);
      if (act && node == 0) cmax[lc] = bits;
    }
  } else if (act && want_cfl) {
    double dn;
    if constexpr (kFast) dn = cfl_denom_f32<Sys, N>(in, typename Sys::FConst(in.ph), uf, u);
    else dn = cfl_denom<Sys, N>(in, u);
    // advection-diffusion: the denominator is the instance's constant, folded below
    if constexpr (Sys::ID != kSysAD) atomicMax(&cmax[lc], (unsigned long long)__double_as_longlong(dn));
  }

  // ------------------------------------------------------------- DMP part
  const bool want_dmp = limiter && mode != kCellCfl;
  if (want_dmp) {
    // Cells whose limiter is active keep their min/max from the subcell data
    // (get_min_max, Euler/limiter.f90:134-139) in the priming pass.
    const bool from_lh = act && (mode == kCellPrime || mode == kCellPrimeLimited) && a.status[par][valid ? cell : 0] != 0;
    bool f32red = false;  // the cell's partial min/max are in REDf (FP32)
    if constexpr (kFast) {
      if (act) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          U[v * P2 + node] = u[v];
          Uf[v * P2 + node] = du[v];
          if constexpr (!kSeg) atomicMax(&amax[v], __float_as_uint(fabsf(du[v])));
        }
      }
      if constexpr (kSeg) {
        // du = 0 in lanes of inactive cells
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const unsigned m = seg_max<P2>(__float_as_uint(fabsf(du[v])));
          if (act && node == 0) amax[v] = m;
        }
      }
      __syncthreads();
      // FP32 projections of the deviations when their error bound stays
      // within the DMP's absolute tolerance (1e-4) for every variable;
      // otherwise this cell takes the FP64 projections in the reference's
      // order (the FP64 path's values bit for bit).
      float err[V];
      bool f32ok = true;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float am = __uint_as_float(amax[v]);
        err[v] = op.perr * am + op.pdev * (fabsf(ubf[v]) + 2.0f * am);
        f32ok = f32ok && err[v] <= 1.0e-4f;
      }
      if (act && !from_lh) {
        if (f32ok) Proj<N, V, float>::template ypass<true>(Uf, LYf, LBf, opsf, opsf + S * P, node, P2);
        else Proj<N, V, double>::template ypass<false>(U, LY, LB, opsm, opsm + S * P, node, P2);
      }
      __syncthreads();
      bool posfail = false;
      if (act) {
        if (from_lh) {
          double mn[V], mx[V];
#pragma unroll
          for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
          const double* L = a.lh[par] + (size_t)cell * S * S * V;
          for (int idx = node; idx < S * S; idx += P2)
#pragma unroll
            for (int v = 0; v < V; ++v) { mn[v] = fmin(mn[v], L[idx * V + v]); mx[v] = fmax(mx[v], L[idx * V + v]); }
#pragma unroll
          for (int v = 0; v < V; ++v) {
            RED[v * P2 + node] = mn[v];
            RED[(V + v) * P2 + node] = mx[v];
          }
        } else if (f32ok) {
          float mn[V], mx[V];
#pragma unroll
          for (int v = 0; v < V; ++v) { mn[v] = du[v]; mx[v] = du[v]; }
          Proj<N, V, float>::template xpass_minmax_f32<Sys>(LYf, LBf, opsf, opsf + S * P, U, opsm,
                                                            typename Sys::FConst(in.ph), err, ubf, in.ph, node, P2,
                                                            mn, mx, posfail);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            REDf[v * P2 + node] = mn[v];
            REDf[(V + v) * P2 + node] = mx[v];
          }
        } else {
          double mn[V], mx[V];
#pragma unroll
          for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
          Proj<N, V, double>::template xpass_minmax<Sys, false>(U, LY, LB, opsm, opsm + S * P, in.ph, node, P2, mn, mx,
                                                                posfail);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            RED[v * P2 + node] = mn[v];
            RED[(V + v) * P2 + node] = mx[v];
          }
        }
        if (posfail) atomicOr(&cflag[lc], 1);
      }
      f32red = f32ok && !from_lh;
    } else {
      if (act) {
#pragma unroll
        for (int v = 0; v < V; ++v) U[v * P2 + node] = u[v];
      }
      __syncthreads();
      const double* lim = opsm;
      const double* lob = opsm + S * P;
      if (act && !from_lh) Proj<N, V, double>::template ypass<false>(U, LY, LB, lim, lob, node, P2);
      __syncthreads();
      double mn[V], mx[V];
      bool posfail = false;
#pragma unroll
      for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
      if (act) {
        if (from_lh) {
          const double* L = a.lh[par] + (size_t)cell * S * S * V;
          for (int idx = node; idx < S * S; idx += P2)
#pragma unroll
            for (int v = 0; v < V; ++v) { mn[v] = fmin(mn[v], L[idx * V + v]); mx[v] = fmax(mx[v], L[idx * V + v]); }
        } else {
          Proj<N, V, double>::template xpass_minmax<Sys, false>(U, LY, LB, lim, lob, in.ph, node, P2, mn, mx, posfail);
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
          RED[v * P2 + node] = mn[v];
          RED[(V + v) * P2 + node] = mx[v];
        }
        if (posfail) atomicOr(&cflag[lc], 1);
      }
    }
    __syncthreads();
    if (act && node < V) {
      const int v = node;
      double cmn, cmx;
      const double ubar = kFast ? (double)ubs[v] : 0.0;  // the cell's FP32 reference state (FP32-mixed)
      // FP32 projections: the cell's deviation min/max from its FP32 reference
      // state ubar, and a bound on |ubar + fmn - FP64 value| (and fmx): the
      // projections' bound as formed above (rounded up), plus the FP64
      // roundings of the reference-order values (generously 1e-12 relative)
      float fmn = 0.0f, fmx = 0.0f, ecell = 0.0f;
      if (f32red) {
        fmn = REDf[v * P2];
        fmx = REDf[(V + v) * P2];
#pragma unroll
        for (int k = 1; k < P2; ++k) { fmn = fminf(fmn, REDf[v * P2 + k]); fmx = fmaxf(fmx, REDf[(V + v) * P2 + k]); }
        cmn = ubar + (double)fmn;
        cmx = ubar + (double)fmx;
        const float am = __uint_as_float(amax[v]);
        ecell = (op.perr * am + op.pdev * (fabsf(ubs[v]) + 2.0f * am)) * 1.0001f + 1.0e-12f * (fabsf(ubs[v]) + am);
      } else {
        cmn = RED[v * P2];
        cmx = RED[(V + v) * P2];
#pragma unroll
        for (int k = 1; k < P2; ++k) { cmn = fmin(cmn, RED[v * P2 + k]); cmx = fmax(cmx, RED[(V + v) * P2 + k]); }
      }
      if (mode == kCellPrime || mode == kCellPrimeLimited) {
        a.mm[par][(size_t)cell * 2 * V + v] = cmn;
        a.mm[par][(size_t)cell * 2 * V + V + v] = cmx;
        if (a.mme[0]) a.mme[par][(size_t)cell * V + v] = ecell;
      } else {
        double lmin, lmax, argmax;
        float en = 0.0f;
        if (mode == kCellInitDmp) {
          // Euler/initialize.f90:291-294: the cell's own nodal min/max
          lmin = U[v * P2];
          lmax = U[v * P2];
          for (int k = 1; k < P2; ++k) { lmin = fmin(lmin, U[v * P2 + k]); lmax = fmax(lmax, U[v * P2 + k]); }
          argmax = 1.0e-1;
        } else {
          // get_min_max step 2: the neighbourhood bounds folded at the start
          lmin = nlmin;
          lmax = nlmax;
          en = nen;
          argmax = 0.0;
          if (a.lminmax) {
            a.lminmax[(size_t)cell * 2 * V + v] = lmin;
            a.lminmax[(size_t)cell * 2 * V + V + v] = lmax;
          }
          // candidate min/max for the next step (status 0)
          a.mm[par ^ 1][(size_t)cell * 2 * V + v] = cmn;
          a.mm[par ^ 1][(size_t)cell * 2 * V + V + v] = cmx;
          if (a.mme[0]) a.mme[par ^ 1][(size_t)cell * V + v] = ecell;
        }
        if (a.mme[0] == nullptr || (!f32red && en == 0.0f)) {
          // FP64 values (FP32-wide mode: FP32 projections taken as they are);
          // Euler/limiter.f90:210-220
          const double ldiff = fmax(fmax(1.0e-4, 1.0e-3 * (lmax - lmin)), argmax);
          if (cmn < lmin - ldiff || cmx > lmax + ldiff) atomicOr(&cflag[lc], 2);
        } else {
          // FP32-mixed: the same comparisons in FP32, in the deviation space
          // of the cell's FP32 reference state ub (FP64 work is the costly
          // part of this kernel).  |own - FP64 value| <= ecell; |lmin - its
          // FP64 value| <= en and likewise lmax, so the thresholds move by at
          // most en (1 + 2e-3); the FP32 forms of lmin - ub, lmax - ub, ldiff,
          // the thresholds and the differences add at most 2.5e-7 of the
          // magnitudes involved, and the FP32 constants 1e-4 and 0.1 differ
          // from their FP64 values by less than 1e-11 and 1e-8 of themselves.
          // A comparison decides here only when it holds by that margin;
          // otherwise k_settle decides the cell from FP64 values (bit 4).
          const double ub = ubar;
          const float Lmin = (float)(lmin - ub), Lmax = (float)(lmax - ub);
          const float ld = fmaxf(fmaxf(1.0e-4f, 1.0e-3f * (Lmax - Lmin)), mode == kCellInitDmp ? 0.1f : 0.0f);
          const float dl = Lmin - ld, dh = Lmax + ld;
          const float xl = f32red ? fmn : (float)(cmn - ub), xh = f32red ? fmx : (float)(cmx - ub);
          const float e = ecell + 1.002f * en + 2.5e-7f * (fabsf(Lmin) + fabsf(Lmax) + ld) + 1.0e-11f +
                          1.0e-12f * fabsf(ubs[v]);
          const float ml = e + 1.2e-7f * fabsf(xl), mh = e + 1.2e-7f * fabsf(xh);
          const float gl = xl - dl, gh = dh - xh;  // >= 0: not below lmin - ldiff / not above lmax + ldiff
          if (gl < -ml || gh < -mh) atomicOr(&cflag[lc], 2);
          else if (!(gl >= ml) || !(gh >= mh)) atomicOr(&cflag[lc], 4);
        }
      }
    }
    __syncthreads();
    if constexpr (kFast) {
      // FP32-mixed: a cell whose DMP the error bounds left open (bit 4) and
      // that nothing else marked goes on the list k_settle decides from FP64
      // values; here it counts as not troubled
      if (act && node == 0 && a.settle && (cflag[lc] & 7) == 4 &&
          (mode == kCellFused || mode == kCellUpdate || mode == kCellInitDmp))
        a.settle[atomicAdd(&a.list_count[1], 1)] = (int)cell;
    }
    if (act && mode != kCellPrime && mode != kCellPrimeLimited) {
      const bool bad = (cflag[lc] & 3) != 0;
      if (mode == kCellInitDmp) {
        if (bad) {
          // Euler/initialize.f90:296-317: status 1, Lh = NewLh = initial subcell data
          if (node == 0) {
            a.status[0][cell] = 1;
            a.status[1][cell] = 1;
            atomicAdd(&a.st[kc].n_recompute, 1);
          }
          if (a.lh_ic) {
            const size_t o = (size_t)cell * S * S * V;
            for (int idx = node; idx < S * S * V; idx += P2) {
              a.lh[0][o + idx] = a.lh_ic[o + idx];
              a.lh[1][o + idx] = a.lh_ic[o + idx];
            }
          }
        }
      } else if (node == 0) {
        a.troubled[cell] = bad ? 1 : 0;
        if (bad) atomicAdd(&a.st[kc].n_recompute, 1);
      }
    }
  } else {
    __syncthreads();
  }

  // ------------------------------------------------ CFL per cell / instance
  if (!want_cfl) return;
  if (limiter && (mode == kCellFused || mode == kCellUpdate)) {
    if (act && node == 0) a.denom[cell] = __longlong_as_double((long long)cmax[lc]);
    return;
  }
  // fold the CTA's cells per instance: the node-0 thread of the first cell of
  // each instance in this CTA folds that instance's cells (a contiguous run)
  // and issues one atomic
  if (act && node == 0 && (lc == 0 || cell - 1 < in.cell_base)) {
    unsigned long long m = 0ull;
    if constexpr (Sys::ID == kSysAD) {
      m = (unsigned long long)__double_as_longlong(in.ad_denom);
    } else {
      const long long end = in.cell_base + (long long)in.imax * in.jmax;
      for (int c = lc; c < CPB && cell + (c - lc) < end; ++c) m = m > cmax[c] ? m : cmax[c];
    }
    atomicMax(&a.st[kc].denom_next, m);
  }
}


}  // namespace aderdg
