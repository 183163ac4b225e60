// limiter.cuh -- K4: a posteriori subcell limiter.
//
// K4a k_mark: spread_recompute + allocate_limiter (Euler/limiter.f90:302-354)
//     as a gather per cell, compaction of the cells to recompute into a list,
//     and the CFL fold of the cells the limiter leaves untouched.
// K4b k_subcell: subcell_recompute (Euler/limiter.f90:411-647,
//     Baer-Nunziato/limiter.f90:416-596) for every listed cell, one CTA per
//     cell, persistent over the list; then put_subcell_data, the DMP of
//     recompute = 2 cells, the next step's min/max and CFL contribution.
//     update_limiter (Lh = NewLh) is the parity flip of the Lh buffers.
// Compiled with --fmad=false, reference operation order throughout.  The FP64
// and FP32-mixed modes run K4b in FP64 (T = double); the FP32-mixed mode adds
// the settling of DMP comparisons against neighbourhood bounds that carry an
// FP32 error bound.  The FP32-wide mode runs the re-solve in FP32 (T = float).
#pragma once

#include "cells.cuh"
#include "common.cuh"
#include "physics.cuh"

namespace aderdg {

template <class Sys, int N>
__global__ void __launch_bounds__(256) k_mark(BatchArgs a) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = c < a.ncells ? find_inst_cell(a.inst, a.ninst, c) : -1;
  const bool act = k >= 0 && a.st[k].active;
  unsigned long long val = 0ull;
  if (act) {
    const InstDesc& in = a.inst[k];
    const int par = parity(a.st[k]);
    const long long lc = c - in.cell_base;
    const int ci = (int)(lc % in.imax), cj = (int)(lc / in.imax);
    int rec = 0;
    if (a.troubled[c]) {
      rec = 1;
    } else {
      // face neighbours (Face2Neigh, Euler/initialize.f90:210-213)
      const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
      for (int f = 0; f < 4; ++f) {
        const int in_ = nb_index(ci, di[f], in.imax, in.bc[0], in.bc[1]);
        const int jn_ = nb_index(cj, dj[f], in.jmax, in.bc[2], in.bc[3]);
        if (a.troubled[in.cell_base + in_ + (long long)in.imax * jn_]) rec = 2;
      }
    }
    a.recompute[c] = rec;
    a.status[par ^ 1][c] = rec == 1 ? 1 : 0;
    if (rec > 0) {
      const int pos = atomicAdd(a.list_count, 1);
      a.list[pos] = (int)c;
      atomicAdd(&a.st[k].n_list, 1);
    } else {
      val = (unsigned long long)__double_as_longlong(a.denom[c]);
    }
  }
  // warp fold of the CFL denominators when the warp holds one instance
  const unsigned full = 0xffffffffu;
  const int k0 = __shfl_sync(full, k, 0);
  const bool same = __all_sync(full, k == k0 || k < 0);
  if (same) {
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_down_sync(full, val, o);
      val = val > other ? val : other;
    }
    if ((threadIdx.x & 31) == 0 && k0 >= 0 && val) atomicMax(&a.st[k0].denom_next, val);
  } else if (act && val) {
    atomicMax(&a.st[k].denom_next, val);
  }
}

template <class Sys, int N, class T>
struct SubCfg {
  static constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V;
  static constexpr int R = S + 4;  // room of the gathered subcells -1 .. S+2 (1-based; Euler reads 0 .. S+1)
  static constexpr int H = S + 2;  // reconstructed region: 0 .. S+1
  static constexpr int THREADS = 128;
  // CTAs per SM the register allocation aims at.  FP32: one more than the
  // unconstrained allocation allows where that does not spill.  FP64 (the
  // FP64 pipe bounds it): as many as shared memory admits, up to 4 (Euler:
  // 128 registers; Baer-Nunziato N = 2 and 3: 4 at 128 registers, about 130
  // bytes spilled, 8% and 2% faster than 3 unspilled; N = 4: 2; N = 5: 1), so
  // that the CTAs' phases without FP64 work (gather loads, barriers) overlap
  // other CTAs' arithmetic.
  static constexpr int MIN_BLOCKS = sizeof(T) == 4 ? (Sys::ID == kSysBN ? (N == 3 ? 4 : N == 2 ? 5 : 1) : 6)
                                                   : (Sys::ID == kSysBN ? (N <= 3 ? 4 : N == 4 ? 2 : 1) : 4);
  static constexpr int NE = (S + 1) * S;               // x edges (and y edges) of the subgrid
  static constexpr int NEF = (Sys::ID == kSysBN ? 4 : 2) * V * NE;  // edge fluxes (+ BN fluctuations)
  // compute-type (T) elements: sub0 [V][R*R]; the reconstructed states wLx
  // wRx wLy wRy [4][V][H*H] (Baer-Nunziato: then the half-step increment
  // [V][H*H] and the volume-fraction slopes [2][H*H], which its finite-volume
  // update reads; the other slopes live in registers); the edge fluxes; the
  // operators uh2lim [S*P], lim2uh [P*S], uh2lob [P*P] in T.  Arrays whose
  // lifetimes do not meet share room: the gather stages the 3x3
  // neighbourhood's uh [9][V][P2] and its y pass [9][V][P][S] in the room of
  // the states and edge fluxes, formed after it; subuh1 [V][S*S] takes wLx's
  // room, luhy [V][P][S] wRx's and the FP32 DMP of the new polynomial (UN, LY,
  // LB) wLy's, all after the edge fluxes.
  static constexpr int TW = V * H * H;
  static constexpr int TSTATE = 4 * TW + (Sys::ID == kSysBN ? TW + 2 * H * H : 0);
  static_assert(9 * V * P2 + 9 * V * P * S <= TSTATE + NEF, "gather staging room");
  static_assert(V * S * S <= TW && V * S * P <= TW, "subuh1 / luhy room");
  static_assert(V * P2 + V * S * P + V * P * P <= 2 * TW, "FP32 DMP room");
  static constexpr int TEL = V * R * R + TSTATE + NEF + 2 * S * P + P * P;
  static constexpr int TBYTES = ((TEL * (int)sizeof(T) + 15) / 16) * 16;
  // FP64 elements: new polynomial UN [V][P2], DMP y pass LY [V][S][P], LB
  // [V][P][P], reduction [2][V][warps] -- all used after the finite-volume
  // update, so in the FP64 re-solve they take the edge fluxes' room, which
  // that update was the last to read -- and the operators uh2lim, uh2lob (FP64)
  static constexpr int OPS_DBL = S * P + P * P;
  static constexpr int DMP_DBL = V * P2 + V * S * P + V * P * P + 2 * V * (THREADS / 32);
  static constexpr bool DMP_IN_EF = sizeof(T) == 8 && DMP_DBL <= NEF;
  static constexpr int DEL = (DMP_IN_EF ? 0 : DMP_DBL) + OPS_DBL;
  // misc: flags, CFL max, neighbour cells and their status
  static constexpr int MISC = 16 + 9 * 8 + 9 * 4 + 4 * V + 12;
  static constexpr int SMEM_BYTES = TBYTES + DEL * 8 + MISC;
};

// minmod, Euler/limiter.f90:384-405
template <class T>
__device__ __forceinline__ T minmod(T a, T b) {
  if (a * b <= T(0)) return T(0);
  return (tabs(a) < tabs(b)) ? a : b;
}
// The same decisions on the FP64 bit patterns (integer pipe, not the FP64
// pipe): 0 when the signs differ or either is 0, else the smaller magnitude
// (magnitude bits order like the magnitudes).  It differs from minmod only
// where a * b underflows to 0 for same-signed |a b| < 2^-1074 (the smaller
// slope instead of 0).
__device__ __forceinline__ double minmod_bits(double a, double b) {
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  const long long ma = ia & 0x7fffffffffffffffLL, mb = ib & 0x7fffffffffffffffLL;
  if ((ia ^ ib) < 0 || ma == 0 || mb == 0) return 0.0;
  return ma < mb ? a : b;
}

// Subgrid Rusanov flux (Euler/limiter.f90:361-378; BN :359-383 adds D = B~ dQ);
// kRcp: the reciprocal-sharing physics forms (FP32-mixed mode)
template <class Sys, class T, bool kRcp = false>
__device__ __forceinline__ void rusanov_s(const PhysC<T>& pc, const T* QL, const T* QR, int d, T* F, T* D) {
  constexpr int V = Sys::V;
  T FLf[2 * V], FRf[2 * V], smax;
  if constexpr (kRcp) {
    // the flux along d only (the other direction's would be multiplied by 0)
    T eL, eR;
    Sys::flux_dir_eig_r(pc, QL, d, FLf, eL);
    Sys::flux_dir_eig_r(pc, QR, d, FRf, eR);
    smax = tmax(eL, eR);
#pragma unroll
    for (int v = 0; v < V; ++v) F[v] = T(0.5) * (FLf[v] + FRf[v]) - T(0.5) * smax * (QR[v] - QL[v]);
  } else {
    smax = tmax(Sys::max_eig(pc, QL, d), Sys::max_eig(pc, QR, d));
    Sys::flux(pc, QL, FLf);
    Sys::flux(pc, QR, FRf);
    const T nv0 = d == 0 ? T(1) : T(0), nv1 = d == 0 ? T(0) : T(1);
#pragma unroll
    for (int v = 0; v < V; ++v)
      F[v] = T(0.5) * ((FLf[v] + FRf[v]) * nv0 + (FLf[V + v] + FRf[V + v]) * nv1) - T(0.5) * smax * (QR[v] - QL[v]);
  }
  if constexpr (Sys::ID == kSysBN) {
    if constexpr (kRcp) BNSys::roe_times_jump_r(pc, QL, QR, d, D);
    else BNSys::roe_times_jump(pc, QL, QR, d, D);
  }
}

// Warp-wide min/max of V values per lane (butterfly), then lane 0 of warp w
// stores them at red[v * NW + w] (min) and red[(V + v) * NW + w] (max).
template <class R, int V, int NW>
__device__ __forceinline__ void warp_minmax_store(R* mn, R* mx, R* red, int t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int v = 0; v < V; ++v) {
      mn[v] = tmin(mn[v], __shfl_xor_sync(0xffffffffu, mn[v], o));
      mx[v] = tmax(mx[v], __shfl_xor_sync(0xffffffffu, mx[v], o));
    }
  if ((t & 31) == 0)
#pragma unroll
    for (int v = 0; v < V; ++v) {
      red[v * NW + (t >> 5)] = mn[v];
      red[(V + v) * NW + (t >> 5)] = mx[v];
    }
}

// T = double: the reference's FP64 arithmetic in its order (bit for bit),
// or, with kRcp (the FP32-mixed mode, instantiated with fused multiply-adds in
// predictor_tu.cu), FP64 with the reciprocal-sharing physics forms and
// multiplications by 1/ldx in place of divisions; the DMP projections keep
// the reference order in both.
// T = float: the FP32-wide mode; the subcell re-solve, the DMP projections
// of the new polynomial (while their error bound allows) and the CFL
// eigenvalues (where the FP32 pressure is settled) in FP32; the state, Lh
// and min/max in FP64.
template <class Sys, int N, class T, bool kRcp = false>
__global__ void __launch_bounds__(SubCfg<Sys, N, T>::THREADS, SubCfg<Sys, N, T>::MIN_BLOCKS) k_subcell(BatchArgs a, DevOps<N, double> op, FaceConst fc) {
  using C = SubCfg<Sys, N, T>;
  constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V, R = C::R, H = C::H, NT = C::THREADS, NE = C::NE;
  constexpr int NW = NT / 32;  // warps
  constexpr bool BN = Sys::ID == kSysBN;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sub0 = reinterpret_cast<T*>(smem_raw);
  T* wLx = sub0 + V * R * R;
  T* wRx = wLx + C::TW;
  T* wLy = wRx + C::TW;
  T* wRy = wLy + C::TW;
  T* slt = wRy + C::TW;              // BN: half-step increment [V][H*H]
  T* sa8 = slt + C::TW;              // BN: volume-fraction slopes x [H*H], y [H*H]
  T* EF = wLx + C::TSTATE;           // x edges: F [V][NE] (BN: then D [V][NE]); then the y edges
  T* limT = EF + C::NEF;             // uh2lim (s,k) at [s + S*k]
  T* l2uT = limT + S * P;            // lim2uh (k,s) at [k + P*s]
  T* lobT = l2uT + S * P;            // uh2lob (q,k) at [q + P*k]
  T* sub1 = wLx;                     // [V][S*S], after the edge fluxes
  T* LUY = wRx;                      // [V][P][S]: luhy(v, iii, s) at (v*P + s)*S + iii
  T* NB = wLx;                       // gather staging: [9][V][P2]
  T* LYN = NB + 9 * V * P2;          // [9][V][P][S]: sum_m uh(k, m) uh2lim(s, m) at ((n*V + v)*P + k)*S + s
  double* UN = C::DMP_IN_EF ? reinterpret_cast<double*>(EF) : reinterpret_cast<double*>(smem_raw + C::TBYTES);  // [V][P2]
  double* LY = UN + V * P2;          // DMP y pass [V][S][P]
  double* LB = LY + V * S * P;       // [V][P][P]
  double* red = LB + V * P * P;      // [2][V][NW]
  double* opsm = C::DMP_IN_EF ? reinterpret_cast<double*>(smem_raw + C::TBYTES) : red + 2 * V * NW;  // uh2lim, uh2lob (FP64)
  unsigned char* misc = reinterpret_cast<unsigned char*>(opsm + C::OPS_DBL);
  int* flag = reinterpret_cast<int*>(misc);
  unsigned long long* cmaxp = reinterpret_cast<unsigned long long*>(misc + 8);
  long long* nbc = reinterpret_cast<long long*>(misc + 16);  // 3x3 neighbour cells, n = (bi+1) + 3 (bj+1)
  int* nbs = reinterpret_cast<int*>(misc + 16 + 9 * 8);     // their status (0: project olduh)
  unsigned* amax = reinterpret_cast<unsigned*>(nbs + 9);     // FP32-wide: max |UN - UN(node 0)| per variable
  float* UNf = reinterpret_cast<float*>(wLy);                // FP32 DMP (after the re-solve)
  float* LYf = UNf + V * P2;
  float* LBf = LYf + V * S * P;
  float* redf = reinterpret_cast<float*>(red);              // [2][V][NW]

  const int t = threadIdx.x;
  for (int k = t; k < C::OPS_DBL; k += NT) opsm[k] = k < S * P ? op.uh2lim[k] : op.uh2lob[k - S * P];
  for (int k = t; k < S * P; k += NT) {
    limT[k] = (T)op.uh2lim[k];
    l2uT[k] = (T)op.lim2uh[k];
  }
  for (int k = t; k < P * P; k += NT) lobT[k] = (T)op.uh2lob[k];
  __syncthreads();
  auto SU = [&](int v, int ii, int jj) -> T& { return sub0[v * R * R + (ii + 1) + R * (jj + 1)]; };  // ii,jj in -1..S+2
  auto hx = [&](int v, int ii, int jj) { return v * H * H + ii + H * jj; };                         // ii,jj in 0..S+1

  const int count = *a.list_count;
  for (int li = blockIdx.x; li < count; li += gridDim.x) {
    const long long c = a.list[li];
    const int k = find_inst_cell(a.inst, a.ninst, c);
    const InstDesc& in = a.inst[k];
    const InstState& st = a.st[k];
    const Phys ph = in.ph;
    const PhysC<T> pc(ph);
    const int par = parity(st);
    const long long lc = c - in.cell_base;
    const int ci = (int)(lc % in.imax), cj = (int)(lc / in.imax);
    const int rec = a.recompute[c];
    const T dt = (T)st.dt;
    const T ldx0 = (T)(in.dx / (double)S), ldx1 = (T)(in.dy / (double)S);
    const T ix0 = T(1) / ldx0, ix1 = T(1) / ldx1;  // kRcp only
    auto divx = [&](T q) -> T { if constexpr (kRcp) return q * ix0; else return q / ldx0; };
    auto divy = [&](T q) -> T { if constexpr (kRcp) return q * ix1; else return q / ldx1; };
    // the flux of Q into F[d * V + v]; kRcp: along d only (the MUSCL half step
    // uses the x flux of the x-reconstructed states and the y flux of the
    // y-reconstructed ones), otherwise both directions as the reference
    auto flux = [&](const T* Q, int d, T* F) {
      if constexpr (kRcp) {
        T e;
        Sys::flux_dir_eig_r(pc, Q, d, F + d * V, e);
      } else {
        Sys::flux(pc, Q, F);
      }
    };
    auto ncp = [&](const T* Q, T ax, T ay, T* Sr) {
      if constexpr (Sys::ID == kSysBN) {
        if constexpr (kRcp) BNSys::src_ncp_r(pc, Q, ax, ay, Sr);
        else BNSys::src_ncp(pc, Q, ax, ay, Sr);
      }
    };
    const bool dmr = (Sys::ID == kSysEuler) && in.bc_mode == 1;

    // ---- gather the subcell data of the 3x3 neighbourhood (only the strip
    // the reconstruction reads): get_subcell_data of olduh (sum-factorised:
    // the y contraction of each neighbour once, then x; the reference's
    // summation order) or Lh of limited cells
    if (t < 9) {
      const int bi = t % 3 - 1, bj = t / 3 - 1;
      const int in_ = nb_index(ci, bi, in.imax, in.bc[0], in.bc[1]);
      const int jn_ = nb_index(cj, bj, in.jmax, in.bc[2], in.bc[3]);
      const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
      nbc[t] = nc;
      nbs[t] = a.status[par][nc];
    }
    if (t == 0) {
      flag[0] = 0;
      *cmaxp = 0ull;
    }
    if (t < V) amax[t] = 0u;
    __syncthreads();
    // Euler's interior slopes read one ring of neighbour subcells, beside the
    // cell's edges only (neighbours n = 1, 3, 5, 7); Baer-Nunziato's halo
    // slopes read two rings beside the edges and the first ring's corners
    // (all nine neighbours)
    constexpr int NNB = BN ? 9 : 5;
    for (int p = t; p < NNB * P2 * V; p += NT) {
      const int m = p / (P2 * V), r = p - m * (P2 * V);
      const int n = BN ? m : (m == 0 ? 1 : m == 4 ? 7 : m + 2);
      const int node = r / V, v = r - node * V;
      if (nbs[n] == 0) NB[(n * V + v) * P2 + node] = (T)a.uh[par][(size_t)nbc[n] * P2 * V + r];
    }
    __syncthreads();
    // the items actually read, enumerated densely (no idle lanes): all S
    // rows of the neighbours beside the cell (n = 3, 4, 5), and the rows
    // nearest to the cell of those below and above -- Baer-Nunziato: two of
    // n = 1 (subcell rows S-2, S-1) and of n = 7 (rows 0, 1), one of the
    // corner neighbours n = 0, 2 (row S-1) and n = 6, 8 (row 0); Euler: one
    // of n = 1 (row S-1) and of n = 7 (row 0); LYN keeps the full
    // [9][V][P][S] index
    constexpr int NMID = 3 * V * P * S, NROW = V * P, NOUT = BN ? 8 : 2;
    for (int q = t; q < NMID + NOUT * NROW; q += NT) {
      int n, v, kk, sb;
      if (q < NMID) {
        n = 3 + q / (V * P * S);
        const int r = q % (V * P * S);
        v = r / (P * S);
        kk = (r / S) % P;
        sb = r % S;
      } else if constexpr (BN) {
        // rows 0..7: (n, sb) = (1, S-2) (1, S-1) (7, 0) (7, 1) (0, S-1) (2, S-1) (6, 0) (8, 0)
        const int q2 = q - NMID, row = q2 / NROW, r2 = q2 % NROW;
        n = row < 2 ? 1 : row < 4 ? 7 : row == 4 ? 0 : row == 5 ? 2 : row == 6 ? 6 : 8;
        v = r2 / P;
        kk = r2 % P;
        sb = row < 2 ? S - 2 + row : row < 4 ? row - 2 : row < 6 ? S - 1 : 0;
      } else {
        const int q2 = q - NMID, r2 = q2 % NROW;
        n = q2 < NROW ? 1 : 7;
        v = r2 / P;
        kk = r2 % P;
        sb = n == 1 ? S - 1 : 0;
      }
      if (nbs[n] != 0) continue;
      const T* u = NB + (n * V + v) * P2;
      T ly = T(0);
#pragma unroll
      for (int m = 0; m < P; ++m) ly = ly + u[kk + P * m] * limT[sb + S * m];
      LYN[((n * V + v) * P + kk) * S + sb] = ly;
    }
    __syncthreads();
    // Baer-Nunziato: subcells 0 .. S+1 in both directions, then the four
    // strips of the second ring beside the edges (columns -1 and S+2 of rows
    // 1..S, rows -1 and S+2 of columns 1..S); Euler: the S x S interior and
    // the four strips beside it (columns 1..S of rows 0..S+1, then columns 0
    // and S+1 of rows 1..S)
    constexpr int NX = BN ? H * H + 4 * S : S * S + 4 * S;
    for (int p = t; p < NX; p += NT) {
      int ii, jj;
      if constexpr (BN) {
        if (p < H * H) {
          ii = p % H;
          jj = p / H;
        } else {
          const int p2 = p - H * H, side = p2 / S, o = 1 + p2 % S;
          ii = side == 0 ? -1 : side == 1 ? S + 2 : o;
          jj = side < 2 ? o : (side == 2 ? -1 : S + 2);
        }
      } else if (p < S * (S + 2)) {
        ii = 1 + p % S;
        jj = p / S;
      } else {
        const int p2 = p - S * (S + 2);
        ii = p2 < S ? 0 : S + 1;
        jj = 1 + p2 % S;
      }
      const int bi = ii < 1 ? -1 : (ii > S ? 1 : 0), bj = jj < 1 ? -1 : (jj > S ? 1 : 0);
      const int sa = ii - 1 - bi * S, sb = jj - 1 - bj * S;
      const int n = (bi + 1) + 3 * (bj + 1);
      T val[V];
      if (nbs[n] == 0) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const T* ly = LYN + (size_t)(n * V + v) * P * S + sb;
          T acc = T(0);
#pragma unroll
          for (int kk = 0; kk < P; ++kk) acc = acc + ly[kk * S] * limT[sa + S * kk];
          val[v] = acc;
        }
      } else {
        const double* L = a.lh[par] + ((size_t)nbc[n] * S * S + sa + S * sb) * V;
#pragma unroll
        for (int v = 0; v < V; ++v) val[v] = (T)L[v];
      }
      if constexpr (Sys::ID == kSysEuler) {
        if (dmr) {  // Euler/limiter.f90:487-522, applied in the reference's order
          T Qbc[4], Vb[4];
          if (ci == 0 && ii <= 0) {
            for (int v = 0; v < 4; ++v) Vb[v] = (T)fc.Va[v];
            EulerSys::prim2cons(pc, Vb, Qbc);
            for (int v = 0; v < 4; ++v) val[v] = Qbc[v];
          }
          if (cj == 0 && jj <= 0 && (double)(ci + 1) * in.dx > 1.0 / 6.0) val[2] = -val[2];
          if (cj == in.jmax - 1 && jj >= S + 1) {
            const double x_sw = fc.xsw0 + fc.xsw1 * st.time;
            const double* src = ((double)(ci + 1) * in.dx <= x_sw) ? fc.Va : fc.Vb;
            for (int v = 0; v < 4; ++v) Vb[v] = (T)src[v];
            EulerSys::prim2cons(pc, Vb, Qbc);
            for (int v = 0; v < 4; ++v) val[v] = Qbc[v];
          }
        }
      }
#pragma unroll
      for (int v = 0; v < V; ++v) SU(v, ii, jj) = val[v];
    }
    __syncthreads();

    // ---- MUSCL-Hancock reconstruction on subcells 0..S+1; the slopes of
    // one direction at a time in registers.  The S*S interior subcells come
    // first, then the ring of halo subcells, so that the interior ones fill
    // whole warps: Euler's halo subcells have zero slopes (Euler/limiter.f90:
    // 529-536), so their two face states per direction are the subcell value,
    // the half-step flux differences vanish exactly and their evolved face
    // states are the subcell value itself; they are copied, and only the
    // warps holding interior subcells evaluate fluxes.
    for (int p = t; p < H * H; p += NT) {
      int ii, jj;
      if (p < S * S) {
        ii = 1 + p % S;
        jj = 1 + p / S;
      } else {
        const int r = p - S * S;  // the ring: bottom row, top row, left column, right column
        if (r < H) { ii = r; jj = 0; }
        else if (r < 2 * H) { ii = r - H; jj = H - 1; }
        else if (r < 2 * H + S) { ii = 0; jj = 1 + (r - 2 * H); }
        else { ii = H - 1; jj = 1 + (r - 2 * H - S); }
      }
      const bool interior = p < S * S;
      // the corners of the ring feed no edge (Euler does not gather them)
      if (!interior && (ii == 0 || ii == H - 1) && (jj == 0 || jj == H - 1)) continue;
      if (!BN && !interior) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const T q = SU(v, ii, jj);
          wLx[hx(v, ii, jj)] = q;
          wRx[hx(v, ii, jj)] = q;
          wLy[hx(v, ii, jj)] = q;
          wRy[hx(v, ii, jj)] = q;
        }
        continue;
      }
      T Qt[V], FL[2 * V], FR[2 * V];
      // Euler computes slopes for interior subcells only (halo slopes stay 0,
      // Euler/limiter.f90:529-536); BN also on the halo (BN :486-492)
      // FP32-mixed (FP64 re-solve): minmod on the bit patterns
      auto mm = [](T a, T b) -> T {
        if constexpr (kRcp && sizeof(T) == 8) return minmod_bits(a, b);
        else return minmod(a, b);
      };
      auto slope_x = [&](int v) -> T {
        return (BN || interior) ? mm(SU(v, ii + 1, jj) - SU(v, ii, jj), SU(v, ii, jj) - SU(v, ii - 1, jj)) : T(0);
      };
      auto slope_y = [&](int v) -> T {
        return (BN || interior) ? mm(SU(v, ii, jj + 1) - SU(v, ii, jj), SU(v, ii, jj) - SU(v, ii, jj - 1)) : T(0);
      };
      T q0[V], wl[V], wr[V], sl[V];
#pragma unroll
      for (int v = 0; v < V; ++v) q0[v] = SU(v, ii, jj);
      T src[V];
      if constexpr (BN) {
        // Baer-Nunziato/limiter.f90:494-497
        const T ax = slope_x(8), ay = slope_y(8);
        sa8[ii + H * jj] = ax;
        sa8[H * H + ii + H * jj] = ay;
        ncp(q0, divx(ax), divy(ay), src);
      }
#pragma unroll
      for (int v = 0; v < V; ++v) sl[v] = slope_x(v);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        wl[v] = q0[v] - T(0.5) * sl[v];
        wr[v] = q0[v] + T(0.5) * sl[v];
      }
      flux(wl, 0, FL);
      flux(wr, 0, FR);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if constexpr (BN) Qt[v] = src[v] - divx(FR[v] - FL[v]);
        else Qt[v] = -divx(FR[v] - FL[v]);
        wLx[hx(v, ii, jj)] = wl[v];
        wRx[hx(v, ii, jj)] = wr[v];
      }
#pragma unroll
      for (int v = 0; v < V; ++v) sl[v] = slope_y(v);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        wl[v] = q0[v] - T(0.5) * sl[v];
        wr[v] = q0[v] + T(0.5) * sl[v];
      }
      flux(wl, 1, FL);
      flux(wr, 1, FR);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        Qt[v] = Qt[v] - divy(FR[V + v] - FL[V + v]);
        if constexpr (BN) slt[hx(v, ii, jj)] = Qt[v];
        wLx[hx(v, ii, jj)] = wLx[hx(v, ii, jj)] + T(0.5) * dt * Qt[v];
        wRx[hx(v, ii, jj)] = wRx[hx(v, ii, jj)] + T(0.5) * dt * Qt[v];
        wLy[hx(v, ii, jj)] = wl[v] + T(0.5) * dt * Qt[v];
        wRy[hx(v, ii, jj)] = wr[v] + T(0.5) * dt * Qt[v];
      }
    }
    __syncthreads();

    // ---- edge fluxes Fx(1..S+1, 1..S), Fy(1..S, 1..S+1) (Euler/limiter.f90:571-588);
    // BN's four Rusanov fluxes per subcell (Baer-Nunziato/limiter.f90:526-545)
    // are those of its edges, each formed once here from the same states
    {
      T* EX = EF;
      T* EY = EF + (BN ? 2 : 1) * V * NE;
      for (int p = t; p < 2 * NE; p += NT) {
        const bool xd = p < NE;
        const int q = xd ? p : p - NE;
        T QL[V], QR[V], F[V], Dd[V];
        int ii, jj;
        if (xd) { ii = q % (S + 1) + 1; jj = q / (S + 1) + 1; }
        else { ii = q % S + 1; jj = q / S + 1; }
#pragma unroll
        for (int v = 0; v < V; ++v) {
          QL[v] = xd ? wRx[hx(v, ii - 1, jj)] : wRy[hx(v, ii, jj - 1)];
          QR[v] = xd ? wLx[hx(v, ii, jj)] : wLy[hx(v, ii, jj)];
        }
        rusanov_s<Sys, T, kRcp>(pc, QL, QR, xd ? 0 : 1, F, Dd);
        T* dst = xd ? EX : EY;
#pragma unroll
        for (int v = 0; v < V; ++v) dst[v * NE + q] = F[v];
        if constexpr (BN) {
#pragma unroll
          for (int v = 0; v < V; ++v) dst[(V + v) * NE + q] = Dd[v];
        }
      }
      __syncthreads();
      for (int p = t; p < S * S; p += NT) {
        const int ii = p % S + 1, jj = p / S + 1;
        const int xp = ii + (S + 1) * (jj - 1), xm = (ii - 1) + (S + 1) * (jj - 1);
        const int yp = (ii - 1) + S * jj, ym = (ii - 1) + S * (jj - 1);
        if constexpr (!BN) {
          // first-order FV update, Euler/limiter.f90:592-597
#pragma unroll
          for (int v = 0; v < V; ++v)
            sub1[v * S * S + p] = SU(v, ii, jj) - divx(dt) * (EX[v * NE + xp] - EX[v * NE + xm]) -
                                  divy(dt) * (EY[v * NE + yp] - EY[v * NE + ym]);
        } else {
          T qh[V], src[V];
#pragma unroll
          for (int v = 0; v < V; ++v) qh[v] = SU(v, ii, jj) + T(0.5) * dt * slt[hx(v, ii, jj)];
          ncp(qh, divx(sa8[ii + H * jj]), divy(sa8[H * H + ii + H * jj]), src);
#pragma unroll
          for (int v = 0; v < V; ++v)
            sub1[v * S * S + p] = SU(v, ii, jj) - divx(dt) * (EX[v * NE + xp] - EX[v * NE + xm]) -
                                  divy(dt) * (EY[v * NE + yp] - EY[v * NE + ym]) -
                                  divx(dt) * T(0.5) * (EX[(V + v) * NE + xp] + EX[(V + v) * NE + xm]) -
                                  divy(dt) * T(0.5) * (EY[(V + v) * NE + yp] + EY[(V + v) * NE + ym]) +
                                  dt * src[v];
        }
      }
    }
    __syncthreads();

    // ---- put_subcell_data (Euler/limiter.f90:74-98): luhy then luh
    for (int p = t; p < S * P; p += NT) {
      const int iii = p % S, s = p / S;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        T acc = T(0);
        for (int kk = 0; kk < S; ++kk) acc = acc + sub1[v * S * S + iii + S * kk] * l2uT[s + P * kk];
        LUY[(v * P + s) * S + iii] = acc;
      }
    }
    __syncthreads();
    double* uout = a.uh[par ^ 1] + (size_t)c * P2 * V;
    for (int p = t; p < P2; p += NT) {
      const int s1 = p % P, jjj = p / P;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        T acc = T(0);
        for (int kk = 0; kk < S; ++kk) acc = acc + LUY[(v * P + jjj) * S + kk] * l2uT[s1 + P * kk];
        UN[v * P2 + p] = (double)acc;
        uout[p * V + v] = (double)acc;
      }
    }
    __syncthreads();
    // ---- DMP of the new polynomial: recompute = 2 cells only (a recompute =
    // 1 cell is limited whatever it gives, and its next min/max come from
    // its subcell data), uniform per CTA.
    const bool dmp = rec == 2;
    if constexpr (sizeof(T) == 4) {
      // FP32-wide DMP: deviations from the new polynomial's node-0 state
      if (dmp) {
        for (int p = t; p < P2; p += NT)
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float d = (float)(UN[v * P2 + p] - UN[v * P2]);
            UNf[v * P2 + p] = d;
            atomicMax(&amax[v], __float_as_uint(fabsf(d)));
          }
      }
      __syncthreads();
    }
    // FP32-wide (T = float): FP32 projections when their error bound stays
    // within the DMP's absolute tolerance, else FP64 (as in the cell kernel).
    float err[V];
    bool f32 = false;
    if constexpr (sizeof(T) == 4) {
      f32 = true;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        err[v] = op.perr * __uint_as_float(amax[v]);
        f32 = f32 && err[v] <= 1.0e-4f;
      }
    }
    if constexpr (sizeof(T) == 4) {
      if (dmp && f32) Proj<N, V, float>::template ypass<true>(UNf, LYf, LBf, limT, lobT, t, NT);
    }
    if (dmp && !f32) Proj<N, V, double>::ypass(UN, LY, LB, opsm, opsm + S * P, t, NT);
    __syncthreads();
    double mn[V], mx[V];
    bool posfail = false;
    if (!dmp) {
      // no projections: the CFL part below only
    } else if (f32) {
      float fmn[V], fmx[V];
#pragma unroll
      for (int v = 0; v < V; ++v) { fmn[v] = __int_as_float(0x7f800000); fmx[v] = -__int_as_float(0x7f800000); }
      for (int p = t; p < P2; p += NT)
#pragma unroll
        for (int v = 0; v < V; ++v) { fmn[v] = fminf(fmn[v], UNf[v * P2 + p]); fmx[v] = fmaxf(fmx[v], UNf[v * P2 + p]); }
      if constexpr (sizeof(T) == 4) {
        float ubf[V];
#pragma unroll
        for (int v = 0; v < V; ++v) ubf[v] = (float)UN[v * P2];
        Proj<N, V, float>::template xpass_minmax_f32<Sys>(LYf, LBf, limT, lobT, UN, opsm, typename Sys::FConst(ph), err,
                                                          ubf, ph, t, NT, fmn, fmx, posfail);
      }
      warp_minmax_store<float, V, NW>(fmn, fmx, redf, t);
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
      Proj<N, V, double>::template xpass_minmax<Sys>(UN, LY, LB, opsm, opsm + S * P, ph, t, NT, mn, mx, posfail);
      warp_minmax_store<double, V, NW>(mn, mx, red, t);
    }
    // CFL denominator of the new polynomial (FP32-wide: FP32 eigenvalues
    // where the FP32 pressure is settled; FP64 in the other modes)
    for (int p = t; p < P2; p += NT) {
      double Q[V];
#pragma unroll
      for (int v = 0; v < V; ++v) Q[v] = UN[v * P2 + p];
      double dn;
      if constexpr (sizeof(T) == 4) {
        float q[V];
#pragma unroll
        for (int v = 0; v < V; ++v) q[v] = (float)Q[v];
        dn = cfl_denom_f32<Sys, N>(in, typename Sys::FConst(ph), q, Q);
      } else {
        dn = cfl_denom<Sys, N>(in, Q);
      }
      atomicMax(cmaxp, (unsigned long long)__double_as_longlong(dn));
    }
    if (posfail) atomicOr(&flag[0], 1);
    __syncthreads();
    double* mmo = a.mm[par ^ 1] + (size_t)c * 2 * V;
    double dmn = 0.0, dmx = 0.0;  // thread v < V: min/max of the new polynomial's variable v
    if (dmp && t < V) {
      const int v = t;
      double cmn, cmx;
      if (f32) {
        float fmn = redf[v * NW], fmx = redf[(V + v) * NW];
        for (int q = 1; q < NW; ++q) { fmn = fminf(fmn, redf[v * NW + q]); fmx = fmaxf(fmx, redf[(V + v) * NW + q]); }
        cmn = UN[v * P2] + (double)fmn;
        cmx = UN[v * P2] + (double)fmx;
      } else {
        cmn = red[v * NW];
        cmx = red[(V + v) * NW];
        for (int q = 1; q < NW; ++q) { cmn = fmin(cmn, red[v * NW + q]); cmx = fmax(cmx, red[(V + v) * NW + q]); }
      }
      dmn = cmn;
      dmx = cmx;
      if (rec == 2) {
        const double* mmi = a.mm[par];
        double lmin = mmi[(size_t)c * 2 * V + v], lmax = mmi[(size_t)c * 2 * V + V + v];
        float en = 0.0f;  // FP32-mixed: largest error bound of the folded min/max
        for (int jj = -1; jj <= 1; ++jj)
          for (int ii = -1; ii <= 1; ++ii) {
            const int in_ = nb_index(ci, ii, in.imax, in.bc[0], in.bc[1]);
            const int jn_ = nb_index(cj, jj, in.jmax, in.bc[2], in.bc[3]);
            const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
            lmin = fmin(lmin, mmi[(size_t)nc * 2 * V + v]);
            lmax = fmax(lmax, mmi[(size_t)nc * 2 * V + V + v]);
            if (a.mme[0]) en = fmaxf(en, a.mme[par][(size_t)nc * V + v]);
          }
        const double ldiff = fmax(fmax(1.0e-4, 1.0e-3 * (lmax - lmin)), 0.0);
        if (en == 0.0f) {
          if (cmn < lmin - ldiff || cmx > lmax + ldiff) atomicOr(&flag[0], 2);
        } else {
          // FP32-mixed: the own values are FP64; the neighbourhood bounds
          // carry at most en, so the threshold moves by at most en (1 + 2e-3).
          // Comparisons inside that margin are settled below (bit 4).
          const double M = 1.002 * (double)en + 1.0e-13 * (fabs(lmin) + fabs(lmax) + fabs(cmn) + fabs(cmx));
          if (cmn < lmin - ldiff - M || cmx > lmax + ldiff + M) atomicOr(&flag[0], 2);
          else if (!(cmn >= lmin - ldiff + M) || !(cmx <= lmax + ldiff - M)) atomicOr(&flag[0], 4);
        }
      }
    }
    __syncthreads();
    if constexpr (sizeof(T) == 8) {
      if (rec == 2 && a.mme[0] != nullptr && (flag[0] & 7) == 4) {
        // FP32-mixed, a recompute = 2 DMP the bounds left open: the min/max
        // of every neighbour whose stored values carry an error bound are
        // recomputed from its start-of-step state in FP64 reference order,
        // so that the decision is the FP64 path's on this state
        if (t == 0) atomicAdd(&a.st[k].n_settled, 1);
        double elmin = kInf, elmax = -kInf;
        for (int n = 0; n < 9; ++n) {
          const long long nc = nbc[n];
          bool comp = false;
          if (nbs[n] == 0) {
#pragma unroll
            for (int v = 0; v < V; ++v) comp = comp || a.mme[par][(size_t)nc * V + v] > 0.0f;
          }
          if (comp) {
            const double* un = a.uh[par] + (size_t)nc * P2 * V;
            for (int p = t; p < P2 * V; p += NT) {
              const int node = p / V, v = p - node * V;
              UN[v * P2 + node] = un[p];
            }
          }
          __syncthreads();
          if (comp) Proj<N, V, double>::ypass(UN, LY, LB, opsm, opsm + S * P, t, NT);
          __syncthreads();
          double nmn[V], nmx[V];
#pragma unroll
          for (int v = 0; v < V; ++v) { nmn[v] = kInf; nmx[v] = -kInf; }
          bool pdummy = false;
          if (comp) Proj<N, V, double>::template xpass_minmax<Sys>(UN, LY, LB, opsm, opsm + S * P, ph, t, NT, nmn, nmx, pdummy);
          warp_minmax_store<double, V, NW>(nmn, nmx, red, t);
          __syncthreads();
          if (t < V) {
            const int v = t;
            double lo, hi;
            if (comp) {
              lo = red[v * NW];
              hi = red[(V + v) * NW];
              for (int q = 1; q < NW; ++q) { lo = fmin(lo, red[v * NW + q]); hi = fmax(hi, red[(V + v) * NW + q]); }
            } else {
              lo = a.mm[par][(size_t)nc * 2 * V + v];
              hi = a.mm[par][(size_t)nc * 2 * V + V + v];
            }
            elmin = fmin(elmin, lo);
            elmax = fmax(elmax, hi);
          }
          __syncthreads();
        }
        if (t < V) {
          const double ldiff = fmax(fmax(1.0e-4, 1.0e-3 * (elmax - elmin)), 0.0);
          if (dmn < elmin - ldiff || dmx > elmax + ldiff) atomicOr(&flag[0], 2);
        }
        __syncthreads();
      }
    }
    // status: recompute 1 -> limited; recompute 2 -> limited only when the DMP fails
    const bool limited = rec == 1 || (rec == 2 && (flag[0] & 3) != 0);
    // min/max over the new subcell data (get_min_max of the next step), in T
    T* redt = reinterpret_cast<T*>(red);
    if (limited) {
      double* nl = a.lh[par ^ 1] + (size_t)c * S * S * V;
      for (int p = t; p < S * S; p += NT)
#pragma unroll
        for (int v = 0; v < V; ++v) nl[p * V + v] = (double)sub1[v * S * S + p];
      T tmn[V], tmx[V];
#pragma unroll
      for (int v = 0; v < V; ++v) { tmn[v] = T(kInf); tmx[v] = T(-kInf); }
      for (int p = t; p < S * S; p += NT)
#pragma unroll
        for (int v = 0; v < V; ++v) {
          tmn[v] = tmin(tmn[v], sub1[v * S * S + p]);
          tmx[v] = tmax(tmx[v], sub1[v * S * S + p]);
        }
      warp_minmax_store<T, V, NW>(tmn, tmx, redt, t);
    }
    __syncthreads();
    if (t < V) {
      const int v = t;
      double cmn = dmn, cmx = dmx;
      if (limited) {
        T lo = redt[v * NW], hi = redt[(V + v) * NW];
        for (int q = 1; q < NW; ++q) { lo = tmin(lo, redt[v * NW + q]); hi = tmax(hi, redt[(V + v) * NW + q]); }
        cmn = (double)lo;
        cmx = (double)hi;
      }
      mmo[v] = cmn;
      mmo[V + v] = cmx;
      if (a.mme[0]) a.mme[par ^ 1][(size_t)c * V + v] = 0.0f;  // FP64 values
    }
    if (t == 0) {
      a.status[par ^ 1][c] = limited ? 1 : 0;
      atomicMax(&a.st[k].denom_next, *cmaxp);
    }
    __syncthreads();
  }
}


// FP32-mixed: the DMP decisions k_cells left open (a.settle, a.list_count[1]
// entries), from FP64 values in the reference's order.  One CTA per listed
// cell, persistent over the list.  The cell's own subcell / Gauss-Lobatto /
// nodal min and max come from its new state (fused step: uh[par ^ 1]; initial
// DMP: uh[par]); the neighbourhood bounds (get_min_max, Euler/limiter.f90:
// 104-171) from the stored min/max where they are FP64 values (error bound 0,
// or limited cells, whose min/max come from Lh) and from the neighbour's
// start-of-step state otherwise.  The decision (Euler/limiter.f90:206-220) is
// then the FP64 path's on this state, bit for bit; a troubled cell is marked
// as k_cells marks it, and the cell's min/max for the next step become the
// FP64 values.  The initial DMP compares against the cell's own nodal
// min/max with argmax 0.1 (Euler/initialize.f90:287-307).
template <class Sys, int N>
__global__ void __launch_bounds__(128) k_settle(BatchArgs a, DevOps<N, double> op) {
  constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V, NT = 128, NW = NT / 32;
  __shared__ double U[V * P2], LY[V * S * P], LB[V * P * P], red[2 * V * NW], ops[S * P + P * P];
  __shared__ int flag;
  const int t = threadIdx.x;
  const int count = a.list_count[1];
  if (count == 0) return;
  for (int k = t; k < S * P + P * P; k += NT) ops[k] = k < S * P ? op.uh2lim[k] : op.uh2lob[k - S * P];
  const bool init = a.mode == kCellInitDmp;
  // FP64 min/max of the projections of the state U (all threads take part)
  auto minmax = [&](const Phys& ph, double* lo, double* hi) {
    __syncthreads();
    Proj<N, V, double>::ypass(U, LY, LB, ops, ops + S * P, t, NT);
    __syncthreads();
    double mn[V], mx[V];
#pragma unroll
    for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
    bool pdummy = false;  // positivity was decided by k_cells, exactly
    Proj<N, V, double>::template xpass_minmax<Sys>(U, LY, LB, ops, ops + S * P, ph, t, NT, mn, mx, pdummy);
    warp_minmax_store<double, V, NW>(mn, mx, red, t);
    __syncthreads();
    if (t < V) {
      double l = red[t * NW], h = red[(V + t) * NW];
      for (int q = 1; q < NW; ++q) { l = fmin(l, red[t * NW + q]); h = fmax(h, red[(V + t) * NW + q]); }
      *lo = l;
      *hi = h;
    }
  };
  for (int li = blockIdx.x; li < count; li += gridDim.x) {
    const long long cell = a.settle[li];
    const int k = find_inst_cell(a.inst, a.ninst, cell);
    const InstDesc& in = a.inst[k];
    const int par = parity(a.st[k]);
    const long long lc = cell - in.cell_base;
    const int ci = (int)(lc % in.imax), cj = (int)(lc / in.imax);
    const double* un = (init ? a.uh[par] : a.uh[par ^ 1]) + (size_t)cell * P2 * V;
    __syncthreads();  // the previous cell's readers of U are done
    for (int p = t; p < P2 * V; p += NT) U[(p % V) * P2 + p / V] = un[p];
    double cmn = 0.0, cmx = 0.0, lmin = kInf, lmax = -kInf;
    minmax(in.ph, &cmn, &cmx);
    if (init) {
      if (t < V)
        for (int q = 0; q < P2; ++q) { lmin = fmin(lmin, U[t * P2 + q]); lmax = fmax(lmax, U[t * P2 + q]); }
    } else {
      for (int n = 0; n < 9; ++n) {
        const int in_ = nb_index(ci, n % 3 - 1, in.imax, in.bc[0], in.bc[1]);
        const int jn_ = nb_index(cj, n / 3 - 1, in.jmax, in.bc[2], in.bc[3]);
        const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
        bool comp = false;
        if (a.status[par][nc] == 0) {
#pragma unroll
          for (int v = 0; v < V; ++v) comp = comp || a.mme[par][(size_t)nc * V + v] > 0.0f;
        }
        double lo = 0.0, hi = 0.0;
        if (comp) {  // uniform over the CTA
          __syncthreads();
          const double* nu = a.uh[par] + (size_t)nc * P2 * V;
          for (int p = t; p < P2 * V; p += NT) U[(p % V) * P2 + p / V] = nu[p];
          minmax(in.ph, &lo, &hi);
        } else if (t < V) {
          lo = a.mm[par][(size_t)nc * 2 * V + t];
          hi = a.mm[par][(size_t)nc * 2 * V + V + t];
        }
        if (t < V) {
          lmin = fmin(lmin, lo);
          lmax = fmax(lmax, hi);
        }
      }
    }
    if (t == 0) flag = 0;
    __syncthreads();
    if (t < V) {
      const double ldiff = fmax(fmax(1.0e-4, 1.0e-3 * (lmax - lmin)), init ? 1.0e-1 : 0.0);
      if (cmn < lmin - ldiff || cmx > lmax + ldiff) atomicOr(&flag, 1);
      if (!init) {
        a.mm[par ^ 1][(size_t)cell * 2 * V + t] = cmn;
        a.mm[par ^ 1][(size_t)cell * 2 * V + V + t] = cmx;
        a.mme[par ^ 1][(size_t)cell * V + t] = 0.0f;
        if (a.lminmax) {
          a.lminmax[(size_t)cell * 2 * V + t] = lmin;
          a.lminmax[(size_t)cell * 2 * V + V + t] = lmax;
        }
      }
    }
    __syncthreads();
    if (t == 0) atomicAdd(&a.st[k].n_settled, 1);
    if (flag) {
      if (init) {
        // as k_cells' initial limiter: status 1, Lh = the initial subcell data
        if (t == 0) {
          a.status[0][cell] = 1;
          a.status[1][cell] = 1;
          atomicAdd(&a.st[k].n_recompute, 1);
        }
        if (a.lh_ic) {
          const size_t o = (size_t)cell * S * S * V;
          for (int q = t; q < S * S * V; q += NT) {
            a.lh[0][o + q] = a.lh_ic[o + q];
            a.lh[1][o + q] = a.lh_ic[o + q];
          }
        }
      } else if (t == 0) {
        a.troubled[cell] = 1;
        atomicAdd(&a.st[k].n_recompute, 1);
      }
    }
  }
}

}  // namespace aderdg
