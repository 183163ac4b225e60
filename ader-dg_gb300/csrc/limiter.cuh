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
// Compiled with --fmad=false, reference operation order throughout.
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

template <class Sys, int N>
struct SubCfg {
  static constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V;
  static constexpr int R = S + 4;  // gathered region: subcells -1 .. S+2 (1-based)
  static constexpr int H = S + 2;  // reconstructed region: 0 .. S+1
  static constexpr int THREADS = 128;
  // doubles: sub0 [V][R*R], slopes x/y/t + wLx wRx wLy wRy [7][V][H*H], edge fluxes [2][V][(S+1)*S],
  // subuh1 [V][S*S], put_subcell_data / DMP scratch
  static constexpr int SCRATCH = V * S * P + V * P2 + V * S * P + V * P * P;
  static constexpr int DBL = V * R * R + 7 * V * H * H + 2 * V * (S + 1) * S + V * S * S + SCRATCH + 2 * V * THREADS;
  static constexpr int SMEM_BYTES = DBL * 8 + 64;
};

// minmod, Euler/limiter.f90:384-405
__device__ __forceinline__ double minmod(double a, double b) {
  if (a * b <= 0.0) return 0.0;
  return (fabs(a) < fabs(b)) ? a : b;
}

// Subgrid Rusanov flux (Euler/limiter.f90:361-378; BN :359-383 adds D = B~ dQ)
template <class Sys>
__device__ __forceinline__ void rusanov_s(const Phys& ph, const double* QL, const double* QR, int d, double* F, double* D) {
  constexpr int V = Sys::V;
  const double smax = fmax(Sys::max_eig(ph, QL, d), Sys::max_eig(ph, QR, d));
  double FLf[2 * V], FRf[2 * V];
  Sys::flux(ph, QL, FLf);
  Sys::flux(ph, QR, FRf);
  const double nv0 = d == 0 ? 1.0 : 0.0, nv1 = d == 0 ? 0.0 : 1.0;
#pragma unroll
  for (int v = 0; v < V; ++v)
    F[v] = 0.5 * ((FLf[v] + FRf[v]) * nv0 + (FLf[V + v] + FRf[V + v]) * nv1) - 0.5 * smax * (QR[v] - QL[v]);
  if constexpr (Sys::ID == kSysBN) BNSys::roe_times_jump(ph, QL, QR, d, D);
}

template <class Sys, int N>
__global__ void __launch_bounds__(SubCfg<Sys, N>::THREADS) k_subcell(BatchArgs a, DevOps<N, double> op, FaceConst fc) {
  using C = SubCfg<Sys, N>;
  constexpr int P = N + 1, P2 = P * P, S = 2 * N + 1, V = Sys::V, R = C::R, H = C::H, NT = C::THREADS;
  constexpr bool BN = Sys::ID == kSysBN;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sub0 = reinterpret_cast<double*>(smem_raw);
  double* slx = sub0 + V * R * R;
  double* sly = slx + V * H * H;
  double* slt = sly + V * H * H;
  double* wLx = slt + V * H * H;
  double* wRx = wLx + V * H * H;
  double* wLy = wRx + V * H * H;
  double* wRy = wLy + V * H * H;
  double* Fx = wRy + V * H * H;
  double* Fy = Fx + V * (S + 1) * S;
  double* sub1 = Fy + V * (S + 1) * S;
  double* scr = sub1 + V * S * S;
  double* red = scr + C::SCRATCH;
  int* flag = reinterpret_cast<int*>(red + 2 * V * NT);
  unsigned long long* cmaxp = reinterpret_cast<unsigned long long*>(flag + 2);

  const int t = threadIdx.x;
  auto SU = [&](int v, int ii, int jj) -> double& { return sub0[v * R * R + (ii + 1) + R * (jj + 1)]; };  // ii,jj in -1..S+2
  auto hx = [&](int v, int ii, int jj) { return v * H * H + ii + H * jj; };                              // ii,jj in 0..S+1

  const int count = *a.list_count;
  for (int li = blockIdx.x; li < count; li += gridDim.x) {
    const long long c = a.list[li];
    const int k = find_inst_cell(a.inst, a.ninst, c);
    const InstDesc& in = a.inst[k];
    const InstState& st = a.st[k];
    const Phys ph = in.ph;
    const int par = parity(st);
    const long long lc = c - in.cell_base;
    const int ci = (int)(lc % in.imax), cj = (int)(lc / in.imax);
    const int rec = a.recompute[c];
    const double dt = st.dt;
    const double ldx0 = in.dx / (double)S, ldx1 = in.dy / (double)S;
    const bool dmr = (Sys::ID == kSysEuler) && in.bc_mode == 1;

    // ---- gather the subcell data of the 3x3 neighbourhood (only the strip
    // the reconstruction reads): olduh projections or Lh of limited cells
    for (int p = t; p < R * R; p += NT) {
      const int ii = p % R - 1, jj = p / R - 1;
      const int bi = ii < 1 ? -1 : (ii > S ? 1 : 0), bj = jj < 1 ? -1 : (jj > S ? 1 : 0);
      const int sa = ii - 1 - bi * S, sb = jj - 1 - bj * S;
      const int in_ = nb_index(ci, bi, in.imax, in.bc[0], in.bc[1]);
      const int jn_ = nb_index(cj, bj, in.jmax, in.bc[2], in.bc[3]);
      const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
      double val[V];
      if (a.status[par][nc] == 0) {
        // get_subcell_data of olduh at subcell (sa, sb): y contraction then x
        const double* uo = a.uh[par] + (size_t)nc * P2 * V;
#pragma unroll
        for (int v = 0; v < V; ++v) {
          double acc = 0.0;
#pragma unroll
          for (int kk = 0; kk < P; ++kk) {
            double ly = 0.0;
#pragma unroll
            for (int m = 0; m < P; ++m) ly = ly + uo[(kk + P * m) * V + v] * op.uh2lim[sb + S * m];
            acc = acc + ly * op.uh2lim[sa + S * kk];
          }
          val[v] = acc;
        }
      } else {
        const double* L = a.lh[par] + ((size_t)nc * S * S + sa + S * sb) * V;
#pragma unroll
        for (int v = 0; v < V; ++v) val[v] = L[v];
      }
      if constexpr (Sys::ID == kSysEuler) {
        if (dmr) {  // Euler/limiter.f90:487-522, applied in the reference's order
          double Qbc[4];
          if (ci == 0 && ii <= 0) {
            EulerSys::prim2cons(ph, fc.Va, Qbc);
            for (int v = 0; v < 4; ++v) val[v] = Qbc[v];
          }
          if (cj == 0 && jj <= 0 && (double)(ci + 1) * in.dx > 1.0 / 6.0) val[2] = -val[2];
          if (cj == in.jmax - 1 && jj >= S + 1) {
            const double x_sw = fc.xsw0 + fc.xsw1 * st.time;
            EulerSys::prim2cons(ph, ((double)(ci + 1) * in.dx <= x_sw) ? fc.Va : fc.Vb, Qbc);
            for (int v = 0; v < 4; ++v) val[v] = Qbc[v];
          }
        }
      }
#pragma unroll
      for (int v = 0; v < V; ++v) SU(v, ii, jj) = val[v];
    }
    if (t == 0) {
      flag[0] = 0;
      *cmaxp = 0ull;
    }
    __syncthreads();

    // ---- MUSCL-Hancock reconstruction on subcells 0..S+1
    for (int p = t; p < H * H; p += NT) {
      const int ii = p % H, jj = p / H;
      double Qt[V], FLx[2 * V], FRx[2 * V], FLy[2 * V], FRy[2 * V];
      const bool interior = ii >= 1 && ii <= S && jj >= 1 && jj <= S;
      // Euler computes slopes for interior subcells only (halo slopes stay 0,
      // Euler/limiter.f90:529-536); BN also on the halo (BN :486-492)
#pragma unroll
      for (int v = 0; v < V; ++v) {
        double sx = 0.0, sy = 0.0;
        if (BN || interior) {
          sx = minmod(SU(v, ii + 1, jj) - SU(v, ii, jj), SU(v, ii, jj) - SU(v, ii - 1, jj));
          sy = minmod(SU(v, ii, jj + 1) - SU(v, ii, jj), SU(v, ii, jj) - SU(v, ii, jj - 1));
        }
        slx[hx(v, ii, jj)] = sx;
        sly[hx(v, ii, jj)] = sy;
      }
      double q0[V], wl[V], wr[V];
#pragma unroll
      for (int v = 0; v < V; ++v) q0[v] = SU(v, ii, jj);
      double src[V];
      if constexpr (BN) {
        // Baer-Nunziato/limiter.f90:494-497
        BNSys::src_ncp(ph, q0, slx[hx(8, ii, jj)] / ldx0, sly[hx(8, ii, jj)] / ldx1, src);
      }
#pragma unroll
      for (int v = 0; v < V; ++v) {
        wl[v] = q0[v] - 0.5 * slx[hx(v, ii, jj)];
        wr[v] = q0[v] + 0.5 * slx[hx(v, ii, jj)];
      }
      Sys::flux(ph, wl, FLx);
      Sys::flux(ph, wr, FRx);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        if constexpr (BN) Qt[v] = src[v] - (FRx[v] - FLx[v]) / ldx0;
        else Qt[v] = -(FRx[v] - FLx[v]) / ldx0;
        wLx[hx(v, ii, jj)] = wl[v];
        wRx[hx(v, ii, jj)] = wr[v];
      }
#pragma unroll
      for (int v = 0; v < V; ++v) {
        wl[v] = q0[v] - 0.5 * sly[hx(v, ii, jj)];
        wr[v] = q0[v] + 0.5 * sly[hx(v, ii, jj)];
      }
      Sys::flux(ph, wl, FLy);
      Sys::flux(ph, wr, FRy);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        Qt[v] = Qt[v] - (FRy[V + v] - FLy[V + v]) / ldx1;
        slt[hx(v, ii, jj)] = Qt[v];
        wLx[hx(v, ii, jj)] = wLx[hx(v, ii, jj)] + 0.5 * dt * Qt[v];
        wRx[hx(v, ii, jj)] = wRx[hx(v, ii, jj)] + 0.5 * dt * Qt[v];
        wLy[hx(v, ii, jj)] = wl[v] + 0.5 * dt * Qt[v];
        wRy[hx(v, ii, jj)] = wr[v] + 0.5 * dt * Qt[v];
      }
    }
    __syncthreads();

    if constexpr (!BN) {
      // edge fluxes Fx(1..S+1, 1..S), Fy(1..S, 1..S+1), Euler/limiter.f90:571-588
      for (int p = t; p < 2 * (S + 1) * S; p += NT) {
        const bool xd = p < (S + 1) * S;
        const int q = xd ? p : p - (S + 1) * S;
        double QL[V], QR[V], F[V], Dd[V];
        int ii, jj;
        if (xd) { ii = q % (S + 1) + 1; jj = q / (S + 1) + 1; }
        else { ii = q % S + 1; jj = q / S + 1; }
#pragma unroll
        for (int v = 0; v < V; ++v) {
          QL[v] = xd ? wRx[hx(v, ii - 1, jj)] : wRy[hx(v, ii, jj - 1)];
          QR[v] = xd ? wLx[hx(v, ii, jj)] : wLy[hx(v, ii, jj)];
        }
        rusanov_s<Sys>(ph, QL, QR, xd ? 0 : 1, F, Dd);
        double* dst = xd ? Fx : Fy;
#pragma unroll
        for (int v = 0; v < V; ++v) dst[v * (S + 1) * S + q] = F[v];
      }
      __syncthreads();
      // first-order FV update, Euler/limiter.f90:592-597
      for (int p = t; p < S * S; p += NT) {
        const int ii = p % S + 1, jj = p / S + 1;
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const double fxp = Fx[v * (S + 1) * S + ii + (S + 1) * (jj - 1)];
          const double fxm = Fx[v * (S + 1) * S + (ii - 1) + (S + 1) * (jj - 1)];
          const double fyp = Fy[v * (S + 1) * S + (ii - 1) + S * jj];
          const double fym = Fy[v * (S + 1) * S + (ii - 1) + S * (jj - 1)];
          sub1[v * S * S + p] = SU(v, ii, jj) - dt / ldx0 * (fxp - fxm) - dt / ldx1 * (fyp - fym);
        }
      }
    } else {
      // Baer-Nunziato/limiter.f90:526-545: four fluxes per subcell
      for (int p = t; p < S * S; p += NT) {
        const int ii = p % S + 1, jj = p / S + 1;
        double qh[V], src[V], fpl[V], fmi[V], gpl[V], gmi[V], Dpx[V], Dmx[V], Dpy[V], Dmy[V], QL[V], QR[V];
#pragma unroll
        for (int v = 0; v < V; ++v) qh[v] = SU(v, ii, jj) + 0.5 * dt * slt[hx(v, ii, jj)];
        BNSys::src_ncp(ph, qh, slx[hx(8, ii, jj)] / ldx0, sly[hx(8, ii, jj)] / ldx1, src);
#pragma unroll
        for (int v = 0; v < V; ++v) { QL[v] = wRx[hx(v, ii, jj)]; QR[v] = wLx[hx(v, ii + 1, jj)]; }
        rusanov_s<Sys>(ph, QL, QR, 0, fpl, Dpx);
#pragma unroll
        for (int v = 0; v < V; ++v) { QL[v] = wRx[hx(v, ii - 1, jj)]; QR[v] = wLx[hx(v, ii, jj)]; }
        rusanov_s<Sys>(ph, QL, QR, 0, fmi, Dmx);
#pragma unroll
        for (int v = 0; v < V; ++v) { QL[v] = wRy[hx(v, ii, jj)]; QR[v] = wLy[hx(v, ii, jj + 1)]; }
        rusanov_s<Sys>(ph, QL, QR, 1, gpl, Dpy);
#pragma unroll
        for (int v = 0; v < V; ++v) { QL[v] = wRy[hx(v, ii, jj - 1)]; QR[v] = wLy[hx(v, ii, jj)]; }
        rusanov_s<Sys>(ph, QL, QR, 1, gmi, Dmy);
#pragma unroll
        for (int v = 0; v < V; ++v)
          sub1[v * S * S + p] = SU(v, ii, jj) - dt / ldx0 * (fpl[v] - fmi[v]) - dt / ldx1 * (gpl[v] - gmi[v]) -
                                dt / ldx0 * 0.5 * (Dpx[v] + Dmx[v]) - dt / ldx1 * 0.5 * (Dpy[v] + Dmy[v]) + dt * src[v];
      }
    }
    __syncthreads();

    // ---- put_subcell_data (Euler/limiter.f90:74-98): luhy then luh
    double* LUY = scr;                 // [V][P][S]: luhy(v, iii, s) at (v*P + s)*S + iii
    double* UN = scr + V * S * P;      // [V][P2]
    double* LY = UN + V * P2;          // DMP y pass [V][S][P]
    double* LB = LY + V * S * P;       // [V][P][P]
    for (int p = t; p < S * P; p += NT) {
      const int iii = p % S, s = p / S;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        double acc = 0.0;
        for (int kk = 0; kk < S; ++kk) acc = acc + sub1[v * S * S + iii + S * kk] * op.lim2uh[s + P * kk];
        LUY[(v * P + s) * S + iii] = acc;
      }
    }
    __syncthreads();
    double* uout = a.uh[par ^ 1] + (size_t)c * P2 * V;
    for (int p = t; p < P2; p += NT) {
      const int s1 = p % P, jjj = p / P;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        double acc = 0.0;
        for (int kk = 0; kk < S; ++kk) acc = acc + LUY[(v * P + jjj) * S + kk] * op.lim2uh[s1 + P * kk];
        UN[v * P2 + p] = acc;
        uout[p * V + v] = acc;
      }
    }
    __syncthreads();

    // ---- DMP of the new polynomial (recompute = 2) and the next min/max
    Proj<N, V>::ypass(UN, LY, LB, op, t, NT);
    __syncthreads();
    double mn[V], mx[V];
    bool posfail = false;
#pragma unroll
    for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
    Proj<N, V>::template xpass_minmax<Sys>(UN, LY, LB, op, ph, t, NT, mn, mx, posfail);
#pragma unroll
    for (int v = 0; v < V; ++v) { red[v * NT + t] = mn[v]; red[(V + v) * NT + t] = mx[v]; }
    if (posfail) atomicOr(&flag[0], 1);
    // CFL denominator of the new polynomial
    for (int p = t; p < P2; p += NT) {
      double Q[V];
#pragma unroll
      for (int v = 0; v < V; ++v) Q[v] = UN[v * P2 + p];
      atomicMax(cmaxp, (unsigned long long)__double_as_longlong(cfl_denom<Sys, N>(in, Q)));
    }
    __syncthreads();
    double* mmo = a.mm[par ^ 1] + (size_t)c * 2 * V;
    if (t < V) {
      const int v = t;
      double cmn = red[v * NT], cmx = red[(V + v) * NT];
      for (int q = 1; q < NT; ++q) { cmn = fmin(cmn, red[v * NT + q]); cmx = fmax(cmx, red[(V + v) * NT + q]); }
      red[v * NT] = cmn;
      red[(V + v) * NT] = cmx;
      if (rec == 2) {
        const double* mmi = a.mm[par];
        double lmin = mmi[(size_t)c * 2 * V + v], lmax = mmi[(size_t)c * 2 * V + V + v];
        for (int jj = -1; jj <= 1; ++jj)
          for (int ii = -1; ii <= 1; ++ii) {
            const int in_ = nb_index(ci, ii, in.imax, in.bc[0], in.bc[1]);
            const int jn_ = nb_index(cj, jj, in.jmax, in.bc[2], in.bc[3]);
            const long long nc = in.cell_base + in_ + (long long)in.imax * jn_;
            lmin = fmin(lmin, mmi[(size_t)nc * 2 * V + v]);
            lmax = fmax(lmax, mmi[(size_t)nc * 2 * V + V + v]);
          }
        const double ldiff = fmax(fmax(1.0e-4, 1.0e-3 * (lmax - lmin)), 0.0);
        if (cmn < lmin - ldiff || cmx > lmax + ldiff) atomicOr(&flag[0], 2);
      }
    }
    __syncthreads();
    // status: recompute 1 -> limited; recompute 2 -> limited only when the DMP fails
    const bool limited = rec == 1 || (rec == 2 && flag[0] != 0);
    if (limited) {
      double* nl = a.lh[par ^ 1] + (size_t)c * S * S * V;
      for (int p = t; p < S * S; p += NT)
#pragma unroll
        for (int v = 0; v < V; ++v) nl[p * V + v] = sub1[v * S * S + p];
      // min/max over the new subcell data (get_min_max of the next step)
      for (int v = 0; v < V; ++v) { mn[v] = kInf; mx[v] = -kInf; }
      for (int p = t; p < S * S; p += NT)
#pragma unroll
        for (int v = 0; v < V; ++v) { mn[v] = fmin(mn[v], sub1[v * S * S + p]); mx[v] = fmax(mx[v], sub1[v * S * S + p]); }
    }
    __syncthreads();
    if (limited) {
#pragma unroll
      for (int v = 0; v < V; ++v) { red[v * NT + t] = mn[v]; red[(V + v) * NT + t] = mx[v]; }
    }
    __syncthreads();
    if (t < V) {
      const int v = t;
      double cmn = red[v * NT], cmx = red[(V + v) * NT];
      if (limited)
        for (int q = 1; q < NT; ++q) { cmn = fmin(cmn, red[v * NT + q]); cmx = fmax(cmx, red[(V + v) * NT + q]); }
      mmo[v] = cmn;
      mmo[V + v] = cmx;
    }
    if (t == 0) {
      a.status[par ^ 1][c] = limited ? 1 : 0;
      atomicMax(&a.st[k].denom_next, *cmaxp);
    }
    __syncthreads();
  }
}

}  // namespace aderdg
