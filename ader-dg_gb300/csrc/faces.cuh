// faces.cuh -- K2: numerical fluxes once per face quadrature point, with the
// boundary conditions inlined.
//
// Reference: Euler/riemann_problem.f90:10-116 (Rusanov, double Mach
// reflection boundaries), Baer-Nunziato/riemann_problem.f90:9-80
// (path-conservative Rusanov fluctuations Dm/Dp), and
// Advection-Diffusion/riemann_problem.f90:8-113 (viscous LLF).  One thread per
// (face, point); the x faces of all instances come first, then the y faces.
// R is the storage type of the face states and fluxes, CT the compute type.
// FP64 (R = CT = double) is compiled with --fmad=false: every value agrees bit
// for bit with the reference expression evaluated in FP64 from the same face
// states.  The FP32 modes store states and fluxes in FP32; Euler and
// advection-diffusion compute in FP32, and Baer-Nunziato computes its
// path-conservative flux (Roe-matrix path integral included) in FP64 in the
// FP32-mixed mode (CT = double, instantiated with fused multiply-adds in
// predictor_tu.cu) and in FP32 in the FP32-wide mode.
#pragma once

#include "common.cuh"
#include "physics.cuh"

namespace aderdg {

// instance owning an x / y face, or -1 (faces between instances of a batch)
__device__ __forceinline__ int find_inst_fx(const InstDesc* inst, int n, long long f) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (inst[mid].fx_base <= f) lo = mid; else hi = mid - 1;
  }
  const InstDesc& d = inst[lo];
  if (f < d.fx_base || f - d.fx_base >= (long long)(d.imax + 1) * d.jmax) return -1;
  return lo;
}
__device__ __forceinline__ int find_inst_fy(const InstDesc* inst, int n, long long f) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (inst[mid].fy_base <= f) lo = mid; else hi = mid - 1;
  }
  const InstDesc& d = inst[lo];
  if (f < d.fy_base || f - d.fy_base >= (long long)d.imax * (d.jmax + 1)) return -1;
  return lo;
}

template <int V, class R, class T>
__device__ __forceinline__ void load_face_state(const R* qb, const R* fb, long long cell, int P, int l, int f, T* Q, T* F) {
  const size_t o = (((size_t)cell * 4 + f) * P + l) * V;  // [cell][face][point][v]
#pragma unroll
  for (int v = 0; v < V; ++v) {
    Q[v] = widen<T>(qb[o + v]);
    if (F) F[v] = widen<T>(fb[o + v]);
  }
}

// Euler double Mach reflection boundary state: Q = prim2cons(Vp), F = flux(Q)
// along axis d (matmul(Fbc, nv) of Euler/riemann_problem.f90:43-46).
template <class T>
__device__ __forceinline__ void dmr_state(const PhysC<T>& pc, const double* Vpd, int d, T* Q, T* F) {
  T Fb[8], Vp[4];
  for (int v = 0; v < 4; ++v) Vp[v] = (T)Vpd[v];
  EulerSys::prim2cons(pc, Vp, Q);
  EulerSys::flux(pc, Q, Fb);
  for (int v = 0; v < 4; ++v) F[v] = Fb[d * 4 + v];
}

// Euler Rusanov pieces in the compute type T (FP32 in the FP32 modes)
template <class T>
__device__ __forceinline__ T euler_max_eig_t(T gamma, const T* Q, int d) {
  const T u = (d == 0 ? Q[1] : Q[2]) / Q[0];
  const T p = (gamma - T(1)) * (Q[3] - T(0.5) * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
  const T c = sqrt(gamma * p / Q[0]);
  return fmax(fmax(fabs(u - c), fabs(u)), fabs(u + c));
}
template <class T>
__device__ __forceinline__ void euler_bc_state_t(T gamma, const double* Vp, int d, T* Q, T* F) {
  Q[0] = T(Vp[0]);
  Q[1] = T(Vp[0] * Vp[1]);
  Q[2] = T(Vp[0] * Vp[2]);
  Q[3] = T(Vp[3] / (double(gamma) - 1) + 0.5 * Vp[0] * (Vp[1] * Vp[1] + Vp[2] * Vp[2]));
  const T irho = T(1) / Q[0];
  const T p = (gamma - T(1)) * (Q[3] - T(0.5) * (Q[1] * Q[1] + Q[2] * Q[2]) * irho);
  const T un = (d == 0 ? Q[1] : Q[2]);
  F[0] = un;
  F[1] = irho * un * Q[1] + (d == 0 ? p : T(0));
  F[2] = irho * un * Q[2] + (d == 1 ? p : T(0));
  F[3] = irho * un * (Q[3] + p);
}

// FP32-mixed faces for Euler: boundary logic as in k_faces, arithmetic in FP32
template <int N>
__device__ void faces_euler_fp32(const BatchArgs& a, const FaceConst& fc, const InstDesc& in, int k, bool xdir, int i,
                                 int j, int l, long long face) {
  constexpr int P = N + 1, V = 4;
  const float* qb = reinterpret_cast<const float*>(a.qbnd);
  const float* fb = reinterpret_cast<const float*>(a.fbnd);
  const int I = in.imax, J = in.jmax;
  auto cid = [&](int ci, int cj) { return in.cell_base + (long long)ci + (long long)I * cj; };
  auto load = [&](long long c, int f, float* Q, float* F) {
    const size_t o = (((size_t)c * 4 + f) * P + l) * V;
#pragma unroll
    for (int v = 0; v < V; ++v) { Q[v] = qb[o + v]; F[v] = fb[o + v]; }
  };
  const float gamma = (float)in.ph.gamma;
  const int d = xdir ? 0 : 1, pos = xdir ? i : j, last = xdir ? I : J;
  const int bcl = in.bc[xdir ? 0 : 2], bcr = in.bc[xdir ? 1 : 3];
  const int fl = xdir ? 0 : 2, fr = xdir ? 1 : 3;
  const bool is_dmr = in.bc_mode == 1;
  float QL[V], QR[V], FL[V], FR[V];
  const long long cR = cid(i, j);
  if (pos == 0) {
    if (is_dmr && xdir) {
      euler_bc_state_t<float>(gamma, fc.Va, 0, QL, FL);
      load(cR, fl, QR, FR);
    } else if (is_dmr) {
      load(cR, fl, QL, FL);
      if (!((double)(i + 1) * in.dx <= 1.0 / 6.0)) {
        QL[2] = -QL[2];
        FL[0] = -FL[0];
        FL[1] = -FL[1];
        FL[3] = -FL[3];
      }
      load(cR, fl, QR, FR);
    } else if (bcl == 3) {
      load(xdir ? cid(I - 1, j) : cid(i, J - 1), fr, QL, FL);
      load(cR, fl, QR, FR);
    } else {
      load(cR, fl, QL, FL);
      load(cR, fl, QR, FR);
    }
  } else if (pos == last) {
    const long long cLast = xdir ? cid(I - 1, j) : cid(i, J - 1);
    load(cLast, fr, QL, FL);
    if (is_dmr && !xdir) {
      const double x_sw = fc.xsw0 + fc.xsw1 * a.st[k].time;
      euler_bc_state_t<float>(gamma, ((double)(i + 1) * in.dx <= x_sw) ? fc.Va : fc.Vb, 1, QR, FR);
    } else if (!is_dmr && bcr == 3) {
      load(xdir ? cid(0, j) : cid(i, 0), fl, QR, FR);
    } else {
      load(cLast, fr, QR, FR);
    }
  } else {
    load(xdir ? cid(i - 1, j) : cid(i, j - 1), fr, QL, FL);
    load(cR, fl, QR, FR);
  }
  const float smax = fmaxf(euler_max_eig_t<float>(gamma, QL, d), euler_max_eig_t<float>(gamma, QR, d));
  float* dst = reinterpret_cast<float*>(xdir ? a.fu : a.gu) + ((size_t)face * P + l) * V;
#pragma unroll
  for (int v = 0; v < V; ++v) dst[v] = 0.5f * (FL[v] + FR[v]) - 0.5f * smax * (QR[v] - QL[v]);
}

template <class Sys, int N, class R, class CT>
__global__ void __launch_bounds__(256) k_faces(BatchArgs a, FaceConst fc) {
  constexpr int P = N + 1, V = Sys::V;
  const long long nx = a.nfx * P, ny = a.nfy * P;
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nx + ny) return;
  const R* qb = reinterpret_cast<const R*>(a.qbnd);
  const R* fb = reinterpret_cast<const R*>(a.fbnd);
  // x and y face points interleave warp by warp, so that the x faces and the
  // y faces of the same cells run at the same time: a cell's face states lie
  // side by side ([cell][P][4 faces][V]) and each DRAM burst then serves both
  // directions instead of being fetched once per direction
  const long long mw = (nx < ny ? nx : ny) >> 5;  // interleaved warp pairs
  bool xdir;
  long long g;
  if (gid < 64 * mw) {
    const long long w = gid >> 5;
    xdir = (w & 1) == 0;
    g = (w >> 1) * 32 + (gid & 31);
  } else {
    // the rest: x points [32 mw, nx), then y points [32 mw, ny)
    const long long r = gid - 64 * mw, rx = nx - 32 * mw;
    xdir = r < rx;
    g = 32 * mw + (xdir ? r : r - rx);
  }
  const long long face = g / P;
  const int l = (int)(g - face * P);
  const int k = xdir ? find_inst_fx(a.inst, a.ninst, face) : find_inst_fy(a.inst, a.ninst, face);
  if (k < 0) return;
  const InstDesc& in = a.inst[k];
  if (!a.st[k].active) return;
  const Phys ph = in.ph;
  const int I = in.imax, J = in.jmax;
  const long long lf = face - (xdir ? in.fx_base : in.fy_base);
  int i, j;
  if (xdir) { i = (int)(lf % (I + 1)); j = (int)(lf / (I + 1)); }
  else { i = (int)(lf % I); j = (int)(lf / I); }
  auto cid = [&](int ci, int cj) { return in.cell_base + (long long)ci + (long long)I * cj; };
  const int d = xdir ? 0 : 1;
  const int nfaces_side = xdir ? I : J;  // index of the last face along d is nfaces_side
  const int pos = xdir ? i : j;
  const int bcl = in.bc[xdir ? 0 : 2], bcr = in.bc[xdir ? 1 : 3];
  const int fl = xdir ? 0 : 2, fr = xdir ? 1 : 3;  // left/bottom and right/top face ids
  const size_t out = ((size_t)face * P + l) * V;
  if constexpr (Sys::ID == kSysEuler && sizeof(R) == 4) {
    static_assert(sizeof(CT) == 4, "Euler's FP32-storage faces compute in FP32");
    faces_euler_fp32<N>(a, fc, in, k, xdir, i, j, l, face);
    return;
  }

  if constexpr (Sys::ID == kSysAD) {
    // Advection-Diffusion/riemann_problem.f90 with PDEViscLLFRiemannSolver (pde.f90:121-152);
    // compute type: FP64 (reference order), FP32 in the FP32 modes
    CT QL[1], QR[1], gL[2], gR[2];
    auto get = [&](long long c, int f, CT* Q, CT* gq) {
      const size_t o = (((size_t)c * 4 + f) * P + l);
      Q[0] = (CT)qb[o];
      gq[0] = (CT)fb[o * 2 + 0];
      gq[1] = (CT)fb[o * 2 + 1];
    };
    const long long cL = xdir ? cid(i - 1, j) : cid(i, j - 1);
    const long long cR = cid(i, j);
    if (pos == 0) {
      if (bcl == 1) {
        get(cR, fl, QL, gL);
        get(cR, fl, QR, gR);
      } else if (bcl == 2) {
        if (xdir) {
          // QR from the right face of cell IMAX, QL = -QR + 2 sin(pi y),
          // y = (j-1 + xi_l) dy (Advection-Diffusion/riemann_problem.f90:37-40)
          get(cid(I - 1, j), 1, QR, gR);
          const double y = ((double)j + fc.xi[l]) * in.dy;
          QL[0] = -QR[0] + (CT)(2.0 * sin(fc.pi * y));
        } else {
          get(cR, fl, QR, gR);
          QL[0] = -QR[0];
        }
        gL[0] = gR[0];
        gL[1] = gR[1];
      } else {
        get(xdir ? cid(I - 1, j) : cid(i, J - 1), fr, QL, gL);
        get(cR, fl, QR, gR);
      }
    } else if (pos == nfaces_side) {
      const long long cLast = xdir ? cid(I - 1, j) : cid(i, J - 1);
      if (bcr == 1) {
        get(cLast, fr, QL, gL);
        get(cLast, fr, QR, gR);
      } else if (bcr == 2) {
        get(cLast, fr, QL, gL);
        QR[0] = -QL[0];
        gR[0] = gL[0];
        gR[1] = gL[1];
      } else {
        get(cLast, fr, QL, gL);
        get(xdir ? cid(0, j) : cid(i, 0), fl, QR, gR);
      }
    } else {
      get(cL, fr, QL, gL);
      get(cR, fl, QR, gR);
    }
    const CT nv0 = xdir ? CT(1) : CT(0), nv1 = xdir ? CT(0) : CT(1);
    // smax = max(|c.n|) + 2 eta a, eta = (2N+1) / (dx sqrt(pi/2)): formed on the host
    const CT smax = (CT)in.ad_smax[xdir ? 0 : 1];
    const CT cx = (CT)ph.cx, cy = (CT)ph.cy, ca = (CT)ph.a;
    const CT FL0 = cx * QL[0] + -ca * gL[0], FL1 = cy * QL[0] + -ca * gL[1];
    const CT FR0 = cx * QR[0] + -ca * gR[0], FR1 = cy * QR[0] + -ca * gR[1];
    R* dst = reinterpret_cast<R*>(xdir ? a.fu : a.gu);
    dst[out] = (R)(CT(0.5) * ((FL0 + FR0) * nv0 + (FL1 + FR1) * nv1) - CT(0.5) * smax * (QR[0] - QL[0]));
  } else {
    // Euler (FP64) and Baer-Nunziato (FP64 or FP32 compute, see above)
    const PhysC<CT> pc(ph);
    CT QL[V], QR[V], FL[V], FR[V];
    const bool is_dmr = (Sys::ID == kSysEuler) && in.bc_mode == 1;
    const long long cL = xdir ? cid(i - 1, j) : cid(i, j - 1);
    const long long cR = cid(i, j);
    if (pos == 0) {
      if (is_dmr) {
        if (xdir) {  // inflow, Euler/riemann_problem.f90:41-48
          dmr_state(pc, fc.Va, 0, QL, FL);
          load_face_state<V, R>(qb, fb, cR, P, l, fl, QR, FR);
        } else {     // transmissive / reflective wall, :76-86
          load_face_state<V, R>(qb, fb, cR, P, l, fl, QL, FL);
          if (!((double)(i + 1) * in.dx <= 1.0 / 6.0)) {
            QL[2] = -QL[2];
            FL[0] = -FL[0];
            FL[1] = -FL[1];
            FL[3] = -FL[3];
          }
          load_face_state<V, R>(qb, fb, cR, P, l, fl, QR, FR);
        }
      } else if (bcl == 3) {
        load_face_state<V, R>(qb, fb, xdir ? cid(I - 1, j) : cid(i, J - 1), P, l, fr, QL, FL);
        load_face_state<V, R>(qb, fb, cR, P, l, fl, QR, FR);
      } else {
        load_face_state<V, R>(qb, fb, cR, P, l, fl, QL, FL);
        load_face_state<V, R>(qb, fb, cR, P, l, fl, QR, FR);
      }
    } else if (pos == nfaces_side) {
      const long long cLast = xdir ? cid(I - 1, j) : cid(i, J - 1);
      load_face_state<V, R>(qb, fb, cLast, P, l, fr, QL, FL);
      if (is_dmr && !xdir) {  // time-dependent top boundary, :88-100
        const double x_sw = fc.xsw0 + fc.xsw1 * a.st[k].time;
        dmr_state(pc, ((double)(i + 1) * in.dx <= x_sw) ? fc.Va : fc.Vb, 1, QR, FR);
      } else if (!is_dmr && bcr == 3) {
        load_face_state<V, R>(qb, fb, xdir ? cid(0, j) : cid(i, 0), P, l, fl, QR, FR);
      } else {
        load_face_state<V, R>(qb, fb, cLast, P, l, fr, QR, FR);
      }
    } else {
      load_face_state<V, R>(qb, fb, cL, P, l, fr, QL, FL);
      load_face_state<V, R>(qb, fb, cR, P, l, fl, QR, FR);
    }
    // FP32-mixed Baer-Nunziato: FP64 with the reciprocal-sharing forms
    constexpr bool kRcp = sizeof(R) == 4 && sizeof(CT) == 8;
    // Rusanov: smax from both sides' eigenvalues (Euler/pde.f90:97-114)
    CT smax;
    if constexpr (kRcp) smax = tmax(Sys::max_eig_r(pc, QL, d), Sys::max_eig_r(pc, QR, d));
    else smax = tmax(Sys::max_eig(pc, QL, d), Sys::max_eig(pc, QR, d));
    if constexpr (Sys::ID == kSysBN) {
      // path-conservative fluctuations, Baer-Nunziato/pde.f90:326-353
      CT D[9];
      if constexpr (kRcp) BNSys::roe_times_jump_r(pc, QL, QR, d, D);
      else BNSys::roe_times_jump(pc, QL, QR, d, D);
      R* dm = reinterpret_cast<R*>(xdir ? a.fu : a.gu);
      R* dp = reinterpret_cast<R*>(xdir ? a.fp : a.gp);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const CT base = CT(0.5) * (FL[v] + FR[v]) - CT(0.5) * smax * (QR[v] - QL[v]);
        dm[out + v] = (R)(base - CT(0.5) * D[v]);
        dp[out + v] = (R)(base + CT(0.5) * D[v]);
      }
    } else {
      R* dst = reinterpret_cast<R*>(xdir ? a.fu : a.gu);
#pragma unroll
      for (int v = 0; v < V; ++v) dst[out + v] = (R)(CT(0.5) * (FL[v] + FR[v]) - CT(0.5) * smax * (QR[v] - QL[v]));
    }
  }
}

}  // namespace aderdg
