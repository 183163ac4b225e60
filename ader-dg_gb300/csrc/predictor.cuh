// predictor.cuh -- K1: cell-local space-time predictor (Picard iteration),
// fused with the volume integral and the face extrapolation.
//
// Reference: Euler/space_time_predictor.f90:8-123,
// Baer-Nunziato/space_time_predictor.f90:8-143,
// Advection-Diffusion/space_time_predictor.f90:10-155, and
// volume_integral.f90 of each solver.
//
// Mapping: one thread per spatial node (i,j) of a cell, CPB cells per CTA.
// Each thread keeps its node's time column q(l, v), l = 0..N, in registers;
// the flux-derivative contractions in x and y are the only operations that
// cross nodes and go through shared memory once per Picard iteration.
//
// Algebra (same as the reference, regrouped for fused multiply-adds):
//   rhs(l)  = w_i w_j F0(l) u - w_l w_j dt/dx (Fx Kxi)_i - w_l w_i dt/dy (Fy Kxi)_j  [+ w_i w_j w_l dt S(l)]
//   q(l')   = 1/(w_i w_j) sum_l iK1(l',l) rhs(l)
//           = g(l') u - sum_l T(l',l) b_l,   b_l = sum_k Dx(i,k) Fx(k,j,l) + sum_k Dy(j,k) Fy(i,k,l) [- dt S(l)]
// with T(l',l) = iK1(l',l) w_l, g = iK1 F0, Dx(i,k) = Kxi(k,i) dt/(dx w_i).
// The first iteration starts from q(l) = u for every l, so its fluxes and
// contractions are evaluated once instead of N+1 times.  The last iteration
// only needs the time average qhi = sum_l' w_l' q(l'), contracted directly.
// Fhi (and Shi) are the time averages of the last iteration's fluxes, as in
// the reference, where lFh is not recomputed after the final iK1 update.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "physics.cuh"

namespace aderdg {

// Shape of the FP32 predictor that the tuner (aderdg/tuner.py) picks per
// (system, N, precision): kCta scales the cells per CTA (+1: twice the
// threads, -1: half), kBlocks adds to the CTAs per SM the register
// allocation aims at, kUnroll unrolls the middle Picard iterations, and
// kNoRowCol contracts per node instead of by rows and columns, and kMma runs
// the row/column pass on the tensor cores (mma_pass).  PredTune<> is the
// hand-measured default.
template <int kCta = 0, int kBlocks = 0, bool kUnroll = false, bool kNoRowCol = false, bool kMma = false>
struct PredTune {
  static constexpr int CTA = kCta, BLOCKS = kBlocks;
  static constexpr bool UNROLL = kUnroll, NO_ROWCOL = kNoRowCol, MMA = kMma;
};
// the tuner's candidates, variant 0 the default
template <int K>
using PredVariant = typename std::conditional<
    K == 1, PredTune<1>,
    typename std::conditional<
        K == 2, PredTune<-1>,
        typename std::conditional<K == 3, PredTune<0, 1>,
                                  typename std::conditional<K == 4, PredTune<0, 0, true>,
                                                            typename std::conditional<K == 5, PredTune<0, 0, false, true>,
                                                                                      typename std::conditional<K == 6, PredTune<0, 0, false, false, true>,
                                                                                                                PredTune<>>::type>::type>::type>::type>::type>::type;
constexpr int kPredVariants = 7;

template <class Sys, int N, class R, class Tune = PredTune<>>
struct PredCfg {
  static constexpr int P = N + 1, P2 = P * P, V = Sys::V;
  // variables of one node padded to whole 16-byte vectors (AD: scalar)
  static constexpr int VEC = 16 / (int)sizeof(R);
  // flux components stored and contracted: Baer-Nunziato's volume fraction
  // has no conservative flux (its ninth component is 0, Baer-Nunziato/pde.f90:74-119),
  // so FP32 stores 8 (two float4) where that is faster (N <= 4; at N = 5
  // the larger cells-per-CTA it allows spill registers); elsewhere all 9 (measured)
  static constexpr int VF = (Sys::ID == kSysBN && sizeof(R) == 4 && N <= 4) ? 8 : V;
  // FP32: pad to whole float4; FP64: double2 when VF is even
  static constexpr int VP = (VF == 1) ? 1 : (sizeof(R) == 4 ? ((VF + VEC - 1) / VEC) * VEC : VF);
  // Flux buffer layout.  FP64 and AD: [P][2][P2][VP], a node's variables
  // contiguous.  FP32 Euler / Baer-Nunziato: each 16-byte chunk of the node
  // vectors in a plane of its own, [chunk][P][2][P2] float4, so that the eight
  // lanes of a quarter-warp (one 16-byte access each) address eight different
  // bank groups; with the chunks interleaved, lanes j and j+1 of a row
  // contraction met in the same group (2-way conflicts on Baer-Nunziato's
  // stores and x contraction).  PC_PAD pads the planes and CE_PAD the cells
  // (float4): the values that leave no conflict, or the fewest, in the
  // stores and both contractions at this degree's cells-per-CTA.
  static constexpr bool PLANAR = sizeof(R) == 4 && VF > 1;
  static constexpr int NCH = PLANAR ? VP / 4 : 1;
  // Row/column contraction (FP32 Euler / Baer-Nunziato, P >= 4): in the
  // Picard iterations 2..N each thread also contracts one x row and one y
  // column of one time level (the level its i names, the row / column its j
  // names) in registers, in place, and the node's thread reads back the two
  // contracted vectors per level: 8 P^2 accesses of 16 bytes per level and
  // cell instead of (2P + 2) P^2 with every node reading its 2P neighbours.
  // The x levels then the y levels, each level padded to XL / YL nodes; at
  // P >= 5 the y pass takes level j and column i (the lanes of a quarter-warp
  // then meet no bank group twice at these paddings).
  static constexpr bool ROWCOL = PLANAR && P >= 4 && !Tune::NO_ROWCOL;
  static constexpr bool MMA = ROWCOL && Tune::MMA;  // the row/column pass on the tensor cores
  static constexpr int XL = ROWCOL ? P2 + ((P == 5) ? 0 : 1) : 2 * P2;  // nodes from x level to x level
  static constexpr int YL = ROWCOL ? P2 + ((P == 5) ? 4 : 2) : 2 * P2;
  static constexpr int Y0 = ROWCOL ? P * XL : P2;  // node offset of the y fluxes of level 0
  static constexpr int PC_PAD = (PLANAR && !ROWCOL && Sys::ID == kSysBN) ? (P == 2 ? 1 : 0) : 0;
  static constexpr int CE_PAD =
      !PLANAR   ? 0
      : ROWCOL  ? (P == 5 ? (Sys::ID == kSysBN ? 5 : 3) : (P == 6 && Sys::ID == kSysEuler) ? 2 : 0)
                : (Sys::ID == kSysBN ? (P == 3 ? 1 : 0) : (P == 2 ? 4 : P == 3 ? 6 : 0));
  static constexpr int PLANE = (ROWCOL ? Y0 + P * YL : 2 * P * P2) + PC_PAD;  // float4 per chunk plane
  static constexpr int NS = PLANAR ? 4 : VP;            // elements from node to node
  static constexpr int CS = PLANAR ? 4 * PLANE : VEC;   // elements from chunk to chunk of a node
  static constexpr int FLUX_ELEMS = PLANAR ? 4 * NCH * PLANE : 2 * VP * P * P2;
  // shared-memory elements per cell: flux buffer (+ BN volume fraction [P][P2];
  // AD: flux [P][2][P2] + state [P][P2]), rounded to 16 bytes (+ CE_PAD);
  // the epilogue reuses it as [V][P2] x 3 (AD: x 5)
  static constexpr int RAW = (Sys::ID == kSysAD) ? 3 * P * P2 : FLUX_ELEMS + (Sys::ID == kSysBN ? P * P2 : 0);
  static constexpr int CELL_ELEMS = ((RAW + VEC - 1) / VEC) * VEC + 4 * CE_PAD;
  static_assert(CELL_ELEMS >= 3 * V * P2 && (Sys::ID != kSysAD || CELL_ELEMS >= 5 * P2), "epilogue layout");
  // FP32 up to N = 4: CTAs of at most 128 threads, twice as many per SM (each
  // Picard iteration's barriers then wait on fewer warps); N = 5 keeps 256,
  // whose 36-thread cells fill 128 badly; FP64 is pipe-bound either way
  static constexpr int MAX_THREADS0 = (sizeof(R) == 4 && N <= 4) ? 128 : 256;
  static constexpr int MAX_THREADS = Tune::CTA > 0 ? 2 * MAX_THREADS0 : Tune::CTA < 0 ? MAX_THREADS0 / 2 : MAX_THREADS0;
  static constexpr int SMEM_BUDGET = 100 * 1024;
  static constexpr int CPB_T = MAX_THREADS / P2;
  static constexpr int CPB_S = SMEM_BUDGET / (CELL_ELEMS * (int)sizeof(R));
  static constexpr int CPB = (CPB_T < CPB_S ? CPB_T : CPB_S) < 1 ? 1 : (CPB_T < CPB_S ? CPB_T : CPB_S);
  static constexpr int THREADS = ((CPB * P2 + 31) / 32) * 32;
  // FP32: CTAs per SM the register allocation aims at, measured per system
  // and degree (more resident warps hide the shared-memory latency of the
  // contractions; Baer-Nunziato's time column does not fit in fewer
  // registers without spilling at N >= 3); FP64 is pipe-bound either way
  static constexpr int BLOCK_UNITS =
      (Sys::ID == kSysAD ? 4 : Sys::ID == kSysEuler ? (N <= 3 ? 4 : 3) : (N <= 2 ? 3 : 2)) + Tune::BLOCKS;
  static constexpr int MIN_BLOCKS =
      (sizeof(R) == 4 && THREADS > 64) ? (BLOCK_UNITS * 256 / MAX_THREADS < 1 ? 1 : BLOCK_UNITS * 256 / MAX_THREADS)
                                       : 1;
  // the middle Picard iterations: a loop (default) or unrolled
  static constexpr int UNROLL = (Tune::UNROLL && P > 3) ? P - 2 : 1;
  // threads past CPB*P2 (the tail of the last warp) take part in the barriers
  // and get a scratch slot of their own so they never touch a real cell's data
  static constexpr int SLOTS = CPB + (THREADS > CPB * P2 ? 1 : 0);
  static constexpr int SMEM_BYTES = SLOTS * CELL_ELEMS * (int)sizeof(R);
};

// Loads the VP (padded) variables of one node with 16-byte vector loads;
// chunk q of the node at p + q * CS.
template <class R, int VP, int CS = 16 / (int)sizeof(R)>
__device__ __forceinline__ void vload(const R* __restrict__ p, R* out) {
  if constexpr (VP % (16 / sizeof(R)) != 0) {
#pragma unroll
    for (int q = 0; q < VP; ++q) out[q] = p[q];
  } else if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int q = 0; q < VP / 4; ++q) {
      const float4 t = *reinterpret_cast<const float4*>(p + q * CS);
      out[4 * q] = t.x; out[4 * q + 1] = t.y; out[4 * q + 2] = t.z; out[4 * q + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < VP / 2; ++q) {
      const double2 t = *reinterpret_cast<const double2*>(p + q * CS);
      out[2 * q] = t.x; out[2 * q + 1] = t.y;
    }
  }
}

// Stores V variables of one node as VP (padded) values with 16-byte vector
// stores where VP allows; chunk q of the node at p + q * CS.
template <class R, int V, int VP, int CS = 16 / (int)sizeof(R)>
__device__ __forceinline__ void vstore(R* __restrict__ p, const R* in) {
  if constexpr (VP % (16 / sizeof(R)) != 0) {
#pragma unroll
    for (int q = 0; q < (V < VP ? V : VP); ++q) p[q] = in[q];
  } else if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int q = 0; q < VP / 4; ++q) {
      float4 t;
      t.x = 4 * q + 0 < V ? in[4 * q + 0] : 0.0f;
      t.y = 4 * q + 1 < V ? in[4 * q + 1] : 0.0f;
      t.z = 4 * q + 2 < V ? in[4 * q + 2] : 0.0f;
      t.w = 4 * q + 3 < V ? in[4 * q + 3] : 0.0f;
      *reinterpret_cast<float4*>(p + q * CS) = t;
    }
  } else {
#pragma unroll
    for (int q = 0; q < VP / 2; ++q) {
      double2 t;
      t.x = 2 * q + 0 < V ? in[2 * q + 0] : 0.0;
      t.y = 2 * q + 1 < V ? in[2 * q + 1] : 0.0;
      *reinterpret_cast<double2*>(p + q * CS) = t;
    }
  }
}

// Flux-derivative contraction of time level l into b[v]; the x fluxes of
// level l start at node l*XL, the y fluxes at node Y0 + l*YL, nodes NS
// elements apart, a node's chunks CS elements apart (default: [P][2][P2]).
template <int V, int VP, int P, class R, int NS = VP, int CS = 16 / (int)sizeof(R), int XL = 2 * P * P,
          int YL = 2 * P * P, int Y0 = P * P>
__device__ __forceinline__ void contract(const R* __restrict__ cs, int l, int i, int j, const R* Dx, const R* Dy, R* b) {
  const R* fx = cs + (size_t)l * XL * NS;
  const R* fy = cs + ((size_t)Y0 + (size_t)l * YL) * NS;
#pragma unroll
  for (int v = 0; v < V; ++v) b[v] = R(0);
#pragma unroll
  for (int k = 0; k < P; ++k) {
    R f[VP];
    vload<R, VP, CS>(fx + (k + P * j) * NS, f);
#pragma unroll
    for (int v = 0; v < V; ++v) b[v] = fma(Dx[k], f[v], b[v]);
  }
#pragma unroll
  for (int k = 0; k < P; ++k) {
    R f[VP];
    vload<R, VP, CS>(fy + (i + P * k) * NS, f);
#pragma unroll
    for (int v = 0; v < V; ++v) b[v] = fma(Dy[k], f[v], b[v]);
  }
}

// Row/column pass of the Picard iterations 2..N (PredCfg::ROWCOL): the
// thread of node (i, j) contracts x row j of time level i and y column c of
// time level m in place (c = j, m = i for P = 4; c = i, m = j above),
// X(o, j) <- sum_k Kxi(k, o) X(k, j) and Y(c, o) <- sum_k Kxi(k, o) Y(c, k),
// each 16-byte chunk loaded once for all P outputs; the node's thread applies
// dt/(dx w_i), dt/(dy w_j) when it reads the results back.
template <class C, class Ops>
__device__ __forceinline__ void rowcol_pass(float* __restrict__ cs, int i, int j, const Ops& op) {
  constexpr int P = C::P;
  auto line = [&](float* p, int stride) {
    float4 f[P];
#pragma unroll
    for (int k = 0; k < P; ++k) f[k] = *reinterpret_cast<const float4*>(p + k * stride);
#pragma unroll
    for (int o = 0; o < P; ++o) {
      const float m0 = op.Kxi[P * o];
      float4 s = make_float4(m0 * f[0].x, m0 * f[0].y, m0 * f[0].z, m0 * f[0].w);
#pragma unroll
      for (int k = 1; k < P; ++k) {
        const float m = op.Kxi[k + P * o];
        s.x = fmaf(m, f[k].x, s.x);
        s.y = fmaf(m, f[k].y, s.y);
        s.z = fmaf(m, f[k].z, s.z);
        s.w = fmaf(m, f[k].w, s.w);
      }
      *reinterpret_cast<float4*>(p + o * stride) = s;
    }
  };
#pragma unroll
  for (int c = 0; c < C::NCH; ++c) {
    line(cs + c * C::CS + ((size_t)i * C::XL + P * j) * 4, 4);
    const int m = P >= 5 ? j : i, col = P >= 5 ? i : j;
    line(cs + c * C::CS + ((size_t)C::Y0 + (size_t)m * C::YL + col) * 4, 4 * P);
  }
}

// TF32 part of an FP32 value (round to nearest, ties away) as the .b32 operand of mma.sync
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// D += A B, one warp: A 16x8 TF32 (row-major fragment a0..a3), B 8x8 TF32
// (column fragment b0, b1), D 16x8 FP32
__device__ __forceinline__ void mma_tf32(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Tensor-core form of the row/column pass (PredTune kMma): every x row and y
// column of every time level of the CTA's cells (the lines rowcol_pass
// contracts), 16 lines to one mma.sync m16n8k8 tile, X(o) <- sum_k Kxi(k, o)
// X(k) with k padded from P to 8 and the P outputs to 8.  Each FP32 value is
// split into a TF32 high part and a TF32 low part, and three products are
// accumulated in FP32 (lo*hi + hi*lo + hi*hi; the dropped lo*lo term is
// below FP32 rounding), so the results carry FP32 accuracy.  Line L (v
// fastest) = (cell, chunk, direction, level, row or column, component v);
// the lines are read and written in place, and the node's thread applies
// dt/(dx w_i), dt/(dy w_j) when it reads them back, as after rowcol_pass.
template <class C, class Ops>
__device__ __forceinline__ void mma_pass(float* __restrict__ sm, int t, const Ops& op) {
  constexpr int P = C::P;
  static_assert(P <= 8, "one k8 step");
  constexpr int LPC = C::NCH * 2 * P * P * 4;  // lines per cell
  constexpr int LINES = C::CPB * LPC, TILES = (LINES + 15) / 16, NW = C::THREADS / 32;
  const int lane = t & 31, w = t >> 5, g = lane >> 2, q = lane & 3;
  // B(k, o) = Kxi(k, o) = op.Kxi[k + P o]: b0 (k = q, o = g), b1 (k = q + 4, o = g)
  const float b0 = (g < P) ? op.Kxi[q + P * g] : 0.0f;
  const float b1 = (g < P && q + 4 < P) ? op.Kxi[q + 4 + P * g] : 0.0f;
  const uint32_t bh0 = to_tf32(b0), bh1 = to_tf32(b1);
  const uint32_t bl0 = to_tf32(b0 - __uint_as_float(bh0)), bl1 = to_tf32(b1 - __uint_as_float(bh1));
  auto line = [&](int L, int& base, int& stride) {
    const int v = L & 3, r1 = L >> 2;
    const int r = r1 % P, r2 = r1 / P;
    const int l = r2 % P, r3 = r2 / P;
    const int d = r3 & 1, r4 = r3 >> 1;
    const int ch = r4 % C::NCH, c = r4 / C::NCH;
    const int cb = c * C::CELL_ELEMS + ch * C::CS + v;
    if (d == 0) { base = cb + (l * C::XL + P * r) * 4; stride = 4; }
    else { base = cb + (C::Y0 + l * C::YL + r) * 4; stride = 4 * P; }
  };
  for (int tile = w; tile < TILES; tile += NW) {
    const int L0 = tile * 16 + g, L1 = L0 + 8;
    const bool ok0 = L0 < LINES, ok1 = L1 < LINES;
    int s0 = 0, d0 = 0, s1 = 0, d1 = 0;
    if (ok0) line(L0, s0, d0);
    if (ok1) line(L1, s1, d1);
    // A fragment: a0 (row g, k = q), a1 (row g + 8, k = q), a2 (row g, k = q + 4), a3 (row g + 8, k = q + 4)
    float af[4];
    af[0] = ok0 ? sm[s0 + q * d0] : 0.0f;
    af[1] = ok1 ? sm[s1 + q * d1] : 0.0f;
    af[2] = (ok0 && q + 4 < P) ? sm[s0 + (q + 4) * d0] : 0.0f;
    af[3] = (ok1 && q + 4 < P) ? sm[s1 + (q + 4) * d1] : 0.0f;
    uint32_t ah[4], al[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      ah[e] = to_tf32(af[e]);
      al[e] = to_tf32(af[e] - __uint_as_float(ah[e]));
    }
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    mma_tf32(acc, al, bh0, bh1);
    mma_tf32(acc, ah, bl0, bl1);
    mma_tf32(acc, ah, bh0, bh1);
    __syncwarp();  // every lane's loads of these lines precede the stores
    // D fragment: d0, d1 (row g, o = 2q, 2q + 1), d2, d3 (row g + 8, o = 2q, 2q + 1)
    const int o = 2 * q;
    if (ok0 && o < P) sm[s0 + o * d0] = acc[0];
    if (ok0 && o + 1 < P) sm[s0 + (o + 1) * d0] = acc[1];
    if (ok1 && o < P) sm[s1 + o * d1] = acc[2];
    if (ok1 && o + 1 < P) sm[s1 + (o + 1) * d1] = acc[3];
  }
}

// Volume integral (duh; kVolume) and face extrapolation (qbnd, fbnd /
// gradQbnd) of one cell from the time averages in shared memory cs: Q [V][P2], FX [V][P2],
// FY [V][P2] (AD: + GX, GY); Sh is the node's time-averaged -NCP (BN).  Called
// by the P2 threads of the cell (node = 0..P2-1).
template <class Sys, int N, class R, bool kVolume>
__device__ __forceinline__ void predictor_outputs(const BatchArgs& a, const DevOps<N, R>& op, const InstDesc& in,
                                                  const R* cs, long long cell, int node, int i, int j, const R* Sh) {
  constexpr int P = N + 1, P2 = P * P, V = Sys::V;
  const R* sQ = cs;
  const R* sX = cs + V * P2;
  const R* sY = cs + 2 * V * P2;
  if constexpr (kVolume) {
    // volume integral: duh = (w_j/dx) sum_k Kxi(i,k) Fhi_x(k,j) + (w_i/dy) sum_k Kxi(j,k) Fhi_y(i,k) [+ w_i w_j Shi]
    // duh is stored in the compute precision R (FP32 in the FP32 modes)
    R vx, vy;
    if constexpr (sizeof(R) == 4) {
      vx = op.w[j] * R(in.idxf);
      vy = op.w[i] * R(in.idyf);
    } else {
      vx = op.w[j] / R(in.dx);
      vy = op.w[i] / R(in.dy);
    }
    R* dst = reinterpret_cast<R*>(a.duh) + ((size_t)cell * P2 + node) * V;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      R sxv = R(0), syv = R(0);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        sxv = fma(op.Kxi[i + P * k], sX[v * P2 + k + P * j], sxv);
        syv = fma(op.Kxi[j + P * k], sY[v * P2 + i + P * k], syv);
      }
      R d = sxv * vx + syv * vy;
      if constexpr (Sys::ID == kSysBN) d = fma(op.w[i] * op.w[j], Sh[v], d);
      dst[v] = d;
    }
  }
  // face extrapolation: faces 0 left, 1 right (x), 2 bottom, 3 top (y); point l
  R* qb = reinterpret_cast<R*>(a.qbnd);
  R* fb = reinterpret_cast<R*>(a.fbnd);
  for (int idx = node; idx < 4 * P; idx += P2) {
    const int f = idx / P, l = idx - f * P;
    const R* c = (f == 0 || f == 2) ? op.FL : op.FR;
    const size_t o = ((size_t)cell * 4 + f) * P + l;  // [cell][face][point]
    const bool xdir = f < 2;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      R sq = R(0), sf = R(0);
#pragma unroll
      for (int m = 0; m < P; ++m) {
        const int nd = xdir ? (m + P * l) : (l + P * m);
        sq = fma(c[m], sQ[v * P2 + nd], sq);
        if constexpr (Sys::ID != kSysAD) sf = fma(c[m], (xdir ? sX : sY)[v * P2 + nd], sf);
      }
      qb[o * V + v] = sq;
      if constexpr (Sys::ID != kSysAD) fb[o * V + v] = sf;
    }
    if constexpr (Sys::ID == kSysAD) {
      // gradQbnd(v,d,f,l)
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        R sg = R(0);
#pragma unroll
        for (int m = 0; m < P; ++m) {
          const int nd = xdir ? (m + P * l) : (l + P * m);
          sg = fma(c[m], cs[(3 + d) * P2 + nd], sg);
        }
        fb[o * 2 + d] = sg;
      }
    }
  }
}

template <class Sys, int N, class R, bool kPhase, class Tune = PredTune<>>
__global__ void __launch_bounds__(PredCfg<Sys, N, R, Tune>::THREADS, PredCfg<Sys, N, R, Tune>::MIN_BLOCKS)
    k_predictor(BatchArgs a, DevOps<N, R> op) {
  using C = PredCfg<Sys, N, R, Tune>;
  constexpr int P = N + 1, P2 = P * P, V = Sys::V, CPB = C::CPB, VP = C::VP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sm = reinterpret_cast<R*>(smem_raw);

  const int t = threadIdx.x;
  const int lc = t / P2;
  const int node = t - lc * P2;
  const int i = node % P, j = node / P;
  const long long cell = a.cell0 + (long long)blockIdx.x * CPB + lc;
  const bool in_cta = lc < CPB;
  const int k_found = (in_cta && cell < a.ncells) ? find_inst_cell(a.inst, a.ninst, cell) : -1;
  const bool valid = k_found >= 0;
  R* cs = sm + (size_t)(lc < CPB ? lc : CPB) * C::CELL_ELEMS;  // lc >= CPB: the scratch slot

  const int k_inst = valid ? k_found : 0;
  const InstDesc& in = a.inst[k_inst];
  const bool act = valid && a.st[k_inst].active;
  if (!__syncthreads_or(act)) return;  // nothing to do in this CTA (finished or absent instances)
  const double dt = act ? a.st[k_inst].dt : 0.0;
  const double* uh_in = a.uh[valid ? parity(a.st[k_inst]) : 0];
  const Phys ph = in.ph;
  const typename Sys::template PConst<R> pc(ph);

  // per-thread contraction rows: Dx(i,k) = Kxi(k,i) dt/(dx w_i), Dy(j,k) likewise
  R Dx[P], Dy[P], Gx[P], Gy[P];
  R cxw, cyw;  // dt/(dx w_i), dt/(dy w_j)
  {
    // FP32: the reciprocals 1/dx, 1/dy held in FP32 (no FP64 divisions per thread)
    R idx, idy;
    if constexpr (sizeof(R) == 4) {
      idx = in.idxf;
      idy = in.idyf;
      const R dtf = R(dt);
      cxw = dtf * idx / op.w[i];
      cyw = dtf * idy / op.w[j];
    } else {
      idx = R(1) / R(in.dx);
      idy = R(1) / R(in.dy);
      cxw = R(dt / in.dx) / op.w[i];
      cyw = R(dt / in.dy) / op.w[j];
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
      Dx[k] = op.Kxi[k + P * i] * cxw;
      Dy[k] = op.Kxi[k + P * j] * cyw;
      // gradient rows dudx(i,k)/dx (BN volume fraction, AD state)
      if constexpr (sizeof(R) == 4) {
        Gx[k] = op.dudx[i + P * k] * idx;
        Gy[k] = op.dudx[j + P * k] * idy;
      } else {
        Gx[k] = op.dudx[i + P * k] / R(in.dx);
        Gy[k] = op.dudx[j + P * k] / R(in.dy);
      }
    }
  }

  R u[V];
  {
    const double* src = uh_in + ((size_t)(valid ? cell : 0) * P2 + node) * V;
#pragma unroll
    for (int v = 0; v < V; ++v) u[v] = act ? R(src[v]) : R(1);
  }
  const R rdt = R(dt);

  R q[P][V];
  R Fh[2][V];   // time-averaged fluxes of the last iteration
  R Sh[V];      // BN: time-averaged -NCP of the last iteration
  R Gh[2];      // AD: time-averaged gradient of the last iteration
  R qh[V];      // time-averaged state

  auto fidx = [&](int l, int d, int v) {
    return ((d == 0 ? (size_t)l * C::XL : (size_t)C::Y0 + (size_t)l * C::YL) + node) * C::NS + v;
  };

  if constexpr (Sys::ID == kSysAD) {
    // -------------------------------------------------------------- AD
    // state buffer [P][P2] after the flux buffer [P][2][P2]
    R* qs = cs + 2 * P * P2;
    const R ca = R(ph.a), ccx = R(ph.cx), ccy = R(ph.cy);
    const bool fused = ph.ad_fused != 0;
    // iteration 1: constant in time
    qs[node] = u[0];
    __syncthreads();
    {
      R gx = R(0), gy = R(0);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        gx = fma(Gx[k], qs[k + P * j], gx);
        gy = fma(Gy[k], qs[i + P * k], gy);
      }
      R fx = -ca * gx, fy = -ca * gy;
      if (fused) {
        fx = fma(ccx, u[0], fx);
        fy = fma(ccy, u[0], fy);
      }
      cs[node] = fx;
      cs[P2 + node] = fy;
    }
    __syncthreads();
    {
      R b[1];
      contract<1, VP, P>(cs, 0, i, j, Dx, Dy, b);
#pragma unroll
      for (int l = 0; l < P; ++l) q[l][0] = op.g[l] * u[0] - op.ts[l] * b[0];
    }
    __syncthreads();
    // the Picard iterations 2..P; the last one is instantiated apart, so that
    // its time averages (Fh, qh, ...) hold no registers in the others
    auto picard = [&](auto last_tag) {
      constexpr bool last = decltype(last_tag)::value;

#pragma unroll
      for (int l = 0; l < P; ++l) qs[l * P2 + node] = q[l][0];
      __syncthreads();
      // last iteration: the time levels' fluxes combined (H = sum_l tw_l F_l) and contracted once
      R hx = R(0), hy = R(0);
      if constexpr (last) { Fh[0][0] = Fh[1][0] = R(0); Gh[0] = Gh[1] = R(0); }
#pragma unroll
      for (int l = 0; l < P; ++l) {
        R gx = R(0), gy = R(0);
#pragma unroll
        for (int k = 0; k < P; ++k) {
          gx = fma(Gx[k], qs[l * P2 + k + P * j], gx);
          gy = fma(Gy[k], qs[l * P2 + i + P * k], gy);
        }
        R fx = -ca * gx, fy = -ca * gy;
        if (fused) {
          fx = fma(ccx, q[l][0], fx);
          fy = fma(ccy, q[l][0], fy);
        }
        if constexpr (!last) {
          cs[fidx(l, 0, 0)] = fx;
          cs[fidx(l, 1, 0)] = fy;
        } else {
          Fh[0][0] = fma(op.w[l], fx, Fh[0][0]);
          Fh[1][0] = fma(op.w[l], fy, Fh[1][0]);
          Gh[0] = fma(op.w[l], gx, Gh[0]);
          Gh[1] = fma(op.w[l], gy, Gh[1]);
          hx = fma(op.tw[l], fx, hx);
          hy = fma(op.tw[l], fy, hy);
        }
      }
      if constexpr (last) {
        cs[fidx(0, 0, 0)] = hx;
        cs[fidx(0, 1, 0)] = hy;
      }
      __syncthreads();
      if constexpr (!last) {
#pragma unroll
        for (int l = 0; l < P; ++l) q[l][0] = op.g[l] * u[0];
#pragma unroll
        for (int l = 0; l < P; ++l) {
          R b[1];
          contract<1, VP, P>(cs, l, i, j, Dx, Dy, b);
#pragma unroll
          for (int lp = 0; lp < P; ++lp) q[lp][0] = fma(-op.T[lp + P * l], b[0], q[lp][0]);
        }
      } else {
        R b[1];
        contract<1, VP, P>(cs, 0, i, j, Dx, Dy, b);
        qh[0] = op.wg * u[0] - b[0];
      }
      __syncthreads();
    };
#pragma unroll C::UNROLL
    for (int it = 2; it < P; ++it) picard(std::false_type{});
    picard(std::true_type{});
  } else {
    // ------------------------------------------------- Euler / Baer-Nunziato
    constexpr bool BN = Sys::ID == kSysBN;
    R* as = cs + C::FLUX_ELEMS;            // BN volume fraction [P][P2]
    R pg[P], us[P], vs[P];                // BN: NCP scalars per time level
    // contraction of level l at this node: b = sum_k Dx Fx + sum_k Dy Fy (+ BN: ax, ay)
    auto node_contract = [&](int l, R* b, R& ax, R& ay) {
      contract<C::VF, VP, P, R, C::NS, C::CS, C::XL, C::YL, C::Y0>(cs, l, i, j, Dx, Dy, b);
      if constexpr (BN) {
        ax = R(0);
        ay = R(0);
#pragma unroll
        for (int k = 0; k < P; ++k) {
          ax = fma(Gx[k], as[l * P2 + k + P * j], ax);
          ay = fma(Gy[k], as[l * P2 + i + P * k], ay);
        }
      }
#pragma unroll
      for (int v = C::VF; v < V; ++v) b[v] = R(0);
    };
    // the same b from the row/column pass's results (PredCfg::ROWCOL)
    auto node_gather = [&](int l, R* b, R& ax, R& ay) {
      R bx[VP], by[VP];
      vload<R, VP, C::CS>(cs + fidx(l, 0, 0), bx);
      vload<R, VP, C::CS>(cs + fidx(l, 1, 0), by);
#pragma unroll
      for (int v = 0; v < C::VF; ++v) b[v] = fma(cxw, bx[v], cyw * by[v]);
      if constexpr (BN) {
        ax = R(0);
        ay = R(0);
#pragma unroll
        for (int k = 0; k < P; ++k) {
          ax = fma(Gx[k], as[l * P2 + k + P * j], ax);
          ay = fma(Gy[k], as[l * P2 + i + P * k], ay);
        }
      }
#pragma unroll
      for (int v = C::VF; v < V; ++v) b[v] = R(0);
    };
    // iteration 1: the state is constant in time
    {
      R Fx[V], Fy[V];
      if constexpr (BN) {
        Sys::template pflux<R>(pc, u, Fx, Fy, pg[0], us[0], vs[0]);
        as[node] = u[8];
      } else {
        Sys::template pflux<R>(pc, u, Fx, Fy);
      }
      vstore<R, V, VP, C::CS>(cs + fidx(0, 0, 0), Fx);
      vstore<R, V, VP, C::CS>(cs + fidx(0, 1, 0), Fy);
      __syncthreads();
      R b[V], ax, ay;
      node_contract(0, b, ax, ay);
      if constexpr (BN) {
        R n[9];
        BNSys::pncp<R>(pg[0], us[0], vs[0], ax, ay, n);
#pragma unroll
        for (int v = 0; v < V; ++v) b[v] = fma(rdt, n[v], b[v]);
      }
#pragma unroll
      for (int l = 0; l < P; ++l)
#pragma unroll
        for (int v = 0; v < V; ++v) q[l][v] = op.g[l] * u[v] - op.ts[l] * b[v];
      __syncthreads();
    }
    // the Picard iterations 2..P; the last one is instantiated apart, so that
    // its time averages (Fh, qh, ...) hold no registers in the others
    auto picard = [&](auto last_tag) {
      constexpr bool last = decltype(last_tag)::value;

      // last iteration: the contraction is linear, so the time levels' fluxes
      // are combined first (H = sum_l tw_l F_l) and contracted once
      R Hx[V], Hy[V];
      if constexpr (last) {
#pragma unroll
        for (int v = 0; v < V; ++v) { Fh[0][v] = R(0); Fh[1][v] = R(0); Hx[v] = R(0); Hy[v] = R(0); }
      }
#pragma unroll
      for (int l = 0; l < P; ++l) {
        R Fx[V], Fy[V];
        if constexpr (BN) {
          Sys::template pflux<R>(pc, q[l], Fx, Fy, pg[l], us[l], vs[l]);
          as[l * P2 + node] = q[l][8];
        } else {
          Sys::template pflux<R>(pc, q[l], Fx, Fy);
        }
        if constexpr (!last) {
          vstore<R, V, VP, C::CS>(cs + fidx(l, 0, 0), Fx);
          vstore<R, V, VP, C::CS>(cs + fidx(l, 1, 0), Fy);
        } else {
#pragma unroll
          for (int v = 0; v < V; ++v) {
            Fh[0][v] = fma(op.w[l], Fx[v], Fh[0][v]);
            Fh[1][v] = fma(op.w[l], Fy[v], Fh[1][v]);
            Hx[v] = fma(op.tw[l], Fx[v], Hx[v]);
            Hy[v] = fma(op.tw[l], Fy[v], Hy[v]);
          }
        }
      }
      if constexpr (last) {
        vstore<R, V, VP, C::CS>(cs + fidx(0, 0, 0), Hx);
        vstore<R, V, VP, C::CS>(cs + fidx(0, 1, 0), Hy);
      }
      __syncthreads();
      if constexpr (!last) {
        if constexpr (C::MMA) {
          mma_pass<C>(sm, t, op);
          __syncthreads();
        } else if constexpr (C::ROWCOL) {
          rowcol_pass<C>(cs, i, j, op);
          __syncthreads();
        }
#pragma unroll
        for (int l = 0; l < P; ++l)
#pragma unroll
          for (int v = 0; v < V; ++v) q[l][v] = op.g[l] * u[v];
      } else {
#pragma unroll
        for (int v = 0; v < V; ++v) { qh[v] = op.wg * u[v]; Sh[v] = R(0); }
      }
      if constexpr (!last) {
#pragma unroll
        for (int l = 0; l < P; ++l) {
          R b[V], ax, ay;
          if constexpr (C::ROWCOL)
            node_gather(l, b, ax, ay);
          else
            node_contract(l, b, ax, ay);
          if constexpr (BN) {
            R n[9];
            BNSys::pncp<R>(pg[l], us[l], vs[l], ax, ay, n);
#pragma unroll
            for (int v = 0; v < V; ++v) b[v] = fma(rdt, n[v], b[v]);
          }
#pragma unroll
          for (int lp = 0; lp < P; ++lp)
#pragma unroll
            for (int v = 0; v < V; ++v) q[lp][v] = fma(-op.T[lp + P * l], b[v], q[lp][v]);
        }
      } else {
        // qh = wg u - sum_l tw_l (D F_l + dt NCP_l) = wg u - D H - dt sum_l tw_l NCP_l
        R b[V];
        contract<C::VF, VP, P, R, C::NS, C::CS, C::XL, C::YL, C::Y0>(cs, 0, i, j, Dx, Dy, b);
#pragma unroll
        for (int v = 0; v < C::VF; ++v) qh[v] = qh[v] - b[v];
        if constexpr (BN) {
#pragma unroll
          for (int l = 0; l < P; ++l) {
            R ax = R(0), ay = R(0);
#pragma unroll
            for (int k = 0; k < P; ++k) {
              ax = fma(Gx[k], as[l * P2 + k + P * j], ax);
              ay = fma(Gy[k], as[l * P2 + i + P * k], ay);
            }
            R n[9];
            BNSys::pncp<R>(pg[l], us[l], vs[l], ax, ay, n);
            const R c = op.tw[l] * rdt;
#pragma unroll
            for (int v = 0; v < V; ++v) {
              Sh[v] = fma(-op.w[l], n[v], Sh[v]);
              qh[v] = fma(-c, n[v], qh[v]);
            }
          }
        }
      }
      __syncthreads();
    };
#pragma unroll C::UNROLL
    for (int it = 2; it < P; ++it) picard(std::false_type{});
    picard(std::true_type{});
  }

  // ------------------------------------------------------------- epilogue
  // shared layout per cell: Q [V][P2], FX [V][P2], FY [V][P2] (AD: + GX, GY)
  R* sQ = cs;
  R* sX = cs + V * P2;
  R* sY = cs + 2 * V * P2;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    sQ[v * P2 + node] = qh[v];
    sX[v * P2 + node] = Fh[0][v];
    sY[v * P2 + node] = Fh[1][v];
  }
  if constexpr (Sys::ID == kSysAD) {
    cs[3 * P2 + node] = Gh[0];
    cs[4 * P2 + node] = Gh[1];
  }
  __syncthreads();
  if (!act) return;

  if constexpr (kPhase) {
    // qhi(v,i,j), Fhi(v,d,i,j), Shi(v,i,j) in the reference layout
    const size_t base = (size_t)cell * P2 + node;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      a.qhi[base * V + v] = (double)qh[v];
      a.fhi[(base * 2 + 0) * V + v] = (double)Fh[0][v];
      a.fhi[(base * 2 + 1) * V + v] = (double)Fh[1][v];
      if constexpr (Sys::ID == kSysBN) a.shi[base * V + v] = (double)Sh[v];
    }
    predictor_outputs<Sys, N, R, false>(a, op, in, cs, cell, node, i, j, Sh);
  } else {
    predictor_outputs<Sys, N, R, true>(a, op, in, cs, cell, node, i, j, Sh);
  }
}

}  // namespace aderdg
