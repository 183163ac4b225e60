// setup.cpp -- host construction of the 1D ADER-DG operators and the initial
// fields.
//
// The operators must come out bit-identical to the reference's, so the
// published algorithms are kept with the reference's operation order
// (each step is noted with the reference file:line it has to agree with):
// Newton iteration on the Legendre recurrence for Gauss-Legendre and
// Gauss-Lobatto nodes, Lagrange products for the basis, Gauss-Jordan with
// column pivoting for the inverses, and the constrained least-squares
// reconstruction for the subcell-to-DG map.
#include "setup.h"
#include "ic_eval.h"

#include <cmath>

#include "../../include/aderdg_gpu.h"

namespace aderdg {
namespace {

const double kPi = 4.0 * std::atan(1.0);

// Column-major dense matrix.
struct Mat {
  int r = 0, c = 0;
  std::vector<double> a;
  Mat() = default;
  Mat(int rows, int cols) : r(rows), c(cols), a((size_t)rows * cols, 0.0) {}
  double& operator()(int i, int j) { return a[(size_t)i + (size_t)r * j]; }
  double operator()(int i, int j) const { return a[(size_t)i + (size_t)r * j]; }
};

// Gauss-Legendre nodes/weights on [x1,x2] (quadrature.f90:8-44).
void gauss_legendre(double x1, double x2, int n, double* x, double* w) {
  const double mid = 0.5 * (x2 + x1), half = 0.5 * (x2 - x1);
  for (int i = 1; i <= (n + 1) / 2; ++i) {
    double z = std::cos(kPi * (i - 0.25) / (n + 0.5));
    double z_prev, dp, pn;
    for (;;) {
      double pa = 1.0, pb = 0.0;  // P_k, P_{k-1}
      for (int k = 1; k <= n; ++k) {
        double pc = pb;
        pb = pa;
        pa = ((2.0 * k - 1.0) * z * pb - (k - 1.0) * pc) / (double)k;
      }
      pn = pa;
      dp = (double)n * (z * pa - pb) / (z * z - 1.0);
      z_prev = z;
      z = z_prev - pn / dp;
      if (!(std::fabs(z - z_prev) > 1.0e-15)) break;
    }
    x[i - 1] = mid - half * z;
    x[n - i] = mid + half * z;
    w[i - 1] = 2.0 * half / ((1.0 - z * z) * dp * dp);
    w[n - i] = w[i - 1];
  }
}

// Gauss-Lobatto nodes/weights on [x1,x2] (quadrature.f90:47-101).
void gauss_lobatto(double x1, double x2, int np, double* x, double* w) {
  const int n = np - 1;
  std::vector<double> prev(np);
  Mat L(np, np + 1);  // L(i,k) = P_{k-1}(x_i), k = 1..np
  for (int i = 0; i <= n; ++i) x[i] = std::cos(kPi * (double)i / (double)n);
  for (int iter = 0; iter < 100000; ++iter) {
    for (int i = 0; i < np; ++i) prev[i] = x[i];
    for (int i = 0; i < np; ++i) {
      L(i, 1) = 1.0;
      L(i, 2) = x[i];
    }
    for (int k = 2; k <= n; ++k)
      for (int i = 0; i < np; ++i) L(i, k + 1) = ((2 * k - 1) * x[i] * L(i, k) - (k - 1) * L(i, k - 1)) / (double)k;
    double change = 0.0;
    for (int i = 0; i < np; ++i) {
      x[i] = prev[i] - (x[i] * L(i, np) - L(i, n)) / (np * L(i, np));
      change = std::fmax(change, std::fabs(x[i] - prev[i]));
    }
    if (change <= 1.0e-15) break;
  }
  for (int i = 0; i < np; ++i) {
    w[i] = 2.0 / ((double)(n * np) * (L(i, np) * L(i, np)));
    w[i] = 0.5 * w[i] * (x2 - x1);
    x[i] = x1 + 0.5 * (x[i] + 1.0) * (x2 - x1);
  }
}

// Lagrange basis through nodes and its derivative at s (basis.f90:9-41).
void lagrange(const std::vector<double>& nodes, double s, double* phi, double* dphi) {
  const int P = (int)nodes.size();
  for (int m = 0; m < P; ++m) {
    double v = 1.0;
    for (int j = 0; j < P; ++j)
      if (j != m) v = v * (s - nodes[j]) / (nodes[m] - nodes[j]);
    phi[m] = v;
    double d = 0.0;
    for (int i = 0; i < P; ++i) {
      if (i == m) continue;
      double t = 1.0;
      for (int j = 0; j < P; ++j)
        if (j != i && j != m) t = t * (s - nodes[j]) / (nodes[m] - nodes[j]);
      d = d + t / (nodes[m] - nodes[i]);
    }
    dphi[m] = d;
  }
}

// Inverse by Gauss-Jordan elimination with column pivoting on the transposed
// augmented matrix (la.f90:8-65).  Returns false when a pivot is <= 1e-15.
bool invert(const Mat& A, Mat& inv) {
  const int n = A.r;
  Mat C(2 * n, n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) C(i, j) = A(j, i);
  for (int i = 0; i < n; ++i) C(n + i, i) = 1.0;
  std::vector<double> col(2 * n);
  for (int i = 0; i < n; ++i) {
    int piv_col = i;
    for (int j = i + 1; j < n; ++j)
      if (std::fabs(C(i, j)) > std::fabs(C(i, piv_col))) piv_col = j;
    for (int k = 0; k < 2 * n; ++k) col[k] = C(k, piv_col);
    for (int k = 0; k < 2 * n; ++k) C(k, piv_col) = C(k, i);
    for (int k = 0; k < 2 * n; ++k) C(k, i) = col[k];
    if (std::fabs(C(i, i)) <= 1.0e-15) return false;
    const double r = 1.0 / C(i, i);
    for (int k = 0; k < 2 * n; ++k) C(k, i) = C(k, i) * r;
    for (int j = i + 1; j < n; ++j) {
      const double f = C(i, j);
      for (int k = 0; k < 2 * n; ++k) C(k, j) = C(k, j) - f * C(k, i);
    }
  }
  for (int i = n - 1; i >= 0; --i)
    for (int j = i - 1; j >= 0; --j) {
      const double f = C(i, j);
      for (int k = 0; k < 2 * n; ++k) C(k, j) = C(k, j) - f * C(k, i);
    }
  inv = Mat(n, n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv(i, j) = C(n + j, i);
  return true;
}

}  // namespace

double pi_value() { return kPi; }

double pnpm_cfl(int N) {
  static const double t[10] = {1.0, 0.33, 0.17, 0.1, 0.069, 0.045, 0.038, 0.03, 0.02, 0.015};
  return (N >= 0 && N <= 9) ? t[N] : 0.0;
}

bool build_ops(int N, HostOps& o, std::string* err) {
  if (N < 1 || N > 9) {
    if (err) *err = "N out of range";
    return false;
  }
  const int P = N + 1, S = 2 * N + 1;
  o.N = N;
  o.P = P;
  o.S = S;
  o.xi.assign(P, 0.0);
  o.w.assign(P, 0.0);
  gauss_legendre(0.0, 1.0, P, o.xi.data(), o.w.data());

  // mass and stiffness matrices by quadrature (Euler/initialize.f90:94-102)
  std::vector<double> phi(P), dphi(P);
  Mat M(P, P), K(P, P);
  for (int g = 0; g < P; ++g) {
    lagrange(o.xi, o.xi[g], phi.data(), dphi.data());
    for (int k = 0; k < P; ++k)
      for (int l = 0; l < P; ++l) {
        M(k, l) = M(k, l) + o.w[g] * phi[k] * phi[l];
        K(k, l) = K(k, l) + o.w[g] * dphi[k] * phi[l];
      }
  }
  Mat iM;
  if (!invert(M, iM)) {
    if (err) *err = "singular mass matrix";
    return false;
  }
  o.Kxi = K.a;
  o.dudx.assign(P * P, 0.0);  // iMM * Kxi^T
  for (int a = 0; a < P; ++a)
    for (int b = 0; b < P; ++b) {
      double s = 0.0;
      for (int c = 0; c < P; ++c) s = s + iM(a, c) * K(b, c);
      o.dudx[a + P * b] = s;
    }
  std::vector<double> phi0(P), phi1(P);
  lagrange(o.xi, 0.0, phi0.data(), dphi.data());
  lagrange(o.xi, 1.0, phi1.data(), dphi.data());
  o.F0 = phi0;
  o.FL = phi0;
  o.FR = phi1;
  Mat K1(P, P);  // F1 - Kxi with F1 = phi(1) phi(1)^T (Euler/initialize.f90:108-128)
  for (int k = 0; k < P; ++k)
    for (int l = 0; l < P; ++l) K1(k, l) = phi1[k] * phi1[l] - K(k, l);
  Mat iK1;
  if (!invert(K1, iK1)) {
    if (err) *err = "singular time matrix";
    return false;
  }
  o.K1 = K1.a;
  o.iK1 = iK1.a;

  // subcell limiter maps (Euler/initialize.f90:171-213)
  Mat U(S, P);
  const double h = 1.0 / (double)S;
  for (int s = 1; s <= S; ++s) {
    const double left = (double)(s - 1) * h;
    for (int q = 0; q < P; ++q) {
      lagrange(o.xi, left + h * o.xi[q], phi.data(), dphi.data());
      for (int c = 0; c < P; ++c) U(s - 1, c) = U(s - 1, c) + o.w[q] * phi[c];
    }
  }
  Mat A(P + 1, P + 1), R(P + 1, S);
  for (int a = 0; a < P; ++a)
    for (int b = 0; b < P; ++b) {
      double acc = 0.0;
      for (int k = 0; k < S; ++k) acc = acc + U(k, a) * U(k, b);
      A(a, b) = 2 * acc;
    }
  for (int b = 0; b < P; ++b) A(P, b) = o.w[b];
  for (int a = 0; a < P; ++a) A(a, P) = -o.w[a];
  Mat iA;
  if (!invert(A, iA)) {
    if (err) *err = "singular least-squares matrix";
    return false;
  }
  for (int a = 0; a < P; ++a)
    for (int s = 0; s < S; ++s) R(a, s) = 2.0 * U(s, a);
  for (int s = 0; s < S; ++s) R(P, s) = h;
  o.lim2uh.assign(P * S, 0.0);
  for (int a = 0; a < P; ++a)
    for (int s = 0; s < S; ++s) {
      double acc = 0.0;
      for (int c = 0; c <= P; ++c) acc = acc + iA(a, c) * R(c, s);
      o.lim2uh[a + P * s] = acc;
    }
  o.uh2lim = U.a;
  std::vector<double> xl(P), wl(P);
  gauss_lobatto(0.0, 1.0, P, xl.data(), wl.data());
  o.uh2lob.assign(P * P, 0.0);
  for (int q = 0; q < P; ++q) {
    lagrange(o.xi, xl[q], phi.data(), dphi.data());
    for (int c = 0; c < P; ++c) o.uh2lob[q + P * c] = phi[c];
  }
  o.xilimbary.assign(S, 0.0);
  for (int s = 1; s <= S; ++s) o.xilimbary[s - 1] = 0.0 + 0.5 / (double)S + (double)(s - 1) * 1.0 / (double)S;
  return true;
}

}  // namespace aderdg

// ---------------------------------------------------------------------------
// Initial fields (ic_eval.h) at the Gauss-Legendre nodes of every cell and at
// the subcell barycentres (Euler/initialize.f90:262-307).
extern "C" int aderdg_project_initial_condition(const aderdg_config* cfg, int ic, const double* params, double* uh,
                                                double* lh_ic) {
  if (!cfg || !uh || cfg->imax < 1 || cfg->jmax < 1) return ADERDG_EINVAL;
  aderdg::HostOps ops;
  if (!aderdg::build_ops(cfg->N, ops, nullptr)) return ADERDG_EINVAL;
  double zero[32] = {0};
  const double* p = params ? params : zero;
  const int V = cfg->system == ADERDG_SYS_ADVDIFF ? 1 : cfg->system == ADERDG_SYS_EULER ? 4 : 9;
  const int P = ops.P, S = ops.S, I = cfg->imax, J = cfg->jmax;
  const double dx = (cfg->xr[0] - cfg->xl[0]) / I, dy = (cfg->xr[1] - cfg->xl[1]) / J;
  double u[9];
  for (int j = 0; j < J; ++j)
    for (int i = 0; i < I; ++i) {
      // cell corner = centre - dx/2 (Euler/initialize.f90:264-266)
      const double x0 = (cfg->xl[0] + ((double)i + 0.5) * dx) - 0.5 * dx;
      const double y0 = (cfg->xl[1] + ((double)j + 0.5) * dy) - 0.5 * dy;
      const long cell = (long)i + (long)I * j;
      for (int l = 0; l < P; ++l)
        for (int k = 0; k < P; ++k) {
          if (aderdg::eval_ic(*cfg, ic, p, aderdg::kPi, x0 + ops.xi[k] * dx, y0 + ops.xi[l] * dy, u))
            return ADERDG_EINVAL;
          for (int v = 0; v < V; ++v) uh[v + V * (k + P * (l + P * cell))] = u[v];
        }
      if (lh_ic)
        for (int b = 0; b < S; ++b)
          for (int a = 0; a < S; ++a) {
            if (aderdg::eval_ic(*cfg, ic, p, aderdg::kPi, x0 + ops.xilimbary[a] * dx, y0 + ops.xilimbary[b] * dy, u))
              return ADERDG_EINVAL;
            for (int v = 0; v < V; ++v) lh_ic[v + V * (a + S * (b + S * cell))] = u[v];
          }
    }
  return ADERDG_OK;
}

extern "C" int aderdg_operator(int N, int which, double* out) {
  aderdg::HostOps o;
  if (!out || !aderdg::build_ops(N, o, nullptr)) return ADERDG_EINVAL;
  const std::vector<double>* v = nullptr;
  switch (which) {
    case ADERDG_OP_XI: v = &o.xi; break;
    case ADERDG_OP_W: v = &o.w; break;
    case ADERDG_OP_KXI: v = &o.Kxi; break;
    case ADERDG_OP_DUDX: v = &o.dudx; break;
    case ADERDG_OP_IK1: v = &o.iK1; break;
    case ADERDG_OP_F0: v = &o.F0; break;
    case ADERDG_OP_FL: v = &o.FL; break;
    case ADERDG_OP_FR: v = &o.FR; break;
    case ADERDG_OP_UH2LIM: v = &o.uh2lim; break;
    case ADERDG_OP_LIM2UH: v = &o.lim2uh; break;
    case ADERDG_OP_UH2LOB: v = &o.uh2lob; break;
    case ADERDG_OP_XILIMBARY: v = &o.xilimbary; break;
    default: return ADERDG_EINVAL;
  }
  for (size_t k = 0; k < v->size(); ++k) out[k] = (*v)[k];
  return (int)v->size();
}
