// setup.h -- host-side set-up of the ADER-DG step: 1D operators and initial
// fields.  Runs once per context on the host in FP64; nothing here is on the
// hot path.
#pragma once

#include <string>
#include <vector>

namespace aderdg {

// One-dimensional operators of the nodal Gauss-Legendre basis of degree N,
// as built by Euler/initialize.f90:88-131 (predictor) and :171-213 (subcell
// limiter).  Matrices are column-major, first index fastest, as in Fortran.
struct HostOps {
  int N = 0, P = 0, S = 0;
  std::vector<double> xi, w;         // Gauss-Legendre nodes and weights on [0,1]
  std::vector<double> Kxi, dudx;     // stiffness matrix and derivative operator (P x P)
  std::vector<double> K1, iK1;       // time matrix F1 - Kxi and its inverse
  std::vector<double> F0, FL, FR;    // phi(0), phi(0), phi(1)
  std::vector<double> uh2lim;        // S x P: DG -> subcell averages
  std::vector<double> lim2uh;        // P x S: subcell averages -> DG (constrained LSQ)
  std::vector<double> uh2lob;        // P x P: DG -> Gauss-Lobatto point values
  std::vector<double> xilimbary;     // S subcell barycentres on [0,1]
};

bool build_ops(int N, HostOps& ops, std::string* err);

// Maximum CFL numbers of the PNPM schemes, Euler/ader_dg.f90:28.
double pnpm_cfl(int N);

// pi = 4 atan(1) as the host computes it (the initial fields use this value
// on the host and on the device alike).
double pi_value();

}  // namespace aderdg
