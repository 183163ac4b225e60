// registry.cu -- collects the per-(system, N) launch tables built by the
// predictor and exact translation units.
#include "tables.h"

namespace aderdg {

#define ADERDG_DECL(S, NN)                             \
  void register_predictor_##S##_##NN(KernelTable& t); \
  void register_exact_##S##_##NN(KernelTable& t);
#define ADERDG_DECL_N(S) ADERDG_DECL(S, 1) ADERDG_DECL(S, 2) ADERDG_DECL(S, 3) ADERDG_DECL(S, 4) ADERDG_DECL(S, 5)
ADERDG_DECL_N(0)
ADERDG_DECL_N(1)
ADERDG_DECL_N(2)

namespace {
struct Registry {
  KernelTable t[3][6];
  Registry() {
#define ADERDG_REG(S, NN)                    \
  register_predictor_##S##_##NN(t[S][NN]); \
  register_exact_##S##_##NN(t[S][NN]);
#define ADERDG_REG_N(S) ADERDG_REG(S, 1) ADERDG_REG(S, 2) ADERDG_REG(S, 3) ADERDG_REG(S, 4) ADERDG_REG(S, 5)
    ADERDG_REG_N(0)
    ADERDG_REG_N(1)
    ADERDG_REG_N(2)
  }
};
}  // namespace

const KernelTable* kernel_table(int sys, int N) {
  static Registry reg;
  if (sys < 0 || sys > 2 || N < 1 || N > 5) return nullptr;
  const KernelTable* t = &reg.t[sys][N];
  return t->predictor ? t : nullptr;
}

}  // namespace aderdg
