// registry.cu -- collects the per-(system, N) launch tables built by the
// predictor and exact translation units.
#include "tables.h"

namespace aderdg {

#define ADERDG_DECL(S, NN)                             \
  void register_predictor_##S##_##NN(KernelTable& t); \
  void register_exact_##S##_##NN(KernelTable& t);     \
  void register_cellsvar_##S##_##NN(KernelTable& t);  \
  void register_predvar_##S##_##NN##_1(KernelTable& t); \
  void register_predvar_##S##_##NN##_2(KernelTable& t); \
  void register_predvar_##S##_##NN##_3(KernelTable& t); \
  void register_predvar_##S##_##NN##_4(KernelTable& t); \
  void register_predvar_##S##_##NN##_5(KernelTable& t); \
  void register_predvar_##S##_##NN##_6(KernelTable& t);
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
  register_exact_##S##_##NN(t[S][NN]);     \
  register_cellsvar_##S##_##NN(t[S][NN]);  \
  register_predvar_##S##_##NN##_1(t[S][NN]); \
  register_predvar_##S##_##NN##_2(t[S][NN]); \
  register_predvar_##S##_##NN##_3(t[S][NN]); \
  register_predvar_##S##_##NN##_4(t[S][NN]); \
  register_predvar_##S##_##NN##_5(t[S][NN]); \
  register_predvar_##S##_##NN##_6(t[S][NN]);
#define ADERDG_REG_N(S) ADERDG_REG(S, 1) ADERDG_REG(S, 2) ADERDG_REG(S, 3) ADERDG_REG(S, 4) ADERDG_REG(S, 5)
    ADERDG_REG_N(0)
    ADERDG_REG_N(1)
    ADERDG_REG_N(2)
  }
};
}  // namespace

// the tuner's table: [system][N][precision], zeros = the defaults; ints read
// at every launch, written rarely (atomically per field)
namespace {
aderdg_tuning g_tune[3][6][3] = {};
}  // namespace

aderdg_tuning tuning_of(int sys, int N, int precision) {
  if (sys < 0 || sys > 2 || N < 1 || N > 5 || precision < 0 || precision > 2) return aderdg_tuning{};
  const aderdg_tuning& t = g_tune[sys][N][precision];
  aderdg_tuning r;
  r.predictor = __atomic_load_n(&t.predictor, __ATOMIC_RELAXED);
  r.cells = __atomic_load_n(&t.cells, __ATOMIC_RELAXED);
  r.subcell_per_sm = __atomic_load_n(&t.subcell_per_sm, __ATOMIC_RELAXED);
  return r;
}

const KernelTable* kernel_table(int sys, int N) {
  static Registry reg;
  if (sys < 0 || sys > 2 || N < 1 || N > 5) return nullptr;
  const KernelTable* t = &reg.t[sys][N];
  return t->predictor ? t : nullptr;
}

}  // namespace aderdg

extern "C" {

int aderdg_set_tuning(int system, int N, int precision, const aderdg_tuning* t) {
  if (!t || system < 0 || system > 2 || N < 1 || N > 5 || precision < 0 || precision > 2) return ADERDG_EINVAL;
  if (t->predictor < 0 || t->predictor >= aderdg::kPredVariantsMax || t->cells < 0 ||
      t->cells >= aderdg::kCellVariantsMax || t->subcell_per_sm < 0 || t->subcell_per_sm > 64)
    return ADERDG_EINVAL;
  aderdg_tuning& d = aderdg::g_tune[system][N][precision];
  __atomic_store_n(&d.predictor, t->predictor, __ATOMIC_RELAXED);
  __atomic_store_n(&d.cells, t->cells, __ATOMIC_RELAXED);
  __atomic_store_n(&d.subcell_per_sm, t->subcell_per_sm, __ATOMIC_RELAXED);
  return ADERDG_OK;
}

int aderdg_get_tuning(int system, int N, int precision, aderdg_tuning* t) {
  if (!t || system < 0 || system > 2 || N < 1 || N > 5 || precision < 0 || precision > 2) return ADERDG_EINVAL;
  *t = aderdg::tuning_of(system, N, precision);
  return ADERDG_OK;
}

int aderdg_tuning_variants(int* n_predictor, int* n_cells) {
  if (n_predictor) *n_predictor = aderdg::kPredVariantsMax;
  if (n_cells) *n_cells = aderdg::kCellVariantsMax;
  return ADERDG_OK;
}

}  // extern "C"
