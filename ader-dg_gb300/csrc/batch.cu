// batch.cu -- many independent simulations of one (system, N, precision,
// limiter) stepped by the same launches.
//
// A batch owns a pool of "units" (one unit = one cell slot in every per-cell
// array).  A simulation with an IMAX x JMAX grid occupies (IMAX+1)(JMAX+1)
// consecutive units from a first-fit free list: its cells, x faces and
// y faces all index from the same base, so one sorted instance table serves
// every kernel.  Gaps between simulations are skipped by the kernels (no
// instance owns them).  Each simulation keeps its own time, CFL time step,
// end time, step budget and limiter state; finished ones stop by themselves
// and are released by the host, new ones are admitted while others run.
//
// Stepping is asynchronous: aderdg_batch_launch enqueues graph replays of one
// step on the batch's stream and returns; aderdg_batch_sync waits and reads
// the per-simulation state back.  Batches of different (system, N) thus run
// concurrently on their own streams.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aderdg_gpu.h"
#include "control.cuh"
#include "ic_eval.h"
#include "tables.h"

namespace aderdg {
void set_last_error(const std::string& msg);
int validate_config(const aderdg_config* c, std::string* why);
FaceConst make_face_const(const HostOps& ops);
InstDesc make_inst_desc(const aderdg_config* cfg);
}  // namespace aderdg

using aderdg::BatchArgs;
using aderdg::InstDesc;
using aderdg::InstState;

struct aderdg_batch {
  int system = 0, N = 0, precision = 0, limiter = 0, V = 0, P = 0, S = 0;
  long long capacity = 0;  // units
  int max_inst = 0, n_used = 0;
  const aderdg::KernelTable* kt = nullptr;
  aderdg::HostOps ops;
  std::vector<unsigned char> ops64, ops32;
  aderdg::FaceConst fc{};
  cudaStream_t stream = nullptr;
  int num_sms = 0, subcell_grid = 0;
  InstDesc* d_inst = nullptr;
  InstState* d_st = nullptr;
  InstDesc* d_inst_scr = nullptr;     // scratch copies for the table edits on the device
  InstState* d_st_scr = nullptr;
  InstState* h_st = nullptr;          // pinned, max_inst entries (table order)
  bool st_stale = false;              // h_st predates a table edit: pull before reading it
  std::vector<InstDesc> h_inst;       // table order: used entries sorted by base, then unused
  std::vector<int> slot_at;           // table position -> slot id
  std::vector<int> pos_of;            // slot id -> table position (-1: free)
  std::vector<aderdg_config> cfg_of;  // slot id -> its configuration
  std::vector<std::pair<long long, long long>> free_ranges;  // (base, size), sorted
  long long hw = 0;                   // end of the highest occupied unit
  BatchArgs args{};
  std::vector<void*> allocs;
  size_t bytes = 0;
  cudaGraphExec_t gexec = nullptr;
  long long graph_hw = -1;
  // set when an admission or release failed after editing the instance table:
  // the host and device tables may then disagree, so the batch refuses
  // further work (ADERDG_ESTATE) instead of stepping a table it cannot trust
  bool broken = false;
  std::string err;
};

namespace {

constexpr long long kUnusedBase = (1ll << 62);

int bfail(aderdg_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  aderdg::set_last_error(msg);
  return code;
}
// marks the batch unusable after a failure that left its table edited
int bbreak(aderdg_batch* b, int code) {
  b->broken = true;
  b->err = "batch unusable after a failed admission or release: " + b->err;
  aderdg::set_last_error(b->err);
  return code;
}
int bcheck(aderdg_batch* b) {
  if (b && b->broken) return bfail(b, ADERDG_ESTATE, b->err);
  return ADERDG_OK;
}
int bcuda(aderdg_batch* b, const char* what, cudaError_t e) {
  return bfail(b, ADERDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define BK(b, call)                                          \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return bcuda((b), #call, e_);     \
  } while (0)

int nvar(int sys) { return sys == ADERDG_SYS_ADVDIFF ? 1 : sys == ADERDG_SYS_EULER ? 4 : 9; }

// bytes per unit of every per-cell array of a batch
long long unit_bytes(int system, int N, int precision, int limiter) {
  const long long V = nvar(system), P = N + 1, S = 2 * N + 1;
  const long long rb = precision != ADERDG_FP64 ? 4 : 8;
  long long b = 8 * V * P * P * 2 + rb * V * P * P;                 // uh[2], duh
  b += rb * P * 4 * V * (system == ADERDG_SYS_ADVDIFF ? 3 : 2);     // qbnd, fbnd / gradQbnd
  b += rb * P * V * (system == ADERDG_SYS_BN ? 4 : 2);              // face fluxes
  if (limiter && system != ADERDG_SYS_ADVDIFF) {
    b += 8 * V * S * S * 2 + 4 * 2 + 8 * 2 * V * 2 + 1 + 4 + 4 + 8;  // Lh[2], status[2], mm[2], flags, list, denom
    if (precision == ADERDG_FP32_MIXED) b += 4 * V * 2 + 4;           // mme[2], settle list
  }
  return b;
}

template <class T>
int balloc(aderdg_batch* b, T** p, size_t n) {
  *p = nullptr;
  if (n == 0) return ADERDG_OK;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T));
  if (e != cudaSuccess) return bfail(b, ADERDG_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  // zeroed in the batch's stream: a plain cudaMemset runs on the legacy
  // default stream, which the batch's non-blocking stream does not wait for
  e = cudaMemsetAsync(q, 0, n * sizeof(T), b->stream);
  if (e != cudaSuccess) return bcuda(b, "cudaMemsetAsync", e);
  b->allocs.push_back(q);
  b->bytes += n * sizeof(T);
  *p = static_cast<T*>(q);
  return ADERDG_OK;
}

void bfree_all(aderdg_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  for (void* p : b->allocs) cudaFree(p);
  b->allocs.clear();
  if (b->h_st) cudaFreeHost(b->h_st);
  if (b->stream) cudaStreamDestroy(b->stream);
}

cudaError_t bcontrol(aderdg_batch* b, int mode, int only) {
  const int threads = 128, blocks = (b->max_inst + threads - 1) / threads;
  aderdg::k_control<<<blocks, threads, 0, b->stream>>>(b->d_inst, b->d_st, b->max_inst, b->args.list_count, mode, only);
  return cudaGetLastError();
}

int push_table(aderdg_batch* b) {
  BK(b, cudaMemcpyAsync(b->d_inst, b->h_inst.data(), sizeof(InstDesc) * b->max_inst, cudaMemcpyHostToDevice, b->stream));
  BK(b, cudaMemcpyAsync(b->d_st, b->h_st, sizeof(InstState) * b->max_inst, cudaMemcpyHostToDevice, b->stream));
  BK(b, cudaStreamSynchronize(b->stream));
  return ADERDG_OK;
}
int pull_states(aderdg_batch* b) {
  BK(b, cudaMemcpyAsync(b->h_st, b->d_st, sizeof(InstState) * b->max_inst, cudaMemcpyDeviceToHost, b->stream));
  BK(b, cudaStreamSynchronize(b->stream));
  b->st_stale = false;
  return ADERDG_OK;
}

// Table edits on the device, in stream order with the steps already queued,
// so that admission and release never wait for the GPU.  The device table
// (descriptors and the live states) of n used entries gets an entry inserted
// at pos (the rest move up one) or removed from pos (the rest move down one,
// `fresh` fills the freed last entry), staged through scratch copies.
template <class T>
__device__ __forceinline__ void copy_words(T* dst, const T* src, int w) {
  reinterpret_cast<unsigned long long*>(dst)[w] = reinterpret_cast<const unsigned long long*>(src)[w];
}
static_assert(sizeof(InstDesc) % 8 == 0 && sizeof(InstState) % 8 == 0, "table entries copied as 8-byte words");

__global__ void k_table_stage(const InstDesc* ti, const InstState* ts, InstDesc* si, InstState* ss, int n, int pos,
                              int insert, InstDesc fi, InstState fs) {
  constexpr int WI = sizeof(InstDesc) / 8, WS = sizeof(InstState) / 8;
  const int end = insert ? n + 1 : n;
  const long long total = (long long)(end - pos) * (WI + WS);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
    const int p = pos + (int)(k / (WI + WS)), w = (int)(k % (WI + WS));
    const bool fresh = insert ? p == pos : p == n - 1;
    const int q = insert ? p - 1 : p + 1;  // source entry of a moved one
    if (w < WI) copy_words(&si[p], fresh ? &fi : &ti[q], w);
    else copy_words(&ss[p], fresh ? &fs : &ts[q], w - WI);
  }
}

__global__ void k_table_commit(InstDesc* ti, InstState* ts, const InstDesc* si, const InstState* ss, int lo, int hi) {
  constexpr int WI = sizeof(InstDesc) / 8, WS = sizeof(InstState) / 8;
  const long long total = (long long)(hi - lo) * (WI + WS);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
    const int p = lo + (int)(k / (WI + WS)), w = (int)(k % (WI + WS));
    if (w < WI) copy_words(&ti[p], &si[p], w);
    else copy_words(&ts[p], &ss[p], w - WI);
  }
}

// n: used entries before the edit
int btable_edit(aderdg_batch* b, int n, int pos, bool insert, const InstDesc& fi, const InstState& fs) {
  const int end = insert ? n + 1 : n;
  if (end <= pos) return ADERDG_OK;
  const long long words = (long long)(end - pos) * ((sizeof(InstDesc) + sizeof(InstState)) / 8);
  const unsigned blocks = (unsigned)std::min<long long>((words + 255) / 256, 64);
  k_table_stage<<<blocks, 256, 0, b->stream>>>(b->d_inst, b->d_st, b->d_inst_scr, b->d_st_scr, n, pos, insert ? 1 : 0,
                                               fi, fs);
  BK(b, cudaGetLastError());
  k_table_commit<<<blocks, 256, 0, b->stream>>>(b->d_inst, b->d_st, b->d_inst_scr, b->d_st_scr, pos, end);
  BK(b, cudaGetLastError());
  b->st_stale = true;
  return ADERDG_OK;
}

const void* bpred_ops(aderdg_batch* b) { return b->precision ? b->ops32.data() : b->ops64.data(); }

int blaunch_step(aderdg_batch* b) {
  BatchArgs a = b->args;
  a.ncells = b->hw;
  a.nfx = b->hw;
  a.nfy = b->hw;
  a.mode = aderdg::kCellFused;
  BK(b, bcontrol(b, aderdg::kCtlBegin, -1));
  BK(b, aderdg::launch_predictor(b->kt, a, bpred_ops(b), b->precision, b->stream));
  BK(b, aderdg::launch_faces(b->kt, a, b->fc, b->precision, b->stream));
  BK(b, aderdg::launch_cells(b->kt, a, b->ops64.data(), b->precision, b->stream));
  if (a.settle) BK(b, b->kt->settle(a, b->ops64.data(), b->num_sms, b->stream));
  if (b->limiter) {
    BK(b, b->kt->mark(a, b->stream));
    BK(b, aderdg::launch_subcell(b->kt, a, b->ops64.data(), b->fc, b->subcell_grid, b->num_sms, b->precision, b->stream));
  }
  BK(b, bcontrol(b, aderdg::kCtlEnd, -1));
  return ADERDG_OK;
}

int bensure_graph(aderdg_batch* b) {
  if (b->gexec && b->graph_hw == b->hw) return ADERDG_OK;
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  cudaGraph_t g = nullptr;
  BK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int r = blaunch_step(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (r) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return bcuda(b, "cudaStreamEndCapture", e);
  e = cudaGraphInstantiate(&b->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bcuda(b, "cudaGraphInstantiate", e);
  b->graph_hw = b->hw;
  return ADERDG_OK;
}

// K3 over one instance's cells only (priming modes)
int bcells_one(aderdg_batch* b, int pos, int mode, const double* lh_ic) {
  const InstDesc& in = b->h_inst[pos];
  BatchArgs a = b->args;
  a.mode = mode;
  a.cell0 = in.cell_base;
  a.ncells = in.cell_base + (long long)in.imax * in.jmax;
  a.only_inst = pos;
  a.lh_ic = lh_ic;
  BK(b, aderdg::launch_cells(b->kt, a, b->ops64.data(), b->precision, b->stream));
  if (a.settle && mode == aderdg::kCellInitDmp) BK(b, b->kt->settle(a, b->ops64.data(), b->num_sms, b->stream));
  return ADERDG_OK;
}

int bprime_one(aderdg_batch* b, int pos) {
  BK(b, bcontrol(b, aderdg::kCtlPrimeReset, pos));
  int r = bcells_one(b, pos, aderdg::kCellPrime, nullptr);
  if (r) return r;
  BK(b, bcontrol(b, aderdg::kCtlPrimeCommit, pos));
  return ADERDG_OK;
}

void recompute_hw(aderdg_batch* b) {
  b->hw = 0;
  for (int p = 0; p < b->n_used; ++p) {
    const InstDesc& d = b->h_inst[p];
    b->hw = std::max(b->hw, d.cell_base + (long long)(d.imax + 1) * (d.jmax + 1));
  }
}

}  // namespace

extern "C" {

long aderdg_batch_unit_bytes(int system, int N, int precision, int limiter) {
  if (system < 0 || system > 2 || N < 1 || N > 5) return ADERDG_EINVAL;
  return (long)unit_bytes(system, N, precision, limiter);
}

int aderdg_batch_create(int system, int N, int precision, int limiter, long capacity_units, int max_instances,
                        aderdg_batch** out) {
  if (!out) return bfail(nullptr, ADERDG_EINVAL, "null output pointer");
  *out = nullptr;
  if (system < 0 || system > 2 || N < 1 || N > 5 || capacity_units < 4 || max_instances < 1 ||
      (precision != ADERDG_FP64 && precision != ADERDG_FP32_MIXED && precision != ADERDG_FP32_WIDE))
    return bfail(nullptr, ADERDG_EINVAL, "bad batch parameters");
  const aderdg::KernelTable* kt = aderdg::kernel_table(system, N);
  if (!kt) return bfail(nullptr, ADERDG_EUNSUPPORTED, "no kernels built for this (system, N)");
  aderdg_batch* b = new aderdg_batch();
  b->system = system;
  b->N = N;
  b->precision = precision;
  b->limiter = (limiter != 0 && system != ADERDG_SYS_ADVDIFF) ? 1 : 0;
  b->V = nvar(system);
  b->P = N + 1;
  b->S = 2 * N + 1;
  b->capacity = capacity_units;
  b->max_inst = max_instances;
  b->kt = kt;
  std::string why;
  auto bail = [&](int code) {
    bfree_all(b);
    delete b;
    return code;
  };
  if (!aderdg::build_ops(N, b->ops, &why)) return bail(bfail(nullptr, ADERDG_EINVAL, why));
  b->fc = aderdg::make_face_const(b->ops);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_st, sizeof(InstState) * max_instances);
  if (e != cudaSuccess) return bail(bcuda(nullptr, "batch set-up", e));
  std::memset(b->h_st, 0, sizeof(InstState) * max_instances);
  const size_t U = (size_t)capacity_units, V = b->V, P = b->P, S = b->S;
  const size_t rb = precision ? 4 : 8;
  BatchArgs& a = b->args;
  std::memset(&a, 0, sizeof(a));
  int r = balloc(b, &b->d_inst, (size_t)max_instances);
  if (!r) r = balloc(b, &b->d_st, (size_t)max_instances);
  if (!r) r = balloc(b, &b->d_inst_scr, (size_t)max_instances);
  if (!r) r = balloc(b, &b->d_st_scr, (size_t)max_instances);
  if (!r) r = balloc(b, &a.uh[0], U * P * P * V);
  if (!r) r = balloc(b, &a.uh[1], U * P * P * V);
  // duh and the face fluxes hold FP32 values in the FP32 modes: half the doubles
  auto stor = [&](size_t n) { return precision ? (n + 1) / 2 : n; };
  if (!r) r = balloc(b, &a.duh, stor(U * P * P * V));
  unsigned char *qb = nullptr, *fb = nullptr;
  if (!r) r = balloc(b, &qb, U * P * 4 * V * rb);
  if (!r) r = balloc(b, &fb, U * P * 4 * V * rb * (system == ADERDG_SYS_ADVDIFF ? 2 : 1));
  a.qbnd = qb;
  a.fbnd = fb;
  if (!r) r = balloc(b, &a.fu, stor(U * P * V));
  if (!r) r = balloc(b, &a.gu, stor(U * P * V));
  if (!r && system == ADERDG_SYS_BN) r = balloc(b, &a.fp, stor(U * P * V));
  if (!r && system == ADERDG_SYS_BN) r = balloc(b, &a.gp, stor(U * P * V));
  if (!r) r = balloc(b, &a.list_count, 2);
  if (b->limiter) {
    if (!r) r = balloc(b, &a.status[0], U);
    if (!r) r = balloc(b, &a.status[1], U);
    if (!r) r = balloc(b, &a.lh[0], U * S * S * V);
    if (!r) r = balloc(b, &a.lh[1], U * S * S * V);
    if (!r) r = balloc(b, &a.mm[0], U * 2 * V);
    if (!r) r = balloc(b, &a.mm[1], U * 2 * V);
    if (!r && precision == ADERDG_FP32_MIXED) r = balloc(b, &a.mme[0], U * V);
    if (!r && precision == ADERDG_FP32_MIXED) r = balloc(b, &a.mme[1], U * V);
    if (!r && precision == ADERDG_FP32_MIXED) r = balloc(b, &a.settle, U);
    // no lminmax: the neighbourhood bounds are an introspection output of
    // the single-simulation API only
    if (!r) r = balloc(b, &a.troubled, U);
    if (!r) r = balloc(b, &a.recompute, U);
    if (!r) r = balloc(b, &a.list, U);
    if (!r) r = balloc(b, &a.denom, U);
  }
  if (r) return bail(r);
  a.inst = b->d_inst;
  a.st = b->d_st;
  a.ninst = max_instances;
  a.only_inst = -1;
  b->h_inst.assign(max_instances, InstDesc{});
  for (auto& d : b->h_inst) {
    d.imax = d.jmax = 1;
    d.cell_base = d.fx_base = d.fy_base = kUnusedBase;
  }
  b->slot_at.assign(max_instances, -1);
  b->pos_of.assign(max_instances, -1);
  b->cfg_of.assign(max_instances, aderdg_config{});
  b->free_ranges.push_back({0, capacity_units});
  b->ops64.assign(kt->ops64_size, 0);
  kt->make_ops64(b->ops, b->ops64.data());
  if (precision) {
    b->ops32.assign(kt->ops32_size, 0);
    kt->make_ops32(b->ops, b->ops32.data());
  }
  if (b->limiter) b->subcell_grid = aderdg::subcell_grid_of(kt, b->num_sms, b->precision);
  {  // kernel attributes before any capture
    BatchArgs z = a;
    z.ncells = z.nfx = z.nfy = 0;
    kt->predictor(z, bpred_ops(b), precision ? 1 : 0, false, b->stream);
    kt->cells(z, b->ops64.data(), precision ? 1 : 0, b->stream);
    aderdg::launch_predictor(kt, z, bpred_ops(b), precision, b->stream);
    aderdg::launch_cells(kt, z, b->ops64.data(), precision, b->stream);
  }
  r = push_table(b);
  if (r) return bail(r);
  *out = b;
  return ADERDG_OK;
}

int aderdg_batch_destroy(aderdg_batch* b) {
  if (!b) return ADERDG_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  bfree_all(b);
  delete b;
  return ADERDG_OK;
}

namespace {

// Admission of one simulation: its initial state comes from host arrays
// (uh, lh_ic) or, with ic >= 0, is evaluated on the device.
int badmit_fill(aderdg_batch* b, const aderdg_config* cfg, const double* uh, const double* lh_ic, int ic,
                const double* params, long long base, int pos);

int badmit(aderdg_batch* b, const aderdg_config* cfg, const double* uh, const double* lh_ic, int ic,
           const double* params, double tend, long max_steps, int* slot) {
  if (!b || !cfg || !slot || (ic < 0 && !uh)) return bfail(b, ADERDG_EINVAL, "null argument");
  if (int r = bcheck(b)) return r;
  if (ic >= 0) {
    double p[32] = {0};
    if (params) std::memcpy(p, params, sizeof(p));
    if (!aderdg::ic_valid(cfg->system, ic, p))
      return bfail(b, ADERDG_EINVAL, "initial field " + std::to_string(ic) + " is not defined for this system");
  }
  std::string why;
  int r = aderdg::validate_config(cfg, &why);
  if (r) return bfail(b, r, why);
  const int lim = (cfg->limiter != 0 && cfg->system != ADERDG_SYS_ADVDIFF) ? 1 : 0;
  if (cfg->system != b->system || cfg->N != b->N || cfg->precision != b->precision || lim != b->limiter)
    return bfail(b, ADERDG_EINVAL, "simulation does not match the batch's (system, N, precision, limiter)");
  if (b->n_used >= b->max_inst) return bfail(b, ADERDG_ENOSPACE, "batch instance table full");
  const long long need = (long long)(cfg->imax + 1) * (cfg->jmax + 1);
  long long base = -1;
  for (auto it = b->free_ranges.begin(); it != b->free_ranges.end(); ++it)
    if (it->second >= need) {
      base = it->first;
      it->first += need;
      it->second -= need;
      if (it->second == 0) b->free_ranges.erase(it);
      break;
    }
  if (base < 0) return bfail(b, ADERDG_ENOSPACE, "no free range of " + std::to_string(need) + " units");
  // insert into the table, keeping it sorted by base: the descriptors on the
  // host, the device table (descriptors and live states) by a table edit in
  // stream order after the steps already queued
  const int n_before = b->n_used;
  int pos = 0;
  while (pos < b->n_used && b->h_inst[pos].cell_base < base) ++pos;
  for (int p = b->n_used; p > pos; --p) {
    b->h_inst[p] = b->h_inst[p - 1];
    b->slot_at[p] = b->slot_at[p - 1];
    b->pos_of[b->slot_at[p]] = p;
  }
  int s = 0;
  while (b->pos_of[s] >= 0) ++s;
  b->slot_at[pos] = s;
  b->pos_of[s] = pos;
  b->cfg_of[s] = *cfg;
  ++b->n_used;
  InstDesc& in = b->h_inst[pos];
  in = aderdg::make_inst_desc(cfg);
  in.cell_base = in.fx_base = in.fy_base = base;
  InstState st;
  std::memset(&st, 0, sizeof(st));
  st.time = 0.0;
  st.tend = tend;
  st.max_steps = max_steps;
  recompute_hw(b);
  r = btable_edit(b, n_before, pos, true, in, st);
  if (!r) r = badmit_fill(b, cfg, uh, lh_ic, ic, params, base, pos);
  if (r) return bbreak(b, r);
  *slot = s;
  return ADERDG_OK;
}

// the new simulation's state and its priming, after its table entry
int badmit_fill(aderdg_batch* b, const aderdg_config* cfg, const double* uh, const double* lh_ic, int ic,
                const double* params, long long base, int pos) {
  int r = ADERDG_OK;
  // state of the new simulation (parity 0); host-given subcell candidates of
  // the initial limiter are staged in the next-parity Lh slab of this
  // simulation, device-evaluated ones are formed after the initial DMP for the
  // cells it limits only
  const size_t cells = (size_t)cfg->imax * cfg->jmax, P2V = (size_t)b->P * b->P * b->V, S2V = (size_t)b->S * b->S * b->V;
  double* uh_dst = b->args.uh[0] + (size_t)base * P2V;
  double* lh_stage = b->limiter ? b->args.lh[1] + (size_t)base * S2V : nullptr;
  bool staged = false;
  const bool lazy_lh = ic >= 0 && b->limiter;
  if (ic >= 0) {
    std::string why;
    cudaError_t e = aderdg::launch_initial_field(*cfg, ic, params, uh_dst, nullptr, b->stream, &why);
    if (e != cudaSuccess) return bcuda(b, ("initial field: " + why).c_str(), e);
  } else {
    BK(b, cudaMemcpyAsync(uh_dst, uh, cells * P2V * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  if (b->limiter) {
    BK(b, cudaMemsetAsync(b->args.status[0] + base, 0, cells * sizeof(int), b->stream));
    BK(b, cudaMemsetAsync(b->args.status[1] + base, 0, cells * sizeof(int), b->stream));
  }
  r = bprime_one(b, pos);
  if (r) return r;
  if (b->limiter && ic < 0 && lh_ic) {
    BK(b, cudaMemcpyAsync(lh_stage, lh_ic, cells * S2V * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    staged = true;
  }
  if (staged || lazy_lh) {
    BK(b, bcontrol(b, aderdg::kCtlPrimeReset, pos));
    r = bcells_one(b, pos, aderdg::kCellInitDmp, staged ? b->args.lh[1] : nullptr);
    if (r) return r;
    if (lazy_lh) {
      std::string why;
      cudaError_t e = aderdg::launch_initial_lh(*cfg, ic, params, b->args.status[0] + base,
                                                b->args.lh[0] + (size_t)base * S2V, b->args.lh[1] + (size_t)base * S2V,
                                                b->stream, &why);
      if (e != cudaSuccess) return bcuda(b, ("initial limiter: " + why).c_str(), e);
    }
    // the limited cells' min/max from their subcell data; the others' and the
    // CFL denominator (uh only) stay those of the first priming pass
    r = bcells_one(b, pos, aderdg::kCellPrimeLimited, nullptr);
    if (r) return r;
  }
  // nothing waits for the GPU (the host mirror of the states is refreshed at
  // the next sync or query), except that host arrays are copied before the
  // call returns, so that the caller may reuse them
  if (ic < 0) BK(b, cudaStreamSynchronize(b->stream));
  return ADERDG_OK;
}

}  // namespace

int aderdg_batch_admit(aderdg_batch* b, const aderdg_config* cfg, const double* uh, const double* lh_ic, double tend,
                       long max_steps, int* slot) {
  return badmit(b, cfg, uh, lh_ic, -1, nullptr, tend, max_steps, slot);
}

int aderdg_batch_admit_ic(aderdg_batch* b, const aderdg_config* cfg, int ic, const double* params, double tend,
                          long max_steps, int* slot) {
  if (ic < 0) return bfail(b, ADERDG_EINVAL, "bad initial field id");
  return badmit(b, cfg, nullptr, nullptr, ic, params, tend, max_steps, slot);
}

int aderdg_batch_release(aderdg_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->max_inst || b->pos_of[slot] < 0) return bfail(b, ADERDG_EINVAL, "bad slot");
  if (int r = bcheck(b)) return r;
  const int pos = b->pos_of[slot];
  const int n_before = b->n_used;
  const InstDesc in = b->h_inst[pos];
  const long long size = (long long)(in.imax + 1) * (in.jmax + 1);
  for (int p = pos; p < b->n_used - 1; ++p) {
    b->h_inst[p] = b->h_inst[p + 1];
    b->slot_at[p] = b->slot_at[p + 1];
    b->pos_of[b->slot_at[p]] = p;
  }
  --b->n_used;
  InstDesc& d = b->h_inst[b->n_used];
  d = InstDesc{};
  d.imax = d.jmax = 1;
  d.cell_base = d.fx_base = d.fy_base = kUnusedBase;
  InstState zero;
  std::memset(&zero, 0, sizeof(zero));
  int r = btable_edit(b, n_before, pos, false, d, zero);
  if (r) return bbreak(b, r);
  b->slot_at[b->n_used] = -1;
  b->pos_of[slot] = -1;
  // return the range to the free list, merging neighbours
  auto& fr = b->free_ranges;
  fr.push_back({in.cell_base, size});
  std::sort(fr.begin(), fr.end());
  std::vector<std::pair<long long, long long>> merged;
  for (auto& x : fr) {
    if (!merged.empty() && merged.back().first + merged.back().second == x.first) merged.back().second += x.second;
    else merged.push_back(x);
  }
  fr.swap(merged);
  recompute_hw(b);
  return ADERDG_OK;
}

int aderdg_batch_launch(aderdg_batch* b, int steps) {
  if (!b) return bfail(b, ADERDG_EINVAL, "null batch");
  if (int r = bcheck(b)) return r;
  if (steps <= 0 || b->n_used == 0) return ADERDG_OK;
  int r = bensure_graph(b);
  if (r) return r;
  for (int s = 0; s < steps; ++s) BK(b, cudaGraphLaunch(b->gexec, b->stream));
  return ADERDG_OK;
}

int aderdg_batch_run_timed(aderdg_batch* const* batches, int n, int steps, double* ms) {
  if (!batches || n <= 0 || !ms) return bfail(nullptr, ADERDG_EINVAL, "null argument");
  for (int k = 0; k < n; ++k) {
    if (!batches[k]) return bfail(nullptr, ADERDG_EINVAL, "null batch");
    if (int r = bcheck(batches[k])) return r;
  }
  aderdg_batch* b0 = batches[0];
  for (int k = 0; k < n; ++k) {
    if (batches[k]->n_used == 0) continue;
    int r = bensure_graph(batches[k]);
    if (r) return r;
  }
  cudaStream_t ts = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<cudaEvent_t> done((size_t)n, nullptr);
  cudaError_t e = cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int k = 0; k < n && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
  // every batch stream starts after e0 on the timing stream; e1 follows all of them
  if (e == cudaSuccess) e = cudaEventRecord(e0, ts);
  for (int k = 0; k < n && e == cudaSuccess; ++k) {
    aderdg_batch* b = batches[k];
    e = cudaStreamWaitEvent(b->stream, e0, 0);
    for (int s = 0; s < steps && e == cudaSuccess && b->n_used > 0; ++s) e = cudaGraphLaunch(b->gexec, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(done[k], b->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ts, done[k], 0);
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, ts);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float f = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
  for (auto d : done)
    if (d) cudaEventDestroy(d);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (ts) cudaStreamDestroy(ts);
  if (e != cudaSuccess) return bcuda(b0, "aderdg_batch_run_timed", e);
  *ms = (double)f;
  return ADERDG_OK;
}

int aderdg_batch_ready(aderdg_batch* b, int* ready) {
  if (!b || !ready) return bfail(b, ADERDG_EINVAL, "null argument");
  if (int r = bcheck(b)) return r;
  const cudaError_t e = cudaStreamQuery(b->stream);
  if (e == cudaErrorNotReady) {
    *ready = 0;
    return ADERDG_OK;
  }
  if (e != cudaSuccess) return bbreak(b, bcuda(b, "cudaStreamQuery", e));
  *ready = 1;
  return ADERDG_OK;
}

int aderdg_batch_sync(aderdg_batch* b, int* n_running) {
  if (!b) return bfail(b, ADERDG_EINVAL, "null batch");
  int r = pull_states(b);
  if (r) return r;
  int n = 0;
  for (int p = 0; p < b->n_used; ++p) {
    const InstState& s = b->h_st[p];
    const bool done = !(s.time < s.tend) || s.nonfinite || (s.max_steps > 0 && s.steps >= s.max_steps);
    n += done ? 0 : 1;
  }
  if (n_running) *n_running = n;
  return ADERDG_OK;
}

int aderdg_batch_query(aderdg_batch* b, int slot, double* time, double* dt, long* steps, int* done) {
  if (!b || slot < 0 || slot >= b->max_inst || b->pos_of[slot] < 0) return bfail(b, ADERDG_EINVAL, "bad slot");
  if (b->st_stale) {
    const int r = pull_states(b);
    if (r) return r;
  }
  const InstState& s = b->h_st[b->pos_of[slot]];
  if (time) *time = s.time;
  if (dt) *dt = s.dt;
  if (steps) *steps = (long)s.steps;
  if (done) *done = (!(s.time < s.tend) || s.nonfinite || (s.max_steps > 0 && s.steps >= s.max_steps)) ? 1 : 0;
  if (s.nonfinite) return bfail(b, ADERDG_ENONFINITE, "the time step became non-finite");
  return ADERDG_OK;
}

int aderdg_batch_counters(aderdg_batch* b, int* n_recompute, int* n_listed, int* n_settled) {
  if (!b) return bfail(b, ADERDG_EINVAL, "null batch");
  int r = pull_states(b);
  if (r) return r;
  long long a = 0, l = 0, s = 0;
  for (int p = 0; p < b->n_used; ++p) {
    a += b->h_st[p].n_recompute;
    l += b->h_st[p].n_list;
    s += b->h_st[p].n_settled;
  }
  if (n_recompute) *n_recompute = (int)a;
  if (n_listed) *n_listed = (int)l;
  if (n_settled) *n_settled = (int)s;
  return ADERDG_OK;
}

int aderdg_batch_download_status(aderdg_batch* b, int slot, int* status) {
  if (!b || !status || slot < 0 || slot >= b->max_inst || b->pos_of[slot] < 0)
    return bfail(b, ADERDG_EINVAL, "bad slot");
  int r = pull_states(b);
  if (r) return r;
  const int pos = b->pos_of[slot];
  const InstDesc& in = b->h_inst[pos];
  const size_t cells = (size_t)in.imax * in.jmax;
  if (!b->limiter) {
    std::memset(status, 0, cells * sizeof(int));
    return ADERDG_OK;
  }
  const int par = (int)(b->h_st[pos].steps & 1);
  BK(b, cudaMemcpyAsync(status, b->args.status[par] + in.cell_base, cells * sizeof(int), cudaMemcpyDeviceToHost,
                        b->stream));
  BK(b, cudaStreamSynchronize(b->stream));
  return ADERDG_OK;
}

int aderdg_batch_download(aderdg_batch* b, int slot, double* uh) {
  if (!b || !uh || slot < 0 || slot >= b->max_inst || b->pos_of[slot] < 0) return bfail(b, ADERDG_EINVAL, "bad slot");
  int r = pull_states(b);
  if (r) return r;
  const int pos = b->pos_of[slot];
  const InstDesc& in = b->h_inst[pos];
  const int par = (int)(b->h_st[pos].steps & 1);
  const size_t cells = (size_t)in.imax * in.jmax, P2V = (size_t)b->P * b->P * b->V;
  BK(b, cudaMemcpyAsync(uh, b->args.uh[par] + (size_t)in.cell_base * P2V, cells * P2V * sizeof(double),
                        cudaMemcpyDeviceToHost, b->stream));
  BK(b, cudaStreamSynchronize(b->stream));
  return ADERDG_OK;
}

int aderdg_batch_cell_averages(aderdg_batch* b, int slot, int primitive, double* out) {
  if (!b || !out || slot < 0 || slot >= b->max_inst || b->pos_of[slot] < 0) return bfail(b, ADERDG_EINVAL, "bad slot");
  int r = pull_states(b);
  if (r) return r;
  const int pos = b->pos_of[slot];
  const InstDesc& in = b->h_inst[pos];
  const int par = (int)(b->h_st[pos].steps & 1);
  const size_t cells = (size_t)in.imax * in.jmax, P2V = (size_t)b->P * b->P * b->V;
  double* tmp = nullptr;
  BK(b, cudaMallocAsync(&tmp, cells * b->V * sizeof(double), b->stream));
  std::string why;
  cudaError_t e = aderdg::launch_cell_averages(b->cfg_of[slot], b->args.uh[par] + (size_t)in.cell_base * P2V,
                                               primitive, tmp, b->stream, &why);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, tmp, cells * b->V * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
  cudaFreeAsync(tmp, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, ("cell averages: " + why).c_str(), e);
  return ADERDG_OK;
}

int aderdg_batch_info(aderdg_batch* b, long* used_units, long* capacity_units, long* device_bytes, int* n_instances) {
  if (!b) return bfail(b, ADERDG_EINVAL, "null batch");
  long long used = 0;
  for (int p = 0; p < b->n_used; ++p) used += (long long)(b->h_inst[p].imax + 1) * (b->h_inst[p].jmax + 1);
  if (used_units) *used_units = (long)used;
  if (capacity_units) *capacity_units = (long)b->capacity;
  if (device_bytes) *device_bytes = (long)b->bytes;
  if (n_instances) *n_instances = b->n_used;
  return ADERDG_OK;
}

int aderdg_batch_profile(aderdg_batch* b, double* phase_ms) {
  if (!b || !phase_ms) return bfail(b, ADERDG_EINVAL, "null argument");
  if (b->n_used == 0) {
    for (int k = 0; k < 7; ++k) phase_ms[k] = 0.0;
    return ADERDG_OK;
  }
  BatchArgs a = b->args;
  a.ncells = a.nfx = a.nfy = b->hw;
  a.mode = aderdg::kCellFused;
  cudaEvent_t ev[8];
  for (auto& e : ev) BK(b, cudaEventCreate(&e));
  BK(b, cudaEventRecord(ev[0], b->stream));
  BK(b, bcontrol(b, aderdg::kCtlBegin, -1));
  BK(b, cudaEventRecord(ev[1], b->stream));
  BK(b, aderdg::launch_predictor(b->kt, a, bpred_ops(b), b->precision, b->stream));
  BK(b, cudaEventRecord(ev[2], b->stream));
  BK(b, aderdg::launch_faces(b->kt, a, b->fc, b->precision, b->stream));
  BK(b, cudaEventRecord(ev[3], b->stream));
  BK(b, aderdg::launch_cells(b->kt, a, b->ops64.data(), b->precision, b->stream));
  if (a.settle) BK(b, b->kt->settle(a, b->ops64.data(), b->num_sms, b->stream));
  BK(b, cudaEventRecord(ev[4], b->stream));
  if (b->limiter) BK(b, b->kt->mark(a, b->stream));
  BK(b, cudaEventRecord(ev[5], b->stream));
  if (b->limiter)
    BK(b, aderdg::launch_subcell(b->kt, a, b->ops64.data(), b->fc, b->subcell_grid, b->num_sms, b->precision, b->stream));
  BK(b, cudaEventRecord(ev[6], b->stream));
  BK(b, bcontrol(b, aderdg::kCtlEnd, -1));
  BK(b, cudaEventRecord(ev[7], b->stream));
  BK(b, cudaStreamSynchronize(b->stream));
  for (int k = 0; k < 7; ++k) {
    float ms = 0.f;
    BK(b, cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
    phase_ms[k] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return pull_states(b);
}

const char* aderdg_batch_last_error(aderdg_batch* b) { return b ? b->err.c_str() : ""; }

}  // extern "C"
