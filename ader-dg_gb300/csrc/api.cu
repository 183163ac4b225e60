// api.cu -- the C ABI of include/aderdg_gpu.h: context lifecycle, the phase
// API (one call per reference phase), the fused step and the graph-captured
// run loop.  Host code only; the kernels live in predictor_tu.cu and
// exact_tu.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aderdg_gpu.h"
#include "control.cuh"
#include "tables.h"

using aderdg::BatchArgs;
using aderdg::InstDesc;
using aderdg::InstState;
using aderdg::KernelTable;

struct aderdg_ctx {
  aderdg_config cfg{};
  int V = 0, P = 0, S = 0;
  long long ncells = 0, nfx = 0, nfy = 0;
  bool limiter = false, fp32 = false;  // fp32: FP32 predictor and intermediates (both FP32 modes)
  int prec = ADERDG_FP64;
  aderdg::HostOps ops;
  std::vector<unsigned char> ops64, ops32;
  const KernelTable* kt = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0, num_sms = 0, subcell_grid = 0;
  InstDesc h_inst{};
  InstState* h_st = nullptr;  // pinned mirror of the device state
  InstDesc* d_inst = nullptr;
  InstState* d_st = nullptr;
  BatchArgs args{};
  aderdg::FaceConst fc{};
  std::vector<void*> allocs;
  size_t bytes = 0;
  bool uploaded = false;
  bool pending = false;  // between element_update and the limiter commit (phase API)
  cudaGraphExec_t gexec = nullptr;
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  std::string err;
};

namespace {

thread_local std::string g_err;

int fail(aderdg_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  g_err = msg;
  return code;
}
int fail_cuda(aderdg_ctx* ctx, const char* what, cudaError_t e) {
  return fail(ctx, ADERDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(ctx, call)                                          \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return fail_cuda((ctx), #call, e_); \
  } while (0)

template <class T>
int dalloc(aderdg_ctx* c, T** p, size_t n) {
  *p = nullptr;
  if (n == 0) return ADERDG_OK;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T));
  if (e != cudaSuccess) return fail(c, ADERDG_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  // zeroed in the context's stream: a plain cudaMemset runs on the legacy
  // default stream, which the context's non-blocking stream does not wait for
  e = cudaMemsetAsync(q, 0, n * sizeof(T), c->stream);
  if (e != cudaSuccess) {
    cudaFree(q);
    return fail_cuda(c, "cudaMemset", e);
  }
  c->allocs.push_back(q);
  c->bytes += n * sizeof(T);
  *p = static_cast<T*>(q);
  return ADERDG_OK;
}

int nvar(int sys) { return sys == ADERDG_SYS_ADVDIFF ? 1 : sys == ADERDG_SYS_EULER ? 4 : 9; }

int validate(const aderdg_config* c, std::string* why) {
  if (!c) return *why = "null config", ADERDG_EINVAL;
  if (c->system < 0 || c->system > 2) return *why = "unknown system", ADERDG_EINVAL;
  if (c->N < 1 || c->N > 5) return *why = "N must be in 1..5", ADERDG_EUNSUPPORTED;
  if (c->imax < 1 || c->jmax < 1) return *why = "imax and jmax must be >= 1", ADERDG_EINVAL;
  if ((long long)c->imax * c->jmax > (1ll << 31) / 64) return *why = "grid too large", ADERDG_EINVAL;
  if (!(c->xr[0] > c->xl[0]) || !(c->xr[1] > c->xl[1])) return *why = "empty domain", ADERDG_EINVAL;
  if (!(c->cfl > 0.0)) return *why = "cfl must be positive", ADERDG_EINVAL;
  if (c->precision != ADERDG_FP64 && c->precision != ADERDG_FP32_MIXED && c->precision != ADERDG_FP32_WIDE)
    return *why = "bad precision", ADERDG_EINVAL;
  if (c->bc_mode != 0 && !(c->bc_mode == 1 && c->system == ADERDG_SYS_EULER))
    return *why = "bc_mode 1 (double Mach reflection) is Euler only", ADERDG_EINVAL;
  for (int s = 0; s < 4; ++s) {
    if (c->bc[s] < 1 || c->bc[s] > 3) return *why = "boundary codes are 1, 2 or 3", ADERDG_EINVAL;
    if (c->bc[s] == 2 && c->system != ADERDG_SYS_ADVDIFF) return *why = "boundary code 2 is advection-diffusion only", ADERDG_EINVAL;
  }
  if (c->system == ADERDG_SYS_EULER && !(c->gamma > 1.0)) return *why = "gamma must exceed 1", ADERDG_EINVAL;
  if (c->system == ADERDG_SYS_BN && (!(c->gamma_s > 1.0) || !(c->gamma_g > 1.0))) return *why = "gammas must exceed 1", ADERDG_EINVAL;
  return ADERDG_OK;
}

cudaError_t control(aderdg_ctx* c, int mode) {
  aderdg::k_control<<<1, 32, 0, c->stream>>>(c->d_inst, c->d_st, 1, c->args.list_count, mode, -1);
  return cudaGetLastError();
}

const void* pred_ops(aderdg_ctx* c) { return c->fp32 ? c->ops32.data() : c->ops64.data(); }

int push_state(aderdg_ctx* c) {
  CK(c, cudaMemcpyAsync(c->d_st, c->h_st, sizeof(InstState), cudaMemcpyHostToDevice, c->stream));
  return ADERDG_OK;
}
int pull_state(aderdg_ctx* c) {
  CK(c, cudaMemcpyAsync(c->h_st, c->d_st, sizeof(InstState), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return ADERDG_OK;
}
int cur_par(aderdg_ctx* c) { return (int)(c->h_st->steps & 1); }

int cells(aderdg_ctx* c, int mode) {
  c->args.mode = mode;
  CK(c, aderdg::launch_cells(c->kt, c->args, c->ops64.data(), c->prec, c->stream));
  // FP32-mixed: the DMP decisions the FP32 bounds left open
  if (c->args.settle && (mode == aderdg::kCellFused || mode == aderdg::kCellUpdate || mode == aderdg::kCellInitDmp))
    CK(c, c->kt->settle(c->args, c->ops64.data(), c->num_sms, c->stream));
  return ADERDG_OK;
}

// min/max of the current state for the DMP neighbourhood and the CFL
// denominators (get_min_max step 1 + calc_time_step's node loop)
int prime(aderdg_ctx* c) {
  CK(c, control(c, aderdg::kCtlPrimeReset));
  int r = cells(c, aderdg::kCellPrime);
  if (r) return r;
  CK(c, control(c, aderdg::kCtlPrimeCommit));
  return ADERDG_OK;
}

int set_clock(aderdg_ctx* c, double time, double tend) {
  if (c->h_st->time != time || c->h_st->tend != tend) {
    c->h_st->time = time;
    c->h_st->tend = tend;
    c->h_st->nonfinite = 0;
    return push_state(c);
  }
  return ADERDG_OK;
}

// one fused loop body of main.f90
int launch_step(aderdg_ctx* c) {
  CK(c, control(c, aderdg::kCtlBegin));
  CK(c, aderdg::launch_predictor(c->kt, c->args, pred_ops(c), c->prec, c->stream));
  CK(c, aderdg::launch_faces(c->kt, c->args, c->fc, c->prec, c->stream));
  int r = cells(c, aderdg::kCellFused);
  if (r) return r;
  if (c->limiter) {
    CK(c, c->kt->mark(c->args, c->stream));
    CK(c, aderdg::launch_subcell(c->kt, c->args, c->ops64.data(), c->fc, c->subcell_grid, c->num_sms, c->prec, c->stream));
  }
  CK(c, control(c, aderdg::kCtlEnd));
  return ADERDG_OK;
}

void free_all(aderdg_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->flush_buf) cudaFree(c->flush_buf);
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
  if (c->h_st) cudaFreeHost(c->h_st);
  if (c->stream) cudaStreamDestroy(c->stream);
}

int ensure_graph(aderdg_ctx* c) {
  if (c->gexec) return ADERDG_OK;
  cudaGraph_t g = nullptr;
  CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int r = launch_step(c);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (r) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail_cuda(c, "cudaStreamEndCapture", e);
  e = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail_cuda(c, "cudaGraphInstantiate", e);
  return ADERDG_OK;
}

__global__ void k_flush(unsigned int* p, size_t n, unsigned int v) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = v + (unsigned)k;
}

int ensure_phase_buffers(aderdg_ctx* c) {
  if (c->args.qhi) return ADERDG_OK;
  const size_t n = (size_t)c->ncells * c->P * c->P * c->V;
  int r = dalloc(c, &c->args.qhi, n);
  if (!r) r = dalloc(c, &c->args.fhi, 2 * n);
  if (!r && c->cfg.system == ADERDG_SYS_BN) r = dalloc(c, &c->args.shi, n);
  return r;
}

}  // namespace

namespace aderdg {
void set_last_error(const std::string& msg) { g_err = msg; }
int validate_config(const aderdg_config* c, std::string* why) { return validate(c, why); }
// Instance description of a configuration (cell and face bases 0).
InstDesc make_inst_desc(const aderdg_config* cfg) {
  InstDesc in{};
  in.imax = cfg->imax;
  in.jmax = cfg->jmax;
  in.cell_base = in.fx_base = in.fy_base = 0;
  in.dx = (cfg->xr[0] - cfg->xl[0]) / cfg->imax;  // dx = (xR-xL)/VMAX, Euler/initialize.f90:45-46
  in.dy = (cfg->xr[1] - cfg->xl[1]) / cfg->jmax;
  in.idxf = (float)(1.0 / in.dx);
  in.idyf = (float)(1.0 / in.dy);
  in.xl0 = cfg->xl[0];
  in.xl1 = cfg->xl[1];
  for (int s = 0; s < 4; ++s) in.bc[s] = cfg->bc[s];
  in.bc_mode = cfg->bc_mode;
  in.cfl_pnpm = cfg->cfl * pnpm_cfl(cfg->N);
  in.ph.gamma = cfg->gamma;
  in.ph.gs = cfg->gamma_s;
  in.ph.gg = cfg->gamma_g;
  in.ph.ps = cfg->pi_s;
  in.ph.pg = cfg->pi_g;
  in.ph.cx = cfg->cx;
  in.ph.cy = cfg->cy;
  in.ph.a = cfg->a;
  in.ph.ad_fused = cfg->ad_flux_mode;
  for (int k = 0; k < 8; ++k) in.ph.f32c[k] = 0.0f;
  if (cfg->system == ADERDG_SYS_EULER) {
    in.ph.f32c[0] = (float)(cfg->gamma - 1.0);
    in.ph.f32c[1] = (float)cfg->gamma;
  } else if (cfg->system == ADERDG_SYS_BN) {
    const double gs = cfg->gamma_s, gg = cfg->gamma_g, ps = cfg->pi_s, pg = cfg->pi_g;
    const float c[8] = {(float)gs, (float)gg, (float)(gs - 1.0), (float)(gg - 1.0), (float)(gs * ps), (float)(gg * pg),
                        (float)ps, (float)pg};
    for (int k = 0; k < 8; ++k) in.ph.f32c[k] = c[k];
  }
  if (cfg->system == ADERDG_SYS_ADVDIFF) {
    // the expressions of the face kernel and of calc_time_step, evaluated once
    const double pi = 4.0 * std::atan(1.0);
    const double factor = (double)(2 * cfg->N + 1);
    const double eta = factor / (in.dx * std::sqrt(0.5 * pi));
    for (int d = 0; d < 2; ++d) {
      const double nv0 = d == 0 ? 1.0 : 0.0, nv1 = d == 0 ? 0.0 : 1.0;
      const double LL = cfg->cx * nv0 + cfg->cy * nv1, LR = LL;
      const double smax_c = std::fmax(std::fabs(LL), std::fabs(LR));
      const double smax_v = std::fmax(cfg->a, cfg->a);
      in.ad_smax[d] = smax_c + 2.0 * eta * smax_v;
    }
    const double smax_v = std::fabs(cfg->a);
    const double ex = std::fabs(cfg->cx * 1.0 + cfg->cy * 0.0), ey = std::fabs(cfg->cx * 0.0 + cfg->cy * 1.0);
    double denom = 0.0;
    denom = denom + (ex + 2.0 * smax_v * factor / in.dx) / in.dx;
    denom = denom + (ey + 2.0 * smax_v * factor / in.dy) / in.dy;
    in.ad_denom = denom;
  }
  return in;
}

FaceConst make_face_const(const HostOps& ops) {
  const double pi = 4.0 * std::atan(1.0);
  FaceConst fc{};
  fc.Va[0] = 8.0;
  fc.Va[1] = 8.25 * std::cos(pi / 6.0);
  fc.Va[2] = -8.25 * std::sin(pi / 6.0);
  fc.Va[3] = 116.5;
  fc.Vb[0] = 1.4;
  fc.Vb[1] = 0.0;
  fc.Vb[2] = 0.0;
  fc.Vb[3] = 1.0;
  fc.xsw0 = 1.0 / 6.0 + 1.0 / std::tan(pi / 3.0);  // Euler/riemann_problem.f90:1-8
  fc.xsw1 = 10.0 / std::sin(pi / 3.0);
  fc.pi = pi;
  for (int k = 0; k < ops.P && k < 10; ++k) fc.xi[k] = ops.xi[k];
  return fc;
}
}  // namespace aderdg

extern "C" {

const char* aderdg_last_error(aderdg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

int aderdg_create(const aderdg_config* cfg, aderdg_ctx** out) {
  if (!out) return fail(nullptr, ADERDG_EINVAL, "null output pointer");
  *out = nullptr;
  std::string why;
  int r = validate(cfg, &why);
  if (r) return fail(nullptr, r, why);
  const KernelTable* kt = aderdg::kernel_table(cfg->system, cfg->N);
  if (!kt) return fail(nullptr, ADERDG_EUNSUPPORTED, "no kernels built for this (system, N)");
  aderdg_ctx* c = new aderdg_ctx();
  c->cfg = *cfg;
  c->kt = kt;
  c->V = nvar(cfg->system);
  c->P = cfg->N + 1;
  c->S = 2 * cfg->N + 1;
  c->ncells = (long long)cfg->imax * cfg->jmax;
  c->nfx = (long long)(cfg->imax + 1) * cfg->jmax;
  c->nfy = (long long)cfg->imax * (cfg->jmax + 1);
  c->limiter = cfg->limiter != 0 && cfg->system != ADERDG_SYS_ADVDIFF;
  c->fp32 = cfg->precision != ADERDG_FP64;
  c->prec = cfg->precision;
  if (!aderdg::build_ops(cfg->N, c->ops, &why)) {
    delete c;
    return fail(nullptr, ADERDG_EINVAL, why);
  }
  auto bail = [&](int code) {
    free_all(c);
    delete c;
    return code;
  };
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return bail(fail_cuda(nullptr, "cudaGetDevice", e));
  e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) return bail(fail_cuda(nullptr, "cudaDeviceGetAttribute", e));
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(fail_cuda(nullptr, "cudaStreamCreate", e));
  e = cudaMallocHost(&c->h_st, sizeof(InstState));
  if (e != cudaSuccess) return bail(fail(nullptr, ADERDG_ENOMEM, "cudaMallocHost"));
  std::memset(c->h_st, 0, sizeof(InstState));

  const int V = c->V, P = c->P, S = c->S;
  const size_t nc = (size_t)c->ncells, st_elems = nc * P * P * V;
  const size_t rb = c->fp32 ? sizeof(float) : sizeof(double);
  BatchArgs& a = c->args;
  std::memset(&a, 0, sizeof(a));
  r = dalloc(c, &c->d_inst, 1);
  if (!r) r = dalloc(c, &c->d_st, 1);
  if (!r) r = dalloc(c, &a.uh[0], st_elems);
  if (!r) r = dalloc(c, &a.uh[1], st_elems);
  // duh and the face fluxes hold FP32 values in the FP32 modes: half the doubles
  auto stor = [&](size_t n) { return c->fp32 ? (n + 1) / 2 : n; };
  if (!r) r = dalloc(c, &a.duh, stor(st_elems));
  unsigned char *qb = nullptr, *fb = nullptr;
  const size_t nbnd = nc * P * 4 * V;
  if (!r) r = dalloc(c, &qb, nbnd * rb);
  if (!r) r = dalloc(c, &fb, nbnd * rb * (cfg->system == ADERDG_SYS_ADVDIFF ? 2 : 1));
  a.qbnd = qb;
  a.fbnd = fb;
  if (!r) r = dalloc(c, &a.fu, stor((size_t)c->nfx * P * V));
  if (!r) r = dalloc(c, &a.gu, stor((size_t)c->nfy * P * V));
  if (!r && cfg->system == ADERDG_SYS_BN) r = dalloc(c, &a.fp, stor((size_t)c->nfx * P * V));
  if (!r && cfg->system == ADERDG_SYS_BN) r = dalloc(c, &a.gp, stor((size_t)c->nfy * P * V));
  if (!r) r = dalloc(c, &a.list_count, 2);
  if (c->limiter) {
    if (!r) r = dalloc(c, &a.status[0], nc);
    if (!r) r = dalloc(c, &a.status[1], nc);
    if (!r) r = dalloc(c, &a.lh[0], nc * S * S * V);
    if (!r) r = dalloc(c, &a.lh[1], nc * S * S * V);
    if (!r) r = dalloc(c, &a.mm[0], nc * 2 * V);
    if (!r) r = dalloc(c, &a.mm[1], nc * 2 * V);
    if (!r && c->prec == ADERDG_FP32_MIXED) r = dalloc(c, &a.mme[0], nc * V);
    if (!r && c->prec == ADERDG_FP32_MIXED) r = dalloc(c, &a.mme[1], nc * V);
    if (!r && c->prec == ADERDG_FP32_MIXED) r = dalloc(c, &a.settle, nc);
    if (!r) r = dalloc(c, &a.lminmax, nc * 2 * V);
    if (!r) r = dalloc(c, &a.troubled, nc);
    if (!r) r = dalloc(c, &a.recompute, nc);
    if (!r) r = dalloc(c, &a.list, nc);
    if (!r) r = dalloc(c, &a.denom, nc);
  }
  if (r) return bail(r);
  a.inst = c->d_inst;
  a.st = c->d_st;
  a.ninst = 1;
  a.cell0 = 0;
  a.only_inst = -1;
  a.ncells = c->ncells;
  a.nfx = c->nfx;
  a.nfy = c->nfy;

  InstDesc& in = c->h_inst;
  in = aderdg::make_inst_desc(cfg);
  e = cudaMemcpyAsync(c->d_inst, &in, sizeof(InstDesc), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return bail(fail_cuda(nullptr, "cudaMemcpy inst", e));

  c->fc = aderdg::make_face_const(c->ops);

  c->ops64.assign(kt->ops64_size, 0);
  kt->make_ops64(c->ops, c->ops64.data());
  if (c->fp32) {
    c->ops32.assign(kt->ops32_size, 0);
    kt->make_ops32(c->ops, c->ops32.data());
  }
  if (c->limiter) c->subcell_grid = aderdg::subcell_grid_of(kt, c->num_sms, c->prec);
  // set kernel attributes now, outside any later stream capture
  {
    BatchArgs z = a;
    z.ncells = 0;
    z.nfx = z.nfy = 0;
    if (kt->predictor(z, pred_ops(c), c->fp32 ? 1 : 0, false, c->stream) != cudaSuccess ||
        aderdg::launch_predictor(kt, z, pred_ops(c), c->prec, c->stream) != cudaSuccess ||
        aderdg::launch_cells(kt, z, c->ops64.data(), c->prec, c->stream) != cudaSuccess ||
        kt->cells(z, c->ops64.data(), 0, c->stream) != cudaSuccess || kt->cells(z, c->ops64.data(), 1, c->stream) != cudaSuccess)
      return bail(fail(nullptr, ADERDG_ECUDA, "kernel attribute setup failed"));
    if (!c->fp32) kt->predictor(z, pred_ops(c), 0, true, c->stream);
  }
  *out = c;
  return ADERDG_OK;
}

int aderdg_destroy(aderdg_ctx* ctx) {
  if (!ctx) return ADERDG_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  delete ctx;
  return ADERDG_OK;
}

int aderdg_upload(aderdg_ctx* c, const double* uh) {
  if (!c || !uh) return fail(c, ADERDG_EINVAL, "null argument");
  const int par = cur_par(c);
  const size_t n = (size_t)c->ncells * c->P * c->P * c->V;
  CK(c, cudaMemcpyAsync(c->args.uh[par], uh, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->limiter) {
    CK(c, cudaMemsetAsync(c->args.status[0], 0, c->ncells * sizeof(int), c->stream));
    CK(c, cudaMemsetAsync(c->args.status[1], 0, c->ncells * sizeof(int), c->stream));
  }
  c->pending = false;
  int r = prime(c);
  if (r) return r;
  r = pull_state(c);
  if (r) return r;
  c->uploaded = true;
  return ADERDG_OK;
}

int aderdg_init_limiter(aderdg_ctx* c, const double* lh_ic, int* n_limited) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (n_limited) *n_limited = 0;
  if (!c->limiter) return ADERDG_OK;
  double* tmp = nullptr;
  const size_t n = (size_t)c->ncells * c->S * c->S * c->V;
  if (lh_ic) {
    CK(c, cudaMalloc(&tmp, n * sizeof(double)));
    CK(c, cudaMemcpyAsync(tmp, lh_ic, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  c->args.lh_ic = tmp;
  CK(c, control(c, aderdg::kCtlPrimeReset));
  int r = cells(c, aderdg::kCellInitDmp);
  c->args.lh_ic = nullptr;
  if (!r) r = pull_state(c);
  if (tmp) cudaFree(tmp);
  if (r) return r;
  if (n_limited) *n_limited = c->h_st->n_recompute;
  r = prime(c);
  if (!r) r = pull_state(c);
  return r;
}

int aderdg_initial_condition(aderdg_ctx* c, int ic, const double* params, int* n_limited) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (n_limited) *n_limited = 0;
  const int par = cur_par(c);
  // the subcell candidates are formed after the initial DMP, for the cells it
  // limits only, in both Lh buffers
  std::string why;
  cudaError_t e = aderdg::launch_initial_field(c->cfg, ic, params, c->args.uh[par], nullptr, c->stream, &why);
  if (e == cudaErrorInvalidValue && !why.empty()) return fail(c, ADERDG_EINVAL, why);
  if (e != cudaSuccess) return fail_cuda(c, "initial field", e);
  if (c->limiter) {
    CK(c, cudaMemsetAsync(c->args.status[0], 0, c->ncells * sizeof(int), c->stream));
    CK(c, cudaMemsetAsync(c->args.status[1], 0, c->ncells * sizeof(int), c->stream));
  }
  c->pending = false;
  int r = prime(c);
  if (!r) r = pull_state(c);
  if (r) return r;
  c->uploaded = true;
  if (!c->limiter) return ADERDG_OK;
  c->args.lh_ic = nullptr;
  CK(c, control(c, aderdg::kCtlPrimeReset));
  r = cells(c, aderdg::kCellInitDmp);
  if (r) return r;
  e = aderdg::launch_initial_lh(c->cfg, ic, params, c->args.status[0], c->args.lh[0], c->args.lh[1], c->stream, &why);
  if (e != cudaSuccess) return fail_cuda(c, "initial limiter", e);
  r = pull_state(c);
  if (r) return r;
  if (n_limited) *n_limited = c->h_st->n_recompute;
  r = prime(c);
  if (!r) r = pull_state(c);
  return r;
}

int aderdg_cell_averages(aderdg_ctx* c, int primitive, double* out) {
  if (!c || !out) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "no state yet");
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  const size_t n = (size_t)c->ncells * c->V;
  double* tmp = nullptr;
  CK(c, cudaMallocAsync(&tmp, n * sizeof(double), c->stream));
  std::string why;
  cudaError_t e = aderdg::launch_cell_averages(c->cfg, c->args.uh[par], primitive, tmp, c->stream, &why);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(tmp, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail_cuda(c, ("cell averages: " + why).c_str(), e);
  return ADERDG_OK;
}

int aderdg_error_norms(aderdg_ctx* c, int ic, const double* params, int var, double* norms) {
  if (!c || !norms) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "no state yet");
  int r = pull_state(c);
  if (r) return r;
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  double* sums = nullptr;
  CK(c, cudaMallocAsync(&sums, 3 * sizeof(double), c->stream));
  CK(c, cudaMemsetAsync(sums, 0, 3 * sizeof(double), c->stream));
  std::string why;
  cudaError_t e = aderdg::launch_error_norms(c->cfg, c->args.uh[par], ic, params, var, c->h_st->time, sums,
                                             reinterpret_cast<unsigned long long*>(sums + 2), c->stream, &why);
  double h[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(sums, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaErrorInvalidValue && !why.empty()) return fail(c, ADERDG_EINVAL, why);
  if (e != cudaSuccess) return fail_cuda(c, "error norms", e);
  const double ncells = (double)c->ncells;
  norms[0] = h[0] / ncells;             // mean |e| (L1 per cell)
  norms[1] = std::sqrt(h[1] / ncells);  // root mean square
  norms[2] = h[2];                      // max |e| (analyze_soln)
  return ADERDG_OK;
}

int aderdg_upload_limiter(aderdg_ctx* c, const int* status, const double* lh) {
  if (!c || !status || !lh) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->limiter) return ADERDG_OK;
  const int par = cur_par(c);
  CK(c, cudaMemcpyAsync(c->args.status[par], status, c->ncells * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaMemcpyAsync(c->args.lh[par], lh, (size_t)c->ncells * c->S * c->S * c->V * sizeof(double),
                        cudaMemcpyHostToDevice, c->stream));
  int r = prime(c);
  if (!r) r = pull_state(c);
  return r;
}

int aderdg_download_limiter(aderdg_ctx* c, int* status, double* lh) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->limiter) return fail(c, ADERDG_ESTATE, "limiter is off");
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  if (status) CK(c, cudaMemcpyAsync(status, c->args.status[par], c->ncells * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (lh)
    CK(c, cudaMemcpyAsync(lh, c->args.lh[par], (size_t)c->ncells * c->S * c->S * c->V * sizeof(double),
                          cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return ADERDG_OK;
}

int aderdg_download(aderdg_ctx* c, double* uh, int* status) {
  if (!c || !uh) return fail(c, ADERDG_EINVAL, "null argument");
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  CK(c, cudaMemcpyAsync(uh, c->args.uh[par], (size_t)c->ncells * c->P * c->P * c->V * sizeof(double),
                        cudaMemcpyDeviceToHost, c->stream));
  if (status) {
    if (c->limiter)
      CK(c, cudaMemcpyAsync(status, c->args.status[par], c->ncells * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    else
      std::memset(status, 0, c->ncells * sizeof(int));
  }
  CK(c, cudaStreamSynchronize(c->stream));
  return ADERDG_OK;
}

// ------------------------------------------------------------ phase API
int aderdg_calc_time_step(aderdg_ctx* c, double time, double tend, double* dt) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the step (aderdg_limiter) first");
  c->h_st->time = time;
  c->h_st->tend = tend;
  c->h_st->nonfinite = 0;
  int r = push_state(c);
  if (r) return r;
  CK(c, control(c, aderdg::kCtlPrimeReset));
  r = cells(c, aderdg::kCellCfl);
  if (r) return r;
  CK(c, control(c, aderdg::kCtlCalcDt));
  r = pull_state(c);
  if (r) return r;
  if (dt) *dt = c->h_st->dt;
  return ADERDG_OK;
}

int aderdg_set_time_step(aderdg_ctx* c, double time, double dt) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the step first");
  c->h_st->time = time;
  c->h_st->dt = dt;
  c->h_st->active = 1;
  return push_state(c);
}

int aderdg_limiter_prepare(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (!c->limiter) return ADERDG_OK;
  // get_min_max step 1 into the current min/max buffer; the CFL accumulator
  // it also feeds is cleared again by the next calc_time_step
  CK(c, control(c, aderdg::kCtlPrimeReset));
  return cells(c, aderdg::kCellPrime);
}

int aderdg_space_time_predictor(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->fp32) return fail(c, ADERDG_EUNSUPPORTED, "the phase API runs in FP64 only");
  int r = ensure_phase_buffers(c);
  if (r) return r;
  CK(c, c->kt->predictor(c->args, c->ops64.data(), 0, true, c->stream));
  return ADERDG_OK;
}

int aderdg_volume_integral(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->args.fhi) return fail(c, ADERDG_ESTATE, "run aderdg_space_time_predictor first");
  CK(c, c->kt->volume(c->args, c->ops64.data(), c->stream));
  return ADERDG_OK;
}

int aderdg_riemann_problem(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  CK(c, aderdg::launch_faces(c->kt, c->args, c->fc, c->prec, c->stream));
  return ADERDG_OK;
}

int aderdg_surface_integral(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  return cells(c, aderdg::kCellSurface);
}

int aderdg_element_update(aderdg_ctx* c, int* n_recompute) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (c->pending) return fail(c, ADERDG_ESTATE, "element update already applied");
  CK(c, cudaMemsetAsync(&c->d_st->n_recompute, 0, sizeof(int), c->stream));
  CK(c, cudaMemsetAsync(&c->d_st->denom_next, 0, sizeof(unsigned long long), c->stream));
  int r = cells(c, aderdg::kCellUpdate);
  if (r) return r;
  if (!c->limiter) CK(c, control(c, aderdg::kCtlEnd));
  r = pull_state(c);
  if (r) return r;
  c->pending = c->limiter;
  if (n_recompute) *n_recompute = c->h_st->n_recompute;
  return ADERDG_OK;
}

int aderdg_limiter(aderdg_ctx* c) {
  if (!c) return fail(c, ADERDG_EINVAL, "null context");
  if (!c->limiter) return ADERDG_OK;
  if (!c->pending) return fail(c, ADERDG_ESTATE, "run aderdg_element_update first");
  CK(c, cudaMemsetAsync(c->args.list_count, 0, sizeof(int), c->stream));
  CK(c, c->kt->mark(c->args, c->stream));
  CK(c, aderdg::launch_subcell(c->kt, c->args, c->ops64.data(), c->fc, c->subcell_grid, c->num_sms, c->prec, c->stream));
  CK(c, control(c, aderdg::kCtlEnd));
  c->pending = false;
  return pull_state(c);
}

// ------------------------------------------------------------ fused API
int aderdg_step(aderdg_ctx* c, double* time, double tend, double* dt, int* n_recompute) {
  if (!c || !time) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the phase-API step first");
  int r = set_clock(c, *time, tend);
  if (r) return r;
  r = launch_step(c);
  if (r) return r;
  r = pull_state(c);
  if (r) return r;
  *time = c->h_st->time;
  if (dt) *dt = c->h_st->dt;
  if (n_recompute) *n_recompute = c->h_st->n_recompute;
  if (c->h_st->nonfinite) return fail(c, ADERDG_ENONFINITE, "the time step became non-finite");
  return ADERDG_OK;
}

int aderdg_run(aderdg_ctx* c, double* time, double tend, int max_steps, int sync_every, int* steps_done) {
  if (!c || !time) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the phase-API step first");
  if (steps_done) *steps_done = 0;
  if (max_steps <= 0) return ADERDG_OK;
  if (sync_every <= 0) sync_every = 64;
  int r = set_clock(c, *time, tend);
  if (r) return r;
  r = ensure_graph(c);
  if (r) return r;
  const long long steps0 = c->h_st->steps;
  int launched = 0;
  while (launched < max_steps) {
    const int n = std::min(sync_every, max_steps - launched);
    for (int s = 0; s < n; ++s) CK(c, cudaGraphLaunch(c->gexec, c->stream));
    launched += n;
    r = pull_state(c);
    if (r) return r;
    if (c->h_st->nonfinite || !(c->h_st->time < tend)) break;
  }
  *time = c->h_st->time;
  if (steps_done) *steps_done = (int)(c->h_st->steps - steps0);
  if (c->h_st->nonfinite) return fail(c, ADERDG_ENONFINITE, "the time step became non-finite");
  return ADERDG_OK;
}

int aderdg_step_host(aderdg_ctx* c, double* uh, double* time, double tend, double* dt, int* n_recompute) {
  if (!c || !uh || !time) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the phase-API step first");
  const size_t n = (size_t)c->ncells * c->P * c->P * c->V * sizeof(double);
  CK(c, cudaMemcpyAsync(c->args.uh[cur_par(c)], uh, n, cudaMemcpyHostToDevice, c->stream));
  int r = prime(c);
  if (!r) r = set_clock(c, *time, tend);
  if (!r) r = ensure_graph(c);
  if (r) return r;
  CK(c, cudaGraphLaunch(c->gexec, c->stream));
  CK(c, cudaMemcpyAsync(c->h_st, c->d_st, sizeof(InstState), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  CK(c, cudaMemcpyAsync(uh, c->args.uh[cur_par(c)], n, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  *time = c->h_st->time;
  if (dt) *dt = c->h_st->dt;
  if (n_recompute) *n_recompute = c->h_st->n_recompute;
  if (c->h_st->nonfinite) return fail(c, ADERDG_ENONFINITE, "the time step became non-finite");
  return ADERDG_OK;
}

int aderdg_time_steps(aderdg_ctx* c, double* time, double tend, int steps, int flush_l2, double* step_ms) {
  if (!c || !time || !step_ms) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the phase-API step first");
  int r = set_clock(c, *time, tend);
  if (!r) r = ensure_graph(c);
  if (r) return r;
  if (flush_l2 && !c->flush_buf) {
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device);
    c->flush_bytes = (size_t)std::max(l2, 1 << 20) * 2;
    CK(c, cudaMalloc(&c->flush_buf, c->flush_bytes));
  }
  std::vector<cudaEvent_t> ev(2 * (size_t)steps);
  for (auto& e : ev) CK(c, cudaEventCreate(&e));
  CK(c, cudaStreamSynchronize(c->stream));
  for (int s = 0; s < steps; ++s) {
    if (flush_l2) {
      const size_t nw = c->flush_bytes / 4;
      k_flush<<<c->num_sms * 4, 256, 0, c->stream>>>(static_cast<unsigned int*>(c->flush_buf), nw, (unsigned)s);
      CK(c, cudaGetLastError());
    }
    CK(c, cudaEventRecord(ev[2 * s], c->stream));
    CK(c, cudaGraphLaunch(c->gexec, c->stream));
    CK(c, cudaEventRecord(ev[2 * s + 1], c->stream));
  }
  CK(c, cudaStreamSynchronize(c->stream));
  for (int s = 0; s < steps; ++s) {
    float ms = 0.f;
    CK(c, cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]));
    step_ms[s] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  r = pull_state(c);
  if (r) return r;
  *time = c->h_st->time;
  if (c->h_st->nonfinite) return fail(c, ADERDG_ENONFINITE, "the time step became non-finite");
  return ADERDG_OK;
}

int aderdg_profile_step(aderdg_ctx* c, double* time, double tend, double* phase_ms) {
  if (!c || !time || !phase_ms) return fail(c, ADERDG_EINVAL, "null argument");
  if (!c->uploaded) return fail(c, ADERDG_ESTATE, "upload uh first");
  if (c->pending) return fail(c, ADERDG_ESTATE, "finish the phase-API step first");
  int r = set_clock(c, *time, tend);
  if (r) return r;
  cudaEvent_t ev[8];
  for (auto& e : ev) CK(c, cudaEventCreate(&e));
  CK(c, cudaEventRecord(ev[0], c->stream));
  CK(c, control(c, aderdg::kCtlBegin));
  CK(c, cudaEventRecord(ev[1], c->stream));
  CK(c, aderdg::launch_predictor(c->kt, c->args, pred_ops(c), c->prec, c->stream));
  CK(c, cudaEventRecord(ev[2], c->stream));
  CK(c, aderdg::launch_faces(c->kt, c->args, c->fc, c->prec, c->stream));
  CK(c, cudaEventRecord(ev[3], c->stream));
  r = cells(c, aderdg::kCellFused);
  if (r) return r;
  CK(c, cudaEventRecord(ev[4], c->stream));
  if (c->limiter) CK(c, c->kt->mark(c->args, c->stream));
  CK(c, cudaEventRecord(ev[5], c->stream));
  if (c->limiter)
    CK(c, aderdg::launch_subcell(c->kt, c->args, c->ops64.data(), c->fc, c->subcell_grid, c->num_sms, c->prec, c->stream));
  CK(c, cudaEventRecord(ev[6], c->stream));
  CK(c, control(c, aderdg::kCtlEnd));
  CK(c, cudaEventRecord(ev[7], c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 7; ++k) {
    float ms = 0.f;
    CK(c, cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
    phase_ms[k] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  r = pull_state(c);
  if (r) return r;
  *time = c->h_st->time;
  return ADERDG_OK;
}

// ------------------------------------------------------------ introspection
long aderdg_array_size(aderdg_ctx* c, int which) {
  if (!c) return ADERDG_EINVAL;
  const long nc = (long)c->ncells, V = c->V, P = c->P, S = c->S;
  switch (which) {
    case ADERDG_A_UH:
    case ADERDG_A_DUH:
    case ADERDG_A_QHI: return nc * P * P * V;
    case ADERDG_A_FHI: return 2 * nc * P * P * V;
    case ADERDG_A_SHI: return c->cfg.system == ADERDG_SYS_BN ? nc * P * P * V : ADERDG_EINVAL;
    case ADERDG_A_QBND: return nc * P * 4 * V;
    case ADERDG_A_FBND: return c->cfg.system == ADERDG_SYS_ADVDIFF ? ADERDG_EINVAL : nc * P * 4 * V;
    case ADERDG_A_GRADQBND: return c->cfg.system == ADERDG_SYS_ADVDIFF ? nc * P * 4 * 2 * V : ADERDG_EINVAL;
    case ADERDG_A_FU: return (long)c->nfx * P * V;
    case ADERDG_A_GU: return (long)c->nfy * P * V;
    case ADERDG_A_FP: return c->cfg.system == ADERDG_SYS_BN ? (long)c->nfx * P * V : ADERDG_EINVAL;
    case ADERDG_A_GP: return c->cfg.system == ADERDG_SYS_BN ? (long)c->nfy * P * V : ADERDG_EINVAL;
    case ADERDG_A_LH: return c->limiter ? nc * S * S * V : ADERDG_EINVAL;
    case ADERDG_A_LMIN:
    case ADERDG_A_LMAX: return c->limiter ? nc * V : ADERDG_EINVAL;
    case ADERDG_A_RECOMPUTE:
    case ADERDG_A_STATUS: return c->limiter ? nc : ADERDG_EINVAL;
  }
  return ADERDG_EINVAL;
}

namespace {

// The face states are stored face-major on the device ([cell][face][point][e])
// and exchanged in the reference's order qbnd(e, face, point, cell); e runs
// over V values (2 V for gradQbnd).  0 for the other arrays.
int face_state_width(const aderdg_ctx* c, int which) {
  if (which == ADERDG_A_QBND || which == ADERDG_A_FBND) return c->V;
  if (which == ADERDG_A_GRADQBND) return 2 * c->V;
  return 0;
}

void face_order(const double* src, double* dst, long ncells, int P, int E, bool to_reference) {
  for (long cc = 0; cc < ncells; ++cc)
    for (int f = 0; f < 4; ++f)
      for (int l = 0; l < P; ++l) {
        const size_t mine = (((size_t)cc * 4 + f) * P + l) * E, ref = (((size_t)cc * P + l) * 4 + f) * E;
        const double* s = src + (to_reference ? mine : ref);
        double* d = dst + (to_reference ? ref : mine);
        for (int e = 0; e < E; ++e) d[e] = s[e];
      }
}

}  // namespace

int aderdg_get_array(aderdg_ctx* c, int which, void* out) {
  if (!c || !out) return fail(c, ADERDG_EINVAL, "null argument");
  const long n = aderdg_array_size(c, which);
  if (n < 0) return fail(c, ADERDG_EINVAL, "array not available for this configuration");
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  const BatchArgs& a = c->args;
  const void* src = nullptr;
  size_t esz = sizeof(double);
  bool narrow = false;  // FP32 storage (the mixed mode's intermediates) widened to double
  switch (which) {
    case ADERDG_A_UH: src = a.uh[par]; break;
    case ADERDG_A_DUH: src = a.duh; narrow = c->fp32; break;
    case ADERDG_A_QHI: src = a.qhi; break;
    case ADERDG_A_FHI: src = a.fhi; break;
    case ADERDG_A_SHI: src = a.shi; break;
    case ADERDG_A_QBND: src = a.qbnd; narrow = c->fp32; break;
    case ADERDG_A_FBND:
    case ADERDG_A_GRADQBND: src = a.fbnd; narrow = c->fp32; break;
    case ADERDG_A_FU: src = a.fu; narrow = c->fp32; break;
    case ADERDG_A_GU: src = a.gu; narrow = c->fp32; break;
    case ADERDG_A_FP: src = a.fp; narrow = c->fp32; break;
    case ADERDG_A_GP: src = a.gp; narrow = c->fp32; break;
    case ADERDG_A_LH: src = a.lh[par]; break;
    case ADERDG_A_RECOMPUTE: src = a.recompute; esz = sizeof(int); break;
    case ADERDG_A_STATUS: src = a.status[par]; esz = sizeof(int); break;
    case ADERDG_A_LMIN:
    case ADERDG_A_LMAX: {
      std::vector<double> mm((size_t)n * 2);
      CK(c, cudaMemcpyAsync(mm.data(), a.lminmax, mm.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      CK(c, cudaStreamSynchronize(c->stream));
      const int V = c->V, off = which == ADERDG_A_LMIN ? 0 : V;
      double* o = static_cast<double*>(out);
      for (long cc = 0; cc < (long)c->ncells; ++cc)
        for (int v = 0; v < V; ++v) o[cc * V + v] = mm[(size_t)cc * 2 * V + off + v];
      return ADERDG_OK;
    }
  }
  if (!src) return fail(c, ADERDG_ESTATE, "array not computed yet");
  if (narrow) {
    std::vector<float> tmp((size_t)n);
    CK(c, cudaMemcpyAsync(tmp.data(), src, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    double* o = static_cast<double*>(out);
    for (long k = 0; k < n; ++k) o[k] = (double)tmp[k];
  } else {
    CK(c, cudaMemcpyAsync(out, src, n * esz, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  if (const int E = face_state_width(c, which)) {
    double* o = static_cast<double*>(out);
    std::vector<double> mine(o, o + n);
    face_order(mine.data(), o, (long)c->ncells, c->P, E, true);
  }
  return ADERDG_OK;
}

int aderdg_set_array(aderdg_ctx* c, int which, const void* in) {
  if (!c || !in) return fail(c, ADERDG_EINVAL, "null argument");
  const long n = aderdg_array_size(c, which);
  if (n < 0) return fail(c, ADERDG_EINVAL, "array not available for this configuration");
  const int par = cur_par(c) ^ (c->pending ? 1 : 0);
  BatchArgs& a = c->args;
  void* dst = nullptr;
  size_t esz = sizeof(double);
  bool narrow = false;
  switch (which) {
    case ADERDG_A_UH: dst = a.uh[par]; break;
    case ADERDG_A_DUH: dst = a.duh; narrow = c->fp32; break;
    case ADERDG_A_QHI: dst = a.qhi; break;
    case ADERDG_A_FHI: dst = a.fhi; break;
    case ADERDG_A_SHI: dst = a.shi; break;
    case ADERDG_A_QBND: dst = a.qbnd; narrow = c->fp32; break;
    case ADERDG_A_FBND:
    case ADERDG_A_GRADQBND: dst = a.fbnd; narrow = c->fp32; break;
    case ADERDG_A_FU: dst = a.fu; narrow = c->fp32; break;
    case ADERDG_A_GU: dst = a.gu; narrow = c->fp32; break;
    case ADERDG_A_FP: dst = a.fp; narrow = c->fp32; break;
    case ADERDG_A_GP: dst = a.gp; narrow = c->fp32; break;
    case ADERDG_A_LH: dst = a.lh[par]; break;
    case ADERDG_A_RECOMPUTE: dst = a.recompute; esz = sizeof(int); break;
    case ADERDG_A_STATUS: dst = a.status[par]; esz = sizeof(int); break;
    default: return fail(c, ADERDG_EINVAL, "array is read-only");
  }
  if (!dst) return fail(c, ADERDG_ESTATE, "array not allocated yet");
  std::vector<double> mine;
  if (const int E = face_state_width(c, which)) {
    mine.resize((size_t)n);
    face_order(static_cast<const double*>(in), mine.data(), (long)c->ncells, c->P, E, false);
    in = mine.data();
  }
  if (narrow) {
    std::vector<float> tmp((size_t)n);
    const double* s = static_cast<const double*>(in);
    for (long k = 0; k < n; ++k) tmp[k] = (float)s[k];
    CK(c, cudaMemcpyAsync(dst, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return ADERDG_OK;
  }
  CK(c, cudaMemcpyAsync(dst, in, n * esz, cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return ADERDG_OK;
}

int aderdg_get_info(aderdg_ctx* c, aderdg_info* info) {
  if (!c || !info) return fail(c, ADERDG_EINVAL, "null argument");
  int r = pull_state(c);
  if (r) return r;
  info->cells = (long)c->ncells;
  info->dofs = (long)c->ncells * c->P * c->P * c->V;
  info->device_bytes = (long)c->bytes;
  info->steps = (long)c->h_st->steps;
  info->time = c->h_st->time;
  info->dt = c->h_st->dt;
  info->n_recompute = c->h_st->n_recompute;
  info->n_settled = c->h_st->n_settled;
  info->n_listed = c->h_st->n_list;
  info->n_limited = 0;
  if (c->limiter) {
    std::vector<int> st((size_t)c->ncells);
    const int par = cur_par(c) ^ (c->pending ? 1 : 0);
    CK(c, cudaMemcpyAsync(st.data(), c->args.status[par], st.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    for (int s : st) info->n_limited += s != 0;
  }
  return ADERDG_OK;
}

}  // extern "C"
