// api.cu -- host implementation of the C ABI declared in include/gbnde.h.
//
// A context owns the parameters (flat ComponentArray order plus a transposed
// copy for the VJPs), one CUDA stream and the device workspace of the last
// forward solve (stage buffers, saved states, checkpoints, step log), which
// gbnde_backward consumes. Buffers grow on demand and are reused.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <vector>

#include "gbnde.h"
#include "kernels.h"
#include "tc_args.h"

namespace gbnde {
int launch_reduce_mu(const float* mu_acc, int nblk, int P, float* out, cudaStream_t st);
struct MsSeg {
  double t0, t1;
  int save_off, nsave;
};
struct MsArgs {
  MlpDev mlp;
  int S, nseg, TM, LD, ntiles;
  double abstol, reltol;
  long long maxiters;
  int MS;
  const MsSeg* segs;
  const double* saveat;
  const float* u0;
  float* usave;
  float* dense;
  double* steplog;
  int* nacc;
  int* retcode;
  long long* counters;
  const float* dLdu;
  float* dLdu0;
  float* bar;
  float* mu_acc;
  int P;
};
int launch_ms_fwd(const MsArgs& a, int grid, size_t smem, cudaStream_t st);
int launch_ms_bwd(const MsArgs& a, int grid, size_t smem, cudaStream_t st);

int launch_transpose_params(const MlpDev& m, const float* p, float* wtr, cudaStream_t st);
int launch_loss(const float* usave, const float* target, size_t n, int kind, float* dL,
                double* partial, int nblk, cudaStream_t st);
int launch_adam(float* p, float* m, float* v, const float* g, size_t n, double lr, double b1, double b2,
                double eps, long long step, cudaStream_t st);
int launch_plan_intervals(Interval* iv, int niv, const double* steplog, const long long* fcounters,
                          const int* fstatus, long long dense_slots, long long maxsteps, int* flags,
                          cudaStream_t st);
int launch_ms_loss(const float* u, const float* d, const int* colseg, const int* segoff, const int* segn,
                   const int* nxt, int S, int ncol, int kind, double cont, float* dL, double* part, int nblk,
                   cudaStream_t st);
int launch_loss_finalize(const double* part, int nblk, size_t n, int kind, double* out, cudaStream_t st);
int launch_adam_graph(float* p, float* m, float* v, const float* g, size_t n, double lr, double b1, double b2,
                      double eps, const double* coef, const int* flags, const int* bstatus, cudaStream_t st);

// Launches of one eager training step, recorded for the graph-mode step,
// which replays them inside one captured CUDA graph.
struct StepRecord {
  bool fwd = false, bwd = false, loss = false, tc = false, bwd_tc_on = false;
  bool wide = false;  // the tensor-core kernels ran in stash mode (fwd_tcw / bwd_tcw)
  FwdTcwArgs fwd_tcw{};
  FwdTcArgs fwd_tc{};
  FwdArgs fwd_f32{};
  int fwd_grid = 0;
  size_t fwd_smem = 0;
  BwdTcArgs bwd_tc{};
  BwdArgs bwd_f32{};
  int bwd_grid = 0;
  size_t bwd_smem = 0;
  int red_stride = 0;  // tensor-core form: per-CTA mu slot stride
  float* dp = nullptr;
  const float* l_us = nullptr;
  const float* l_tg = nullptr;
  size_t l_n = 0;
  int l_kind = 0;
  float* l_dl = nullptr;
  double* l_part = nullptr;
  int l_nblk = 0;
};
}  // namespace gbnde

using namespace gbnde;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess)                                                               \
      return fail(GBNDE_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), \
                  __FILE__, __LINE__);                                                   \
  } while (0)

struct DBuf {
  void* p = nullptr;
  size_t n = 0;
  int ensure(size_t bytes) {
    if (bytes <= n) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(GBNDE_ERR_NOMEM, "cudaMalloc(%zu) failed", bytes);
    }
    n = bytes;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

}  // namespace

struct gbnde_ctx {
  int device = 0;
  int precision = GBNDE_PREC_FP32;
  gbnde_mlp_desc desc{};
  size_t P = 0;
  int S = 0;  // state dimension
  cudaStream_t stream = nullptr;
  MlpDev mlp{};
  DBuf params, wtr;
  bool have_params = false;
  // forward workspace
  DBuf u0, ubuf, kbuf, usave, ckpt, ckpt_step, steplog, trace, partials, sync, counters, saveat_d, bnd_d;
  // backward workspace
  DBuf dldu, dldu0, dldp, lam, ub, kl, ku, ibuf, mu_acc, mu_stage, iv_d, bsync, bcounters, loss_part;
  // last forward
  bool have_fwd = false;
  int B = 0, nsave = 0;
  double t0 = 0, t1 = 0, abstol = 0, reltol = 0;
  long long maxiters = 0;
  int sensealg = 0;
  std::vector<double> saveat;
  std::vector<double> steps;  // 2*naccept
  std::vector<int> ckstep;
  long long naccept = 0;
  long long nattempt = 0;
  long long last_naccept = 0;
  bool rerun_guard = false;
  int final_cur = 0;
  bool dense_tl = false;  // the last forward kept its dense slots in the tile layout (BF16 form)
  int fwd_retcode = 0;
  const float* usave_dev = nullptr;  // saved states of the last forward (device)
  cudaStream_t own_stream = nullptr;
  // tensor-core form: split-BF16 weight images per layer
  DBuf wimg;
  size_t wimg_off[GBNDE_MAX_LAYERS] = {};
  int npad[GBNDE_MAX_LAYERS] = {}, nchunk[GBNDE_MAX_LAYERS] = {};
  size_t wtimg_off[GBNDE_MAX_LAYERS] = {};
  int npadT[GBNDE_MAX_LAYERS] = {}, nchunkT[GBNDE_MAX_LAYERS] = {};
  bool tc_shape_ok = false;
  bool tc_bwd_ok = false;  // tensor-core adjoint covers this model
  // stash mode (fwd_tcw / bwd_tcw): state up to 256, widths up to 1024, time
  // row; weight images per 256-row N-block of each layer (W and W^T)
  bool tc_wide = false, tc_wide_bwd = false;
  bool fwd_wide = false;  // the last forward ran on the stash engine (its adjoint follows)
  bool ffj_tc_ok = false; // FFJORD (Hutchinson trace) on the stash engine: d + 1 <= 64, identity output
  DBuf ttrs;              // FFJORD on the stash engine: per-CTA row scratch
  int force_wide = -1;    // autotuner: -1 tuned/default, 0 single-accumulator, 1 stash engine
  std::map<std::pair<int, int>, int> tuned_tc;  // (S, B) -> 1: stash engine measured faster
  int nsc = 1;  // 64-component chunks of the state in the tensor-core kernels
  size_t wb_off[GBNDE_MAX_LAYERS][4] = {}, wbT_off[GBNDE_MAX_LAYERS][4] = {};
  int wb_npad[GBNDE_MAX_LAYERS][4] = {}, wbT_npad[GBNDE_MAX_LAYERS][4] = {};
  DBuf stash;
  DBuf timg, thscr, tmucomp, tlamcomp, txst;
  size_t timg_cleared = 0;  // bytes of timg set to zero since its allocation
  DBuf tr_us, tr_dl, tr_du0, tr_dp;  // training-step scratch
  // graph-mode training step
  bool recording = false;
  StepRecord rec;
  cudaGraphExec_t gexec = nullptr;
  std::vector<char> gkey;   // the arguments the graph was captured for
  DBuf gstat;               // device: loss (double), Adam coefficients (2 doubles), flags (ints)
  double* gpin = nullptr;   // pinned host mirror of the Adam coefficients
  bool graph_failed = false;
  int f32time = 0;  // Float32 time of the last forward solve (its adjoint follows)
  // autotuner (FP32 kernels): rows per tile chosen by timing, per (S, B)
  int tm_force_fwd = 0, tm_force_bwd = 0;
  std::map<std::pair<int, int>, std::pair<int, int>> tuned;
  // multiple shooting workspace
  DBuf ms_segs, ms_saveat, ms_u0, ms_usave, ms_dense, ms_steplog, ms_nacc, ms_ret, ms_cnt, ms_dldu,
      ms_dldu0, ms_bar, ms_mu, ms_dldp;
  bool ms_have = false;
  bool ms_saves = false;  // ms_usave holds the saves of the last multishoot forward
  // multiple-shooting loss on the device: the data, the column/segment maps
  // and the per-block partials; ms_dl_ok: ms_dldu holds the last loss's cotangent
  DBuf ms_data, ms_map, ms_part;
  std::vector<gbnde_segment> ms_hsegs;
  bool ms_dl_ok = false;
  // FFJORD
  DBuf ffnoise, ffu0, ffus;
  int fS = 0;          // state dim of the last forward (d + 1 for FFJORD)
  int ff_on = 0, ff_d = 0, ff_exact = 0;
  int ff_reg = 0;      // FFJORD with the |f|^2 and |e^T J| rows
  int ff_reg_g2 = 0;   // the |e^T J| row's cotangent is nonzero (set by the backward)
  int ms_S = 0, ms_nseg = 0, ms_nsave = 0, ms_MS = 0;
  // dense stage storage of the last forward
  DBuf comp, dense;
  long long dense_slots = 0;
  bool dense_valid = false;
  size_t stage_cap = 0;  // gbnde_set_stage_memory: bytes the dense stage storage may take (0: a quarter of free)
  int grid_cap = 0;      // gbnde_set_grid_cap: CTAs of the tensor-core kernels (0: one per SM)
  DBuf ckcomp, trep;     // tensor-core form: compensation at the checkpoints; replay state of the adjoint
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double fwd_ms = 0.0, bwd_ms = 0.0;
};

namespace {
// The weight-gradient images' padding rows and blocks are never written (the
// products that read them land in accumulator rows and columns that are not
// stored), so the image buffer is set to zero once per allocation rather than
// at every adjoint launch.
int clear_images(gbnde_ctx* c) {
  if (c->timg_cleared == c->timg.n) return 0;
  if (cudaMemsetAsync(c->timg.p, 0, c->timg.n, c->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(GBNDE_ERR_CUDA, "clearing the weight-gradient images failed");
  }
  c->timg_cleared = c->timg.n;
  return 0;
}
}  // namespace

namespace {

// CTAs for ntiles tiles on at most gmax CTAs: the fewest that keep the number
// of tile rounds (a CTA loops over its tiles), so that no CTA idles in the
// last round and the others contend less for L2 (FFJORD, B = 65536: 512 tiles
// on 128 CTAs in 61.3 ms against 64.0 ms on 152).
int balanced_grid(int ntiles, int gmax) {
  const int rounds = (ntiles + gmax - 1) / gmax;
  return (ntiles + rounds - 1) / rounds;
}

int set_device(gbnde_ctx* c) {
  CK(cudaSetDevice(c->device));
  return 0;
}

int choose_tm(int maxdim_rows_total, size_t budget, int* TM) {
  // rows_total feature rows of TM+4 floats must fit the budget
  for (int tm = 64; tm >= 8; tm /= 2) {
    if ((size_t)maxdim_rows_total * (tm + 4) * sizeof(float) <= budget) {
      *TM = tm;
      return 0;
    }
  }
  return -1;
}

// dynamic shared memory of the FP32 kernels: the 227 KB a CTA may hold, less
// 1 KB for their static reduction arrays
constexpr size_t kSmemBudget = 227 * 1024 - 1024;
// the packed multiple-shooting kernels hold more static shared memory
constexpr size_t kSmemBudgetMs = 200 * 1024;

}  // namespace

extern "C" {

const char* gbnde_strerror(int code) {
  switch (code) {
    case GBNDE_OK: return "ok";
    case GBNDE_ERR_INVALID: return "invalid argument";
    case GBNDE_ERR_CUDA: return "CUDA error";
    case GBNDE_ERR_NOMEM: return "out of memory";
    case GBNDE_ERR_UNSUPPORTED: return "unsupported";
    case GBNDE_ERR_STATE: return "invalid call order";
    case GBNDE_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown error";
  }
}

const char* gbnde_last_error(void) { return g_last_error.c_str(); }

int gbnde_create(gbnde_ctx** out, const gbnde_mlp_desc* mlp, int precision, int device) {
  if (!out || !mlp) return fail(GBNDE_ERR_INVALID, "null argument");
  *out = nullptr;
  if (mlp->nlayers < 1 || mlp->nlayers > GBNDE_MAX_LAYERS)
    return fail(GBNDE_ERR_INVALID, "nlayers must be in [1, %d]", GBNDE_MAX_LAYERS);
  for (int l = 0; l <= mlp->nlayers; ++l)
    if (mlp->dims[l] < 1 || mlp->dims[l] > 4096)
      return fail(GBNDE_ERR_INVALID, "dims[%d] = %d out of range", l, mlp->dims[l]);
  for (int l = 0; l < mlp->nlayers; ++l)
    if (mlp->act[l] < GBNDE_ACT_IDENTITY || mlp->act[l] > GBNDE_ACT_SOFTPLUS)
      return fail(GBNDE_ERR_INVALID, "act[%d] = %d unknown", l, mlp->act[l]);
  const int S = mlp->dims[0] - (mlp->time_input ? 1 : 0);
  if (S < 1 || mlp->dims[mlp->nlayers] != S)
    return fail(GBNDE_ERR_INVALID, "output dim %d must equal state dim %d", mlp->dims[mlp->nlayers], S);
  if (precision != GBNDE_PREC_FP32 && precision != GBNDE_PREC_BF16)
    return fail(GBNDE_ERR_INVALID, "unknown precision %d", precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(GBNDE_ERR_CUDA, "no CUDA device available");
  }
  if (device < 0 || device >= ndev) return fail(GBNDE_ERR_INVALID, "device %d out of range", device);
  gbnde_ctx* c = new gbnde_ctx();
  c->device = device;
  c->precision = precision;
  c->desc = *mlp;
  c->S = S;
  if (int r = set_device(c)) {
    delete c;
    return r;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(GBNDE_ERR_CUDA, "cudaStreamCreate failed");
  }
  c->own_stream = c->stream;
  for (auto& e : c->ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete c;
      return fail(GBNDE_ERR_CUDA, "cudaEventCreate failed");
    }
  }
  size_t off = 0;
  MlpDev& m = c->mlp;
  m.nlayers = mlp->nlayers;
  m.cube = mlp->cube_input;
  m.timein = mlp->time_input;
  m.maxdim = 0;
  for (int l = 0; l <= mlp->nlayers; ++l) {
    m.dims[l] = mlp->dims[l];
    m.maxdim = std::max(m.maxdim, mlp->dims[l]);
  }
  for (int l = 0; l < mlp->nlayers; ++l) {
    m.act[l] = mlp->act[l];
    m.woff[l] = (long long)off;
    off += (size_t)mlp->dims[l] * mlp->dims[l + 1];
    m.boff[l] = (long long)off;
    off += (size_t)mlp->dims[l + 1];
  }
  c->P = off;
  // shapes the tensor-core engine covers: state <= 64, hidden widths <= 256
  c->tc_shape_ok = !mlp->time_input && S <= 64 && mlp->dims[0] <= 64;
  for (int l = 1; l < mlp->nlayers; ++l) c->tc_shape_ok = c->tc_shape_ok && mlp->dims[l] <= 256;
  // the tensor-core adjoint also needs an identity output layer and <= 256 on
  // the N side of every weight-gradient product
  c->tc_bwd_ok = c->tc_shape_ok && mlp->act[mlp->nlayers - 1] == GBNDE_ACT_IDENTITY;
  for (int l = 0; l < mlp->nlayers; ++l)
    c->tc_bwd_ok = c->tc_bwd_ok && std::min(mlp->dims[l], mlp->dims[l + 1]) <= 256;
  // beyond that, stash mode: state <= 256, every width <= 1024 (16 K-chunks,
  // 4 N-blocks), no cube prefix; its adjoint needs an identity output layer
  // (tc_wide: the stash engine covers the model; shapes the single-accumulator
  // engine covers too run on it unless the autotuner measured the stash engine faster)
  if (precision == GBNDE_PREC_BF16) {
    bool w = S <= 256 && !mlp->cube_input;
    for (int l = 0; l <= mlp->nlayers; ++l) w = w && mlp->dims[l] <= 1024;
    c->tc_wide = w;
    c->tc_wide_bwd = w && mlp->act[mlp->nlayers - 1] == GBNDE_ACT_IDENTITY;
    c->nsc = (S + 63) / 64;
    c->ffj_tc_ok = c->tc_wide_bwd && S + 1 <= 64;
  }
  if (precision == GBNDE_PREC_BF16 && !c->tc_shape_ok && !c->tc_wide) {
    gbnde_destroy(c);
    return fail(GBNDE_ERR_UNSUPPORTED,
                "BF16 form supports state dim <= 256 and widths <= 1024 (no cube prefix beyond state 64 / "
                "width 256)");
  }
  *out = c;
  return 0;
}

void gbnde_destroy(gbnde_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  DBuf* bufs[] = {&c->params, &c->wtr, &c->u0, &c->ubuf, &c->kbuf, &c->usave, &c->ckpt,
                  &c->ckpt_step, &c->steplog, &c->trace, &c->partials, &c->sync, &c->counters, &c->saveat_d,
                  &c->bnd_d, &c->dldu, &c->dldu0, &c->dldp, &c->lam, &c->ub, &c->kl, &c->ku,
                  &c->ibuf, &c->mu_acc, &c->mu_stage, &c->iv_d, &c->bsync, &c->bcounters,
                  &c->loss_part, &c->wimg, &c->comp, &c->dense, &c->timg, &c->thscr,
                  &c->tmucomp, &c->tlamcomp, &c->ms_segs, &c->ms_saveat, &c->ms_u0,
                  &c->ms_usave, &c->ms_dense, &c->ms_steplog, &c->ms_nacc, &c->ms_ret, &c->ms_cnt,
                  &c->ms_dldu, &c->ms_dldu0, &c->ms_bar, &c->ms_mu, &c->ms_dldp, &c->ffnoise,
                  &c->ffu0, &c->ffus, &c->tr_us, &c->tr_dl, &c->tr_du0, &c->tr_dp, &c->stash,
                  &c->ms_data, &c->ms_map, &c->ms_part, &c->ckcomp, &c->trep, &c->txst};
  for (DBuf* b : bufs) b->release();
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->gpin) cudaFreeHost(c->gpin);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

size_t gbnde_nparams(const gbnde_ctx* c) { return c ? c->P : 0; }

static int bind_params(gbnde_ctx* c) {
  MlpDev& m = c->mlp;
  const float* p = c->params.as<float>();
  size_t toff = 0;
  for (int l = 0; l < m.nlayers; ++l) {
    m.Wt[l] = p + m.woff[l];
    m.bias[l] = p + m.boff[l];
    m.W[l] = c->wtr.as<float>() + toff;
    toff += (size_t)m.dims[l] * m.dims[l + 1];
  }
  if (launch_transpose_params(m, p, c->wtr.as<float>(), c->stream))
    return fail(GBNDE_ERR_CUDA, "transpose kernel launch failed");
  if (c->precision == GBNDE_PREC_BF16 && c->tc_wide) {
    // per 256-row N-block: W rows [256 b, ...) of layer l (forward), W^T rows
    // (input features) [256 b, ...) (VJP)
    for (int l = 0; l < m.nlayers; ++l) {
      const int in = m.dims[l], out = m.dims[l + 1];
      for (int b = 0; b * 256 < out; ++b)
        if (launch_prep_weight_image(m.W[l] + (size_t)256 * b * in, std::min(256, out - 256 * b), in,
                                     c->wb_npad[l][b], c->wimg.as<uint8_t>() + c->wb_off[l][b], c->stream))
          return fail(GBNDE_ERR_CUDA, "weight image kernel launch failed");
      for (int b = 0; b * 256 < in; ++b)
        if (launch_prep_weight_image(m.Wt[l] + (size_t)256 * b * out, std::min(256, in - 256 * b), out,
                                     c->wbT_npad[l][b], c->wimg.as<uint8_t>() + c->wbT_off[l][b], c->stream))
          return fail(GBNDE_ERR_CUDA, "weight image kernel launch failed");
    }
  }
  if (c->precision == GBNDE_PREC_BF16 && c->tc_shape_ok) {
    for (int l = 0; l < m.nlayers; ++l) {
      if (launch_prep_weight_image(m.W[l], m.dims[l + 1], m.dims[l], c->npad[l],
                                   c->wimg.as<uint8_t>() + c->wimg_off[l], c->stream))
        return fail(GBNDE_ERR_CUDA, "weight image kernel launch failed");
      if (launch_prep_weight_image(m.Wt[l], m.dims[l], m.dims[l + 1], c->npadT[l],
                                   c->wimg.as<uint8_t>() + c->wtimg_off[l], c->stream))
        return fail(GBNDE_ERR_CUDA, "weight image kernel launch failed");
    }
  }
  c->have_params = true;
  return 0;
}

static int alloc_params(gbnde_ctx* c) {
  if (int r = c->params.ensure(c->P * sizeof(float))) return r;
  if (int r = c->wtr.ensure(c->P * sizeof(float))) return r;
  // one image buffer: the single-accumulator engine's images, then the stash
  // engine's per-N-block images (both where both engines cover the model)
  size_t off = 0;
  if (c->precision == GBNDE_PREC_BF16 && c->tc_shape_ok) {
    for (int l = 0; l < c->mlp.nlayers; ++l) {
      c->npad[l] = (c->mlp.dims[l + 1] + 15) / 16 * 16;
      c->nchunk[l] = (c->mlp.dims[l] + 63) / 64;
      c->wimg_off[l] = off;
      off += (size_t)c->nchunk[l] * 2 * c->npad[l] * 128;
    }
    // transposed weights W^T (N = in, K = out) for the VJP chain
    for (int l = 0; l < c->mlp.nlayers; ++l) {
      c->npadT[l] = (c->mlp.dims[l] + 15) / 16 * 16;
      c->nchunkT[l] = (c->mlp.dims[l + 1] + 63) / 64;
      c->wtimg_off[l] = off;
      off += (size_t)c->nchunkT[l] * 2 * c->npadT[l] * 128;
    }
  }
  if (c->precision == GBNDE_PREC_BF16 && c->tc_wide) {
    for (int l = 0; l < c->mlp.nlayers; ++l) {
      const int in = c->mlp.dims[l], out = c->mlp.dims[l + 1];
      for (int b = 0; b * 256 < out; ++b) {
        c->wb_npad[l][b] = (std::min(256, out - 256 * b) + 15) / 16 * 16;
        c->wb_off[l][b] = off;
        off += (size_t)((in + 63) / 64) * 2 * c->wb_npad[l][b] * 128;
      }
      for (int b = 0; b * 256 < in; ++b) {
        c->wbT_npad[l][b] = (std::min(256, in - 256 * b) + 15) / 16 * 16;
        c->wbT_off[l][b] = off;
        off += (size_t)((out + 63) / 64) * 2 * c->wbT_npad[l][b] * 128;
      }
    }
  }
  if (off)
    if (int r = c->wimg.ensure(off)) return r;
  return 0;
}

int gbnde_set_stage_memory(gbnde_ctx* c, size_t max_bytes) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  c->stage_cap = max_bytes;
  return 0;
}

int gbnde_set_grid_cap(gbnde_ctx* c, int max_ctas) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  if (max_ctas < 0) return fail(GBNDE_ERR_INVALID, "grid cap %d < 0", max_ctas);
  c->grid_cap = max_ctas;
  return 0;
}

int gbnde_set_params(gbnde_ctx* c, const float* p, size_t n) {
  if (!c || !p) return fail(GBNDE_ERR_INVALID, "null argument");
  if (n != c->P) return fail(GBNDE_ERR_INVALID, "expected %zu parameters, got %zu", c->P, n);
  if (int r = set_device(c)) return r;
  if (int r = alloc_params(c)) return r;
  CK(cudaMemcpyAsync(c->params.p, p, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  return bind_params(c);
}

int gbnde_set_params_device(gbnde_ctx* c, const float* p, size_t n) {
  if (!c || !p) return fail(GBNDE_ERR_INVALID, "null argument");
  if (n != c->P) return fail(GBNDE_ERR_INVALID, "expected %zu parameters, got %zu", c->P, n);
  if (int r = set_device(c)) return r;
  if (int r = alloc_params(c)) return r;
  CK(cudaMemcpyAsync(c->params.p, p, n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
  return bind_params(c);
}

static int validate_desc(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B) {
  if (!d) return fail(GBNDE_ERR_INVALID, "null solve descriptor");
  if (S != c->S + (c->ff_on ? (c->ff_reg ? 3 : 1) : 0))
    return fail(GBNDE_ERR_INVALID, "state dim %d does not match the model (%d)", S, c->S);
  if (B < 1) return fail(GBNDE_ERR_INVALID, "batch must be >= 1");
  if (!(d->t1 != d->t0)) return fail(GBNDE_ERR_INVALID, "tspan must satisfy t1 != t0");
  if (!(d->abstol > 0) || !(d->reltol >= 0)) return fail(GBNDE_ERR_INVALID, "tolerances must be positive");
  if (d->nsave < 1 || !d->saveat) return fail(GBNDE_ERR_INVALID, "saveat must hold >= 1 time");
  const double tdir = d->t1 > d->t0 ? 1.0 : -1.0;
  for (int i = 0; i < d->nsave; ++i) {
    const double s = d->saveat[i];
    if (!(tdir * (s - d->t0) >= 0 && tdir * (d->t1 - s) >= 0))
      return fail(GBNDE_ERR_INVALID, "saveat[%d] = %g outside tspan", i, s);
    if (i > 0 && tdir * (s - d->saveat[i - 1]) < 0)
      return fail(GBNDE_ERR_INVALID, "saveat must be ordered from t0 to t1");
  }
  if (tdir < 0 && c->precision == GBNDE_PREC_BF16 && !c->ff_on)
    return fail(GBNDE_ERR_UNSUPPORTED, "reverse time spans run in the FP32 form");
  if (d->sensealg != GBNDE_SENSE_INTERPOLATING && d->sensealg != GBNDE_SENSE_BACKSOLVE &&
      d->sensealg != GBNDE_SENSE_GAUSS)
    return fail(GBNDE_ERR_INVALID, "unknown sensealg %d", d->sensealg);
  if ((long long)B * S > (1LL << 31)) return fail(GBNDE_ERR_UNSUPPORTED, "S*B too large");
  if (d->flags & ~GBNDE_FLAG_FP32_TIME) return fail(GBNDE_ERR_INVALID, "unknown flags 0x%x", d->flags);
  if ((d->flags & GBNDE_FLAG_FP32_TIME) && c->precision != GBNDE_PREC_FP32)
    return fail(GBNDE_ERR_UNSUPPORTED, "Float32 time is a mode of the FP32 form");
  return 0;
}

static int forward_impl(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0,
                        bool u0_host, float* usave, bool usave_host, gbnde_stats* stats) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  if (!c->have_params) return fail(GBNDE_ERR_STATE, "parameters not set");
  if (int r = validate_desc(c, d, S, B)) return r;
  if (int r = set_device(c)) return r;
  if (c->precision != GBNDE_PREC_FP32 && c->precision != GBNDE_PREC_BF16)
    return fail(GBNDE_ERR_UNSUPPORTED, "precision");
  c->have_fwd = false;
  const size_t SB = (size_t)S * B;
  const int nsave = d->nsave;
  const long long maxiters = d->maxiters > 0 ? d->maxiters : 100000;
  // checkpoint boundaries: t0 and every save point but the last
  std::vector<double> bnd;
  bnd.push_back(d->t0);
  for (int i = 0; i + 1 < nsave; ++i)
    if (d->saveat[i] > d->t0) bnd.push_back(d->saveat[i]);
  const int nb = (int)bnd.size();

  int sumdims = 0;
  for (int l = 0; l <= c->mlp.nlayers; ++l) sumdims += c->mlp.dims[l];
  const int frows = c->ff_on ? 2 * sumdims + c->mlp.maxdim + 1 + (c->ff_reg ? c->mlp.maxdim + 2 : 0)
                             : 2 * c->mlp.maxdim;
  int TM = 0;
  if (choose_tm(frows, kSmemBudget, &TM)) return fail(GBNDE_ERR_UNSUPPORTED, "layer too wide");
  while (TM > 8 && TM / 2 >= B) TM /= 2;  // small batches: no tile rows past the batch
  {
    int want = c->tm_force_fwd;
    auto it = c->tuned.find({S, B});
    if (!want && it != c->tuned.end()) want = it->second.first;
    if (want > 0 && (size_t)frows * (want + 4) * sizeof(float) <= kSmemBudget) TM = want;
    else if (c->tm_force_fwd) return fail(GBNDE_ERR_UNSUPPORTED, "%d tile rows do not fit", want);
  }
  const int LD = TM + 4;
  const size_t smem = (size_t)frows * LD * sizeof(float);
  // FFJORD with the Hutchinson trace runs on the stash engine where it covers the model
  const bool ffj_tc =
      c->precision == GBNDE_PREC_BF16 && c->ff_on && c->ffj_tc_ok && !c->ff_exact && !c->ff_reg;
  const bool tcform = c->precision == GBNDE_PREC_BF16 && (!c->ff_on || ffj_tc);
  bool wide = tcform && c->tc_wide && (!c->tc_shape_ok || ffj_tc);
  if (tcform && c->tc_wide && c->tc_shape_ok && !ffj_tc) {
    if (c->force_wide >= 0) wide = c->force_wide == 1;
    else {
      auto it = c->tuned_tc.find({S, B});
      wide = it != c->tuned_tc.end() && it->second == 1;
    }
  }
  const int ntiles = tcform ? (B + 127) / 128 : (B + TM - 1) / TM;
  int gmax = 0;
  if (tcform) {
    if (max_grid_fwd_tc(&gmax)) return fail(GBNDE_ERR_CUDA, "occupancy query failed (tc)");
    if (c->grid_cap > 0) gmax = std::min(gmax, c->grid_cap);
  } else if (max_grid_fwd_f32(smem, &gmax)) {
    return fail(GBNDE_ERR_CUDA, "occupancy query failed");
  }
  const int grid = tcform ? balanced_grid(ntiles, gmax) : std::min(gmax, ntiles);

  int r = 0;
  // dense stage storage: one slot (u_n, k1..k7) per accepted step, within a
  // quarter of the free device memory
  // dense stage storage: one slot (u_n, k1..k7) per accepted step. Sized from
  // the step count of the previous solve (at least 64 slots), within a
  // quarter of the free device memory; grows only when a solve needs more.
  // the BF16 form keeps its internal vectors (state, stages, dense slots) in
  // the tile layout: ntiles * 128 rows x 64 components each
  const size_t SBv = tcform ? (size_t)ntiles * c->nsc * tc::kTileVec : SB;
  const size_t slot = 8 * SBv * sizeof(float);
  const long long cap_slots = c->stage_cap ? (long long)(c->stage_cap / slot) : (long long)1 << 62;
  auto size_dense = [&](long long want) {
    want = std::min<long long>(std::max<long long>(want, 64), maxiters + 1);
    want = std::min(want, cap_slots);
    const long long have_now = (long long)(c->dense.n / slot);
    if (have_now > cap_slots) c->dense.release();
    if (want > (long long)(c->dense.n / slot)) {
      size_t freeb = 0, totb = 0;
      cudaMemGetInfo(&freeb, &totb);
      const long long budget = (long long)((freeb / 4) / slot) + (long long)(c->dense.n / slot);
      long long ns = std::min(want, budget);
      if (ns > (long long)(c->dense.n / slot)) {
        c->dense.release();
        if (ns >= 2 && c->dense.ensure((size_t)ns * slot)) {
          cudaGetLastError();
          c->dense.release();
        }
      }
    }
    c->dense_slots = (long long)(c->dense.n / slot);
    if (c->dense_slots < 2) c->dense_slots = 0;
  };
  size_dense(2 * c->last_naccept + 8);
  if (tcform && (r = c->comp.ensure(2 * SBv * 4))) return r;
  if (u0_host && (r = c->u0.ensure(SB * 4))) return r;
  if ((r = c->ubuf.ensure(2 * SBv * 4)) || (r = c->kbuf.ensure(7 * SBv * 4))) return r;
  if (usave_host && (r = c->usave.ensure(SB * nsave * 4))) return r;
  if ((r = c->ckpt.ensure(SB * nb * 4)) || (r = c->ckpt_step.ensure(nb * sizeof(int)))) return r;
  if (tcform && !wide && (r = c->ckcomp.ensure(SBv * nb * 4))) return r;
  const long long maxsteps = std::min<long long>(maxiters, 1LL << 22);
  if ((r = c->steplog.ensure(2 * maxsteps * sizeof(double)))) return r;
  if ((r = c->trace.ensure(4 * maxsteps * sizeof(double)))) return r;
  if ((r = c->partials.ensure(4 * (size_t)grid * sizeof(double)))) return r;
  if ((r = c->sync.ensure(64)) || (r = c->counters.ensure(CT_NSLOTS * sizeof(long long) + 16))) return r;
  if ((r = c->saveat_d.ensure(nsave * sizeof(double))) || (r = c->bnd_d.ensure(nb * sizeof(double)))) return r;

  cudaStream_t st = c->stream;
  const float* u0d = u0;
  if (u0_host) {
    CK(cudaMemcpyAsync(c->u0.p, u0, SB * 4, cudaMemcpyHostToDevice, st));
    u0d = c->u0.as<float>();
  }
  float* usd = usave_host ? c->usave.as<float>() : usave;
  CK(cudaMemcpyAsync(c->saveat_d.p, d->saveat, nsave * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->bnd_d.p, bnd.data(), nb * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(c->sync.p, 0, 64, st));
  CK(cudaMemsetAsync(c->counters.p, 0, CT_NSLOTS * sizeof(long long) + 16, st));

  FwdArgs a{};
  a.mlp = c->mlp;
  a.S = S;
  a.B = B;
  a.TM = TM;
  a.LD = LD;
  a.ntiles = ntiles;
  a.t0 = d->t0;
  a.t1 = d->t1;
  a.abstol = d->abstol;
  a.reltol = d->reltol;
  a.dt0 = d->dt0;
  a.f32time = (d->flags & GBNDE_FLAG_FP32_TIME) ? 1 : 0;
  a.dtmin = d->dtmin > 0 ? d->dtmin : 0.0;
  a.dtmax = std::fabs(d->t1 - d->t0);
  a.maxiters = maxiters;
  a.saveat = c->saveat_d.as<double>();
  a.nsave = nsave;
  a.bnd = c->bnd_d.as<double>();
  a.nbnd = nb;
  a.u0 = u0d;
  a.ubuf[0] = c->ubuf.as<float>();
  a.ubuf[1] = c->ubuf.as<float>() + SBv;
  for (int j = 0; j < 7; ++j) a.kbuf[j] = c->kbuf.as<float>() + j * SBv;
  a.usave = usd;
  a.ckpt = c->ckpt.as<float>();
  a.max_ckpt = nb;
  a.ckpt_step = c->ckpt_step.as<int>();
  a.steplog = c->steplog.as<double>();
  a.maxsteps = maxsteps;
  a.trace = c->trace.as<double>();
  a.partials = c->partials.as<double>();
  a.bar = c->sync.as<unsigned int>();
  a.status = reinterpret_cast<int*>(c->sync.as<char>() + 16);
  a.counters = c->counters.as<long long>();
  a.tfinal = reinterpret_cast<double*>(c->counters.as<char>() + CT_NSLOTS * sizeof(long long));
  a.dense = c->dense_slots > 0 ? c->dense.as<float>() : nullptr;
  a.dense_slots = c->dense_slots;
  a.ffj = c->ff_on;
  a.ffd = c->ff_d;
  a.exact = c->ff_exact;
  a.ffreg = c->ff_on && c->ff_reg;
  a.noise = c->ff_on ? c->ffnoise.as<float>() : nullptr;
  if (wide && (r = c->stash.ensure((size_t)grid * tc::kStashCta))) return r;
  CK(cudaEventRecord(c->ev[0], st));
  if (wide) {
    FwdTcwArgs wa{};
    FwdTcArgs& ta = wa.t;
    ta.f = a;
    ta.f.ntiles = ntiles;
    ta.f.TM = 128;
    // per layer its N-block ops; FFJORD: the primal blocks (stash buffer
    // l % 2), then the tangent blocks on the same weights (buffer 2 + l % 2)
    int n = 0;
    for (int l = 0; l < c->mlp.nlayers; ++l) {
      const int out = c->mlp.dims[l + 1];
      for (int chain = 0; chain < (ffj_tc ? 2 : 1); ++chain)
        for (int b = 0; b * 256 < out; ++b) {
          if (n >= tc::kMaxOps) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
          tc::GemmOp& o = ta.ops.op[n++];
          o.kind = 3;
          // the tangent chain (FFJORD's J e, read only through the trace)
          // issues three split products, and its stash chunks carry two pieces
          o.nprod = chain == 1 ? 3 : 0;
          o.wimg = c->wimg.as<uint8_t>() + c->wb_off[l][b];
          o.npad = c->wb_npad[l][b];
          o.nchunk = (c->mlp.dims[l] + 63) / 64;
          o.sbuf = 2 * chain + (l & 1);
          o.first_nb = b == 0;
          o.aimg = c->stash.as<uint8_t>() + (size_t)o.sbuf * tc::kStashChunks * tc::kASlotBytes;
          o.cta_stride = tc::kStashCta;
          o.img_off = -1;
        }
      ta.bias[l] = c->mlp.bias[l];
    }
    ta.ops.nops = n;
    if (ffj_tc) {
      int hv = 0;
      for (int l = 1; l < c->mlp.nlayers; ++l) hv += tc::kCW * ((c->mlp.dims[l] + 63) / 64);
      wa.hvals = hv + 4;
      if ((r = c->thscr.ensure((size_t)grid * tc::kEpiThreads * wa.hvals * 4)) ||
          (r = c->ttrs.ensure((size_t)grid * 512 * 4)))
        return r;
      wa.hscr = c->thscr.as<float>();
      wa.trs = c->ttrs.as<float>();
    }
    ta.comp[0] = c->comp.as<float>();
    ta.comp[1] = c->comp.as<float>() + SBv;
    ta.dense = a.dense;
    ta.dense_slots = a.dense_slots;
    ta.kring = c->kbuf.as<float>();
    wa.stash = c->stash.as<uint8_t>();
    wa.nsc = c->nsc;
    if (c->recording) {
      c->rec.fwd = true;
      c->rec.tc = true;
      c->rec.wide = true;
      c->rec.fwd_tcw = wa;
      c->rec.fwd_grid = grid;
    }
    if (launch_fwd_tcw(wa, grid, st)) {
      cudaError_t e = cudaGetLastError();
      return fail(GBNDE_ERR_CUDA, "forward (tc, stash mode) launch failed: %s", cudaGetErrorString(e));
    }
  } else if (tcform) {
    FwdTcArgs ta{};
    ta.f = a;
    ta.f.ntiles = ntiles;
    ta.f.TM = 128;
    ta.ops.nops = c->mlp.nlayers;
    for (int l = 0; l < c->mlp.nlayers; ++l) {
      ta.ops.op[l].wimg = c->wimg.as<uint8_t>() + c->wimg_off[l];
      ta.ops.op[l].npad = c->npad[l];
      ta.ops.op[l].nchunk = c->nchunk[l];
      ta.ops.op[l].kind = 0;
      ta.bias[l] = c->mlp.bias[l];
    }
    ta.comp[0] = c->comp.as<float>();
    ta.comp[1] = c->comp.as<float>() + SBv;
    ta.dense = a.dense;
    ta.dense_slots = a.dense_slots;
    ta.kring = c->kbuf.as<float>();
    ta.ckcomp = c->ckcomp.as<float>();
    if (c->recording) {
      c->rec.fwd = true;
      c->rec.tc = true;
      c->rec.wide = false;
      c->rec.fwd_tc = ta;
      c->rec.fwd_grid = grid;
    }
    if (launch_fwd_tc(ta, grid, st)) {
      cudaError_t e = cudaGetLastError();
      return fail(GBNDE_ERR_CUDA, "forward (tc) launch failed: %s", cudaGetErrorString(e));
    }
  } else {
    if (c->recording) {
      c->rec.fwd = true;
      c->rec.tc = false;
      c->rec.fwd_f32 = a;
      c->rec.fwd_grid = grid;
      c->rec.fwd_smem = smem;
    }
    if (launch_fwd_f32(a, grid, smem, st)) {
      cudaError_t e = cudaGetLastError();
      return fail(GBNDE_ERR_CUDA, "forward launch failed: %s", cudaGetErrorString(e));
    }
  }
  CK(cudaEventRecord(c->ev[1], st));
  long long cnt[CT_NSLOTS + 2];
  int status[4];
  CK(cudaMemcpyAsync(cnt, c->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(status, a.status, sizeof status, cudaMemcpyDeviceToHost, st));
  if (usave_host) CK(cudaMemcpyAsync(usave, usd, SB * nsave * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    c->fwd_ms = ms;
  }
  double tfinal;
  std::memcpy(&tfinal, &cnt[CT_NSLOTS], sizeof(double));
  const long long nacc = cnt[CT_NACCEPT];
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->nf = cnt[CT_NF];
    stats->naccept = nacc;
    stats->nreject = cnt[CT_NREJECT];
    stats->retcode = status[ST_RETCODE];
    stats->t_final = tfinal;
    stats->fwd_path = tcform ? GBNDE_PATH_TC : GBNDE_PATH_FP32;
  }
  c->fwd_retcode = status[ST_RETCODE];
  if (status[ST_BARRIER]) return fail(GBNDE_ERR_TIMEOUT, "forward grid barrier timed out");
  // keep what the backward pass needs
  const long long nlog = std::min(nacc, maxsteps);
  c->steps.resize(2 * nlog);
  if (nlog) CK(cudaMemcpy(c->steps.data(), c->steplog.p, 2 * nlog * sizeof(double), cudaMemcpyDeviceToHost));
  const int nck = (int)cnt[CT_NCKPT];
  c->ckstep.resize(nck);
  if (nck) CK(cudaMemcpy(c->ckstep.data(), c->ckpt_step.p, nck * sizeof(int), cudaMemcpyDeviceToHost));
  c->naccept = nacc;
  c->nattempt = std::min(cnt[CT_NATTEMPT], maxsteps);
  c->final_cur = (int)cnt[5];
  c->B = B;
  c->nsave = nsave;
  c->t0 = d->t0;
  c->f32time = (d->flags & GBNDE_FLAG_FP32_TIME) ? 1 : 0;
  c->t1 = d->t1;
  c->abstol = d->abstol;
  c->reltol = d->reltol;
  c->maxiters = maxiters;
  c->sensealg = d->sensealg;
  c->saveat.assign(d->saveat, d->saveat + nsave);
  c->have_fwd = (status[ST_RETCODE] == GBNDE_RET_SUCCESS) && nacc <= maxsteps;
  c->dense_valid = c->dense_slots > 0 && nacc < c->dense_slots;
  c->dense_tl = tcform;
  c->fwd_wide = wide;
  c->last_naccept = nacc;
  c->fS = S;
  if (c->have_fwd && !c->dense_valid && !c->rerun_guard && c->dense_slots < cap_slots) {
    // the solve outgrew the dense stage storage: grow it and solve again once
    // (the backward then interpolates the stored stages instead of recomputing)
    c->rerun_guard = true;
    const int rr = forward_impl(c, d, S, B, u0, u0_host, usave, usave_host, stats);
    c->rerun_guard = false;
    return rr;
  }
  c->usave_dev = usd;
  return 0;
}

// Backward intervals, from the last save time down to t0, with the recorded
// forward steps that cover each and the checkpoint to restart them from.
static int build_intervals(gbnde_ctx* c, std::vector<Interval>& ivs, int* max_slots,
                           int* save_last, int* nsave_last) {
  std::vector<double> times;  // distinct save times and t0, increasing
  times.push_back(c->t0);
  for (double s : c->saveat)
    if (s > times.back()) times.push_back(s);
  const double tlast = c->saveat.back();
  *save_last = 0;
  *nsave_last = 0;
  for (int i = 0; i < c->nsave; ++i)
    if (c->saveat[i] == tlast) {
      if (*nsave_last == 0) *save_last = i;
      ++*nsave_last;
    }
  const long long ns = c->naccept;
  auto step_tn = [&](long long n) { return c->steps[2 * n]; };
  *max_slots = 1;
  ivs.clear();
  for (int k = (int)times.size() - 1; k >= 1; --k) {
    const double lo = times[k - 1], hi = times[k];
    if (hi > tlast) continue;
    Interval iv{};
    iv.t_lo = lo;
    iv.t_hi = hi;
    // step containing lo: last n with t_n <= lo; step containing hi: last n with t_n < hi
    long long nlo = 0, nhi = 0;
    for (long long n = 0; n < ns; ++n) {
      if (step_tn(n) <= lo) nlo = n;
      if (step_tn(n) < hi) nhi = n;
    }
    iv.nlo = (int)nlo;
    iv.nhi = (int)nhi;
    auto it = std::find(c->ckstep.begin(), c->ckstep.end(), (int)nlo);
    if (c->sensealg != GBNDE_SENSE_BACKSOLVE && it == c->ckstep.end())
      return fail(GBNDE_ERR_STATE, "no checkpoint for forward step %lld", nlo);
    iv.ckpt = it == c->ckstep.end() ? 0 : (int)(it - c->ckstep.begin());
    iv.save_lo = -1;
    iv.nsave_lo = 0;
    for (int i = 0; i < c->nsave; ++i)
      if (c->saveat[i] == lo) {
        if (iv.nsave_lo == 0) iv.save_lo = i;
        ++iv.nsave_lo;
      }
    *max_slots = std::max(*max_slots, iv.nhi - iv.nlo + 1);
    ivs.push_back(iv);
  }
  return 0;
}

// Tensor-core adjoint: op list, scratch images and launch. `base` carries the
// intervals, cotangents and state buffers prepared for the FP32 kernel.
static int backward_tc(gbnde_ctx* c, const BwdArgs& base, cudaStream_t st, float* dp_d) {
  const MlpDev& m = c->mlp;
  const int L = m.nlayers;
  const int B = c->B;
  const int P = (int)c->P;
  int gmax = 0;
  if (max_grid_fwd_tc(&gmax)) return fail(GBNDE_ERR_CUDA, "occupancy query failed (tc)");
  if (c->grid_cap > 0) gmax = std::min(gmax, c->grid_cap);
  const int ntiles = (B + 127) / 128;
  const int grid = balanced_grid(ntiles, gmax);
  // tiles per CTA: each keeps its own stage images (the tile index travels in
  // 8 bits of the evaluation command)
  const int tpc = (ntiles + grid - 1) / grid;
  if (tpc > 255) return fail(GBNDE_ERR_UNSUPPORTED, "tensor-core adjoint: more than 255 tiles per SM");
  const size_t SBt = (size_t)ntiles * tc::kTileVec;  // tile-layout vectors
  BwdTcArgs t{};
  t.b = base;
  t.b.ntiles = ntiles;
  t.b.TM = 128;
  // weight-gradient operand images per CTA
  size_t off = 0;
  for (int l = 0; l < L; ++l) {
    const int out = m.dims[l + 1], in = m.dims[l];
    // the smaller side is the M side (128-row halves), the larger the N side
    // (up to 256 columns): fewer, wider products (each tcgen05.mma costs about
    // the same to issue whatever its N, so two N = 64 ops cost twice one
    // N = 256 op although they do half its work)
    t.a_isA[l] = in < out ? 1 : 0;
    const int mside = t.a_isA[l] ? in : out;
    t.nh[l] = (mside + 127) / 128;
    // per 64-trajectory block (2 of them): the M side in 128-row halves of
    // 16 KB per piece, the N side in 64-feature blocks of 8 KB per piece
    // (one FP16 piece: the epilogue writes the images itself)
    auto img_bytes = [&](int dim, int isA) -> size_t {
      return isA ? (size_t)2 * t.nh[l] * 16384 : (size_t)2 * ((dim + 63) / 64) * 8192;
    };
    t.aoff[l] = (long long)off;
    off += img_bytes(in, t.a_isA[l]);
    t.doff[l] = (long long)off;
    off += img_bytes(out, !t.a_isA[l]);
  }
  t.img_cta = off;
  int hv = 0;
  for (int l = 1; l < L; ++l) {
    t.hoff[l] = hv;
    hv += tc::kCW * ((m.dims[l] + 63) / 64);  // per epilogue thread
  }
  t.hx = hv;
  hv += tc::kCW;
  t.hvals = hv;
  int nb = 0;
  for (int l = 0; l < L; ++l) {
    t.boffp[l] = nb;
    nb += 64 * ((m.dims[l + 1] + 63) / 64);
  }
  t.nbias = nb;
  int r = 0;
  t.tpc = tpc;
  if ((r = c->timg.ensure((size_t)grid * tpc * tc::kImgSlots * t.img_cta)) ||
      (r = c->thscr.ensure((size_t)grid * tc::kEpiThreads * t.hvals * 4)) ||
      (r = c->tlamcomp.ensure(2 * SBt * 4)) ||
      (r = c->mu_acc.ensure((size_t)grid * P * 4)) || (r = c->mu_stage.ensure((size_t)grid * 3 * P * 4)) ||
      (r = c->txst.ensure(6 * SBt * 4)))
    return r;
  if ((r = clear_images(c))) return r;
  t.xst = c->txst.as<float>();
  // per-CTA quadrature slots padded to a multiple of 4 floats (float4 sweeps)
  const int Ppad = (P + 3) / 4 * 4;
  t.b.P = Ppad;
  if ((r = c->mu_acc.ensure((size_t)grid * Ppad * 4)) || (r = c->mu_stage.ensure((size_t)grid * 3 * 4 * t.nbias * 4)))
    return r;
  t.b.mu_acc = c->mu_acc.as<float>();
  t.b.mu_stage = c->mu_stage.as<float>();
  t.pbias = c->mu_stage.as<float>();
  t.img = c->timg.as<uint8_t>();
  t.hscr = c->thscr.as<float>();
  t.mu_comp = nullptr;  // plain FP32 accumulation (no compensation) in this engine
  t.lam_comp[0] = c->tlamcomp.as<float>();
  t.lam_comp[1] = c->tlamcomp.as<float>() + SBt;
  // dense storage, or (O(checkpoints) mode) replay of each interval into b.ibuf
  const bool replay = base.dense == nullptr;
  t.b.dense = replay ? nullptr : c->dense.as<float>();
  if (replay) {
    if ((r = c->trep.ensure(2 * SBt * 4))) return r;
    t.rep[0] = c->trep.as<float>();
    t.rep[1] = c->trep.as<float>() + SBt;
    t.ckcomp = c->ckcomp.as<float>();
  }
  for (int l = 0; l < L; ++l) {
    tc::GemmOp& o = t.fwops.op[l];
    o.kind = 0;
    o.wimg = c->wimg.as<uint8_t>() + c->wimg_off[l];
    o.npad = c->npad[l];
    o.nchunk = c->nchunk[l];
    o.img_off = -1;
  }
  t.fwops.nops = L;
  for (int l = 0; l < L; ++l) t.bias[l] = m.bias[l];
  // op lists: forward recompute + VJP chain (per evaluation), and the
  // stage-stacked weight gradients (per accepted step: K = 6 stages x 128)
  // Every chain operand is also a weight-gradient image: forward op l's A is
  // a_l (image aoff[l]), VJP op l's A is delta_{l+1} (image doff[l]); the MMA
  // warp copies the chunks to the stage's slot. The output layer's forward
  // op is copy-only: a_{L-1} passes through the ring just to reach its image.
  int n = 0;
  if (2 * L > tc::kMaxOps) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
  // The adjoint's chain GEMMs (recompute and VJP) issue three of the five
  // split products: their 16-bit operands keep the gradient within 1e-5 of
  // the five-product form, while the forward needs all five (its error
  // estimate reaches the rounding noise of fewer). The replay list (fwops)
  // keeps five: it must reproduce the forward's steps exactly.
  // The epilogue writes the weight-gradient images (FP16) itself, so the
  // chain ops copy nothing, and the output layer is not recomputed: the
  // list is the forward ops of layers 0..L-2, then the VJP ops of L-1..0.
  for (int l = 0; l < L - 1; ++l) {
    tc::GemmOp& o = t.ops.op[n++];
    o.kind = 0;
    o.nprod = 3;
    o.wimg = c->wimg.as<uint8_t>() + c->wimg_off[l];
    o.npad = c->npad[l];
    o.nchunk = c->nchunk[l];
    o.img_off = -1;
  }
  for (int l = L - 1; l >= 0; --l) {
    tc::GemmOp& o = t.ops.op[n++];
    o.kind = 0;
    o.nprod = 3;
    o.wimg = c->wimg.as<uint8_t>() + c->wtimg_off[l];
    o.npad = c->npadT[l];
    o.nchunk = c->nchunkT[l];
    o.img_off = -1;
  }
  t.ops.nops = n;
  t.ops7 = t.ops;  // (unused: an evaluation that reuses activations starts at the VJP ops)
  n = 0;
  t.dw_chunks = 0;
  for (int l = 0; l < L; ++l) {
    const int out = m.dims[l + 1], in = m.dims[l];
    const int nside = t.a_isA[l] ? out : in;
    const int nblk = (nside + 63) / 64;
    const long long aimg = t.a_isA[l] ? t.aoff[l] : t.doff[l];
    const long long bimg = t.a_isA[l] ? t.doff[l] : t.aoff[l];
    for (int hh = 0; hh < t.nh[l]; ++hh) {
      if (n >= tc::kMaxOps) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
      tc::GemmOp& o = t.dwops.op[n++];
      o.kind = 1;
      o.aimg = t.img + aimg + (size_t)hh * 16384;
      o.wimg = t.img + bimg;
      o.cta_stride = (size_t)tpc * tc::kImgSlots * t.img_cta;
      o.slot_stride = t.img_cta;
      o.a_bytes = 16384;
      o.a_step = (uint32_t)(t.nh[l] * 16384);
      o.b_step = (uint32_t)(nblk * 8192);
      o.nblk_b = nblk;
      o.img_pieces = 1;
      o.img_f16 = 1;
      o.npad = (nside + 15) / 16 * 16;
      o.nchunk = 2 * 6 * tpc;  // K = (tile, stage, 64-trajectory block)
      o.first_dw = 0;
      o.img_off = -1;
      t.dw_chunks += o.nchunk;
    }
  }
  t.dwops.nops = n;
  CK(cudaEventRecord(c->ev[2], st));
  if (c->recording) {
    c->rec.bwd = !replay;  // an O(checkpoints) step runs eagerly
    c->rec.bwd_tc_on = true;
    c->rec.bwd_tc = t;
    c->rec.bwd_grid = grid;
    c->rec.red_stride = Ppad;
    c->rec.dp = dp_d;
  }
  if (launch_bwd_tc(t, grid, st)) {
    cudaError_t e = cudaGetLastError();
    return fail(GBNDE_ERR_CUDA, "backward (tc) launch failed: %s", cudaGetErrorString(e));
  }
  CK(cudaEventRecord(c->ev[3], st));
  if (launch_reduce_mu_comp(t.b.mu_acc, t.mu_comp, grid, Ppad, P, dp_d, st))
    return fail(GBNDE_ERR_CUDA, "reduce launch failed");
  return 0;
}

// Stash-mode tensor-core adjoint (bwd_tcw.cu): N-block op lists, images and
// launch. `base` carries the intervals, cotangents and state buffers.
static int backward_tcw(gbnde_ctx* c, const BwdArgs& base, cudaStream_t st, float* dp_d) {
  const MlpDev& m = c->mlp;
  const int L = m.nlayers;
  const int B = c->B, S = c->S;
  const int P = (int)c->P;
  int gmax = 0;
  if (max_grid_fwd_tc(&gmax)) return fail(GBNDE_ERR_CUDA, "occupancy query failed (tc)");
  if (c->grid_cap > 0) gmax = std::min(gmax, c->grid_cap);
  const int ntiles = (B + 127) / 128;
  const int grid = balanced_grid(ntiles, gmax);
  const int tpc = (ntiles + grid - 1) / grid;
  if (tpc > 255) return fail(GBNDE_ERR_UNSUPPORTED, "tensor-core adjoint: more than 255 tiles per SM");
  const size_t SBt = (size_t)ntiles * c->nsc * tc::kTileVec;
  BwdTcwArgs w{};
  BwdTcArgs& t = w.t;
  t.b = base;
  t.b.ntiles = ntiles;
  t.b.TM = 128;
  // weight-gradient images: per layer a_l and delta_{l+1}; the larger side is
  // the M side (128-row halves), the other the N side (64-column blocks)
  size_t off = 0;
  int nblkN[GBNDE_MAX_LAYERS] = {};
  for (int l = 0; l < L; ++l) {
    const int out = m.dims[l + 1], in = m.dims[l];
    // the smaller side is the M side (128-row halves), the larger the N side
    // (up to 256 columns): fewer, wider products (each tcgen05.mma costs about
    // the same to issue whatever its N, so two N = 64 ops cost twice one
    // N = 256 op although they do half its work)
    t.a_isA[l] = in < out ? 1 : 0;
    const int mside = t.a_isA[l] ? in : out;
    t.nh[l] = (mside + 127) / 128;
    nblkN[l] = ((t.a_isA[l] ? out : in) + 63) / 64;
    // per 64-trajectory block (2 of them): the M side in 128-row halves of
    // 16 KB per piece, the N side in 64-feature blocks of 8 KB per piece
    auto img_bytes = [&](int dim, int isA) -> size_t {
      return isA ? (size_t)2 * t.nh[l] * tc::kImgPieces * 16384
                 : (size_t)2 * tc::kImgPieces * ((dim + 63) / 64) * 8192;
    };
    t.aoff[l] = (long long)off;
    off += img_bytes(in, t.a_isA[l]);
    t.doff[l] = (long long)off;
    off += img_bytes(out, !t.a_isA[l]);
  }
  // FFJORD: a second operand pair per layer (adot_l, pdotbar_l), laid out
  // after the first pair's images, one pair's bytes further
  const bool ffj = c->ff_on != 0;
  const size_t img0 = off;
  t.img_cta = ffj ? 2 * off : off;
  int hv = 0;
  for (int l = 1; l < L; ++l) {
    t.hoff[l] = hv;
    hv += tc::kCW * ((m.dims[l] + 63) / 64);
  }
  t.hx = hv;
  if (ffj)
    for (int l = 0; l + 1 < L; ++l) {  // the tangent pre-activations pdot_l
      t.hoff2[l] = hv;
      hv += tc::kCW * ((m.dims[l + 1] + 63) / 64);
    }
  t.hvals = hv + 4;
  int nb = 0;
  for (int l = 0; l < L; ++l) {
    t.boffp[l] = nb;
    nb += 64 * ((m.dims[l + 1] + 63) / 64);
  }
  t.nbias = nb;
  t.tpc = tpc;
  const int Ppad = (P + 3) / 4 * 4;
  t.b.P = Ppad;
  int r = 0;
  if ((r = c->timg.ensure((size_t)grid * tpc * tc::kImgSlots * t.img_cta)) ||
      (r = c->thscr.ensure((size_t)grid * tc::kEpiThreads * t.hvals * 4)) ||
      (r = c->tlamcomp.ensure(2 * SBt * 4)) ||
      (r = c->mu_acc.ensure((size_t)grid * Ppad * 4)) || (r = c->mu_stage.ensure((size_t)grid * 3 * 4 * t.nbias * 4)) ||
      (r = c->stash.ensure((size_t)grid * tc::kStashCta)))
    return r;
  if ((r = clear_images(c))) return r;
  t.b.mu_acc = c->mu_acc.as<float>();
  t.b.mu_stage = c->mu_stage.as<float>();
  t.pbias = c->mu_stage.as<float>();
  t.img = c->timg.as<uint8_t>();
  t.hscr = c->thscr.as<float>();
  t.mu_comp = nullptr;  // plain FP32 accumulation (no compensation)
  t.lam_comp[0] = c->tlamcomp.as<float>();
  t.lam_comp[1] = c->tlamcomp.as<float>() + SBt;
  t.b.dense = c->dense.as<float>();
  for (int l = 0; l < L; ++l) t.bias[l] = m.bias[l];
  uint8_t* stash = c->stash.as<uint8_t>();
  auto stash_op = [&](tc::GemmOp& o, int sbuf, int first) {
    o.sbuf = sbuf;
    o.first_nb = first;
    o.aimg = stash + (size_t)sbuf * tc::kStashChunks * tc::kASlotBytes;
    o.cta_stride = tc::kStashCta;
  };
  // evaluation list: forward recompute of layers 0..L-2 (a_l in buffer l % 2,
  // image of a_l from the first N-block op), a copy-only op for a_{L-1}, then
  // the VJP layers L-1..0 (delta_{l+1} in buffer (l + 1) % 2, image from the
  // first N-block op; layer 0 only over the state inputs)
  int n = 0;
  auto next_op = [&](tc::OpList& lst) -> tc::GemmOp* {
    if (n >= tc::kMaxOps) return nullptr;
    tc::GemmOp* o = &lst.op[n++];
    *o = tc::GemmOp{};
    return o;
  };
  // chain ops: chain 0 the primal operands (a_l, pbar_l: images aoff / doff,
  // stash buffers 0/1), chain 1 FFJORD's tangent operands (adot_l, pdotbar_l:
  // images one pair further, stash buffers 2/3)
  auto chain_op = [&](int kind, int l, int b, int chain, bool vjp) -> tc::GemmOp* {
    tc::GemmOp* o = next_op(t.ops);
    if (!o) return nullptr;
    const int in = m.dims[l], out = m.dims[l + 1];
    const int k = vjp ? out : in;  // K of the op: the operand's width
    o->kind = kind;
    o->nprod = 3;  // the adjoint's chains: three split products (as in the single-accumulator engine)
    if (kind == 3) {
      o->wimg = c->wimg.as<uint8_t>() + (vjp ? c->wbT_off[l][b] : c->wb_off[l][b]);
      o->npad = vjp ? c->wbT_npad[l][b] : c->wb_npad[l][b];  // the image's row padding
    }
    o->nchunk = (k + 63) / 64;
    stash_op(*o, 2 * chain + ((vjp ? l + 1 : l) & 1), b == 0);
    o->img_off = b == 0 ? (int)((vjp ? t.doff[l] : t.aoff[l]) + (chain ? img0 : 0)) : -1;
    o->img_isA = (uint8_t)(vjp ? !t.a_isA[l] : t.a_isA[l]);
    o->img_nblk = (uint8_t)((k + 63) / 64);
    o->img_nh = (uint16_t)t.nh[l];
    return o;
  };
  const int nchains = ffj ? 2 : 1;
  // evaluation list: forward recompute of layers 0..L-2 (per chain; operand
  // images from the first N-block op), copy-only ops for a_{L-1} (and
  // adot_{L-1}), then the VJP layers L-1..0 over their inputs (layer 0 only
  // over the state inputs; FFJORD: the abar / achk ops of an N-block in a
  // row, then a copy-only op for pdotbar_0's image)
  for (int l = 0; l < L - 1; ++l)
    for (int ch = 0; ch < nchains; ++ch)
      for (int b = 0; b * 256 < m.dims[l + 1]; ++b)
        if (!chain_op(3, l, b, ch, false)) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
  for (int ch = 0; ch < nchains; ++ch)
    if (!chain_op(4, L - 1, 0, ch, false)) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
  for (int l = L - 1; l >= 0; --l) {
    const int nout = l == 0 ? S : m.dims[l];  // inputs whose cotangent is needed
    for (int b = 0; b * 256 < nout; ++b)
      for (int ch = 0; ch < (l == 0 ? 1 : nchains); ++ch)
        if (!chain_op(3, l, b, ch, true)) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
  }
  if (ffj) {
    // pdotbar_0 feeds no product, only layer 0's second weight-gradient pair
    tc::GemmOp* o = next_op(t.ops);
    if (!o) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
    o->kind = 4;
    o->nchunk = (m.dims[1] + 63) / 64;
    stash_op(*o, 2 + 1, 1);
    o->img_off = (int)(t.doff[0] + img0);
    o->img_isA = (uint8_t)(!t.a_isA[0]);
    o->img_nblk = (uint8_t)((m.dims[1] + 63) / 64);
    o->img_nh = (uint16_t)t.nh[0];
  }
  t.ops.nops = n;
  t.ops7 = t.ops;
  // weight gradients of an accepted step: per layer, M halves x N-blocks
  n = 0;
  t.dw_chunks = 0;
  for (int l = 0; l < L; ++l) {
    const int out = m.dims[l + 1], in = m.dims[l];
    const int nside = t.a_isA[l] ? out : in;
    const int nblk = nblkN[l];
    const long long aimg = t.a_isA[l] ? t.aoff[l] : t.doff[l];
    const long long bimg = t.a_isA[l] ? t.doff[l] : t.aoff[l];
    for (int hh = 0; hh < t.nh[l]; ++hh) {
      for (int nbk = 0; nbk * 256 < nside; ++nbk) {
        tc::GemmOp* o = next_op(t.dwops);
        if (!o) return fail(GBNDE_ERR_UNSUPPORTED, "too many tensor-core ops");
        const int nbb = std::min(4, nblk - 4 * nbk);
        o->kind = 1;
        o->aimg = t.img + aimg + (size_t)hh * tc::kImgPieces * 16384;
        o->wimg = t.img + bimg;
        o->cta_stride = (size_t)tpc * tc::kImgSlots * t.img_cta;
        o->slot_stride = t.img_cta;
        o->a_bytes = tc::kImgPieces * 16384;
        o->a_step = (uint32_t)(t.nh[l] * tc::kImgPieces * 16384);
        o->b_step = (uint32_t)(tc::kImgPieces * nblk * 8192);
        o->nblk_b = nbb;
        o->b_off0 = (uint32_t)(4 * nbk * 8192);
        o->b_pstride = (uint32_t)(nblk * 8192);
        o->npad = (std::min(256, nside - 256 * nbk) + 15) / 16 * 16;
        o->nchunk = 2 * 6 * tpc * nchains;
        o->npairs = nchains;
        o->pair_aoff = (uint32_t)img0;
        o->pair_boff = (uint32_t)img0;
        o->first_dw = 0;
        o->img_off = -1;
        t.dw_chunks += o->nchunk;
      }
    }
  }
  t.dwops.nops = n;
  w.stash = stash;
  w.nsc = c->nsc;
  if (ffj) {
    if ((r = c->ttrs.ensure((size_t)grid * 512 * 4))) return r;
    w.trs = c->ttrs.as<float>();
  }
  CK(cudaEventRecord(c->ev[2], st));
  if (launch_bwd_tcw(w, grid, st)) {
    cudaError_t e = cudaGetLastError();
    return fail(GBNDE_ERR_CUDA, "backward (tc, stash mode) launch failed: %s", cudaGetErrorString(e));
  }
  CK(cudaEventRecord(c->ev[3], st));
  if (launch_reduce_mu_comp(t.b.mu_acc, t.mu_comp, grid, Ppad, P, dp_d, st))
    return fail(GBNDE_ERR_CUDA, "reduce launch failed");
  return 0;
}

static int backward_impl(gbnde_ctx* c, const float* dLdu, bool in_host, float* dLdu0,
                         float* dLdp, bool out_host, gbnde_stats* stats) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  if (!c->have_fwd) return fail(GBNDE_ERR_STATE, "backward needs a successful forward solve first");
  if (!(c->t1 > c->t0)) return fail(GBNDE_ERR_UNSUPPORTED, "gradients of reverse time spans");
  if (!dLdu || !dLdu0 || !dLdp) return fail(GBNDE_ERR_INVALID, "null argument");
  if (int r = set_device(c)) return r;
  const int S = c->fS, B = c->B, nsave = c->nsave;
  const size_t SB = (size_t)S * B;
  const int P = (int)c->P;
  if (c->ff_on && (c->sensealg != GBNDE_SENSE_INTERPOLATING || !c->dense_valid))
    return fail(GBNDE_ERR_UNSUPPORTED, "FFJORD gradients use InterpolatingAdjoint with stored stages");
  std::vector<Interval> ivs;
  int max_slots = 1, save_last = 0, nsave_last = 0;
  if (int r = build_intervals(c, ivs, &max_slots, &save_last, &nsave_last)) return r;
  const bool backsolve = c->sensealg == GBNDE_SENSE_BACKSOLVE;
  const bool gauss = c->sensealg == GBNDE_SENSE_GAUSS;
  // tensor-core adjoint: on the dense stage storage, or (single-accumulator
  // engine, after a tensor-core forward) replaying each interval from its checkpoint
  const bool tc_replay = c->precision == GBNDE_PREC_BF16 && c->tc_bwd_ok && !backsolve && !gauss &&
                         !c->dense_valid && c->dense_tl && !c->fwd_wide && !c->ff_on;
  const bool ffj_tc = c->ff_on && c->fwd_wide && c->dense_tl && c->ffj_tc_ok && !c->ff_exact && !c->ff_reg;
  const bool tcbwd = (c->precision == GBNDE_PREC_BF16 && (c->fwd_wide ? c->tc_wide_bwd : c->tc_bwd_ok) &&
                      !backsolve && !gauss && c->dense_valid && (!c->ff_on || ffj_tc)) ||
                     tc_replay;
  // the FP32 adjoint reads dense slots only in its own layout; after a
  // tensor-core forward it recomputes each interval from the checkpoints
  const bool dense_f32 = c->dense_valid && !backsolve && !c->dense_tl;
  const size_t SBv = tcbwd ? (size_t)((B + 127) / 128) * c->nsc * tc::kTileVec : SB;

  int rows = 0;
  for (int l = 0; l <= c->mlp.nlayers; ++l) rows += c->mlp.dims[l];
  // activations of every layer, two work buffers and, with the cube prefix,
  // the state before it
  rows = c->ff_on ? 2 * rows + 4 * c->mlp.maxdim + 1 + (c->ff_reg ? 3 : 0)
                  : rows + 2 * c->mlp.maxdim + (c->mlp.cube ? S : 0);
  int TM = 0;
  if (choose_tm(rows, kSmemBudget, &TM)) return fail(GBNDE_ERR_UNSUPPORTED, "network too wide");
  while (TM > 8 && TM / 2 >= B) TM /= 2;
  {
    int want = c->tm_force_bwd;
    auto it = c->tuned.find({S, B});
    if (!want && it != c->tuned.end()) want = it->second.second;
    if (want > 0 && (size_t)rows * (want + 4) * sizeof(float) <= kSmemBudget) TM = want;
    else if (c->tm_force_bwd) return fail(GBNDE_ERR_UNSUPPORTED, "%d tile rows do not fit", want);
  }
  const int LD = TM + 4;
  size_t smem = (size_t)rows * LD * sizeof(float);
  // a small model's pending quadrature (3 x P floats) fits beside the tile in
  // shared memory: the per-stage weight-gradient sums then make no global
  // round trips (the batch-1 spiral: P = 252)
  int pb_smem_off = 0;
  if (smem + (size_t)3 * P * sizeof(float) <= std::min<size_t>(kSmemBudget, 64 * 1024)) {
    pb_smem_off = rows * LD;
    smem += (size_t)3 * P * sizeof(float);
  }
  const int ntiles = (B + TM - 1) / TM;
  int gmax = 0;
  if (max_grid_bwd_f32(smem, &gmax)) return fail(GBNDE_ERR_CUDA, "occupancy query failed");
  const int grid = std::min(gmax, ntiles);

  int r = 0;
  if (in_host && (r = c->dldu.ensure(SB * nsave * 4))) return r;
  if (out_host && ((r = c->dldu0.ensure(SB * 4)) || (r = c->dldp.ensure((size_t)P * 4)))) return r;
  if ((r = c->lam.ensure(2 * SBv * 4)) || (r = c->kl.ensure(7 * SBv * 4))) return r;
  if (backsolve && ((r = c->ub.ensure(2 * SB * 4)) || (r = c->ku.ensure(7 * SB * 4)))) return r;
  if (!tcbwd && !backsolve && !dense_f32 && (r = c->ibuf.ensure((size_t)max_slots * 8 * SB * 4))) return r;
  if (tc_replay && (r = c->ibuf.ensure((size_t)max_slots * 8 * SBv * 4))) return r;
  if ((r = c->mu_acc.ensure((size_t)grid * P * 4)) || (r = c->mu_stage.ensure((size_t)grid * 3 * P * 4))) return r;
  if ((r = c->iv_d.ensure(std::max<size_t>(1, ivs.size()) * sizeof(Interval)))) return r;
  if ((r = c->bsync.ensure(64)) || (r = c->bcounters.ensure(CT_NSLOTS * sizeof(long long)))) return r;
  if ((r = c->partials.ensure(4 * (size_t)grid * sizeof(double)))) return r;

  cudaStream_t st = c->stream;
  const float* dldu_d = dLdu;
  if (in_host) {
    CK(cudaMemcpyAsync(c->dldu.p, dLdu, SB * nsave * 4, cudaMemcpyHostToDevice, st));
    dldu_d = c->dldu.as<float>();
  }
  float* du0_d = out_host ? c->dldu0.as<float>() : dLdu0;
  float* dp_d = out_host ? c->dldp.as<float>() : dLdp;
  if (!ivs.empty())
    CK(cudaMemcpyAsync(c->iv_d.p, ivs.data(), ivs.size() * sizeof(Interval), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(c->bsync.p, 0, 64, st));
  CK(cudaMemsetAsync(c->bcounters.p, 0, CT_NSLOTS * sizeof(long long), st));

  BwdArgs a{};
  a.mlp = c->mlp;
  a.S = S;
  a.B = B;
  a.TM = TM;
  a.LD = LD;
  a.ntiles = ntiles;
  a.P = P;
  a.sensealg = c->sensealg;
  a.t0 = c->t0;
  a.abstol = c->abstol;
  a.reltol = c->reltol;
  a.dtmax = c->saveat.back() - c->t0;
  a.f32time = c->f32time;
  a.maxiters = c->maxiters;
  a.iv = c->iv_d.as<Interval>();
  a.niv = (int)ivs.size();
  a.fsteps = c->steplog.as<double>();
  a.nfsteps = c->naccept;
  a.ckpt = c->ckpt.as<float>();
  a.usave = c->usave_dev;
  a.dLdu = dldu_d;
  a.saveat = c->saveat_d.as<double>();
  a.nsave = nsave;
  a.save_last = save_last;
  a.nsave_last = nsave_last;
  a.ibuf = c->ibuf.as<float>();
  a.ibuf_slots = max_slots;
  a.dense = (tcbwd && !tc_replay) || dense_f32 ? c->dense.as<float>() : nullptr;
  a.lam[0] = c->lam.as<float>();
  a.lam[1] = c->lam.as<float>() + SBv;
  a.ub[0] = backsolve ? c->ub.as<float>() : nullptr;
  a.ub[1] = backsolve ? c->ub.as<float>() + SB : nullptr;
  for (int j = 0; j < 7; ++j) {
    a.kl[j] = c->kl.as<float>() + j * SBv;
    a.ku[j] = backsolve ? c->ku.as<float>() + j * SB : nullptr;
    a.kf[j] = nullptr;
  }
  a.mu_acc = c->mu_acc.as<float>();
  a.mu_stage = c->mu_stage.as<float>();
  a.pb_smem_off = pb_smem_off;
  a.dLdu0 = du0_d;
  a.partials = c->partials.as<double>();
  a.bar = c->bsync.as<unsigned int>();
  a.status = reinterpret_cast<int*>(c->bsync.as<char>() + 16);
  a.counters = c->bcounters.as<long long>();
  a.ffj = c->ff_on;
  a.ffd = c->ff_d;
  a.exact = c->ff_exact;
  a.ffreg = (c->ff_on && c->ff_reg) ? (1 | (c->ff_reg_g2 ? 2 : 0)) : 0;
  a.noise = c->ff_on ? c->ffnoise.as<float>() : nullptr;
  if (tcbwd && c->fwd_wide) {
    if (c->recording) c->rec.bwd = false;  // stash-mode steps run eagerly
    if (int rr = backward_tcw(c, a, st, dp_d)) return rr;
  } else if (tcbwd) {
    if (int rr = backward_tc(c, a, st, dp_d)) return rr;
  } else {
    CK(cudaEventRecord(c->ev[2], st));
    if (c->recording) {
      c->rec.bwd = true;
      c->rec.bwd_tc_on = false;
      c->rec.bwd_f32 = a;
      c->rec.bwd_grid = grid;
      c->rec.bwd_smem = smem;
      c->rec.dp = dp_d;
    }
    if (launch_bwd_f32(a, grid, smem, st)) {
      cudaError_t e = cudaGetLastError();
      return fail(GBNDE_ERR_CUDA, "backward launch failed: %s", cudaGetErrorString(e));
    }
    CK(cudaEventRecord(c->ev[3], st));
    if (launch_reduce_mu(a.mu_acc, grid, P, dp_d, st)) return fail(GBNDE_ERR_CUDA, "reduce launch failed");
  }
  long long cnt[CT_NSLOTS];
  int status[4];
  CK(cudaMemcpyAsync(cnt, c->bcounters.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(status, a.status, sizeof status, cudaMemcpyDeviceToHost, st));
  if (out_host) {
    CK(cudaMemcpyAsync(dLdu0, du0_d, SB * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(dLdp, dp_d, (size_t)P * 4, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
    c->bwd_ms = ms;
  }
  if (stats) {
    stats->nf_adj = cnt[CT_NF];
    stats->naccept_adj = cnt[CT_NACCEPT];
    stats->nreject_adj = cnt[CT_NREJECT];
    stats->nf_recompute = cnt[CT_NRECOMP];
    stats->nf_adj_vjp = cnt[CT_NVJP];
    stats->retcode_adj = status[ST_RETCODE];
    stats->adj_path = tc_replay ? GBNDE_PATH_TC_RECOMPUTE
                      : tcbwd     ? GBNDE_PATH_TC
                      : (a.dense != nullptr || backsolve) ? GBNDE_PATH_FP32 : GBNDE_PATH_FP32_RECOMPUTE;
  }
  if (status[ST_BARRIER]) return fail(GBNDE_ERR_TIMEOUT, "backward grid barrier timed out");
  return 0;
}

static MsArgs ms_args(gbnde_ctx* c, int TM) {
  MsArgs m{};
  m.mlp = c->mlp;
  m.S = c->ms_S;
  m.nseg = c->ms_nseg;
  m.TM = TM;
  m.LD = TM + 4;
  m.ntiles = (c->ms_nseg + TM - 1) / TM;
  m.MS = c->ms_MS;
  m.segs = c->ms_segs.as<MsSeg>();
  m.saveat = c->ms_saveat.as<double>();
  m.u0 = c->ms_u0.as<float>();
  m.usave = c->ms_usave.as<float>();
  m.dense = c->ms_dense.as<float>();
  m.steplog = c->ms_steplog.as<double>();
  m.nacc = c->ms_nacc.as<int>();
  m.retcode = c->ms_ret.as<int>();
  m.counters = c->ms_cnt.as<long long>();
  return m;
}

// Segments per tile: the largest power of two up to `fit` (and 64) that still
// leaves about as many tiles as SMs. The segments are short and each carries
// its own controller, so the launches are latency-bound and parallelism across
// SMs pays: 3973 segments run as 125 tiles of 32 (74.2 gradient evaluations/s)
// against 63 tiles of 64 (50.3), 249 of 16 (69.0) or 497 of 8 (58.4).
static int ms_tile_rows(int fit, int nseg) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int tm = std::min(fit, 64);
  while (tm > 8 && (nseg + tm - 1) / tm < (3 * nsm) / 4) tm /= 2;
  return tm;
}

static int ms_grid(int ntiles) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, std::min(ntiles, nsm));
}

int gbnde_multishoot_forward(gbnde_ctx* c, int S, int nseg, const gbnde_segment* segs,
                             const double* saveat, int nsave_total, const float* u0, double abstol,
                             double reltol, long long maxiters, float* usave, int* retcodes,
                             gbnde_stats* stats) {
  if (!c || !segs || !saveat || !u0) return fail(GBNDE_ERR_INVALID, "null argument");
  if (!c->have_params) return fail(GBNDE_ERR_STATE, "parameters not set");
  if (S != c->S || nseg < 1 || nsave_total < 1) return fail(GBNDE_ERR_INVALID, "bad sizes");
  if (c->mlp.timein) return fail(GBNDE_ERR_UNSUPPORTED, "multiple shooting with a time input");
  if (!(abstol > 0) || !(reltol >= 0)) return fail(GBNDE_ERR_INVALID, "tolerances must be positive");
  for (int i = 0; i < nseg; ++i) {
    const gbnde_segment& g = segs[i];
    if (!(g.t1 >= g.t0) || g.nsave < 1 || g.save_off < 0 || g.save_off + g.nsave > nsave_total)
      return fail(GBNDE_ERR_INVALID, "segment %d is malformed", i);
    for (int q = 0; q < g.nsave; ++q) {
      const double s = saveat[g.save_off + q];
      if (!(s >= g.t0 && s <= g.t1) || (q > 0 && s < saveat[g.save_off + q - 1]))
        return fail(GBNDE_ERR_INVALID, "segment %d: save times must be increasing inside [t0, t1]", i);
    }
  }
  if (int r = set_device(c)) return r;
  c->ms_have = false;
  c->ms_dl_ok = false;
  c->ms_saves = false;
  c->ms_hsegs.assign(segs, segs + nseg);
  c->ms_S = S;
  c->ms_nseg = nseg;
  c->ms_nsave = nsave_total;
  c->ms_MS = 256;
  const size_t SN = (size_t)S * nseg;
  int TM = 0;
  if (choose_tm(2 * c->mlp.maxdim, kSmemBudgetMs, &TM)) return fail(GBNDE_ERR_UNSUPPORTED, "layer too wide");
  TM = ms_tile_rows(TM, nseg);
  const size_t smem = (size_t)2 * c->mlp.maxdim * (TM + 4) * sizeof(float);
  int r = 0;
  if ((r = c->ms_segs.ensure(nseg * sizeof(MsSeg))) || (r = c->ms_saveat.ensure(nsave_total * sizeof(double))) ||
      (r = c->ms_u0.ensure(SN * 4)) || (r = c->ms_usave.ensure((size_t)S * nsave_total * 4)) ||
      (r = c->ms_dense.ensure((size_t)nseg * (c->ms_MS + 1) * 8 * S * 4)) ||
      (r = c->ms_steplog.ensure((size_t)nseg * c->ms_MS * 2 * sizeof(double))) ||
      (r = c->ms_nacc.ensure(nseg * sizeof(int))) || (r = c->ms_ret.ensure(nseg * sizeof(int))) ||
      (r = c->ms_cnt.ensure(8 * sizeof(long long))))
    return r;
  cudaStream_t st = c->stream;
  static_assert(sizeof(MsSeg) == sizeof(gbnde_segment), "segment layout");
  CK(cudaMemcpyAsync(c->ms_segs.p, segs, nseg * sizeof(MsSeg), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->ms_saveat.p, saveat, nsave_total * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->ms_u0.p, u0, SN * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(c->ms_usave.p, 0, (size_t)S * nsave_total * 4, st));
  CK(cudaMemsetAsync(c->ms_cnt.p, 0, 8 * sizeof(long long), st));
  MsArgs m = ms_args(c, TM);
  m.abstol = abstol;
  m.reltol = reltol;
  m.maxiters = maxiters > 0 ? maxiters : 100000;
  const int grid = ms_grid(m.ntiles);
  CK(cudaEventRecord(c->ev[0], st));
  if (launch_ms_fwd(m, grid, smem, st)) return fail(GBNDE_ERR_CUDA, "multishoot forward launch failed");
  CK(cudaEventRecord(c->ev[1], st));
  long long cnt[8];
  CK(cudaMemcpyAsync(cnt, c->ms_cnt.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
  if (usave) CK(cudaMemcpyAsync(usave, c->ms_usave.p, (size_t)S * nsave_total * 4, cudaMemcpyDeviceToHost, st));
  std::vector<int> ret(nseg);
  CK(cudaMemcpyAsync(ret.data(), c->ms_ret.p, nseg * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->fwd_ms = ms;
  int worst = GBNDE_RET_SUCCESS;
  for (int i = 0; i < nseg; ++i) {
    if (retcodes) retcodes[i] = ret[i];
    if (ret[i] != GBNDE_RET_SUCCESS) worst = ret[i];
  }
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->nf = cnt[0];
    stats->naccept = cnt[1];
    stats->nreject = cnt[2];
    stats->retcode = worst;
    stats->fwd_path = GBNDE_PATH_FP32;
  }
  c->ms_have = (worst == GBNDE_RET_SUCCESS);
  c->ms_saves = true;
  return 0;
}

int gbnde_multishoot_saves(gbnde_ctx* c, float* usave) {
  if (!c || !usave) return fail(GBNDE_ERR_INVALID, "null argument");
  if (!c->ms_saves) return fail(GBNDE_ERR_STATE, "no multishoot forward to read the saves of");
  if (int r = set_device(c)) return r;
  CK(cudaMemcpyAsync(usave, c->ms_usave.p, (size_t)c->ms_S * c->ms_nsave * 4, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int gbnde_multishoot_loss(gbnde_ctx* c, const float* data, const int* seg_next, int loss_kind,
                          double continuity_term, double* loss) {
  if (!c || !data || !seg_next || !loss) return fail(GBNDE_ERR_INVALID, "null argument");
  if (loss_kind != 0 && loss_kind != 1) return fail(GBNDE_ERR_INVALID, "loss_kind must be 0 or 1");
  if (!c->ms_have) return fail(GBNDE_ERR_STATE, "the loss needs a successful multishoot forward first");
  if (int r = set_device(c)) return r;
  const int S = c->ms_S, nseg = c->ms_nseg, ncol = c->ms_nsave;
  // column -> segment, segment offsets/lengths and successors (every save
  // column belongs to exactly one segment; a segment is continued by at most
  // one other)
  std::vector<int> map((size_t)ncol + 3 * (size_t)nseg, -1);
  int* colseg = map.data();
  int* segoff = colseg + ncol;
  int* segn = segoff + nseg;
  int* nxt = segn + nseg;
  std::vector<char> taken(nseg, 0);
  for (int g = 0; g < nseg; ++g) {
    const gbnde_segment& q = c->ms_hsegs[g];
    segoff[g] = q.save_off;
    segn[g] = q.nsave;
    for (int k = 0; k < q.nsave; ++k) {
      if (colseg[q.save_off + k] != -1) return fail(GBNDE_ERR_INVALID, "save column %d is in two segments", q.save_off + k);
      colseg[q.save_off + k] = g;
    }
    const int nx = seg_next[g];
    if (nx < -1 || nx >= nseg || nx == g || (nx >= 0 && taken[nx]))
      return fail(GBNDE_ERR_INVALID, "seg_next[%d] = %d is not a segment that continues it", g, nx);
    if (nx >= 0) taken[nx] = 1;
    nxt[g] = nx;
  }
  for (int j = 0; j < ncol; ++j)
    if (colseg[j] < 0) return fail(GBNDE_ERR_INVALID, "save column %d is in no segment", j);
  const int nblk = std::max(1, std::min(1024, (int)(((size_t)S * ncol + 255) / 256)));
  int r = 0;
  if ((r = c->ms_data.ensure((size_t)S * ncol * 4)) || (r = c->ms_map.ensure(map.size() * sizeof(int))) ||
      (r = c->ms_part.ensure(nblk * sizeof(double))) || (r = c->ms_dldu.ensure((size_t)S * ncol * 4)))
    return r;
  cudaStream_t st = c->stream;
  CK(cudaMemcpyAsync(c->ms_data.p, data, (size_t)S * ncol * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->ms_map.p, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  const int* dm = c->ms_map.as<int>();
  if (launch_ms_loss(c->ms_usave.as<float>(), c->ms_data.as<float>(), dm, dm + ncol, dm + ncol + nseg,
                     dm + ncol + 2 * nseg, S, ncol, loss_kind, continuity_term, c->ms_dldu.as<float>(),
                     c->ms_part.as<double>(), nblk, st))
    return fail(GBNDE_ERR_CUDA, "multishoot loss launch failed");
  std::vector<double> part(nblk);
  CK(cudaMemcpyAsync(part.data(), c->ms_part.p, nblk * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  double s = 0.0;
  for (double x : part) s += x;
  *loss = s;
  c->ms_dl_ok = true;
  return 0;
}

int gbnde_multishoot_backward(gbnde_ctx* c, const float* dLdu, float* dLdu0, float* dLdp,
                              gbnde_stats* stats) {
  if (!c || !dLdp) return fail(GBNDE_ERR_INVALID, "null argument");
  if (!c->ms_have) return fail(GBNDE_ERR_STATE, "backward needs a successful multishoot forward first");
  if (!dLdu && !c->ms_dl_ok)
    return fail(GBNDE_ERR_STATE, "dL_dusave = NULL needs a gbnde_multishoot_loss after the forward");
  if (int r = set_device(c)) return r;
  const int S = c->ms_S, nseg = c->ms_nseg;
  const size_t SN = (size_t)S * nseg;
  const int P = (int)c->P;
  int rows = 0;
  for (int l = 0; l <= c->mlp.nlayers; ++l) rows += c->mlp.dims[l];
  rows = c->ff_on ? 2 * rows + 4 * c->mlp.maxdim + 1 : rows + 2 * c->mlp.maxdim + S;
  int TM = 0;
  if (choose_tm(rows, kSmemBudgetMs, &TM)) return fail(GBNDE_ERR_UNSUPPORTED, "network too wide");
  TM = ms_tile_rows(TM, nseg);
  const size_t smem = (size_t)rows * (TM + 4) * sizeof(float);
  MsArgs m = ms_args(c, TM);
  const int grid = ms_grid(m.ntiles);
  int r = 0;
  if ((r = c->ms_dldu.ensure((size_t)S * c->ms_nsave * 4)) || (r = c->ms_dldu0.ensure(SN * 4)) ||
      (r = c->ms_bar.ensure(SN * 9 * 4)) || (r = c->ms_mu.ensure((size_t)grid * P * 4)) ||
      (r = c->ms_dldp.ensure((size_t)P * 4)))
    return r;
  cudaStream_t st = c->stream;
  if (dLdu) {
    CK(cudaMemcpyAsync(c->ms_dldu.p, dLdu, (size_t)S * c->ms_nsave * 4, cudaMemcpyHostToDevice, st));
    c->ms_dl_ok = false;  // the device cotangent is now the caller's
  }
  m.dLdu = c->ms_dldu.as<float>();
  m.dLdu0 = c->ms_dldu0.as<float>();
  m.bar = c->ms_bar.as<float>();
  m.mu_acc = c->ms_mu.as<float>();
  m.P = P;
  CK(cudaEventRecord(c->ev[2], st));
  if (launch_ms_bwd(m, grid, smem, st)) return fail(GBNDE_ERR_CUDA, "multishoot backward launch failed");
  if (launch_reduce_mu(m.mu_acc, grid, P, c->ms_dldp.as<float>(), st)) return fail(GBNDE_ERR_CUDA, "reduce failed");
  CK(cudaEventRecord(c->ev[3], st));
  if (dLdu0) CK(cudaMemcpyAsync(dLdu0, c->ms_dldu0.p, SN * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(dLdp, c->ms_dldp.p, (size_t)P * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
  c->bwd_ms = ms;
  if (stats) {
    stats->retcode_adj = GBNDE_RET_SUCCESS;
    stats->adj_path = GBNDE_PATH_FP32;
  }
  return 0;
}

int gbnde_forward(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0,
                  float* usave, gbnde_stats* stats) {
  if (!c || !u0 || !usave) return fail(GBNDE_ERR_INVALID, "null argument");
  c->ff_on = 0;
  return forward_impl(c, d, S, B, u0, true, usave, true, stats);
}

int gbnde_forward_device(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0,
                         float* usave, gbnde_stats* stats) {
  if (!c || !u0 || !usave) return fail(GBNDE_ERR_INVALID, "null argument");
  c->ff_on = 0;
  return forward_impl(c, d, S, B, u0, false, usave, false, stats);
}

namespace {

// FFJORD forward: the augmented system [z; delta_logp (; |f|^2; |e^T J|)] from
// (x, 0) over [t0, t1], keeping the end state; logpx for the standard-normal
// base, z(t1) and the two regulariser integrals when reg.
int ffjord_forward_impl(gbnde_ctx* c, const gbnde_solve_desc* desc, int d, int B, const float* x,
                        const float* noise, int exact, int reg, float* logpx, float* zT, float* rf, float* rj,
                        gbnde_stats* stats) {
  if (!c || !desc || !x || !logpx) return fail(GBNDE_ERR_INVALID, "null argument");
  if (d != c->S) return fail(GBNDE_ERR_INVALID, "data dim %d does not match the model (%d)", d, c->S);
  if (c->mlp.cube) return fail(GBNDE_ERR_UNSUPPORTED, "FFJORD with a cube prefix");
  if (!exact && !noise) return fail(GBNDE_ERR_INVALID, "the Hutchinson trace needs noise");
  if (int r = set_device(c)) return r;
  const int S = d + (reg ? 3 : 1);
  const size_t SB = (size_t)S * B;
  int r = 0;
  if ((r = c->ffu0.ensure(SB * 4)) || (r = c->ffus.ensure(SB * 4)) ||
      (noise && (r = c->ffnoise.ensure((size_t)d * B * 4))))
    return r;
  std::vector<float> y0(SB, 0.f);
  for (int b = 0; b < B; ++b)
    for (int s = 0; s < d; ++s) y0[(size_t)b * S + s] = x[(size_t)b * d + s];
  CK(cudaMemcpy(c->ffu0.p, y0.data(), SB * 4, cudaMemcpyHostToDevice));
  if (noise) CK(cudaMemcpy(c->ffnoise.p, noise, (size_t)d * B * 4, cudaMemcpyHostToDevice));
  gbnde_solve_desc dd = *desc;
  const double tend = desc->t1;
  dd.saveat = &tend;
  dd.nsave = 1;
  dd.sensealg = GBNDE_SENSE_INTERPOLATING;
  c->ff_on = 1;
  c->ff_d = d;
  c->ff_exact = exact ? 1 : 0;
  c->ff_reg = reg ? 1 : 0;
  c->ff_reg_g2 = 0;
  r = forward_impl(c, &dd, S, B, c->ffu0.as<float>(), false, c->ffus.as<float>(), false, stats);
  if (r) return r;
  std::vector<float> yT(SB);
  CK(cudaMemcpy(yT.data(), c->ffus.p, SB * 4, cudaMemcpyDeviceToHost));
  const double lognorm = 0.5 * d * std::log(6.283185307179586);  // log(2 pi)
  for (int b = 0; b < B; ++b) {
    double q = 0.0;
    for (int s = 0; s < d; ++s) {
      const double z = yT[(size_t)b * S + s];
      q += z * z;
      if (zT) zT[(size_t)b * d + s] = (float)z;
    }
    logpx[b] = (float)(-0.5 * q - lognorm - (double)yT[(size_t)b * S + d]);
    if (reg && rf) rf[b] = yT[(size_t)b * S + d + 1];
    if (reg && rj) rj[b] = yT[(size_t)b * S + d + 2];
  }
  return 0;
}

int ffjord_backward_impl(gbnde_ctx* c, const float* dLdlogpx, const float* dLdzT, const float* dLdrf,
                         const float* dLdrj, float* dLdx, float* dLdp, gbnde_stats* stats) {
  if (!c || !dLdlogpx || !dLdx || !dLdp) return fail(GBNDE_ERR_INVALID, "null argument");
  if (!c->ff_on || !c->have_fwd) return fail(GBNDE_ERR_STATE, "backward needs a successful FFJORD forward");
  if (int r = set_device(c)) return r;
  const int d = c->ff_d, S = d + (c->ff_reg ? 3 : 1), B = c->B;
  const size_t SB = (size_t)S * B;
  std::vector<float> yT(SB), g(SB), du0(SB);
  CK(cudaMemcpy(yT.data(), c->ffus.p, SB * 4, cudaMemcpyDeviceToHost));
  int g2 = 0;
  for (int b = 0; b < B; ++b) {
    const float gl = dLdlogpx[b];
    for (int s = 0; s < d; ++s)
      g[(size_t)b * S + s] = -yT[(size_t)b * S + s] * gl + (dLdzT ? dLdzT[(size_t)b * d + s] : 0.f);
    g[(size_t)b * S + d] = -gl;
    if (c->ff_reg) {
      g[(size_t)b * S + d + 1] = dLdrf ? dLdrf[b] : 0.f;
      g[(size_t)b * S + d + 2] = dLdrj ? dLdrj[b] : 0.f;
      g2 |= (dLdrj && dLdrj[b] != 0.f);
    }
  }
  c->ff_reg_g2 = g2;
  const int r = backward_impl(c, g.data(), true, du0.data(), dLdp, true, stats);
  if (r) return r;
  for (int b = 0; b < B; ++b)
    for (int s = 0; s < d; ++s) dLdx[(size_t)b * d + s] = du0[(size_t)b * S + s];
  return 0;
}

}  // namespace

int gbnde_ffjord_forward(gbnde_ctx* c, const gbnde_solve_desc* desc, int d, int B, const float* x,
                         const float* noise, float* logpx, float* zT, gbnde_stats* stats) {
  return ffjord_forward_impl(c, desc, d, B, x, noise, noise ? 0 : 1, 0, logpx, zT, nullptr, nullptr, stats);
}

int gbnde_ffjord_forward_reg(gbnde_ctx* c, const gbnde_solve_desc* desc, int d, int B, const float* x,
                             const float* noise, int exact_trace, float* logpx, float* zT, float* reg_f2,
                             float* reg_ej, gbnde_stats* stats) {
  if (!noise) return fail(GBNDE_ERR_INVALID, "the |e^T J| row needs noise");
  return ffjord_forward_impl(c, desc, d, B, x, noise, exact_trace ? 1 : 0, 1, logpx, zT, reg_f2, reg_ej,
                             stats);
}

int gbnde_ffjord_backward(gbnde_ctx* c, const float* dLdlogpx, const float* dLdzT, float* dLdx, float* dLdp,
                          gbnde_stats* stats) {
  return ffjord_backward_impl(c, dLdlogpx, dLdzT, nullptr, nullptr, dLdx, dLdp, stats);
}

int gbnde_ffjord_backward_reg(gbnde_ctx* c, const float* dLdlogpx, const float* dLdzT, const float* dL_dreg_f2,
                              const float* dL_dreg_ej, float* dLdx, float* dLdp, gbnde_stats* stats) {
  if (c && c->ff_on && !c->ff_reg)
    return fail(GBNDE_ERR_STATE, "the last FFJORD forward ran without the regulariser rows");
  return ffjord_backward_impl(c, dLdlogpx, dLdzT, dL_dreg_f2, dL_dreg_ej, dLdx, dLdp, stats);
}

int gbnde_backward(gbnde_ctx* c, const float* dLdu, float* dLdu0, float* dLdp, gbnde_stats* stats) {
  return backward_impl(c, dLdu, true, dLdu0, dLdp, true, stats);
}

int gbnde_backward_device(gbnde_ctx* c, const float* dLdu, float* dLdu0, float* dLdp,
                          gbnde_stats* stats) {
  return backward_impl(c, dLdu, false, dLdu0, dLdp, false, stats);
}

int gbnde_loss_device(gbnde_ctx* c, const float* usave, const float* target, int kind,
                      float* dLdu, double* loss) {
  if (!c || !usave || !target || !dLdu || !loss) return fail(GBNDE_ERR_INVALID, "null argument");
  if (!c->have_fwd) return fail(GBNDE_ERR_STATE, "loss needs a forward solve first");
  if (kind != 0 && kind != 1) return fail(GBNDE_ERR_INVALID, "unknown loss kind %d", kind);
  if (int r = set_device(c)) return r;
  const size_t n = (size_t)c->S * c->B * c->nsave;
  const int nblk = 304;
  if (int r = c->loss_part.ensure(nblk * sizeof(double))) return r;
  if (c->recording) {
    c->rec.loss = true;
    c->rec.l_us = usave;
    c->rec.l_tg = target;
    c->rec.l_n = n;
    c->rec.l_kind = kind;
    c->rec.l_dl = dLdu;
    c->rec.l_part = c->loss_part.as<double>();
    c->rec.l_nblk = nblk;
  }
  if (launch_loss(usave, target, n, kind, dLdu, c->loss_part.as<double>(), nblk, c->stream))
    return fail(GBNDE_ERR_CUDA, "loss launch failed");
  std::vector<double> part(nblk);
  CK(cudaMemcpyAsync(part.data(), c->loss_part.p, nblk * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double s = 0.0;
  for (double v : part) s += v;
  *loss = (kind == 1) ? s / (double)n : s;
  return 0;
}

int gbnde_train_step(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0,
                     const float* target, int kind, const gbnde_adam* opt, long long step, float* p,
                     float* m, float* v, double* loss, gbnde_stats* stats) {
  if (!c || !d || !u0 || !target || !opt || !p || !m || !v || !loss)
    return fail(GBNDE_ERR_INVALID, "null argument");
  if (step < 1) return fail(GBNDE_ERR_INVALID, "step counts from 1");
  if (!(opt->lr > 0) || !(opt->beta1 >= 0 && opt->beta1 < 1) || !(opt->beta2 >= 0 && opt->beta2 < 1) ||
      !(opt->eps > 0))
    return fail(GBNDE_ERR_INVALID, "Adam needs lr > 0, 0 <= beta1, beta2 < 1 and eps > 0");
  if (kind != 0 && kind != 1) return fail(GBNDE_ERR_INVALID, "unknown loss kind %d", kind);
  if (int r = set_device(c)) return r;
  if (d->nsave < 1 || B < 1 || S < 1) return fail(GBNDE_ERR_INVALID, "empty problem");
  const size_t SB = (size_t)S * B, nsv = (size_t)SB * d->nsave;
  int r = 0;
  if ((r = c->tr_us.ensure(nsv * 4)) || (r = c->tr_dl.ensure(nsv * 4)) || (r = c->tr_du0.ensure(SB * 4)) ||
      (r = c->tr_dp.ensure(c->P * 4)))
    return r;
  if ((r = gbnde_set_params_device(c, p, c->P))) return r;
  gbnde_stats sf{}, sb{};
  if ((r = gbnde_forward_device(c, d, S, B, u0, c->tr_us.as<float>(), &sf))) return r;
  *loss = INFINITY;
  if (sf.retcode == GBNDE_RET_SUCCESS) {
    if ((r = gbnde_loss_device(c, c->tr_us.as<float>(), target, kind, c->tr_dl.as<float>(), loss))) return r;
    if ((r = gbnde_backward_device(c, c->tr_dl.as<float>(), c->tr_du0.as<float>(), c->tr_dp.as<float>(), &sb)))
      return r;
    sf.nf_recompute = sb.nf_recompute;
    sf.nf_adj = sb.nf_adj;
    sf.nf_adj_vjp = sb.nf_adj_vjp;
    sf.naccept_adj = sb.naccept_adj;
    sf.nreject_adj = sb.nreject_adj;
    sf.retcode_adj = sb.retcode_adj;
    sf.adj_path = sb.adj_path;
    // a failed solve leaves the parameters unchanged (its loss is Inf)
    if (sb.retcode_adj == GBNDE_RET_SUCCESS) {
      if (launch_adam(p, m, v, c->tr_dp.as<float>(), c->P, opt->lr, opt->beta1, opt->beta2, opt->eps, step,
                      c->stream))
        return fail(GBNDE_ERR_CUDA, "Adam launch failed");
      if ((r = gbnde_set_params_device(c, p, c->P))) return r;
      CK(cudaStreamSynchronize(c->stream));
    } else {
      *loss = INFINITY;
    }
  }
  if (stats) *stats = sf;
  return 0;
}

}  // extern "C"

namespace {

// Captures the recorded step (parameter upload, forward, loss, interval plan,
// adjoint, reduction, Adam) into one CUDA graph on the context's stream.
int capture_step(gbnde_ctx* c, const gbnde_adam* opt, float* p, float* m, float* v) {
  StepRecord& R = c->rec;
  const BwdArgs& b = R.bwd_tc_on ? R.bwd_tc.b : R.bwd_f32;
  const FwdArgs& f = R.tc ? (R.wide ? R.fwd_tcw.t.f : R.fwd_tc.f) : R.fwd_f32;
  if (R.wide) return -1;  // stash-mode steps run eagerly
  if (!R.fwd || !R.bwd || !R.loss || !f.dense || !b.dense) return -1;  // the adjoint must read dense storage
  if (c->gstat.ensure(64)) return -1;
  if (!c->gpin && cudaMallocHost(&c->gpin, 2 * sizeof(double)) != cudaSuccess) {
    c->gpin = nullptr;
    cudaGetLastError();
    return -1;
  }
  double* gloss = c->gstat.as<double>();
  double* gcoef = gloss + 1;
  int* gflags = reinterpret_cast<int*>(gloss + 3);
  cudaStream_t st = c->stream;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  bool ok = cudaMemcpyAsync(c->params.p, p, c->P * sizeof(float), cudaMemcpyDeviceToDevice, st) == cudaSuccess;
  ok = ok && bind_params(c) == 0;
  ok = ok && cudaMemsetAsync(c->sync.p, 0, 64, st) == cudaSuccess;
  ok = ok && cudaMemsetAsync(c->counters.p, 0, CT_NSLOTS * sizeof(long long) + 16, st) == cudaSuccess;
  ok = ok && (R.tc ? launch_fwd_tc(R.fwd_tc, R.fwd_grid, st) : launch_fwd_f32(R.fwd_f32, R.fwd_grid, R.fwd_smem, st)) == 0;
  ok = ok && launch_loss(R.l_us, R.l_tg, R.l_n, R.l_kind, R.l_dl, R.l_part, R.l_nblk, st) == 0;
  ok = ok && launch_loss_finalize(R.l_part, R.l_nblk, R.l_n, R.l_kind, gloss, st) == 0;
  ok = ok && cudaMemsetAsync(c->bsync.p, 0, 64, st) == cudaSuccess;
  ok = ok && cudaMemsetAsync(c->bcounters.p, 0, CT_NSLOTS * sizeof(long long), st) == cudaSuccess;
  ok = ok && launch_plan_intervals(const_cast<Interval*>(b.iv), b.niv, b.fsteps, f.counters, f.status, f.dense_slots, f.maxsteps, gflags,
                                   st) == 0;
  ok = ok && (R.bwd_tc_on ? launch_bwd_tc(R.bwd_tc, R.bwd_grid, st)
                          : launch_bwd_f32(R.bwd_f32, R.bwd_grid, R.bwd_smem, st)) == 0;
  ok = ok && (R.bwd_tc_on ? launch_reduce_mu_comp(b.mu_acc, R.bwd_tc.mu_comp, R.bwd_grid, R.red_stride, (int)c->P,
                                                  R.dp, st)
                          : launch_reduce_mu(b.mu_acc, R.bwd_grid, (int)c->P, R.dp, st)) == 0;
  ok = ok && launch_adam_graph(p, m, v, R.dp, c->P, opt->lr, opt->beta1, opt->beta2, opt->eps, gcoef, gflags,
                               b.status, st) == 0;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  if (!ok || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return -1;
  }
  const cudaError_t ei = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) {
    c->gexec = nullptr;
    cudaGetLastError();
    return -1;
  }
  return 0;
}

template <class T>
void key_put(std::vector<char>& k, const T& x) {
  const char* p = reinterpret_cast<const char*>(&x);
  k.insert(k.end(), p, p + sizeof(T));
}

}  // namespace

extern "C" {

int gbnde_graph_train_step(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0,
                           const float* target, int kind, const gbnde_adam* opt, long long step, float* p,
                           float* m, float* v, double* loss, gbnde_stats* stats, int* graphed) {
  if (graphed) *graphed = 0;
  if (!c || !d || !u0 || !target || !opt || !p || !m || !v || !loss)
    return fail(GBNDE_ERR_INVALID, "null argument");
  if (step < 1) return fail(GBNDE_ERR_INVALID, "step counts from 1");
  if (!d->saveat || d->nsave < 1) return fail(GBNDE_ERR_INVALID, "saveat must hold >= 1 time");
  if (int r = set_device(c)) return r;
  // the graph is tied to these arguments (pointers included)
  std::vector<char> key;
  key_put(key, d->t0); key_put(key, d->t1); key_put(key, d->abstol); key_put(key, d->reltol);
  key_put(key, d->dt0); key_put(key, d->dtmin); key_put(key, d->maxiters); key_put(key, d->nsave);
  key_put(key, d->sensealg); key_put(key, d->flags);
  for (int i = 0; i < d->nsave; ++i) key_put(key, d->saveat[i]);
  key_put(key, S); key_put(key, B); key_put(key, u0); key_put(key, target); key_put(key, kind);
  key_put(key, opt->lr); key_put(key, opt->beta1); key_put(key, opt->beta2); key_put(key, opt->eps);
  key_put(key, p); key_put(key, m); key_put(key, v);
  if (!(c->gexec && key == c->gkey)) {
    // an eager step that records its launches, then the capture
    if (c->gexec) {
      cudaGraphExecDestroy(c->gexec);
      c->gexec = nullptr;
    }
    c->gkey.clear();
    c->rec = StepRecord{};
    c->recording = true;
    gbnde_stats se{};
    const int r = gbnde_train_step(c, d, S, B, u0, target, kind, opt, step, p, m, v, loss, &se);
    c->recording = false;
    if (stats) *stats = se;
    if (r) return r;
    if (se.retcode == GBNDE_RET_SUCCESS && se.retcode_adj == GBNDE_RET_SUCCESS && !c->graph_failed) {
      if (capture_step(c, opt, p, m, v) == 0) c->gkey = key;
      else c->graph_failed = true;  // this context keeps stepping eagerly
    }
    return 0;
  }
  // replay: the Adam bias corrections of this step, then the graph
  c->gpin[0] = 1.0 / (1.0 - std::pow(opt->beta1, (double)step));
  c->gpin[1] = 1.0 / (1.0 - std::pow(opt->beta2, (double)step));
  cudaStream_t st = c->stream;
  double* gloss = c->gstat.as<double>();
  CK(cudaMemcpyAsync(gloss + 1, c->gpin, 2 * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaGraphLaunch(c->gexec, st));
  double gl[4];
  long long fc[CT_NSLOTS], bc[CT_NSLOTS];
  int fs[4], bs[4];
  const StepRecord& R = c->rec;
  const FwdArgs& f = R.tc ? (R.wide ? R.fwd_tcw.t.f : R.fwd_tc.f) : R.fwd_f32;
  const BwdArgs& b = R.bwd_tc_on ? R.bwd_tc.b : R.bwd_f32;
  CK(cudaMemcpyAsync(gl, gloss, sizeof gl, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(fc, f.counters, sizeof fc, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(fs, f.status, sizeof fs, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(bc, b.counters, sizeof bc, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(bs, b.status, sizeof bs, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  int flags[2];
  std::memcpy(flags, &gl[3], sizeof flags);
  // the host-side record of the last forward is not refreshed by a replay
  c->have_fwd = false;
  if (flags[0] != 0 || fs[ST_RETCODE] != GBNDE_RET_SUCCESS || bs[ST_RETCODE] != GBNDE_RET_SUCCESS) {
    // a failed solve or outgrown stage storage: nothing was updated; redo the
    // step eagerly (which also regrows the storage) and capture again later
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->gkey.clear();
    return gbnde_train_step(c, d, S, B, u0, target, kind, opt, step, p, m, v, loss, stats);
  }
  *loss = gl[0];
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->nf = fc[CT_NF];
    stats->naccept = fc[CT_NACCEPT];
    stats->nreject = fc[CT_NREJECT];
    stats->nf_adj = bc[CT_NF];
    stats->nf_adj_vjp = bc[CT_NVJP];
    stats->nf_recompute = bc[CT_NRECOMP];
    stats->naccept_adj = bc[CT_NACCEPT];
    stats->nreject_adj = bc[CT_NREJECT];
    stats->retcode = fs[ST_RETCODE];
    stats->retcode_adj = bs[ST_RETCODE];
    stats->fwd_path = c->rec.tc ? GBNDE_PATH_TC : GBNDE_PATH_FP32;
    stats->adj_path = c->rec.bwd_tc_on ? GBNDE_PATH_TC : GBNDE_PATH_FP32;
  }
  if (graphed) *graphed = 1;
  return 0;
}

int gbnde_autotune(gbnde_ctx* c, const gbnde_solve_desc* d, int S, int B, const float* u0, int* tiles) {
  if (!c || !d || !u0) return fail(GBNDE_ERR_INVALID, "null argument");
  if (int r = validate_desc(c, d, S, B)) return r;
  if (int r = set_device(c)) return r;
  if (!c->have_params) return fail(GBNDE_ERR_STATE, "parameters not set");
  c->ff_on = 0;
  const bool tcform = c->precision == GBNDE_PREC_BF16;
  const size_t SB = (size_t)S * B, nsv = SB * d->nsave;
  int r = 0;
  if ((r = c->tr_us.ensure(nsv * 4)) || (r = c->tr_dl.ensure(nsv * 4)) || (r = c->tr_du0.ensure(SB * 4)) ||
      (r = c->tr_dp.ensure(c->P * 4)))
    return r;
  float* us = c->tr_us.as<float>();
  float* dl = c->tr_dl.as<float>();
  if (tcform) {
    // The tensor-core kernels run 128-trajectory tiles, one CTA per SM
    // (tensor memory is allocated whole). What there is to choose is the
    // engine, where both cover the model: the single-accumulator engine
    // (operands through shared memory, activation reuse in the adjoint) or the
    // stash engine (operands through a global stash, N-blocked layers). Each
    // runs a forward solve and its adjoint three times; the faster (last two)
    // is kept for this (S, B).
    int mode = c->tc_shape_ok ? 0 : 1;
    if (c->tc_shape_ok && c->tc_wide && c->tc_wide_bwd == c->tc_bwd_ok) {
      double best = 1e300;
      for (int w = 0; w < 2; ++w) {
        c->force_wide = w;
        double tsum = 0.0;
        bool okc = true;
        for (int rep = 0; rep < 3 && okc; ++rep) {
          gbnde_stats st{}, sb{};
          double L = 0.0;
          if (forward_impl(c, d, S, B, u0, false, us, false, &st) || st.retcode != GBNDE_RET_SUCCESS ||
              cudaMemsetAsync(dl, 0, nsv * 4, c->stream) != cudaSuccess || gbnde_loss_device(c, us, dl, 1, dl, &L) ||
              backward_impl(c, dl, false, c->tr_du0.as<float>(), c->tr_dp.as<float>(), false, &sb) ||
              sb.retcode_adj != GBNDE_RET_SUCCESS)
            okc = false;
          else if (rep > 0) tsum += c->fwd_ms + c->bwd_ms;
        }
        cudaGetLastError();
        if (okc && tsum < best) { best = tsum; mode = w; }
      }
      c->force_wide = -1;
      c->tuned_tc[{S, B}] = mode;
      if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
      }
      c->gkey.clear();
      g_last_error.clear();
    }
    if (tiles) {
      tiles[0] = 128;
      tiles[1] = mode;
    }
    return 0;
  }
  const int cand[4] = {8, 16, 32, 64};
  c->tuned.erase({S, B});
  // forward: fastest rows per tile over two timed solves each
  double best = 1e300;
  int best_f = 0;
  for (int tm : cand) {
    c->tm_force_fwd = tm;
    double tsum = 0.0;
    bool okc = true;
    for (int rep = 0; rep < 3 && okc; ++rep) {
      gbnde_stats st{};
      if (forward_impl(c, d, S, B, u0, false, us, false, &st) || st.retcode != GBNDE_RET_SUCCESS) okc = false;
      else if (rep > 0) tsum += c->fwd_ms;
    }
    cudaGetLastError();
    if (okc && tsum < best) { best = tsum; best_f = tm; }
  }
  c->tm_force_fwd = best_f;
  // backward: the cotangent of the mean square of the saved states
  int best_b = 0;
  best = 1e300;
  for (int tm : cand) {
    c->tm_force_bwd = tm;
    double tsum = 0.0;
    bool okc = true;
    for (int rep = 0; rep < 3 && okc; ++rep) {
      gbnde_stats st{}, sb{};
      double L = 0.0;
      if (forward_impl(c, d, S, B, u0, false, us, false, &st) || st.retcode != GBNDE_RET_SUCCESS ||
          cudaMemsetAsync(dl, 0, nsv * 4, c->stream) != cudaSuccess ||
          gbnde_loss_device(c, us, dl, 1, dl, &L) ||
          backward_impl(c, dl, false, c->tr_du0.as<float>(), c->tr_dp.as<float>(), false, &sb) ||
          sb.retcode_adj != GBNDE_RET_SUCCESS)
        okc = false;
      else if (rep > 0) tsum += c->bwd_ms;
    }
    cudaGetLastError();
    if (okc && tsum < best) { best = tsum; best_b = tm; }
  }
  c->tm_force_fwd = c->tm_force_bwd = 0;
  if (!best_f || !best_b) return fail(GBNDE_ERR_UNSUPPORTED, "no tile size ran for this shape");
  c->tuned[{S, B}] = {best_f, best_b};
  // a captured training step holds the old tile sizes: capture again
  if (c->gexec) {
    cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
  }
  c->gkey.clear();
  if (tiles) {
    tiles[0] = best_f;
    tiles[1] = best_b;
  }
  g_last_error.clear();
  return 0;
}

long long gbnde_forward_trace(gbnde_ctx* c, double* out4, long long cap) {
  if (!c || c->nattempt <= 0) return 0;
  const long long n = std::min(c->nattempt, cap);
  if (out4 && n > 0 &&
      cudaMemcpy(out4, c->trace.p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return c->nattempt;
}

void* gbnde_stream(gbnde_ctx* c) { return c ? (void*)c->stream : nullptr; }

int gbnde_set_stream(gbnde_ctx* c, void* stream) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return 0;
}

int gbnde_last_kernel_ms(gbnde_ctx* c, double* fwd_ms, double* bwd_ms) {
  if (!c) return fail(GBNDE_ERR_INVALID, "null context");
  if (fwd_ms) *fwd_ms = c->fwd_ms;
  if (bwd_ms) *bwd_ms = c->bwd_ms;
  return 0;
}

long long gbnde_forward_steps(gbnde_ctx* c, double* t, double* h, long long cap) {
  if (!c || !c->have_fwd) return 0;
  const long long n = (long long)c->steps.size() / 2;
  for (long long i = 0; i < std::min(n, cap); ++i) {
    if (t) t[i] = c->steps[2 * i];
    if (h) h[i] = c->steps[2 * i + 1];
  }
  return n;
}

}  // extern "C"
