// aux.cu -- small helper kernels: transposed weight copy for the VJPs and the
// fused save-point loss with its cotangent.
#include <algorithm>
#include <cmath>

#include "kernels.h"

namespace gbnde {

struct TransposeArgs {
  const float* src[GBNDE_MAX_LAYERS];
  float* dst[GBNDE_MAX_LAYERS];
  int K[GBNDE_MAX_LAYERS], N[GBNDE_MAX_LAYERS];
  int nlayers;
};

// dst[n*K + k] = src[k*N + n] for every layer (Lux [in][out] -> [out][in]).
__global__ void transpose_params_kernel(TransposeArgs a) {
  for (int l = 0; l < a.nlayers; ++l) {
    const int K = a.K[l], N = a.N[l];
    const size_t tot = (size_t)K * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot;
         i += (size_t)gridDim.x * blockDim.x) {
      const size_t n = i / K, k = i - n * K;
      a.dst[l][i] = a.src[l][k * N + n];
    }
  }
}

int launch_transpose_params(const MlpDev& m, const float* p, float* wtr, cudaStream_t st) {
  TransposeArgs a{};
  a.nlayers = m.nlayers;
  size_t toff = 0;
  for (int l = 0; l < m.nlayers; ++l) {
    a.src[l] = p + m.woff[l];
    a.dst[l] = wtr + toff;
    a.K[l] = m.dims[l];
    a.N[l] = m.dims[l + 1];
    toff += (size_t)m.dims[l] * m.dims[l + 1];
  }
  transpose_params_kernel<<<256, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// loss = sum (u - target)^2 (kind 0) or its mean (kind 1); dL = dloss/du.
// One FP64 partial per block, summed on the host in block order.
__global__ void loss_kernel(const float* __restrict__ u, const float* __restrict__ tg, size_t n,
                            int kind, float* __restrict__ dL, double* __restrict__ part) {
  __shared__ double red[40];
  const float scale = (kind == 1) ? (float)(2.0 / (double)n) : 2.f;
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
  double s = 0.0;
  size_t done = 0;
  if (((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(tg) | reinterpret_cast<uintptr_t>(dL)) & 15) == 0) {
    // 128-bit accesses; the squares go into two compensated (Kahan) FP32 sums
    // per thread (a few hundred terms each), added in FP64 at the end
    const size_t n4 = n / 4;
    const float4* u4 = reinterpret_cast<const float4*>(u);
    const float4* t4 = reinterpret_cast<const float4*>(tg);
    float4* d4 = reinterpret_cast<float4*>(dL);
    float a0 = 0.f, c0 = 0.f, a1 = 0.f, c1 = 0.f;
    auto kadd = [](float& acc, float& cmp, float x) {
      const float y = x - cmp;
      const float t2 = acc + y;
      cmp = (t2 - acc) - y;
      acc = t2;
    };
    for (size_t i = tid; i < n4; i += nth) {
      const float4 x = __ldcs(u4 + i), y = __ldcs(t4 + i);
      const float e0 = x.x - y.x, e1 = x.y - y.y, e2 = x.z - y.z, e3 = x.w - y.w;
      __stcs(d4 + i, make_float4(scale * e0, scale * e1, scale * e2, scale * e3));
      kadd(a0, c0, fmaf(e0, e0, e1 * e1));
      kadd(a1, c1, fmaf(e2, e2, e3 * e3));
    }
    s = ((double)a0 - (double)c0) + ((double)a1 - (double)c1);
    done = n4 * 4;
  }
  for (size_t i = done + tid; i < n; i += nth) {
    const float d = u[i] - tg[i];
    s += (double)d * (double)d;
    dL[i] = scale * d;
  }
  s = block_sum_double(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

int launch_loss(const float* usave, const float* target, size_t n, int kind, float* dL,
                double* partial, int nblk, cudaStream_t st) {
  loss_kernel<<<nblk, 256, 0, st>>>(usave, target, n, kind, dL, partial);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Multiple-shooting loss over the packed saves (S x nsave columns, one per
// save of every segment, in segment order; src/multiple_shooting.jl:69-81):
// column j of segment g adds w_g * sum_s (u - d)^2 (w_g = 1 or 1 / (S n_g)),
// and the last column of a segment g whose trajectory continues in segment
// nxt[g] adds cont * sum_s |u[j] - d[first column of nxt[g]]| (the default
// continuity loss, :243). dL is written once per element (the fit term and,
// on a segment's last column, the continuity term of that same column), so
// nothing is accumulated concurrently. One FP64 partial per block.
struct MsLossArgs {
  const float* u;       // S x ncol predictions
  const float* d;       // S x ncol data, same packing
  const int* colseg;    // segment of each column
  const int* segoff;    // first column of each segment
  const int* segn;      // columns of each segment
  const int* nxt;       // next segment of the same trajectory, or -1
  int S, ncol, kind;
  double cont;
  float* dL;
  double* part;
};

__global__ void ms_loss_kernel(MsLossArgs a) {
  __shared__ double red[40];
  const size_t n = (size_t)a.S * a.ncol;
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i / a.S), r = (int)(i - (size_t)j * a.S);
    const int g = a.colseg[j];
    const double w = a.kind == 1 ? 1.0 / ((double)a.S * a.segn[g]) : 1.0;
    const float e = a.u[i] - a.d[i];
    s += w * (double)e * (double)e;
    float gr = (float)(2.0 * w) * e;
    const int nx = a.nxt[g];
    if (nx >= 0 && j == a.segoff[g] + a.segn[g] - 1) {
      const float c = a.u[i] - a.d[(size_t)a.segoff[nx] * a.S + r];
      s += a.cont * fabs((double)c);
      gr += (float)a.cont * (c > 0.f ? 1.f : (c < 0.f ? -1.f : 0.f));
    }
    a.dL[i] = gr;
  }
  s = block_sum_double(s, red);
  if (threadIdx.x == 0) a.part[blockIdx.x] = s;
}

int launch_ms_loss(const float* u, const float* d, const int* colseg, const int* segoff, const int* segn,
                   const int* nxt, int S, int ncol, int kind, double cont, float* dL, double* part, int nblk,
                   cudaStream_t st) {
  MsLossArgs a{u, d, colseg, segoff, segn, nxt, S, ncol, kind, cont, dL, part};
  ms_loss_kernel<<<nblk, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Adam on n parameters: moments in FP32, the update in FP32 with the bias
// corrections c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t) computed on the host.
__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, size_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
    const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

int launch_adam(float* p, float* m, float* v, const float* g, size_t n, double lr, double b1, double b2,
                double eps, long long step, cudaStream_t st) {
  const double c1 = 1.0 / (1.0 - pow(b1, (double)step)), c2 = 1.0 / (1.0 - pow(b2, (double)step));
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 1216);
  adam_kernel<<<blocks, 256, 0, st>>>(p, m, v, g, n, (float)lr, (float)b1, (float)b2, (float)eps, (float)c1,
                                      (float)c2);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---- graph-mode training step helpers ---------------------------------------------
// Inside one captured CUDA graph nothing goes back to the host between the
// solves, so the host-side pieces of an eager step move to the device:

// Backward interval plan from the forward's step log: for each interval
// [t_lo, t_hi] (static, uploaded once) the forward steps covering it. A
// forward that failed, or took more steps than the dense storage holds,
// leaves every interval on step 0 (so the adjoint stays in bounds) and raises
// flags[0]; the host then redoes the step outside the graph.
__global__ void plan_intervals_kernel(Interval* iv, int niv, const double* steplog, const long long* fcounters,
                                      const int* fstatus, long long dense_slots, long long maxsteps, int* flags) {
  const long long ns = fcounters[CT_NACCEPT];
  const bool bad = fstatus[ST_RETCODE] != GBNDE_RET_SUCCESS || ns < 1 || ns >= dense_slots || ns > maxsteps;
  if (blockIdx.x == 0 && threadIdx.x == 0) flags[0] = bad ? 1 : 0;
  for (int k = threadIdx.x; k < niv; k += blockDim.x) {
    int nlo = 0, nhi = 0;
    if (!bad) {
      const double lo = iv[k].t_lo, hi = iv[k].t_hi;
      for (long long n = 0; n < ns; ++n) {
        const double tn = steplog[2 * n];
        if (tn <= lo) nlo = (int)n;
        if (tn < hi) nhi = (int)n;
      }
    }
    iv[k].nlo = nlo;
    iv[k].nhi = nhi;
    iv[k].ckpt = 0;
  }
}

int launch_plan_intervals(Interval* iv, int niv, const double* steplog, const long long* fcounters,
                          const int* fstatus, long long dense_slots, long long maxsteps, int* flags,
                          cudaStream_t st) {
  plan_intervals_kernel<<<1, 128, 0, st>>>(iv, niv, steplog, fcounters, fstatus, dense_slots, maxsteps, flags);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The loss from its per-block partials, in block order (the same sum the
// host forms after an eager step).
__global__ void loss_finalize_kernel(const double* part, int nblk, size_t n, int kind, double* out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nblk; ++i) s += part[i];
    out[0] = (kind == 1) ? s / (double)n : s;
  }
}

int launch_loss_finalize(const double* part, int nblk, size_t n, int kind, double* out, cudaStream_t st) {
  loss_finalize_kernel<<<1, 32, 0, st>>>(part, nblk, n, kind, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Adam with the bias corrections read from device memory (coef[0] =
// 1/(1 - b1^t), coef[1] = 1/(1 - b2^t), written before each graph launch);
// skipped when the forward or the adjoint failed.
__global__ void adam_graph_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                  const float* __restrict__ g, size_t n, float lr, float b1, float b2, float eps,
                                  const double* coef, const int* flags, const int* bstatus) {
  if (flags[0] != 0 || bstatus[ST_RETCODE] != GBNDE_RET_SUCCESS) return;
  const float c1 = (float)coef[0], c2 = (float)coef[1];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
    const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

int launch_adam_graph(float* p, float* m, float* v, const float* g, size_t n, double lr, double b1, double b2,
                      double eps, const double* coef, const int* flags, const int* bstatus, cudaStream_t st) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 1216);
  adam_graph_kernel<<<blocks, 256, 0, st>>>(p, m, v, g, n, (float)lr, (float)b1, (float)b2, (float)eps, coef, flags,
                                            bstatus);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde

// ---- bounded-wait self-test ------------------------------------------------------
// Two CTAs meet at the solvers' grid barrier; with `absent` = 0 or 1 that CTA
// returns first and never arrives, so the other's wait runs out after
// limit_ns and records the barrier timeout, as a solve would report it. No
// fault, no trap: the waiting CTA leaves its loop and the kernel ends.
namespace gbnde {
namespace {
__global__ void barrier_selftest_kernel(unsigned int* counter, int* status, int absent,
                                        unsigned long long limit_ns, unsigned long long* waited) {
  if ((int)blockIdx.x == absent) return;
  unsigned int gen = 0;
  const unsigned long long t0 = globaltimer_ns();
  grid_barrier_ns(counter, gen, status, limit_ns);
  if (threadIdx.x == 0) atomicMax(waited, globaltimer_ns() - t0);
}
}  // namespace
}  // namespace gbnde

extern "C" int gbnde_barrier_selftest(int absent, double limit_ms, int* timed_out, double* waited_ms) {
  if (!timed_out || !waited_ms || absent < -1 || absent > 1 || !(limit_ms > 0.0) || limit_ms > 1000.0)
    return GBNDE_ERR_INVALID;
  struct Blk {
    unsigned int counter;
    int status[gbnde::ST_NSLOTS];
    unsigned long long waited;
  };
  Blk* d = nullptr;
  if (cudaMalloc(&d, sizeof(Blk)) != cudaSuccess) return GBNDE_ERR_NOMEM;
  int rc = GBNDE_OK;
  if (cudaMemset(d, 0, sizeof(Blk)) != cudaSuccess) rc = GBNDE_ERR_CUDA;
  if (rc == GBNDE_OK) {
    unsigned int* counter = &d->counter;
    int* status = d->status;
    unsigned long long* waited = &d->waited;
    unsigned long long limit_ns = (unsigned long long)(limit_ms * 1e6);
    void* args[] = {(void*)&counter, (void*)&status, (void*)&absent, (void*)&limit_ns, (void*)&waited};
    // cooperative: both CTAs are resident, so only the absent one can keep the other waiting
    if (cudaLaunchCooperativeKernel((const void*)gbnde::barrier_selftest_kernel, dim3(2), dim3(64), args, 0,
                                    nullptr) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
      rc = GBNDE_ERR_CUDA;
  }
  Blk h{};
  if (rc == GBNDE_OK && cudaMemcpy(&h, d, sizeof(Blk), cudaMemcpyDeviceToHost) != cudaSuccess) rc = GBNDE_ERR_CUDA;
  cudaFree(d);
  if (rc != GBNDE_OK) return rc;
  *timed_out = h.status[gbnde::ST_BARRIER];
  *waited_ms = (double)h.waited / 1e6;
  return GBNDE_OK;
}
