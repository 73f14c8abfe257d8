// noalloc.cu -- the save-point loss (sum or mean of squared errors and its
// cotangent) for callers that are not allowed to allocate device memory.
//
// Who needs this: real-time loops cannot afford the implicit device-wide
// synchronisation of cudaMalloc/cudaFree in the middle of an iteration, and
// hosts that own every device byte through their own pool (a Julia or Python
// framework's caching allocator with a fixed budget) forbid allocations
// outside it. gbnde_loss_device needs a context, and a context allocates. This
// entry point takes only caller-owned buffers and keeps its scratch (one FP64
// partial sum per chunk of the input) in a fixed array compiled into the
// library.
//
// The call launches a kernel, copies the partial sums to the host and
// synchronises the stream before it returns, so it is an ordinary host-side
// call: it must not be made from a stream callback (a host function enqueued
// with cudaLaunchHostFunc may make no CUDA calls).
//
// The scratch array lives in every device that loads the library, for the
// life of the process (kMaxChunks doubles = 32 KB). All calls on a device
// share it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race on it and may return wrong losses. Every
// partial a call reads is written earlier in the same call, so nothing needs
// clearing between calls.
#include <mutex>

#include "kernels.h"

namespace gbnde {

namespace {

constexpr int kNoAllocThreads = 256;
constexpr long long kChunk = 65536;        // input elements per block
constexpr int kMaxChunks = 4096;           // => at most 2^28 elements per call
constexpr int kMaxDevices = 64;

// File-scope scratch: per-chunk FP64 partial sums of the squared errors.
static __device__ __align__(256) double g_loss_scratch[kMaxChunks];

std::mutex g_mu;
double* g_dev_ptr[kMaxDevices] = {};

// Per-device address of the scratch array (the host symbol is only a
// stand-in): looked up once per device, with that device current.
int scratch_ptr(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBNDE_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GBNDE_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_dev_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_loss_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return GBNDE_ERR_CUDA;
    }
    g_dev_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_dev_ptr[dev];
  return 0;
}

// Block b handles elements [b*kChunk, (b+1)*kChunk): writes dL and the FP64
// partial sum of squared errors of its chunk into scratch[b].
__global__ void __launch_bounds__(kNoAllocThreads) loss_noalloc_kernel(
    const float* __restrict__ u, const float* __restrict__ tg, long long n, float scale,
    float* __restrict__ dL, double* __restrict__ scratch) {
  __shared__ double red[40];
  const long long lo = (long long)blockIdx.x * kChunk;
  const long long hi = lo + kChunk < n ? lo + kChunk : n;
  double s = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const float d = u[i] - tg[i];
    s += (double)d * (double)d;
    dL[i] = scale * d;
  }
  s = block_sum_double(s, red);
  if (threadIdx.x == 0) scratch[blockIdx.x] = s;
}

}  // namespace
}  // namespace gbnde

extern "C" int gbnde_loss_noalloc(const float* u, const float* target, size_t n, int kind,
                                  float* dL, double* loss, void* stream) {
  using namespace gbnde;
  if (!u || !target || !dL || !loss || n == 0) return GBNDE_ERR_INVALID;
  if (kind != 0 && kind != 1) return GBNDE_ERR_INVALID;
  // unsigned comparison: every size_t above the limit is refused (a signed
  // cast would let sizes above LLONG_MAX wrap negative and pass)
  if (n > (size_t)kChunk * (size_t)kMaxChunks) return GBNDE_ERR_UNSUPPORTED;
  double* scratch = nullptr;
  if (int r = scratch_ptr(&scratch)) return r;
  const int nchunks = (int)(((long long)n + kChunk - 1) / kChunk);
  const float scale = (kind == 1) ? (float)(2.0 / (double)n) : 2.f;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  loss_noalloc_kernel<<<nchunks, kNoAllocThreads, 0, st>>>(u, target, (long long)n, scale, dL, scratch);
  if (cudaGetLastError() != cudaSuccess) return GBNDE_ERR_CUDA;
  double part[kMaxChunks];
  if (cudaMemcpyAsync(part, scratch, (size_t)nchunks * sizeof(double), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return GBNDE_ERR_CUDA;
  }
  double s = 0.0;
  for (int b = 0; b < nchunks; ++b) s += part[b];
  *loss = (kind == 1) ? s / (double)n : s;
  return 0;
}
