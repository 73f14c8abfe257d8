// tc_gemm.cu -- weight-image preparation for the tensor-core RHS and a
// self-test GEMM of the tcgen05 building blocks.
//
// Split-BF16 products. A Dense layer z = W a in the BF16 form is evaluated as
//   W_hi a_hi + W_hi a_mid + W_lo a_hi + W_hi a_lo + W_lo a_mid
// with W = W_hi + W_lo and a = a_hi + a_mid + a_lo (bf16 pieces), accumulated
// in FP32 in tensor memory. A single bf16 product would leave ~2^-9 relative
// noise in every stage of the right-hand side; the embedded Tsit5 error
// estimate reads that noise as local error and shrinks the step until it
// drowns it (over 100x more steps at abstol 1e-7). The five products bring the
// noise to the FP32 level.
//
// Weight image: for every layer, K is cut into chunks of 64 (zero padded),
// each chunk stored as two pieces (hi, lo) of N rows x 128 bytes in the
// K-major SW128 layout of the MMA B operand, so one bulk copy moves a chunk.
#include "kernels.h"
#include "tc_ptx.cuh"

namespace gbnde {

// W [N][K] fp32 row-major (K contiguous) -> image [chunk][piece][Npad x 128 B].
__global__ void prep_weight_image_kernel(const float* __restrict__ W, int N, int K, int Npad,
                                         uint8_t* __restrict__ img) {
  const int nchunk = (K + 63) / 64;
  const int total = nchunk * Npad * 8;  // 16-byte groups per piece
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int j = i % 8, n = (i / 8) % Npad, c = i / (8 * Npad);
    float x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = c * 64 + j * 8 + e;
      x[e] = (n < N && k < K) ? W[(size_t)n * K + k] : 0.f;
    }
    uint4 hi = tc::pack8_bf16(x);
    const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&hi);
    float r[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) r[e] = x[e] - __bfloat162float(hb[e]);
    uint4 lo = tc::pack8_bf16(r);
    const size_t piece = (size_t)Npad * 128;
    uint8_t* base = img + (size_t)c * 2 * piece;
    const uint32_t off = tc::sw128_offset(n, j);
    *reinterpret_cast<uint4*>(base + off) = hi;
    *reinterpret_cast<uint4*>(base + piece + off) = lo;
  }
}

int launch_prep_weight_image(const float* W, int N, int K, int Npad, uint8_t* img,
                             cudaStream_t st) {
  prep_weight_image_kernel<<<128, 256, 0, st>>>(W, N, K, Npad, img);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---- self-test: D[128 x N] = A[128 x K] W[N x K]^T ---------------------------------
// mode 0: single bf16 product; mode 1: the five split products.
__global__ void __launch_bounds__(256, 1) tc_selftest_kernel(const float* __restrict__ A,
                                                             const uint8_t* __restrict__ img,
                                                             int N, int K, int mode,
                                                             float* __restrict__ D, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;                   // 3 pieces x 16 KB
  uint8_t* sB = smem + 3 * 16384;       // 2 pieces x N*128
  __shared__ uint64_t bar_b, bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
  if (tid == 0) {
    s_err = 0;
    tc::mbar_init(&bar_b, 1);
    tc::mbar_init(&bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_bf16(128, N);
  const size_t piece = (size_t)N * 128;
  const int nchunk = (K + 63) / 64;
  volatile int* verr = &s_err;
  for (int c = 0; c < nchunk && !*verr; ++c) {
    // A chunk: row r = tid/2, 32 columns per thread, split into pieces
    {
      const int r = tid >> 1, half = tid & 1;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = half * 4 + q;
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int k = c * 64 + j * 8 + e;
          x[e] = (k < K) ? A[(size_t)r * K + k] : 0.f;
        }
        uint4 hi, mid, lo;
        tc::split3_bf16(x, hi, mid, lo);
        const uint32_t off = tc::sw128_offset(r, j);
        *reinterpret_cast<uint4*>(sA + off) = hi;
        *reinterpret_cast<uint4*>(sA + 16384 + off) = mid;
        *reinterpret_cast<uint4*>(sA + 32768 + off) = lo;
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::mbar_arrive_expect_tx(&bar_b, (uint32_t)(2 * piece));
      tc::bulk_g2s(sB, img + (size_t)c * 2 * piece, (uint32_t)(2 * piece), &bar_b);
      if (tc::mbar_wait(&bar_b, c & 1, verr)) {
        tc::tc_fence_after();
        const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
        // (A piece, B piece) pairs
        const int pa[5] = {0, 1, 0, 2, 1};
        const int pb[5] = {0, 0, 1, 0, 1};
        const int nprod = mode == 0 ? 1 : 5;
        for (int pr = 0; pr < nprod; ++pr) {
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = tc::sdesc_sw128(a0 + pa[pr] * 16384 + kk * 32);
            const uint64_t bd = tc::sdesc_sw128(b0 + pb[pr] * (uint32_t)piece + kk * 32);
            tc::mma_bf16(tmem, ad, bd, idesc, (c > 0 || pr > 0 || kk > 0) ? 1u : 0u);
          }
        }
        tc::mma_commit(&bar_mma);
      }
    }
    __syncthreads();
    tc::mbar_wait(&bar_mma, c & 1, verr);
    tc::tc_fence_after();
    __syncthreads();
  }
  // drain: warps 0..3 read their 32 lanes
  if (warp < 4 && !*verr) {
    for (int cb = 0; cb < N; cb += 32) {
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
      const int r = warp * 32 + lane;
      for (int i = 0; i < 32 && cb + i < N; ++i) D[(size_t)r * N + cb + i] = v[i];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
  if (tid == 0) *err = s_err;
}

// ---- self-test of MN-major operands (the weight-gradient products) -----------------
// D[128 x N] = G^T A where G is [128 (K) x 128 (M)] and A is [128 (K) x N],
// both stored trajectory-major: per 64-wide K chunk, per piece, MN blocks of
// 64 columns (64 rows x 128 B each, SW128). Products: hi.hi + hi.lo + lo.hi.
__global__ void __launch_bounds__(256, 1) tc_selftest_mn_kernel(const float* __restrict__ G,
                                                                const float* __restrict__ A, int N,
                                                                float* __restrict__ D, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nbA = 2, nbB = N / 64;
  uint8_t* sA = smem;                       // 2 pieces x nbA blocks x 8 KB
  uint8_t* sB = smem + 2 * nbA * 8192;      // 2 pieces x nbB blocks x 8 KB
  __shared__ uint64_t bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    s_err = 0;
    tc::mbar_init(&bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 256);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  volatile int* verr = &s_err;
  for (int kc = 0; kc < 2; ++kc) {
    // rows k in [64kc, 64kc+64): thread -> (row, 16-byte group)
    for (int idx = tid; idx < 64 * (128 / 8); idx += 256) {
      const int r = idx / 16, j = idx % 16;  // j: 16-byte group across 128 columns
      float x[8];
      for (int e = 0; e < 8; ++e) x[e] = G[(size_t)(64 * kc + r) * 128 + 8 * j + e];
      uint4 hi = tc::pack8_bf16(x);
      const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&hi);
      float rr[8];
      for (int e = 0; e < 8; ++e) rr[e] = x[e] - __bfloat162float(hb[e]);
      uint4 lo = tc::pack8_bf16(rr);
      const int blk = j / 8, jj = j % 8;
      const uint32_t off = blk * 8192 + tc::sw128_offset(r, jj);
      *reinterpret_cast<uint4*>(sA + off) = hi;
      *reinterpret_cast<uint4*>(sA + nbA * 8192 + off) = lo;
    }
    for (int idx = tid; idx < 64 * (N / 8); idx += 256) {
      const int r = idx / (N / 8), j = idx % (N / 8);
      float x[8];
      for (int e = 0; e < 8; ++e) x[e] = A[(size_t)(64 * kc + r) * N + 8 * j + e];
      uint4 hi = tc::pack8_bf16(x);
      const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&hi);
      float rr[8];
      for (int e = 0; e < 8; ++e) rr[e] = x[e] - __bfloat162float(hb[e]);
      uint4 lo = tc::pack8_bf16(rr);
      const int blk = j / 8, jj = j % 8;
      const uint32_t off = blk * 8192 + tc::sw128_offset(r, jj);
      *reinterpret_cast<uint4*>(sB + off) = hi;
      *reinterpret_cast<uint4*>(sB + nbB * 8192 + off) = lo;
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
      const uint32_t idesc = tc::idesc_bf16_mn(128, N);
      const int pa[3] = {0, 0, 1};
      const int pb[3] = {0, 1, 0};
      for (int pr = 0; pr < 3; ++pr)
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ad = tc::sdesc_sw128_mn(a0 + pa[pr] * nbA * 8192 + kk * 2048, 8192);
          const uint64_t bd = tc::sdesc_sw128_mn(b0 + pb[pr] * nbB * 8192 + kk * 2048, 8192);
          tc::mma_bf16(tmem, ad, bd, idesc, (kc > 0 || pr > 0 || kk > 0) ? 1u : 0u);
        }
      tc::mma_commit(&bar_mma);
    }
    __syncthreads();
    tc::mbar_wait(&bar_mma, kc & 1, verr);
    tc::tc_fence_after();
    __syncthreads();
  }
  if (warp < 4 && !*verr) {
    for (int cb = 0; cb < N; cb += 32) {
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
      const int r = warp * 32 + lane;
      for (int i = 0; i < 32; ++i) D[(size_t)r * N + cb + i] = v[i];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
  if (tid == 0) *err = s_err;
}

}  // namespace gbnde

extern "C" int gbnde_tc_selftest(const float* A, const float* W, int N, int K, int mode, float* D) {
  using namespace gbnde;
  if (!A || !W || !D || (N != 64 && N != 128 && N != 256) || K < 1 || K > 1024 || mode < 0 || mode > 2)
    return GBNDE_ERR_INVALID;
  if (mode == 2 && K != 128) return GBNDE_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GBNDE_ERR_CUDA;
  }
  const int nchunk = (K + 63) / 64;
  float *dA = nullptr, *dW = nullptr, *dD = nullptr;
  uint8_t* img = nullptr;
  int* derr = nullptr;
  int rc = GBNDE_OK;
  const size_t imgbytes = (size_t)nchunk * 2 * N * 128;
  const size_t smem = 1024 + 3 * 16384 + 2 * (size_t)N * 128;
  if (cudaMalloc(&dA, 128 * (size_t)K * 4) || cudaMalloc(&dW, (size_t)N * K * 4) ||
      cudaMalloc(&dD, 128 * (size_t)N * 4) || cudaMalloc(&img, imgbytes) || cudaMalloc(&derr, 4)) {
    rc = GBNDE_ERR_NOMEM;
  } else {
    cudaMemcpy(dA, A, 128 * (size_t)K * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dW, W, (size_t)N * K * 4, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 4);
    cudaMemset(dD, 0, 128 * (size_t)N * 4);
    if (mode == 2) {
      // A: K x 128 (rows k, columns m), W: K x N
      const size_t smem2 = 1024 + 2 * 2 * 8192 + 2 * (size_t)(N / 64) * 8192;
      cudaFuncSetAttribute(tc_selftest_mn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
      tc_selftest_mn_kernel<<<1, 256, smem2>>>(dA, dW, N, dD, derr);
    } else {
      launch_prep_weight_image(dW, N, K, N, img, 0);
      cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      tc_selftest_kernel<<<1, 256, smem>>>(dA, img, N, K, mode, dD, derr);
    }
    int herr = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) {
      rc = GBNDE_ERR_CUDA;
    } else {
      cudaMemcpy(D, dD, 128 * (size_t)N * 4, cudaMemcpyDeviceToHost);
      cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
      if (herr) rc = GBNDE_ERR_TIMEOUT;
    }
  }
  cudaFree(dA);
  cudaFree(dW);
  cudaFree(dD);
  cudaFree(img);
  cudaFree(derr);
  return rc;
}

// ---- activation self-test: the tensor-core epilogue's activation beside the
// library's (tanhf / log1pf(expf)) on the same inputs ------------------------
namespace gbnde {
__global__ void act_selftest_kernel(const float* __restrict__ x, int n, int act, float* __restrict__ ytc,
                                    float* __restrict__ ylib) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ytc[i] = act_apply_tc(x[i], act);
  ylib[i] = act_apply(x[i], act);
}
}  // namespace gbnde

extern "C" int gbnde_act_selftest(const float* x, int n, int act, float* y_tc, float* y_lib) {
  using namespace gbnde;
  if (!x || !y_tc || !y_lib || n < 1 || act < GBNDE_ACT_IDENTITY || act > GBNDE_ACT_SOFTPLUS)
    return GBNDE_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GBNDE_ERR_CUDA;
  }
  float *dx = nullptr, *d1 = nullptr, *d2 = nullptr;
  const size_t bytes = (size_t)n * 4;
  int rc = GBNDE_OK;
  if (cudaMalloc(&dx, bytes) || cudaMalloc(&d1, bytes) || cudaMalloc(&d2, bytes)) {
    rc = GBNDE_ERR_NOMEM;
  } else if (cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = GBNDE_ERR_CUDA;
  } else {
    act_selftest_kernel<<<(n + 255) / 256, 256>>>(dx, n, act, d1, d2);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(y_tc, d1, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(y_lib, d2, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = GBNDE_ERR_CUDA;
  }
  cudaFree(dx);
  cudaFree(d1);
  cudaFree(d2);
  cudaGetLastError();
  return rc;
}
