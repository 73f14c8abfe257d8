// common.cuh -- pieces shared by the GB300 neural-ODE kernels:
// Tsit5 tableau in constant memory, the PI step-size controller, the bounded
// grid barrier of the persistent kernels and FP64 block reductions.
//
// Tableau: Tsitouras (2011) 5(4) pair with its free 4th-order interpolant, the
// method OrdinaryDiffEq calls Tsit5 (what the reference passes as `alg`,
// test/BasicNeuralDE/neural_de_tests.jl:43). Controller: PI control with
// beta1 = 7/50, beta2 = 2/25, qmin = 1/5, qmax = 10, gamma = 9/10,
// qoldinit = 1e-4 (the integrator's documented defaults for order 5).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbnde.h"

namespace gbnde {

// ---------------------------------------------------------------------------
// Tableau (host copies; the kernels read the __constant__ mirrors)
// ---------------------------------------------------------------------------
struct Tableau {
  double c[7];
  double a[7][7];
  double b[7];
  double btilde[7];
  double r[7][4];  // b_i(theta) = sum_m r[i][m] theta^(m+1)
};

// Each translation unit holds its own initialised copy (no relocatable device
// code needed). Values: Tsitouras (2011), btilde = b - bhat.
static __constant__ Tableau c_tab = {
    {0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0},
    {{0, 0, 0, 0, 0, 0, 0},
     {0.161, 0, 0, 0, 0, 0, 0},
     {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0, 0},
     {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0, 0},
     {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0, 0},
     {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401,
      -0.028269050394068383, 0, 0},
     {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
      2.324710524099774, 0}},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
     2.324710524099774, 0.0},
    {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
     -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 1.0 / 66.0},
    {{1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216},
     {0.0, 0.13169999999999998, -0.2234, 0.1017},
     {0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253},
     {0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902},
     {0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928},
     {0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661},
     {0.0, 1.5, -4.0, 2.5}},
};

constexpr double kBeta1 = 7.0 / 50.0;
constexpr double kBeta2 = 2.0 / 25.0;
constexpr double kQmin = 1.0 / 5.0;
constexpr double kQmax = 10.0;
constexpr double kGamma = 9.0 / 10.0;
constexpr double kQoldInit = 1.0e-4;

// Device-side status words (one int array per launch).
enum StatusSlot { ST_RETCODE = 0, ST_BARRIER = 1, ST_NSLOTS = 4 };

// Barrier wait limit (nanoseconds of %globaltimer) before the kernel gives up.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier for a cooperative (co-resident) launch. `counter` starts
// at 0 for the launch; generation g waits for g*gridDim.x arrivals. Waits at
// most kBarrierTimeoutNs, then records ST_BARRIER and returns false; every
// caller then leaves its loop, so the kernel ends instead of hanging.
__device__ __forceinline__ bool grid_barrier_ns(unsigned int* counter, unsigned int& gen, int* status,
                                                unsigned long long limit_ns) {
  __syncthreads();
  gen += 1;
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(counter, 1u);
    const unsigned int target = gen * gridDim.x;
    const unsigned long long t_start = globaltimer_ns();
    int ok = 1;
    while (ld_acquire_u32(counter) < target) {
      if (*((volatile int*)&status[ST_BARRIER]) != 0) { ok = 0; break; }
      if (globaltimer_ns() - t_start > limit_ns) {
        atomicExch(&status[ST_BARRIER], 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(unsigned int* counter, unsigned int& gen, int* status) {
  return grid_barrier_ns(counter, gen, status, kBarrierTimeoutNs);
}

// Deterministic block sum of a double: warp butterflies (commutative pairs give
// bit-identical results in every lane) then a fixed-order pass over warps.
__device__ __forceinline__ double block_sum_double(double v, double* scratch /* >= 32 */) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < nw; ++i) s += scratch[i];
    scratch[32] = s;
  }
  __syncthreads();
  s = scratch[32];
  __syncthreads();
  return s;
}

// Sum of per-CTA partials written before a grid barrier, in the same order in
// every CTA, so that every CTA takes the same controller decision.
__device__ __forceinline__ double grid_partials_sum(const double* partials, int n,
                                                    double* scratch) {
  double v = 0.0;
  if (threadIdx.x < 32) {
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(partials + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) scratch[33] = v;
  }
  __syncthreads();
  v = scratch[33];
  __syncthreads();
  return v;
}

// The value x as the nearest Float32 when `on` (the Float32-time mode: t, dt,
// the error estimate and qold are kept as Float32 values), else unchanged.
__device__ __forceinline__ double rt32(double x, int on) { return on ? (double)(float)x : x; }

// The step controller's scalar FP64 work (step size, stage coefficients and
// times, the norm's square root, the PI update, save weights) runs on one
// thread of a CTA: FP64 executes at a small fraction of the FP32 rate on this
// GPU, and every warp of the CTA would repeat it. The results reach the other
// threads through this block of shared memory, read after a barrier.
struct StepCtl {
  double t, h, habs, tnew, d1, dt0;
  double tst[7];  // stage times (tst[0]: the initial step's probe time)
  float ha[6][6], hbt[7], hb[7], hf;
  int go, clipped, accept, ret, nsv, need_ckpt, exact;
};

// PI controller (FP64). Returns q, writes q11.
__device__ __forceinline__ double pi_q(double eest, double qold, double* q11) {
  if (eest == 0.0) {
    *q11 = 0.0;
    return 1.0 / kQmax;
  }
  const double a = pow(eest, kBeta1);
  *q11 = a;
  double q = a / pow(qold, kBeta2);
  q = fmax(1.0 / kQmax, fmin(1.0 / kQmin, q / kGamma));
  return q;
}

__device__ __forceinline__ float act_apply(float z, int act) {
  if (act == GBNDE_ACT_TANH) return tanhf(z);
  if (act == GBNDE_ACT_SOFTPLUS) return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));
  return z;
}

// tanh for the tensor-core epilogues from the identity
//   tanh x = sign(x) (1 - 2 / (exp(2|x|) + 1)),
// with exp(2|x|) = 2^(2|x| / ln 2) from the ex2.approx instruction and
// 1/(e + 1) from rcp.approx refined by one Newton step (q <- q (2 - d q)).
// Branch-free: 8 instructions, 2 of them on the special-function unit.
// Its error is absolute, a few units of 2^-24 (largest near 0, where the
// relative error grows like 2^-24/|x|): the size of the FP32 rounding of
// O(1) activations, which is what the next layer's GEMM sees. Tested against
// the library tanhf over [-12, 12].
__device__ __forceinline__ float tanh_tc(float x) {
  const float ax = fabsf(x);
  // clamp keeps exp finite (tanh(10) rounds to 1) and lets NaN through
  const float axc = ax > 10.f ? 10.f : ax;
  float e, q;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(axc * 2.8853900817779268f));  // 2/ln 2
  const float d = e + 1.f;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q) : "f"(d));
  q = q * fmaf(-d, q, 2.f);
  return copysignf(fmaf(-2.f, q, 1.f), x);
}

__device__ __forceinline__ float act_apply_tc(float z, int act) {
  if (act == GBNDE_ACT_TANH) return tanh_tc(z);
  if (act == GBNDE_ACT_SOFTPLUS) return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));
  return z;
}

// Activations as types, so that a loop over elements can be compiled for one
// activation: `with_act(code, [&](auto A) { ... A.f(z) ... A.d(y) ... })`
// takes the branch on the (uniform) activation code once, outside the loop.
// With the code tested per element, the compiler evaluates every
// activation's formula for every element and selects.
// f: the activation; d: act'(z) from the output y; d2: act''(z) from y.
struct ActIdentity {
  __device__ __forceinline__ float f(float z) const { return z; }
  __device__ __forceinline__ float d(float) const { return 1.f; }
  __device__ __forceinline__ float d2(float) const { return 0.f; }
};
struct ActTanh {
  __device__ __forceinline__ float f(float z) const { return tanhf(z); }
  __device__ __forceinline__ float d(float y) const { return 1.f - y * y; }
  __device__ __forceinline__ float d2(float y) const { return -2.f * y * (1.f - y * y); }
};
struct ActSoftplus {
  __device__ __forceinline__ float f(float z) const { return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))); }
  __device__ __forceinline__ float d(float y) const { return -expm1f(-y); }
  __device__ __forceinline__ float d2(float y) const {
    const float sg = -expm1f(-y);
    return sg * (1.f - sg);
  }
};
template <class F>
__device__ __forceinline__ void with_act(int act, F&& fn) {
  if (act == GBNDE_ACT_TANH) fn(ActTanh{});
  else if (act == GBNDE_ACT_SOFTPLUS) fn(ActSoftplus{});
  else fn(ActIdentity{});
}


// Free interpolant weights b_i(theta) (FP64 in, FP32 out).
__device__ __forceinline__ void interp_weights(double th, float* bw) {
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    const double* r = c_tab.r[i];
    bw[i] = (float)(th * (r[0] + th * (r[1] + th * (r[2] + th * r[3]))));
  }
}

}  // namespace gbnde
