// mlp_simt.cuh -- FP32 SIMT evaluation of the Lux Dense chain on a tile of
// trajectories held in shared memory (the plain-FP32 form of the right-hand
// side `dudt(u, p, t) = model(u, p)`, src/neural_de.jl:50).
//
// Tile layout in shared memory: feature-major, buf[f * LD + m] for feature f
// and trajectory m of the tile (LD = TM + 4). A Dense layer y = act(W x + b)
// reads the weight in the Lux memory order, W^T as [in][out] (the column-major
// out x in matrix of ComponentArray(ps)), so a thread's output columns are
// contiguous in global memory.
#pragma once
#include "common.cuh"

namespace gbnde {

struct MlpDev {
  int nlayers;
  int dims[GBNDE_MAX_LAYERS + 1];
  int act[GBNDE_MAX_LAYERS];
  int cube;
  int timein;
  int maxdim;
  const float* Wt[GBNDE_MAX_LAYERS];    // [in][out]  (Lux order)
  const float* W[GBNDE_MAX_LAYERS];     // [out][in]  (transposed copy, for VJPs)
  const float* bias[GBNDE_MAX_LAYERS];
  long long woff[GBNDE_MAX_LAYERS];     // offset of layer weight in the flat vector
  long long boff[GBNDE_MAX_LAYERS];     // offset of layer bias in the flat vector
};

// out[n][m] = act(sum_k Wt[k][n] * in[k][m] + b[n]) for rows m < TM, cols n < N.
// Thread micro-tile: RM trajectories x RN outputs.
template <int RM, int RN>
__device__ __forceinline__ void dense_fwd_tile(const float* __restrict__ Wt,
                                               const float* __restrict__ bias, int K, int N,
                                               int act, const float* in_s, float* out_s, int LD,
                                               int TM) {
  const int rgroups = TM / RM;
  const int cgroups = blockDim.x / rgroups;
  const int tm = threadIdx.x % rgroups, tn = threadIdx.x / rgroups;
  const int m0 = tm * RM;
  const bool vecw = (RN % 4 == 0) && ((N & 3) == 0) && ((reinterpret_cast<uintptr_t>(Wt) & 15) == 0);
  for (int nbase = 0; nbase < N; nbase += cgroups * RN) {
    const int n0 = nbase + tn * RN;
    if (n0 >= N) continue;
    float acc[RM][RN];
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < RN; ++j) acc[i][j] = 0.f;
    const bool full = (n0 + RN <= N);
    for (int k = 0; k < K; ++k) {
      float a[RM], w[RN];
      const float* ip = in_s + k * LD + m0;
#pragma unroll
      for (int i = 0; i < RM; i += 4) {
        const float4 v = *reinterpret_cast<const float4*>(ip + i);
        a[i] = v.x; a[i + 1] = v.y; a[i + 2] = v.z; a[i + 3] = v.w;
      }
      const float* wp = Wt + (size_t)k * N + n0;
      if (vecw && full) {
#pragma unroll
        for (int j = 0; j < RN; j += 4) {
          const float4 v = __ldg(reinterpret_cast<const float4*>(wp + j));
          w[j] = v.x; w[j + 1] = v.y; w[j + 2] = v.z; w[j + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int j = 0; j < RN; ++j) w[j] = (n0 + j < N) ? __ldg(wp + j) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
    }
    with_act(act, [&](auto A) {
#pragma unroll
      for (int j = 0; j < RN; ++j) {
        if (n0 + j < N) {
          const float bb = bias ? __ldg(bias + n0 + j) : 0.f;
          float* op = out_s + (n0 + j) * LD + m0;
#pragma unroll
          for (int i = 0; i < RM; i += 4) {
            float4 v;
            v.x = A.f(acc[i][j] + bb);
            v.y = A.f(acc[i + 1][j] + bb);
            v.z = A.f(acc[i + 2][j] + bb);
            v.w = A.f(acc[i + 3][j] + bb);
            *reinterpret_cast<float4*>(op + i) = v;
          }
        }
      }
    });
  }
}

// Skinny layers (few outputs, long K; small batches such as the batch-1
// spiral fit): each output (trajectory m, column n) is summed by a group of G
// lanes of one warp over a strided share of K and reduced with shuffles in a
// fixed order, so that a long dot product is not one thread's serial chain.
// Every lane of a warp runs the same number of rounds (the shuffles need the
// whole warp); lanes past the last output compute nothing.
template <int G>
__device__ __forceinline__ void dense_fwd_splitk(const float* __restrict__ Wt, const float* __restrict__ bias,
                                                 int K, int N, int act, const float* in_s, float* out_s,
                                                 int LD, int TM) {
  const int lg = threadIdx.x % G, grp = threadIdx.x / G, ngrp = blockDim.x / G;
  const int nout = N * TM;
  with_act(act, [&](auto A) {
    for (int ob = 0; ob < nout; ob += ngrp) {
      const int o = ob + grp;
      const bool mine = o < nout;
      const int n = mine ? o / TM : 0, m = mine ? o - (o / TM) * TM : 0;
      float sum = 0.f;
      if (mine)
        for (int k = lg; k < K; k += G) sum = fmaf(in_s[k * LD + m], __ldg(Wt + (size_t)k * N + n), sum);
#pragma unroll
      for (int off = G / 2; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off, G);
      if (mine && lg == 0) out_s[n * LD + m] = A.f(sum + (bias ? __ldg(bias + n) : 0.f));
    }
  });
}

__device__ __forceinline__ void dense_fwd(const float* Wt, const float* bias, int K, int N, int act,
                                          const float* in_s, float* out_s, int LD, int TM) {
  const int rgroups = TM / 8;
  const int cgroups = blockDim.x / rgroups;
  // few outputs per thread and a long K: split K over lanes (the rounds of
  // the per-thread path would be one thread's K-long serial chain)
  if (K >= 16 && N * TM * 4 <= (int)blockDim.x) {
    const int per = (int)blockDim.x / (N * TM);
    if (per >= 32) dense_fwd_splitk<32>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
    else if (per >= 16) dense_fwd_splitk<16>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
    else if (per >= 8) dense_fwd_splitk<8>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
    else dense_fwd_splitk<4>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
    return;
  }
  if (N >= cgroups * 8)
    dense_fwd_tile<8, 8>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
  else if (N >= cgroups * 4)
    dense_fwd_tile<8, 4>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
  else if (N >= cgroups * 2)
    dense_fwd_tile<8, 2>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
  else
    dense_fwd_tile<8, 1>(Wt, bias, K, N, act, in_s, out_s, LD, TM);
}

// Whole chain on the tile. Input in bufA rows [0, dims[0]); when keep != null,
// layer l's output goes to keep[l] (distinct buffers, for the VJP); otherwise
// the two buffers alternate. Returns the buffer holding the output.
__device__ __forceinline__ float* mlp_fwd_tile(const MlpDev& m, float* bufA, float* bufB, int LD,
                                               int TM, float** keep) {
  float* in = bufA;
  float* out = bufB;
  for (int l = 0; l < m.nlayers; ++l) {
    if (keep) out = keep[l];
    dense_fwd(m.Wt[l], m.bias[l], m.dims[l], m.dims[l + 1], m.act[l], in, out, LD, TM);
    __syncthreads();
    if (keep) {
      in = out;
    } else {
      float* t = in;
      in = out;
      out = t;
    }
  }
  return in;
}


// P[k*N + n] += c * sum_m g[n][m] * a[k][m] for n < N, k < K: the batch-summed
// weight gradient of one Dense layer (Lux order: element (out n, in k) of the
// column-major out x in weight sits at k*N + n). Each thread owns 8 x 8
// micro-tiles; lanes take consecutive n so the read-modify-write is coalesced.
__device__ __forceinline__ void dw_accum(float* __restrict__ P, const float* g, const float* a,
                                         int N, int K, int LD, int TM, float c) {
  const int tnc = (N + 7) >> 3, tkc = (K + 7) >> 3;
  for (int mt = threadIdx.x; mt < tnc * tkc; mt += blockDim.x) {
    const int n0 = (mt % tnc) * 8, k0 = (mt / tnc) * 8;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int m = 0; m < TM; m += 4) {
      float4 gv[8], av[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        gv[i] = *reinterpret_cast<const float4*>(g + min(n0 + i, N - 1) * LD + m);
        av[i] = *reinterpret_cast<const float4*>(a + min(k0 + i, K - 1) * LD + m);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float s = acc[i][j];
          s = fmaf(gv[i].x, av[j].x, s);
          s = fmaf(gv[i].y, av[j].y, s);
          s = fmaf(gv[i].z, av[j].z, s);
          s = fmaf(gv[i].w, av[j].w, s);
          acc[i][j] = s;
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (k0 + j >= K) continue;
      float* row = P + (size_t)(k0 + j) * N;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (n0 + i < N) row[n0 + i] += c * acc[i][j];
    }
  }
}

// P[n] += c * sum_m g[n][m]: the batch-summed bias gradient.
__device__ __forceinline__ void db_accum(float* __restrict__ P, const float* g, int N, int LD,
                                         int TM, float c) {
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    float s = 0.f;
    for (int m = 0; m < TM; ++m) s += g[n * LD + m];
    P[n] += c * s;
  }
}

// Vector-Jacobian product of the chain on a tile. act[0..L] hold the layer
// inputs/outputs of the forward pass (act[0] = chain input), gA holds the
// cotangent of the output (rows [0, dims[L])). When P != null the parameter
// cotangent (weights and biases, Lux order) is accumulated into P scaled by
// c. Returns the buffer holding the cotangent of the chain input
// (rows [0, dims[0])).
__device__ __forceinline__ float* mlp_vjp_tile(const MlpDev& m, float* const* act, float* gA,
                                               float* gB, int LD, int TM, float* P, float c) {
  float* g = gA;
  float* o = gB;
  for (int l = m.nlayers - 1; l >= 0; --l) {
    const int N = m.dims[l + 1], K = m.dims[l];
    if (m.act[l] != GBNDE_ACT_IDENTITY) {
      const float* y = act[l + 1];
      with_act(m.act[l], [&](auto A) {
        for (int e = threadIdx.x; e < N * TM; e += blockDim.x) {
          const int n = e / TM, mm = e - n * TM;
          g[n * LD + mm] *= A.d(y[n * LD + mm]);
        }
      });
      __syncthreads();
    }
    if (P) {
      dw_accum(P + m.woff[l], g, act[l], N, K, LD, TM, c);
      db_accum(P + m.boff[l], g, N, LD, TM, c);
    }
    // o[k][m] = sum_n W[n][k] g[n][m]
    dense_fwd(m.W[l], nullptr, N, K, GBNDE_ACT_IDENTITY, g, o, LD, TM);
    __syncthreads();
    float* t = g;
    g = o;
    o = t;
  }
  return g;
}


// ---- FFJORD: directional derivative and its reverse pass ------------------------------
//
// act'' from the output y: tanh -> -2 y (1 - y^2); softplus -> s (1 - s) with
// s = 1 - exp(-y); identity -> 0.
__device__ __forceinline__ float act_deriv2_from_out(float y, int act) {
  if (act == GBNDE_ACT_TANH) return -2.f * y * (1.f - y * y);
  if (act == GBNDE_ACT_SOFTPLUS) {
    const float sg = -expm1f(-y);
    return sg * (1.f - sg);
  }
  return 0.f;
}

// Tangent of the chain along the input direction held in zd[0] (feature-major,
// rows [0, dims[0])): zd[l+1] = W_l adot_l with adot_0 = zd[0] and
// adot_l = act'(act[l]) * zd[l] for l >= 1. act[0..L] must hold the primal
// activations. tmp: one buffer of maxdim rows.
__device__ __forceinline__ void mlp_tangent_tile(const MlpDev& m, float* const* act, float* const* zd,
                                                 float* tmp, int LD, int TM) {
  for (int l = 0; l < m.nlayers; ++l) {
    const int K = m.dims[l];
    const float* in = zd[0];
    if (l > 0) {
      with_act(m.act[l - 1], [&](auto A) {
        for (int e = threadIdx.x; e < K * TM; e += blockDim.x) {
          const int k = e / TM, mm = e - k * TM;
          tmp[k * LD + mm] = A.d(act[l][k * LD + mm]) * zd[l][k * LD + mm];
        }
      });
      __syncthreads();
      in = tmp;
    }
    dense_fwd(m.Wt[l], nullptr, K, m.dims[l + 1], GBNDE_ACT_IDENTITY, in, zd[l + 1], LD, TM);
    __syncthreads();
  }
}

// P[k*N + n] += c * sum_m g[n][m] * (act'(y[k][m]) * x[k][m]) : the weight
// gradient of the tangent chain (operand adot = act'(y) * zdot).
__device__ __forceinline__ void dw_accum_scaled(float* __restrict__ P, const float* g, const float* x,
                                                const float* y, int actcode, int N, int K, int LD,
                                                int TM, float c) {
  const int tnc = (N + 7) >> 3, tkc = (K + 7) >> 3;
  with_act(y ? actcode : GBNDE_ACT_IDENTITY, [&](auto A) {
  for (int mt = threadIdx.x; mt < tnc * tkc; mt += blockDim.x) {
    const int n0 = (mt % tnc) * 8, k0 = (mt / tnc) * 8;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int mm = 0; mm < TM; ++mm) {
      float gv[8], av[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        gv[i] = g[min(n0 + i, N - 1) * LD + mm];
        const int kk = min(k0 + i, K - 1) * LD + mm;
        av[i] = (y ? A.d(y[kk]) : 1.f) * x[kk];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(gv[i], av[j], acc[i][j]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (k0 + j >= K) continue;
      float* row = P + (size_t)(k0 + j) * N;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (n0 + i < N) row[n0 + i] += c * acc[i][j];
    }
  }
  });
}

// Reverse pass through the primal chain and its tangent (reverse over forward).
// Inputs: act[0..L] primal activations, zd[0..L] tangents (zd[0] = input
// direction), abar (rows dims[L]) cotangent of the primal output, tbar (rows
// dims[L]) cotangent of the tangent output. Buffers abar/abar2 and tbar/tbar2
// are ping-pong pairs of maxdim rows. Accumulates the parameter cotangent
// into P scaled by c (when P != null). Returns the buffer with the cotangent
// of the primal input (rows dims[0]).
__device__ __forceinline__ float* ffjord_vjp_tile(const MlpDev& m, float* const* act, float* const* zd,
                                                  float* abar, float* abar2, float* tbar, float* tbar2,
                                                  int LD, int TM, float* P, float c) {
  for (int l = m.nlayers - 1; l >= 0; --l) {
    const int N = m.dims[l + 1], K = m.dims[l];
    const int code = m.act[l];
    const float* y = act[l + 1];
    const float* zl = zd[l + 1];
    // tbar <- tbar * act'(y) (= zdot bar); abar <- tbar_in * act''(y) * zdot + abar * act'(y) (= z bar)
    with_act(code, [&](auto A) {
      for (int e = threadIdx.x; e < N * TM; e += blockDim.x) {
        const int n = e / TM, mm = e - n * TM, o = n * LD + mm;
        const float d1 = A.d(y[o]), d2 = A.d2(y[o]);
        const float tb = tbar[o];
        abar[o] = fmaf(tb * d2, zl[o], abar[o] * d1);
        tbar[o] = tb * d1;
      }
    });
    __syncthreads();
    if (P) {
      dw_accum(P + m.woff[l], abar, act[l], N, K, LD, TM, c);
      dw_accum_scaled(P + m.woff[l], tbar, zd[l], l > 0 ? act[l] : nullptr, l > 0 ? m.act[l - 1] : 0, N, K,
                      LD, TM, c);
      db_accum(P + m.boff[l], abar, N, LD, TM, c);
    }
    __syncthreads();
    dense_fwd(m.W[l], nullptr, N, K, GBNDE_ACT_IDENTITY, abar, abar2, LD, TM);
    dense_fwd(m.W[l], nullptr, N, K, GBNDE_ACT_IDENTITY, tbar, tbar2, LD, TM);
    __syncthreads();
    float* t1 = abar;
    abar = abar2;
    abar2 = t1;
    float* t2 = tbar;
    tbar = tbar2;
    tbar2 = t2;
  }
  return abar;
}

}  // namespace gbnde
