// bwd_tcw.cu -- persistent InterpolatingAdjoint solve, BF16 tensor-core form,
// in stash mode: state dim up to 256, widths up to 1024, optional time row.
//
// The algorithm is that of bwd_tc.cu (the pullback of SciMLSensitivity's rrule
// on `solve` for sensealg = InterpolatingAdjoint(), src/neural_de.jl:57):
// reverse-time Tsit5 on lam with the PI controller over lam, the save points
// as stops where lam jumps by dL/du(t_i), u(t) from the forward's dense stage
// storage, and the parameter quadrature mu with the Tsit5 weights over
// accepted steps -- weight gradients as stage-stacked products once per
// accepted step (K = 6 stages x 128 trajectories per tile), bias gradients as
// column sums into per-CTA pending buffers, Kahan-compensated mu.
//
// What differs from the single-accumulator kernel:
//  * every chain operand (layer inputs a_l of the forward recompute, the
//    cotangents delta_{l+1} of the VJP chain) is written by the epilogue
//    into the CTA's stash (tc_engine.cuh, stash mode): a_l and delta_l into
//    buffer l % 2, so consecutive layers alternate buffers in both chains;
//  * a layer with more than 256 outputs (forward) or inputs (VJP) runs as
//    N-block ops of at most 256 accumulator columns that share the stash
//    chunks; the first N-block op of each layer copies the chunks to the
//    stage's weight-gradient image;
//  * weight-gradient ops are N-blocked too (B image read block-wise);
//  * state vectors are kept in 64-component chunks (virtual tiles
//    T * nsc + c), and every evaluation runs in full (no reuse of the
//    previous evaluation's activations).
//
// FFJORD mode (b.ffj; state [z; delta_logp], d + 1 <= 64): the right-hand
// side is g = [f(z [, t]); -e . (J e)] (src/ffjord.jl:81-136), and the VJP
// with cotangent [lam_z; lam_D] runs reverse mode over the forward's primal
// chain a_{l+1} = act(p_l), p_l = W_l a_l + b_l, and tangent chain
// adot_{l+1} = act'(p_l) pdot_l, pdot_l = W_l adot_l (adot_0 = e):
//   abar_L = lam_z, achk_L = -lam_D e;   per layer, from the top:
//   pdotbar_l = achk_{l+1} act'(p_l),
//   pbar_l = abar_{l+1} act'(p_l) + achk_{l+1} act''(p_l) pdot_l,
//   abar_l = W_l^T pbar_l,  achk_l = W_l^T pdotbar_l,
//   dW_l += pbar_l a_l^T + pdotbar_l adot_l^T,  db_l += pbar_l,
// with kl_z = abar_0 on the z inputs and kl_D = 0. The primal and tangent
// chains use stash buffers 0/1 and 2/3; the two VJP ops of an N-block
// (abar and achk) are drained together (both accumulator regions); the
// weight-gradient ops stack both operand pairs along K.
#include "tc_args.h"

namespace gbnde {

namespace {

struct ThrW {
  int r, ch, q, lane;
};

__device__ __forceinline__ int nmine_of(int S, int c, int ch) {
  return min(tc::kCW, max(0, S - 64 * c - tc::kCW * ch));
}
__device__ __forceinline__ void ldv_api(const float* p, int n, float* x) {
#pragma unroll
  for (int i = 0; i < tc::kCW; ++i) x[i] = (i < n) ? p[i] : 0.f;
}
__device__ __forceinline__ void stv_api(float* p, int n, const float* x) {
#pragma unroll
  for (int i = 0; i < tc::kCW; ++i)
    if (i < n) p[i] = x[i];
}

// Thread-private FP32 activation scratch, slot-major (float4 slot k of thread
// t at hs4[k * kEpiThreads + t]).
__device__ __forceinline__ void hs_ldv(const float4* hs4, int k0, float* x) {
  const uint64_t pol = tc::policy_evict_first();
#pragma unroll
  for (int j = 0; j < tc::kCW / 4; ++j) {
    const float4 q = tc::ld_v4f_hint(hs4 + (size_t)(k0 + j) * tc::kEpiThreads + threadIdx.x, pol);
    x[4 * j] = q.x; x[4 * j + 1] = q.y; x[4 * j + 2] = q.z; x[4 * j + 3] = q.w;
  }
}
__device__ __forceinline__ void hs_stv(float4* hs4, int k0, const float* x) {
  const uint64_t pol = tc::policy_evict_last();
#pragma unroll
  for (int j = 0; j < tc::kCW / 4; ++j) {
    uint4 u;
    u.x = __float_as_uint(x[4 * j]);
    u.y = __float_as_uint(x[4 * j + 1]);
    u.z = __float_as_uint(x[4 * j + 2]);
    u.w = __float_as_uint(x[4 * j + 3]);
    tc::st_v4_hint(hs4 + (size_t)(k0 + j) * tc::kEpiThreads + threadIdx.x, u, pol);
  }
}

__device__ __forceinline__ bool epi_grid_barrier(const BwdArgs& a, unsigned int& gen, int* okflag) {
  tc::epi_bar();
  gen += 1;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(a.bar, 1u);
    const unsigned int target = gen * gridDim.x;
    const unsigned long long t0 = globaltimer_ns();
    int ok = 1;
    while (ld_acquire_u32(a.bar) < target) {
      if (*((volatile int*)&a.status[ST_BARRIER]) != 0) { ok = 0; break; }
      if (globaltimer_ns() - t0 > kBarrierTimeoutNs) {
        atomicExch(&a.status[ST_BARRIER], 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    *okflag = ok;
  }
  tc::epi_bar();
  return *okflag != 0;
}

__device__ __forceinline__ double epi_partials_sum(const double* p, int n, tc::Shared& sh) {
  if (threadIdx.x < 32) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(p + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) sh.red[16] = v;
  }
  tc::epi_bar();
  const double v = sh.red[16];
  tc::epi_bar();
  return v;
}

// Column sums over the warp's 32 trajectory rows of kCW values per lane:
// after the butterfly, lane j holds the sum of value j % kCW over the 32 lanes.
__device__ __forceinline__ float warp_colsum(float* v, int lane) {
#pragma unroll
  for (int s = tc::kCW / 2; s >= 1; s >>= 1) {
#pragma unroll
    for (int i = 0; i < s; ++i) {
      const bool up = (lane & s) != 0;
      const float send = up ? v[i] : v[i + s];
      const float keep = up ? v[i + s] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
#pragma unroll
  for (int s = tc::kCW; s < 32; s <<= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], s);
  return v[0];
}

}  // namespace

__global__ void __launch_bounds__(tc::kThreads, 1) bwd_tcw_kernel(BwdTcwArgs W) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* aring = smem;
  uint8_t* wring = smem + tc::kARing * tc::kASlotBytes;
  __shared__ tc::Shared sh;
  __shared__ int s_ok;
  __shared__ float s_ha[6][6], s_hb[6][7], s_hbt[7];
  __shared__ int s_n[6];
  __shared__ StepCtl s_ctl;
  const BwdTcArgs& A = W.t;
  const BwdArgs& a = A.b;
  const int warp = threadIdx.x >> 5;

  tc::init_shared(sh);
  if (warp == tc::kMmaWarp) tc::tmem_alloc(&sh.tmem_base, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp >= tc::kMmaWarp) {
    tc::regs_give_ctl();
    if (warp == tc::kMmaWarp)
      tc::mma_loop_cmd(A.ops, A.dwops, A.ops, A.ops, sh, aring, wring,
                       A.img + (size_t)blockIdx.x * A.tpc * tc::kImgSlots * A.img_cta, A.img_cta);
    else if (warp == tc::kTmaWarp) tc::tma_loop_cmd(A.ops, A.dwops, A.ops, A.ops, sh, aring, wring);
  } else {
    tc::regs_take_epi();
    // ======================= epilogue warps =======================
    const MlpDev& m = a.mlp;
    const int L = m.nlayers;
    const int S = a.S, G = gridDim.x, nsc = W.nsc;
    const size_t SB = (size_t)S * a.B;
    const double Nn = (double)SB;
    const bool timein = m.timein != 0;
    const bool ffj = a.ffj != 0;
    const int netS = ffj ? a.ffd : S;  // state inputs of the network (z without delta_logp)
    float* trs = ffj ? W.trs + (size_t)blockIdx.x * 512 : nullptr;
    ThrW th;
    th.lane = threadIdx.x & 31;
    th.q = warp & 3;
    th.r = 32 * th.q + th.lane;
    th.ch = warp >> 2;
    const uint32_t lane_base = ((uint32_t)(th.q * 32)) << 16;
    uint8_t* stash = W.stash + (size_t)blockIdx.x * tc::kStashCta;
    tc::EpiState es;
    tc::epi_state_init(es);
    unsigned int gen = 0;
    int par = 0, cur = 0;
    int ret = GBNDE_RET_SUCCESS;
    long long nf_adj = 0, nacc = 0, nrej = 0, iter = 0;
    double dt = 0.0, qold = kQoldInit;
    bool swp = false, ok = true;
    uint8_t* img = A.img + (size_t)blockIdx.x * A.tpc * tc::kImgSlots * A.img_cta;
    int fs = 0;
    float4* hs4 = reinterpret_cast<float4*>(A.hscr + (size_t)blockIdx.x * tc::kEpiThreads * A.hvals);
    float* mu_acc = a.mu_acc + (size_t)blockIdx.x * a.P;
    float* Pb[3] = {A.pbias + (size_t)blockIdx.x * 12 * A.nbias, A.pbias + ((size_t)blockIdx.x * 12 + 4) * A.nbias,
                    A.pbias + ((size_t)blockIdx.x * 12 + 8) * A.nbias};
    int iP1 = 0, iP7 = 2;
    float* Pmid = Pb[1];
    tc::CmdPoster cmdp;

    auto klb = [&](int j) -> float* {
      if (j == 0) return swp ? a.kl[6] : a.kl[0];
      if (j == 6) return swp ? a.kl[0] : a.kl[6];
      return a.kl[j];
    };
    const size_t SBt = (size_t)a.ntiles * nsc * tc::kTileVec;
    auto gofs = [&](int tile, int c) -> size_t {
      return ((size_t)tile * 128 + th.r) * S + 64 * c + tc::kCW * th.ch;
    };
    auto tofs = [&](int tile, int c) -> size_t { return tc::tl_offset_cw(tile * nsc + c, th.ch, th.r); };
    auto rowok = [&](int tile) -> bool { return tile * 128 + th.r < a.B; };
    auto zero_cta = [&](float* p) {
      float4* p4 = reinterpret_cast<float4*>(p);
      for (size_t i = threadIdx.x; i < (size_t)a.P / 4; i += tc::kEpiThreads) p4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    };
    auto zero_bias = [&](float* p) {
      for (int i = threadIdx.x; i < 4 * A.nbias; i += tc::kEpiThreads) p[i] = 0.f;
    };

    // (the images' padding rows and blocks are never written: the host clears
    // the image buffer once when it is allocated)
    zero_cta(mu_acc);
    asm volatile("fence.proxy.async.global;" ::: "memory");
    for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
      if (!rowok(tile)) continue;
      for (int c = 0; c < nsc; ++c) {
        const int nm = nmine_of(S, c, th.ch);
        float v[tc::kCW], z[tc::kCW];
        for (int i = 0; i < tc::kCW; ++i) { v[i] = 0.f; z[i] = 0.f; }
        for (int qq = 0; qq < a.nsave_last; ++qq) {
          float d[tc::kCW];
          ldv_api(a.dLdu + (size_t)(a.save_last + qq) * SB + gofs(tile, c), nm, d);
          for (int i = 0; i < tc::kCW; ++i) v[i] += d[i];
        }
        tc::tl_stv(a.lam[0] + tofs(tile, c), v);
        tc::tl_stv(A.lam_comp[0] + tofs(tile, c), z);
      }
    }
    tc::epi_bar();

    // ---- adjoint right-hand side of one tile --------------------------------------------
    // in_x(c, x): this thread's columns of input chunk c of the network at u(t)
    // (time row included); in_lam(c, y): its columns of state chunk c of the
    // stage's lam. out_kl(c, kl): the stage's kl chunk c (lam^T df/du). slot:
    // image slot of the stage's weight-gradient operands (-1: none); P / cw:
    // pending bias quadrature buffer and the stage weight (P == nullptr: no
    // quadrature). The VJP chain runs on cw * lam (it is linear), so its chunks
    // double as the weight-gradient images; kl is divided by cw at the end.
    auto adj_eval = [&](int tile, int slot, float* P, float cw, auto&& in_x, auto&& in_lam,
                        auto&& out_kl) -> bool {
      const uint32_t tj = (uint32_t)((tile - (int)blockIdx.x) / G);
      if (threadIdx.x == 0 &&
          !tc::epi_post(cmdp, sh, tc::CMD_EVAL | ((uint32_t)(slot + 1) << 8) | (tj << 24)))
        return false;
      // forward recompute: a_0 = (x [, t]) into buffer 0, a_{l+1} into buffer (l + 1) % 2
      const int kc0 = (m.dims[0] + 63) / 64;
      for (int c = 0; c < kc0; ++c) {
        float x[tc::kCW];
        in_x(c, x);
        tc::stash_write<2>(stash, sh, 0, c, th.r, th.ch, x);
      }
      for (int l = 0; l < L - 1; ++l) {
        const int N = m.dims[l + 1];
        const int ob = (l + 1) & 1;
        for (int b = 0; b * 256 < N; ++b) {
          uint32_t col;
          if (!tc::epi_wait_acc(es, sh, &col)) return false;
          const int nch = (min(256, N - 256 * b) + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
            float v[tc::kCW], bc[tc::kCW];
            tc::load_bias_cw(A.bias[l], n0, N, bc);
            tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
            tc::bias_act_cw(v, bc, m.act[l], n0, N);
            hs_stv(hs4, (A.hoff[l + 1] + tc::kCW * (4 * b + cc)) / 4, v);
            tc::stash_write<2>(stash, sh, ob, 4 * b + cc, th.r, th.ch, v);
          }
          tc::epi_release_acc(es, sh);
        }
      }
      // a_{L-1} reaches its image through a copy-only op. delta_L = cw lam
      // (identity output layer) into buffer L % 2, with its bias column sums
      const float cs = P ? cw : 1.f;
      for (int c = 0; c < nsc; ++c) {
        float v[tc::kCW];
        in_lam(c, v);
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) v[i] *= cs;
        tc::stash_write<2>(stash, sh, L & 1, c, th.r, th.ch, v);
        if (P) {
          const float s = warp_colsum(v, th.lane);
          if (th.lane < tc::kCW && 64 * c + tc::kCW * th.ch + th.lane < S)
            tc::red_add(P + th.q * A.nbias + A.boffp[L - 1] + 64 * c + tc::kCW * th.ch + th.lane, s);
        }
      }
      // VJP chain: g_l = W_l^T delta_{l+1} in N-blocks over the inputs of
      // layer l; delta_l = g_l * act'(z_l) into buffer l % 2
      for (int l = L - 1; l >= 1; --l) {
        const int N = m.dims[l];
        for (int b = 0; b * 256 < N; ++b) {
          uint32_t col;
          if (!tc::epi_wait_acc(es, sh, &col)) return false;
          const int nch = (min(256, N - 256 * b) + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
            float v[tc::kCW], h[tc::kCW];
            hs_ldv(hs4, (A.hoff[l] + tc::kCW * (4 * b + cc)) / 4, h);
            tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
            tc::deriv_mul_cw(v, h, m.act[l - 1], n0, N);
            tc::stash_write<2>(stash, sh, l & 1, 4 * b + cc, th.r, th.ch, v);
            if (P) {
              const float s = warp_colsum(v, th.lane);
              if (th.lane < tc::kCW) tc::red_add(P + th.q * A.nbias + A.boffp[l - 1] + n0 + th.lane, s);
            }
          }
          tc::epi_release_acc(es, sh);
        }
      }
      // kl = W_0^T delta_1 on the state inputs (the time row's is not needed)
      const float inv = 1.f / cs;
      for (int b = 0; b * 256 < S; ++b) {
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        const int nch = (min(256, S - 256 * b) + 63) / 64;
        for (int cc = 0; cc < nch; ++cc) {
          float v[tc::kCW];
          tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
          const int c = 4 * b + cc;
          const int nm = nmine_of(S, c, th.ch);
#pragma unroll
          for (int i = 0; i < tc::kCW; ++i) v[i] = (i < nm) ? v[i] * inv : 0.f;
          out_kl(c, v);
        }
        tc::epi_release_acc(es, sh);
      }
      return true;
    };

    // ---- FFJORD adjoint right-hand side of one tile (same contract as adj_eval) -----------
    // scratch per thread: a_l (l = 1..L-1) at hoff[l], pdot_l (l = 0..L-2) at hoff2[l]
    auto adj_eval_ffj = [&](int tile, int slot, float* P, float cw, auto&& in_x, auto&& in_lam,
                            auto&& out_kl) -> bool {
      const int d = a.ffd;
      const uint32_t tj = (uint32_t)((tile - (int)blockIdx.x) / G);
      if (threadIdx.x == 0 &&
          !tc::epi_post(cmdp, sh, tc::CMD_EVAL | ((uint32_t)(slot + 1) << 8) | (tj << 24)))
        return false;
      const float* erow = (rowok(tile) && a.noise != nullptr) ? a.noise + ((size_t)tile * 128 + th.r) * d : nullptr;
      // forward recompute of both chains: a_0 = (z [, t]) into buffer 0, adot_0 = e into buffer 2
      {
        float x[tc::kCW];
        in_x(0, x);
        tc::stash_write<2>(stash, sh, 0, 0, th.r, th.ch, x);
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) {
          const int col = tc::kCW * th.ch + i;
          x[i] = (erow != nullptr && col < d) ? erow[col] : 0.f;
        }
        tc::stash_write<2>(stash, sh, 2, 0, th.r, th.ch, x);
      }
      for (int l = 0; l < L - 1; ++l) {
        const int N = m.dims[l + 1];
        const int ob = (l + 1) & 1;
        for (int b = 0; b * 256 < N; ++b) {  // primal
          uint32_t col;
          if (!tc::epi_wait_acc(es, sh, &col)) return false;
          const int nch = (min(256, N - 256 * b) + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
            float v[tc::kCW], bc[tc::kCW];
            tc::load_bias_cw(A.bias[l], n0, N, bc);
            tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
            tc::bias_act_cw(v, bc, m.act[l], n0, N);
            hs_stv(hs4, (A.hoff[l + 1] + tc::kCW * (4 * b + cc)) / 4, v);
            tc::stash_write<2>(stash, sh, ob, 4 * b + cc, th.r, th.ch, v);
          }
          tc::epi_release_acc(es, sh);
        }
        for (int b = 0; b * 256 < N; ++b) {  // tangent: pdot_l kept, adot_{l+1} = act' pdot_l
          uint32_t col;
          if (!tc::epi_wait_acc(es, sh, &col)) return false;
          const int nch = (min(256, N - 256 * b) + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
            float v[tc::kCW], y[tc::kCW];
            tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
            hs_stv(hs4, (A.hoff2[l] + tc::kCW * (4 * b + cc)) / 4, v);
            hs_ldv(hs4, (A.hoff[l + 1] + tc::kCW * (4 * b + cc)) / 4, y);
            tc::deriv_mul_cw(v, y, m.act[l], n0, N);
            tc::stash_write<2>(stash, sh, 2 + ob, 4 * b + cc, th.r, th.ch, v);
          }
          tc::epi_release_acc(es, sh);
        }
      }
      // a_{L-1} and adot_{L-1} reach their images through copy-only ops.
      // Output cotangents (identity output layer): pbar_{L-1} = cw lam_z into
      // buffer L % 2 (with its bias column sums), pdotbar_{L-1} = -cw lam_D e
      // into buffer 2 + L % 2; lam_D (row d of the state) comes from the thread
      // owning that column, through the CTA's scratch.
      const float cs = P ? cw : 1.f;
      {
        float y[tc::kCW];
        in_lam(0, y);
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i)
          if (tc::kCW * th.ch + i == d) trs[th.r] = y[i];
        tc::epi_bar();
        const float lamD = trs[th.r];
        tc::epi_bar();
        float v[tc::kCW];
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) {
          const int col = tc::kCW * th.ch + i;
          v[i] = col < d ? cs * y[i] : 0.f;
          y[i] = (erow != nullptr && col < d) ? -cs * lamD * erow[col] : 0.f;
        }
        tc::stash_write<2>(stash, sh, L & 1, 0, th.r, th.ch, v);
        tc::stash_write<2>(stash, sh, 2 + (L & 1), 0, th.r, th.ch, y);
        if (P) {
          const float sm = warp_colsum(v, th.lane);
          if (th.lane < tc::kCW && tc::kCW * th.ch + th.lane < d)
            tc::red_add(P + th.q * A.nbias + A.boffp[L - 1] + tc::kCW * th.ch + th.lane, sm);
        }
      }
      // VJP pairs per N-block over the inputs of layer l (l >= 1): abar_l and
      // achk_l drained together into pbar_{l-1} (buffer l % 2, bias sums) and
      // pdotbar_{l-1} (buffer 2 + l % 2)
      for (int l = L - 1; l >= 1; --l) {
        const int N = m.dims[l];
        const int act = m.act[l - 1];
        for (int b = 0; b * 256 < N; ++b) {
          const int r0 = (int)(es.g & 1), r1 = r0 ^ 1;
          if (!tc::mbar_wait(&sh.acc_full[r0], es.use[r0] & 1, &sh.err)) return false;
          if (!tc::mbar_wait(&sh.acc_full[r1], es.use[r1] & 1, &sh.err)) return false;
          tc::tc_fence_after();
          const uint32_t c0 = (uint32_t)(r0 * 256), c1 = (uint32_t)(r1 * 256);
          const int nch = (min(256, N - 256 * b) + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
            const uint32_t co = (uint32_t)(64 * cc + tc::kCW * th.ch);
            float ab[tc::kCW], ak[tc::kCW];
            tc::tmem_ld_cw(sh.tmem_base + lane_base + c0 + co, ab);
            tc::tmem_ld_cw(sh.tmem_base + lane_base + c1 + co, ak);
            const int ka = (A.hoff[l] + tc::kCW * (4 * b + cc)) / 4;
            const int kp = (A.hoff2[l - 1] + tc::kCW * (4 * b + cc)) / 4;
#pragma unroll
            for (int j = 0; j < tc::kCW / 4; ++j) {
              const float4 a4 = hs4[(size_t)(ka + j) * tc::kEpiThreads + threadIdx.x];
              const float4 p4 = hs4[(size_t)(kp + j) * tc::kEpiThreads + threadIdx.x];
              const float av[4] = {a4.x, a4.y, a4.z, a4.w}, pv[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const int i = 4 * j + q;
                float s1 = 1.f, s2 = 0.f;
                if (act == GBNDE_ACT_TANH) {
                  s1 = fmaf(-av[q], av[q], 1.f);
                  s2 = -2.f * av[q] * s1;
                } else if (act == GBNDE_ACT_SOFTPLUS) {
                  s1 = -expm1f(-av[q]);
                  s2 = s1 * (1.f - s1);
                }
                const bool inside = n0 + i < N;
                const float pb = fmaf(ak[i] * s2, pv[q], ab[i] * s1);
                ab[i] = inside ? pb : 0.f;           // pbar_{l-1}
                ak[i] = inside ? ak[i] * s1 : 0.f;   // pdotbar_{l-1}
              }
            }
            tc::stash_write<2>(stash, sh, 2 + (l & 1), 4 * b + cc, th.r, th.ch, ak);
            tc::stash_write<2>(stash, sh, l & 1, 4 * b + cc, th.r, th.ch, ab);
            if (P) {
              const float sm = warp_colsum(ab, th.lane);
              if (th.lane < tc::kCW) tc::red_add(P + th.q * A.nbias + A.boffp[l - 1] + n0 + th.lane, sm);
            }
          }
          tc::epi_release_acc(es, sh);
          tc::epi_release_acc(es, sh);
        }
      }
      // kl_z = abar_0 on the z inputs; kl_D = 0
      const float inv = 1.f / cs;
      for (int b = 0; b * 256 < d; ++b) {
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        float v[tc::kCW];
        tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(tc::kCW * th.ch), v);
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) v[i] = (tc::kCW * th.ch + i < d) ? v[i] * inv : 0.f;
        out_kl(0, v);
        tc::epi_release_acc(es, sh);
      }
      return true;
    };
    auto adj = [&](int tile, int slot, float* P, float cw, auto&& in_x, auto&& in_lam, auto&& out_kl) -> bool {
      if (ffj) return adj_eval_ffj(tile, slot, P, cw, in_x, in_lam, out_kl);
      return adj_eval(tile, slot, P, cw, in_x, in_lam, out_kl);
    };

    // ---- weight gradients of an accepted step ------------------------------------------
    // mu += H * accumulator, plain FP32 per CTA (a compensated sum doubled the
    // read-modify-write traffic for rounding far below the BF16 images')
    auto commit_step = [&](float Hf) -> bool {
      tc::epi_bar();
      if (threadIdx.x == 0 && !tc::epi_post(cmdp, sh, tc::CMD_DW | ((uint32_t)fs << 8))) return false;
      float v[tc::kCW];
      for (int l = 0; l < L; ++l) {
        const int out = m.dims[l + 1], in = m.dims[l];
        const int isA = A.a_isA[l];
        const int Nn2 = isA ? out : in;  // N side of the dW ops
        float* __restrict__ Pw = mu_acc + m.woff[l];
        for (int hh = 0; hh < A.nh[l]; ++hh) {
          const int mrow = 128 * hh + th.r;  // M-side feature of this lane
          for (int nb = 0; nb * 256 < Nn2; ++nb) {
            uint32_t col;
            if (!tc::epi_wait_acc(es, sh, &col)) return false;
            const int nch = (min(256, Nn2 - 256 * nb) + 63) / 64;
            for (int cc = 0; cc < nch; ++cc) {
              const int n0 = 256 * nb + 64 * cc + tc::kCW * th.ch;  // N-side feature of element 0
              tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
              const bool vec = isA && mrow < in && n0 + tc::kCW <= out &&
                               (reinterpret_cast<uintptr_t>(Pw + (size_t)mrow * out + n0) & 15) == 0;
              if (vec) {
                const size_t o = (size_t)mrow * out + n0;
#pragma unroll
                for (int i = 0; i < tc::kCW; i += 4) {
                  const float4 a4 = *reinterpret_cast<const float4*>(Pw + o + i);
                  *reinterpret_cast<float4*>(Pw + o + i) =
                      make_float4(fmaf(Hf, v[i], a4.x), fmaf(Hf, v[i + 1], a4.y), fmaf(Hf, v[i + 2], a4.z),
                                  fmaf(Hf, v[i + 3], a4.w));
                }
              } else {
#pragma unroll
                for (int i = 0; i < tc::kCW; ++i) {
                  const int n = n0 + i;
                  const bool okp = isA ? (mrow < in && n < out) : (mrow < out && n < in);
                  if (!okp) continue;
                  const size_t o = isA ? (size_t)mrow * out + n : (size_t)n * out + mrow;
                  Pw[o] = fmaf(Hf, v[i], Pw[o]);
                }
              }
            }
            tc::epi_release_acc(es, sh);
          }
        }
      }
      const float* P1 = Pb[iP1];
      for (int f = threadIdx.x; f < A.nbias; f += tc::kEpiThreads) {
        int l = 0;
        while (l + 1 < L && f >= A.boffp[l + 1]) ++l;
        const int o = f - A.boffp[l];
        if (o < m.dims[l + 1])
          mu_acc[m.boff[l] + o] +=
              Hf * ((((__ldcg(P1 + f) + __ldcg(P1 + A.nbias + f)) + __ldcg(P1 + 2 * A.nbias + f)) +
                     __ldcg(P1 + 3 * A.nbias + f)) +
                    (((__ldcg(Pmid + f) + __ldcg(Pmid + A.nbias + f)) + __ldcg(Pmid + 2 * A.nbias + f)) +
                     __ldcg(Pmid + 3 * A.nbias + f)));
      }
      tc::epi_bar();
      return true;
    };

    auto dense_setup = [&](const Interval& iv, double t, int* nstep, float* hb) {
      int n = iv.nlo;
      while (n < iv.nhi && a.fsteps[2 * (n + 1)] <= t) ++n;
      const double tn = a.fsteps[2 * n], h = a.fsteps[2 * n + 1];
      float bw[7];
      interp_weights((t - tn) / h, bw);
      for (int j = 0; j < 7; ++j) hb[j] = (float)(h * (double)bw[j]);
      *nstep = n;
    };
    // network input chunk c at u(t) (dense output of step n with weights hb)
    auto dense_x = [&](int tile, int c, int n, const float* hb, double tq, float* x) {
      if (c < nsc) {
        const float* slot = a.dense + (size_t)n * 8 * SBt + tofs(tile, c);
        float u[tc::kCW];
        tc::tl_ldv(slot, u);
        for (int j = 0; j < 7; ++j) {
          float k[tc::kCW];
          tc::tl_ldv(slot + (size_t)(j + 1) * SBt, k);
#pragma unroll
          for (int q = 0; q < tc::kCW; ++q) u[q] = fmaf(hb[j], k[q], u[q]);
        }
#pragma unroll
        for (int q = 0; q < tc::kCW; ++q) x[q] = u[q];
      } else {
#pragma unroll
        for (int q = 0; q < tc::kCW; ++q) x[q] = 0.f;
      }
      if (timein || netS != S)
#pragma unroll
        for (int q = 0; q < tc::kCW; ++q) {
          const int col = 64 * c + tc::kCW * th.ch + q;
          if (col == netS) x[q] = timein ? (float)tq : 0.f;
          else if (col > netS && col < S) x[q] = 0.f;
        }
    };

    for (int ivi = 0; ivi < a.niv && ok && ret == GBNDE_RET_SUCCESS; ++ivi) {
      const Interval iv = a.iv[ivi];
      double t = iv.t_hi;
      const double t_lo = iv.t_lo;
      // ---- FSAL stage at the interval start: kl1 and P1 = b1 * mu ----
      {
        zero_bias(Pb[iP1]);
        if (threadIdx.x == 0) dense_setup(iv, t, &s_n[0], s_hb[0]);
        tc::epi_bar();
        const int n = s_n[0];
        float hb[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) hb[j] = s_hb[0][j];
        for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
          const bool v = rowok(tile);
          ok = adj(
              tile, fs, Pb[iP1], (float)c_tab.b[0],
              [&](int c, float* x) {
                dense_x(tile, c, n, hb, t, x);
                if (!v)
                  for (int q = 0; q < tc::kCW; ++q) x[q] = 0.f;
              },
              [&](int c, float* y) {
                if (v) tc::tl_ldv(a.lam[cur] + tofs(tile, c), y);
                else
                  for (int q = 0; q < tc::kCW; ++q) y[q] = 0.f;
              },
              [&](int c, const float* kl) {
                if (v) tc::tl_stv(klb(0) + tofs(tile, c), kl);
              });
        }
        ++nf_adj;
        if (!ok) break;
      }
      // ---- initial step (first interval) ----
      // The controller's scalar FP64 work runs in warp 0 (every lane computes
      // the same values; lane 0 publishes them in s_ctl): FP64 executes at a
      // small fraction of the FP32 rate, and each epilogue warp would repeat
      // it. t, dt and qold are kept by warp 0 only. Per-thread parts of the
      // norms are FP32 sums of a thread's own components; the sums across
      // threads and CTAs are FP64.
      if (ivi == 0) {
        float p0 = 0.f, p1 = 0.f;
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
          if (!rowok(tile)) continue;
          for (int c = 0; c < nsc; ++c) {
            const int nm = nmine_of(S, c, th.ch);
            float l[tc::kCW], f[tc::kCW];
            tc::tl_ldv(a.lam[cur] + tofs(tile, c), l);
            tc::tl_ldv(klb(0) + tofs(tile, c), f);
            for (int i = 0; i < tc::kCW; ++i) {
              if (i >= nm) continue;
              const float sk = (float)a.abstol + fabsf(l[i]) * (float)a.reltol;
              const float xx = l[i] / sk, yy = f[i] / sk;
              p0 = fmaf(xx, xx, p0);
              p1 = fmaf(yy, yy, p1);
            }
          }
        }
        const double s0 = tc::epi_sum0_f(p0, sh);
        const double s1 = tc::epi_sum0_f(p1, sh);
        double* pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) {
          pp[blockIdx.x] = s0;
          pp[G + blockIdx.x] = s1;
        }
        if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        {
          const double q0 = tc::epi_partials_sum0(pp, G), q1 = tc::epi_partials_sum0(pp + G, G);
          if (threadIdx.x == 0) {
            const double d0 = sqrt(q0 / Nn), d1 = sqrt(q1 / Nn);
            double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
            dt0 = fmin(dt0, a.dtmax);
            s_ctl.d1 = d1;
            s_ctl.dt0 = dt0;
            s_ctl.hf = (float)dt0;
            s_ctl.tst[0] = t - dt0;
            dense_setup(iv, t - dt0, &s_n[0], s_hb[0]);
          }
        }
        tc::epi_bar();
        par ^= 1;
        const float hf = s_ctl.hf;
        const double tp = s_ctl.tst[0];
        const int n = s_n[0];
        float hb[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) hb[j] = s_hb[0][j];
        float p2 = 0.f;
        for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
          const bool v = rowok(tile);
          ok = adj(
              tile, -1, nullptr, 0.f,
              [&](int c, float* x) {
                dense_x(tile, c, n, hb, tp, x);
                if (!v)
                  for (int q = 0; q < tc::kCW; ++q) x[q] = 0.f;
              },
              [&](int c, float* y) {
                if (!v) {
                  for (int q = 0; q < tc::kCW; ++q) y[q] = 0.f;
                  return;
                }
                float l[tc::kCW], f0[tc::kCW];
                tc::tl_ldv(a.lam[cur] + tofs(tile, c), l);
                tc::tl_ldv(klb(0) + tofs(tile, c), f0);
                for (int q = 0; q < tc::kCW; ++q) y[q] = l[q] + hf * f0[q];
              },
              [&](int c, const float* f1) {
                if (!v) return;
                const int nm = nmine_of(S, c, th.ch);
                float l[tc::kCW], f0[tc::kCW];
                tc::tl_ldv(a.lam[cur] + tofs(tile, c), l);
                tc::tl_ldv(klb(0) + tofs(tile, c), f0);
                for (int i = 0; i < tc::kCW; ++i) {
                  if (i >= nm) continue;
                  const float sk = (float)a.abstol + fabsf(l[i]) * (float)a.reltol;
                  const float z = (f1[i] - f0[i]) / sk;
                  p2 = fmaf(z, z, p2);
                }
              });
        }
        ++nf_adj;
        if (!ok) break;
        const double s2 = tc::epi_sum0_f(p2, sh);
        pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) pp[blockIdx.x] = s2;
        if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        {
          const double q2 = tc::epi_partials_sum0(pp, G);
          if (threadIdx.x == 0) s_ctl.d1 = fmax(s_ctl.d1, sqrt(q2 / Nn) / s_ctl.dt0);
          tc::epi_bar();
          if (threadIdx.x < 32) {
            const double dt0 = s_ctl.dt0, mm = s_ctl.d1;
            const double dt1 = (mm <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(mm)) / 5.0);
            dt = fmin(100.0 * dt0, fmin(dt1, a.dtmax));
          }
        }
        par ^= 1;
      }
      // ---- adaptive steps down to t_lo ----
      while (ok) {
        zero_bias(Pmid);
        if (threadIdx.x < 32) {
          // warp 0: the step, its stage times, coefficients and interpolation weights
          const double rem = t - t_lo;
          const bool clipped = dt >= rem;
          const double H = clipped ? rem : dt;
          if (threadIdx.x == 0) {
            s_ctl.go = t > t_lo;
            s_ctl.clipped = clipped;
            s_ctl.h = H;
            s_ctl.hf = (float)H;
            for (int i = 1; i < 7; ++i) s_ctl.tst[i] = t - c_tab.c[i] * H;
          }
          if (t > t_lo) {
            if (threadIdx.x < 6) {
              const int i = threadIdx.x + 1;
              for (int j = 0; j < 6; ++j) s_ha[i - 1][j] = (float)(H * c_tab.a[i][j]);
              dense_setup(iv, t - c_tab.c[i] * H, &s_n[i - 1], s_hb[i - 1]);
            } else if (threadIdx.x == 6) {
              for (int j = 0; j < 7; ++j) s_hbt[j] = (float)(H * c_tab.btilde[j]);
            }
          }
        }
        tc::epi_bar();
        if (!s_ctl.go) break;
        if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
        ++iter;
        const float* lcur = a.lam[cur];
        float* lnew = a.lam[cur ^ 1];
        const float* ccur = A.lam_comp[cur];
        float* cnew = A.lam_comp[cur ^ 1];
        float perr = 0.f;
        for (int i = 1; i < 7 && ok; ++i) {
          float* P = (i < 6) ? Pmid : Pb[iP7];
          const int slot = (i < 6) ? i : tc::kImgSlots - 1 - fs;
          if (i == 6) {
            zero_bias(P);
            tc::epi_bar();
          }
          const float cw = (i < 6) ? (float)c_tab.b[i] : (float)c_tab.b[0];
          const int n = s_n[i - 1];
          const double ti = s_ctl.tst[i];
          for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
            const bool v = rowok(tile);
            ok = adj(
                tile, slot, P, cw,
                [&](int c, float* x) {
                  float hb[7];
#pragma unroll
                  for (int j = 0; j < 7; ++j) hb[j] = s_hb[i - 1][j];
                  dense_x(tile, c, n, hb, ti, x);
                  if (!v)
                    for (int q = 0; q < tc::kCW; ++q) x[q] = 0.f;
                },
                [&](int c, float* Y) {
                  if (!v) {
                    for (int q = 0; q < tc::kCW; ++q) Y[q] = 0.f;
                    return;
                  }
                  const size_t g = tofs(tile, c);
                  float lv[tc::kCW], sv[tc::kCW];
                  tc::tl_ldv(lcur + g, lv);
                  tc::tl_ldv(ccur + g, sv);
                  for (int j = 0; j < 6; ++j) {
                    if (j >= i) break;
                    float kj[tc::kCW];
                    tc::tl_ldv(klb(j) + g, kj);
                    const float hj = s_ha[i - 1][j];
#pragma unroll
                    for (int q = 0; q < tc::kCW; ++q) sv[q] = fmaf(hj, kj[q], sv[q]);
                  }
#pragma unroll
                  for (int q = 0; q < tc::kCW; ++q) Y[q] = lv[q] + sv[q];
                  if (i == 6) {
                    // the embedded error estimate's sum over k1..k6 (parked in the k7
                    // slot), the new lam and its compensation
                    float lt[tc::kCW], cn[tc::kCW];
#pragma unroll
                    for (int q = 0; q < tc::kCW; ++q) lt[q] = 0.f;
                    for (int j = 0; j < 6; ++j) {
                      float kj[tc::kCW];
                      tc::tl_ldv(klb(j) + g, kj);
                      const float bj = s_hbt[j];
#pragma unroll
                      for (int q = 0; q < tc::kCW; ++q) lt[q] = fmaf(bj, kj[q], lt[q]);
                    }
#pragma unroll
                    for (int q = 0; q < tc::kCW; ++q) cn[q] = sv[q] - (Y[q] - lv[q]);
                    tc::tl_stv(klb(6) + g, lt);
                    tc::tl_stv(lnew + g, Y);
                    tc::tl_stv(cnew + g, cn);
                  }
                },
                [&](int c, const float* kl) {
                  if (!v) return;
                  const size_t g = tofs(tile, c);
                  if (i == 6) {
                    const int nm = nmine_of(S, c, th.ch);
                    float lt[tc::kCW], lv[tc::kCW], yv[tc::kCW];
                    tc::tl_ldv(klb(6) + g, lt);
                    tc::tl_ldv(lcur + g, lv);
                    tc::tl_ldv(lnew + g, yv);
                    const float hbt6 = s_hbt[6];
                    for (int q = 0; q < tc::kCW; ++q) {
                      if (q >= nm) continue;
                      const float e = fmaf(hbt6, kl[q], lt[q]);
                      const float sc = (float)a.abstol + fmaxf(fabsf(lv[q]), fabsf(yv[q])) * (float)a.reltol;
                      const float rr = e / sc;
                      perr = isfinite(yv[q]) ? fmaf(rr, rr, perr) : INFINITY;
                    }
                  }
                  tc::tl_stv(klb(i) + g, kl);
                });
          }
          ++nf_adj;
        }
        if (!ok) break;
        const double se = tc::epi_sum0_f(perr, sh);
        double* pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) pp[blockIdx.x] = se;
        if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        {
          // error norm and PI controller (warp 0)
          const double qe = tc::epi_partials_sum0(pp, G);
          if (threadIdx.x < 32) {
            const double eest = sqrt(qe / Nn);
            const double H = s_ctl.h;
            int rc = GBNDE_RET_SUCCESS, acc = 0;
            if (!isfinite(eest)) {
              rc = GBNDE_RET_UNSTABLE;
            } else {
              double q11;
              double q = pi_q(eest, qold, &q11);
              if (eest <= 1.0) {
                acc = 1;
                t = s_ctl.clipped ? t_lo : t - H;
                if (q >= 1.0 && q <= 1.0) q = 1.0;
                qold = fmax(eest, kQoldInit);
                dt = fmin(H / q, a.dtmax);
              } else {
                dt = H / fmin(1.0 / kQmin, q11 / kGamma);
              }
            }
            __syncwarp();
            if (threadIdx.x == 0) {
              s_ctl.ret = rc;
              s_ctl.accept = acc;
            }
          }
          tc::epi_bar();
        }
        par ^= 1;
        if (s_ctl.ret != GBNDE_RET_SUCCESS) { ret = s_ctl.ret; break; }
        if (s_ctl.accept) {
          if (!commit_step(s_ctl.hf)) { ok = false; break; }
          const int tmp = iP1;
          iP1 = iP7;
          iP7 = tmp;
          fs = tc::kImgSlots - 1 - fs;
          ++nacc;
          cur ^= 1;
          swp = !swp;
        } else {
          ++nrej;
        }
      }
      if (!ok || ret != GBNDE_RET_SUCCESS) break;
      // ---- jump at t_lo ----
      if (iv.nsave_lo > 0) {
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
          if (!rowok(tile)) continue;
          for (int c = 0; c < nsc; ++c) {
            const int nm = nmine_of(S, c, th.ch);
            float v[tc::kCW];
            tc::tl_ldv(a.lam[cur] + tofs(tile, c), v);
            for (int qq = 0; qq < iv.nsave_lo; ++qq) {
              float d[tc::kCW];
              ldv_api(a.dLdu + (size_t)(iv.save_lo + qq) * SB + gofs(tile, c), nm, d);
              for (int i = 0; i < tc::kCW; ++i) v[i] += d[i];
            }
            tc::tl_stv(a.lam[cur] + tofs(tile, c), v);
          }
        }
      }
    }
    if (!ok && ret == GBNDE_RET_SUCCESS) ret = GBNDE_RET_BARRIER_TIMEOUT;
    if (ret == GBNDE_RET_SUCCESS) {
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
        if (rowok(tile))
          for (int c = 0; c < nsc; ++c) {
            float v[tc::kCW];
            tc::tl_ldv(a.lam[cur] + tofs(tile, c), v);
            stv_api(a.dLdu0 + gofs(tile, c), nmine_of(S, c, th.ch), v);
          }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.counters[CT_NF] = nf_adj;
      a.counters[CT_NVJP] = 0;
      a.counters[CT_NACCEPT] = nacc;
      a.counters[CT_NREJECT] = nrej;
      a.counters[CT_NRECOMP] = 0;
      const int e = ((volatile int*)&sh.err)[0];
      a.status[ST_RETCODE] = (a.status[ST_BARRIER] != 0 || e != 0) ? GBNDE_RET_BARRIER_TIMEOUT : ret;
      if (e) a.status[2] = e;
    }
    tc::epi_bar();
    if (threadIdx.x == 0) ((volatile int*)&sh.stop)[0] = 1;
  }
  __syncthreads();
  tc::tc_fence_after();
  if (warp == tc::kMmaWarp) tc::tmem_dealloc(sh.tmem_base, 512);
}

int launch_bwd_tcw(const BwdTcwArgs& a, int grid, cudaStream_t st) {
  if (tc_check_regs((const void*)bwd_tcw_kernel)) return -1;
  cudaError_t e = cudaFuncSetAttribute(bwd_tcw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes);
  if (e != cudaSuccess) return -1;
  void* args[] = {(void*)&a};
  e = cudaLaunchCooperativeKernel((const void*)bwd_tcw_kernel, dim3(grid), dim3(tc::kThreads), args,
                                  tc::kSmemBytes, st);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
