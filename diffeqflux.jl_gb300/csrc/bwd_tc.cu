// bwd_tc.cu -- persistent InterpolatingAdjoint solve, BF16 tensor-core form.
//
// Same adjoint algorithm as bwd_f32.cu (the pullback of SciMLSensitivity's
// rrule on `solve` for sensealg = InterpolatingAdjoint(), src/neural_de.jl:57):
// reverse-time Tsit5 on lam with the PI controller over lam, the save points
// as stops where lam jumps by dL/du(t_i), and the parameter quadrature mu with
// the Tsit5 weights over accepted steps. u(t) is the free interpolant of the
// forward's dense stage storage (one slot per accepted forward step).
//
// One adjoint right-hand side on a tile of 128 trajectories is a list of
// tensor-core ops (tc_engine.cuh, command mode):
//   forward recompute  z_l = W_l a_{l-1},          l = 1..L-1   (5 split products)
//   VJP chain          g_l = W_l^T delta_{l+1},    l = L..1     (5 split products)
//                      delta_l = g_l * act'(z_l), delta_L = lam, kl = g_1
// The VJP chain runs on b_s lam (b_s: the stage's quadrature weight; it is
// linear, so kl is divided by b_s at the end). The A chunks of the activations
// a_l and of the weighted cotangents b_s delta_{l+1} (their first two split
// pieces) are bulk-copied by the MMA warp from shared memory into the image
// slot of the stage. Once a step is
// accepted, one weight-gradient op per layer (and 128-row half) runs over
// the six stages' images stacked along K (K = 6 x 128 trajectories, MN-major
// operands, 3 split products),
//   sum_s b_s dW_l(s) = sum_s b_s delta_{l+1}(s) a_l(s)^T,
// and the epilogue adds H times that accumulator to the CTA's mu
// (Kahan-compensated, each element owned by one thread): one drain per
// accepted step instead of one per stage, and no weight-gradient work at all
// for rejected steps. Stage 7 of a step is stage
// 1 of the next (FSAL): its images go to the second of two stage-1 slots,
// already weighted by b_1. Bias gradients are column sums of the cotangents
// (warp butterfly reductions) added into small per-CTA pending buffers, one
// row per 32-row group of the tile (one adder per element: deterministic).
// lam uses compensated (TwoSum) sums; t, H and the controller are FP64.
//
// O(checkpoints) mode (no dense storage, b.dense == null): at the start of
// every save interval the CTA replays that interval's accepted forward steps
// for its own tiles on the tensor cores (forward op list, CMD_FWD), from the
// checkpoint's state and compensation with the recorded step sizes -- the
// same arithmetic as the forward kernel, so the replayed stages are
// bit-identical -- into the interval buffer b.ibuf, which u(t) is then
// interpolated from. Each CTA reads only its own tiles, so no grid-wide sync
// is needed between the replay and the adjoint steps.
#include <cuda_fp16.h>

#include "tc_args.h"

namespace gbnde {


namespace {

struct Thr {
  int r, ch, nmine, q, lane;
};

__device__ __forceinline__ void ldv(const float* p, int n, bool vec, float* x) {
  if (vec) {
#pragma unroll
    for (int i = 0; i < tc::kCW; i += 4) {
      const float4 v = *reinterpret_cast<const float4*>(p + i);
      x[i] = v.x; x[i + 1] = v.y; x[i + 2] = v.z; x[i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < tc::kCW; ++i) x[i] = (i < n) ? p[i] : 0.f;
  }
}

__device__ __forceinline__ void stv(float* p, int n, bool vec, const float* x) {
  if (vec) {
#pragma unroll
    for (int i = 0; i < tc::kCW; i += 4)
      *reinterpret_cast<float4*>(p + i) = make_float4(x[i], x[i + 1], x[i + 2], x[i + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < tc::kCW; ++i)
      if (i < n) p[i] = x[i];
  }
}

// Thread-private FP32 scratch in slot-major layout: float4 slot k of thread t
// at hs4[k * kEpiThreads + t], so the 32 lanes of a warp touch 512 contiguous
// bytes. kCW values (kCW / 4 slots) per call.
__device__ __forceinline__ void hs_ldv(const float4* hs4, int k0, float* x) {
  const uint64_t pol = tc::policy_evict_first();  // last use
#pragma unroll
  for (int j = 0; j < tc::kCW / 4; ++j) {
    const float4 q = tc::ld_v4f_hint(hs4 + (size_t)(k0 + j) * tc::kEpiThreads + threadIdx.x, pol);
    x[4 * j] = q.x; x[4 * j + 1] = q.y; x[4 * j + 2] = q.z; x[4 * j + 3] = q.w;
  }
}
__device__ __forceinline__ void hs_stv(float4* hs4, int k0, const float* x) {
  const uint64_t pol = tc::policy_evict_last();  // read back within the evaluation
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

// kCW values of this thread's row into the next chain A chunk (split BF16
// pieces) of the shared-memory ring.
// NP = 3: all three pieces (the forward list's five products); NP = 2: hi and
// mid only, for chunks that only three-product GEMMs read (the adjoint's
// chains), whose lo piece is never loaded.
template <int NP = 3>
__device__ __forceinline__ bool emit(tc::EpiState& e, tc::Shared& sh, uint8_t* aring, const Thr& th,
                                     const float* x) {
  constexpr int nu = tc::kCW / 8;  // 16-byte units per piece
  uint4 hi[nu], mid[nu], lo[nu];
#pragma unroll
  for (int j = 0; j < nu; ++j) {
    if constexpr (NP == 3) tc::split3_bf16(x + 8 * j, hi[j], mid[j], lo[j]);
    else tc::split2_bf16(x + 8 * j, hi[j], mid[j]);
  }
  {
    if (!tc::mbar_wait(&sh.a_empty[e.aslot], e.aph ^ 1, &sh.err)) return false;
    uint8_t* base = aring + e.aslot * tc::kASlotBytes;
#pragma unroll
    for (int j = 0; j < nu; ++j) {
      const uint32_t off = tc::sw128_offset(th.r, nu * th.ch + j);
      *reinterpret_cast<uint4*>(base + off) = hi[j];
      *reinterpret_cast<uint4*>(base + 16384 + off) = mid[j];
      if constexpr (NP == 3) *reinterpret_cast<uint4*>(base + 32768 + off) = lo[j];
    }
    tc::epi_warp_arrive_smem(&sh.a_full[e.aslot]);
    if (++e.aslot == tc::kARing) { e.aslot = 0; e.aph ^= 1; }
  }
  return true;
}

// This thread's kCW columns (trajectory row r, column group ch) of K chunk cc
// (64 features) of a weight-gradient operand image, as FP16 times `scale`.
// The image is made of 8 KB blocks of 64 trajectories x 64 features (128-byte
// rows, SW128 swizzle), arranged as the weight-gradient ops read them: on the M
// side [trajectory block][128-row half][two 64-feature blocks], on the N side
// [trajectory block][64-feature block]. Streaming stores (the step's commit
// reads them once). Returns false if a value does not fit FP16.
__device__ __forceinline__ bool img_put_f16(uint8_t* base, int isA, int nh, int nblk, int cc, int r, int ch,
                                            const float* v, float scale) {
  const int kc = r >> 6, rr = r & 63;
  const size_t blk = isA ? (size_t)(kc * nh + (cc >> 1)) * 16384 + (size_t)(cc & 1) * 8192
                         : (size_t)(kc * nblk + cc) * 8192;
  uint8_t* p = base + blk;
  bool fine = true;
#pragma unroll
  for (int j = 0; j < tc::kCW / 8; ++j) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float a0 = v[8 * j + 2 * i] * scale, a1 = v[8 * j + 2 * i + 1] * scale;
      fine = fine && fabsf(a0) <= 65504.f && fabsf(a1) <= 65504.f;
      const __half2 h2 = __floats2half2_rn(a0, a1);
      w[i] = *reinterpret_cast<const uint32_t*>(&h2);
    }
    __stcs(reinterpret_cast<uint4*>(p + tc::sw128_offset(rr, (tc::kCW / 8) * ch + j)),
           make_uint4(w[0], w[1], w[2], w[3]));
  }
  return fine;
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

__global__ void __launch_bounds__(tc::kThreads, 1) bwd_tc_kernel(BwdTcArgs A) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* aring = smem;
  uint8_t* wring = smem + tc::kARing * tc::kASlotBytes;
  __shared__ tc::Shared sh;
  __shared__ int s_ok;
  // per-step scalars of stages 2..7, computed once by one warp: h a_ij, the
  // interpolation weights h b_j(theta) and forward slot of each stage time,
  // and the error weights h btilde_j
  __shared__ float s_ha[6][6], s_hb[6][7], s_hbt[7];
  __shared__ int s_n[6];
  __shared__ StepCtl s_ctl;
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
      tc::mma_loop_cmd(A.ops, A.dwops, A.ops7, A.fwops, sh, aring, wring,
                       A.img + (size_t)blockIdx.x * A.tpc * tc::kImgSlots * A.img_cta, A.img_cta);
    else if (warp == tc::kTmaWarp) tc::tma_loop_cmd(A.ops, A.dwops, A.ops7, A.fwops, sh, aring, wring);
  } else {
    tc::regs_take_epi();
    // ======================= epilogue warps =======================
    const MlpDev& m = a.mlp;
    const int L = m.nlayers;
    const int S = a.S, G = gridDim.x;
    const size_t SB = (size_t)S * a.B;
    const double Nn = (double)SB;
    Thr th;
    th.lane = threadIdx.x & 31;
    th.q = warp & 3;
    th.r = 32 * th.q + th.lane;
    th.ch = warp >> 2;
    th.nmine = min(tc::kCW, max(0, S - tc::kCW * th.ch));
    const bool vec = (S % 4 == 0) && th.nmine == tc::kCW;
    const uint32_t lane_base = ((uint32_t)(th.q * 32)) << 16;
    tc::EpiState es;
    tc::epi_state_init(es);
    unsigned int gen = 0;
    int par = 0, cur = 0;
    int ret = GBNDE_RET_SUCCESS;
    long long nf_adj = 0, nacc = 0, nrej = 0, iter = 0, nf_vjp = 0;
    double dt = 0.0, qold = kQoldInit;
    bool swp = false, ok = true;
    // image slots of this CTA: stage 1 in slot fs (0 or 6), stages 2..6 in
    // slots 1..5, stage 7 in slot 6 - fs (stage 1 of the next step)
    uint8_t* img = A.img + (size_t)blockIdx.x * A.tpc * tc::kImgSlots * A.img_cta;
    int fs = 0;
    // scale of the cotangent images over the current save interval (a power
    // of two, inv_isc its inverse) and whether an image value overflowed FP16
    float isc = 1.f, inv_isc = 1.f;
    float4* hs4 = reinterpret_cast<float4*>(A.hscr + (size_t)blockIdx.x * tc::kEpiThreads * A.hvals);
    float* mu_acc = a.mu_acc + (size_t)blockIdx.x * a.P;
    // pending bias quadrature: stage 1, stages 2..6, stage 7; each holds one
    // nbias row per 32-row group of the tile (rows q = warp % 4), into which
    // that group's warps add their column sums (one adder per element, so the
    // sums are deterministic); the step commit adds the four rows
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
    // lam, its compensation, the stages and the dense forward slots use the
    // tile layout; the cotangents dL/du(t_i) and dL/du0 the API layout
    const size_t SBt = (size_t)a.ntiles * tc::kTileVec;
    const bool c67_same = c_tab.c[5] == c_tab.c[6];  // stages 6 and 7 at one time (Tsit5: c = 1)
    auto gofs = [&](int tile) -> size_t { return ((size_t)tile * 128 + th.r) * S + tc::kCW * th.ch; };
    auto tofs = [&](int tile) -> size_t { return tc::tl_offset_cw(tile, th.ch, th.r); };
    auto valid = [&](int tile) -> bool { return tile * 128 + th.r < a.B && th.nmine > 0; };
    // P is a multiple of 4 floats per CTA slot (the host pads it)
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
    // the weight-gradient images are read by the producer warp (async proxy)
    asm volatile("fence.proxy.async.global;" ::: "memory");
    for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
      if (!valid(tile)) continue;
      float v[tc::kCW], z[tc::kCW];
      for (int i = 0; i < tc::kCW; ++i) { v[i] = 0.f; z[i] = 0.f; }
      for (int qq = 0; qq < a.nsave_last; ++qq) {
        float d[tc::kCW];
        ldv(a.dLdu + (size_t)(a.save_last + qq) * SB + gofs(tile), th.nmine, vec, d);
        for (int i = 0; i < tc::kCW; ++i) v[i] += d[i];
      }
      tc::tl_stv(a.lam[0] + tofs(tile), v);
      tc::tl_stv(A.lam_comp[0] + tofs(tile), z);
    }
    tc::epi_bar();

    // ---- adjoint right-hand side of one tile ------------------------------------------
    // lam_in: stage input lam (own components), x: u(t) (own components).
    // slot: image slot of the stage's weight-gradient operands (-1: none);
    // P/c: pending bias quadrature buffer and the stage weight (P == nullptr:
    // no quadrature). The cotangent images carry the weight c and the
    // interval's scale isc.
    // vjp_only: the activations of u(t) are those of the previous evaluation
    // (same t and u, in the activation scratch, and their images already in
    // `slot`): only the VJP ops run (x is not read).
    // reemit: the previous evaluation was at the same t and u(t) (Tsit5's
    // stages 6 and 7 share c = 1): the activation images of this stage are
    // written from x and the stored activations instead of being recomputed,
    // and only the VJP ops run.
    // tile: the tile being evaluated (its index within the CTA selects the
    // CTA's image set for that tile).
    // The weight-gradient images (FP16, one piece) are written here, with
    // plain stores, as each operand chunk is formed: a_0 = x (or x^3) and the
    // recomputed activations a_1 .. a_{L-1}, and the cotangents delta_L ..
    // delta_1. a_{L-1} feeds no GEMM of the evaluation (the output layer is
    // not recomputed), so it only goes to its image.
    auto adj_eval = [&](const float* lam_in, const float* x, int slot, float* P, float c, float* kl,
                        bool vjp_only, int tile, bool reemit) -> bool {
      const uint32_t tj = (uint32_t)((tile - (int)blockIdx.x) / G);
      const bool skip_fwd = vjp_only || reemit;
      if (threadIdx.x == 0 &&
          !tc::epi_post(cmdp, sh, tc::CMD_EVAL | ((uint32_t)(slot + 1) << 8) |
                                      ((skip_fwd ? (uint32_t)(L - 1) : 0u) << 16) | (tj << 24)))
        return false;
      uint8_t* simg = slot >= 0 ? img + ((size_t)tj * tc::kImgSlots + slot) * A.img_cta : nullptr;
      // image chunk cc of operand a_l (act = 1) or delta_{l+1} (act = 0) of layer l
      auto put = [&](int l, bool act, int cc, const float* val, float scale) {
        if (!simg) return;
        const int isA = act ? A.a_isA[l] : !A.a_isA[l];
        const int dim = act ? m.dims[l] : m.dims[l + 1];
        if (!img_put_f16(simg + (act ? A.aoff[l] : A.doff[l]), isA, A.nh[l], (dim + 63) / 64, cc, th.r, th.ch,
                         val, scale))
          atomicExch(&a.status[3], 1);  // seen by CTA 0 after the last grid barrier
      };
      float v[tc::kCW];
      if (reemit && !vjp_only) {
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) {
          const float y = (i < th.nmine) ? x[i] : 0.f;
          v[i] = m.cube ? y * y * y : y;
        }
        put(0, true, 0, v, 1.f);
        for (int l = 0; l < L - 1; ++l) {
          const int nch = (m.dims[l + 1] + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            hs_ldv(hs4, (A.hoff[l + 1] + tc::kCW * cc) / 4, v);
            put(l + 1, true, cc, v, 1.f);
          }
        }
      } else if (!vjp_only) {
      // a_0 = x (or x^3)
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) {
        const float y = (i < th.nmine) ? x[i] : 0.f;
        v[i] = m.cube ? y * y * y : y;
      }
      if (m.cube) hs_stv(hs4, A.hx / 4, x);  // for the chain rule through x^3 at the end
      if (!emit<2>(es, sh, aring, th, v)) return false;
      put(0, true, 0, v, 1.f);
      // forward recompute of the hidden layers
      for (int l = 0; l < L - 1; ++l) {
        const int N = m.dims[l + 1];
        const float* b = A.bias[l];
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        const int nch = (N + 63) / 64;
        // (the bias is loaded just before use: prefetching it a chunk ahead
        // costs registers the epilogue does not have, measured slower)
        for (int cc = 0; cc < nch; ++cc) {
          const int n0 = 64 * cc + tc::kCW * th.ch;
          float bc[tc::kCW];
          tc::load_bias_cw(b, n0, N, bc);
          tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
          tc::bias_act_cw(v, bc, m.act[l], n0, N);
          hs_stv(hs4, (A.hoff[l + 1] + tc::kCW * cc) / 4, v);
          if (l + 1 < L - 1 && !emit<2>(es, sh, aring, th, v)) return false;
          put(l + 1, true, cc, v, 1.f);
        }
        tc::epi_release_acc(es, sh);
      }
      }
      // delta_L = c lam (identity output layer). The VJP chain is linear in
      // its input, so every cotangent below carries the stage weight c (and
      // the images the scale isc), and kl is divided by c at the end.
      const float cs = P ? c : 1.f;
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) v[i] = (i < th.nmine) ? cs * lam_in[i] : 0.f;
      if (!emit<2>(es, sh, aring, th, v)) return false;
      put(L - 1, false, 0, v, isc);
      if (P) {
        float w[tc::kCW];
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) w[i] = v[i];
        const float s = warp_colsum(w, th.lane);
        if (th.lane < tc::kCW) tc::red_add(P + th.q * A.nbias + A.boffp[L - 1] + tc::kCW * th.ch + th.lane, s);
      }
      // VJP chain
      for (int l = L - 1; l >= 1; --l) {
        const int N = m.dims[l];
        const int nch = (N + 63) / 64;
        // the stored activations are loaded per chunk just before use (a
        // chunk-ahead prefetch costs registers and measured slower)
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        for (int cc = 0; cc < nch; ++cc) {
          const int n0 = 64 * cc + tc::kCW * th.ch;
          float h[tc::kCW];
          hs_ldv(hs4, (A.hoff[l] + tc::kCW * cc) / 4, h);
          tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
          tc::deriv_mul_cw(v, h, m.act[l - 1], n0, N);
          if (!emit<2>(es, sh, aring, th, v)) return false;
          put(l - 1, false, cc, v, isc);
          if (P) {
            const float s = warp_colsum(v, th.lane);
            if (th.lane < tc::kCW) tc::red_add(P + th.q * A.nbias + A.boffp[l - 1] + n0 + th.lane, s);
          }
        }
        tc::epi_release_acc(es, sh);
      }
      // kl = W_1^T delta_1 (times 3 x^2 for the cube prefix)
      {
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(tc::kCW * th.ch), v);
        const float inv = 1.f / cs;
#pragma unroll
        for (int i = 0; i < tc::kCW; ++i) kl[i] = (i < th.nmine) ? v[i] * inv : 0.f;
        if (m.cube) {
          float xc[tc::kCW];
          hs_ldv(hs4, A.hx / 4, xc);
#pragma unroll
          for (int i = 0; i < tc::kCW; ++i) kl[i] *= 3.f * xc[i] * xc[i];
        }
        tc::epi_release_acc(es, sh);
      }
      return true;
    };

    // ---- weight gradients of an accepted step -------------------------------------
    // One stage-stacked op per layer and 128-row half; mu += H * accumulator,
    // each mu element owned by one thread of the CTA. Then the bias quadrature
    // mu_b += H (P1 + Pmid).
    auto commit_step = [&](float Hf0) -> bool {
      // the images' FP16 writes are complete and ordered before the
      // producer's bulk loads of them (async proxy)
      asm volatile("fence.proxy.async.global;" ::: "memory");
      // the cotangent images carry the interval's scale isc (a power of two)
      const float Hf = Hf0 * inv_isc;
      tc::epi_bar();
      if (threadIdx.x == 0 && !tc::epi_post(cmdp, sh, tc::CMD_DW | ((uint32_t)fs << 8))) return false;
      tc::epi_skip_a(es, A.dw_chunks);
      // mu += H * accumulator, plain FP32 (19-odd accepted steps per solve add
      // about 1e-6 of rounding, far inside the FP16 images' 2e-4; a compensated
      // sum doubled the per-step read-modify-write traffic of mu)
      float v[tc::kCW];
      for (int l = 0; l < L; ++l) {
        const int out = m.dims[l + 1], in = m.dims[l];
        const int isA = A.a_isA[l];
        const int Nn2 = isA ? out : in;  // N side of the dW op
        float* __restrict__ Pw = mu_acc + m.woff[l];
        for (int hh = 0; hh < A.nh[l]; ++hh) {
          const int mrow = 128 * hh + th.r;  // M-side feature of this lane
          // element i of chunk cc of this lane: isA -> row mrow (in feature),
          // kCW consecutive out features; else row mrow (out feature), in
          // features at stride `out`
          auto addr = [&](int cc, int i, bool* okp) -> size_t {
            const int n0 = 64 * cc + tc::kCW * th.ch;
            *okp = isA ? (mrow < in && n0 + i < out) : (mrow < out && n0 + i < in);
            return isA ? (size_t)mrow * out + n0 + i : (size_t)(n0 + i) * out + mrow;
          };
          float av[tc::kCW];
          // a full row of kCW contiguous, 16-byte aligned elements (isA)
          auto vec4 = [&](int cc) -> bool {
            const int n0 = 64 * cc + tc::kCW * th.ch;
            return isA && mrow < in && n0 + tc::kCW <= out &&
                   (reinterpret_cast<uintptr_t>(Pw + (size_t)mrow * out + n0) & 15) == 0;
          };
          auto fetch = [&](int cc) {
            if (vec4(cc)) {
              const size_t o = (size_t)mrow * out + 64 * cc + tc::kCW * th.ch;
#pragma unroll
              for (int i = 0; i < tc::kCW; i += 4) {
                const float4 a4 = *reinterpret_cast<const float4*>(Pw + o + i);
                av[i] = a4.x; av[i + 1] = a4.y; av[i + 2] = a4.z; av[i + 3] = a4.w;
              }
              return;
            }
#pragma unroll
            for (int i = 0; i < tc::kCW; ++i) {
              bool okp;
              const size_t o = addr(cc, i, &okp);
              av[i] = okp ? Pw[o] : 0.f;
            }
          };
          // the first chunk's mu is read while the accumulator is computed
          fetch(0);
          uint32_t col;
          if (!tc::epi_wait_acc(es, sh, &col)) return false;
          const int nch = (Nn2 + 63) / 64;
          for (int cc = 0; cc < nch; ++cc) {
            if (cc > 0) fetch(cc);
            tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
            if (vec4(cc)) {
              const size_t o = (size_t)mrow * out + 64 * cc + tc::kCW * th.ch;
#pragma unroll
              for (int i = 0; i < tc::kCW; i += 4)
                *reinterpret_cast<float4*>(Pw + o + i) =
                    make_float4(fmaf(Hf, v[i], av[i]), fmaf(Hf, v[i + 1], av[i + 1]), fmaf(Hf, v[i + 2], av[i + 2]),
                                fmaf(Hf, v[i + 3], av[i + 3]));
            } else {
#pragma unroll
              for (int i = 0; i < tc::kCW; ++i) {
                bool okp;
                const size_t o = addr(cc, i, &okp);
                if (okp) Pw[o] = fmaf(Hf, v[i], av[i]);
              }
            }
          }
          tc::epi_release_acc(es, sh);
        }
      }
      // bias quadrature (pending buffers were summed by L2 adds: read them from L2)
      const float* P1 = Pb[iP1];
      for (int f = threadIdx.x; f < A.nbias; f += tc::kEpiThreads) {
        int l = 0;
        while (l + 1 < L && f >= A.boffp[l + 1]) ++l;
        const int o = f - A.boffp[l];
        if (o < m.dims[l + 1])
          mu_acc[m.boff[l] + o] +=
              Hf0 * ((((__ldcg(P1 + f) + __ldcg(P1 + A.nbias + f)) + __ldcg(P1 + 2 * A.nbias + f)) +
                      __ldcg(P1 + 3 * A.nbias + f)) +
                     (((__ldcg(Pmid + f) + __ldcg(Pmid + A.nbias + f)) + __ldcg(Pmid + 2 * A.nbias + f)) +
                      __ldcg(Pmid + 3 * A.nbias + f)));
      }
      tc::epi_bar();
      return true;
    };

    // u(t) from the dense forward slots: step n, weights hb
    auto dense_setup = [&](const Interval& iv, double t, int* nstep, float* hb) {
      int n = iv.nlo;
      while (n < iv.nhi && a.fsteps[2 * (n + 1)] <= t) ++n;
      const double tn = a.fsteps[2 * n], h = a.fsteps[2 * n + 1];
      float bw[7];
      interp_weights((t - tn) / h, bw);
      for (int j = 0; j < 7; ++j) hb[j] = (float)(h * (double)bw[j]);
      *nstep = n;
    };
    // dense slot of forward step n: the forward's storage, or the replayed
    // interval's buffer (slot n - nlo of the current interval)
    int nlo_cur = 0;
    auto slot_of = [&](int n) -> const float* {
      return a.dense ? a.dense + (size_t)n * 8 * SBt : a.ibuf + (size_t)(n - nlo_cur) * 8 * SBt;
    };
    auto dense_u = [&](int tile, int n, const float* hb, float* x) {
      const float* slot = slot_of(n);
      const size_t g = tofs(tile);
      // u_n + sum_j hb_j k_j, in two parts of kPart components and batches of
      // four vectors (u_n, k1..k3 then k4..k7), each batch in flight together
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        const float* sp = slot + g;
        float v8[8][tc::kPart];
#pragma unroll
        for (int j = 0; j < 8; ++j) tc::tl_ldp(sp + (size_t)j * SBt, hf, v8[j]);
#pragma unroll
        for (int q = 0; q < tc::kPart; ++q) {
          float e = 0.f;
#pragma unroll
          for (int j = 0; j < 7; ++j) e = fmaf(hb[j], v8[j + 1][q], e);
          x[tc::kPart * hf + q] = v8[0][q] + e;
        }
      }
    };

    // u(t) at the six stage times of an adjoint step (s_n, s_hb), into xst:
    // a forward slot's eight vectors are loaded once for all the stages that
    // interpolate in it (usually all six), instead of once per stage. One
    // float4 group of the thread's components at a time; the arithmetic is
    // dense_u's.
    auto stage_u = [&](int tile) {
      const size_t g = tofs(tile);
#pragma unroll 1
      for (int jg = 0; jg < tc::kCW / 4; ++jg) {
        float4 v8[8];
        int cur_n = -1;
#pragma unroll 1
        for (int i = 0; i < 6; ++i) {
          const int n = s_n[i];
          if (n != cur_n) {
            const float* sp = slot_of(n) + g + jg * 512;
#pragma unroll
            for (int j = 0; j < 8; ++j) v8[j] = *reinterpret_cast<const float4*>(sp + (size_t)j * SBt);
            cur_n = n;
          }
          float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int j = 0; j < 7; ++j) {
            const float w = s_hb[i][j];
            e.x = fmaf(w, v8[j + 1].x, e.x);
            e.y = fmaf(w, v8[j + 1].y, e.y);
            e.z = fmaf(w, v8[j + 1].z, e.z);
            e.w = fmaf(w, v8[j + 1].w, e.w);
          }
          *reinterpret_cast<float4*>(A.xst + (size_t)i * SBt + g + jg * 512) =
              make_float4(v8[0].x + e.x, v8[0].y + e.y, v8[0].z + e.z, v8[0].w + e.w);
        }
      }
    };

    // The plain right-hand side of one tile (the forward list): Y -> kout,
    // with the forward kernel's arithmetic.
    auto fwd_eval = [&](const float* Y, float* kout) -> bool {
      if (threadIdx.x == 0 && !tc::epi_post(cmdp, sh, tc::CMD_FWD)) return false;
      float v[tc::kCW];
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) {
        const float y = (i < th.nmine) ? Y[i] : 0.f;
        v[i] = m.cube ? y * y * y : y;
      }
      if (!emit(es, sh, aring, th, v)) return false;
      for (int l = 0; l < L - 1; ++l) {
        const int N = m.dims[l + 1];
        uint32_t col;
        if (!tc::epi_wait_acc(es, sh, &col)) return false;
        for (int cc = 0; cc < (N + 63) / 64; ++cc) {
          const int n0 = 64 * cc + tc::kCW * th.ch;
          float bc[tc::kCW];
          tc::load_bias_cw(A.bias[l], n0, N, bc);
          tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
          tc::bias_act_cw(v, bc, m.act[l], n0, N);
          if (!emit(es, sh, aring, th, v)) return false;
        }
        tc::epi_release_acc(es, sh);
      }
      uint32_t col;
      if (!tc::epi_wait_acc(es, sh, &col)) return false;
      float bc[tc::kCW];
      tc::load_bias_cw(A.bias[L - 1], tc::kCW * th.ch, m.dims[L], bc);
      tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(tc::kCW * th.ch), v);
      tc::bias_act_cw(v, bc, m.act[L - 1], tc::kCW * th.ch, m.dims[L]);
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) kout[i] = (i < th.nmine) ? v[i] : 0.f;
      tc::epi_release_acc(es, sh);
      return true;
    };
    long long nf_rec = 0;
    // Replay of the interval's forward steps nlo..nhi from its checkpoint into
    // b.ibuf (slot j = step nlo + j: u_n, k1..k7), as fwd_tc.cu computes them.
    auto replay = [&](const Interval& iv) -> bool {
      long long evals = 0;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        const bool v = valid(tile);
        const size_t g = tofs(tile);
        float* ru = A.rep[0];
        float* rc = A.rep[1];
        {
          float u[tc::kCW], cp[tc::kCW], k[tc::kCW];
          if (v) {
            ldv(a.ckpt + (size_t)iv.ckpt * SB + gofs(tile), th.nmine, vec, u);
            tc::tl_ldv(A.ckcomp + (size_t)iv.ckpt * SBt + g, cp);
          } else {
            for (int i = 0; i < tc::kCW; ++i) u[i] = cp[i] = 0.f;
          }
          tc::tl_stv(ru + g, u);
          tc::tl_stv(rc + g, cp);
          tc::tl_stv(a.ibuf + g, u);
          if (!fwd_eval(u, k)) return false;
          ++evals;
          tc::tl_stv(a.ibuf + SBt + g, k);
        }
        for (int n = iv.nlo; n <= iv.nhi; ++n) {
          float* slot = a.ibuf + (size_t)(n - iv.nlo) * 8 * SBt;
          const double h = a.fsteps[2 * n + 1];
          for (int i = 1; i < 7; ++i) {
            float ha[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) ha[j] = (float)(h * c_tab.a[i][j]);
            float u[tc::kCW], sv[tc::kCW], Y[tc::kCW], k[tc::kCW];
            if (v) {
              tc::tl_ldv(ru + g, u);
              tc::tl_ldv(rc + g, sv);
#pragma unroll
              for (int j = 0; j < 6; ++j) {
                if (j >= i) break;
                float kj[tc::kCW];
                tc::tl_ldv(slot + (size_t)(1 + j) * SBt + g, kj);
#pragma unroll
                for (int q = 0; q < tc::kCW; ++q) sv[q] = fmaf(ha[j], kj[q], sv[q]);
              }
#pragma unroll
              for (int q = 0; q < tc::kCW; ++q) Y[q] = u[q] + sv[q];
              if (i == 6) {
                float cn[tc::kCW];
#pragma unroll
                for (int q = 0; q < tc::kCW; ++q) cn[q] = sv[q] - (Y[q] - u[q]);
                tc::tl_stv(ru + g, Y);
                tc::tl_stv(rc + g, cn);
              }
            } else {
#pragma unroll
              for (int q = 0; q < tc::kCW; ++q) Y[q] = 0.f;
            }
            if (!fwd_eval(Y, k)) return false;
            ++evals;
            tc::tl_stv(slot + (size_t)(1 + i) * SBt + g, k);
          }
          if (n < iv.nhi) {
            // the next slot: its state, and k7 as its k1 (FSAL)
            float* nx = slot + 8 * SBt;
            float un[tc::kCW], k7[tc::kCW];
            tc::tl_ldv(ru + g, un);
            tc::tl_ldv(slot + 7 * SBt + g, k7);
            tc::tl_stv(nx + g, un);
            tc::tl_stv(nx + SBt + g, k7);
          }
        }
      }
      if (blockIdx.x == 0) nf_rec += evals / ((a.ntiles + G - 1 - blockIdx.x) / G);
      return true;
    };

    for (int ivi = 0; ivi < a.niv && ok && ret == GBNDE_RET_SUCCESS; ++ivi) {
      const Interval iv = a.iv[ivi];
      double t = iv.t_hi;
      const double t_lo = iv.t_lo;
      if (!a.dense) {
        nlo_cur = iv.nlo;
        if (!replay(iv)) { ok = false; break; }
      }
      // ---- the interval's image scale: the power of two that takes this
      // CTA's largest |lam| (after the jump) into [2^7, 2^8). FP16 reaches
      // 2^16, which leaves the cotangents of the inner layers and lam's
      // growth over the interval 256x; values below 2^-22 of the largest
      // keep full precision. A value that does not fit ends the solve with
      // an error instead of a wrong gradient.
      {
        float mx = 0.f;
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
          if (!valid(tile)) continue;
          float lv[tc::kCW];
          tc::tl_ldv(a.lam[cur] + tofs(tile), lv);
#pragma unroll
          for (int i = 0; i < tc::kCW; ++i)
            if (i < th.nmine) mx = fmaxf(mx, fabsf(lv[i]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (th.lane == 0) sh.red[warp] = (double)mx;
        tc::epi_bar();
        if (threadIdx.x == 0) {
          float m2 = 0.f;
          for (int w = 0; w < tc::kEpiWarps; ++w) m2 = fmaxf(m2, (float)sh.red[w]);
          int e = 0;
          if (m2 > 0.f && isfinite(m2)) {
            frexpf(m2, &e);  // m2 in [2^(e-1), 2^e)
            e = 8 - e;
          }
          s_ctl.exact = max(-120, min(120, e));
        }
        tc::epi_bar();
        isc = ldexpf(1.f, s_ctl.exact);
        inv_isc = ldexpf(1.f, -s_ctl.exact);
      }
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
          float lam[tc::kCW], x[tc::kCW], kl[tc::kCW];
          const bool v = valid(tile);
          // after the first interval, the last evaluation was the previous
          // step's stage 7 at this same t (the interval boundary), on this
          // CTA's only tile: its activations are reused, the jump changed lam only
          const bool reuse = ivi > 0 && G >= a.ntiles;
          if (v) {
            tc::tl_ldv(a.lam[cur] + tofs(tile), lam);
            if (!reuse) dense_u(tile, n, hb, x);
          } else {
            for (int i = 0; i < tc::kCW; ++i) lam[i] = x[i] = 0.f;
          }
          ok = adj_eval(lam, x, fs, Pb[iP1], (float)c_tab.b[0], kl, reuse, tile, false);
          if (reuse && tile == (int)blockIdx.x) ++nf_vjp;
          if (v) tc::tl_stv(klb(0) + tofs(tile), kl);
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
          if (!valid(tile)) continue;
          float l[tc::kCW], f[tc::kCW];
          tc::tl_ldv(a.lam[cur] + tofs(tile), l);
          tc::tl_ldv(klb(0) + tofs(tile), f);
          #pragma unroll
          for (int i = 0; i < tc::kCW; ++i) {
            if (i >= th.nmine) continue;
            const float sk = (float)a.abstol + fabsf(l[i]) * (float)a.reltol;
            const float xx = l[i] / sk, yy = f[i] / sk;
            p0 = fmaf(xx, xx, p0);
            p1 = fmaf(yy, yy, p1);
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
            dense_setup(iv, t - dt0, &s_n[0], s_hb[0]);
          }
        }
        tc::epi_bar();
        par ^= 1;
        const float hf = s_ctl.hf;
        const int n = s_n[0];
        float hb[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) hb[j] = s_hb[0][j];
        float p2 = 0.f;
        for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
          const bool v = valid(tile);
          float l[tc::kCW], f0[tc::kCW], x[tc::kCW], f1[tc::kCW];
          if (v) {
            tc::tl_ldv(a.lam[cur] + tofs(tile), l);
            tc::tl_ldv(klb(0) + tofs(tile), f0);
            dense_u(tile, n, hb, x);
          } else {
            for (int i = 0; i < tc::kCW; ++i) l[i] = f0[i] = x[i] = 0.f;
          }
          float li[tc::kCW];
          for (int i = 0; i < tc::kCW; ++i) li[i] = l[i] + hf * f0[i];
          ok = adj_eval(li, x, -1, nullptr, 0.f, f1, false, tile, false);
          if (v) {
            #pragma unroll
            for (int i = 0; i < tc::kCW; ++i) {
              if (i >= th.nmine) continue;
              const float sk = (float)a.abstol + fabsf(l[i]) * (float)a.reltol;
              const float z = (f1[i] - f0[i]) / sk;
              p2 = fmaf(z, z, p2);
            }
          }
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
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
          if (valid(tile)) stage_u(tile);
        float perr = 0.f;
        for (int i = 1; i < 7 && ok; ++i) {
          float ha[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) ha[j] = s_ha[i - 1][j];
          float* P = (i < 6) ? Pmid : Pb[iP7];
          const int slot = (i < 6) ? i : tc::kImgSlots - 1 - fs;
          if (i == 6) {
            zero_bias(P);
            tc::epi_bar();
          }
          const float cw = (i < 6) ? (float)c_tab.b[i] : (float)c_tab.b[0];
          for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
            const bool v = valid(tile);
            const size_t g = tofs(tile);  // tile layout
            float Y[tc::kCW], x[tc::kCW], kl[tc::kCW];
            if (v) {
              // Y = lam + (comp + sum_j h a_ij k_j), in two parts of kPart
              // components whose loads are all in flight together
#pragma unroll
              for (int hf = 0; hf < 2; ++hf) {
                float lv[tc::kPart], sv[tc::kPart], kv[6][tc::kPart];
                tc::tl_ldp(lcur + g, hf, lv);
                tc::tl_ldp(ccur + g, hf, sv);
#pragma unroll
                for (int j = 0; j < 6; ++j)
                  if (j < i) tc::tl_ldp(klb(j) + g, hf, kv[j]);
#pragma unroll
                for (int q = 0; q < tc::kPart; ++q) {
                  float sq = sv[q];
#pragma unroll
                  for (int j = 0; j < 6; ++j)
                    if (j < i) sq = fmaf(ha[j], kv[j][q], sq);
                  sv[q] = sq;
                  Y[tc::kPart * hf + q] = lv[q] + sq;
                }
                if (i == 6) {
                  // stage 7 reads k1..k6 anyway: the embedded error
                  // estimate's sum over them is formed here and parked in
                  // the k7 slot; the new lam and its compensation are stored
                  float lt[tc::kPart], cn[tc::kPart];
#pragma unroll
                  for (int q = 0; q < tc::kPart; ++q) {
                    float e = 0.f;
#pragma unroll
                    for (int j = 0; j < 6; ++j) e = fmaf(s_hbt[j], kv[j][q], e);
                    lt[q] = e;
                    cn[q] = sv[q] - (Y[tc::kPart * hf + q] - lv[q]);
                  }
                  tc::tl_stp(klb(6) + g, hf, lt);
                  tc::tl_stp(lnew + g, hf, Y + tc::kPart * hf);
                  tc::tl_stp(cnew + g, hf, cn);
                }
              }
              tc::tl_ldv(A.xst + (size_t)(i - 1) * SBt + g, x);
            } else {
              for (int q = 0; q < tc::kCW; ++q) Y[q] = x[q] = 0.f;
            }
            // stage 7 (i == 6) is at the same time as stage 6 (c6 = c7 = 1): on
            // a CTA's only tile its activations are re-emitted, not recomputed
            const bool re = i == 6 && G >= a.ntiles && c67_same;
            ok = adj_eval(Y, x, slot, P, cw, kl, false, tile, re);
            if (re) ++nf_vjp;
            if (v) {
              if (i == 6) {
                // lam, the stage value and the error sum over k1..k6 again
                // (stored above): nothing of the stage arithmetic stays in
                // registers across adj_eval
                const float hbt6 = s_hbt[6];
#pragma unroll
                for (int hf = 0; hf < 2; ++hf) {
                  float lt[tc::kPart], lv[tc::kPart], yv[tc::kPart];
                  tc::tl_ldp(klb(6) + g, hf, lt);
                  tc::tl_ldp(lcur + g, hf, lv);
                  tc::tl_ldp(lnew + g, hf, yv);
#pragma unroll
                  for (int q = 0; q < tc::kPart; ++q) {
                    if (tc::kPart * hf + q >= th.nmine) continue;
                    const float e = fmaf(hbt6, kl[tc::kPart * hf + q], lt[q]);
                    const float sc = (float)a.abstol + fmaxf(fabsf(lv[q]), fabsf(yv[q])) * (float)a.reltol;
                    const float rr = e / sc;
                    perr = isfinite(yv[q]) ? fmaf(rr, rr, perr) : INFINITY;
                  }
                }
                tc::tl_stv(klb(i) + g, kl);
              } else {
                tc::tl_stv(klb(i) + g, kl);
              }
            }
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
          if (!valid(tile)) continue;
          float v[tc::kCW];
          tc::tl_ldv(a.lam[cur] + tofs(tile), v);
          for (int qq = 0; qq < iv.nsave_lo; ++qq) {
            float d[tc::kCW];
            ldv(a.dLdu + (size_t)(iv.save_lo + qq) * SB + gofs(tile), th.nmine, vec, d);
            for (int i = 0; i < tc::kCW; ++i) v[i] += d[i];
          }
          tc::tl_stv(a.lam[cur] + tofs(tile), v);
        }
      }
    }
    if (!ok && ret == GBNDE_RET_SUCCESS) ret = GBNDE_RET_BARRIER_TIMEOUT;
    if (ret == GBNDE_RET_SUCCESS) {
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
        if (valid(tile)) {
          float v[tc::kCW];
          tc::tl_ldv(a.lam[cur] + tofs(tile), v);
          stv(a.dLdu0 + gofs(tile), th.nmine, vec, v);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.counters[CT_NF] = nf_adj;
      a.counters[CT_NVJP] = nf_vjp;
      a.counters[CT_NACCEPT] = nacc;
      a.counters[CT_NREJECT] = nrej;
      a.counters[CT_NRECOMP] = nf_rec;
      const int e = ((volatile int*)&sh.err)[0];
      // a weight-gradient image value that did not fit FP16 (status word 3,
      // set before the solve's last grid barrier) makes the gradient invalid
      if (ret == GBNDE_RET_SUCCESS && ((volatile int*)a.status)[3] != 0) ret = GBNDE_RET_UNSTABLE;
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

// dLdp[i] = sum over CTAs of (mu_acc - mu_comp) (mu_comp == nullptr: mu_acc
// alone), in CTA order, as a compensated (Kahan) FP32 sum: FP64 arithmetic is
// slow on this GPU and made this pass compute-bound; the compensation keeps
// the sum of the ~100 per-CTA terms to FP32 rounding. Per-CTA slots are
// `stride` floats apart; `P` parameters are written.
__global__ void reduce_mu_comp_kernel(const float* __restrict__ acc, const float* __restrict__ comp,
                                      int nblk, int stride, int P, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  float s = 0.f, c = 0.f;
  auto add = [&](float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  };
  for (int b = 0; b < nblk; ++b) {
    const size_t o = (size_t)b * stride + i;
    // both parts of the CTA's compensated sum enter as terms
    add(__ldcs(acc + o));
    if (comp) add(-__ldcs(comp + o));
  }
  out[i] = s - c;
}

int launch_bwd_tc(const BwdTcArgs& a, int grid, cudaStream_t st) {
  if (tc_check_regs((const void*)bwd_tc_kernel)) return -1;
  cudaError_t e = cudaFuncSetAttribute(bwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes);
  if (e != cudaSuccess) return -1;
  void* args[] = {(void*)&a};
  e = cudaLaunchCooperativeKernel((const void*)bwd_tc_kernel, dim3(grid), dim3(tc::kThreads), args,
                                  tc::kSmemBytes, st);
  return e == cudaSuccess ? 0 : -1;
}

int launch_reduce_mu_comp(const float* acc, const float* comp, int nblk, int stride, int P, float* out,
                          cudaStream_t st) {
  reduce_mu_comp_kernel<<<(P + 255) / 256, 256, 0, st>>>(acc, comp, nblk, stride, P, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
