// fwd_tcw.cu -- persistent Tsit5 forward solve, BF16 tensor-core form, for
// networks beyond the single-accumulator engine: state dim up to 256, hidden
// widths up to 1024, optionally t appended as an input row.
//
// Same algorithm and controller as fwd_tc.cu (the integrator loop of
// `solve(prob, Tsit5(); saveat, abstol, reltol)` at src/neural_de.jl:55-58).
// The right-hand side runs on the tensor-core engine in stash mode
// (tc_engine.cuh): every layer input is written by the epilogue into the
// CTA's global stash as split-BF16 64-column chunks, and a layer wider than
// 256 outputs is computed as several N-block ops (at most 256 TMEM columns
// each) that all bulk-load the same stash chunks. Layer l's input lives in
// stash buffer l % 2.
//
// State vectors are kept in 64-component chunks: chunk c of tile T is the
// "virtual tile" T * nsc + c of the tile layout (tc::tl_offset_cw), so the
// per-thread stage arithmetic is that of the single-chunk kernel, repeated
// over the chunks. Epilogue thread (warp w, lane l) owns trajectory row
// r = 32 (w % 4) + l and columns kCW (w / 4) .. + kCW of every chunk.
#include "tc_args.h"

namespace gbnde {

namespace {

struct ThrW {
  int r, ch;
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
// t at hs4[k * kEpiThreads + t]): contiguous per warp.
__device__ __forceinline__ void hs_ldv(const float4* hs4, int k0, float* x) {
#pragma unroll
  for (int j = 0; j < tc::kCW / 4; ++j) {
    const float4 q = hs4[(size_t)(k0 + j) * tc::kEpiThreads + threadIdx.x];
    x[4 * j] = q.x; x[4 * j + 1] = q.y; x[4 * j + 2] = q.z; x[4 * j + 3] = q.w;
  }
}
__device__ __forceinline__ void hs_stv(float4* hs4, int k0, const float* x) {
#pragma unroll
  for (int j = 0; j < tc::kCW / 4; ++j)
    hs4[(size_t)(k0 + j) * tc::kEpiThreads + threadIdx.x] = make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
}

__device__ __forceinline__ bool epi_grid_barrier(const FwdArgs& a, unsigned int& gen, int* okflag) {
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

}  // namespace

// One right-hand side of a tile on the stash engine. in(c, x) fills this
// thread's kCW columns of input chunk c (c < kc0); out(c, v) receives its
// kCW columns of output chunk c (c < nsc). Returns false if a wait gave up.
template <class In, class Out>
__device__ __forceinline__ bool epi_rhs_w(const FwdTcwArgs& A, tc::EpiState& e, tc::Shared& sh, uint8_t* stash,
                                          const ThrW& th, In&& in, Out&& out) {
  const MlpDev& m = A.t.f.mlp;
  const uint32_t lane_base = ((uint32_t)((threadIdx.x >> 5) & 3) * 32) << 16;
  const int kc0 = (m.dims[0] + 63) / 64;
  for (int c = 0; c < kc0; ++c) {
    float x[tc::kCW];
    in(c, x);
    tc::stash_write(stash, sh, 0, c, th.r, th.ch, x);
  }
  for (int l = 0; l < m.nlayers - 1; ++l) {
    const int N = m.dims[l + 1];
    const int nb = (N + 255) / 256;
    const int ob = (l + 1) & 1;
    for (int b = 0; b < nb; ++b) {
      uint32_t col;
      if (!tc::epi_wait_acc(e, sh, &col)) return false;
      const int nch = (min(256, N - 256 * b) + 63) / 64;
      for (int cc = 0; cc < nch; ++cc) {
        const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
        float v[tc::kCW], bc[tc::kCW];
        tc::load_bias_cw(A.t.bias[l], n0, N, bc);
        tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
        tc::bias_act_cw(v, bc, m.act[l], n0, N);
        tc::stash_write(stash, sh, ob, 4 * b + cc, th.r, th.ch, v);
      }
      tc::epi_release_acc(e, sh);
    }
  }
  {
    const int L = m.nlayers, N = m.dims[L];
    uint32_t col;
    if (!tc::epi_wait_acc(e, sh, &col)) return false;
    for (int c = 0; c < (N + 63) / 64; ++c) {
      const int n0 = 64 * c + tc::kCW * th.ch;
      float v[tc::kCW], bc[tc::kCW];
      tc::load_bias_cw(A.t.bias[L - 1], n0, N, bc);
      tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
      tc::bias_act_cw(v, bc, m.act[L - 1], n0, N);
      out(c, v);
    }
    tc::epi_release_acc(e, sh);
  }
  return true;
}

// FFJORD right-hand side of one tile (state [z; delta_logp], d = ffd rows of
// z, d + 1 <= 64): [f(z [, t]); -e . (J e)] with the Hutchinson direction e of
// the trajectory (src/ffjord.jl:81-115, e fixed per solve). The primal chain
// a_{l+1} = act(W_l a_l + b_l) and the tangent chain
// adot_{l+1} = act'(.) (W_l adot_l) (the forward-mode derivative along e) run
// interleaved per layer on the same weights: P_l from stash buffer l % 2, T_l
// from buffer 2 + l % 2. The primal activations go to the thread's scratch
// for the tangent drain's act'. in(c, x) fills the network input chunk c;
// out(0, k) receives the state chunk of the derivative (f and, at row d,
// minus the trace estimate, reduced over the row's four column groups through
// the CTA's slice of trs).
template <class In, class Out>
__device__ __forceinline__ bool epi_rhs_ffj(const FwdTcwArgs& A, tc::EpiState& e, tc::Shared& sh, uint8_t* stash,
                                            const ThrW& th, float4* hs4, const float* erow, float* trs, In&& in,
                                            Out&& out) {
  const MlpDev& m = A.t.f.mlp;
  const int L = m.nlayers, d = A.t.f.ffd;
  const uint32_t lane_base = ((uint32_t)((threadIdx.x >> 5) & 3) * 32) << 16;
  const int kc0 = (m.dims[0] + 63) / 64;
  for (int c = 0; c < kc0; ++c) {
    float x[tc::kCW];
    in(c, x);
    tc::stash_write(stash, sh, 0, c, th.r, th.ch, x);
#pragma unroll
    for (int i = 0; i < tc::kCW; ++i) {
      const int col = 64 * c + tc::kCW * th.ch + i;
      x[i] = (erow != nullptr && col < d) ? erow[col] : 0.f;
    }
    tc::stash_write<2>(stash, sh, 2, c, th.r, th.ch, x);
  }
  int hoff = 0;
  for (int l = 0; l < L - 1; ++l) {
    const int N = m.dims[l + 1];
    const int ob = (l + 1) & 1;
    for (int b = 0; b * 256 < N; ++b) {  // primal P_l
      uint32_t col;
      if (!tc::epi_wait_acc(e, sh, &col)) return false;
      const int nch = (min(256, N - 256 * b) + 63) / 64;
      for (int cc = 0; cc < nch; ++cc) {
        const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
        float v[tc::kCW], bc[tc::kCW];
        tc::load_bias_cw(A.t.bias[l], n0, N, bc);
        tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
        tc::bias_act_cw(v, bc, m.act[l], n0, N);
        hs_stv(hs4, (hoff + tc::kCW * (4 * b + cc)) / 4, v);
        tc::stash_write(stash, sh, ob, 4 * b + cc, th.r, th.ch, v);
      }
      tc::epi_release_acc(e, sh);
    }
    for (int b = 0; b * 256 < N; ++b) {  // tangent T_l
      uint32_t col;
      if (!tc::epi_wait_acc(e, sh, &col)) return false;
      const int nch = (min(256, N - 256 * b) + 63) / 64;
      for (int cc = 0; cc < nch; ++cc) {
        const int n0 = 256 * b + 64 * cc + tc::kCW * th.ch;
        float v[tc::kCW], y[tc::kCW];
        hs_ldv(hs4, (hoff + tc::kCW * (4 * b + cc)) / 4, y);
        tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(64 * cc + tc::kCW * th.ch), v);
        tc::deriv_mul_cw(v, y, m.act[l], n0, N);
        tc::stash_write<2>(stash, sh, 2 + ob, 4 * b + cc, th.r, th.ch, v);
      }
      tc::epi_release_acc(e, sh);
    }
    hoff += tc::kCW * ((N + 63) / 64);
  }
  // output layer (d outputs, one chunk): f from P, J e from T
  const int n0 = tc::kCW * th.ch;
  float f[tc::kCW];
  {
    uint32_t col;
    if (!tc::epi_wait_acc(e, sh, &col)) return false;
    float bc[tc::kCW];
    tc::load_bias_cw(A.t.bias[L - 1], n0, d, bc);
    tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, f);
    tc::bias_act_cw(f, bc, m.act[L - 1], n0, d);
    tc::epi_release_acc(e, sh);
  }
  float part = 0.f;
  {
    uint32_t col;
    if (!tc::epi_wait_acc(e, sh, &col)) return false;
    float v[tc::kCW];
    tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
    tc::deriv_mul_cw(v, f, m.act[L - 1], n0, d);
#pragma unroll
    for (int i = 0; i < tc::kCW; ++i)
      if (erow != nullptr && n0 + i < d) part = fmaf(erow[n0 + i], v[i], part);
    tc::epi_release_acc(e, sh);
  }
  // the row's trace: its four column groups' parts, in a fixed order
  trs[th.ch * 128 + th.r] = part;
  tc::epi_bar();
  const float tr = ((trs[th.r] + trs[128 + th.r]) + trs[256 + th.r]) + trs[384 + th.r];
  tc::epi_bar();
#pragma unroll
  for (int i = 0; i < tc::kCW; ++i)
    if (n0 + i == d) f[i] = -tr;
  out(0, f);
  return true;
}

__global__ void __launch_bounds__(tc::kThreads, 1) fwd_tcw_kernel(FwdTcwArgs A) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* aring = smem;
  uint8_t* wring = smem + tc::kARing * tc::kASlotBytes;
  __shared__ tc::Shared sh;
  __shared__ int s_ok;
  __shared__ StepCtl s_ctl;
  const FwdArgs& a = A.t.f;
  const int warp = threadIdx.x >> 5;

  tc::init_shared(sh);
  if (warp == tc::kMmaWarp) tc::tmem_alloc(&sh.tmem_base, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp >= tc::kMmaWarp) {
    tc::regs_give_ctl();
    if (warp == tc::kMmaWarp) tc::mma_loop(A.t.ops, sh, aring, wring);
    else if (warp == tc::kTmaWarp) tc::tma_loop(A.t.ops, sh, aring, wring);
  } else {
    tc::regs_take_epi();
    // ======================= epilogue warps =======================
    const int S = a.S, G = gridDim.x, nsc = A.nsc;
    const size_t SB = (size_t)S * a.B;
    const double N = (double)SB;
    const double tdir = a.t1 >= a.t0 ? 1.0 : -1.0;
    const bool timein = a.mlp.timein != 0;
    // state inputs of the network: the whole state, or z without FFJORD's
    // delta_logp row (the time row, if any, takes column netS)
    const int netS = a.ffj ? a.ffd : S;
    ThrW th;
    th.r = 32 * (warp & 3) + (threadIdx.x & 31);
    th.ch = warp >> 2;
    uint8_t* stash = A.stash + (size_t)blockIdx.x * tc::kStashCta;
    float4* hs4 = a.ffj ? reinterpret_cast<float4*>(A.hscr + (size_t)blockIdx.x * tc::kEpiThreads * A.hvals) : nullptr;
    float* trs = a.ffj ? A.trs + (size_t)blockIdx.x * 512 : nullptr;
    tc::EpiState es;
    tc::epi_state_init(es);
    unsigned int gen = 0;
    int par = 0, cur = 0;
    int ret = GBNDE_RET_SUCCESS;
    long long nf = 0, naccept = 0, nreject = 0, iter = 0;
    const bool dense = A.t.dense != nullptr;
    const size_t SBt = (size_t)a.ntiles * nsc * tc::kTileVec;
    auto kptr = [&](int j) -> float* {
      if (dense) return A.t.dense + ((size_t)min(naccept, A.t.dense_slots - 1) * 8 + 1 + j) * SBt;
      return A.t.kring + (size_t)j * SBt;
    };
    // chunk c of tile T: the API offset of this thread's first component and
    // the tile-layout offset of virtual tile T * nsc + c
    auto gofs = [&](int tile, int c) -> size_t {
      return ((size_t)tile * 128 + th.r) * S + 64 * c + tc::kCW * th.ch;
    };
    auto tofs = [&](int tile, int c) -> size_t { return tc::tl_offset_cw(tile * nsc + c, th.ch, th.r); };
    auto rowok = [&](int tile) -> bool { return tile * 128 + th.r < a.B; };
    // input chunk c >= nsc (the time row when S is a multiple of 64): t at
    // column S, zeros elsewhere; inside the state chunks the time column
    // (S % 64 != 0) is filled by the callers
    auto tcol = [&](int c, double tt, float* x) {
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) x[i] = (timein && 64 * c + tc::kCW * th.ch + i == netS) ? (float)tt : 0.f;
    };
    auto with_t = [&](int c, double tt, float* x) {
      if (!timein && netS == S) return;
#pragma unroll
      for (int i = 0; i < tc::kCW; ++i) {
        const int col = 64 * c + tc::kCW * th.ch + i;
        if (col == netS) x[i] = timein ? (float)tt : 0.f;
        else if (col > netS && col < S) x[i] = 0.f;
      }
    };
    // one right-hand side of a tile: the MLP, or FFJORD's augmented one
    auto rhs = [&](int tile, auto&& in, auto&& out) -> bool {
      if (a.ffj) {
        const float* erow =
            (rowok(tile) && a.noise != nullptr) ? a.noise + ((size_t)tile * 128 + th.r) * a.ffd : nullptr;
        return epi_rhs_ffj(A, es, sh, stash, th, hs4, erow, trs, in, out);
      }
      return epi_rhs_w(A, es, sh, stash, th, in, out);
    };
    bool ok = true;

    // ---- k1 = f(u0); state, compensation and slot 0 ---------------------------
    for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
      const bool v = rowok(tile);
      ok = rhs(
          tile,
          [&](int c, float* x) {
            if (c >= nsc) { tcol(c, a.t0, x); return; }
            const int nm = nmine_of(S, c, th.ch);
            if (v) ldv_api(a.u0 + gofs(tile, c), nm, x);
            else
              for (int i = 0; i < tc::kCW; ++i) x[i] = 0.f;
            float z[tc::kCW];
            for (int i = 0; i < tc::kCW; ++i) z[i] = 0.f;
            const size_t tg = tofs(tile, c);
            tc::tl_stv(a.ubuf[0] + tg, x);
            tc::tl_stv(A.t.comp[0] + tg, z);
            if (dense) tc::tl_stv(A.t.dense + tg, x);
            with_t(c, a.t0, x);
          },
          [&](int c, const float* k) {
            float kk[tc::kCW];
            const int nm = nmine_of(S, c, th.ch);
            for (int i = 0; i < tc::kCW; ++i) kk[i] = (v && i < nm) ? k[i] : 0.f;
            tc::tl_stv(kptr(0) + tofs(tile, c), kk);
          });
    }
    nf = 1;
    int isave = 0;
    while (isave < a.nsave && a.saveat[isave] == a.t0) {
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
        if (rowok(tile))
          for (int c = 0; c < nsc; ++c) {
            float Y[tc::kCW];
            const int nm = nmine_of(S, c, th.ch);
            ldv_api(a.u0 + gofs(tile, c), nm, Y);
            stv_api(a.usave + (size_t)isave * SB + gofs(tile, c), nm, Y);
          }
      ++isave;
    }
    if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }

    // ---- initial step ---------------------------------------------------------------
    // The controller's scalar FP64 work (norms, the initial step, the PI
    // update, stage coefficients and times, save weights) runs on epilogue
    // thread 0 and reaches the others through shared memory (s_ctl): FP64
    // executes at a small fraction of the FP32 rate, and each of the epilogue
    // warps would repeat it. Per-thread parts of the norms are FP32 sums of a
    // thread's own components; the sums across threads and CTAs are FP64.
    double dt;  // thread 0's controller state (t, dt, qold) is the one used
    dt = a.dt0;
    if (!(a.dt0 > 0.0)) {
      float p0 = 0.f, p1 = 0.f;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        if (!rowok(tile)) continue;
        for (int c = 0; c < nsc; ++c) {
          const int nm = nmine_of(S, c, th.ch);
          float u[tc::kCW], f[tc::kCW];
          tc::tl_ldv(a.ubuf[0] + tofs(tile, c), u);
          tc::tl_ldv(kptr(0) + tofs(tile, c), f);
          for (int i = 0; i < tc::kCW; ++i) {
            if (i >= nm) continue;
            const float sk = (float)a.abstol + fabsf(u[i]) * (float)a.reltol;
            const float x = u[i] / sk, y = f[i] / sk;
            p0 = fmaf(x, x, p0);
            p1 = fmaf(y, y, p1);
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
      if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      {
        const double q0 = tc::epi_partials_sum0(pp, G), q1 = tc::epi_partials_sum0(pp + G, G);
        if (threadIdx.x == 0) {
          const double d0 = sqrt(q0 / N), d1 = sqrt(q1 / N);
          double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? fmax(a.dtmin, 1e-6) : 0.01 * (d0 / d1);
          dt0 = fmin(dt0, a.dtmax);
          s_ctl.d1 = d1;
          s_ctl.dt0 = dt0;
          s_ctl.hf = (float)(tdir * dt0);
          s_ctl.tst[0] = a.t0 + tdir * dt0;
        }
      }
      tc::epi_bar();
      par ^= 1;
      const float hf = s_ctl.hf;
      const double t1p = s_ctl.tst[0];
      float p2 = 0.f;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
        const bool v = rowok(tile);
        ok = rhs(
            tile,
            [&](int c, float* x) {
              if (c >= nsc) { tcol(c, t1p, x); return; }
              float u[tc::kCW], f0[tc::kCW];
              tc::tl_ldv(a.ubuf[0] + tofs(tile, c), u);
              tc::tl_ldv(kptr(0) + tofs(tile, c), f0);
              for (int i = 0; i < tc::kCW; ++i) x[i] = u[i] + hf * f0[i];
              with_t(c, t1p, x);
            },
            [&](int c, const float* f1) {
              if (!v) return;
              const int nm = nmine_of(S, c, th.ch);
              float u[tc::kCW], f0[tc::kCW];
              tc::tl_ldv(a.ubuf[0] + tofs(tile, c), u);
              tc::tl_ldv(kptr(0) + tofs(tile, c), f0);
              for (int i = 0; i < tc::kCW; ++i) {
                if (i >= nm) continue;
                const float sk = (float)a.abstol + fabsf(u[i]) * (float)a.reltol;
                const float z = (f1[i] - f0[i]) / sk;
                p2 = fmaf(z, z, p2);
              }
            });
      }
      nf += 1;
      if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      const double s2 = tc::epi_sum0_f(p2, sh);
      pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = s2;
      if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      {
        const double q2 = tc::epi_partials_sum0(pp, G);
        if (threadIdx.x == 0) {
          const double dt0 = s_ctl.dt0;
          const double d2 = sqrt(q2 / N) / dt0;
          const double mm = fmax(s_ctl.d1, d2);
          const double dt1 = (mm <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(mm)) / 5.0);
          dt = fmax(a.dtmin, fmin(100.0 * dt0, fmin(dt1, a.dtmax)));
        }
      }
      par ^= 1;
    }

    // ---- step loop ---------------------------------------------------------------------
    {
      double t = a.t0, qold = kQoldInit;
      int ib = 0, nck = 0;
      for (;;) {
        // step setup (thread 0): continue?, the step size, the stage coefficients and times
        if (threadIdx.x == 0) {
          s_ctl.go = tdir * (a.t1 - t) > 0.0;
          const double rem = fabs(a.t1 - t);
          s_ctl.clipped = dt >= rem;
          s_ctl.habs = s_ctl.clipped ? rem : dt;
          const double h = tdir * s_ctl.habs;
          s_ctl.t = t;
          s_ctl.h = h;
          for (int i = 1; i < 7; ++i) {
            for (int j = 0; j < i; ++j) s_ctl.ha[i - 1][j] = (float)(h * c_tab.a[i][j]);
            s_ctl.tst[i] = t + c_tab.c[i] * h;
          }
          for (int j = 0; j < 7; ++j) s_ctl.hbt[j] = (float)(h * c_tab.btilde[j]);
        }
        tc::epi_bar();
        if (!s_ctl.go) break;
        if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
        ++iter;
        const float* ucur = a.ubuf[cur];
        float* unew = a.ubuf[cur ^ 1];
        const float* ccur = A.t.comp[cur];
        float* cnew = A.t.comp[cur ^ 1];
        float perr = 0.f;
        for (int i = 1; i < 7 && ok; ++i) {
          float ha[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) ha[j] = j < i ? s_ctl.ha[i - 1][j] : 0.f;
          float hbt[7];
#pragma unroll
          for (int j = 0; j < 7; ++j) hbt[j] = s_ctl.hbt[j];
          const double ti = s_ctl.tst[i];
          for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
            const bool v = rowok(tile);
            ok = rhs(
                tile,
                [&](int c, float* Y) {
                  if (c >= nsc) { tcol(c, ti, Y); return; }
                  const size_t g = tofs(tile, c);
                  float u[tc::kCW], s[tc::kCW];
                  tc::tl_ldv(ucur + g, u);
                  tc::tl_ldv(ccur + g, s);
                  if (i < 6) {
                    for (int j = 0; j < 5; ++j) {
                      if (j >= i) break;
                      float kj[tc::kCW];
                      tc::tl_ldv(kptr(j) + g, kj);
#pragma unroll
                      for (int q = 0; q < tc::kCW; ++q) s[q] = fmaf(ha[j], kj[q], s[q]);
                    }
                  } else {
                    // the embedded error estimate's sum over k1..k6, parked in the k7 slot
                    float ut[tc::kCW];
#pragma unroll
                    for (int q = 0; q < tc::kCW; ++q) ut[q] = 0.f;
                    for (int j = 0; j < 6; ++j) {
                      float kj[tc::kCW];
                      tc::tl_ldv(kptr(j) + g, kj);
#pragma unroll
                      for (int q = 0; q < tc::kCW; ++q) {
                        s[q] = fmaf(ha[j], kj[q], s[q]);
                        ut[q] = fmaf(hbt[j], kj[q], ut[q]);
                      }
                    }
                    tc::tl_stv(kptr(6) + g, ut);
                  }
#pragma unroll
                  for (int q = 0; q < tc::kCW; ++q) Y[q] = u[q] + s[q];
                  if (i == 6) {
                    float cn[tc::kCW];
#pragma unroll
                    for (int q = 0; q < tc::kCW; ++q) cn[q] = s[q] - (Y[q] - u[q]);
                    tc::tl_stv(unew + g, Y);
                    tc::tl_stv(cnew + g, cn);
                  }
                  if (!v)
                    for (int q = 0; q < tc::kCW; ++q) Y[q] = 0.f;
                  with_t(c, ti, Y);
                },
                [&](int c, const float* kin) {
                  if (!v) return;
                  const int nm = nmine_of(S, c, th.ch);
                  const size_t g = tofs(tile, c);
                  float k[tc::kCW];
                  for (int q = 0; q < tc::kCW; ++q) k[q] = (q < nm) ? kin[q] : 0.f;
                  if (i == 6) {
                    float ut[tc::kCW], u[tc::kCW], Y[tc::kCW];
                    tc::tl_ldv(kptr(6) + g, ut);
                    tc::tl_ldv(ucur + g, u);
                    tc::tl_ldv(unew + g, Y);
                    for (int q = 0; q < tc::kCW; ++q) {
                      if (q >= nm) continue;
                      const float e = fmaf(hbt[6], k[q], ut[q]);
                      const float sc = (float)a.abstol + fmaxf(fabsf(u[q]), fabsf(Y[q])) * (float)a.reltol;
                      const float rr = e / sc;
                      perr = isfinite(Y[q]) ? fmaf(rr, rr, perr) : INFINITY;
                    }
                  }
                  tc::tl_stv(kptr(i) + g, k);
                });
          }
        }
        if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        nf += 6;
        const double se = tc::epi_sum0_f(perr, sh);
        double* pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) pp[blockIdx.x] = se;
        if (!epi_grid_barrier(a, gen, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        {
          // error norm, PI controller, saves and checkpoints of the step (thread 0)
          const double qe = tc::epi_partials_sum0(pp, G);
          if (threadIdx.x == 0) {
            const double eest = sqrt(qe / N);
            const double h = s_ctl.h, habs = s_ctl.habs;
            s_ctl.ret = GBNDE_RET_SUCCESS;
            s_ctl.accept = 0;
            if (!isfinite(eest)) {
              s_ctl.ret = GBNDE_RET_UNSTABLE;
            } else {
              double q11;
              double q = pi_q(eest, qold, &q11);
              if (blockIdx.x == 0 && iter - 1 < a.maxsteps) {
                double* tr = a.trace + 4 * (iter - 1);
                tr[0] = t;
                tr[1] = h;
                tr[2] = eest;
                tr[3] = eest <= 1.0 ? 1.0 : 0.0;
              }
              if (eest <= 1.0) {
                const double tnew = s_ctl.clipped ? a.t1 : t + h;
                s_ctl.accept = 1;
                s_ctl.tnew = tnew;
                int ns = 0;
                while (isave + ns < a.nsave && tdir * (a.saveat[isave + ns] - tnew) <= 0.0) ++ns;
                s_ctl.nsv = ns;
                bool need = false;
                while (ib < a.nbnd && tdir * (a.bnd[ib] - tnew) < 0.0) { need = true; ++ib; }
                s_ctl.need_ckpt = need;
                if (blockIdx.x == 0 && naccept < a.maxsteps) {
                  a.steplog[2 * naccept] = t;
                  a.steplog[2 * naccept + 1] = h;
                }
                t = tnew;
                if (q >= 1.0 && q <= 1.0) q = 1.0;
                qold = fmax(eest, kQoldInit);
                dt = fmax(fmin(habs / q, a.dtmax), a.dtmin);
              } else {
                dt = habs / fmin(1.0 / kQmin, q11 / kGamma);
                if (a.dtmin > 0.0 && dt <= a.dtmin) s_ctl.ret = GBNDE_RET_DTLESSTHANMIN;
              }
            }
          }
          tc::epi_bar();
        }
        par ^= 1;
        if (s_ctl.ret != GBNDE_RET_SUCCESS) {
          ret = s_ctl.ret;
          if (ret == GBNDE_RET_DTLESSTHANMIN) ++nreject;
          break;
        }
        if (s_ctl.accept) {
          const int nsv = s_ctl.nsv;
          for (int k = 0; k < nsv; ++k, ++isave) {
            if (threadIdx.x == 0) {
              const double sv = a.saveat[isave];
              s_ctl.exact = sv == s_ctl.tnew;
              if (!s_ctl.exact) {
                float bw[7];
                interp_weights((sv - s_ctl.t) / s_ctl.h, bw);
                for (int j = 0; j < 7; ++j) s_ctl.hb[j] = (float)(s_ctl.h * (double)bw[j]);
              }
            }
            tc::epi_bar();
            const bool exact = s_ctl.exact;
            float hb[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) hb[j] = s_ctl.hb[j];
            float* dst = a.usave + (size_t)isave * SB;
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
              if (!rowok(tile)) continue;
              for (int c = 0; c < nsc; ++c) {
                const size_t tg = tofs(tile, c);
                float o[tc::kCW];
                if (exact) {
                  tc::tl_ldv(unew + tg, o);
                } else {
                  // u + (comp + sum_j hb_j k_j), one float4 group of the
                  // thread's components at a time, its nine loads in flight
#pragma unroll
                  for (int jg = 0; jg < tc::kCW / 4; ++jg) {
                    float4 v9[9];
                    v9[0] = *reinterpret_cast<const float4*>(ucur + tg + jg * 512);
                    v9[1] = *reinterpret_cast<const float4*>(ccur + tg + jg * 512);
#pragma unroll
                    for (int j = 0; j < 7; ++j) v9[2 + j] = *reinterpret_cast<const float4*>(kptr(j) + tg + jg * 512);
                    float4 e = v9[1];
#pragma unroll
                    for (int j = 0; j < 7; ++j) {
                      e.x = fmaf(hb[j], v9[2 + j].x, e.x);
                      e.y = fmaf(hb[j], v9[2 + j].y, e.y);
                      e.z = fmaf(hb[j], v9[2 + j].z, e.z);
                      e.w = fmaf(hb[j], v9[2 + j].w, e.w);
                    }
                    o[4 * jg] = v9[0].x + e.x;
                    o[4 * jg + 1] = v9[0].y + e.y;
                    o[4 * jg + 2] = v9[0].z + e.z;
                    o[4 * jg + 3] = v9[0].w + e.w;
                  }
                }
                stv_api(dst + gofs(tile, c), nmine_of(S, c, th.ch), o);
              }
            }
            tc::epi_bar();  // s_ctl.hb is rewritten for the next save
          }
          if (s_ctl.need_ckpt && nck < a.max_ckpt) {
            float* dst = a.ckpt + (size_t)nck * SB;
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
              if (rowok(tile))
                for (int c = 0; c < nsc; ++c) {
                  float u[tc::kCW];
                  tc::tl_ldv(ucur + tofs(tile, c), u);
                  stv_api(dst + gofs(tile, c), nmine_of(S, c, th.ch), u);
                }
            if (blockIdx.x == 0 && threadIdx.x == 0) a.ckpt_step[nck] = (int)naccept;
            ++nck;
          }
          // FSAL: k7 becomes k1 of the next step (next dense slot, or in place)
          const float* k7 = kptr(6);
          ++naccept;
          for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
            if (!rowok(tile)) continue;
            for (int c = 0; c < nsc; ++c) {
              const size_t g = tofs(tile, c);
              float kk[tc::kCW];
              tc::tl_ldv(k7 + g, kk);
              if (dense && naccept < A.t.dense_slots) {
                float un[tc::kCW];
                tc::tl_ldv(unew + g, un);
                tc::tl_stv(A.t.dense + (size_t)naccept * 8 * SBt + g, un);
              }
              tc::tl_stv(kptr(0) + g, kk);
            }
          }
          cur ^= 1;
        } else {
          ++nreject;
        }
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.counters[CT_NCKPT] = nck;
        a.counters[CT_NATTEMPT] = iter;
        *a.tfinal = t;
      }
    }
  epi_done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.counters[CT_NF] = nf;
      a.counters[CT_NACCEPT] = naccept;
      a.counters[CT_NREJECT] = nreject;
      a.counters[5] = cur;
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

int launch_fwd_tcw(const FwdTcwArgs& a, int grid, cudaStream_t st) {
  if (tc_check_regs((const void*)fwd_tcw_kernel)) return -1;
  cudaError_t e = cudaFuncSetAttribute(fwd_tcw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes);
  if (e != cudaSuccess) return -1;
  void* args[] = {(void*)&a};
  e = cudaLaunchCooperativeKernel((const void*)fwd_tcw_kernel, dim3(grid), dim3(tc::kThreads), args,
                                  tc::kSmemBytes, st);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
