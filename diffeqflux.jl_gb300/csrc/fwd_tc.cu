// fwd_tc.cu -- persistent Tsit5 forward solve, BF16 tensor-core form.
//
// Same algorithm and controller as the plain FP32 kernel (fwd_f32.cu), which
// replaces the integrator loop of `solve(prob, Tsit5(); saveat, abstol,
// reltol)` at src/neural_de.jl:55-58, with the MLP right-hand side evaluated
// by the tensor-core engine (tc_engine.cuh): split-BF16 tcgen05 GEMMs with
// FP32 accumulation in tensor memory, weights streamed by bulk copies.
//
// Epilogue thread (warp w, lane l) owns trajectory row r = 32*(w%4) + l of the
// 128-trajectory tile and state components [kCW*(w/4), kCW*(w/4)+kCW); every
// state/stage value a thread touches in global memory is its own, so the
// stage arithmetic needs no synchronisation. State updates use a compensated
// (TwoSum) sum whose low-order part is carried across steps. t, h, the error
// reduction and the controller are FP64.
//
// Dense stage storage: with `dense` set, accepted step n keeps (u_n, k1..k7)
// in slot n -- the forward dense output the InterpolatingAdjoint backward
// interpolates, so no recompute is needed.
#include "tc_args.h"

namespace gbnde {


namespace {

struct Thr {
  int r, ch, nmine;
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

// Grid barrier run by the epilogue warps only (the MMA and producer warps keep
// running their loops).
__device__ __forceinline__ bool epi_grid_barrier(const FwdArgs& a, unsigned int& gen, tc::Shared& sh,
                                                 int* okflag) {
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

// Right-hand side of one tile on the tensor cores. Y: this thread's state
// components. Returns false if a wait gave up.
__device__ __forceinline__ bool epi_rhs(const FwdTcArgs& A, tc::EpiState& e, tc::Shared& sh,
                                        uint8_t* aring, const Thr& th, const float* Y, float* kout) {
  const MlpDev& m = A.f.mlp;
  float x[tc::kCW];
#pragma unroll
  for (int i = 0; i < tc::kCW; ++i) {
    const float y = (i < th.nmine) ? Y[i] : 0.f;
    x[i] = m.cube ? y * y * y : y;
  }
  if (!tc::epi_write_a(e, sh, aring, th.r, th.ch, x)) return false;
  const uint32_t lane_base = ((uint32_t)((threadIdx.x >> 5) & 3) * 32) << 16;
  for (int l = 0; l < m.nlayers - 1; ++l) {
    const int N = m.dims[l + 1];
    const int act = m.act[l];
    const float* b = A.bias[l];
    uint32_t col;
    if (!tc::epi_wait_acc(e, sh, &col)) return false;
    const int nch = (N + 63) / 64;
    for (int c = 0; c < nch; ++c) {
      float v[tc::kCW], bc[tc::kCW];
      const int n0 = 64 * c + tc::kCW * th.ch;
      tc::load_bias_cw(b, n0, N, bc);
      tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)n0, v);
      tc::bias_act_cw(v, bc, act, n0, N);
      if (!tc::epi_write_a(e, sh, aring, th.r, th.ch, v)) return false;
    }
    tc::epi_release_acc(e, sh);
  }
  {
    const float* b = A.bias[m.nlayers - 1];
    uint32_t col;
    if (!tc::epi_wait_acc(e, sh, &col)) return false;
    float v[tc::kCW], bc[tc::kCW];
    tc::load_bias_cw(b, tc::kCW * th.ch, m.dims[m.nlayers], bc);
    tc::tmem_ld_cw(sh.tmem_base + lane_base + col + (uint32_t)(tc::kCW * th.ch), v);
    // output layer: bias and its activation (identity for most models)
    tc::bias_act_cw(v, bc, m.act[m.nlayers - 1], tc::kCW * th.ch, m.dims[m.nlayers]);
#pragma unroll
    for (int i = 0; i < tc::kCW; ++i) kout[i] = (i < th.nmine) ? v[i] : 0.f;
    tc::epi_release_acc(e, sh);
  }
  return true;
}

}  // namespace

__global__ void __launch_bounds__(tc::kThreads, 1) fwd_tc_kernel(FwdTcArgs A) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* aring = smem;
  uint8_t* wring = smem + tc::kARing * tc::kASlotBytes;
  __shared__ tc::Shared sh;
  __shared__ int s_ok;
  __shared__ StepCtl s_ctl;
  const FwdArgs& a = A.f;
  const int warp = threadIdx.x >> 5;

  tc::init_shared(sh);
  if (warp == tc::kMmaWarp) tc::tmem_alloc(&sh.tmem_base, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp >= tc::kMmaWarp) {
    tc::regs_give_ctl();
    if (warp == tc::kMmaWarp) tc::mma_loop(A.ops, sh, aring, wring);
    else if (warp == tc::kTmaWarp) tc::tma_loop(A.ops, sh, aring, wring);
  } else {
    tc::regs_take_epi();
    // ======================= epilogue warps =======================
    const int S = a.S, G = gridDim.x;
    const size_t SB = (size_t)S * a.B;
    const double N = (double)SB;
    const double tdir = a.t1 >= a.t0 ? 1.0 : -1.0;
    Thr th;
    th.r = 32 * (warp & 3) + (threadIdx.x & 31);
    th.ch = warp >> 2;
    th.nmine = min(tc::kCW, max(0, S - tc::kCW * th.ch));
    const bool vec = (S % 4 == 0) && th.nmine == tc::kCW;
    tc::EpiState es;
    tc::epi_state_init(es);
    unsigned int gen = 0;
    int par = 0, cur = 0;
    int ret = GBNDE_RET_SUCCESS;
    long long nf = 0, naccept = 0, nreject = 0, iter = 0;
    const bool dense = A.dense != nullptr;
    // stage buffer j of the current attempt (slot = accepted-step index)
    // internal vectors (state, compensation, stages, dense slots) use the
    // tile layout; u0, the saved states and the checkpoints the API layout
    const size_t SBt = (size_t)a.ntiles * tc::kTileVec;
    auto kptr = [&](int j) -> float* {
      if (dense) return A.dense + ((size_t)min(naccept, A.dense_slots - 1) * 8 + 1 + j) * SBt;
      return A.kring + (size_t)j * SBt;
    };
    auto gofs = [&](int tile) -> size_t { return ((size_t)tile * 128 + th.r) * S + tc::kCW * th.ch; };
    auto tofs = [&](int tile) -> size_t { return tc::tl_offset_cw(tile, th.ch, th.r); };
    auto valid = [&](int tile) -> bool { return tile * 128 + th.r < a.B && th.nmine > 0; };
    bool ok = true;

    // ---- k1 = f(u0); state, compensation and slot 0 ---------------------------
    for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
      float Y[tc::kCW], k[tc::kCW];
      const bool v = valid(tile);
      const size_t g = gofs(tile);
      if (v) ldv(a.u0 + g, th.nmine, vec, Y);
      else
        for (int i = 0; i < tc::kCW; ++i) Y[i] = 0.f;
      ok = epi_rhs(A, es, sh, aring, th, Y, k);
      if (v) {
        float z[tc::kCW];
        for (int i = 0; i < tc::kCW; ++i) z[i] = 0.f;
        const size_t tg = tofs(tile);
        tc::tl_stv(a.ubuf[0] + tg, Y);
        tc::tl_stv(A.comp[0] + tg, z);
        if (dense) tc::tl_stv(A.dense + tg, Y);
        tc::tl_stv(kptr(0) + tg, k);
      }
    }
    nf = 1;
    int isave = 0;
    while (isave < a.nsave && a.saveat[isave] == a.t0) {
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
        if (valid(tile)) {
          float Y[tc::kCW];
          ldv(a.u0 + gofs(tile), th.nmine, vec, Y);
          stv(a.usave + (size_t)isave * SB + gofs(tile), th.nmine, vec, Y);
        }
      ++isave;
    }
    if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }

    // ---- initial step ---------------------------------------------------------------
    // The controller's scalar FP64 work (norms, the initial step, the PI
    // update, stage coefficients, save weights) runs on epilogue thread 0 and
    // reaches the others through shared memory (s_ctl): FP64 executes at a
    // small fraction of the FP32 rate, and each of the epilogue warps would
    // repeat it. Per-thread parts of the norms are FP32 sums of a thread's
    // own components; the sums across threads and CTAs are FP64.
    double dt;  // thread 0's controller state (t, dt, qold) is the one used
    dt = a.dt0;
    if (!(a.dt0 > 0.0)) {
      float p0 = 0.f, p1 = 0.f;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        if (!valid(tile)) continue;
        float u[tc::kCW], f[tc::kCW];
        ldv(a.u0 + gofs(tile), th.nmine, vec, u);
        tc::tl_ldv(kptr(0) + tofs(tile), f);
        #pragma unroll
        for (int i = 0; i < tc::kCW; ++i) {
          if (i >= th.nmine) continue;
          const float sk = (float)a.abstol + fabsf(u[i]) * (float)a.reltol;
          const float x = u[i] / sk, y = f[i] / sk;
          p0 = fmaf(x, x, p0);
          p1 = fmaf(y, y, p1);
        }
      }
      const double s0 = tc::epi_sum0_f(p0, sh);
      const double s1 = tc::epi_sum0_f(p1, sh);
      double* pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) {
        pp[blockIdx.x] = s0;
        pp[G + blockIdx.x] = s1;
      }
      if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      {
        const double q0 = tc::epi_partials_sum0(pp, G), q1 = tc::epi_partials_sum0(pp + G, G);
        if (threadIdx.x == 0) {
          const double d0 = sqrt(q0 / N), d1 = sqrt(q1 / N);
          double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? fmax(a.dtmin, 1e-6) : 0.01 * (d0 / d1);
          dt0 = fmin(dt0, a.dtmax);
          s_ctl.d1 = d1;
          s_ctl.dt0 = dt0;
          s_ctl.hf = (float)(tdir * dt0);
        }
      }
      tc::epi_bar();
      par ^= 1;
      const float hf = s_ctl.hf;
      float p2 = 0.f;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
        const bool v = valid(tile);
        float u[tc::kCW], f0[tc::kCW], Y[tc::kCW], f1[tc::kCW];
        if (v) {
          ldv(a.u0 + gofs(tile), th.nmine, vec, u);
          tc::tl_ldv(kptr(0) + tofs(tile), f0);
        } else {
          for (int i = 0; i < tc::kCW; ++i) u[i] = f0[i] = 0.f;
        }
        for (int i = 0; i < tc::kCW; ++i) Y[i] = u[i] + hf * f0[i];
        ok = epi_rhs(A, es, sh, aring, th, Y, f1);
        if (v) {
          #pragma unroll
          for (int i = 0; i < tc::kCW; ++i) {
            if (i >= th.nmine) continue;
            const float sk = (float)a.abstol + fabsf(u[i]) * (float)a.reltol;
            const float z = (f1[i] - f0[i]) / sk;
            p2 = fmaf(z, z, p2);
          }
        }
      }
      nf += 1;
      if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      const double s2 = tc::epi_sum0_f(p2, sh);
      pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = s2;
      if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
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
        // step setup (thread 0): continue?, the step size, the stage coefficients
        if (threadIdx.x == 0) {
          s_ctl.go = tdir * (a.t1 - t) > 0.0;
          const double rem = fabs(a.t1 - t);
          s_ctl.clipped = dt >= rem;
          s_ctl.habs = s_ctl.clipped ? rem : dt;
          const double h = tdir * s_ctl.habs;
          s_ctl.t = t;
          s_ctl.h = h;
          for (int i = 1; i < 7; ++i)
            for (int j = 0; j < i; ++j) s_ctl.ha[i - 1][j] = (float)(h * c_tab.a[i][j]);
          for (int j = 0; j < 7; ++j) s_ctl.hbt[j] = (float)(h * c_tab.btilde[j]);
        }
        tc::epi_bar();
        if (!s_ctl.go) break;
        if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
        ++iter;
        const float* ucur = a.ubuf[cur];
        float* unew = a.ubuf[cur ^ 1];
        const float* ccur = A.comp[cur];
        float* cnew = A.comp[cur ^ 1];
        float perr = 0.f;
        for (int i = 1; i < 7 && ok; ++i) {
          float ha[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) ha[j] = j < i ? s_ctl.ha[i - 1][j] : 0.f;
          float hbt[7];
#pragma unroll
          for (int j = 0; j < 7; ++j) hbt[j] = s_ctl.hbt[j];
          for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += G) {
            const bool v = valid(tile);
            const size_t g = tofs(tile);  // tile layout
            float u[tc::kCW], s[tc::kCW], Y[tc::kCW], k[tc::kCW];
            if (v) {
              tc::tl_ldv(ucur + g, u);
              tc::tl_ldv(ccur + g, s);
              if (i < 6) {
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                  if (j >= i) break;
                  float kj[tc::kCW];
                  tc::tl_ldv(kptr(j) + g, kj);
#pragma unroll
                  for (int q = 0; q < tc::kCW; ++q) s[q] = fmaf(ha[j], kj[q], s[q]);
                }
              } else {
                // stage 7 reads k1..k6 anyway: the embedded error estimate's
                // sum over them is formed here and parked in the k7 slot
                float ut[tc::kCW];
#pragma unroll
                for (int q = 0; q < tc::kCW; ++q) ut[q] = 0.f;
#pragma unroll
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
            } else {
#pragma unroll
              for (int q = 0; q < tc::kCW; ++q) Y[q] = 0.f;
            }
            ok = epi_rhs(A, es, sh, aring, th, Y, k);
            if (v) {
              if (i == 6) {
                // u, the stage value and the error sum over k1..k6 again
                // (stored above): nothing of the stage arithmetic stays in
                // registers across epi_rhs
                float ut[tc::kCW];
                tc::tl_ldv(kptr(6) + g, ut);
                tc::tl_ldv(ucur + g, u);
                tc::tl_ldv(unew + g, Y);
#pragma unroll
                for (int q = 0; q < tc::kCW; ++q) ut[q] = fmaf(hbt[6], k[q], ut[q]);
                tc::tl_stv(kptr(i) + g, k);
                #pragma unroll
                for (int q = 0; q < tc::kCW; ++q) {
                  if (q >= th.nmine) continue;
                  const float sc = (float)a.abstol + fmaxf(fabsf(u[q]), fabsf(Y[q])) * (float)a.reltol;
                  const float rr = ut[q] / sc;
                  perr = isfinite(Y[q]) ? fmaf(rr, rr, perr) : INFINITY;
                }
              } else {
                tc::tl_stv(kptr(i) + g, k);
              }
            }
          }
        }
        if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        nf += 6;
        const double se = tc::epi_sum0_f(perr, sh);
        double* pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) pp[blockIdx.x] = se;
        if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
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
              if (!valid(tile)) continue;
              const size_t g = gofs(tile), tg = tofs(tile);
              float o[tc::kCW];
              if (exact) {
                tc::tl_ldv(unew + tg, o);
              } else {
                // u + (comp + sum_j hb_j k_j), one float4 group of the
                // thread's components at a time, its nine loads in flight
                // together
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
              stv(dst + g, th.nmine, vec, o);
            }
            tc::epi_bar();  // s_ctl.hb is rewritten for the next save
          }
          if (s_ctl.need_ckpt && nck < a.max_ckpt) {
            float* dst = a.ckpt + (size_t)nck * SB;
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G)
              if (valid(tile)) {
                float u[tc::kCW];
                tc::tl_ldv(ucur + tofs(tile), u);
                stv(dst + gofs(tile), th.nmine, vec, u);
                if (A.ckcomp) {
                  // and the compensation, so that the adjoint's replay of the
                  // interval from here is bit-identical to this solve
                  float cp[tc::kCW];
                  tc::tl_ldv(ccur + tofs(tile), cp);
                  tc::tl_stv(A.ckcomp + (size_t)nck * SBt + tofs(tile), cp);
                }
              }
            if (blockIdx.x == 0 && threadIdx.x == 0) a.ckpt_step[nck] = (int)naccept;
            ++nck;
          }
          // FSAL: k7 becomes k1 of the next step (next dense slot, or in place)
          const float* k7 = kptr(6);
          ++naccept;
          for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
            if (!valid(tile)) continue;
            const size_t g = tofs(tile);  // tile layout
            float kk[tc::kCW];
            tc::tl_ldv(k7 + g, kk);
            if (dense && naccept < A.dense_slots) {
              float un[tc::kCW];
              tc::tl_ldv(unew + g, un);
              tc::tl_stv(A.dense + (size_t)naccept * 8 * SBt + g, un);
            }
            tc::tl_stv(kptr(0) + g, kk);
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

int tc_check_regs(const void* kernel) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return -1;
  return fa.numRegs == tc::kLaunchRegs ? 0 : -1;
}

int max_grid_fwd_tc(int* grid) {
  if (tc_check_regs((const void*)fwd_tc_kernel)) return -1;
  cudaError_t e = cudaFuncSetAttribute(fwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       tc::kSmemBytes);
  if (e != cudaSuccess) return -1;
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd_tc_kernel, tc::kThreads, tc::kSmemBytes);
  if (e != cudaSuccess || per_sm < 1) return -1;
  *grid = nsm;  // one CTA per SM (tensor memory is allocated whole)
  return 0;
}

int launch_fwd_tc(const FwdTcArgs& a, int grid, cudaStream_t st) {
  if (tc_check_regs((const void*)fwd_tc_kernel)) return -1;
  void* args[] = {(void*)&a};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)fwd_tc_kernel, dim3(grid), dim3(tc::kThreads),
                                              args, tc::kSmemBytes, st);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
