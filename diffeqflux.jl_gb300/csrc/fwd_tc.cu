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
    double dt;
    if (a.dt0 > 0.0) {
      dt = a.dt0;
    } else {
      double p0 = 0.0, p1 = 0.0;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        if (!valid(tile)) continue;
        float u[tc::kCW], f[tc::kCW];
        ldv(a.u0 + gofs(tile), th.nmine, vec, u);
        tc::tl_ldv(kptr(0) + tofs(tile), f);
        #pragma unroll
        for (int i = 0; i < tc::kCW; ++i) {
          if (i >= th.nmine) continue;
          const float sk = (float)a.abstol + fabsf(u[i]) * (float)a.reltol;
          const double x = (double)(u[i] / sk), y = (double)(f[i] / sk);
          p0 += x * x;
          p1 += y * y;
        }
      }
      p0 = tc::epi_sum(p0, sh);
      p1 = tc::epi_sum(p1, sh);
      double* pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) {
        pp[blockIdx.x] = p0;
        pp[G + blockIdx.x] = p1;
      }
      if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      const double d0 = sqrt(epi_partials_sum(pp, G, sh) / N);
      const double d1 = sqrt(epi_partials_sum(pp + G, G, sh) / N);
      par ^= 1;
      double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? fmax(a.dtmin, 1e-6) : 0.01 * (d0 / d1);
      dt0 = fmin(dt0, a.dtmax);
      const float hf = (float)(tdir * dt0);
      double p2 = 0.0;
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
            const double z = (double)((f1[i] - f0[i]) / sk);
            p2 += z * z;
          }
        }
      }
      nf += 1;
      if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      p2 = tc::epi_sum(p2, sh);
      pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = p2;
      if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto epi_done; }
      const double d2 = sqrt(epi_partials_sum(pp, G, sh) / N) / dt0;
      par ^= 1;
      const double mm = fmax(d1, d2);
      const double dt1 = (mm <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(mm)) / 5.0);
      dt = fmax(a.dtmin, fmin(100.0 * dt0, fmin(dt1, a.dtmax)));
    }

    // ---- step loop ---------------------------------------------------------------------
    {
      double t = a.t0, qold = kQoldInit;
      int ib = 0, nck = 0;
      while (tdir * (a.t1 - t) > 0.0) {
        if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
        ++iter;
        const double rem = fabs(a.t1 - t);
        const bool clipped = dt >= rem;
        const double habs = clipped ? rem : dt;
        const double h = tdir * habs;
        const float* ucur = a.ubuf[cur];
        float* unew = a.ubuf[cur ^ 1];
        const float* ccur = A.comp[cur];
        float* cnew = A.comp[cur ^ 1];
        double perr = 0.0;
        for (int i = 1; i < 7 && ok; ++i) {
          float ha[6];
#pragma unroll
          for (int j = 0; j < 6; ++j) ha[j] = (float)(h * c_tab.a[i][j]);
          float hbt[7];
#pragma unroll
          for (int j = 0; j < 7; ++j) hbt[j] = (float)(h * c_tab.btilde[j]);
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
                  const double rr = (double)(ut[q] / sc);
                  perr += isfinite(Y[q]) ? rr * rr : (double)INFINITY;
                }
              } else {
                tc::tl_stv(kptr(i) + g, k);
              }
            }
          }
        }
        if (!ok) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        nf += 6;
        perr = tc::epi_sum(perr, sh);
        double* pp = a.partials + (size_t)par * 2 * G;
        if (threadIdx.x == 0) pp[blockIdx.x] = perr;
        if (!epi_grid_barrier(a, gen, sh, &s_ok)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
        const double eest = sqrt(epi_partials_sum(pp, G, sh) / N);
        par ^= 1;
        if (!isfinite(eest)) { ret = GBNDE_RET_UNSTABLE; break; }
        double q11;
        double q = pi_q(eest, qold, &q11);
        if (blockIdx.x == 0 && threadIdx.x == 0 && iter - 1 < a.maxsteps) {
          double* tr = a.trace + 4 * (iter - 1);
          tr[0] = t;
          tr[1] = h;
          tr[2] = eest;
          tr[3] = eest <= 1.0 ? 1.0 : 0.0;
        }
        if (eest <= 1.0) {
          const double tnew = clipped ? a.t1 : t + h;
          while (isave < a.nsave && tdir * (a.saveat[isave] - tnew) <= 0.0) {
            const double sv = a.saveat[isave];
            float* dst = a.usave + (size_t)isave * SB;
            float hb[7];
            if (sv != tnew) {
              float bw[7];
              interp_weights((sv - t) / h, bw);
              for (int j = 0; j < 7; ++j) hb[j] = (float)(h * (double)bw[j]);
            }
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
              if (!valid(tile)) continue;
              const size_t g = gofs(tile), tg = tofs(tile);
              float o[tc::kCW];
              if (sv == tnew) {
                tc::tl_ldv(unew + tg, o);
              } else {
                float u[tc::kCW];
                tc::tl_ldv(ucur + tg, u);
                tc::tl_ldv(ccur + tg, o);
#pragma unroll
                for (int j = 0; j < 7; ++j) {
                  float kj[tc::kCW];
                  tc::tl_ldv(kptr(j) + tg, kj);
#pragma unroll
                  for (int q = 0; q < tc::kCW; ++q) o[q] = fmaf(hb[j], kj[q], o[q]);
                }
#pragma unroll
                for (int q = 0; q < tc::kCW; ++q) o[q] = u[q] + o[q];
              }
              stv(dst + g, th.nmine, vec, o);
            }
            ++isave;
          }
          bool need = false;
          while (ib < a.nbnd && tdir * (a.bnd[ib] - tnew) < 0.0) { need = true; ++ib; }
          if (need && nck < a.max_ckpt) {
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
          if (blockIdx.x == 0 && threadIdx.x == 0 && naccept < a.maxsteps) {
            a.steplog[2 * naccept] = t;
            a.steplog[2 * naccept + 1] = h;
          }
          // FSAL: k7 becomes k1 of the next step (next dense slot, or in place)
          const float* k7 = kptr(6);
          ++naccept;
          for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
            if (!valid(tile)) continue;
            const size_t g = tofs(tile);  // tile layout
            float kk[tc::kCW];
            tc::tl_ldv(k7 + g, kk);
            tc::tl_stv(kptr(0) + g, kk);
            if (dense && naccept < A.dense_slots) {
              float un[tc::kCW];
              tc::tl_ldv(unew + g, un);
              tc::tl_stv(A.dense + (size_t)naccept * 8 * SBt + g, un);
            }
          }
          cur ^= 1;
          t = tnew;
          if (q >= 1.0 && q <= 1.0) q = 1.0;
          qold = fmax(eest, kQoldInit);
          dt = fmax(fmin(habs / q, a.dtmax), a.dtmin);
        } else {
          ++nreject;
          dt = habs / fmin(1.0 / kQmin, q11 / kGamma);
          if (a.dtmin > 0.0 && dt <= a.dtmin) { ret = GBNDE_RET_DTLESSTHANMIN; break; }
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
