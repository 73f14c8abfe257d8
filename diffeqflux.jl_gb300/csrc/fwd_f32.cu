// fwd_f32.cu -- persistent Tsit5 forward solve, plain FP32 form.
//
// Replaces, for the batched NeuralODE state, the integrator loop that
// `solve(prob, Tsit5(); saveat, abstol, reltol)` runs (src/neural_de.jl:55-58):
// 7-stage FSAL Tsit5 steps, the embedded error estimate with the scaled RMS
// norm over all S*B entries, PI step-size control with one accept/reject
// decision per step for the whole batch, the free interpolant at `saveat`
// points and clipping of the last step to t1.
//
// One cooperative launch does the whole solve. CTAs own tiles of TM
// trajectories; stages of a step need no communication between CTAs, so the
// only grid-wide synchronisation is one barrier per step, after which every
// CTA sums the per-CTA error partials in the same fixed order and takes the
// same controller decision. t, dt and the error reduction are FP64; all
// state and stage arithmetic is FP32.
#include "kernels.h"

namespace gbnde {

namespace {

// Stage buffer j of the current attempt. Dense mode: slot of accepted step
// `n` (k1..k7 at positions 1..7); otherwise a ring of 7 with the FSAL swap.
__device__ __forceinline__ float* kbuf_at(const FwdArgs& a, int j, bool swp, long long n) {
  if (a.dense) {
    const size_t SB = (size_t)a.S * a.B;
    return a.dense + ((size_t)min(n, a.dense_slots - 1) * 8 + 1 + j) * SB;
  }
  if (j == 0) return swp ? a.kbuf[6] : a.kbuf[0];
  if (j == 6) return swp ? a.kbuf[0] : a.kbuf[6];
  return a.kbuf[j];
}
#define kb(a, j, swp) kbuf_at(a, j, swp, naccept)

// Load the MLP input of a tile (feature-major) from a per-element producer.
template <class Fn>
__device__ __forceinline__ void load_tile_input(const FwdArgs& a, int tile, float* bufA,
                                                double tstage, Fn&& val) {
  const int S = a.S, TM = a.TM, LD = a.LD;
  const size_t base = (size_t)tile * TM * S;
  const int nvalid = min(TM, a.B - tile * TM);
  for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
    const int m = e / S, s = e - m * S;
    float v = 0.f;
    if (m < nvalid) v = val(base + e);
    if (a.mlp.cube) v = v * v * v;
    bufA[s * LD + m] = v;
  }
  if (a.mlp.timein) {
    for (int m = threadIdx.x; m < TM; m += blockDim.x) bufA[S * LD + m] = (float)tstage;
  }
  __syncthreads();
}

// Store the tile output (rows [0,S) of `out`) through a per-element consumer.
template <class Fn>
__device__ __forceinline__ void store_tile_output(const FwdArgs& a, int tile, const float* out,
                                                  Fn&& sink) {
  const int S = a.S, TM = a.TM, LD = a.LD;
  const size_t base = (size_t)tile * TM * S;
  const int nvalid = min(TM, a.B - tile * TM);
  for (int e = threadIdx.x; e < nvalid * S; e += blockDim.x) {
    const int m = e / S, s = e - m * S;
    sink(base + e, out[s * LD + m]);
  }
  __syncthreads();
}

__device__ __forceinline__ size_t tile_elems(const FwdArgs& a, int tile) {
  return (size_t)min(a.TM, a.B - tile * a.TM) * a.S;
}

// FFJORD right-hand side of a tile: [f(z, t); -trace(df/dz)], the trace as
// e^T (J e) along the sample's noise e (Hutchinson) or summed over the unit
// directions (exact). With a.ffreg two more rows: |f|^2 and |e^T J|, the
// latter through a reverse pass of the chain from the output cotangent e
// (src/ffjord.jl:131-132). smem: act[0..L], zd[0..L] (sum(dims) rows each),
// tmp (maxdim rows), trace sums (TM); with ffreg also the two row values (TM
// each) and a second work buffer (maxdim rows).
template <class Fn, class Sink>
__device__ __forceinline__ void ffjord_rhs_tile(const FwdArgs& a, int tile, float* smem, double tstage,
                                                Fn&& val, Sink&& sink) {
  const MlpDev& m = a.mlp;
  const int S = a.S, d = a.ffd, TM = a.TM, LD = a.LD;
  float* act[GBNDE_MAX_LAYERS + 1];
  float* zd[GBNDE_MAX_LAYERS + 1];
  float* p = smem;
  for (int l = 0; l <= m.nlayers; ++l) { act[l] = p; p += (size_t)m.dims[l] * LD; }
  for (int l = 0; l <= m.nlayers; ++l) { zd[l] = p; p += (size_t)m.dims[l] * LD; }
  float* tmp = p;
  p += (size_t)m.maxdim * LD;
  float* tr = p;
  p += LD;
  float* rf = p;   // |f|^2
  p += LD;
  float* rj = p;   // |e^T J|
  p += LD;
  float* wk = p;   // second work buffer of the reverse pass
  const size_t base = (size_t)tile * TM * S;
  const int nvalid = min(TM, a.B - tile * TM);
  for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
    const int mm = e / S, s = e - mm * S;
    const float v = (mm < nvalid) ? val(base + e) : 0.f;
    if (s < d) act[0][s * LD + mm] = v;
  }
  if (m.timein)
    for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) act[0][d * LD + mm] = (float)tstage;
  for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) tr[mm] = 0.f;
  __syncthreads();
  mlp_fwd_tile(m, act[0], nullptr, LD, TM, act + 1);
  const int ndir = a.exact ? d : 1;
  const int L = m.nlayers;
  for (int k = 0; k < ndir; ++k) {
    for (int e = threadIdx.x; e < m.dims[0] * TM; e += blockDim.x) {
      const int s = e / TM, mm = e - s * TM;
      float v = 0.f;
      if (s < d && mm < nvalid) v = a.exact ? (s == k ? 1.f : 0.f) : a.noise[((size_t)tile * TM + mm) * d + s];
      zd[0][s * LD + mm] = v;
    }
    __syncthreads();
    mlp_tangent_tile(m, act, zd, tmp, LD, TM);
    with_act(m.act[L - 1], [&](auto A) {
      for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) {
        float s_ = 0.f;
        for (int s = 0; s < d; ++s)
          s_ = fmaf(zd[0][s * LD + mm], A.d(act[L][s * LD + mm]) * zd[L][s * LD + mm], s_);
        tr[mm] += s_;
      }
    });
    __syncthreads();
  }
  if (a.ffreg) {
    // v = J^T e: the chain's reverse pass from the output cotangent e
    for (int e = threadIdx.x; e < d * TM; e += blockDim.x) {
      const int s = e / TM, mm = e - s * TM;
      tmp[s * LD + mm] = mm < nvalid ? a.noise[((size_t)tile * TM + mm) * d + s] : 0.f;
    }
    __syncthreads();
    const float* v = mlp_vjp_tile(m, act, tmp, wk, LD, TM, nullptr, 0.f);
    for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) {
      float sf = 0.f, sj = 0.f;
      for (int s = 0; s < d; ++s) {
        const float f = act[L][s * LD + mm], g = v[s * LD + mm];
        sf = fmaf(f, f, sf);
        sj = fmaf(g, g, sj);
      }
      rf[mm] = sf;
      rj[mm] = sqrtf(sj);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nvalid * S; e += blockDim.x) {
    const int mm = e / S, s = e - mm * S;
    sink(base + e, s < d ? act[L][s * LD + mm] : s == d ? -tr[mm] : s == d + 1 ? rf[mm] : rj[mm]);
  }
  __syncthreads();
}

// One right-hand side of a tile: the NeuralODE chain or the FFJORD system.
template <class Fn, class Sink>
__device__ __forceinline__ void rhs_tile(const FwdArgs& a, int tile, float* smem, double tstage, Fn&& val,
                                         Sink&& sink) {
  if (a.ffj) {
    ffjord_rhs_tile(a, tile, smem, tstage, val, sink);
    return;
  }
  float* bufA = smem;
  float* bufB = smem + (size_t)a.mlp.maxdim * a.LD;
  load_tile_input(a, tile, bufA, tstage, val);
  const float* out = mlp_fwd_tile(a.mlp, bufA, bufB, a.LD, a.TM, nullptr);
  store_tile_output(a, tile, out, sink);
}

}  // namespace

__global__ void __launch_bounds__(256, 1) fwd_f32_kernel(FwdArgs a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ double red[40];
  __shared__ StepCtl s_ctl;  // the step's scalars from thread 0
  const int G = gridDim.x;
  const double N = (double)a.S * (double)a.B;
  const double tdir = a.t1 >= a.t0 ? 1.0 : -1.0;
  unsigned int gen = 0;
  int par = 0;
  bool swp = false;
  int cur = 0;
  int ret = GBNDE_RET_SUCCESS;
  long long nf = 0, naccept = 0, nreject = 0;

  // ---- k1 = f(u0, t0); ubuf[0] = u0 --------------------------------------
  for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
    float* k1 = kb(a, 0, swp);
    rhs_tile(a, tile, smem, a.t0,
             [&](size_t g) {
               const float v = a.u0[g];
               a.ubuf[0][g] = v;
               if (a.dense) a.dense[g] = v;
               return v;
             },
             [&](size_t g, float v) { k1[g] = v; });
  }
  nf = 1;

  int isave = 0;
  while (isave < a.nsave && a.saveat[isave] == a.t0) {
    float* dst = a.usave + (size_t)isave * a.S * a.B;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
      const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
      for (size_t e = threadIdx.x; e < n; e += blockDim.x) dst[base + e] = a.u0[base + e];
    }
    ++isave;
  }

  // ---- initial step (Hairer's algorithm as the integrator implements it) --
  double dt;
  const int f32t = a.f32time;
  if (a.dt0 > 0.0) {
    dt = rt32(a.dt0, f32t);
  } else {
    double p0 = 0.0, p1 = 0.0;
    const float* k1 = kb(a, 0, swp);
    for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
      const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
      for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
        const float u = a.u0[base + e], f = k1[base + e];
        const float sk = (float)a.abstol + fabsf(u) * (float)a.reltol;
        const double x = (double)(u / sk), y = (double)(f / sk);
        p0 += x * x;
        p1 += y * y;
      }
    }
    p0 = block_sum_double(p0, red);
    p1 = block_sum_double(p1, red);
    double* pp = a.partials + (size_t)par * 2 * G;
    if (threadIdx.x == 0) {
      pp[blockIdx.x] = p0;
      pp[G + blockIdx.x] = p1;
    }
    if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto done; }
    {
      const double d0 = sqrt(grid_partials_sum(pp, G, red) / N);
      const double d1 = sqrt(grid_partials_sum(pp + G, G, red) / N);
      par ^= 1;
      const double smalldt = fmax(a.dtmin, 1e-6);
      double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? smalldt : 0.01 * (d0 / d1);
      dt0 = rt32(fmin(dt0, a.dtmax), f32t);
      const float hf = (float)(tdir * dt0);
      // f1 = f(u0 + dt0*f0) into the stage-2 buffer (scratch here)
      float* f1b = kb(a, 1, swp);
      double p2 = 0.0;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        rhs_tile(a, tile, smem, a.t0 + tdir * dt0, [&](size_t g) { return a.u0[g] + hf * k1[g]; },
                 [&](size_t g, float v) {
          f1b[g] = v;
          const float sk = (float)a.abstol + fabsf(a.u0[g]) * (float)a.reltol;
          const double z = (double)((v - k1[g]) / sk);
          p2 += z * z;
        });
      }
      nf += 1;
      p2 = block_sum_double(p2, red);
      pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = p2;
      if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; goto done; }
      const double d2 = sqrt(grid_partials_sum(pp, G, red) / N) / dt0;
      par ^= 1;
      const double m = fmax(d1, d2);
      const double dt1 = (m <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(m)) / 5.0);
      dt = rt32(fmax(a.dtmin, fmin(100.0 * dt0, fmin(dt1, a.dtmax))), f32t);
    }
  }

  // ---- step loop ------------------------------------------------------------
  // The scalar FP64 work of a step (step size, stage coefficients and times,
  // the norm's square root, the PI update, save weights) runs on thread 0 and
  // reaches the others through shared memory; t, dt and qold are thread 0's.
  {
    double t = a.t0, qold = kQoldInit;
    long long iter = 0;
    int ib = 0, nck = 0;
    for (;;) {
      if (threadIdx.x == 0) {
        s_ctl.go = tdir * (a.t1 - t) > 0.0;
        const double rem = rt32(fabs(a.t1 - t), f32t);
        s_ctl.clipped = dt >= rem;
        s_ctl.habs = s_ctl.clipped ? rem : dt;
        const double h = tdir * s_ctl.habs;
        s_ctl.t = t;
        s_ctl.h = h;
        for (int i = 1; i < 7; ++i) {
          for (int j = 0; j < 6; ++j) s_ctl.ha[i - 1][j] = (float)(h * c_tab.a[i][j]);
          s_ctl.tst[i] = t + c_tab.c[i] * h;
        }
        for (int j = 0; j < 7; ++j) s_ctl.hbt[j] = (float)(h * c_tab.btilde[j]);
      }
      __syncthreads();
      if (!s_ctl.go) break;
      if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
      ++iter;
      float* ucur = a.ubuf[cur];
      float* unew = a.ubuf[cur ^ 1];
      double perr = 0.0;
      for (int i = 1; i < 7; ++i) {
        float ha[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) ha[j] = s_ctl.ha[i - 1][j];
        const float* kj[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) kj[j] = kb(a, j, swp);
        float* ki = kb(a, i, swp);
        float hbt[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) hbt[j] = s_ctl.hbt[j];
        const double ts = s_ctl.tst[i];
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
          auto stage_in = [&](size_t g) {
            float s = 0.f;
            for (int j = 0; j < i; ++j) s = fmaf(ha[j], kj[j][g], s);
            const float y = ucur[g] + s;
            if (i == 6) unew[g] = y;
            return y;
          };
          if (i < 6) {
            rhs_tile(a, tile, smem, ts, stage_in, [&](size_t g, float v) { ki[g] = v; });
          } else {
            rhs_tile(a, tile, smem, ts, stage_in, [&](size_t g, float v) {
              ki[g] = v;
              float ut = hbt[6] * v;
#pragma unroll
              for (int j = 0; j < 6; ++j) ut = fmaf(hbt[j], kj[j][g], ut);
              const float uo = ucur[g], un = unew[g];
              const float sc = (float)a.abstol + fmaxf(fabsf(uo), fabsf(un)) * (float)a.reltol;
              const double r = (double)(ut / sc);
              perr += isfinite(un) ? r * r : (double)INFINITY;
            });
          }
        }
      }
      nf += 6;
      perr = block_sum_double(perr, red);
      double* pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = perr;
      if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
      {
        const double qe = grid_partials_sum(pp, G, red);
        if (threadIdx.x == 0) {
          const double eest = rt32(sqrt(qe / N), f32t);
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
              const double tnew = s_ctl.clipped ? a.t1 : rt32(t + h, f32t);
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
              qold = rt32(fmax(eest, kQoldInit), f32t);
              dt = rt32(fmax(fmin(habs / q, a.dtmax), a.dtmin), f32t);
            } else {
              dt = rt32(habs / fmin(1.0 / kQmin, q11 / kGamma), f32t);
              if (a.dtmin > 0.0 && dt <= a.dtmin) s_ctl.ret = GBNDE_RET_DTLESSTHANMIN;
            }
          }
        }
        __syncthreads();
      }
      par ^= 1;
      if (s_ctl.ret != GBNDE_RET_SUCCESS) {
        ret = s_ctl.ret;
        if (ret == GBNDE_RET_DTLESSTHANMIN) ++nreject;
        break;
      }
      if (s_ctl.accept) {
        // saveat points in (t, tnew]
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
          __syncthreads();
          float* dst = a.usave + (size_t)isave * a.S * a.B;
          if (s_ctl.exact) {
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
              const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
              for (size_t e = threadIdx.x; e < n; e += blockDim.x) dst[base + e] = unew[base + e];
            }
          } else {
            float hb[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) hb[j] = s_ctl.hb[j];
            const float* kk[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) kk[j] = kb(a, j, swp);
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
              const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
              for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
                const size_t g = base + e;
                float acc = 0.f;
#pragma unroll
                for (int j = 0; j < 7; ++j) acc = fmaf(hb[j], kk[j][g], acc);
                dst[g] = ucur[g] + acc;
              }
            }
          }
          __syncthreads();  // s_ctl.hb is rewritten for the next save
        }
        // checkpoint the state at the start of this step if it holds a boundary
        if (s_ctl.need_ckpt && nck < a.max_ckpt) {
          float* dst = a.ckpt + (size_t)nck * a.S * a.B;
          for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
            const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
            for (size_t e = threadIdx.x; e < n; e += blockDim.x) dst[base + e] = ucur[base + e];
          }
          if (blockIdx.x == 0 && threadIdx.x == 0) a.ckpt_step[nck] = (int)naccept;
          ++nck;
        }
        ++naccept;
        if (a.dense) {
          const float* k7 = kbuf_at(a, 6, swp, naccept - 1);
          float* k1n = kbuf_at(a, 0, swp, naccept);
          const bool slot_ok = naccept < a.dense_slots;
          float* un = a.dense + (size_t)naccept * 8 * a.S * a.B;
          for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
            const size_t base = (size_t)tile * a.TM * a.S, n = tile_elems(a, tile);
            for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
              k1n[base + e] = k7[base + e];
              if (slot_ok) un[base + e] = unew[base + e];
            }
          }
        } else {
          swp = !swp;
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

done:
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.counters[CT_NF] = nf;
    a.counters[CT_NACCEPT] = naccept;
    a.counters[CT_NREJECT] = nreject;
    a.status[ST_RETCODE] = (a.status[ST_BARRIER] != 0) ? GBNDE_RET_BARRIER_TIMEOUT : ret;
    // which buffer holds the final state: reported through counters slot 5
    a.counters[5] = cur;
  }
}

int max_grid_fwd_f32(size_t smem, int* grid) {
  cudaError_t e = cudaFuncSetAttribute(fwd_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return -1;
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd_f32_kernel, 256, smem);
  if (e != cudaSuccess || per_sm < 1) return -1;
  *grid = per_sm * nsm;
  return 0;
}

int launch_fwd_f32(const FwdArgs& a, int grid, size_t smem, cudaStream_t st) {
  void* args[] = {(void*)&a};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)fwd_f32_kernel, dim3(grid), dim3(256),
                                              args, smem, st);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
