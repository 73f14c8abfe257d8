// ms_f32.cu -- packed multiple shooting: many independent segment solves with
// their own step-size controllers in one launch (FP32 form).
//
// Replaces the sequential per-group solves of `multiple_shoot`
// (src/multiple_shooting.jl:52-62): every group range rg is a solve of
// `remake(prob; tspan = (tsteps[first(rg)], tsteps[last(rg)]),
// u0 = data[:, first(rg)])` with `saveat = tsteps[rg]`. Each segment keeps its
// own Tsit5 step size, PI controller (RMS error norm over its S components)
// and save points, as separate solves would. Segments are the rows of tiles
// that step in lockstep, one attempt per iteration; finished rows are masked.
// No grid-wide synchronisation is needed.
//
// The gradient is the discrete adjoint of the accepted steps: reverse mode
// through the Tsit5 stages and the save-point interpolation with the step
// sizes held fixed -- the discretize-then-differentiate family of sensealgs
// the reference re-exports (ZygoteAdjoint / ReverseDiffAdjoint,
// src/DiffEqFlux.jl:53-54). It is the exact gradient of the computed forward.
#include "kernels.h"

namespace gbnde {

struct MsSeg {
  double t0, t1;
  int save_off, nsave;
};

struct MsArgs {
  MlpDev mlp;
  int S, nseg, TM, LD, ntiles;
  double abstol, reltol;
  long long maxiters;  // attempts per tile
  int MS;              // dense step capacity per segment
  const MsSeg* segs;
  const double* saveat;
  const float* u0;     // S x nseg
  float* usave;        // S x nsave_total
  float* dense;        // [nseg][MS+1][8][S]: u_n, k1..k7
  double* steplog;     // [nseg][MS][2]
  int* nacc;           // [nseg]
  int* retcode;        // [nseg]
  long long* counters; // [0] RHS evaluations (segment-weighted), [1] accepted, [2] rejected
  // backward
  const float* dLdu;   // S x nsave_total
  float* dLdu0;        // S x nseg
  float* bar;          // [nseg][9][S]: ubar, Ybar7, kbar1..kbar7
  float* mu_acc;       // [grid][P]
  int P;
};

namespace {

struct Row {
  double t, dt, qold, h, told, hacc;
  int active, clipped, nacc, isave, ret, accnow, nsv;
};

__device__ __forceinline__ size_t slot_off(const MsArgs& a, int sg, int n, int j) {
  return (((size_t)sg * (a.MS + 1) + n) * 8 + j) * a.S;
}
__device__ __forceinline__ size_t bar_off(const MsArgs& a, int sg, int j) {
  return ((size_t)sg * 9 + j) * a.S;
}

// Deterministic per-row sums: warp w takes rows w, w+8, ...
template <class Fn>
__device__ __forceinline__ void row_sums(int TM, int S, double* out, Fn&& val) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int m = w; m < TM; m += nw) {
    double s = 0.0;
    for (int c = l; c < S; c += 32) s += val(m, c);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) out[m] = s;
  }
  __syncthreads();
}

}  // namespace

// ======================================================================================
// forward
// ======================================================================================
__global__ void __launch_bounds__(256, 1) ms_fwd_f32_kernel(MsArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int S = a.S, TM = a.TM, LD = a.LD;
  float* bufA = smem;
  float* bufB = smem + (size_t)a.mlp.maxdim * LD;
  __shared__ Row rw[64];
  __shared__ double rsum[64], rsum2[64];
  __shared__ int s_any, s_maxsv;
  long long nf = 0, nacc_tot = 0, nrej_tot = 0;

  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
    const int row0 = tile * TM;
    const int nrows = min(TM, a.nseg - row0);
    if (threadIdx.x < TM) {
      Row& r = rw[threadIdx.x];
      r.active = threadIdx.x < nrows;
      r.t = r.active ? a.segs[row0 + threadIdx.x].t0 : 0.0;
      r.qold = kQoldInit;
      r.nacc = 0;
      r.isave = 0;
      r.ret = GBNDE_RET_SUCCESS;
      r.h = 0.0;
      r.accnow = 0;
    }
    __syncthreads();
    // one RHS evaluation of the tile: input per element, output per element
    auto eval = [&](auto&& val, auto&& sink) {
      for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
        const int m = e / S, s = e - m * S;
        float v = (m < nrows) ? val(m, s) : 0.f;
        if (a.mlp.cube) v = v * v * v;
        bufA[s * LD + m] = v;
      }
      if (a.mlp.timein)
        for (int m = threadIdx.x; m < TM; m += blockDim.x) bufA[S * LD + m] = (float)rw[m].t;
      __syncthreads();
      const float* out = mlp_fwd_tile(a.mlp, bufA, bufB, LD, TM, nullptr);
      for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
        const int m = e / S, s = e - m * S;
        sink(m, s, out[s * LD + m]);
      }
      __syncthreads();
    };
    // k1 = f(u0); slot 0 = (u0, k1)
    eval([&](int m, int s) { return a.u0[(size_t)(row0 + m) * S + s]; },
         [&](int m, int s, float v) {
           const int sg = row0 + m;
           a.dense[slot_off(a, sg, 0, 0) + s] = a.u0[(size_t)sg * S + s];
           a.dense[slot_off(a, sg, 0, 1) + s] = v;
         });
    nf += nrows;
    // save points at t0
    for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
      const int m = e / S, s = e - m * S, sg = row0 + m;
      const MsSeg g = a.segs[sg];
      for (int q = 0; q < g.nsave && a.saveat[g.save_off + q] == g.t0; ++q)
        a.usave[(size_t)(g.save_off + q) * S + s] = a.u0[(size_t)sg * S + s];
    }
    if (threadIdx.x < nrows) {
      Row& r = rw[threadIdx.x];
      const MsSeg g = a.segs[row0 + threadIdx.x];
      while (r.isave < g.nsave && a.saveat[g.save_off + r.isave] == g.t0) ++r.isave;
    }
    __syncthreads();
    // initial step of every segment
    row_sums(TM, S, rsum, [&](int m, int c) -> double {
      if (m >= nrows) return 0.0;
      const float u = a.dense[slot_off(a, row0 + m, 0, 0) + c];
      const double x = (double)(u / ((float)a.abstol + fabsf(u) * (float)a.reltol));
      return x * x;
    });
    row_sums(TM, S, rsum2, [&](int m, int c) -> double {
      if (m >= nrows) return 0.0;
      const float u = a.dense[slot_off(a, row0 + m, 0, 0) + c];
      const float f = a.dense[slot_off(a, row0 + m, 0, 1) + c];
      const double y = (double)(f / ((float)a.abstol + fabsf(u) * (float)a.reltol));
      return y * y;
    });
    if (threadIdx.x < nrows) {
      Row& r = rw[threadIdx.x];
      const MsSeg g = a.segs[row0 + threadIdx.x];
      const double d0 = sqrt(rsum[threadIdx.x] / S), d1 = sqrt(rsum2[threadIdx.x] / S);
      double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
      r.h = fmin(dt0, g.t1 - g.t0);
      r.dt = d1;
    }
    __syncthreads();
    eval([&](int m, int s) {
           const int sg = row0 + m;
           return a.dense[slot_off(a, sg, 0, 0) + s] + (float)rw[m].h * a.dense[slot_off(a, sg, 0, 1) + s];
         },
         [&](int m, int s, float v) { a.dense[slot_off(a, row0 + m, 0, 2) + s] = v; });
    nf += nrows;
    row_sums(TM, S, rsum, [&](int m, int c) -> double {
      if (m >= nrows) return 0.0;
      const int sg = row0 + m;
      const float u = a.dense[slot_off(a, sg, 0, 0) + c];
      const float sk = (float)a.abstol + fabsf(u) * (float)a.reltol;
      const double z = (double)((a.dense[slot_off(a, sg, 0, 2) + c] - a.dense[slot_off(a, sg, 0, 1) + c]) / sk);
      return z * z;
    });
    if (threadIdx.x < nrows) {
      Row& r = rw[threadIdx.x];
      const MsSeg g = a.segs[row0 + threadIdx.x];
      const double dt0 = r.h, d1 = r.dt;
      const double d2 = sqrt(rsum[threadIdx.x] / S) / dt0;
      const double mm = fmax(d1, d2);
      const double dt1 = (mm <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(mm)) / 5.0);
      r.dt = fmin(100.0 * dt0, fmin(dt1, g.t1 - g.t0));
      r.active = g.t1 > g.t0;
    }
    __syncthreads();

    // ---- lockstep attempts ------------------------------------------------------------
    for (long long it = 0;; ++it) {
      if (threadIdx.x < TM) {
        Row& r = rw[threadIdx.x];
        if (r.active && it >= a.maxiters) {
          r.ret = GBNDE_RET_MAXITERS;
          r.active = 0;
        }
        if (r.active) {
          const double rem = a.segs[row0 + threadIdx.x].t1 - r.t;
          r.clipped = r.dt >= rem;
          r.h = r.clipped ? rem : r.dt;
        } else {
          r.h = 0.0;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int any = 0;
        for (int m = 0; m < nrows; ++m) any |= rw[m].active;
        s_any = any;
      }
      __syncthreads();
      if (!s_any) break;
      for (int i = 1; i < 7; ++i) {
        eval(
            [&](int m, int s) {
              const Row& r = rw[m];
              if (!r.active) return 0.f;
              const int sg = row0 + m, n = r.nacc;
              float acc = 0.f;
              for (int j = 0; j < i; ++j)
                acc = fmaf((float)(r.h * c_tab.a[i][j]), a.dense[slot_off(a, sg, n, 1 + j) + s], acc);
              const float y = a.dense[slot_off(a, sg, n, 0) + s] + acc;
              if (i == 6) a.dense[slot_off(a, sg, n + 1, 0) + s] = y;
              return y;
            },
            [&](int m, int s, float v) {
              const Row& r = rw[m];
              if (r.active) a.dense[slot_off(a, row0 + m, r.nacc, 1 + i) + s] = v;
            });
        for (int m = 0; m < nrows; ++m) nf += rw[m].active;
      }
      row_sums(TM, S, rsum, [&](int m, int c) -> double {
        const Row& r = rw[m];
        if (m >= nrows || !r.active) return 0.0;
        const int sg = row0 + m, n = r.nacc;
        float ut = 0.f;
        for (int j = 0; j < 7; ++j)
          ut = fmaf((float)(r.h * c_tab.btilde[j]), a.dense[slot_off(a, sg, n, 1 + j) + c], ut);
        const float uo = a.dense[slot_off(a, sg, n, 0) + c], un = a.dense[slot_off(a, sg, n + 1, 0) + c];
        const float sc = (float)a.abstol + fmaxf(fabsf(uo), fabsf(un)) * (float)a.reltol;
        const double rr = (double)(ut / sc);
        return isfinite(un) ? rr * rr : (double)INFINITY;
      });
      // controller of every segment
      if (threadIdx.x < TM) {
        Row& r = rw[threadIdx.x];
        r.accnow = 0;
        r.nsv = 0;
        if (r.active) {
          const int sg = row0 + threadIdx.x;
          const MsSeg g = a.segs[sg];
          const double eest = sqrt(rsum[threadIdx.x] / S);
          if (!isfinite(eest)) {
            r.ret = GBNDE_RET_UNSTABLE;
            r.active = 0;
          } else {
            double q11;
            double q = pi_q(eest, r.qold, &q11);
            if (eest <= 1.0) {
              a.steplog[((size_t)sg * a.MS + r.nacc) * 2] = r.t;
              a.steplog[((size_t)sg * a.MS + r.nacc) * 2 + 1] = r.h;
              r.told = r.t;
              r.hacc = r.h;
              r.t = r.clipped ? g.t1 : r.t + r.h;
              r.nacc += 1;
              r.accnow = 1;
              if (q >= 1.0 && q <= 1.0) q = 1.0;
              r.qold = fmax(eest, kQoldInit);
              r.dt = fmin(r.h / q, g.t1 - g.t0);
              while (r.isave + r.nsv < g.nsave && a.saveat[g.save_off + r.isave + r.nsv] <= r.t) ++r.nsv;
              if (r.clipped) r.active = 0;
              else if (r.nacc >= a.MS) {
                r.ret = GBNDE_RET_MAXITERS;
                r.active = 0;
              }
            } else {
              r.dt = r.h / fmin(1.0 / kQmin, q11 / kGamma);
            }
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int mx = 0;
        for (int m = 0; m < nrows; ++m) {
          mx = max(mx, rw[m].nsv);
          nacc_tot += rw[m].accnow;
          nrej_tot += (rw[m].h > 0.0 && !rw[m].accnow && rw[m].ret == GBNDE_RET_SUCCESS);
        }
        s_maxsv = mx;
      }
      __syncthreads();
      // save points inside the accepted steps; FSAL copy k7 -> next slot's k1
      for (int qv = 0; qv < s_maxsv; ++qv) {
        for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
          const int m = e / S, s = e - m * S;
          const Row& r = rw[m];
          if (!r.accnow || qv >= r.nsv) continue;
          const int sg = row0 + m, n = r.nacc - 1;
          const MsSeg g = a.segs[sg];
          const int si = r.isave + qv;
          const double sv = a.saveat[g.save_off + si];
          float o;
          if (sv == r.t) {
            o = a.dense[slot_off(a, sg, n + 1, 0) + s];
          } else {
            float bw[7];
            interp_weights((sv - r.told) / r.hacc, bw);
            float acc = 0.f;
            for (int j = 0; j < 7; ++j)
              acc = fmaf((float)(r.hacc * (double)bw[j]), a.dense[slot_off(a, sg, n, 1 + j) + s], acc);
            o = a.dense[slot_off(a, sg, n, 0) + s] + acc;
          }
          a.usave[(size_t)(g.save_off + si) * S + s] = o;
        }
      }
      for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
        const int m = e / S, s = e - m * S;
        const Row& r = rw[m];
        if (r.accnow && r.nacc <= a.MS)
          a.dense[slot_off(a, row0 + m, r.nacc, 1) + s] = a.dense[slot_off(a, row0 + m, r.nacc - 1, 7) + s];
      }
      __syncthreads();
      if (threadIdx.x < TM) {
        Row& r = rw[threadIdx.x];
        r.isave += r.nsv;
      }
      __syncthreads();
    }
    if (threadIdx.x < nrows) {
      const Row& r = rw[threadIdx.x];
      a.nacc[row0 + threadIdx.x] = r.nacc;
      a.retcode[row0 + threadIdx.x] = r.ret;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd((unsigned long long*)&a.counters[0], (unsigned long long)nf);
    atomicAdd((unsigned long long*)&a.counters[1], (unsigned long long)nacc_tot);
    atomicAdd((unsigned long long*)&a.counters[2], (unsigned long long)nrej_tot);
  }
}

// ======================================================================================
// discrete adjoint
// ======================================================================================
__global__ void __launch_bounds__(256, 1) ms_bwd_f32_kernel(MsArgs a) {
  extern __shared__ __align__(16) float smem[];
  const int S = a.S, TM = a.TM, LD = a.LD;
  const MlpDev& m = a.mlp;
  float* act[GBNDE_MAX_LAYERS + 1];
  float* p = smem;
  for (int l = 0; l <= m.nlayers; ++l) {
    act[l] = p;
    p += (size_t)m.dims[l] * LD;
  }
  float* gA = p;
  p += (size_t)m.maxdim * LD;
  float* gB = p;
  p += (size_t)m.maxdim * LD;
  float* uraw = p;
  __shared__ int s_n[64];
  __shared__ double s_h[64], s_tn[64], s_tnext[64];
  __shared__ int s_isv[64], s_maxn;
  float* mu = a.mu_acc + (size_t)blockIdx.x * a.P;
  for (int i = threadIdx.x; i < a.P; i += blockDim.x) mu[i] = 0.f;
  __syncthreads();

  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
    const int row0 = tile * TM;
    const int nrows = min(TM, a.nseg - row0);
    // zero the cotangent state, save pointers at the last save
    for (int e = threadIdx.x; e < nrows * 9 * S; e += blockDim.x) a.bar[(size_t)row0 * 9 * S + e] = 0.f;
    if (threadIdx.x < TM) {
      const bool v = threadIdx.x < nrows;
      s_isv[threadIdx.x] = v ? a.segs[row0 + threadIdx.x].nsave - 1 : -1;
    }
    if (threadIdx.x == 0) {
      int mx = 0;
      for (int r = 0; r < nrows; ++r) mx = max(mx, a.nacc[row0 + r]);
      s_maxn = mx;
    }
    __syncthreads();
    // VJP of the tile: input Y (per element), cotangent per element; output
    // J^T cot per element to `sink`; parameter cotangent accumulated into mu.
    auto vjp = [&](auto&& yval, auto&& cot, auto&& sink) {
      for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
        const int mm = e / S, s = e - mm * S;
        float y = 0.f, c = 0.f;
        if (mm < nrows) {
          y = yval(mm, s);
          c = cot(mm, s);
        }
        uraw[s * LD + mm] = y;
        act[0][s * LD + mm] = m.cube ? y * y * y : y;
        gA[s * LD + mm] = c;
      }
      if (m.timein)
        for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) act[0][S * LD + mm] = 0.f;
      __syncthreads();
      mlp_fwd_tile(m, act[0], nullptr, LD, TM, act + 1);
      const float* gi = mlp_vjp_tile(m, act, gA, gB, LD, TM, mu, 1.f);
      for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
        const int mm = e / S, s = e - mm * S;
        float g = gi[s * LD + mm];
        if (m.cube) {
          const float u = uraw[s * LD + mm];
          g *= 3.f * u * u;
        }
        sink(mm, s, g);
      }
      __syncthreads();
    };

    for (int q = 0; q < s_maxn; ++q) {
      if (threadIdx.x < TM) {
        const int r = threadIdx.x;
        int n = -1;
        if (r < nrows) n = a.nacc[row0 + r] - 1 - q;
        s_n[r] = n;
        if (n >= 0) {
          const int sg = row0 + r;
          s_tn[r] = a.steplog[((size_t)sg * a.MS + n) * 2];
          s_h[r] = a.steplog[((size_t)sg * a.MS + n) * 2 + 1];
          s_tnext[r] = (n + 1 < a.nacc[sg]) ? a.steplog[((size_t)sg * a.MS + n + 1) * 2] : a.segs[sg].t1;
        }
      }
      __syncthreads();
      // A: Ybar7 = ubar; ubar = 0; kbar_j (j < 7) = 0 (kbar7 holds the carry); saves in step n
      for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
        const int r = e / S, s = e - r * S;
        const int n = s_n[r];
        if (n < 0) continue;
        const int sg = row0 + r;
        float* B = a.bar;
        float ybar7 = B[bar_off(a, sg, 0) + s];
        float ub = 0.f;
        float kb[7];
        for (int j = 0; j < 6; ++j) kb[j] = 0.f;
        kb[6] = B[bar_off(a, sg, 8) + s];
        const MsSeg g = a.segs[sg];
        for (int si = s_isv[r]; si >= 0; --si) {
          const double sv = a.saveat[g.save_off + si];
          if (!(sv > s_tn[r])) break;
          const float sb = a.dLdu[(size_t)(g.save_off + si) * S + s];
          if (sv == s_tnext[r]) {
            ybar7 += sb;
          } else {
            float bw[7];
            interp_weights((sv - s_tn[r]) / s_h[r], bw);
            ub += sb;
            for (int j = 0; j < 7; ++j) kb[j] = fmaf((float)(s_h[r] * (double)bw[j]), sb, kb[j]);
          }
        }
        B[bar_off(a, sg, 0) + s] = ub;
        B[bar_off(a, sg, 1) + s] = ybar7;
        for (int j = 0; j < 7; ++j) B[bar_off(a, sg, 2 + j) + s] = kb[j];
      }
      __syncthreads();
      if (threadIdx.x < TM) {
        const int r = threadIdx.x, n = s_n[r];
        if (n >= 0) {
          const MsSeg g = a.segs[row0 + r];
          int si = s_isv[r];
          while (si >= 0 && a.saveat[g.save_off + si] > s_tn[r]) --si;
          s_isv[r] = si;
        }
      }
      __syncthreads();
      // B: stages 7..2
      for (int i = 6; i >= 1; --i) {
        vjp(
            [&](int r, int s) -> float {
              const int n = s_n[r];
              if (n < 0) return 0.f;
              const int sg = row0 + r;
              float acc = 0.f;
              for (int j = 0; j < i; ++j)
                acc = fmaf((float)(s_h[r] * c_tab.a[i][j]), a.dense[slot_off(a, sg, n, 1 + j) + s], acc);
              return a.dense[slot_off(a, sg, n, 0) + s] + acc;
            },
            [&](int r, int s) -> float {
              return s_n[r] < 0 ? 0.f : a.bar[bar_off(a, row0 + r, 2 + i) + s];
            },
            [&](int r, int s, float g) {
              const int n = s_n[r];
              if (n < 0) return;
              const int sg = row0 + r;
              float yb = g;
              if (i == 6) yb += a.bar[bar_off(a, sg, 1) + s];
              a.bar[bar_off(a, sg, 0) + s] += yb;
              for (int j = 0; j < i; ++j)
                a.bar[bar_off(a, sg, 2 + j) + s] =
                    fmaf((float)(s_h[r] * c_tab.a[i][j]), yb, a.bar[bar_off(a, sg, 2 + j) + s]);
            });
      }
      // C: kbar1 -> carry into kbar7 of step n-1; for n == 0 take the VJP at u0
      bool any0 = false;
      for (int r = 0; r < nrows; ++r) any0 |= (s_n[r] == 0);
      if (any0) {
        vjp([&](int r, int s) -> float { return s_n[r] == 0 ? a.dense[slot_off(a, row0 + r, 0, 0) + s] : 0.f; },
            [&](int r, int s) -> float { return s_n[r] == 0 ? a.bar[bar_off(a, row0 + r, 2) + s] : 0.f; },
            [&](int r, int s, float g) {
              if (s_n[r] != 0) return;
              const int sg = row0 + r;
              float ub = a.bar[bar_off(a, sg, 0) + s] + g;
              // save points at t0 (copies of u0)
              const MsSeg gg = a.segs[sg];
              for (int si = s_isv[r]; si >= 0; --si)
                if (a.saveat[gg.save_off + si] == gg.t0) ub += a.dLdu[(size_t)(gg.save_off + si) * S + s];
              a.bar[bar_off(a, sg, 0) + s] = ub;
            });
      }
      for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
        const int r = e / S, s = e - r * S;
        if (s_n[r] > 0) {
          const int sg = row0 + r;
          a.bar[bar_off(a, sg, 8) + s] = a.bar[bar_off(a, sg, 2) + s];
        }
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < nrows * S; e += blockDim.x) {
      const int r = e / S, s = e - r * S;
      const int sg = row0 + r;
      float v = a.bar[bar_off(a, sg, 0) + s];
      if (a.nacc[sg] == 0) {
        // no step taken: every save point is a copy of u0
        const MsSeg g = a.segs[sg];
        v = 0.f;
        for (int si = 0; si < g.nsave; ++si) v += a.dLdu[(size_t)(g.save_off + si) * S + s];
      }
      a.dLdu0[(size_t)sg * S + s] = v;
    }
    __syncthreads();
  }
}

int launch_ms_fwd(const MsArgs& a, int grid, size_t smem, cudaStream_t st) {
  if (cudaFuncSetAttribute(ms_fwd_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  ms_fwd_f32_kernel<<<grid, 256, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_ms_bwd(const MsArgs& a, int grid, size_t smem, cudaStream_t st) {
  if (cudaFuncSetAttribute(ms_bwd_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return -1;
  ms_bwd_f32_kernel<<<grid, 256, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
