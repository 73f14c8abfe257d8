// bwd_f32.cu -- persistent continuous-adjoint solve, plain FP32 form.
//
// Replaces the pullback of SciMLSensitivity's rrule on `solve` for the
// sensealgs the DiffEqFlux layers use: InterpolatingAdjoint (the default,
// src/neural_de.jl:57) and BacksolveAdjoint (test/BasicNeuralDE/neural_de_tests.jl:36).
//
// The adjoint ODE is integrated in reverse time tau = -t with the same Tsit5
// tableau and tolerances as the forward solve:
//   d lam / d tau = J(u)^T lam,  d mu / d tau = (df/dp)^T lam,  [Backsolve: d u / d tau = -f(u)]
// from the last save point down to t0, with the save points as stops where
// lam jumps by dL/du(t_i) (and, for Backsolve, u is reset to the saved
// forward state). The error norm covers lam (and u for Backsolve); mu is a
// quadrature with the Tsit5 weights over accepted steps.
//
// InterpolatingAdjoint needs u(t) at every backward stage. The forward kept
// one checkpoint per save interval; here each interval's forward steps are
// recomputed from it with the recorded step sizes (bit-identical to the
// forward solve) into a stage buffer, and u(t) is the free interpolant of
// the forward step containing t -- the dense forward solution, with memory
// O(checkpoints + one interval).
//
// Each CTA accumulates its trajectories' share of mu in its own FP32 slot;
// a deterministic reduction over CTAs follows the launch.
#include "kernels.h"

namespace gbnde {

namespace {

struct Smem {
  float* act[GBNDE_MAX_LAYERS + 1];
  float* gA;
  float* gB;
  float* uraw;  // chain input before the cube prefix (S x LD)
};

__device__ __forceinline__ int nvalid_of(const BwdArgs& a, int tile) {
  return min(a.TM, a.B - tile * a.TM);
}

// Index of the recomputed forward step (within the interval) containing t.
__device__ __forceinline__ int find_step(const BwdArgs& a, const Interval& iv, double t) {
  int n = iv.nlo;
  while (n < iv.nhi && a.fsteps[2 * (n + 1)] <= t) ++n;
  return n;
}

// u(t) weights of the forward step holding tt: hb[j] = h b_j(theta); returns
// the step.
__device__ __forceinline__ int dense_weights_at(const BwdArgs& a, const Interval& iv, double tt, float* hb) {
  const int n = find_step(a, iv, tt);
  const double tn = a.fsteps[2 * n], h = a.fsteps[2 * n + 1];
  float bw[7];
  interp_weights((tt - tn) / h, bw);
  for (int q = 0; q < 7; ++q) hb[q] = (float)(h * (double)bw[q]);
  return n;
}

// The scalar FP64 work of an adjoint step, run by warp 0 (every lane keeps
// the same t, dt and qold) and kept out of line so that its registers do not
// weigh on the tile loops: the step setup (lane i: stage i's time,
// coefficients and u(t) weights; lane 7: the error weights) ...
__device__ __noinline__ void adj_step_setup(const BwdArgs& a, const Interval& iv, double t, double t_lo, double dt,
                                            bool backsolve, StepCtl* c, float (*hb6)[7], int* n6) {
  const int lane = threadIdx.x;
  const bool go = t > t_lo;
  const double rem = rt32(t - t_lo, a.f32time);
  const bool clipped = dt >= rem;
  const double Hs = clipped ? rem : dt;
  if (lane == 0) {
    c->go = go;
    c->clipped = clipped;
    c->t = t;
    c->h = Hs;
    c->hf = (float)Hs;
  }
  if (go && lane >= 1 && lane < 7) {
    const int i = lane;
    const double tt = t - c_tab.c[i] * Hs;
    c->tst[i] = tt;
    for (int q = 0; q < 6; ++q) c->ha[i - 1][q] = (float)(Hs * c_tab.a[i][q]);
    if (!backsolve) n6[i - 1] = dense_weights_at(a, iv, tt, hb6[i - 1]);
  } else if (go && lane == 7) {
    for (int q = 0; q < 7; ++q) c->hbt[q] = (float)(Hs * c_tab.btilde[q]);
  }
}

// ... and the controller after the error norm (qe: the grid's sum of squares):
// accept or reject, the next step size, and for an accepted step with the
// Gauss quadrature its four points (lane gq).
__device__ __noinline__ void adj_step_control(const BwdArgs& a, const Interval& iv, double qe, double Nnorm,
                                              double t_lo, bool gauss, double* t, double* dt, double* qold,
                                              StepCtl* c, float (*hb6)[7], int* n6, float (*bl4)[7]) {
  const int lane = threadIdx.x;
  const double H = c->h;
  const double eest = rt32(sqrt(qe / Nnorm), a.f32time);
  int rc = GBNDE_RET_SUCCESS, acc = 0;
  if (!isfinite(eest)) {
    rc = GBNDE_RET_UNSTABLE;
  } else {
    double q11;
    double q = pi_q(eest, *qold, &q11);
    if (eest <= 1.0) {
      acc = 1;
      if (gauss && lane < 4) {
        const double gth[4] = {0.06943184420297371, 0.33000947820757187, 0.6699905217924281,
                               0.9305681557970262};
        const double gw[4] = {0.17392742256872679, 0.3260725774312732, 0.3260725774312732,
                              0.17392742256872679};
        const int gq = lane;
        const double tt = *t - gth[gq] * H;
        c->tst[gq] = tt;
        float bl[7];
        interp_weights(gth[gq], bl);
        for (int q2 = 0; q2 < 7; ++q2) bl4[gq][q2] = (float)(H * (double)bl[q2]);
        c->hb[gq] = (float)(H * gw[gq]);
        n6[gq] = dense_weights_at(a, iv, tt, hb6[gq]);
      }
      *t = c->clipped ? t_lo : rt32(*t - H, a.f32time);
      if (q >= 1.0 && q <= 1.0) q = 1.0;
      *qold = rt32(fmax(eest, kQoldInit), a.f32time);
      *dt = rt32(fmin(H / q, a.dtmax), a.f32time);
    } else {
      *dt = rt32(H / fmin(1.0 / kQmin, q11 / kGamma), a.f32time);
    }
  }
  __syncwarp();
  if (lane == 0) {
    c->ret = rc;
    c->accept = acc;
  }
}

// Forward RHS on a tile into `out` rows (plain, no kept activations), input
// produced per element.
template <class Fn>
__device__ __forceinline__ const float* fwd_eval_tile(const BwdArgs& a, int tile, Smem& sm,
                                                      double tstage, Fn&& val) {
  const int S = a.S, TM = a.TM, LD = a.LD;
  const size_t base = (size_t)tile * TM * S;
  const int nv = nvalid_of(a, tile);
  float* in = sm.gA;
  for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
    const int m = e / S, s = e - m * S;
    float v = 0.f;
    if (m < nv) v = val(base + e);
    if (a.mlp.cube) v = v * v * v;
    in[s * LD + m] = v;
  }
  if (a.mlp.timein)
    for (int m = threadIdx.x; m < TM; m += blockDim.x) in[S * LD + m] = (float)tstage;
  __syncthreads();
  return mlp_fwd_tile(a.mlp, sm.gA, sm.gB, LD, TM, nullptr);
}

// The |e^T J| row's share of the FFJORD adjoint right-hand side (out of line:
// it runs only with the regulariser rows and keeps its registers out of the
// main kernel). v = J^T e by a reverse pass, w = v / |v| (0 where v = 0), then
// the cotangent of e^T J w with w held fixed: a reverse-over-forward pass
// along w with lam_j e on the tangent output; adds its z rows to kl_out and
// its parameter cotangent to P (scaled by c). act holds the primal pass.
__device__ __noinline__ void ffj_reg_pass(const BwdArgs& a, int tile, float* const* fact, float* const* fzd,
                                          float* const* fcot, const float* flj, float* fnrm, float* kl_out,
                                          float* P, float c) {
  const MlpDev& m = a.mlp;
  const int d = a.ffd, S = a.S, TM = a.TM, LD = a.LD;
  const size_t base = (size_t)tile * TM * S;
  const int nv = nvalid_of(a, tile);
  for (int e = threadIdx.x; e < d * TM; e += blockDim.x) {
    const int s = e / TM, mm = e - s * TM;
    fcot[0][s * LD + mm] = mm < nv ? a.noise[((size_t)tile * TM + mm) * d + s] : 0.f;
  }
  __syncthreads();
  const float* v = mlp_vjp_tile(m, fact, fcot[0], fcot[1], LD, TM, nullptr, 0.f);
  for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) {
    float q = 0.f;
    for (int s = 0; s < d; ++s) q = fmaf(v[s * LD + mm], v[s * LD + mm], q);
    fnrm[mm] = q > 0.f ? 1.f / sqrtf(q) : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < m.dims[0] * TM; e += blockDim.x) {
    const int s = e / TM, mm = e - s * TM;
    fzd[0][s * LD + mm] = s < d ? v[s * LD + mm] * fnrm[mm] : 0.f;
  }
  __syncthreads();
  mlp_tangent_tile(m, fact, fzd, fcot[3], LD, TM);
  for (int e = threadIdx.x; e < d * TM; e += blockDim.x) {
    const int s = e / TM, mm = e - s * TM;
    fcot[0][s * LD + mm] = 0.f;
    fcot[2][s * LD + mm] = mm < nv ? flj[mm] * a.noise[((size_t)tile * TM + mm) * d + s] : 0.f;
  }
  __syncthreads();
  const float* gi = ffjord_vjp_tile(m, fact, fzd, fcot[0], fcot[1], fcot[2], fcot[3], LD, TM, P, c);
  for (int e = threadIdx.x; e < nv * S; e += blockDim.x) {
    const int mm = e / S, s = e - mm * S;
    if (s < d) kl_out[base + e] += gi[s * LD + mm];
  }
  __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(256, 1) bwd_f32_kernel(BwdArgs a) {
  extern __shared__ __align__(16) float smem[];
  __shared__ double red[40];
  // the step's scalars from thread 0 (see StepCtl): stage i's interpolation
  // weights and forward step, or quadrature point q's
  __shared__ StepCtl s_ctl;
  __shared__ float s_hb6[6][7], s_bl4[4][7];
  __shared__ int s_n6[6];
  const int S = a.S, TM = a.TM, LD = a.LD, G = gridDim.x;
  const bool backsolve = (a.sensealg == GBNDE_SENSE_BACKSOLVE);
  // quadrature adjoint: lam only in the solve, mu by Gauss-Legendre per step
  const bool gauss = (a.sensealg == GBNDE_SENSE_GAUSS);
  const double Nnorm = (double)S * (double)a.B * (backsolve ? 2.0 : 1.0);

  Smem sm;
  {
    float* p = smem;
    for (int l = 0; l <= a.mlp.nlayers; ++l) {
      sm.act[l] = p;
      p += (size_t)a.mlp.dims[l] * LD;
    }
    sm.gA = p;
    p += (size_t)a.mlp.maxdim * LD;
    sm.gB = p;
    p += (size_t)a.mlp.maxdim * LD;
    sm.uraw = p;
  }
  float* mu_acc = a.mu_acc + (size_t)blockIdx.x * a.P;
  float* pbase = a.pb_smem_off > 0 ? smem + a.pb_smem_off : a.mu_stage + (size_t)blockIdx.x * 3 * a.P;
  float* Pb[3] = {pbase, pbase + a.P, pbase + 2 * (size_t)a.P};
  int iP1 = 0, iP7 = 2;  // roles of Pb[0] and Pb[2] swap on accept
  float* Pmid = Pb[1];

  unsigned int gen = 0;
  int par = 0, cur = 0;
  bool swp = false;
  int ret = GBNDE_RET_SUCCESS;
  long long nf_adj = 0, nf_rec = 0, nacc = 0, nrej = 0, iter = 0;
  double dt = 0.0, qold = kQoldInit;

  auto klb = [&](int j) -> float* {
    if (j == 0) return swp ? a.kl[6] : a.kl[0];
    if (j == 6) return swp ? a.kl[0] : a.kl[6];
    return a.kl[j];
  };
  auto kub = [&](int j) -> float* {
    if (j == 0) return swp ? a.ku[6] : a.ku[0];
    if (j == 6) return swp ? a.ku[0] : a.ku[6];
    return a.ku[j];
  };

  for (size_t i = threadIdx.x; i < (size_t)a.P; i += blockDim.x) mu_acc[i] = 0.f;

  // lam = dL/du at the last save time; Backsolve: u = saved state there.
  for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
    const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
    for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
      float v = 0.f;
      for (int q = 0; q < a.nsave_last; ++q) v += a.dLdu[(size_t)(a.save_last + q) * S * a.B + base + e];
      a.lam[0][base + e] = v;
      if (backsolve) a.ub[0][base + e] = a.usave[(size_t)a.save_last * S * a.B + base + e];
    }
  }
  __syncthreads();

  // Adjoint RHS on a tile at time `tt`: lam stage from `lamv`, u from `uval`
  // (Interpolating: dense forward output; Backsolve: stage of co-integrated u).
  // Writes kl (J^T lam) and, for Backsolve, ku (-f(u)); accumulates mu into P*c.
  // FFJORD layout: act[0..L], zd[0..L] (sum(dims) rows each), 4 cotangent
  // buffers (maxdim rows each), tmp (maxdim rows).
  float* fact[GBNDE_MAX_LAYERS + 1];
  float* fzd[GBNDE_MAX_LAYERS + 1];
  float* fcot[4];
  float* ftmp = nullptr;
  float* flam = nullptr;  // lam_l per trajectory of the tile
  float* flf = nullptr;   // cotangents of the |f|^2 and |e^T J| rows (ffreg)
  float* flj = nullptr;
  float* fnrm = nullptr;  // |J^T e| per trajectory
  if (a.ffj) {
    float* p = smem;
    for (int l = 0; l <= a.mlp.nlayers; ++l) { fact[l] = p; p += (size_t)a.mlp.dims[l] * LD; }
    for (int l = 0; l <= a.mlp.nlayers; ++l) { fzd[l] = p; p += (size_t)a.mlp.dims[l] * LD; }
    for (int q = 0; q < 4; ++q) { fcot[q] = p; p += (size_t)a.mlp.maxdim * LD; }
    ftmp = fcot[3];  // the tangent pass runs before fcot[3] is used as a cotangent
    flam = p;
    flf = p + LD;
    flj = p + 2 * LD;
    fnrm = p + 3 * LD;
  }
  // FFJORD adjoint right-hand side: cotangent [lam_z; lam_l] of [f; -trace];
  // writes kl = lam_z^T df/dz - lam_l d(trace)/dz (z rows; 0 for the logp row).
  // With the regulariser rows (cotangents lam_f, lam_j; src/ffjord.jl:131-132):
  // |f|^2 adds 2 lam_f f to the primal output's cotangent, and |e^T J| adds the
  // cotangent of e^T J w with w = J^T e / |J^T e| held fixed (d|v| = w^T dv),
  // one more reverse-over-forward pass along w with e lam_j on the tangent
  // output.
  auto ffj_eval = [&](int tile, double tt, auto&& lamv, auto&& uval, float* kl_out, float* P, float c,
                      float* lam_store) {
    const MlpDev& m = a.mlp;
    const int d = a.ffd, L = m.nlayers;
    const size_t base = (size_t)tile * TM * S;
    const int nv = nvalid_of(a, tile);
    for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
      const int mm = e / S, s = e - mm * S;
      float u = 0.f, l = 0.f;
      if (mm < nv) {
        u = uval(base + e);
        l = lamv(base + e);
        if (lam_store) lam_store[base + e] = l;
      }
      if (s < d) {
        fact[0][s * LD + mm] = u;
        fcot[0][s * LD + mm] = l;     // cotangent of f (primal output), rows < d
      } else if (s == d) {
        flam[mm] = l;
      } else if (s == d + 1) {
        flf[mm] = l;
      } else {
        flj[mm] = l;
      }
    }
    if (m.timein)
      for (int mm = threadIdx.x; mm < TM; mm += blockDim.x) fact[0][d * LD + mm] = (float)tt;
    __syncthreads();
    mlp_fwd_tile(m, fact[0], nullptr, LD, TM, fact + 1);
    if (a.ffreg) {
      __syncthreads();
      for (int e = threadIdx.x; e < d * TM; e += blockDim.x) {
        const int s = e / TM, mm = e - s * TM;
        fcot[0][s * LD + mm] = fmaf(2.f * flf[mm], fact[L][s * LD + mm], fcot[0][s * LD + mm]);
      }
      __syncthreads();
    }
    const int ndir = a.exact ? d : 1;
    for (int k = 0; k < ndir; ++k) {
      for (int e = threadIdx.x; e < m.dims[0] * TM; e += blockDim.x) {
        const int s = e / TM, mm = e - s * TM;
        float v = 0.f;
        if (s < d && mm < nv) v = a.exact ? (s == k ? 1.f : 0.f) : a.noise[((size_t)tile * TM + mm) * d + s];
        fzd[0][s * LD + mm] = v;
      }
      __syncthreads();
      mlp_tangent_tile(m, fact, fzd, ftmp, LD, TM);
      // cotangents: primal (first direction only) and tangent output -lam_l e
      for (int e = threadIdx.x; e < d * TM; e += blockDim.x) {
        const int s = e / TM, mm = e - s * TM;
        fcot[2][s * LD + mm] = -flam[mm] * fzd[0][s * LD + mm];
        if (k > 0) fcot[0][s * LD + mm] = 0.f;
      }
      __syncthreads();
      const float* gi = ffjord_vjp_tile(m, fact, fzd, fcot[0], fcot[1], fcot[2], fcot[3], LD, TM, P, c);
      for (int e = threadIdx.x; e < nv * S; e += blockDim.x) {
        const int mm = e / S, s = e - mm * S;
        const float g = s < d ? gi[s * LD + mm] : 0.f;
        kl_out[base + e] = (k == 0) ? g : kl_out[base + e] + g;
      }
      __syncthreads();
    }
    if (a.ffreg & 2) ffj_reg_pass(a, tile, fact, fzd, fcot, flj, fnrm, kl_out, P, c);
  };

  auto adj_eval = [&](int tile, double tt, const Interval& iv, auto&& lamv, auto&& uval,
                      float* kl_out, float* ku_out, float* P, float c, float* lam_store,
                      float* u_store) {
    if (a.ffj) {
      ffj_eval(tile, tt, lamv, uval, kl_out, P, c, lam_store);
      return;
    }
    const size_t base = (size_t)tile * TM * S;
    const int nv = nvalid_of(a, tile);
    // chain input
    float* in = sm.act[0];
    for (int e = threadIdx.x; e < TM * S; e += blockDim.x) {
      const int m = e / S, s = e - m * S;
      float u = 0.f;
      if (m < nv) {
        u = uval(base + e);
        if (u_store) u_store[base + e] = u;
      }
      in[s * LD + m] = a.mlp.cube ? u * u * u : u;
      if (a.mlp.cube) sm.uraw[s * LD + m] = u;  // rows reserved only with the cube prefix
      // lam cotangent of the chain output goes to gA
      float l = 0.f;
      if (m < nv) {
        l = lamv(base + e);
        if (lam_store) lam_store[base + e] = l;
      }
      sm.gA[s * LD + m] = l;
    }
    if (a.mlp.timein)
      for (int m = threadIdx.x; m < TM; m += blockDim.x) in[S * LD + m] = (float)tt;
    __syncthreads();
    mlp_fwd_tile(a.mlp, sm.act[0], nullptr, LD, TM, sm.act + 1);
    const float* fo = sm.act[a.mlp.nlayers];
    const float* gi = mlp_vjp_tile(a.mlp, sm.act, sm.gA, sm.gB, LD, TM, P, c);
    for (int e = threadIdx.x; e < nv * S; e += blockDim.x) {
      const int m = e / S, s = e - m * S;
      float g = gi[s * LD + m];
      if (a.mlp.cube) {
        const float u = sm.uraw[s * LD + m];
        g *= 3.f * u * u;
      }
      if (kl_out) kl_out[base + e] = g;
      if (ku_out) ku_out[base + e] = -fo[s * LD + m];
    }
    __syncthreads();
  };

  for (int ivi = 0; ivi < a.niv && ret == GBNDE_RET_SUCCESS; ++ivi) {
    const Interval iv = a.iv[ivi];
    // ---- recompute the interval's forward steps (InterpolatingAdjoint) ----
    if (!backsolve && !a.dense) {
      const size_t SB = (size_t)S * a.B;
      const int nst = iv.nhi - iv.nlo + 1;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        const size_t base = (size_t)tile * TM * S;
        const int nv = nvalid_of(a, tile);
        for (int j = 0; j < nst; ++j) {
          float* slot = a.ibuf + (size_t)j * 8 * SB;
          float* us = slot;
          float* ks[7];
          for (int q = 0; q < 7; ++q) ks[q] = slot + (size_t)(q + 1) * SB;
          const double tn = a.fsteps[2 * (iv.nlo + j)], h = a.fsteps[2 * (iv.nlo + j) + 1];
          if (j == 0) {
            const float* ck = a.ckpt + (size_t)iv.ckpt * SB;
            const float* fo = fwd_eval_tile(a, tile, sm, tn, [&](size_t g) {
              us[g] = ck[g];
              return ck[g];
            });
            for (int e = threadIdx.x; e < nv * S; e += blockDim.x) {
              const int m = e / S, s = e - m * S;
              ks[0][base + e] = fo[s * LD + m];
            }
            __syncthreads();
          } else {
            float* prev = a.ibuf + (size_t)(j - 1) * 8 * SB;
            for (int e = threadIdx.x; e < nv * S; e += blockDim.x)
              ks[0][base + e] = prev[7 * SB + base + e];
            __syncthreads();
          }
          for (int i = 1; i < 7; ++i) {
            float ha[6];
            for (int q = 0; q < 6; ++q) ha[q] = (float)(h * c_tab.a[i][q]);
            float* nextu = (i == 6 && j + 1 < nst) ? a.ibuf + (size_t)(j + 1) * 8 * SB : nullptr;
            const float* fo = fwd_eval_tile(a, tile, sm, tn + c_tab.c[i] * h, [&](size_t g) {
              float s = 0.f;
              for (int q = 0; q < i; ++q) s = fmaf(ha[q], ks[q][g], s);
              const float y = us[g] + s;
              if (nextu) nextu[g] = y;
              return y;
            });
            for (int e = threadIdx.x; e < nv * S; e += blockDim.x) {
              const int m = e / S, s = e - m * S;
              ks[i][base + e] = fo[s * LD + m];
            }
            __syncthreads();
          }
        }
      }
      nf_rec += 1 + 6LL * nst;
    }

    // ---- backward solve over [t_lo, t_hi] ------------------------------------
    const double t_hi = iv.t_hi, t_lo = iv.t_lo;
    double t = t_hi;
    // dense forward output at time tt for element g
    auto udense = [&](double tt, float* hb, const float** kk, const float*& un) {
      const int n = find_step(a, iv, tt);
      const double tn = a.fsteps[2 * n], h = a.fsteps[2 * n + 1];
      float bw[7];
      interp_weights((tt - tn) / h, bw);
      const size_t SB = (size_t)S * a.B;
      const float* slot = a.dense ? a.dense + (size_t)n * 8 * SB : a.ibuf + (size_t)(n - iv.nlo) * 8 * SB;
      un = slot;
      for (int q = 0; q < 7; ++q) {
        hb[q] = (float)(h * (double)bw[q]);
        kk[q] = slot + (size_t)(q + 1) * SB;
      }
    };

    // FSAL stage at the interval start (after the jump): kl1, mu -> P1
    {
      float* P1 = Pb[iP1];
      for (size_t i = threadIdx.x; i < (size_t)a.P; i += blockDim.x) P1[i] = 0.f;
      if (threadIdx.x == 0 && !backsolve) {
        // u(t) weights on thread 0 (FP64), read by all after the barrier
        const int n = find_step(a, iv, t);
        const double tn = a.fsteps[2 * n], h = a.fsteps[2 * n + 1];
        float bw[7];
        interp_weights((t - tn) / h, bw);
        for (int q = 0; q < 7; ++q) s_hb6[0][q] = (float)(h * (double)bw[q]);
        s_n6[0] = n;
      }
      __syncthreads();
      float hb[7];
      const float* kk[7];
      const float* un = nullptr;
      if (!backsolve) {
        const size_t SB = (size_t)S * a.B;
        un = a.dense ? a.dense + (size_t)s_n6[0] * 8 * SB : a.ibuf + (size_t)(s_n6[0] - iv.nlo) * 8 * SB;
        for (int q = 0; q < 7; ++q) {
          hb[q] = s_hb6[0][q];
          kk[q] = un + (size_t)(q + 1) * SB;
        }
      }
      float* lcur = a.lam[cur];
      float* ucurb = a.ub[cur];
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        adj_eval(tile, t, iv, [&](size_t g) { return lcur[g]; },
                 [&](size_t g) {
                   if (backsolve) return ucurb[g];
                   float acc = 0.f;
                   for (int q = 0; q < 7; ++q) acc = fmaf(hb[q], kk[q][g], acc);
                   return un[g] + acc;
                 },
                 klb(0), backsolve ? kub(0) : nullptr, gauss ? nullptr : P1, (float)c_tab.b[0], nullptr, nullptr);
      }
      ++nf_adj;
    }

    // initial step of the backward solve (first interval only)
    if (ivi == 0) {
      double p0 = 0.0, p1 = 0.0;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
        for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
          const float l = a.lam[cur][base + e], f = klb(0)[base + e];
          const float sk = (float)a.abstol + fabsf(l) * (float)a.reltol;
          const double x = (double)(l / sk), y = (double)(f / sk);
          p0 += x * x;
          p1 += y * y;
          if (backsolve) {
            const float u = a.ub[cur][base + e], fu = kub(0)[base + e];
            const float sku = (float)a.abstol + fabsf(u) * (float)a.reltol;
            const double xu = (double)(u / sku), yu = (double)(fu / sku);
            p0 += xu * xu;
            p1 += yu * yu;
          }
        }
      }
      p0 = block_sum_double(p0, red);
      p1 = block_sum_double(p1, red);
      double* pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) {
        pp[blockIdx.x] = p0;
        pp[G + blockIdx.x] = p1;
      }
      if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
      const double d0 = sqrt(grid_partials_sum(pp, G, red) / Nnorm);
      const double d1 = sqrt(grid_partials_sum(pp + G, G, red) / Nnorm);
      par ^= 1;
      double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * (d0 / d1);
      dt0 = rt32(fmin(dt0, a.dtmax), a.f32time);
      const float hf = (float)dt0;
      const double tp = t - dt0;
      float hb[7];
      const float* kk[7];
      const float* un = nullptr;
      if (!backsolve) udense(tp, hb, kk, un);
      // probe evaluation into stage buffers 1 (scratch), no mu accumulation
      float* lcur = a.lam[cur];
      float* ucurb = a.ub[cur];
      float* k0l = klb(0);
      float* k0u = kub(0);
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        adj_eval(tile, tp, iv, [&](size_t g) { return lcur[g] + hf * k0l[g]; },
                 [&](size_t g) {
                   if (backsolve) return ucurb[g] + hf * k0u[g];
                   float acc = 0.f;
                   for (int q = 0; q < 7; ++q) acc = fmaf(hb[q], kk[q][g], acc);
                   return un[g] + acc;
                 },
                 klb(1), backsolve ? kub(1) : nullptr, nullptr, 0.f, nullptr, nullptr);
      }
      ++nf_adj;
      double p2 = 0.0;
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
        for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
          const float l = lcur[base + e];
          const float sk = (float)a.abstol + fabsf(l) * (float)a.reltol;
          const double z = (double)((klb(1)[base + e] - k0l[base + e]) / sk);
          p2 += z * z;
          if (backsolve) {
            const float u = ucurb[base + e];
            const float sku = (float)a.abstol + fabsf(u) * (float)a.reltol;
            const double zu = (double)((kub(1)[base + e] - k0u[base + e]) / sku);
            p2 += zu * zu;
          }
        }
      }
      p2 = block_sum_double(p2, red);
      pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = p2;
      if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
      const double d2 = sqrt(grid_partials_sum(pp, G, red) / Nnorm) / dt0;
      par ^= 1;
      const double mm = fmax(d1, d2);
      const double dt1 = (mm <= 1e-15) ? fmax(1e-6, dt0 * 1e-3) : pow(10.0, -(2.0 + log10(mm)) / 5.0);
      dt = rt32(fmin(100.0 * dt0, fmin(dt1, a.dtmax)), a.f32time);
    }

    // ---- adaptive steps down to t_lo ----------------------------------------
    // The scalar FP64 work of a step (stage times and coefficients, the
    // forward step and interpolation weights of every stage, the norm's square
    // root, the PI update) runs on thread 0 and reaches the others through
    // shared memory; t, dt and qold are thread 0's.
    auto dense_of = [&](int n) -> const float* {
      const size_t SB = (size_t)S * a.B;
      return a.dense ? a.dense + (size_t)n * 8 * SB : a.ibuf + (size_t)(n - iv.nlo) * 8 * SB;
    };
    for (;;) {
      if (threadIdx.x < 32) adj_step_setup(a, iv, t, t_lo, dt, backsolve, &s_ctl, s_hb6, s_n6);
      __syncthreads();
      if (!s_ctl.go) break;
      if (iter >= a.maxiters) { ret = GBNDE_RET_MAXITERS; break; }
      ++iter;
      float* lcur = a.lam[cur];
      float* lnew = a.lam[cur ^ 1];
      float* ucurb = a.ub[cur];
      float* unewb = a.ub[cur ^ 1];
      for (size_t i = threadIdx.x; i < (size_t)a.P; i += blockDim.x) Pmid[i] = 0.f;
      __syncthreads();
      double perr = 0.0;
      for (int i = 1; i < 7; ++i) {
        const double tt = s_ctl.tst[i];
        float ha[6];
        for (int q = 0; q < 6; ++q) ha[q] = s_ctl.ha[i - 1][q];
        const float* kl[6];
        const float* ku[6];
        for (int q = 0; q < 6; ++q) {
          kl[q] = klb(q);
          ku[q] = kub(q);
        }
        float hb[7];
        const float* kk[7];
        const float* un = nullptr;
        if (!backsolve) {
          un = dense_of(s_n6[i - 1]);
          for (int q = 0; q < 7; ++q) {
            hb[q] = s_hb6[i - 1][q];
            kk[q] = un + (size_t)(q + 1) * S * a.B;
          }
        }
        float* P = gauss ? nullptr : (i < 6) ? Pmid : Pb[iP7];
        if (i == 6 && P) {
          for (size_t q = threadIdx.x; q < (size_t)a.P; q += blockDim.x) P[q] = 0.f;
          __syncthreads();
        }
        const float c = (i < 6) ? (float)c_tab.b[i] : (float)c_tab.b[0];
        for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
          adj_eval(tile, tt, iv,
                   [&](size_t g) {
                     float s = 0.f;
                     for (int q = 0; q < i; ++q) s = fmaf(ha[q], kl[q][g], s);
                     return lcur[g] + s;
                   },
                   [&](size_t g) {
                     if (backsolve) {
                       float s = 0.f;
                       for (int q = 0; q < i; ++q) s = fmaf(ha[q], ku[q][g], s);
                       return ucurb[g] + s;
                     }
                     float acc = 0.f;
                     for (int q = 0; q < 7; ++q) acc = fmaf(hb[q], kk[q][g], acc);
                     return un[g] + acc;
                   },
                   klb(i), backsolve ? kub(i) : nullptr, P, c, (i == 6) ? lnew : nullptr,
                   (i == 6 && backsolve) ? unewb : nullptr);
          if (i == 6) {
            // error contribution of this tile
            float hbt[7];
            for (int q = 0; q < 7; ++q) hbt[q] = s_ctl.hbt[q];
            const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
            for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
              const size_t g = base + e;
              float lt = 0.f;
              for (int q = 0; q < 7; ++q) lt = fmaf(hbt[q], klb(q)[g], lt);
              const float sc = (float)a.abstol + fmaxf(fabsf(lcur[g]), fabsf(lnew[g])) * (float)a.reltol;
              const double r = (double)(lt / sc);
              perr += isfinite(lnew[g]) ? r * r : (double)INFINITY;
              if (backsolve) {
                float ut = 0.f;
                for (int q = 0; q < 7; ++q) ut = fmaf(hbt[q], kub(q)[g], ut);
                const float scu = (float)a.abstol + fmaxf(fabsf(ucurb[g]), fabsf(unewb[g])) * (float)a.reltol;
                const double ru = (double)(ut / scu);
                perr += ru * ru;
              }
            }
            __syncthreads();
          }
        }
        ++nf_adj;
      }
      perr = block_sum_double(perr, red);
      double* pp = a.partials + (size_t)par * 2 * G;
      if (threadIdx.x == 0) pp[blockIdx.x] = perr;
      if (!grid_barrier(a.bar, gen, a.status)) { ret = GBNDE_RET_BARRIER_TIMEOUT; break; }
      {
        const double qe = grid_partials_sum(pp, G, red);
        if (threadIdx.x < 32)
          adj_step_control(a, iv, qe, Nnorm, t_lo, gauss, &t, &dt, &qold, &s_ctl, s_hb6, s_n6, s_bl4);
        __syncthreads();
      }
      par ^= 1;
      if (s_ctl.ret != GBNDE_RET_SUCCESS) { ret = s_ctl.ret; break; }
      if (s_ctl.accept) {
        if (gauss) {
          // mu += int over the step of lam^T df/dp: 4-point Gauss-Legendre on
          // [t - H, t], lam(theta) = lam_n + H sum_j b_j(theta) k_j from this
          // step's stages (the free interpolant), u from the forward
          const float* kl7[7];
          for (int q = 0; q < 7; ++q) kl7[q] = klb(q);
          for (int gq = 0; gq < 4; ++gq) {
            const double tt = s_ctl.tst[gq];
            float bl[7];
            for (int q = 0; q < 7; ++q) bl[q] = s_bl4[gq][q];
            float hb[7];
            const float* kk[7];
            const float* un = dense_of(s_n6[gq]);
            for (int q = 0; q < 7; ++q) {
              hb[q] = s_hb6[gq][q];
              kk[q] = un + (size_t)(q + 1) * S * a.B;
            }
            for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
              adj_eval(tile, tt, iv,
                       [&](size_t g) {
                         float s = 0.f;
                         for (int q = 0; q < 7; ++q) s = fmaf(bl[q], kl7[q][g], s);
                         return lcur[g] + s;
                       },
                       [&](size_t g) {
                         float acc = 0.f;
                         for (int q = 0; q < 7; ++q) acc = fmaf(hb[q], kk[q][g], acc);
                         return un[g] + acc;
                       },
                       nullptr, nullptr, mu_acc, s_ctl.hb[gq], nullptr, nullptr);
            }
            ++nf_adj;
          }
          __syncthreads();
        } else {
          // mu += H * (P1 + Pmid)
          const float Hf = s_ctl.hf;
          const float* P1 = Pb[iP1];
          for (size_t i = threadIdx.x; i < (size_t)a.P; i += blockDim.x)
            mu_acc[i] = fmaf(Hf, P1[i] + Pmid[i], mu_acc[i]);
          __syncthreads();
        }
        const int tmp = iP1;
        iP1 = iP7;
        iP7 = tmp;
        ++nacc;
        cur ^= 1;
        swp = !swp;
      } else {
        ++nrej;
      }
    }
    if (ret != GBNDE_RET_SUCCESS) break;

    // ---- jump at t_lo: lam += dL/du(t_lo); Backsolve: u = saved state -------
    if (iv.nsave_lo > 0) {
      for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
        const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
        for (size_t e = threadIdx.x; e < n; e += blockDim.x) {
          float v = a.lam[cur][base + e];
          for (int q = 0; q < iv.nsave_lo; ++q)
            v += a.dLdu[(size_t)(iv.save_lo + q) * S * a.B + base + e];
          a.lam[cur][base + e] = v;
          if (backsolve) a.ub[cur][base + e] = a.usave[(size_t)iv.save_lo * S * a.B + base + e];
        }
      }
      __syncthreads();
    }
  }

  // dL/du0 = lam(t0)
  if (ret == GBNDE_RET_SUCCESS) {
    for (int tile = blockIdx.x; tile < a.ntiles; tile += G) {
      const size_t base = (size_t)tile * TM * S, n = (size_t)nvalid_of(a, tile) * S;
      for (size_t e = threadIdx.x; e < n; e += blockDim.x) a.dLdu0[base + e] = a.lam[cur][base + e];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.counters[CT_NF] = nf_adj;
    a.counters[CT_NACCEPT] = nacc;
    a.counters[CT_NREJECT] = nrej;
    a.counters[CT_NRECOMP] = nf_rec;
    a.status[ST_RETCODE] = (a.status[ST_BARRIER] != 0) ? GBNDE_RET_BARRIER_TIMEOUT : ret;
  }
}

// dLdp[i] = sum over CTAs of mu_acc[cta][i], in CTA order.
__global__ void reduce_mu_kernel(const float* __restrict__ mu_acc, int nblk, int P,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += mu_acc[(size_t)b * P + i];
  out[i] = s;
}

int max_grid_bwd_f32(size_t smem, int* grid) {
  cudaError_t e = cudaFuncSetAttribute(bwd_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return -1;
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bwd_f32_kernel, 256, smem);
  if (e != cudaSuccess || per_sm < 1) return -1;
  *grid = per_sm * nsm;
  return 0;
}

int launch_bwd_f32(const BwdArgs& a, int grid, size_t smem, cudaStream_t st) {
  void* args[] = {(void*)&a};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)bwd_f32_kernel, dim3(grid), dim3(256),
                                              args, smem, st);
  if (e != cudaSuccess) return -1;
  return 0;
}

int launch_reduce_mu(const float* mu_acc, int nblk, int P, float* out, cudaStream_t st) {
  reduce_mu_kernel<<<(P + 255) / 256, 256, 0, st>>>(mu_acc, nblk, P, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace gbnde
