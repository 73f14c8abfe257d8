// kernels.h -- launch descriptors shared by the host API (api.cu) and the
// kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include "mlp_simt.cuh"

namespace gbnde {

// Counters written by the persistent kernels (device, long long).
enum CounterSlot {
  CT_NF = 0,
  CT_NACCEPT = 1,
  CT_NREJECT = 2,
  CT_NCKPT = 3,
  CT_NRECOMP = 4,
  CT_NATTEMPT = 6,
  CT_NVJP = 7,  // adjoint evaluations that ran the VJP only
  CT_NSLOTS = 8
};

// Forward solve of one batched state (NeuralODE forward).
struct FwdArgs {
  MlpDev mlp;
  int S, B, TM, LD, ntiles;
  double t0, t1, abstol, reltol, dt0, dtmin, dtmax;
  int f32time;           // t, dt, EEst, qold kept as Float32 values (GBNDE_FLAG_FP32_TIME)
  long long maxiters;
  const double* saveat;  // device, nsave
  int nsave;
  const double* bnd;     // checkpoint boundaries (device, nbnd, increasing)
  int nbnd;
  const float* u0;
  float* ubuf[2];
  float* kbuf[7];
  float* usave;          // S*B*nsave
  float* ckpt;           // S*B*max_ckpt
  int max_ckpt;
  int* ckpt_step;        // accepted-step index of each checkpoint
  double* steplog;       // 2*maxsteps: (t_n, h_n)
  long long maxsteps;
  double* trace;         // 4*maxsteps: (t, h, EEst, accepted) per attempt
  float* dense;          // per accepted step n: slot of 8 x S*B floats (u_n, k1..k7), or null
  long long dense_slots;
  double* partials;      // 2*2*grid
  unsigned int* bar;
  int* status;
  long long* counters;
  double* tfinal;
  // FFJORD mode: state = [z (ffd rows); delta_logp], RHS = [f(z); -trace];
  // with ffreg two more rows integrate |f|^2 and |e^T J| (e = noise)
  int ffj, ffd, exact, ffreg;
  const float* noise;    // ffd x B (Hutchinson directions; the e of |e^T J|)
};

// One backward interval of InterpolatingAdjoint: forward steps [nlo, nhi]
// recomputed from checkpoint `ckpt`, backward solve from t_hi down to t_lo.
struct Interval {
  double t_lo, t_hi;
  int nlo, nhi;
  int ckpt;
  int save_lo;   // first saveat index equal to t_lo (-1 if none)
  int nsave_lo;  // number of saveat entries equal to t_lo
  int pad;
};

struct BwdArgs {
  MlpDev mlp;
  int S, B, TM, LD, ntiles;
  int P;                  // number of parameters
  int sensealg;
  double t0, abstol, reltol, dtmax;
  int f32time;            // as FwdArgs::f32time
  long long maxiters;
  const Interval* iv;     // device, niv (ordered from the last interval to the first)
  int niv;
  const double* fsteps;   // forward steplog (t_n, h_n)
  long long nfsteps;
  const float* ckpt;      // forward checkpoints
  const float* usave;     // forward saved states (Backsolve resets)
  const float* dLdu;      // S*B*nsave cotangent
  const double* saveat;
  int nsave;
  int save_last;          // index of the first saveat entry equal to the last time
  int nsave_last;
  float* ibuf;            // interval recompute buffer: slot j = (u_n, k1..k7)
  int ibuf_slots;
  const float* dense;     // forward dense slots (slot n = step n); when set, no recompute
  float* lam[2];          // adjoint state ping-pong
  float* ub[2];           // Backsolve: co-integrated u ping-pong
  float* kl[7];           // adjoint stage buffers (lambda part)
  float* ku[7];           // Backsolve: u part of the stages
  float* kf[7];           // forward recompute stage buffers
  float* mu_acc;          // per-CTA committed parameter gradient [grid][P]
  float* mu_stage;        // per-CTA pending quadrature [grid][3][P]  (P1, Pmid, P7)
  int pb_smem_off;        // > 0: the pending quadrature lives in dynamic shared memory at this
                          //   float offset instead (small models: no global round trips)
  float* dLdu0;           // output S*B
  double* partials;
  unsigned int* bar;
  int* status;
  long long* counters;
  int ffj, ffd, exact;    // FFJORD mode (see FwdArgs)
  int ffreg;              // bit 0: the two regulariser rows; bit 1: the |e^T J|
                          // row has a nonzero cotangent (its extra pass runs)
  const float* noise;
};

int launch_fwd_f32(const FwdArgs& a, int grid, size_t smem, cudaStream_t st);
struct FwdTcArgs;
int launch_fwd_tc(const FwdTcArgs& a, int grid, cudaStream_t st);
int max_grid_fwd_tc(int* grid);
int launch_prep_weight_image(const float* W, int N, int K, int Npad, uint8_t* img, cudaStream_t st);
int max_grid_fwd_f32(size_t smem, int* grid);
int launch_bwd_f32(const BwdArgs& a, int grid, size_t smem, cudaStream_t st);
int max_grid_bwd_f32(size_t smem, int* grid);

}  // namespace gbnde
