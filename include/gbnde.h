/*
 * gbnde.h -- C ABI of the GB300 neural-ODE solver library (libgbnde.so).
 *
 * The library replaces, for one GPU (sm_103a), the arithmetic that the
 * reference reaches through `solve` when a DiffEqFlux layer is called:
 *
 *   NeuralODE (x, p, st) -> (sol, st)        src/neural_de.jl:47-61
 *   FFJORD    (x, ps, st) -> ((logpx,..),st) src/ffjord.jl:138-178
 *   multiple_shoot(p, data, tsteps, ...)     src/multiple_shooting.jl:36-94
 *
 * i.e. OrdinaryDiffEq's Tsit5 + PI controller + saveat interpolation, the
 * SciMLSensitivity InterpolatingAdjoint / BacksolveAdjoint gradient that the
 * layers select (src/neural_de.jl:57, src/ffjord.jl:143) and the Lux Dense
 * chain used as right-hand side. Host code (Julia `ccall`, Python `ctypes`)
 * keeps the layer constructors and call signatures and calls these entry points.
 *
 * Conventions
 *  - All functions return 0 on success or a negative gbnde_error code; they
 *    never throw or exit. gbnde_strerror() names the code, gbnde_last_error()
 *    gives a message for the last failing call on this thread.
 *  - Arrays are column-major like Julia: a state batch is S x B with one
 *    trajectory per column (element (s, b) at b*S + s); saved states are
 *    S x B x nsave. Parameters are the flat vector ComponentArray(ps) gives:
 *    per Dense layer its weight (out x in, column-major) then its bias.
 *  - Functions without the _device suffix take HOST pointers and copy
 *    through pinned staging buffers on the context's stream. The _device
 *    variants take DEVICE pointers (no copies).
 *  - A context is not thread-safe; use one per host thread/task. Different
 *    contexts may run concurrently.
 *  - Solver outcomes come back in gbnde_stats.retcode (gbnde_retcode), which
 *    maps onto SciMLBase.ReturnCode; a failed solve is not an API error.
 */
#ifndef GBNDE_H
#define GBNDE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBNDE_MAX_LAYERS 8

typedef struct gbnde_ctx gbnde_ctx;

typedef enum {
  GBNDE_ACT_IDENTITY = 0,
  GBNDE_ACT_TANH = 1,
  GBNDE_ACT_SOFTPLUS = 2
} gbnde_act;

/* Arithmetic of the MLP right-hand side. FP32: every operation in FP32
 * (the plain drop-in). BF16: GEMMs on the tensor cores with BF16 operands and
 * FP32 accumulation; state, stage sums and adjoint quadrature stay FP32;
 * t, dt and the controller in FP64. */
typedef enum {
  GBNDE_PREC_FP32 = 0,
  GBNDE_PREC_BF16 = 1
} gbnde_precision;

/* sensealg: InterpolatingAdjoint (default of NeuralODE, src/neural_de.jl:57),
 * BacksolveAdjoint (test/BasicNeuralDE/neural_de_tests.jl:36), or the
 * quadrature adjoints QuadratureAdjoint / GaussAdjoint (re-exported at
 * src/DiffEqFlux.jl:53, used at test/AdvancedNeuralDE/second_order_ode_tests.jl:59):
 * the backward solve carries lam only, and dL/dp = int lam^T df/dp dt is
 * integrated separately, here with 4-point Gauss-Legendre over every accepted
 * adjoint step (lam from that step's interpolant, u from the forward's dense
 * output). The quadrature adjoints run in the FP32 adjoint kernel. */
typedef enum {
  GBNDE_SENSE_INTERPOLATING = 0,
  GBNDE_SENSE_BACKSOLVE = 1,
  GBNDE_SENSE_GAUSS = 2
} gbnde_sensealg;

typedef enum {
  GBNDE_OK = 0,
  GBNDE_ERR_INVALID = -1,      /* bad argument */
  GBNDE_ERR_CUDA = -2,         /* CUDA runtime error */
  GBNDE_ERR_NOMEM = -3,        /* device or pinned allocation failed */
  GBNDE_ERR_UNSUPPORTED = -4,  /* shape or feature outside this build */
  GBNDE_ERR_STATE = -5,        /* call order (e.g. backward before forward) */
  GBNDE_ERR_TIMEOUT = -6       /* a device-side wait gave up (see retcode) */
} gbnde_error;

/* Solver outcome, SciMLBase.ReturnCode names in comments. */
typedef enum {
  GBNDE_RET_SUCCESS = 0,        /* Success */
  GBNDE_RET_MAXITERS = 1,       /* MaxIters */
  GBNDE_RET_DTLESSTHANMIN = 2,  /* DtLessThanMin */
  GBNDE_RET_UNSTABLE = 3,       /* Unstable (non-finite state or error) */
  GBNDE_RET_BARRIER_TIMEOUT = 4 /* device grid barrier gave up; no result */
} gbnde_retcode;

/* Chain([x -> x.^3,] Dense(dims[0], dims[1], act[0]), ..., Dense(dims[n-1], dims[n], act[n-1])) */
typedef struct {
  int nlayers;
  int dims[GBNDE_MAX_LAYERS + 1];
  int act[GBNDE_MAX_LAYERS];
  int cube_input;  /* 1: the chain starts with the WrappedFunction x -> x.^3 */
  int time_input;  /* 1: t is appended as an extra input row (FFJORD extension); dims[0] = S + 1 */
} gbnde_mlp_desc;

/* Keyword surface of solve(prob, Tsit5(); saveat, abstol, reltol, dt, dtmin, maxiters, sensealg) */
typedef struct {
  double t0, t1;          /* tspan */
  double abstol, reltol;
  double dt0;             /* <= 0: automatic initial step */
  double dtmin;           /* <= 0: no minimum */
  long long maxiters;     /* <= 0: 100000 */
  const double* saveat;   /* host array of nsave times inside [t0, t1], increasing from t0 */
  int nsave;              /* >= 1 */
  int sensealg;           /* gbnde_sensealg, used by gbnde_backward */
  int flags;              /* 0, or GBNDE_FLAG_FP32_TIME */
} gbnde_solve_desc;

/* gbnde_solve_desc.flags: FP32 form only. t, the step size, the error
 * estimate and qold are kept as Float32 values (rounded after every update),
 * as the reference's integrator does for a Float32 tspan
 * (src/neural_de.jl:52 builds the ODEProblem from the user's tspan); the
 * forward solve and its adjoint both follow it. Without the flag they are
 * FP64 (the BF16 form always). */
#define GBNDE_FLAG_FP32_TIME 1

typedef struct {
  long long nf;           /* RHS evaluations of the forward solve */
  long long naccept;
  long long nreject;
  long long nf_recompute; /* RHS evaluations of the checkpoint recompute (InterpolatingAdjoint) */
  long long nf_adj;       /* adjoint RHS evaluations (each = forward recompute + VJP) */
  long long naccept_adj;
  long long nreject_adj;
  int retcode;            /* gbnde_retcode of the forward solve */
  int retcode_adj;        /* gbnde_retcode of the adjoint solve */
  double t_final;
  long long nf_adj_vjp;   /* adjoint evaluations that ran the VJP products only, reusing the
                             activations of the previous evaluation at the same t and u(t)
                             (interval starts, and stage 7 of every step) */
  int fwd_path;           /* gbnde_path of the forward solve that ran */
  int adj_path;           /* gbnde_path of the adjoint solve that ran */
} gbnde_stats;

/* Which kernels a solve ran on (gbnde_stats.fwd_path / adj_path). A BF16
 * context runs the tensor-core kernels where they cover the model and the
 * solve; the rest (FFJORD, multiple shooting, the Backsolve and quadrature
 * adjoints, and gradients past the tensor-core adjoint's storage) runs on the
 * plain FP32 kernels, and these fields say so. */
typedef enum {
  GBNDE_PATH_NONE = 0,            /* no solve of this kind ran in the call */
  GBNDE_PATH_FP32 = 1,            /* plain FP32 kernels (adjoint: dense stage storage,
                                     or Backsolve's co-integrated u) */
  GBNDE_PATH_FP32_RECOMPUTE = 2,  /* plain FP32 adjoint, each save interval recomputed
                                     from its checkpoint: O(checkpoints) memory */
  GBNDE_PATH_TC = 3,              /* tensor-core (BF16-form) kernels; adjoint on the
                                     forward's dense stage storage */
  GBNDE_PATH_TC_RECOMPUTE = 4     /* tensor-core adjoint, each save interval recomputed on
                                     the tensor-core forward from its checkpoint */
} gbnde_path;

/* ---- context ------------------------------------------------------------ */
/* Replaces the model/parameter setup that StatefulLuxLayer does per call
 * (src/neural_de.jl:48). precision: gbnde_precision. device: CUDA ordinal. */
int gbnde_create(gbnde_ctx** out, const gbnde_mlp_desc* mlp, int precision, int device);
void gbnde_destroy(gbnde_ctx* ctx);
size_t gbnde_nparams(const gbnde_ctx* ctx);
/* p: the flat ComponentArray(ps) vector (src/neural_de.jl:47 `p`). */
int gbnde_set_params(gbnde_ctx* ctx, const float* p, size_t n);
int gbnde_set_params_device(gbnde_ctx* ctx, const float* p_dev, size_t n);

/* Bound on the device memory of the forward's dense stage storage (u_n, k1..k7
 * per accepted step), which the InterpolatingAdjoint reads. 0 (the default):
 * up to a quarter of the free device memory. When a solve needs more, the
 * adjoint recomputes each save interval from its checkpoint instead (memory
 * O(checkpoints)): the FP32 kernel, or the tensor-core adjoint replaying the
 * interval on the tensor cores (gbnde_stats.adj_path says which). No
 * reference counterpart (InterpolatingAdjoint(checkpointing = true) is the
 * reference's memory switch, src/neural_de.jl:57). */
int gbnde_set_stage_memory(gbnde_ctx* ctx, size_t max_bytes);

/* Upper bound on the CTAs of the tensor-core solver kernels (persistent, one
 * CTA per SM, each CTA looping over its 128-trajectory tiles). 0 (the
 * default): one CTA per SM. Fewer CTAs keep the stash engine's per-CTA
 * operand buffers in L2 at large batches (FFJORD, wide layers). No reference
 * counterpart (a tuning knob of this implementation). */
int gbnde_set_grid_cap(gbnde_ctx* ctx, int max_ctas);

/* ---- NeuralODE forward solve ------------------------------------------------
 * Replaces solve(ODEProblem{false}(dudt, x, tspan, p), Tsit5(); saveat, abstol,
 * reltol, ...) at src/neural_de.jl:52-58. u0: S x B. usave: S x B x nsave.
 * Keeps the checkpoints and step log that gbnde_backward needs. */
int gbnde_forward(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int S, int B,
                  const float* u0, float* usave, gbnde_stats* stats);
int gbnde_forward_device(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int S, int B,
                         const float* u0_dev, float* usave_dev, gbnde_stats* stats);

/* ---- adjoint gradient --------------------------------------------------------
 * Replaces the pullback of SciMLSensitivity's rrule on solve for
 * sensealg = InterpolatingAdjoint()/BacksolveAdjoint() (src/neural_de.jl:57).
 * dL_dusave: S x B x nsave cotangent of the saved states of the last forward.
 * Outputs dL/du0 (S x B) and dL/dp (nparams). */
int gbnde_backward(gbnde_ctx* ctx, const float* dL_dusave, float* dL_du0, float* dL_dp,
                   gbnde_stats* stats);
int gbnde_backward_device(gbnde_ctx* ctx, const float* dL_dusave_dev, float* dL_du0_dev,
                          float* dL_dp_dev, gbnde_stats* stats);

/* ---- FFJORD (continuous normalizing flow) ------------------------------------------
 * Replaces __forward_ffjord (src/ffjord.jl:140-178): solves the augmented
 * system [z; delta_logp] with right-hand side [f(z [, t]); -trace(df/dz)] from
 * (x, 0) over [t0, t1], keeping only the end state (:154-157), and returns
 * logpx = logpz(z(t1)) - delta_logp(t1) for the standard-normal base
 * (:171-176). The model is the context's chain with state dim d (time_input
 * appends t to its input). noise: d x B Hutchinson directions, fixed for the
 * solve (monte_carlo = true), or NULL for the exact trace (monte_carlo =
 * false). FP32 arithmetic in both precisions; desc->saveat is ignored. */
int gbnde_ffjord_forward(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int d, int B, const float* x,
                         const float* noise, float* logpx, float* zT, gbnde_stats* stats);
/* Gradient of a loss of logpx (and optionally of z(t1)) through the
 * InterpolatingAdjoint of the last gbnde_ffjord_forward (sensealg at
 * src/ffjord.jl:143). dL_dzT may be NULL. Outputs dL/dx (d x B) and dL/dp. */
int gbnde_ffjord_backward(gbnde_ctx* ctx, const float* dL_dlogpx, const float* dL_dzT, float* dL_dx,
                          float* dL_dp, gbnde_stats* stats);
/* FFJORD with regularize = true (src/ffjord.jl:131-135, :151-168): the
 * augmented system gains two rows that integrate |f|^2 (the sum of squares
 * of the model's d outputs) and |e^T (df/dz)| (the 2-norm of the
 * vector-Jacobian product along the sample's noise e) from 0; reg_f2 and
 * reg_ej (B each, may be NULL) receive their values at t1 -- the lambda1 and
 * lambda2 the reference returns beside logpx. Both rows enter the step-size
 * control like the reference's. noise (d x B) is required: it is the e of
 * |e^T J| and, unless exact_trace, the Hutchinson direction of the trace.
 * Runs on the FP32 kernels in both precisions (gbnde_stats.fwd_path). */
int gbnde_ffjord_forward_reg(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int d, int B, const float* x,
                             const float* noise, int exact_trace, float* logpx, float* zT, float* reg_f2,
                             float* reg_ej, gbnde_stats* stats);
/* Gradient through the last gbnde_ffjord_forward_reg of a loss of logpx,
 * z(t1) and the two regulariser values (dL_dzT, dL_dreg_f2, dL_dreg_ej may be
 * NULL for zero). Outputs dL/dx (d x B) and dL/dp. */
int gbnde_ffjord_backward_reg(gbnde_ctx* ctx, const float* dL_dlogpx, const float* dL_dzT,
                              const float* dL_dreg_f2, const float* dL_dreg_ej, float* dL_dx, float* dL_dp,
                              gbnde_stats* stats);

/* ---- multiple shooting -------------------------------------------------------------
 * Replaces the per-group solves of multiple_shoot (src/multiple_shooting.jl:52-62):
 * segment i solves from u0[:, i] over [t0, t1] with its own adaptive Tsit5
 * step-size control and saves at saveat[save_off .. save_off + nsave - 1]
 * (times inside [t0, t1], increasing). All segments run in one launch.
 * FP32 arithmetic in both precisions. usave: S x nsave_total (column j = save
 * time j), or NULL to keep the saves on the device only (gbnde_multishoot_loss
 * reads them there; gbnde_multishoot_saves copies them out later). retcodes[i]
 * is segment i's gbnde_retcode (the reference turns any failure into an Inf
 * loss, src/multiple_shooting.jl:66-67). */
typedef struct {
  double t0, t1;
  int save_off;
  int nsave;
} gbnde_segment;

int gbnde_multishoot_forward(gbnde_ctx* ctx, int S, int nseg, const gbnde_segment* segs,
                             const double* saveat, int nsave_total, const float* u0,
                             double abstol, double reltol, long long maxiters, float* usave,
                             int* retcodes, gbnde_stats* stats);
/* Copies the saves (S x nsave_total) of the last gbnde_multishoot_forward to
 * host memory: the group predictions of multiple_shoot
 * (src/multiple_shooting.jl:83-93) when the forward kept them on the device. */
int gbnde_multishoot_saves(gbnde_ctx* ctx, float* usave);
/* The loss of multiple_shoot on the device (src/multiple_shooting.jl:69-81):
 * over the saves of the last gbnde_multishoot_forward,
 *   loss = sum_g lf(data_g, pred_g)
 *        + continuity_term * sum_{g : seg_next[g] >= 0} sum(abs, pred_g[:, end] - data_{seg_next[g]}[:, 1])
 * with loss_function lf = sum of squares (loss_kind 0) or their mean over the
 * group's S x nsave entries (loss_kind 1), and the default continuity loss
 * sum(abs, u_end - u_0) (:243). data: S x nsave_total host array packed like
 * the saves (column j = the data point of save j). seg_next[g]: the segment
 * that continues segment g's trajectory (the next group), or -1 for a
 * trajectory's last group. Keeps dL/dusave on the device for
 * gbnde_multishoot_backward(ctx, NULL, ...). The forward must have succeeded
 * (a failed group makes the reference's loss Inf; the caller reports that). */
int gbnde_multishoot_loss(gbnde_ctx* ctx, const float* data, const int* seg_next, int loss_kind,
                          double continuity_term, double* loss);
/* Gradient of a loss of the saved states of the last multiple-shooting forward:
 * the discrete adjoint of its accepted steps (exact gradient of the computed
 * solution). dL_dusave: S x nsave_total host cotangent, or NULL for the one
 * gbnde_multishoot_loss left on the device. Outputs dL/du0 (S x nseg; may be
 * NULL) and dL/dp. */
int gbnde_multishoot_backward(gbnde_ctx* ctx, const float* dL_dusave, float* dL_du0,
                              float* dL_dp, gbnde_stats* stats);

/* ---- fused loss at the save points (device pointers) -------------------------
 * kind 0: sum(abs2, target .- usave) (docs/src/examples/neural_ode.md:41);
 * kind 1: mean(abs2, ...). Writes dL/dusave and the loss (FP64, host). */
int gbnde_loss_device(gbnde_ctx* ctx, const float* usave_dev, const float* target_dev,
                      int kind, float* dL_dusave_dev, double* loss);

/* ---- one training iteration (Adam) ------------------------------------------------
 * One iteration of the reference's training loop (Optimization.solve with
 * OptimizationOptimisers.Adam around the loss, docs/src/examples/neural_ode.md:66-70)
 * on device buffers: forward solve from u0_dev, the fused save-point loss
 * against target_dev (loss_kind 0: sum of squares, 1: mean), the adjoint
 * gradient, then Adam on the parameters in p_dev (nparams floats, updated in
 * place and loaded into the context for the next solve). m_dev and v_dev are
 * the Adam moments (zero before the first step); step is the 1-based
 * iteration count used for the bias corrections:
 *   m = b1 m + (1 - b1) g;  v = b2 v + (1 - b2) g^2;
 *   p -= lr (m / (1 - b1^step)) / (sqrt(v / (1 - b2^step)) + eps).
 * All launches are on the context's stream; the host reads the forward's step
 * log to plan the adjoint intervals (gbnde_graph_train_step moves that plan
 * to the device and replays the whole iteration as one CUDA graph). */
typedef struct {
  double lr, beta1, beta2, eps;
} gbnde_adam;

int gbnde_train_step(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int S, int B, const float* u0_dev,
                     const float* target_dev, int loss_kind, const gbnde_adam* opt, long long step,
                     float* p_dev, float* m_dev, float* v_dev, double* loss, gbnde_stats* stats);

/* The same iteration replayed as one CUDA graph. The first call (and any call
 * whose arguments or buffers differ from the captured ones) runs
 * gbnde_train_step eagerly while recording its launches, then captures
 * parameter upload, forward, loss, an on-device plan of the adjoint
 * intervals, adjoint, reduction and Adam into a graph; later calls launch
 * that graph and read back only the loss and the solver counters. A replay
 * whose solve failed or outgrew the stage storage updates nothing on the
 * device and is redone eagerly. *graphed (may be NULL) is set to 1 when the
 * step ran as a graph replay. Needs an adjoint that reads the dense stage
 * storage (InterpolatingAdjoint, not FFJORD); otherwise every step runs
 * eagerly. After a replay the context holds no forward solve for
 * gbnde_backward. Buffers must stay allocated while the graph is in use. */
int gbnde_graph_train_step(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int S, int B, const float* u0_dev,
                           const float* target_dev, int loss_kind, const gbnde_adam* opt, long long step,
                           float* p_dev, float* m_dev, float* v_dev, double* loss, gbnde_stats* stats,
                           int* graphed);

/* ---- fused loss without any device allocation ----------------------------------
 * No counterpart in the reference. Same loss and cotangent as
 * gbnde_loss_device (kind 0: sum of squared errors, kind 1: their mean) on n
 * floats of caller-owned device memory, for callers that must not allocate:
 * real-time loops that cannot take the device-wide synchronisation of
 * cudaMalloc/cudaFree, and hosts whose own pool owns every device byte. It
 * needs no context: its scratch is a 32 KB array compiled into the library
 * (held on every device that loads it, until the process exits).
 * n <= GBNDE_LOSS_NOALLOC_MAX_N, else GBNDE_ERR_UNSUPPORTED. The first call on a
 * device looks up the scratch address for that device; make that first call
 * before any stream capture. All calls on a device share the scratch: calls
 * whose kernels overlap on the GPU (other streams or host threads) race and
 * may return wrong losses. stream: a cudaStream_t, or NULL for the default
 * stream. The call synchronises that stream and returns after the loss is on
 * the host, so it is made from ordinary host code, never from a stream
 * callback (a host function enqueued with cudaLaunchHostFunc may make no CUDA
 * calls). */
#define GBNDE_LOSS_NOALLOC_MAX_N (4096LL * 65536LL)
int gbnde_loss_noalloc(const float* usave_dev, const float* target_dev, size_t n, int kind,
                       float* dL_dusave_dev, double* loss, void* stream);

/* Accepted steps (t_n, h_n) of the last forward solve; returns the count
 * (may exceed cap; only cap entries are written). */
long long gbnde_forward_steps(gbnde_ctx* ctx, double* t, double* h, long long cap);

/* Attempted steps of the last forward solve, 4 doubles each: t_n, h_n, the
 * error estimate EEst and 1.0 if accepted (the step trace the integrator's
 * controller acted on). Returns the count (only cap entries are written). */
long long gbnde_forward_trace(gbnde_ctx* ctx, double* out4, long long cap);

/* The CUDA stream (cudaStream_t) the context launches on, and a way to use
 * the caller's stream instead (e.g. CUDA.jl's task stream); NULL restores the
 * context's own stream. No reference counterpart (stream plumbing of the host).
 * The context's own stream is destroyed with the context: a host whose
 * allocator keeps per-stream records (torch's pinned-memory allocator records
 * events on every stream a block was used on, also when the block is freed)
 * should hand its own stream to gbnde_set_stream rather than use this one. */
void* gbnde_stream(gbnde_ctx* ctx);
int gbnde_set_stream(gbnde_ctx* ctx, void* stream);

/* Durations (ms, CUDA events on the launching stream) of the last forward and
 * backward solver kernels. No reference counterpart (instrumentation). */
int gbnde_last_kernel_ms(gbnde_ctx* ctx, double* fwd_ms, double* bwd_ms);

/* Autotuner. Times the FP32 form's forward and adjoint kernels on (S, B, u0)
 * at every rows-per-tile choice that fits shared memory (8, 16, 32, 64
 * trajectories per tile) and keeps the fastest of each for this (S, B) in
 * the context; later solves of that shape use them. The cotangent of the
 * timed adjoint is that of the mean square of the saved states. tiles[0] and
 * tiles[1] receive the forward and adjoint choices. The BF16 form runs
 * 128-trajectory tiles, one CTA per SM; there it times the two tensor-core
 * engines where both cover the model (single-accumulator: state <= 64,
 * widths <= 256; stash: state <= 256, widths <= 1024) on a forward solve and
 * its adjoint, keeps the faster for this (S, B), and returns tiles[0] = 128,
 * tiles[1] = the engine (0 single-accumulator, 1 stash).
 * Clobbers the last forward solve (run forward again before a backward).
 * No reference counterpart (the reference's tile sizes are chosen by its
 * array library). */
int gbnde_autotune(gbnde_ctx* ctx, const gbnde_solve_desc* desc, int S, int B,
                   const float* u0_dev, int* tiles);

/* Self-test of the bounded waits (failure detection without a fault): two
 * CTAs meet at the solvers' grid barrier; with absent = 0 or 1 that CTA never
 * arrives and the other gives up after limit_ms (<= 1000), as a solve does
 * after its barrier limit (then retcode BarrierTimeout). absent = -1: both
 * arrive. timed_out: 1 when the wait ran out; waited_ms: how long it waited.
 * No reference counterpart (test support). */
int gbnde_barrier_selftest(int absent, double limit_ms, int* timed_out, double* waited_ms);

/* Self-test of the tensor-core building blocks on the current device:
 * D[128 x N] = A[128 x K] * W[N x K]^T (host arrays, row-major) through bulk
 * copied SW128 weight images, tcgen05.mma into tensor memory and tcgen05.ld.
 * mode 0: one BF16 product; mode 1: the five split-BF16 products of the BF16
 * form. N in {64, 128, 256}, K <= 1024. mode 2: the MN-major weight-gradient
 * form, D = A^T W with A of K x 128 and W of K x N (K = 128), three products.
 * No reference counterpart (diagnostic). */
int gbnde_tc_selftest(const float* A, const float* W, int N, int K, int mode, float* D);

/* Self-test of the activation the tensor-core epilogues evaluate (a tanh
 * built from its Maclaurin series and the exponential identity on the
 * ex2/rcp instructions) beside the library functions the plain FP32 form
 * uses, on n host inputs: y_tc = epilogue activation, y_lib = library
 * activation. act: gbnde_act. No reference counterpart (diagnostic). */
int gbnde_act_selftest(const float* x, int n, int act, float* y_tc, float* y_lib);

const char* gbnde_strerror(int code);
const char* gbnde_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GBNDE_H */
