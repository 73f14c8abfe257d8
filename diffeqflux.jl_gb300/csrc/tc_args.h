// tc_args.h -- launch descriptors of the tensor-core (BF16-form) solver kernels,
// shared by the kernels and the host API.
#pragma once
#include "tc_engine.cuh"

namespace gbnde {

struct FwdTcArgs {
  FwdArgs f;
  tc::OpList ops;
  const float* bias[GBNDE_MAX_LAYERS];
  float* comp[2];       // compensation of the state (ping-pong with ubuf)
  float* dense;         // slots of 8 x S*B floats: u_n, k1..k7 (or null)
  long long dense_slots;
  float* kring;         // 7 x S*B stage buffers when dense == null
  float* ckcomp;        // the state's compensation at each checkpoint (tile layout), or null
};


struct BwdTcArgs {
  BwdArgs b;
  tc::OpList ops;               // one adjoint evaluation: forward recompute + VJP chain
  tc::OpList dwops;             // one accepted step: stage-stacked weight-gradient ops
  tc::OpList ops7;              // an evaluation whose activations are re-emitted (copy-only forward ops)
  int dw_chunks;                // K chunks of all dwops (A-ring slots the producer fills)
  float* pbias;                 // [grid][3][4][nbias] pending bias quadrature: stage 1, 2..6, 7 (x 4 row groups)
  const float* bias[GBNDE_MAX_LAYERS];
  float* lam_comp[2];           // compensation of lam
  float* mu_comp;               // [grid][P] Kahan compensation of mu_acc
  float* hscr;                  // per CTA hvals/4 float4 slots x 256 threads (slot-major, so a
                                //   warp's accesses to one slot are contiguous), fp32 activations
  int hvals;                    // values per thread in hscr
  int hoff[GBNDE_MAX_LAYERS];   // offset of hidden layer l (1..L-1) inside a thread's hscr
  int hx;                       // offset of the 32 state values kept for the cube prefix
  int hoff2[GBNDE_MAX_LAYERS];  // FFJORD (stash mode): offset of the tangent pre-activations pdot_l
  uint8_t* img;                 // [grid][tpc][kImgSlots][img_cta] weight-gradient operand images
  size_t img_cta;               // bytes of one stage's images
  int tpc;                      // 128-trajectory tiles per CTA (image sets per CTA)
  long long aoff[GBNDE_MAX_LAYERS];  // image offset of a_l (l = 0..L-1)
  long long doff[GBNDE_MAX_LAYERS];  // image offset of delta_{l+1} (l = 0..L-1)
  int a_isA[GBNDE_MAX_LAYERS];       // 1: a_l is the A operand (rows = in) of layer l's dW
  int nh[GBNDE_MAX_LAYERS];          // M halves (128 rows) of layer l's dW
  int nbias;
  int boffp[GBNDE_MAX_LAYERS];  // offset of layer l's bias inside a pending-bias row
  // O(checkpoints) mode (b.dense == null): each save interval's forward steps
  // are replayed on the tensor cores (fwops, CMD_FWD) from the checkpoint
  // (b.ckpt: u, API layout; ckcomp: its compensation, tile layout) into the
  // interval buffer b.ibuf (slot j = step nlo + j: u_n, k1..k7, tile layout)
  tc::OpList fwops;
  const float* ckcomp;
  float* rep[2];                // replayed state and its compensation (tile layout)
  float* xst;                   // [6][ntiles * kTileVec] u(t) at the six stage times of the
                                //   current adjoint step (tile layout)
};


int launch_bwd_tc(const BwdTcArgs& a, int grid, cudaStream_t st);

// Stash-mode forward (fwd_tcw.cu): state up to 256 (nsc 64-component chunks),
// widths up to 1024, optional time row. The ops are N-block ops of kind 3.
struct FwdTcwArgs {
  FwdTcArgs t;
  uint8_t* stash;  // [grid][kStashBufs][kStashChunks][kASlotBytes]
  int nsc;         // 64-component chunks of the state
  // FFJORD mode (t.f.ffj): the tangent chain's activation scratch (hvals
  // floats per epilogue thread, slot-major) and the trace partials [grid][512]
  float* hscr;
  int hvals;
  float* trs;
};
int launch_fwd_tcw(const FwdTcwArgs& a, int grid, cudaStream_t st);

// Stash-mode adjoint (bwd_tcw.cu): the BwdTcArgs op lists hold N-block ops
// (kind 3 chain, kind 4 copy-only, kind 1 weight gradients with B blocks).
struct BwdTcwArgs {
  BwdTcArgs t;
  uint8_t* stash;
  int nsc;
  float* trs;  // FFJORD mode: per-CTA scratch of 512 floats (row broadcasts)
};
int launch_bwd_tcw(const BwdTcwArgs& a, int grid, cudaStream_t st);

// 0 if `kernel` was compiled with exactly tc::kLaunchRegs registers per
// thread, the count the warpgroup register split is sized for; -1 otherwise
// (the kernel must then not be launched: its register split would wait for
// registers that the launch never had).
int tc_check_regs(const void* kernel);
int launch_reduce_mu_comp(const float* acc, const float* comp, int nblk, int stride, int P, float* out,
                          cudaStream_t st);

}  // namespace gbnde
