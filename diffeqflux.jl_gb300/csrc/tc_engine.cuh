// tc_engine.cuh -- the tensor-core MLP engine shared by the BF16-form solver
// kernels.
//
// A CTA evaluates GEMM "ops" on a tile of 128 trajectories. An op is
//   D[128 x N] (tensor memory, FP32) = sum over K chunks of the five split
//   products  A_hi W_hi + A_mid W_hi + A_hi W_lo + A_lo W_hi + A_mid W_lo
// where A chunks (128 rows x 64 columns, 3 bf16 pieces) are written into a
// shared-memory ring by the epilogue warps and W chunks (N rows x 64, 2 bf16
// pieces, pre-swizzled image in global memory) are streamed by a producer
// warp with bulk copies. Ops alternate between two 256-column accumulator
// regions so that the epilogue can drain one while the next op accumulates.
//
// Warp roles: kNWG epilogue warpgroups (warps 0 .. 4 kNWG - 1), then one
// control warpgroup: the MMA issuer, the weight producer and two idle warps.
// Epilogue warp w serves the 32 accumulator rows (tensor-memory lanes) of
// w % 4 and column group w / 4 (kCW columns of every 64-column chunk). The
// MMA and producer warps run the op list cyclically until the epilogue
// raises the stop flag. The kernel is launched with kLaunchRegs registers
// per thread; the control warpgroup then gives registers back
// (setmaxnreg.dec to kCtlRegs) and the epilogue warpgroups take them
// (setmaxnreg.inc to kEpiRegs): kEpiThreads * kEpiRegs + 128 * kCtlRegs ==
// kThreads * kLaunchRegs, checked at compile time here and against the
// compiled kernel's register count before every launch (a split above the
// launch's registers would never complete).
#pragma once
#include "kernels.h"
#include "tc_ptx.cuh"

namespace gbnde {
namespace tc {

// Four epilogue warpgroups (16 columns per thread) hide more of the
// epilogue's memory and tensor-memory latency than two (32 columns per
// thread, more registers each): the adjoint kernel runs 6.7 % faster at
// B = 16384, 64-256-256-64, and the forward within 1 %.
#ifndef GBNDE_TC_NWG
#define GBNDE_TC_NWG 4
#endif
constexpr int kNWG = GBNDE_TC_NWG;   // epilogue warpgroups: 2 or 4
static_assert(kNWG == 2 || kNWG == 4, "two or four epilogue warpgroups");
constexpr int kCW = 64 / kNWG;       // columns of each 64-column chunk per epilogue thread
constexpr int kEpiThreads = 128 * kNWG;
constexpr int kEpiWarps = kEpiThreads / 32;  // arrivals of the epilogue on a barrier: one per warp
constexpr int kThreads = kEpiThreads + 128;
constexpr int kMmaWarp = 4 * kNWG;
constexpr int kTmaWarp = kMmaWarp + 1;
// Launch registers: 65536 / kThreads, rounded down to a multiple of 8 and
// within one scheduler's 16384 registers for its share of the warps
// (kThreads / 128 warps each); then the split.
constexpr int kLaunchRegs = kNWG == 2 ? 168 : 96;
#ifndef GBNDE_TC_EPI_REGS
#define GBNDE_TC_EPI_REGS (GBNDE_TC_NWG == 2 ? 224 : 104)
#endif
#ifndef GBNDE_TC_CTL_REGS
#define GBNDE_TC_CTL_REGS (GBNDE_TC_NWG == 2 ? 56 : 64)
#endif
constexpr int kEpiRegs = GBNDE_TC_EPI_REGS;
constexpr int kCtlRegs = GBNDE_TC_CTL_REGS;
static_assert(kEpiThreads * kEpiRegs + (kThreads - kEpiThreads) * kCtlRegs == kThreads * kLaunchRegs,
              "register split must equal the launch's registers");
static_assert(kThreads * kLaunchRegs <= 65536, "launch registers exceed the register file");
constexpr int kASlotBytes = 3 * 16384;   // 3 pieces x 128 rows x 128 B
constexpr int kWSlotBytes = 2 * 32768;   // 2 pieces x 256 rows x 128 B
constexpr int kARing = 2;
constexpr int kWRing = 2;
constexpr int kSmemBytes = 1024 + kARing * kASlotBytes + kWRing * kWSlotBytes;
constexpr int kMaxOps = 64;
constexpr int kCmdRing = 4;
constexpr int kImgSlots = 7;    // weight-gradient image slots per CTA: stages 1..6 + the next stage 1
// Split pieces kept in the weight-gradient images, and the products of a
// weight-gradient op: 1 (hi, one BF16 product) or 2 (hi and mid; hi.hi +
// hi.lo + lo.hi). One piece makes the adjoint 10 % faster at B = 16384,
// 64-256-256-64, but its parameter gradients differ from the FP64 oracle by
// 1.1e-3 to 3e-3 (relative norm) on batches of 130 to 1000 trajectories,
// above the 1e-3 bar; two pieces stay below it on every shape. The chain
// GEMMs keep five products (three make the forward take 23 steps instead of 12).
constexpr int kImgPieces = 2;
// Stash mode (layers wider than one 256-column accumulator): every chain A
// operand goes through a per-CTA global "stash" of two buffers of up to
// kStashChunks K-chunks (ring-slot layout: 3 pieces x 128 rows x 128 B each),
// written by the epilogue with plain stores and bulk-loaded by the producer.
constexpr int kStashChunks = 16;                                   // K <= 1024
constexpr int kStashBufs = 4;  // two per chain: the primal chain and (FFJORD) the tangent chain
constexpr size_t kStashCta = (size_t)kStashBufs * kStashChunks * kASlotBytes;  // bytes per CTA

// kind 0 (chain GEMM): A chunks written by the epilogue (3 pieces, K-major),
//   B = weight image chunks (2 pieces, K-major), five split products.
// kind 1 (weight-gradient GEMM, K = trajectories): A and B both bulk-copied
//   from per-CTA images (kImgPieces pieces, MN-major 64-column blocks):
//   hi.hi, or hi.hi + hi.lo + lo.hi with two pieces.
// kind 2 (copy only, command mode): epilogue-written A chunks that only go to
//   their weight-gradient image; no product, no accumulator, no W chunk.
// kind 3 (stash chain GEMM): as kind 0, but the A chunks are bulk-loaded by
//   the producer from stash buffer `sbuf` (once the epilogue has marked each
//   chunk written), so one layer's input can feed several N-block ops.
// kind 4 (stash copy only): stash A chunks loaded into the ring only to be
//   copied to their weight-gradient image; no product.
struct GemmOp {
  const uint8_t* wimg;  // kind 0: weight image; kind 1: B image base of CTA 0
  const uint8_t* aimg;  // kind 1: A image base of CTA 0
  size_t cta_stride;    // kind 1: bytes between consecutive CTAs' images
  uint32_t a_bytes;     // kind 1: bytes of one A chunk
  uint32_t a_step;      // kind 1: bytes between consecutive A chunks
  uint32_t b_step;      // kind 1: bytes between consecutive B chunks
  int npad;             // N rounded up to 16 (<= 256)
  int nchunk;           // K / 64 (rounded up)
  int kind;
  int nblk_b;           // kind 1: 64-column blocks in a B chunk
  int first_dw;         // kind 1: first weight-gradient op of an evaluation (waits for images)
  size_t slot_stride;   // kind 1: bytes between the image slots of consecutive stages
  // kind 0 in command mode: the A chunks are also the weight-gradient image
  // of this operand (first two split pieces), bulk-copied by the MMA warp to
  // the stage's image slot at byte offset img_off (< 0: no image). Layout:
  // img_isA (rows = M-side features, img_nh 128-row halves) or img_nblk
  // 64-feature blocks.
  int img_off;
  uint8_t img_isA, img_nblk;
  uint16_t img_nh;
  // kind 3 / 4: stash buffer of the A operand, and whether this op is the
  // first reader of that buffer's current contents (the producer then moves
  // to the buffer's next fill); aimg = stash base of CTA 0 for this buffer,
  // cta_stride = bytes between CTAs' stashes
  int sbuf;
  int first_nb;
  // kind 1 with the B side split in N-blocks: B chunk = 2 pieces of nblk_b
  // blocks each, starting b_off0 bytes into each piece, pieces b_pstride
  // bytes apart (b_pstride == 0: one contiguous copy)
  uint32_t b_off0, b_pstride;
  // kind 1: operand pairs stacked along K per stage (FFJORD: (pbar, a) and
  // (pdotbar, adot)); pair q's images sit q * pair_aoff / q * pair_boff
  // bytes after pair 0's in the stage slot (npairs 0 or 1: one pair)
  int npairs;
  uint32_t pair_aoff, pair_boff;
  // kind 0 / 3: split products issued: 0 (all five) or 3 (A_hi W_hi +
  // A_mid W_hi + A_hi W_lo, about 16 bits of both operands)
  int nprod;
  // kind 1: pieces per image chunk (0: kImgPieces, BF16 copies of the chain
  // chunks) and whether the images are FP16 (one piece, written by the
  // epilogue: one FP16 product)
  int img_pieces;
  int img_f16;
};

struct OpList {
  GemmOp op[kMaxOps];
  int nops;
};

struct Shared {
  uint64_t a_full[kARing], a_empty[kARing];
  uint64_t w_full[kWRing], w_empty[kWRing];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t img_ready;
  uint64_t img_done;  // command mode: the MMA warp's image copies of the step have landed
  uint64_t cmd_full[kCmdRing], cmd_empty[kCmdRing];
  uint64_t stash_full[kStashBufs][kStashChunks];  // stash mode: chunk written by all epilogue warps
  uint32_t cmd[kCmdRing];
  uint32_t tmem_base;
  int stop;
  int err;
  double red[24];  // [0, 16): per-warp sums; 16..: broadcasts
};

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory"); }

// Register split between the warpgroups (all four warps of a warpgroup
// execute the same instruction).
__device__ __forceinline__ void regs_take_epi() {
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kEpiRegs));
}
__device__ __forceinline__ void regs_give_ctl() {
  asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kCtlRegs));
}

// Deterministic sum of a double over the epilogue threads.
__device__ __forceinline__ double epi_sum(double v, Shared& sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  epi_bar();
  if ((threadIdx.x & 31) == 0) sh.red[w] = v;
  epi_bar();
  double s = 0.0;
  for (int i = 0; i < kEpiThreads / 32; ++i) s += sh.red[i];
  epi_bar();
  return s;
}

// Sum of one float per epilogue thread, valid in epilogue thread 0 only:
// FP32 within each warp (fixed shuffle order), FP64 over the warps.
__device__ __forceinline__ double epi_sum0_f(float v, Shared& sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) sh.red[w] = (double)v;
  epi_bar();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kEpiThreads / 32; ++i) s += sh.red[i];
  epi_bar();  // sh.red is reused by the next sum
  return s;
}

// Sum of the grid's n per-CTA partials (FP64, in a fixed order), valid in
// epilogue thread 0 only: warp 0 reads them.
__device__ __forceinline__ double epi_partials_sum0(const double* p, int n) {
  double v = 0.0;
  if (threadIdx.x < 32) {
    for (int i = threadIdx.x; i < n; i += 32) v += __ldcg(p + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}

__device__ __forceinline__ void init_shared(Shared& sh) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < kARing; ++i) {
      mbar_init(&sh.a_full[i], kEpiWarps);
      mbar_init(&sh.a_empty[i], 1);
    }
    for (int i = 0; i < kWRing; ++i) {
      mbar_init(&sh.w_full[i], 1);
      mbar_init(&sh.w_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&sh.acc_full[i], 1);
      mbar_init(&sh.acc_empty[i], kEpiWarps);
    }
    mbar_init(&sh.img_ready, kEpiWarps);
    mbar_init(&sh.img_done, 1);
    for (int i = 0; i < kCmdRing; ++i) {
      mbar_init(&sh.cmd_full[i], 1);
      mbar_init(&sh.cmd_empty[i], 2);
    }
    for (int b = 0; b < kStashBufs; ++b)
      for (int i = 0; i < kStashChunks; ++i) mbar_init(&sh.stash_full[b][i], kEpiWarps);
    sh.stop = 0;
    sh.err = 0;
    fence_mbar_init();
  }
}

// ---- tile layout of the solvers' internal state vectors ---------------------------
// The 64 components of a row are two halves of 8 float4 groups each, with
// the rows innermost: tile T, half h, group j, row r at float
// ((T * 2 + h) * 8 + j) * 512 + 4 r. The epilogue thread of row r and column
// group g owns the kCW components from kCW g: kCW / 4 consecutive groups.
// A warp (32 consecutive rows) reading group j touches 512 contiguous bytes,
// where the column-major API layout would touch 32 separate lines. One vector
// holds ntiles * kTileVec floats (components padded to 64, pads kept zero).
constexpr int kTileVec = 128 * 64;
// Offset of the first of the kCW components of column group g, row r.
__device__ __forceinline__ size_t tl_offset_cw(int tile, int g, int r) {
  const int c0 = kCW * g;
  return (size_t)(tile * 2 + (c0 >> 5)) * 4096 + (size_t)((c0 & 31) >> 2) * 512 + (size_t)r * 4;
}
// the kCW components of a thread (kCW / 4 groups)
__device__ __forceinline__ void tl_ldv(const float* p, float* x) {
#pragma unroll
  for (int j = 0; j < kCW / 4; ++j) {
    const float4 q = *reinterpret_cast<const float4*>(p + j * 512);
    x[4 * j] = q.x; x[4 * j + 1] = q.y; x[4 * j + 2] = q.z; x[4 * j + 3] = q.w;
  }
}
__device__ __forceinline__ void tl_stv(float* p, const float* x) {
#pragma unroll
  for (int j = 0; j < kCW / 4; ++j)
    *reinterpret_cast<float4*>(p + j * 512) = make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
}
// Part `part` (0 or 1) of the same: components kPart part .. kPart part + kPart - 1.
constexpr int kPart = kCW / 2;
__device__ __forceinline__ void tl_ldp(const float* p, int part, float* x) {
#pragma unroll
  for (int j = 0; j < kPart / 4; ++j) {
    const float4 q = *reinterpret_cast<const float4*>(p + (part * (kPart / 4) + j) * 512);
    x[4 * j] = q.x; x[4 * j + 1] = q.y; x[4 * j + 2] = q.z; x[4 * j + 3] = q.w;
  }
}
__device__ __forceinline__ void tl_stp(float* p, int part, const float* x) {
#pragma unroll
  for (int j = 0; j < kPart / 4; ++j)
    *reinterpret_cast<float4*>(p + (part * (kPart / 4) + j) * 512) =
        make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
}
// ---- command ring (command mode) -------------------------------------------------
// In command mode the epilogue decides, round by round, which op list the MMA
// and producer warps run next: CMD_EVAL (the evaluation list, once; bits 8-15
// carry the image slot + 1, bits 16-23 the first op to run, so that an
// evaluation can skip a prefix of the list, bits 24-31 the CTA's tile index,
// whose image set the copies go to) or CMD_DW (the weight-gradient list,
// once; bits 8-15 carry the image slot of stage 1).
// Thread 0 of the epilogue posts; the MMA and producer leaders both release
// the slot.
// CMD_EVAL_RE runs the re-emission list instead of the evaluation list: the
// forward ops are copy-only (the epilogue re-emits stored activations, whose
// chunks only go to their images), the VJP ops are the same.
// CMD_FWD runs the forward list (the plain right-hand side, no images): the
// adjoint's replay of a save interval's forward steps from its checkpoint.
enum : uint32_t { CMD_EVAL = 1, CMD_DW = 2, CMD_EVAL_RE = 3, CMD_FWD = 4 };

// Image slot of stacked stage s (0-based) when stage 1 lives in slot f.
__device__ __forceinline__ int stage_slot(int s, int f) { return s == 0 ? f : s; }

// ---- MMA warp ------------------------------------------------------------------------
struct MmaState {
  int aslot = 0, wslot = 0;
  uint32_t aph = 0, wph = 0;
  uint32_t use[2] = {0, 0};
  long long g = 0;
};

// Bulk copies of A chunk c (its first kImgPieces split pieces, rows 0-63 and
// 64-127) of a chain op to its weight-gradient image (same SW128 arrangement
// as the image's 8 KB blocks). Issued by the elected lane. Image layout, per
// 64-trajectory block kc: M side (img_isA) [kc][128-row half][piece][16 KB],
// N side [kc][piece][64-feature block][8 KB].
__device__ __forceinline__ void copy_a_image(const GemmOp& op, int c, const uint8_t* achunk, uint8_t* img_base) {
  const uint64_t pol = policy_evict_first();  // read once, at the step's commit
  uint8_t* dst0 = img_base + op.img_off;
#pragma unroll
  for (int p = 0; p < kImgPieces; ++p) {
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
      const size_t o = op.img_isA
                           ? ((size_t)((kc * op.img_nh + (c >> 1)) * kImgPieces + p)) * 16384 + (size_t)(c & 1) * 8192
                           : ((size_t)((kc * kImgPieces + p) * op.img_nblk + c)) * 8192;
      bulk_s2g(dst0 + o, achunk + p * 16384 + kc * 8192, 8192, pol);
    }
  }
  bulk_commit();
}

// One op: waits for its accumulator region, then for every K chunk for the A
// chunk and the W chunk, and issues the products (and, with img_base, the
// image copies of the A chunks, which must have read the slot before it is
// released). Returns false when the loop must end (stop flag, error or wait
// limit).
__device__ __forceinline__ bool mma_op(const GemmOp& op, MmaState& m, Shared& sh, uint8_t* aring,
                                       uint8_t* wring, uint8_t* img_base = nullptr) {
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  const bool leader = (threadIdx.x & 31) == 0;
  if (op.kind == 2 || op.kind == 4) {
    for (int c = 0; c < op.nchunk; ++c) {
      unsigned long long t0 = 0;
      while (!mbar_try_wait(&sh.a_full[m.aslot], m.aph)) {
        if (*vstop || *verr) return false;
        if (t0 == 0) t0 = globaltimer_ns();
        else if (globaltimer_ns() - t0 > 4 * kWaitTimeoutNs) { *verr = 2; return false; }
      }
      if (leader) {
        if (img_base != nullptr && op.img_off >= 0) {
          copy_a_image(op, c, aring + m.aslot * kASlotBytes, img_base);
          bulk_wait_read_all();
        }
        mbar_arrive(&sh.a_empty[m.aslot]);
      }
      __syncwarp();
      if (++m.aslot == kARing) { m.aslot = 0; m.aph ^= 1; }
    }
    return true;
  }
  const int pa[5] = {0, 1, 0, 2, 1};
  const int pb[5] = {0, 0, 1, 0, 1};
  const int reg = (int)(m.g & 1);
  {
    const uint32_t par = (m.use[reg] & 1) ^ 1;
    while (!mbar_try_wait(&sh.acc_empty[reg], par)) {
      if (*vstop || *verr) return false;
    }
  }
  const uint32_t d = sh.tmem_base + (uint32_t)(reg * 256);
  const bool chain = op.kind == 0 || op.kind == 3;  // K-major chain GEMM (five split products)
  const uint32_t idesc = chain ? idesc_bf16(128, op.npad)
                               : (op.img_f16 ? idesc_f16_mn(128, op.npad) : idesc_bf16_mn(128, op.npad));
  const int wg_products = (op.img_pieces ? op.img_pieces : kImgPieces) == 2 ? 3 : 1;
  const uint32_t wpiece = chain ? (uint32_t)op.npad * 128 : (uint32_t)op.nblk_b * 8192;
  for (int c = 0; c < op.nchunk; ++c) {
    // A chunk ready? (bounded by the stop flag: the epilogue may be done)
    {
      unsigned long long t0 = 0;
      while (!mbar_try_wait(&sh.a_full[m.aslot], m.aph)) {
        if (*vstop || *verr) return false;
        if (t0 == 0) t0 = globaltimer_ns();
        else if (globaltimer_ns() - t0 > 4 * kWaitTimeoutNs) { *verr = 2; return false; }
      }
    }
    if (!mbar_wait(&sh.w_full[m.wslot], m.wph, verr)) return false;
    tc_fence_after();
    if (leader) {
      const uint32_t a0 = smem_u32(aring + m.aslot * kASlotBytes);
      const uint32_t b0 = smem_u32(wring + m.wslot * kWSlotBytes);
      const bool copy = chain && img_base != nullptr && op.img_off >= 0;
      if (copy) copy_a_image(op, c, aring + m.aslot * kASlotBytes, img_base);
      if (chain) {
        const int np = op.nprod == 3 ? 3 : 5;
#pragma unroll
        for (int pr = 0; pr < 5; ++pr) {
          if (pr >= np) break;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = sdesc_sw128(a0 + pa[pr] * 16384 + kk * 32);
            const uint64_t bd = sdesc_sw128(b0 + pb[pr] * wpiece + kk * 32);
            mma_bf16(d, ad, bd, idesc, (c > 0 || pr > 0 || kk > 0) ? 1u : 0u);
          }
        }
      } else {
        // A chunk: kImgPieces x 2 blocks x 8 KB; B chunk: kImgPieces x nblk x
        // 8 KB. Products hi.hi (and hi.lo, lo.hi with two pieces); K step of
        // 16 trajectories = 2048 bytes.
#pragma unroll
        for (int pr = 0; pr < 3; ++pr) {
          if (pr >= wg_products) break;
          const int qa = (pr == 2) ? 1 : 0, qb = (pr == 1) ? 1 : 0;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = sdesc_sw128_mn(a0 + qa * 16384 + kk * 2048, 8192);
            const uint64_t bd = sdesc_sw128_mn(b0 + qb * wpiece + kk * 2048, 8192);
            mma_bf16(d, ad, bd, idesc, (c > 0 || pr > 0 || kk > 0) ? 1u : 0u);
          }
        }
      }
      if (copy) bulk_wait_read_all();
      mma_commit(&sh.a_empty[m.aslot]);
      mma_commit(&sh.w_empty[m.wslot]);
      if (c == op.nchunk - 1) mma_commit(&sh.acc_full[reg]);
    }
    __syncwarp();
    if (++m.aslot == kARing) { m.aslot = 0; m.aph ^= 1; }
    if (++m.wslot == kWRing) { m.wslot = 0; m.wph ^= 1; }
  }
  m.use[reg] += 1;
  ++m.g;
  return true;
}

// Cyclic mode: runs the op list over and over until the stop flag is raised
// (or a wait gives up, which also raises sh.err).
__device__ __forceinline__ void mma_loop(const OpList& ops, Shared& sh, uint8_t* aring, uint8_t* wring) {
  MmaState m;
  while (mma_op(ops.op[m.g % ops.nops], m, sh, aring, wring)) {
  }
}

// Waits for the next command of the ring; false when the loop must end.
__device__ __forceinline__ bool cmd_take(Shared& sh, int& cs, uint32_t& cph, uint32_t* cmd) {
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  while (!mbar_try_wait(&sh.cmd_full[cs], cph)) {
    if (*vstop || *verr) return false;
  }
  *cmd = ((volatile uint32_t*)sh.cmd)[cs];
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(&sh.cmd_empty[cs]);
  if (++cs == kCmdRing) { cs = 0; cph ^= 1; }
  return true;
}

// Command mode: one op list per command. CMD_EVAL carries slot + 1 in bits
// 8-15 (0: no images) and the first op in bits 16-23; `imgs` is this CTA's
// image region, `img_cta` the bytes
// of one slot. Before a CMD_DW round the image copies must have landed: the
// elected lane waits for its bulk groups and signals the producer.
__device__ __forceinline__ void mma_loop_cmd(const OpList& ev, const OpList& dw, const OpList& ev_re,
                                             const OpList& fw, Shared& sh, uint8_t* aring,
                                             uint8_t* wring, uint8_t* imgs, size_t img_cta) {
  MmaState m;
  int cs = 0;
  uint32_t cph = 0, cmd = 0;
  const bool leader = (threadIdx.x & 31) == 0;
  bool ok = true;
  while (ok && cmd_take(sh, cs, cph, &cmd)) {
    const bool isdw = (cmd & 0xffu) == CMD_DW;
    uint8_t* img_base = nullptr;
    if (isdw) {
      if (leader) {
        bulk_wait_all();
        mbar_arrive(&sh.img_done);
      }
      __syncwarp();
    } else if ((cmd & 0xffu) != CMD_FWD && ((cmd >> 8) & 0xffu) != 0) {
      const size_t j = (cmd >> 24) & 0xffu;  // tile of the CTA: its own image set
      img_base = imgs + (j * kImgSlots + (((cmd >> 8) & 0xffu) - 1)) * img_cta;
    }
    const uint32_t kd = cmd & 0xffu;
    const OpList& L = isdw ? dw : (kd == CMD_EVAL_RE ? ev_re : (kd == CMD_FWD ? fw : ev));
    const int first = isdw ? 0 : (int)((cmd >> 16) & 0xffu);
    for (int i = first; i < L.nops && ok; ++i) ok = mma_op(L.op[i], m, sh, aring, wring, img_base);
  }
  if (leader) bulk_wait_all();
}

// ---- producer warp ---------------------------------------------------------------------
// Streams the B chunks of every op (weight images, or weight-gradient B
// images) into the W ring and, for weight-gradient ops, their A chunks into
// the A ring (those slots are completed by one arrive of 256 counts plus the
// transaction bytes, so the ring keeps one protocol with the epilogue).
// The A ring position advances over the epilogue-written chunks as well.
struct TmaState {
  int wslot = 0, aslot = 0;
  uint32_t wph = 0, aph = 0, img_phase = 0;
  long long g = 0;
  uint32_t issued_w[kWRing] = {0, 0};
  int a_pending[kARing] = {0, 0};     // a producer-filled A slot whose copy may be in flight
  uint32_t a_par[kARing] = {0, 0};    // ... and the phase parity of that fill
  // stash mode: per buffer, bit c = phase parity of chunk c's next fill, and
  // the parities of the fill being read (chunks are refilled unevenly: a
  // buffer holds inputs of different widths in turn)
  uint32_t ph[kStashBufs] = {0, 0, 0, 0};
  uint32_t cur[kStashBufs] = {0, 0, 0, 0};
};

__device__ __forceinline__ bool tma_wait_or_stop(Shared& sh, uint64_t* bar, uint32_t par) {
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  while (true) {
    if (mbar_try_wait(bar, par)) return true;
    if (*vstop || *verr) return false;
  }
}

// One op's copies; `f` is the image slot of stage 1 for stage-stacked
// weight-gradient ops (K chunk c: tile c / (12 np) of the CTA, operand pair
// (c % (12 np)) / 12, stage (c % 12) / 2, trajectory block c % 2; np pairs).
__device__ __forceinline__ bool tma_op(const GemmOp& op, TmaState& t, Shared& sh, uint8_t* aring,
                                       uint8_t* wring, int f) {
  const bool leader = (threadIdx.x & 31) == 0;
  if (op.kind == 2) {  // copy only: epilogue-written A chunks, no weights
    for (int c = 0; c < op.nchunk; ++c) {
      t.a_pending[t.aslot] = 0;
      if (++t.aslot == kARing) { t.aslot = 0; t.aph ^= 1; }
    }
    return true;
  }
  if (op.kind == 3 || op.kind == 4) {
    // stash A chunks (and, for kind 3, the weight chunks)
    if (op.first_nb) {
      t.cur[op.sbuf] = t.ph[op.sbuf];
      t.ph[op.sbuf] ^= (op.nchunk >= 32) ? 0xffffffffu : ((1u << op.nchunk) - 1u);
    }
    const uint8_t* sbase = op.aimg + (size_t)blockIdx.x * op.cta_stride;
    const uint32_t wbytes = 2u * (uint32_t)op.npad * 128u;
    // the pieces the op reads: three-product GEMMs and image copies only the
    // first two (hi, mid; the adjoint's stash chunks hold no lo piece)
    const uint32_t abytes = (op.kind == 4 || op.nprod == 3) ? 2u * 16384u : (uint32_t)kASlotBytes;
    for (int c = 0; c < op.nchunk; ++c) {
      // the epilogue's generic-proxy writes of chunk c are complete (each
      // writer fenced them for the async proxy before arriving)
      if (!tma_wait_or_stop(sh, &sh.stash_full[op.sbuf][c], (t.cur[op.sbuf] >> c) & 1u)) return false;
      if (!tma_wait_or_stop(sh, &sh.a_empty[t.aslot], t.aph ^ 1)) return false;
      if (leader) {
        asm volatile("fence.proxy.async.global;" ::: "memory");
        mbar_arrive_expect_tx(&sh.a_full[t.aslot], abytes);
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                         smem_u32(&sh.a_full[t.aslot])),
                     "r"(kEpiWarps - 1)
                     : "memory");
        bulk_g2s(aring + t.aslot * kASlotBytes, sbase + (size_t)c * kASlotBytes, abytes, &sh.a_full[t.aslot]);
      }
      __syncwarp();
      t.a_pending[t.aslot] = 1;
      t.a_par[t.aslot] = t.aph;
      if (++t.aslot == kARing) { t.aslot = 0; t.aph ^= 1; }
      if (op.kind == 4) continue;
      if (!tma_wait_or_stop(sh, &sh.w_empty[t.wslot], t.wph ^ 1)) return false;
      if (leader) {
        mbar_arrive_expect_tx(&sh.w_full[t.wslot], wbytes);
        bulk_g2s(wring + t.wslot * kWSlotBytes, op.wimg + (size_t)c * wbytes, wbytes, &sh.w_full[t.wslot]);
      }
      __syncwarp();
      t.issued_w[t.wslot] += 1;
      if (++t.wslot == kWRing) { t.wslot = 0; t.wph ^= 1; }
    }
    ++t.g;
    return true;
  }
  const uint32_t ipieces = op.img_pieces ? (uint32_t)op.img_pieces : (uint32_t)kImgPieces;
  const uint32_t bbytes =
      op.kind == 0 ? 2u * (uint32_t)op.npad * 128u : ipieces * (uint32_t)op.nblk_b * 8192u;
  const uint8_t* bbase = op.kind == 0 ? op.wimg : op.wimg + (size_t)blockIdx.x * op.cta_stride;
  const uint8_t* abase = op.kind == 0 ? nullptr : op.aimg + (size_t)blockIdx.x * op.cta_stride;
  if (op.kind == 1 && op.first_dw) {
    if (!tma_wait_or_stop(sh, &sh.img_ready, t.img_phase)) return false;
    t.img_phase ^= 1;
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  for (int c = 0; c < op.nchunk; ++c) {
    size_t aoff = 0, boff = 0;
    if (op.kind == 1) {
      // K chunk c: tile j of the CTA, operand pair q, stage s, 64-trajectory block kb
      const int np = op.npairs > 1 ? op.npairs : 1;
      const int j = c / (12 * np), rem = c - 12 * np * j;
      const int q = rem / 12, cw = rem - 12 * q;
      const int s = cw >> 1, kb = cw & 1;
      const size_t slot = ((size_t)j * kImgSlots + stage_slot(s, f)) * op.slot_stride;
      aoff = slot + (size_t)kb * op.a_step + (size_t)q * op.pair_aoff;
      boff = slot + (size_t)kb * op.b_step + (size_t)q * op.pair_boff;
      if (!tma_wait_or_stop(sh, &sh.a_empty[t.aslot], t.aph ^ 1)) return false;
      if (leader) {
        mbar_arrive_expect_tx(&sh.a_full[t.aslot], op.a_bytes);
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                         smem_u32(&sh.a_full[t.aslot])),
                     "r"(kEpiWarps - 1)
                     : "memory");
        bulk_g2s(aring + t.aslot * kASlotBytes, abase + aoff, op.a_bytes, &sh.a_full[t.aslot]);
      }
      __syncwarp();
      t.a_pending[t.aslot] = 1;
      t.a_par[t.aslot] = t.aph;
    } else {
      t.a_pending[t.aslot] = 0;  // an epilogue chunk follows the earlier copy into this slot
    }
    if (++t.aslot == kARing) { t.aslot = 0; t.aph ^= 1; }
    if (!tma_wait_or_stop(sh, &sh.w_empty[t.wslot], t.wph ^ 1)) return false;
    if (leader) {
      mbar_arrive_expect_tx(&sh.w_full[t.wslot], bbytes);
      if (op.kind == 1 && op.b_pstride != 0) {
        // one N-block of the B image: its blocks in each piece
        const uint32_t part = bbytes / ipieces;
        for (uint32_t q = 0; q < ipieces; ++q)
          bulk_g2s(wring + t.wslot * kWSlotBytes + q * part, bbase + boff + op.b_off0 + (size_t)q * op.b_pstride,
                   part, &sh.w_full[t.wslot]);
      } else {
        const uint8_t* src = op.kind == 0 ? bbase + (size_t)c * bbytes : bbase + boff;
        bulk_g2s(wring + t.wslot * kWSlotBytes, src, bbytes, &sh.w_full[t.wslot]);
      }
    }
    __syncwarp();
    t.issued_w[t.wslot] += 1;
    if (++t.wslot == kWRing) { t.wslot = 0; t.wph ^= 1; }
  }
  ++t.g;
  return true;
}

// Every issued copy must have landed before the CTA exits.
__device__ __forceinline__ void tma_drain(TmaState& t, Shared& sh) {
  volatile int* verr = &sh.err;
  // A slot whose last fill was a producer copy: normally the MMA consumed it
  // long ago (the epilogue drains every op). After an early exit the copy may
  // still be in flight; then the slot's phase is that fill's, and the wait
  // below ends when the bytes land. A phase that moved on twice since reads
  // like an unfinished one, so the wait is short and sets no error.
  for (int s = 0; s < kARing; ++s) {
    if (!t.a_pending[s]) continue;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(&sh.a_full[s], t.a_par[s])) {
      if (globaltimer_ns() - t0 > 20000ull) break;
    }
  }
  for (int s = 0; s < kWRing; ++s) {
    if (t.issued_w[s] == 0) continue;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(&sh.w_full[s], (t.issued_w[s] - 1) & 1)) {
      if (globaltimer_ns() - t0 > kWaitTimeoutNs) { *verr = 3; break; }
    }
  }
}

__device__ __forceinline__ void tma_loop(const OpList& ops, Shared& sh, uint8_t* aring, uint8_t* wring) {
  TmaState t;
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  while (!*vstop && !*verr && tma_op(ops.op[t.g % ops.nops], t, sh, aring, wring, 0)) {
  }
  tma_drain(t, sh);
}

__device__ __forceinline__ void tma_loop_cmd(const OpList& ev, const OpList& dw, const OpList& ev_re,
                                             const OpList& fw, Shared& sh, uint8_t* aring,
                                             uint8_t* wring) {
  TmaState t;
  int cs = 0;
  uint32_t cph = 0, cmd = 0, dph = 0;
  bool run = true;
  while (run && cmd_take(sh, cs, cph, &cmd)) {
    const bool isdw = (cmd & 0xffu) == CMD_DW;
    const uint32_t kd = cmd & 0xffu;
    const OpList& L = isdw ? dw : (kd == CMD_EVAL_RE ? ev_re : (kd == CMD_FWD ? fw : ev));
    if (isdw) {
      // the stage images (bulk-copied by the MMA warp) must have landed
      if (!tma_wait_or_stop(sh, &sh.img_done, dph)) break;
      dph ^= 1;
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
    const int first = isdw ? 0 : (int)((cmd >> 16) & 0xffu);
    for (int i = first; i < L.nops && run; ++i)
      run = tma_op(L.op[i], t, sh, aring, wring, (int)((cmd >> 8) & 0xffu));
  }
  tma_drain(t, sh);
}

// ---- epilogue helpers --------------------------------------------------------------------
struct EpiState {
  int aslot;
  uint32_t aph;
  uint32_t use[2];
  long long g;  // ops consumed
};

__device__ __forceinline__ void epi_state_init(EpiState& e) {
  e.aslot = 0;
  e.aph = 0;
  e.use[0] = e.use[1] = 0;
  e.g = 0;
}

// A chunk's shared-memory writes by the warp are complete: each lane fences
// its writes for the async proxy (the tensor cores read the chunk), then one
// lane arrives for the warp. One arrival per warp instead of one per thread
// keeps the 512-thread epilogue off the barrier's serialised arrive path.
__device__ __forceinline__ void epi_warp_arrive_smem(uint64_t* bar) {
  fence_proxy_async_smem();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
}

// Write this thread's kCW columns (its row r, column group ch) of an A chunk:
// values x[0 .. kCW) for columns [kCW*ch, kCW*ch + kCW) of the chunk, split in
// 3 pieces.
__device__ __forceinline__ bool epi_write_a(EpiState& e, Shared& sh, uint8_t* aring, int r, int ch,
                                            const float* x) {
  volatile int* verr = &sh.err;
  // slot free? (phase of its previous consumption)
  if (!mbar_wait(&sh.a_empty[e.aslot], e.aph ^ 1, verr)) return false;
  uint8_t* base = aring + e.aslot * kASlotBytes;
#pragma unroll
  for (int j = 0; j < kCW / 8; ++j) {
    uint4 hi, mid, lo;
    split3_bf16(x + 8 * j, hi, mid, lo);
    const uint32_t off = sw128_offset(r, (kCW / 8) * ch + j);
    *reinterpret_cast<uint4*>(base + off) = hi;
    *reinterpret_cast<uint4*>(base + 16384 + off) = mid;
    *reinterpret_cast<uint4*>(base + 32768 + off) = lo;
  }
  epi_warp_arrive_smem(&sh.a_full[e.aslot]);
  if (++e.aslot == kARing) { e.aslot = 0; e.aph ^= 1; }
  return true;
}

// Stash mode: this thread's kCW columns (row r, column group ch) of K-chunk c
// of stash buffer b, split in 3 pieces, written with plain global stores in
// the ring-slot layout; then fenced for the async proxy (the producer's bulk
// loads) and marked on the chunk's barrier. Every epilogue thread writes its
// part of every chunk of a layer input exactly once per fill.
// NP = 2 writes only the hi and mid pieces: chunks that only three-product
// GEMMs and image copies read (the adjoint's chains).
template <int NP = 3>
__device__ __forceinline__ void stash_write(uint8_t* stash_cta, Shared& sh, int b, int c, int r, int ch,
                                            const float* x) {
  uint8_t* base = stash_cta + ((size_t)b * kStashChunks + c) * kASlotBytes;
#pragma unroll
  for (int j = 0; j < kCW / 8; ++j) {
    uint4 hi, mid, lo;
    if constexpr (NP == 3) split3_bf16(x + 8 * j, hi, mid, lo);
    else split2_bf16(x + 8 * j, hi, mid);
    const uint32_t off = sw128_offset(r, (kCW / 8) * ch + j);
    *reinterpret_cast<uint4*>(base + off) = hi;
    *reinterpret_cast<uint4*>(base + 16384 + off) = mid;
    if constexpr (NP == 3) *reinterpret_cast<uint4*>(base + 32768 + off) = lo;
  }
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(&sh.stash_full[b][c]);
}

// Bias values of columns [n0, n0 + kCW) of a layer with N outputs (zero past
// N), loaded together (vector loads where aligned) so that a single memory
// round trip covers them; callers issue the next chunk's load before working
// on the current one.
__device__ __forceinline__ void load_bias_cw(const float* __restrict__ b, int n0, int N, float* out) {
  const float* p = b + n0;
  if (n0 + kCW <= N && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
    for (int i = 0; i < kCW / 4; ++i) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p) + i);
      out[4 * i] = q.x; out[4 * i + 1] = q.y; out[4 * i + 2] = q.z; out[4 * i + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kCW; ++i) out[i] = (n0 + i < N) ? __ldg(p + i) : 0.f;
  }
}

// v <- act(v + bias) on kCW columns starting at n0 (columns at or past N -> 0,
// the zero padding of the next GEMM's K dimension). The activation branch is
// taken once per chunk, not per element.
__device__ __forceinline__ void bias_act_cw(float* v, const float* bias, int act, int n0, int N) {
  if (act == GBNDE_ACT_TANH) {
#pragma unroll
    for (int i = 0; i < kCW; ++i) v[i] = tanh_tc(v[i] + bias[i]);
  } else if (act == GBNDE_ACT_SOFTPLUS) {
#pragma unroll
    for (int i = 0; i < kCW; ++i) v[i] = act_apply_tc(v[i] + bias[i], GBNDE_ACT_SOFTPLUS);
  } else {
#pragma unroll
    for (int i = 0; i < kCW; ++i) v[i] += bias[i];
  }
  if (n0 + kCW > N) {
#pragma unroll
    for (int i = 0; i < kCW; ++i)
      if (n0 + i >= N) v[i] = 0.f;
  }
}

// v <- v * act'(z) on kCW columns starting at n0, with act' taken from the
// stored activation outputs y (tanh: 1 - y^2; softplus: 1 - exp(-y));
// columns at or past N -> 0. The activation branch is taken once per chunk.
__device__ __forceinline__ void deriv_mul_cw(float* v, const float* y, int act, int n0, int N) {
  if (act == GBNDE_ACT_TANH) {
#pragma unroll
    for (int i = 0; i < kCW; ++i) v[i] *= fmaf(-y[i], y[i], 1.f);
  } else if (act == GBNDE_ACT_SOFTPLUS) {
#pragma unroll
    for (int i = 0; i < kCW; ++i) v[i] *= -expm1f(-y[i]);
  }
  if (n0 + kCW > N) {
#pragma unroll
    for (int i = 0; i < kCW; ++i)
      if (n0 + i >= N) v[i] = 0.f;
  }
}

// TMEM -> registers: this warp's 32 lanes, kCW columns from taddr.
__device__ __forceinline__ void tmem_ld_cw(uint32_t taddr, float* v) {
  if constexpr (kCW == 32) tmem_ld32(taddr, v);
  else tmem_ld16(taddr, v);
}

// Skip A-ring slots that the producer warp fills (weight-gradient ops).
__device__ __forceinline__ void epi_skip_a(EpiState& e, int n) {
  for (int i = 0; i < n; ++i)
    if (++e.aslot == kARing) { e.aslot = 0; e.aph ^= 1; }
}

// Wait for the accumulator of the next op; returns its TMEM column base.
__device__ __forceinline__ bool epi_wait_acc(EpiState& e, Shared& sh, uint32_t* col) {
  const int reg = (int)(e.g & 1);
  if (!mbar_wait(&sh.acc_full[reg], e.use[reg] & 1, &sh.err)) return false;
  tc_fence_after();
  *col = (uint32_t)(reg * 256);
  return true;
}

// Posts a command (thread 0 of the epilogue only). Returns false if the ring
// slot did not come free within the wait limit.
struct CmdPoster {
  int cs = 0;
  uint32_t cph = 0;
};
__device__ __forceinline__ bool epi_post(CmdPoster& p, Shared& sh, uint32_t cmd) {
  if (!mbar_wait(&sh.cmd_empty[p.cs], p.cph ^ 1, &sh.err)) return false;
  ((volatile uint32_t*)sh.cmd)[p.cs] = cmd;
  mbar_arrive(&sh.cmd_full[p.cs]);
  if (++p.cs == kCmdRing) { p.cs = 0; p.cph ^= 1; }
  return true;
}

__device__ __forceinline__ void epi_release_acc(EpiState& e, Shared& sh) {
  const int reg = (int)(e.g & 1);
  tc_fence_before();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(&sh.acc_empty[reg]);
  e.use[reg] += 1;
  e.g += 1;
}

}  // namespace tc
}  // namespace gbnde
