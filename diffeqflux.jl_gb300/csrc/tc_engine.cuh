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
// Warp roles (384 threads, three warpgroups): warps 0-7 epilogue (EPI),
// warp 8 MMA issuer, warp 9 weight producer, warps 10-11 idle. The MMA and
// producer warps run the op list cyclically until the epilogue raises the
// stop flag. The kernel is launched with kLaunchRegs registers per thread;
// the control warpgroup then gives registers back (setmaxnreg.dec to
// kCtlRegs) and the two epilogue warpgroups take them (setmaxnreg.inc to
// kEpiRegs): 256 * kEpiRegs + 128 * kCtlRegs == 384 * kLaunchRegs, checked at
// compile time here and against the compiled kernel's register count before
// every launch (a split above the launch's registers would never complete).
#pragma once
#include "kernels.h"
#include "tc_ptx.cuh"

namespace gbnde {
namespace tc {

constexpr int kEpiThreads = 256;
constexpr int kThreads = 384;
constexpr int kMmaWarp = 8;
constexpr int kTmaWarp = 9;
constexpr int kLaunchRegs = 168;   // 65536 / 384, rounded down to a multiple of 8
constexpr int kEpiRegs = 224;
constexpr int kCtlRegs = 56;
static_assert(kEpiThreads * kEpiRegs + (kThreads - kEpiThreads) * kCtlRegs == kThreads * kLaunchRegs,
              "register split must equal the launch's registers");
static_assert(kThreads * kLaunchRegs <= 65536, "launch registers exceed the register file");
constexpr int kASlotBytes = 3 * 16384;   // 3 pieces x 128 rows x 128 B
constexpr int kWSlotBytes = 2 * 32768;   // 2 pieces x 256 rows x 128 B
constexpr int kARing = 2;
constexpr int kWRing = 2;
constexpr int kSmemBytes = 1024 + kARing * kASlotBytes + kWRing * kWSlotBytes;
constexpr int kMaxOps = 40;

// kind 0 (chain GEMM): A chunks written by the epilogue (3 pieces, K-major),
//   B = weight image chunks (2 pieces, K-major), five split products.
// kind 1 (weight-gradient GEMM, K = trajectories): A and B both bulk-copied
//   from per-CTA images (2 pieces, MN-major 64-column blocks), three products
//   hi.hi + hi.lo + lo.hi.
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
  uint32_t tmem_base;
  int stop;
  int err;
  double red[16];
};

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Register split between the warpgroups (all four warps of a warpgroup
// execute the same instruction).
__device__ __forceinline__ void regs_take_epi() {
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kEpiRegs));
}
__device__ __forceinline__ void regs_give_ctl() {
  asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kCtlRegs));
}

// Deterministic sum of a double over the 256 epilogue threads.
__device__ __forceinline__ double epi_sum(double v, Shared& sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  epi_bar();
  if ((threadIdx.x & 31) == 0) sh.red[w] = v;
  epi_bar();
  double s = 0.0;
  for (int i = 0; i < 8; ++i) s += sh.red[i];
  epi_bar();
  return s;
}

__device__ __forceinline__ void init_shared(Shared& sh) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < kARing; ++i) {
      mbar_init(&sh.a_full[i], kEpiThreads);
      mbar_init(&sh.a_empty[i], 1);
    }
    for (int i = 0; i < kWRing; ++i) {
      mbar_init(&sh.w_full[i], 1);
      mbar_init(&sh.w_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&sh.acc_full[i], 1);
      mbar_init(&sh.acc_empty[i], kEpiThreads);
    }
    mbar_init(&sh.img_ready, kEpiThreads);
    sh.stop = 0;
    sh.err = 0;
    fence_mbar_init();
  }
}

// ---- MMA warp ------------------------------------------------------------------------
// Executes the op list cyclically. Returns when the stop flag is raised (or on
// a wait timeout, which also raises sh.err).
__device__ __forceinline__ void mma_loop(const OpList& ops, Shared& sh, uint8_t* aring,
                                         uint8_t* wring) {
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  const bool leader = (threadIdx.x & 31) == 0;
  int aslot = 0, wslot = 0;
  uint32_t aph = 0, wph = 0;
  uint32_t use[2] = {0, 0};
  long long g = 0;
  const int pa[5] = {0, 1, 0, 2, 1};
  const int pb[5] = {0, 0, 1, 0, 1};
  while (true) {
    const GemmOp& op = ops.op[g % ops.nops];
    const int reg = (int)(g & 1);
    // accumulator region free?
    {
      const uint32_t par = (use[reg] & 1) ^ 1;
      while (!mbar_try_wait(&sh.acc_empty[reg], par)) {
        if (*vstop || *verr) return;
      }
    }
    const uint32_t d = sh.tmem_base + (uint32_t)(reg * 256);
    const uint32_t idesc = op.kind == 0 ? idesc_bf16(128, op.npad) : idesc_bf16_mn(128, op.npad);
    const uint32_t wpiece = op.kind == 0 ? (uint32_t)op.npad * 128 : (uint32_t)op.nblk_b * 8192;
    for (int c = 0; c < op.nchunk; ++c) {
      // A chunk ready? (bounded by the stop flag: the epilogue may be done)
      {
        unsigned long long t0 = 0;
        while (!mbar_try_wait(&sh.a_full[aslot], aph)) {
          if (*vstop || *verr) return;
          if (t0 == 0) t0 = globaltimer_ns();
          else if (globaltimer_ns() - t0 > 4 * kWaitTimeoutNs) { *verr = 2; return; }
        }
      }
      if (!mbar_wait(&sh.w_full[wslot], wph, verr)) return;
      tc_fence_after();
      if (leader) {
        const uint32_t a0 = smem_u32(aring + aslot * kASlotBytes);
        const uint32_t b0 = smem_u32(wring + wslot * kWSlotBytes);
        if (op.kind == 0) {
#pragma unroll
          for (int pr = 0; pr < 5; ++pr) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ad = sdesc_sw128(a0 + pa[pr] * 16384 + kk * 32);
              const uint64_t bd = sdesc_sw128(b0 + pb[pr] * wpiece + kk * 32);
              mma_bf16(d, ad, bd, idesc, (c > 0 || pr > 0 || kk > 0) ? 1u : 0u);
            }
          }
        } else {
          // A chunk: 2 pieces x 2 blocks x 8 KB; B chunk: 2 pieces x nblk x 8 KB.
          // Products hi.hi, hi.lo, lo.hi; K step of 16 trajectories = 2048 bytes.
#pragma unroll
          for (int pr = 0; pr < 3; ++pr) {
            const int qa = (pr == 2) ? 1 : 0, qb = (pr == 1) ? 1 : 0;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ad = sdesc_sw128_mn(a0 + qa * 16384 + kk * 2048, 8192);
              const uint64_t bd = sdesc_sw128_mn(b0 + qb * wpiece + kk * 2048, 8192);
              mma_bf16(d, ad, bd, idesc, (c > 0 || pr > 0 || kk > 0) ? 1u : 0u);
            }
          }
        }
        mma_commit(&sh.a_empty[aslot]);
        mma_commit(&sh.w_empty[wslot]);
        if (c == op.nchunk - 1) mma_commit(&sh.acc_full[reg]);
      }
      __syncwarp();
      if (++aslot == kARing) { aslot = 0; aph ^= 1; }
      if (++wslot == kWRing) { wslot = 0; wph ^= 1; }
    }
    use[reg] += 1;
    ++g;
  }
}

// ---- producer warp ---------------------------------------------------------------------
// Streams the B chunks of every op (weight images, or weight-gradient B
// images) into the W ring and, for weight-gradient ops, their A chunks into
// the A ring (those slots are completed by one arrive of 256 counts plus the
// transaction bytes, so the ring keeps one protocol with the epilogue).
// The A ring position advances over the epilogue-written chunks as well.
__device__ __forceinline__ void tma_loop(const OpList& ops, Shared& sh, uint8_t* aring,
                                         uint8_t* wring) {
  volatile int* verr = &sh.err;
  volatile int* vstop = &sh.stop;
  const bool leader = (threadIdx.x & 31) == 0;
  int wslot = 0, aslot = 0;
  uint32_t wph = 0, aph = 0, img_phase = 0;
  long long g = 0;
  uint32_t issued_w[kWRing] = {0, 0};
  uint32_t issued_a[kARing] = {0, 0};
  auto wait_or_stop = [&](uint64_t* bar, uint32_t par) -> bool {
    while (true) {
      if (mbar_try_wait(bar, par)) return true;
      if (*vstop || *verr) return false;
    }
  };
  bool run = true;
  while (run && !*vstop && !*verr) {
    const GemmOp& op = ops.op[g % ops.nops];
    const uint32_t bbytes = op.kind == 0 ? 2u * (uint32_t)op.npad * 128u : 2u * (uint32_t)op.nblk_b * 8192u;
    const uint8_t* bbase = op.kind == 0 ? op.wimg : op.wimg + (size_t)blockIdx.x * op.cta_stride;
    const uint8_t* abase = op.kind == 0 ? nullptr : op.aimg + (size_t)blockIdx.x * op.cta_stride;
    if (op.kind == 1 && op.first_dw) {
      if (!wait_or_stop(&sh.img_ready, img_phase)) break;
      img_phase ^= 1;
      asm volatile("fence.proxy.async.global;" ::: "memory");
    }
    for (int c = 0; c < op.nchunk; ++c) {
      if (op.kind == 1) {
        if (!wait_or_stop(&sh.a_empty[aslot], aph ^ 1)) { run = false; break; }
        if (leader) {
          mbar_arrive_expect_tx(&sh.a_full[aslot], op.a_bytes);
          asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                           smem_u32(&sh.a_full[aslot])),
                       "r"(kEpiThreads - 1)
                       : "memory");
          bulk_g2s(aring + aslot * kASlotBytes, abase + (size_t)c * op.a_step, op.a_bytes, &sh.a_full[aslot]);
        }
        __syncwarp();
        issued_a[aslot] += 1;
      }
      if (++aslot == kARing) { aslot = 0; aph ^= 1; }
      if (!wait_or_stop(&sh.w_empty[wslot], wph ^ 1)) { run = false; break; }
      if (leader) {
        mbar_arrive_expect_tx(&sh.w_full[wslot], bbytes);
        const uint8_t* src = op.kind == 0 ? bbase + (size_t)c * bbytes : bbase + (size_t)c * op.b_step;
        bulk_g2s(wring + wslot * kWSlotBytes, src, bbytes, &sh.w_full[wslot]);
      }
      __syncwarp();
      issued_w[wslot] += 1;
      if (++wslot == kWRing) { wslot = 0; wph ^= 1; }
    }
    ++g;
  }
  // drain: every issued copy must have landed before the CTA exits
  for (int s = 0; s < kWRing; ++s) {
    if (issued_w[s] == 0) continue;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(&sh.w_full[s], (issued_w[s] - 1) & 1)) {
      if (globaltimer_ns() - t0 > kWaitTimeoutNs) { *verr = 3; break; }
    }
  }
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

// Write this thread's 32 columns (its row r, column half ch) of an A chunk:
// values x[0..31] for columns [32*ch, 32*ch+32) of the chunk, split in 3 pieces.
__device__ __forceinline__ bool epi_write_a(EpiState& e, Shared& sh, uint8_t* aring, int r, int ch,
                                            const float* x) {
  volatile int* verr = &sh.err;
  // slot free? (phase of its previous consumption)
  if (!mbar_wait(&sh.a_empty[e.aslot], e.aph ^ 1, verr)) return false;
  uint8_t* base = aring + e.aslot * kASlotBytes;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint4 hi, mid, lo;
    split3_bf16(x + 8 * j, hi, mid, lo);
    const uint32_t off = sw128_offset(r, 4 * ch + j);
    *reinterpret_cast<uint4*>(base + off) = hi;
    *reinterpret_cast<uint4*>(base + 16384 + off) = mid;
    *reinterpret_cast<uint4*>(base + 32768 + off) = lo;
  }
  fence_proxy_async_smem();
  mbar_arrive(&sh.a_full[e.aslot]);
  if (++e.aslot == kARing) { e.aslot = 0; e.aph ^= 1; }
  return true;
}

// Bias values of columns [n0, n0 + 32) of a layer with N outputs (zero past
// N), loaded together (vector loads where aligned) so that a single memory
// round trip covers them; callers issue the next chunk's load before working
// on the current one.
__device__ __forceinline__ void load_bias32(const float* __restrict__ b, int n0, int N, float* out) {
  const float* p = b + n0;
  if (n0 + 32 <= N && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p) + i);
      out[4 * i] = q.x; out[4 * i + 1] = q.y; out[4 * i + 2] = q.z; out[4 * i + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) out[i] = (n0 + i < N) ? __ldg(p + i) : 0.f;
  }
}

// v <- act(v + bias) on 32 columns starting at n0 (columns at or past N -> 0,
// the zero padding of the next GEMM's K dimension). The activation branch is
// taken once per chunk, not per element.
__device__ __forceinline__ void bias_act32(float* v, const float* bias, int act, int n0, int N) {
  if (act == GBNDE_ACT_TANH) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = tanh_tc(v[i] + bias[i]);
  } else if (act == GBNDE_ACT_SOFTPLUS) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = act_apply_tc(v[i] + bias[i], GBNDE_ACT_SOFTPLUS);
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] += bias[i];
  }
  if (n0 + 32 > N) {
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (n0 + i >= N) v[i] = 0.f;
  }
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

__device__ __forceinline__ void epi_release_acc(EpiState& e, Shared& sh) {
  const int reg = (int)(e.g & 1);
  tc_fence_before();
  mbar_arrive(&sh.acc_empty[reg]);
  e.use[reg] += 1;
  e.g += 1;
}

}  // namespace tc
}  // namespace gbnde
