// tc_ptx.cuh -- inline-PTX wrappers for the Blackwell (sm_100a/sm_103a)
// tensor-core path: mbarriers with bounded waits, bulk (TMA engine) copies,
// TMEM allocation, tcgen05.mma / commit / ld, and the shared-memory and
// instruction descriptors of kind::f16 MMAs with BF16 operands.
//
// Operand layout used throughout: K-major, 128-byte swizzle. A tile of R rows
// x 64 bf16 (128 bytes per row) is stored as R/8 atoms of 8 rows x 128 bytes
// (1024 bytes, the stride-dimension offset); inside an atom the 16-byte chunk
// c of row r sits at chunk position c ^ (r % 8). Buffers are 1024-byte aligned.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace gbnde {
namespace tc {

// Wait limit for every mbarrier wait (ns of %globaltimer).
constexpr unsigned long long kWaitTimeoutNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier -----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on phase `parity`. On timeout sets *err (shared or global
// flag) and returns false; the caller then winds down.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*err) return false;
    if (globaltimer_ns() - t0 > kWaitTimeoutNs) {
      *err = 1;
      return false;
    }
  }
  return true;
}

// ---- bulk copy global -> shared (TMA engine, no tensor map) -----------------------
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gsrc, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---- bulk copy shared -> global (bulk-group completion) ---------------------------
// Both addresses 16-byte aligned, bytes a multiple of 16. The issuing thread
// tracks completion with commit_group / wait_group.
__device__ __forceinline__ void bulk_s2g(void* gdst, const void* smem_src, uint32_t bytes, uint64_t pol) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group.L2::cache_hint [%0], [%1], %2, %3;" ::"l"(gdst),
               "r"(smem_u32(smem_src)), "r"(bytes), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of all committed groups have been read
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// all committed groups have completed (their global writes are done)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---- TMEM -----------------------------------------------------------------------
// Executed by one full warp. Writes the TMEM base address into *slot (smem).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- descriptors ------------------------------------------------------------------
// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, SBO = 1024 bytes.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: 8-row atoms
  d |= (uint64_t)1 << 46;                        // descriptor version (sm_100)
  d |= (uint64_t)2 << 61;                        // SWIZZLE_128B
  return d;
}

// Shared-memory matrix descriptor: MN-major, SWIZZLE_128B. The operand is
// stored as blocks of 64 MN-elements (128-byte rows, one row per K index,
// 8-row swizzle atoms 1024 bytes apart = SBO); consecutive 64-element MN
// blocks are `lbo` bytes apart.
__device__ __forceinline__ uint64_t sdesc_sw128_mn(uint32_t saddr, uint32_t lbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;    // leading byte offset: next 64-element MN block
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset: next 8 K-rows
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                 // D format F32
         | (1u << 7)               // A format BF16
         | (1u << 10)              // B format BF16
         | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Same with both operands MN-major (transpose bits for A and B).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int M, int N) {
  return idesc_bf16(M, N) | (1u << 15) | (1u << 16);
}

// kind::f16 with FP16 operands (A = B = F16, format code 0), both MN-major.
__host__ __device__ constexpr uint32_t idesc_f16_mn(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24) | (1u << 15) | (1u << 16);
}

// ---- MMA --------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on `bar` when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// ---- TMEM -> registers ------------------------------------------------------------
// 32 lanes x 32 columns of 32-bit: lane i of the warp gets row (lane base + i),
// columns [col, col + 32).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 16 columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- swizzled operand stores ----------------------------------------------------------
// Byte offset of (row r, 16-byte chunk c) inside a K-major SW128 tile.
__device__ __forceinline__ uint32_t sw128_offset(int r, int c) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// Pack 8 floats into 8 bf16 (round to nearest even) as one 16-byte chunk.
__device__ __forceinline__ uint4 pack8_bf16(const float* x) {
  uint4 o;
  __nv_bfloat162 h0 = __floats2bfloat162_rn(x[0], x[1]);
  __nv_bfloat162 h1 = __floats2bfloat162_rn(x[2], x[3]);
  __nv_bfloat162 h2 = __floats2bfloat162_rn(x[4], x[5]);
  __nv_bfloat162 h3 = __floats2bfloat162_rn(x[6], x[7]);
  o.x = *reinterpret_cast<uint32_t*>(&h0);
  o.y = *reinterpret_cast<uint32_t*>(&h1);
  o.z = *reinterpret_cast<uint32_t*>(&h2);
  o.w = *reinterpret_cast<uint32_t*>(&h3);
  return o;
}

// Split 8 floats into hi/mid/lo bf16 pieces (x ~= hi + mid + lo) and return the
// three 16-byte chunks.
// The first two of the same pieces (hi, mid), for GEMMs that issue only the
// products A_hi W_hi + A_mid W_hi + A_hi W_lo.
__device__ __forceinline__ void split2_bf16(const float* x, uint4& hi, uint4& mid) {
  float r[8];
  uint4 ph = pack8_bf16(x);
  const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&ph);
#pragma unroll
  for (int i = 0; i < 8; ++i) r[i] = x[i] - __bfloat162float(hb[i]);
  hi = ph;
  mid = pack8_bf16(r);
}

__device__ __forceinline__ void split3_bf16(const float* x, uint4& hi, uint4& mid, uint4& lo) {
  float r[8], h[8];
  uint4 ph = pack8_bf16(x);
  const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&ph);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    h[i] = __bfloat162float(hb[i]);
    r[i] = x[i] - h[i];
  }
  uint4 pm = pack8_bf16(r);
  const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(&pm);
#pragma unroll
  for (int i = 0; i < 8; ++i) r[i] = r[i] - __bfloat162float(mb[i]);
  hi = ph;
  mid = pm;
  lo = pack8_bf16(r);
}

// ---- L2 eviction priority ----------------------------------------------------------
// Cache policies for accesses whose reuse distance is known: data read once
// much later (weight-gradient images) is marked evict-first so that it does
// not push out data read back soon (activation scratch, marked evict-last).
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_v4_hint(void* ptr, uint4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(ptr), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ float4 ld_v4f_hint(const void* ptr, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(ptr), "l"(pol)
               : "memory");
  return v;
}

// Fire-and-forget global add (performed at L2; no value returned, so the
// issuing thread does not wait for the memory round trip). Each address of a
// pending quadrature buffer has one adding thread, so the adds to an address
// happen in that thread's program order: the sums stay deterministic.
__device__ __forceinline__ void red_add(float* p, float a) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(a) : "memory");
}

}  // namespace tc
}  // namespace gbnde
