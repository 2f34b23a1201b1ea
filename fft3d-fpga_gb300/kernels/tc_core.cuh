// tc_core.cuh - Blackwell tensor-core (tcgen05) building blocks written in
// inline PTX: TMEM allocation, shared-memory matrix descriptors, the
// instruction descriptor of kind::f16 MMAs, MMA issue/commit, bounded
// mbarrier waits and TMEM loads.
//
// Operand layout used throughout (K-major, no swizzle): an R x K half-
// precision matrix is stored as 8-row x 16-byte "core matrices"; element
// (r, k) lives at byte (r/8)*SBO + (k/8)*LBO + (r%8)*16 + (k%8)*2 with
// LBO = 128 and SBO = (K/8)*128.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fftgb {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) in the core-matrix layout of an R x K tile
__device__ __forceinline__ int core_off(int r, int k, int K) {
  return (r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// (K-direction core-matrix) byte offset, stride (8-row group) byte offset,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo,
                                              uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // version
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of tcgen05.mma.kind::f16: D = F32, A/B = F16 (0)
// or BF16 (1), both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int ab_bf16, int M, int N) {
  return (1u << 4) | ((uint32_t)ab_bf16 << 7) | ((uint32_t)ab_bf16 << 10) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *smem_slot, uint32_t ncols) {
  asm volatile(
      "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
          smem_u32(smem_slot)),
      "r"(ncols));
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr),
               "r"(ncols));
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc,
                                        uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];\n" ::"r"(smem_u32(mbar)));
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// make generic-proxy shared-memory stores visible to the tensor core
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)),
               "r"(count));
}

// Wait for phase `parity` of the mbarrier, giving up after `limit` polls.
// Returns true when the phase completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *mbar, uint32_t parity,
                                                  uint32_t limit) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// The give-up path of a bounded wait, on demand: thread 0 waits on a fresh
// mbarrier that nothing ever arrives on (no copy, no MMA refers to it), gives
// up after `polls` polls and records the timeout in `status` as the kernels
// record a wait that gave up.  Lets a test check that a timeout reaches the
// host as FFTGB_ETIMEOUT (and valid = false) without leaving any copy in
// flight.
__device__ __forceinline__ void expire_wait(int *status, uint32_t polls) {
  __shared__ __align__(8) uint64_t never;
  if (threadIdx.x == 0) {
    mbar_init(&never, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    if (!mbar_wait_bounded(&never, 0, polls)) atomicExch(status, 1);
  }
}

// 32 consecutive 32-bit TMEM columns of lane (warp quarter base + laneid).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&r)[32]) {
  uint32_t u[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]),
        "=r"(u[6]), "=r"(u[7]), "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]),
        "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]), "=r"(u[16]),
        "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]),
        "=r"(u[22]), "=r"(u[23]), "=r"(u[24]), "=r"(u[25]), "=r"(u[26]),
        "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) r[i] = __uint_as_float(u[i]);
}

// Round-to-nearest splits of x into hi + lo (and for BF16 a third term).
__device__ __forceinline__ void split_f16(float x, __half &hi, __half &lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi,
                                           __nv_bfloat16 &mid,
                                           __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
}

}  // namespace tc
}  // namespace fftgb
