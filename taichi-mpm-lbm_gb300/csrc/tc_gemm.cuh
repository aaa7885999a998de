// Fifth-generation tensor core (tcgen05) building blocks for sm_100+ / sm_103a, in inline PTX:
// tensor-memory allocation, shared-memory operand descriptors, BF16 MMA with FP32
// accumulation in tensor memory, commit to an mbarrier, and loads of the accumulator.
//
// Operands are staged in shared memory in the canonical K-major layout without swizzle:
// "core matrices" of 8 rows x 16 bytes (8 bf16 along K) stored as 128 contiguous bytes.
// For a tile of R rows and Kc columns, core matrix (rb, kb) sits at byte
//   (rb * (Kc / 8) + kb) * 128,
// so core matrices adjacent along K are 128 bytes apart (leading-dimension byte offset,
// LBO) and those adjacent along M/N are Kc * 16 bytes apart (stride byte offset, SBO).
// One MMA consumes K = 16 (two core matrices along K); the next K slice starts 256 bytes on.
//
// Every wait on an mbarrier is bounded: after kWaitCycles clock cycles it gives up, records
// an error code in a caller-provided flag and returns false, so a kernel can release its
// tensor memory and return instead of hanging.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace fsi {
namespace tc {

// Bound of every wait: about one second at the 2 GHz SM clock.
constexpr long long kWaitCycles = 1ll << 31;
// Suspend-time hint of one poll (ns): a waiting thread sleeps instead of spinning, leaving
// the issue slots to the warps that work.
constexpr uint32_t kSuspendNs = 20000;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of a K-major no-swizzle tile with kc columns.
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int kc) {
  return (uint32_t)(((r >> 3) * (kc >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), descriptor version 1
// (bits 46-48 = 0b001), base offset 0, layout type 0 (no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Descriptor of the K slice [16 s, 16 s + 16) of a K-major no-swizzle tile with kc columns.
__device__ __forceinline__ uint64_t tile_desc(uint32_t tile_addr, int kc, int s) {
  return smem_desc(tile_addr + (uint32_t)s * 256u, 128u, (uint32_t)kc * 16u);
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, both operands K-major, dense.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4)                         // D format F32
         | (1u << 7)                       // A format BF16
         | (1u << 10)                      // B format BF16
         | ((uint32_t)(n >> 3) << 17)      // N / 8
         | ((uint32_t)(m >> 4) << 24);     // M / 16
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// One bounded poll of the phase with parity `parity`: the thread is suspended (it issues
// nothing) until the phase completes or kSuspendNs elapse.
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;}"
      : "=r"(done)
      : "r"(a), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return done != 0;
}

// Waits for the phase with parity `parity` to complete; false (and *err set) after
// kWaitCycles SM clock cycles.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  const uint32_t a = smem_addr(bar);
  const long long t0 = clock64();
  while (!mbar_try(a, parity)) {
    if (clock64() - t0 > kWaitCycles) {
      if (err) atomicExch(err, code);
      return false;
    }
  }
  return true;
}

// Arrives once on `bar` (release semantics at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// As mbar_wait, but also gives up (without recording an error) once *abort is non-zero,
// and sets *abort when it times out itself, so that the other roles of a warp-specialised
// kernel stop waiting for it.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t* bar, uint32_t parity,
                                                    volatile int* abort, int* err, int code) {
  const uint32_t a = smem_addr(bar);
  const long long t0 = clock64();
  while (!mbar_try(a, parity)) {
    if (*abort) return false;
    if (clock64() - t0 > kWaitCycles) {
      *abort = 1;
      if (err) atomicExch(err, code);
      return false;
    }
  }
  return true;
}

// ----------------------------------------------------------- tensor memory
// Allocates ncols columns (power of two >= 32) for the CTA; one full warp executes it.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the tensor cores.
__device__ __forceinline__ void fence_smem_for_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A * B^T for one K = 16 slice; issued by a single thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, bool accumulate) {
  asm volatile(
      "{.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrives once on `bar` when all previously issued MMAs of this thread have completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (lane = 32 * (warp % 4) + lane id).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace fsi
