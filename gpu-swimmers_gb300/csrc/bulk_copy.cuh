// bulk_copy.cuh -- one-dimensional bulk copies global -> shared memory
// (cp.async.bulk, the TMA engine's untiled form) completed on an mbarrier.
//
// A copy moves a contiguous run of bytes; source and destination must be
// 16-byte aligned and the size a multiple of 16.  The thread that arms a
// barrier announces the bytes its copies will deliver (expect_tx); the barrier's
// phase completes once they have all landed, and the threads that read the
// buffer wait for that phase.  Every wait is bounded in time: past the limit
// it records an error in the caller's status word and gives up, so a mistake
// in the byte counts shows up as an error status instead of a hung GPU.
#pragma once
#include <cstdint>

namespace lbswim {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes initialised barriers visible to the async proxy (before any copy uses them).
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy writes (a bulk copy into a buffer the threads just read).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// One bounded wait for the phase: the thread is suspended (not spinning) until
// the phase completes or about MBAR_SUSPEND_NS pass.
constexpr uint32_t MBAR_SUSPEND_NS = 100000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity), "r"(MBAR_SUSPEND_NS)
      : "memory");
  return done != 0;
}

// Wait for phase `parity` of the barrier.  The wait is bounded by time
// (MBAR_WAIT_NS of the global timer): past it, the bit `code` is set in *err
// and the wait returns false.  Once that bit is set, later waits of any CTA
// return at once, so a kernel whose copies never complete still ends within
// about one limit (its results are then wrong, and the status says so).
constexpr unsigned long long MBAR_WAIT_NS = 2000000000ull;  // 2 s
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned* err,
                                          unsigned code) {
  if (mbar_try_wait(bar, parity)) return true;
  // try_wait suspends the thread for a while in hardware; the timer and the
  // status word are looked at only every 64 tries
  const unsigned long long t0 = global_ns();
  for (unsigned i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 0) {
      if (err && (*(volatile unsigned*)err & code)) return false;
      if (global_ns() - t0 > MBAR_WAIT_NS) {
        if (err) atomicOr(err, code);
        return false;
      }
    }
  }
}

}  // namespace lbswim
