// hmf_async.cuh -- inline-PTX helpers for sm_103a asynchronous copies:
// mbarriers, tensor (TMA) and bulk copies global -> shared, time-bounded waits.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace hmf {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// An initialised mbarrier must be invalidated before its memory is
// initialised again (re-initialising a valid mbarrier object is undefined):
// every phase must have completed, with no thread waiting on it.
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// try_wait with a suspend-time hint: a thread whose phase is not complete
// sleeps (up to the hint, in ns) until it completes instead of spinning.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity), "r"(100000u)
      : "memory");
  return done != 0;
}

// Tensor maps here live in global memory and are written by host copies
// before a launch (one table per context, rewritten every solve).  The TMA
// unit reads a map through the tensormap proxy, which may still hold the
// 128-byte descriptor an earlier kernel used at the same address (a context
// freed and another allocated in its place, or a table rewritten with other
// arrays), so every thread that issues copies with a map first acquires it
// for that proxy, at system scope because the writer is the host.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

__device__ __forceinline__ void tma_load_plane(float* dst, const CUtensorMap* map, int x, int y, int z,
                                               uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for a completed phase for at most `limit_ns`; false on time-out (the
// caller records the failure instead of hanging).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// Error-flag bit of a requested stall: the first CTA of a copy-pipeline
// kernel that finds it set clears it and, before its first copy wait, waits
// on an mbarrier that nothing completes, so that the bounded wait runs out
// and the kernel's time-out path (stop issuing, drain the copies in flight,
// report) runs on healthy hardware.  Set by the host only on request
// (hmf_inject_wait_stall).
constexpr int kStallRequest = 1 << 16;

// Thread 0 of a CTA, given the error flag's value read at kernel start:
// whether this CTA takes the stall request (exactly one CTA does).
__device__ __forceinline__ bool take_stall_request(int* error_flag, int flag) {
  return error_flag && (flag & kStallRequest) && (atomicAnd(error_flag, ~kStallRequest) & kStallRequest);
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace hmf
