// vk_bulk.cuh -- bulk-copy row loads for the FP64 row passes (sm_103a).
//
// A row of complex doubles lands in the padded shared-memory layout of the
// row transforms (16 elements, then one pad element) by cp.async.bulk: a
// padded chunk of 16 elements is 256 contiguous bytes and every element is
// 16 bytes, so any element range splits at the chunk boundaries into pieces
// whose shared and global addresses are 16-byte aligned and whose sizes are
// multiples of 16 bytes.  One mbarrier per CTA counts the bytes: thread 0
// initialises it and posts the expected byte count before any thread issues
// a piece, the threads issue the pieces, and every thread waits with a
// bounded poll.  A CTA whose wait runs out sets the error word, waits again
// (bounded) for the copies still in flight into its shared memory, and
// returns; the host reports the error word.
#pragma once
#include <stdint.h>
#include "vk_tc.cuh"

namespace vk {

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}

// Thread 0 sets up the CTA's barrier for `bytes` of copies; every thread
// must call it, and no thread issues a copy before it returns.
__device__ __forceinline__ void bulk_begin(uint64_t* bar, uint32_t bytes) {
  if (threadIdx.x == 0) {
    tc::mbar_init(bar);
    tc::mbar_arrive_expect_tx(bar, bytes);
  }
  __syncthreads();
}

// Elements [a, b) of the global row g into the padded row s (element k at
// s[pidx(k)]): one piece per 16-element chunk, the chunks spread over the
// NT threads.
template <int NT>
__device__ __forceinline__ void bulk_row_range(double2* s, const double2* g, int a, int b, uint64_t* bar) {
  if (b <= a) return;
  const int c1 = (b - 1) >> 4;
  for (int ch = (a >> 4) + (int)threadIdx.x; ch <= c1; ch += NT) {
    const int lo = max(a, ch << 4), hi = min(b, (ch + 1) << 4);
    bulk_g2s(s + lo + ch, g + lo, (uint32_t)(hi - lo) * 16u, bar);
  }
}

__device__ __forceinline__ bool bulk_try(uint64_t* bar) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(tc::smem_u32(bar))
      : "memory");
  return done != 0;
}

// Bounded wait for the CTA's copies (phase 0 of bar).  The outcome is the
// same on every thread: false if any thread gave up after `limit` polls, in
// which case the error word is set and the copies in flight have landed (or
// a second bounded wait ran out) when it returns; the caller must return.
__device__ __forceinline__ bool bulk_wait(uint64_t* bar, int* err, unsigned long long limit) {
  bool done = false;
  for (unsigned long long it = 0; it < limit && !done; ++it) done = bulk_try(bar);
  if (!__syncthreads_or(!done)) return true;
  if (threadIdx.x == 0 && err) atomicExch(err, 1);
  for (int it = 0; it < (1 << 24) && !done; ++it) done = bulk_try(bar);
  __syncthreads();
  return false;
}

}  // namespace vk
