// fst_tma.cuh — tensor-memory-accelerator (TMA) plane loads and mbarrier
// waits for sm_103a, in inline PTX.
//
// A plane tile is one z-plane of a box of consecutive fields of a 4D tensor
// (x, y, z, field) described by a CUtensorMap.  One elected thread arms an
// mbarrier with the byte count and issues the copy; every thread then waits
// on the barrier's phase.  Waits are bounded: after FST_TMA_SPIN polls the
// kernel records FST_DEVERR_TMA_TIMEOUT in its error word and the caller
// returns, so a lost copy can never hang the GPU.
#pragma once
#include <cuda.h>  // CUtensorMap (type only; no driver library is linked)
#include <cuda_runtime.h>
#include <stdint.h>

#define FST_TMA_SPIN (1u << 22)
#define FST_DEVERR_TMA_TIMEOUT 1u

namespace fsttma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Make barrier initialisation visible to the async proxy (the TMA unit).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same memory.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// 4D tiled load of the box at (x, y, z, f) into shared memory; completion
// is signalled on `bar` as transaction bytes.  x * 4 bytes must be a
// multiple of 16 (the caller rounds x down to a multiple of 4 floats).
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z, int f) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z), "r"(f)
      : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`.  Returns false (and records the
// timeout in *err) if the phase did not complete within FST_TMA_SPIN polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned int* err) {
  for (uint32_t n = 0; n < FST_TMA_SPIN; ++n) {
    if (mbar_test(bar, parity)) return true;
    if (n > 64) __nanosleep(64);
  }
  if (err) atomicOr(err, FST_DEVERR_TMA_TIMEOUT);
  return false;
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

}  // namespace fsttma
