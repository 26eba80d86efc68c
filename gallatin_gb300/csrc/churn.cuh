// churn.cuh — the mixed-size churn workload (16 B–4 KiB, 50% random frees
// per round, uint32 payload written and checked) as device bodies templated
// over the allocator, so the plain per-thread path of this library and the
// reference build run literally the same request code.
//
// Alloc must provide  void* malloc(uint64_t)  and  void free(void*).
#pragma once
#include <stdint.h>

#include "workload.cuh"

namespace galwl {

// stats[0] mallocs ok, [1] mallocs failed, [2] payload mismatches, [3] frees
__device__ __forceinline__ void warp_count(unsigned long long *ctr, bool flag) {
  unsigned mask;
  asm volatile("activemask.b32 %0;" : "=r"(mask));  // read once, where written
  unsigned b = __ballot_sync(mask, flag);
  int leader = __ffs(mask) - 1;
  if ((int)(threadIdx.x & 31) == leader && b) atomicAdd(ctr, (unsigned long long)__popc(b));
}

template <class Alloc>
__device__ __forceinline__ void churn_malloc_body(Alloc *a, void **ptrs, uint64_t base, uint64_t n,
                                                  uint32_t seed, unsigned long long *stats) {
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  uint64_t slot = base + tid;
  uint64_t size = mixed_size(slot, seed);
  void *p = a->malloc(size);
  if (p) *(volatile uint32_t *)p = payload(slot, seed);
  ptrs[slot] = p;
  warp_count(&stats[0], p != nullptr);
  warp_count(&stats[1], p == nullptr);
}

// all == true frees every live slot (drain); otherwise a fair coin per slot.
template <class Alloc>
__device__ __forceinline__ void churn_free_body(Alloc *a, void **ptrs, uint64_t nslots,
                                                uint32_t round, uint32_t seed, bool all,
                                                unsigned long long *stats) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nslots) return;
  void *p = ptrs[i];
  bool go = p != nullptr && (all || free_coin(i, round, seed));
  bool bad = false;
  if (go) {
    bad = *(volatile uint32_t *)p != payload(i, seed);
    a->free(p);
    ptrs[i] = nullptr;
  }
  warp_count(&stats[2], bad);
  warp_count(&stats[3], go);
}

}  // namespace galwl
