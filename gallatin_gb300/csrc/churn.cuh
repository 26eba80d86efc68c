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

__device__ __forceinline__ void warp_add(unsigned long long *ctr, uint32_t n) {
  unsigned mask;
  asm volatile("activemask.b32 %0;" : "=r"(mask));
  uint32_t total = __reduce_add_sync(mask, n);
  int leader = __ffs(mask) - 1;
  if ((int)(threadIdx.x & 31) == leader && total) atomicAdd(ctr, (unsigned long long)total);
}

// Each thread of the free phase owns FREE_SLOTS consecutive slots: one vector
// load of their pointers, one Philox group of coins for all of them.
constexpr int FREE_SLOTS = 4;

__device__ __forceinline__ uint64_t free_threads(uint64_t nslots) {
  return (nslots + FREE_SLOTS - 1) / FREE_SLOTS;
}

static_assert(FREE_SLOTS % 2 == 0 && FREE_SLOTS <= 128, "slots come in 16-byte pairs within a coin group");

// i0 is a multiple of FREE_SLOTS, so whole pairs are 16-byte aligned
__device__ __forceinline__ void load_slots(void **ptrs, uint64_t i0, uint64_t nslots, void *p[FREE_SLOTS]) {
  if (i0 + FREE_SLOTS <= nslots) {
#pragma unroll
    for (int k = 0; k < FREE_SLOTS; k += 2) {
      ulonglong2 a = *(const ulonglong2 *)(ptrs + i0 + k);
      p[k] = (void *)a.x;
      p[k + 1] = (void *)a.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < FREE_SLOTS; k++) p[k] = i0 + k < nslots ? ptrs[i0 + k] : nullptr;
  }
}

// How an allocator frees one thread's FREE_SLOTS pointers (go[k] selects);
// the default frees them one after another.  An allocator may specialise this
// to overlap the work of the several frees.
template <class Alloc>
struct free_many {
  static __device__ __forceinline__ void run(Alloc *a, void *const (&p)[FREE_SLOTS], const bool (&go)[FREE_SLOTS]) {
#pragma unroll
    for (int k = 0; k < FREE_SLOTS; k++)
      if (go[k]) a->free(p[k]);
  }
};

// all == true frees every live slot (drain); otherwise a fair coin per slot.
template <class Alloc>
__device__ __forceinline__ void churn_free_body(Alloc *a, void **ptrs, uint64_t nslots,
                                                uint32_t round, uint32_t seed, bool all,
                                                unsigned long long *stats) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t i0 = t * FREE_SLOTS;
  if (i0 >= nslots) return;
  void *p[FREE_SLOTS];
  load_slots(ptrs, i0, nslots, p);
  u32x4 coins = all ? u32x4{{~0u, ~0u, ~0u, ~0u}} : free_coin_group(i0 >> 7, round, seed);
  bool go[FREE_SLOTS];
  uint32_t seen[FREE_SLOTS];
  uint32_t nbad = 0, ngo = 0;
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++) go[k] = p[k] != nullptr && coin_bit(coins, i0 + k);
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++) seen[k] = go[k] ? *(const uint32_t *)p[k] : 0u;  // loads in flight together
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++)
    if (go[k]) {
      nbad += seen[k] != payload(i0 + k, seed);
      ptrs[i0 + k] = nullptr;
      ngo++;
    }
  free_many<Alloc>::run(a, p, go);
  warp_add(&stats[2], nbad);
  warp_add(&stats[3], ngo);
}

}  // namespace galwl
