// churn.cuh — the mixed-size churn workload (16 B–4 KiB, 50% random frees
// per round, uint32 payload written and checked) as device bodies templated
// over the allocator, so the plain per-thread path of this library and the
// reference build run literally the same request code.
//
// Alloc must provide  void* malloc(uint64_t)  and  void free(void*).
// PAYLOAD = false gives the allocator-only form: the same requests, frees and
// pointer stores, without the payload word written at malloc and checked at
// free.
#pragma once
#include <stdint.h>

#include "workload.cuh"

namespace galwl {

// Counters of a run: [0] mallocs ok, [1] mallocs failed, [2] payload
// mismatches, [3] frees.  Every warp adds to them, so each counter is kept in
// STAT_SHARDS copies chosen by SM, each in a 32-byte sector of its own (the
// adds of one kernel would otherwise queue on four words); the host sums the
// copies (stat_total).  A buffer holds STAT_WORDS 64-bit words.
constexpr int STAT_SHARDS = 64;
constexpr int STAT_WORDS = STAT_SHARDS * 4 * 4;

__device__ __forceinline__ unsigned long long *stat_word(unsigned long long *stats, int which) {
  uint32_t smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  return stats + ((smid % STAT_SHARDS) * 4 + (uint32_t)which) * 4;
}

inline uint64_t stat_total(const unsigned long long *host_stats, int which) {
  uint64_t t = 0;
  for (int sh = 0; sh < STAT_SHARDS; sh++) t += host_stats[(sh * 4 + which) * 4];
  return t;
}

__device__ __forceinline__ void warp_count(unsigned long long *stats, int which, bool flag) {
  unsigned mask;
  asm volatile("activemask.b32 %0;" : "=r"(mask));  // read once, where written
  unsigned b = __ballot_sync(mask, flag);
  int leader = __ffs(mask) - 1;
  if ((int)(threadIdx.x & 31) == leader && b) atomicAdd(stat_word(stats, which), (unsigned long long)__popc(b));
}

// Slot liveness: bit (i & 31) of live_bits[i >> 5] is set while slot i holds
// a live allocation.  A round's mallocs write the words of their slots, one
// word per warp of 32 consecutive slots; a free phase reads the words (8 MiB
// for 64 Mi slots, so they stay in L2), loads pointer and payload of the
// slots it frees only, and clears their bits.  Slots freed in earlier rounds
// are thus never read again.  Rounds are a multiple of SLOT_ALIGN requests,
// so every warp covers whole words (and whole coin groups) or none.
constexpr uint64_t SLOT_ALIGN = 128;

// one full warp, lane l holding slot (slot & ~31) + l
__device__ __forceinline__ void publish_live(uint32_t *live_bits, uint64_t slot, bool live) {
  const uint32_t b = __ballot_sync(0xFFFFFFFFu, live);
  if ((threadIdx.x & 31) == 0) live_bits[slot >> 5] = b;
}

template <class Alloc, bool PAYLOAD = true>
__device__ __forceinline__ void churn_malloc_body(Alloc *a, void **ptrs, uint32_t *live_bits,
                                                  uint64_t base, uint64_t n, uint32_t seed,
                                                  unsigned long long *stats) {
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;  // whole warps: n is a multiple of SLOT_ALIGN
  uint64_t slot = base + tid;
  uint64_t size = mixed_size(slot, seed);
  void *p = a->malloc(size);
  if (PAYLOAD && p) *(volatile uint32_t *)p = payload(slot, seed);
  ptrs[slot] = p;
  publish_live(live_bits, slot, p != nullptr);
  warp_count(stats, 0, p != nullptr);
  warp_count(stats, 1, p == nullptr);
}

__device__ __forceinline__ void warp_add(unsigned long long *stats, int which, uint32_t n) {
  unsigned mask;
  asm volatile("activemask.b32 %0;" : "=r"(mask));
  uint32_t total = __reduce_add_sync(mask, n);
  int leader = __ffs(mask) - 1;
  if ((int)(threadIdx.x & 31) == leader && total) atomicAdd(stat_word(stats, which), (unsigned long long)total);
}

// Each thread of the free phase owns FREE_SLOTS consecutive slots: one vector
// load of their pointers, one Philox group of coins for all of them.
constexpr int FREE_SLOTS = 4;

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

constexpr uint32_t GROUP_MASK = (1u << FREE_SLOTS) - 1u;
constexpr int GROUPS_PER_WORD = 32 / FREE_SLOTS;
static_assert(32 % FREE_SLOTS == 0, "a thread's slots sit inside one liveness word");

// The slots of i0..i0+FREE_SLOTS-1 to free: live ones, and of those the ones
// whose coin (one Philox call per 128 slots) came up, or all on the drain.
__device__ __forceinline__ uint32_t select_frees(uint32_t word, uint64_t i0, uint32_t round,
                                                 uint32_t seed, bool all) {
  uint32_t sel = (word >> (i0 & 31)) & GROUP_MASK;
  if (sel && !all) {
    u32x4 coins = free_coin_group(i0 >> 7, round, seed);
    sel &= (coins.v[(i0 >> 5) & 3u] >> (i0 & 31)) & GROUP_MASK;
  }
  return sel;
}

// Clears the freed bits: the GROUPS_PER_WORD lanes sharing a word OR their
// masks together and the first of them stores the word.  Full warp.
__device__ __forceinline__ void clear_live(uint32_t *live_bits, uint64_t i0, uint32_t word,
                                           uint32_t sel) {
  uint32_t cleared = sel << (i0 & 31);
#pragma unroll
  for (int o = 1; o < GROUPS_PER_WORD; o <<= 1) cleared |= __shfl_xor_sync(0xFFFFFFFFu, cleared, o);
  if ((threadIdx.x & (GROUPS_PER_WORD - 1)) == 0 && cleared) live_bits[i0 >> 5] = word & ~cleared;
}

// The free phase, persistent: each warp takes 1,024 slots (32 liveness words)
// at a time.  Lane l reads word l, draws its coins (one Philox call gives the
// coins of 128 slots, so word w uses lane w & 3 of group w >> 2) and clears the
// bits it frees; the selected slots go, in slot order, to the warp's list in
// shared memory, and the lanes then free them FREE_SLOTS at a time, lane l
// taking entries l, l + 32, ... so that neighbouring lanes hold neighbouring
// slots (which share blocks).  Dead and unselected slots cost one bit of an
// L2-resident word; every lane has a request to serve while any is left.
// all == true frees every live slot (drain); otherwise a fair coin per slot.
constexpr int WARP_WORDS = 32;
constexpr int WARP_SLOTS = 32 * WARP_WORDS;

// One warp's 1,024 slots from word w0: reads and clears the liveness words of
// the slots it selects and lists the selected slots (offsets from w0 * 32) in
// slot order; returns how many.  Full warp.
__device__ __forceinline__ uint32_t list_selected(uint32_t *live_bits, uint64_t words, uint64_t w0,
                                                  uint32_t round, uint32_t seed, bool all,
                                                  uint16_t *list) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t w = w0 + lane;
  const uint32_t word = w < words ? live_bits[w] : 0u;
  uint32_t sel = word;
  if (sel && !all) sel &= free_coin_group(w >> 2, round, seed).v[w & 3u];
  if (sel) live_bits[w] = word & ~sel;
  const uint32_t n = (uint32_t)__popc(sel);
  uint32_t end = n;  // inclusive scan of the counts
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_up_sync(0xFFFFFFFFu, end, o);
    if ((int)lane >= o) end += v;
  }
  uint32_t pos = end - n;
  for (uint32_t b = sel; b; b &= b - 1u) list[pos++] = (uint16_t)(lane * 32u + (uint32_t)__ffs(b) - 1u);
  __syncwarp();
  return __shfl_sync(0xFFFFFFFFu, end, 31);
}

// Pointers and payload words of list entries j0 + k*32 + lane (k < FREE_SLOTS),
// loads issued together; go[k] marks the entries that exist.
template <bool PAYLOAD = true>
__device__ __forceinline__ void load_listed(void **ptrs, uint64_t w0, const uint16_t *list,
                                            uint32_t total, uint32_t j0, uint32_t seed, void **p,
                                            bool *go, uint32_t &nbad, uint32_t &ngo) {
  const uint32_t lane = threadIdx.x & 31u;
  uint64_t slot[FREE_SLOTS];
  uint32_t seen[FREE_SLOTS];
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++) {
    const uint32_t j = j0 + (uint32_t)k * 32u + lane;
    slot[k] = j < total ? w0 * 32u + list[j] : 0;
    p[k] = j < total ? ptrs[slot[k]] : nullptr;
  }
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++) {
    go[k] = p[k] != nullptr;
    seen[k] = PAYLOAD && go[k] ? *(const uint32_t *)p[k] : 0u;
  }
#pragma unroll
  for (int k = 0; k < FREE_SLOTS; k++)
    if (go[k]) {
      if (PAYLOAD) nbad += seen[k] != payload(slot[k], seed);
      ngo++;
    }
}

template <class Alloc, bool PAYLOAD = true>
__device__ __forceinline__ void churn_free_warps(Alloc *a, void **ptrs, uint32_t *live_bits,
                                                 uint64_t nslots, uint32_t round, uint32_t seed,
                                                 bool all, unsigned long long *stats,
                                                 uint16_t *list /* WARP_SLOTS entries */) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t words = nslots >> 5;
  uint32_t nbad = 0, ngo = 0;
  for (uint64_t w0 = warp * WARP_WORDS; w0 < words; w0 += nwarps * WARP_WORDS) {
    const uint32_t total = list_selected(live_bits, words, w0, round, seed, all, list);
    for (uint32_t j0 = 0; j0 < total; j0 += 32u * FREE_SLOTS) {
      void *p[FREE_SLOTS];
      bool go[FREE_SLOTS];
      load_listed<PAYLOAD>(ptrs, w0, list, total, j0, seed, p, go, nbad, ngo);
      free_many<Alloc>::run(a, p, go);
    }
    __syncwarp();
  }
  warp_add(stats, 2, nbad);
  warp_add(stats, 3, ngo);
}

// The same selection, but the selected pointers are appended to freelist
// (*count entries so far; one atomicAdd per warp and chunk) for a batched
// free call to serve; payloads are checked here.
__device__ __forceinline__ void churn_select_warps(void **ptrs, uint32_t *live_bits, uint64_t lo_slots,
                                                   uint64_t nslots, uint32_t round, uint32_t seed, bool all,
                                                   unsigned long long *stats, uint16_t *list,
                                                   void **freelist, unsigned long long *count) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t words = nslots >> 5;
  uint32_t nbad = 0, ngo = 0;
  for (uint64_t w0 = (lo_slots >> 5) + warp * WARP_WORDS; w0 < words; w0 += nwarps * WARP_WORDS) {
    const uint32_t total = list_selected(live_bits, words, w0, round, seed, all, list);
    if (total == 0) continue;  // warp-uniform
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)total);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    for (uint32_t j0 = 0; j0 < total; j0 += 32u * FREE_SLOTS) {
      void *p[FREE_SLOTS];
      bool go[FREE_SLOTS];
      load_listed(ptrs, w0, list, total, j0, seed, p, go, nbad, ngo);
#pragma unroll
      for (int k = 0; k < FREE_SLOTS; k++) {
        const uint32_t j = j0 + (uint32_t)k * 32u + lane;
        if (j < total) freelist[base + j] = p[k];
      }
    }
    __syncwarp();
  }
  warp_add(stats, 2, nbad);
  warp_add(stats, 3, ngo);
}

}  // namespace galwl
