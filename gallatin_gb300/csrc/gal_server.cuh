// gal_server.cuh — a resident allocator server: producer warps send slice
// requests through per-class rings in device memory and wait for the reply;
// server CTAs drain the rings in batches and claim each batch's slices with
// one atomicAdd per run on the class's pinned block (gal_batch.cuh's
// claim_run, spare blocks included).
//
// Producers and servers wait on one another, so they must be CTAs of ONE
// cooperative launch (cudaLaunchCooperativeKernel, or the cooperative launch
// attribute): only then are all of them resident at the same time.  Separate
// producer and server kernels are not guaranteed to run concurrently, and a
// server spinning on requests from a kernel that has not started would only
// end at its deadline.  Every wait here ends at a %globaltimer deadline, sets
// SERVER_ERR_TIMEOUT in the rings' status word and returns.
//
// Rings: class t has 2^cap_shift entries; position p of class t lives in
// entry p mod 2^cap_shift and holds (lap << 40) | (reply slot + 1), lap =
// p >> cap_shift (mod 2^24), 0 when empty.  A producer reserves positions
// with atomicAdd on the class's tail (one per warp team), waits for its entry
// to be empty (the server of the previous lap clears it) and publishes the
// request; a server takes positions with a CAS on the class's `taken`
// counter, waits for each entry to carry its own lap, answers in the reply
// slot (the pointer, or 1 for no memory) and clears the entry.
#pragma once

#include "gal_batch.cuh"

namespace gal {

static constexpr uint32_t SERVER_ERR_TIMEOUT = 0x1u;
static constexpr int SERVER_RUNS = 8;  // runs a server batch may use per class

struct server_rings {
  unsigned long long *entries;   // [num_trees << cap_shift]
  unsigned long long *tail;      // positions reserved by producers, class t at t * 4 (own sector)
  unsigned long long *taken;     // positions taken by servers, class t at t * 4
  unsigned long long *reply;     // per reply slot: 0 pending, 1 no memory, else the pointer
  uint32_t *producers_left;      // producer CTAs not yet finished
  uint32_t *status;              // SERVER_ERR_* bits
  uint32_t cap_shift;            // ring capacity 2^cap_shift per class
  uint64_t deadline_ns;          // every wait gives up this long after the kernel began
};

GAL_DEVICE_INLINE uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
GAL_DEVICE_INLINE unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
GAL_DEVICE_INLINE void st_release(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
GAL_DEVICE_INLINE unsigned long long ring_entry(uint64_t pos, uint32_t cap_shift, uint64_t slot) {
  return ((unsigned long long)((pos >> cap_shift) & 0xFFFFFFull) << 40) | (slot + 1);
}

// A producer lane's request for `size` bytes, answered by a server CTA of the
// same launch.  `slot` is the lane's own reply slot (one request in flight per
// slot).  Sizes that are not single slices take the per-thread path.  Called
// by any subset of a warp's lanes; `t0` is the kernel's start time.
GAL_DEVICE_INLINE void *server_malloc(const state *s, const server_rings &r, uint64_t size, uint64_t slot,
                                      uint64_t t0) {
  const int bits = ceil_log2(size);
  const int t = (size >> s->min_shift) == 0 ? 0 : bits - (int)s->min_shift;
  if (t >= (int)s->num_trees) return gal::malloc(s, size);
  r.reply[slot] = 0ull;
  const uint32_t callers = active_lanes();
  const uint32_t team = __match_any_sync(callers, t);
  const int leader = __ffs(team) - 1;
  unsigned long long base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(r.tail + (uint64_t)t * 4, (unsigned long long)__popc(team));
  base = __shfl_sync(callers, base, leader);
  const uint64_t pos = base + (uint64_t)__popc(team & lanemask_lt());
  unsigned long long *e = r.entries + ((uint64_t)t << r.cap_shift) + (pos & ((1ull << r.cap_shift) - 1));
  for (uint32_t i = 0; ld_acquire(e) != 0ull; i++) {  // the previous lap's request still unserved
    if (global_ns() - t0 > r.deadline_ns) {
      atomicOr(r.status, SERVER_ERR_TIMEOUT);
      return nullptr;
    }
    __nanosleep(i < 4 ? 64 : 512);
  }
  st_release(e, ring_entry(pos, r.cap_shift, slot));
  unsigned long long v;
  for (uint32_t i = 0; (v = ld_acquire(r.reply + slot)) == 0ull; i++) {
    if (global_ns() - t0 > r.deadline_ns) {
      atomicOr(r.status, SERVER_ERR_TIMEOUT);
      return nullptr;
    }
    __nanosleep(i < 8 ? 32 : 256);
  }
  return v == 1ull ? nullptr : (void *)v;
}

struct server_smem {
  run_cache runs;                    // the block of each class's last run
  unsigned long long first;          // first position of the batch
  uint32_t count;                    // requests in the batch
  uint32_t nruns;
  uint32_t run_blk[SERVER_RUNS], run_start[SERVER_RUNS], run_len[SERVER_RUNS];
  uint32_t spare_slot[SERVER_RUNS];
  uint32_t served, stop;
};

// Takes up to `most` positions of class t that producers have reserved;
// returns how many (first position in *first).  One thread.
GAL_DEVICE_INLINE uint32_t server_take(const server_rings &r, uint32_t t, uint32_t most, unsigned long long *first) {
  unsigned long long *tk = r.taken + (uint64_t)t * 4;
  unsigned long long cur = ld_acquire(tk);
  for (int a = 0; a < 8; a++) {
    const unsigned long long tl = ld_acquire(r.tail + (uint64_t)t * 4);
    if (tl <= cur) return 0;
    const uint32_t m = (uint32_t)min(tl - cur, (unsigned long long)most);
    const unsigned long long seen = atomicCAS(tk, cur, cur + m);
    if (seen == cur) {
      *first = cur;
      return m;
    }
    cur = seen;
  }
  return 0;
}

// The server loop of one CTA (every thread calls it): sweeps the classes,
// serves a batch of up to blockDim.x requests of a class at a time, and
// returns once no producer is left and every reserved position is served,
// or at the deadline.
GAL_DEVICE_INLINE void server_loop(const state *s, const server_rings &r, server_smem &sm, uint64_t t0) {
  const uint32_t T = s->num_trees;
  run_cache_init(sm.runs);
  if (threadIdx.x == 0) sm.stop = 0;
  if (threadIdx.x < SERVER_RUNS) sm.spare_slot[threadIdx.x] = NOBLK;
  __syncthreads();
  for (uint32_t sweep = 0;; sweep++) {
    if (threadIdx.x == 0) sm.served = 0;
    for (uint32_t k = 0; k < T; k++) {
      const uint32_t t = (k + blockIdx.x) % T;  // servers start their sweeps on different classes
      if (threadIdx.x == 0) {
        sm.count = server_take(r, t, blockDim.x, &sm.first);
        sm.nruns = 0;
        uint32_t need = sm.count;
        while (need && sm.nruns < SERVER_RUNS) {  // one atomicAdd per run on the pinned block
          uint32_t blk, start, spare_slot;
          const uint32_t got = claim_run(s, t, need, sm.runs, blk, start, spare_slot);
          sm.spare_slot[sm.nruns] = spare_slot;
          if (!got) break;
          sm.run_blk[sm.nruns] = blk;
          sm.run_start[sm.nruns] = start;
          sm.run_len[sm.nruns] = got;
          sm.nruns++;
          need -= got;
        }
        sm.served += sm.count;
      }
      __syncthreads();
      const uint32_t m = sm.count;
      if (threadIdx.x < m) {
        const uint64_t pos = sm.first + threadIdx.x;
        unsigned long long *e = r.entries + ((uint64_t)t << r.cap_shift) + (pos & ((1ull << r.cap_shift) - 1));
        const unsigned long long lap = (pos >> r.cap_shift) & 0xFFFFFFull;
        unsigned long long v;
        bool ok = true;
        for (uint32_t i = 0; ((v = ld_acquire(e)) >> 40) != lap || v == 0ull; i++) {  // not yet published
          if (global_ns() - t0 > r.deadline_ns) {
            atomicOr(r.status, SERVER_ERR_TIMEOUT);
            ok = false;
            break;
          }
          __nanosleep(i < 4 ? 32 : 256);
        }
        if (ok) {
          uint32_t j = threadIdx.x;
          void *p = nullptr;
          for (uint32_t q = 0; q < sm.nruns; q++) {
            if (j < sm.run_len[q]) {
              p = slice_ptr(s, sm.run_blk[q], sm.run_start[q] + j, t);
              break;
            }
            j -= sm.run_len[q];
          }
          if (!p) p = malloc_slices<false>(s, t, 1, active_lanes());  // the runs fell short
          if (p && s->zero_fill) zero_fill(p, 1ull << (s->min_shift + t));  // the whole slice
          const uint64_t slot = (v & ((1ull << 40) - 1)) - 1;
          st_release(e, 0ull);  // the entry is free for the next lap
          st_release(r.reply + slot, p ? (unsigned long long)p : 1ull);
        }
      }
      __syncthreads();
      if (threadIdx.x == 0)  // spare blocks of the runs that crossed a block's end
        for (uint32_t q = 0; q <= sm.nruns && q < SERVER_RUNS; q++)
          if (sm.spare_slot[q] != NOBLK) {
            refill_spare(s, t, sm.spare_slot[q], thread_linear_id());
            sm.spare_slot[q] = NOBLK;
          }
    }
    if (threadIdx.x == 0) {
      bool done = ld_rlx(r.producers_left) == 0u;
      for (uint32_t t = 0; done && t < T; t++)
        done = ld_acquire(r.taken + (uint64_t)t * 4) >= ld_acquire(r.tail + (uint64_t)t * 4);
      if (done || global_ns() - t0 > r.deadline_ns) sm.stop = 1;
      else if (sm.served == 0) __nanosleep(256);
    }
    __syncthreads();
    if (sm.stop) break;
  }
}

}  // namespace gal
