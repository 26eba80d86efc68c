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
// p >> cap_shift (mod 2^24), while a request waits in it, and lap << 40 (slot
// bits zero) while it is free for that lap.  A producer reserves positions
// with atomicAdd on the class's tail (one per warp team), waits for its entry
// to be free for its own lap (the server of the previous lap hands it on) and
// publishes the request; a server takes positions with a CAS on the class's
// `taken` counter, waits for each entry to carry its own lap's request,
// answers in the reply slot (the pointer, or 1 for no memory) and hands the
// entry to the next lap.  Naming the lap in the free state matters once the
// ring wraps: with a bare "empty", a request of the next lap could take an
// entry whose own lap was still waiting to publish, and a server warp holding
// that position while it answers a batch in order could wait on the server
// warp that needs the later request answered first.
#pragma once

#include "gal_batch.cuh"

namespace gal {

static constexpr uint32_t SERVER_ERR_TIMEOUT = 0x1u;
// positions a server warp takes at once (its lanes answer them 32 at a time):
// with many server warps a take of one warp's width left most takes a few
// requests each, and the warps spent their time contending on the classes'
// `taken` counters instead of answering
static constexpr uint32_t SERVER_BATCH = 256;

struct server_rings {
  unsigned long long *entries;   // [num_trees << cap_shift]
  unsigned long long *tail;      // positions reserved by producers, class t at t * ctr_stride
  unsigned long long *taken;     // positions taken by servers, class t at t * ctr_stride
  unsigned long long *reply;     // per reply slot: 0 pending, 1 no memory, else the pointer
  uint32_t *producers_left;      // producer CTAs not yet finished
  uint32_t *status;              // SERVER_ERR_* bits
  uint32_t cap_shift;            // ring capacity 2^cap_shift per class
  uint32_t ctr_stride;           // words between consecutive classes' counters
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
GAL_DEVICE_INLINE unsigned long long ring_lap(uint64_t pos, uint32_t cap_shift) {
  return (unsigned long long)((pos >> cap_shift) & 0xFFFFFFull);
}
GAL_DEVICE_INLINE unsigned long long ring_entry(uint64_t pos, uint32_t cap_shift, uint64_t slot) {
  return (ring_lap(pos, cap_shift) << 40) | (slot + 1);
}
// the entry free for the lap of `pos` (all zero for lap 0, the state at set-up)
GAL_DEVICE_INLINE unsigned long long ring_free(uint64_t pos, uint32_t cap_shift) {
  return ring_lap(pos, cap_shift) << 40;
}

// A producer lane's request for `size` bytes, sent to the server CTAs of the
// same launch: returns true once the request is in its class's ring (its
// answer then comes from server_wait on the same `slot`), false when it was
// served here (*direct: sizes that are not single slices take the per-thread
// path) or the wait for a free entry ran out (*direct = nullptr).  `slot` is
// a reply slot of the lane's own, with one request in flight per slot; a lane
// may post into several slots before it waits.  Called by any subset of a
// warp's lanes; `t0` is the kernel's start time.
GAL_DEVICE_INLINE bool server_post(const state *s, const server_rings &r, uint64_t size, uint64_t slot, uint64_t t0,
                                   void **direct) {
  const int bits = ceil_log2(size);
  const int t = (size >> s->min_shift) == 0 ? 0 : bits - (int)s->min_shift;
  *direct = nullptr;
  if (t >= (int)s->num_trees) {
    *direct = gal::malloc(s, size);
    return false;
  }
  r.reply[slot] = 0ull;
  const uint32_t callers = active_lanes();
  const uint32_t team = __match_any_sync(callers, t);
  const int leader = __ffs(team) - 1;
  unsigned long long base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(r.tail + (uint64_t)t * r.ctr_stride, (unsigned long long)__popc(team));
  base = __shfl_sync(callers, base, leader);
  const uint64_t pos = base + (uint64_t)__popc(team & lanemask_lt());
  unsigned long long *e = r.entries + ((uint64_t)t << r.cap_shift) + (pos & ((1ull << r.cap_shift) - 1));
  const unsigned long long mine = ring_free(pos, r.cap_shift);
  for (uint32_t i = 0; ld_acquire(e) != mine; i++) {  // the previous lap's request still unserved
    if (global_ns() - t0 > r.deadline_ns) {
      atomicOr(r.status, SERVER_ERR_TIMEOUT);
      return false;
    }
    __nanosleep(i < 4 ? 64 : 512);
  }
  st_release(e, ring_entry(pos, r.cap_shift, slot));
  return true;
}

// The answer to the request posted into `slot` (nullptr: no memory, or the
// wait ran out).
GAL_DEVICE_INLINE void *server_wait(const server_rings &r, uint64_t slot, uint64_t t0) {
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

// One request, posted and waited for.
GAL_DEVICE_INLINE void *server_malloc(const state *s, const server_rings &r, uint64_t size, uint64_t slot,
                                      uint64_t t0) {
  void *direct;
  return server_post(s, r, size, slot, t0, &direct) ? server_wait(r, slot, t0) : direct;
}

// Takes up to `most` positions of class t that producers have reserved;
// returns how many (first position in *first).  One thread.
GAL_DEVICE_INLINE uint32_t server_take(const server_rings &r, uint32_t t, uint32_t most, unsigned long long *first) {
  unsigned long long *tk = r.taken + (uint64_t)t * r.ctr_stride;
  unsigned long long cur = ld_acquire(tk);
  for (int a = 0; a < 8; a++) {
    const unsigned long long tl = ld_acquire(r.tail + (uint64_t)t * r.ctr_stride);
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

// Per server warp, the block of each class's last run (shared memory).
struct server_smem {
  run_cache runs[32];  // indexed by warp within the CTA (up to 1,024 threads)
};

// The server loop (every thread of a server CTA calls it).  Each warp serves
// on its own, without CTA barriers: it sweeps the classes, starting at a
// class of its own, takes a batch of up to SERVER_BATCH reserved positions of
// a class, claims their slices with one atomicAdd per run (lane 0), and the
// lanes answer the requests 32 at a time.  Returns once no producer is left and every reserved
// position is served, or at the deadline.
GAL_DEVICE_INLINE void server_loop(const state *s, const server_rings &r, server_smem &sm, uint64_t t0) {
  const uint32_t T = s->num_trees;
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  run_cache &rc = sm.runs[warp];
  if (lane < GAL_MAX_TREES) {
    rc.blk[lane] = NOBLK;
    rc.slot[lane] = 0;
  }
  __syncwarp();
  const uint32_t first_class = (blockIdx.x * (blockDim.x >> 5) + warp) % T;
  for (uint32_t sweep = 0;; sweep++) {
    uint32_t served = 0;
    for (uint32_t k = 0; k < T; k++) {
      const uint32_t t = (first_class + k) % T;
      unsigned long long first = 0;
      uint32_t m = 0, nruns = 0, spare_slot[2] = {NOBLK, NOBLK};
      uint32_t rb[2] = {NOBLK, NOBLK}, rs[2] = {0, 0}, rl[2] = {0, 0};
      if (lane == 0) {
        m = server_take(r, t, SERVER_BATCH, &first);
        uint32_t need = m;
        while (need && nruns < 2) {  // at most SERVER_BATCH slices: one crossing of a block's end
          uint32_t blk, start, ss;
          const uint32_t got = claim_run(s, t, need, rc, blk, start, ss);
          spare_slot[nruns] = ss;
          if (!got) break;
          rb[nruns] = blk;
          rs[nruns] = start;
          rl[nruns] = got;
          nruns++;
          need -= got;
        }
      }
      m = __shfl_sync(0xFFFFFFFFu, m, 0);
      if (m == 0) continue;
      served += m;
      first = __shfl_sync(0xFFFFFFFFu, first, 0);
      const uint32_t b0 = __shfl_sync(0xFFFFFFFFu, rb[0], 0), b1 = __shfl_sync(0xFFFFFFFFu, rb[1], 0);
      const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, rs[0], 0), s1 = __shfl_sync(0xFFFFFFFFu, rs[1], 0);
      const uint32_t l0 = __shfl_sync(0xFFFFFFFFu, rl[0], 0), l1 = __shfl_sync(0xFFFFFFFFu, rl[1], 0);
      for (uint32_t j = lane; j < ((m + 31u) & ~31u); j += 32u) {  // whole warps each pass
        if (j < m) {
          const uint64_t pos = first + j;
          unsigned long long *e = r.entries + ((uint64_t)t << r.cap_shift) + (pos & ((1ull << r.cap_shift) - 1));
          const unsigned long long lap = ring_lap(pos, r.cap_shift);
          unsigned long long v;
          bool ok = true;
          for (uint32_t i = 0; ((v = ld_acquire(e)) >> 40) != lap || (v & ((1ull << 40) - 1)) == 0ull;
               i++) {  // not yet published
            if (global_ns() - t0 > r.deadline_ns) {
              atomicOr(r.status, SERVER_ERR_TIMEOUT);
              ok = false;
              break;
            }
            __nanosleep(i < 4 ? 32 : 256);
          }
          if (ok) {
            void *p = nullptr;
            if (j < l0) p = slice_ptr(s, b0, s0 + j, t);
            else if (j < l0 + l1) p = slice_ptr(s, b1, s1 + j - l0, t);
            else p = malloc_slices<false>(s, t, 1, active_lanes());  // the runs fell short
            if (p && s->zero_fill) zero_fill(p, 1ull << (s->min_shift + t));  // the whole slice
            const uint64_t slot = (v & ((1ull << 40) - 1)) - 1;
            st_release(e, ring_free(pos + (1ull << r.cap_shift), r.cap_shift));  // free for the next lap
            st_release(r.reply + slot, p ? (unsigned long long)p : 1ull);
          }
        }
        __syncwarp();
      }
      if (lane == 0)  // spare blocks of the runs that crossed a block's end, after the replies
        for (int q = 0; q < 2; q++)
          if (spare_slot[q] != NOBLK) refill_spare(s, t, spare_slot[q], thread_linear_id());
    }
    int stop = 0;
    if (lane == 0) {
      bool done = ld_rlx(r.producers_left) == 0u;
      for (uint32_t t = 0; done && t < T; t++)
        done = ld_acquire(r.taken + (uint64_t)t * r.ctr_stride) >= ld_acquire(r.tail + (uint64_t)t * r.ctr_stride);
      stop = done || global_ns() - t0 > r.deadline_ns;
      if (!stop && served == 0) __nanosleep(256);
    }
    if (__shfl_sync(0xFFFFFFFFu, stop, 0)) break;
  }
}

}  // namespace gal
