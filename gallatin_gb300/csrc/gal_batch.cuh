// gal_batch.cuh — CTA-level aggregation of allocation requests (the batched form).
//
// A CTA collects its threads' requests, ranks them per size class in shared
// memory, and one thread per class claims the whole run of slices with a single
// atomicAdd on the pinned block's malloc word (the per-thread path needs one
// atomic per warp team).  Frees are combined per block through a shared-memory
// hash so each touched block gets one free-counter atomic per CTA.
//
// Both entry points must be reached by every thread of the CTA (they contain
// CTA barriers; with a service warp, by every worker thread: see
// cta_claim_init); threads without work pass has_request = false / ptr = nullptr.
// With gal_config.spare_blocks, a service warp keeps the next block of each
// pinned slot the CTA uses prepared, so a claim that exhausts its block swaps
// the spare in instead of searching the class's segments itself.
// Requests that the aggregated path cannot serve (whole blocks, segment runs,
// multi-slice sizes, or a claim that ran out of attempts) fall back to the
// per-thread gal::malloc / gal::free of gal_device.cuh.
#pragma once

#include "../../include/gallatin_gb300/gal_device.cuh"

namespace gal {

static constexpr int CTA_RUNS = 4;          // block runs a class may use per claim
static constexpr int CTA_CLAIM_ATTEMPTS = 64;

struct cta_claim_smem {
  uint32_t cached[GAL_MAX_TREES];       // block a persistent CTA last claimed from, per class
  uint32_t cached_slot[GAL_MAX_TREES];
  uint32_t refill[GAL_MAX_TREES];       // slot whose spare the service warp should prepare
  uint32_t workers;                     // threads that call cta_malloc (the rest: service warp)
  uint32_t stop;                        // set once the workers are done
  uint32_t count[GAL_MAX_TREES];
  uint32_t nruns[GAL_MAX_TREES];
  uint32_t run_blk[GAL_MAX_TREES][CTA_RUNS];
  uint32_t run_start[GAL_MAX_TREES][CTA_RUNS];
  uint32_t run_len[GAL_MAX_TREES][CTA_RUNS];
};

// Claim `want` slices of class `tree` for this CTA; records up to CTA_RUNS runs.
static __device__ __noinline__ void cta_claim_class(const state *s, uint32_t tree, uint32_t want,
                                             cta_claim_smem &sm) {
  const uint64_t tid = thread_linear_id();
  uint32_t assigned = 0, nruns = 0;
  // a persistent CTA keeps claiming from the block it used last and reads the
  // pinned slot again only after a claim comes back exhausted or foreign
  uint32_t blk = sm.cached[tree], slot = sm.cached_slot[tree];
  for (int attempt = 0; attempt < CTA_CLAIM_ATTEMPTS && assigned < want && nruns < CTA_RUNS;
       attempt++) {
    if (blk == NOBLK) {
      slot = pick_slot(s, tree, blk);
      if (blk == NOBLK) {
        backoff((uint32_t)attempt);
        continue;
      }
    }
    uint32_t need = want - assigned;
    unsigned long long old = atomicAdd(mword_ptr(s, blk), (unsigned long long)need);
    uint64_t cnt = old & 0xFFFFFFFFull;
    if (cnt >= SLICES_PER_BLOCK) {  // exhausted; its crosser is installing a new one
      blk = NOBLK;
      __nanosleep(256);
      continue;
    }
    uint32_t got = (uint32_t)min((uint64_t)need, (uint64_t)SLICES_PER_BLOCK - cnt);
    bool crossed = cnt + need > SLICES_PER_BLOCK - 1;
    uint32_t used = blk;
    if ((uint32_t)(old >> 32) == tree) {
      sm.run_blk[tree][nruns] = blk;
      sm.run_start[tree][nruns] = (uint32_t)cnt;
      sm.run_len[tree][nruns] = got;
      nruns++;
      assigned += got;
    } else {
      credit_frees(s, blk, got);  // foreign block: give the slices back
      blk = NOBLK;
    }
    if (crossed) {
      const uint32_t si = s->slot_base[tree] + slot;
      uint32_t nx = NOBLK;
      if (s->use_spares && sm.workers != blockDim.x) nx = atomicExch(s->spares + si, NOBLK);
      if (nx != NOBLK) {  // the prepared block: one swap
        if (atomicCAS(s->slots + si, used, nx) != used) retire_block(s, nx);
      } else {
        replace_block(s, tree, slot, used, tid);
      }
      if (s->use_spares && sm.workers != blockDim.x) atomicExch(&sm.refill[tree], si);
      blk = NOBLK;
    }
  }
  sm.nruns[tree] = nruns;
  sm.cached[tree] = blk;
  sm.cached_slot[tree] = slot;
}

// Call once at the start of a kernel that uses cta_malloc, before its loop,
// followed by a __syncthreads().  workers: how many threads (a multiple of 32,
// from thread 0) call cta_malloc; the last warp beyond them, if any, runs
// cta_service.  0 = every thread of the CTA calls cta_malloc.
__device__ __forceinline__ void cta_claim_init(cta_claim_smem &sm, uint32_t workers = 0) {
  if (threadIdx.x < GAL_MAX_TREES) {
    sm.cached[threadIdx.x] = NOBLK;
    sm.cached_slot[threadIdx.x] = 0;
    sm.refill[threadIdx.x] = NOBLK;
  }
  if (threadIdx.x == 0) {
    sm.workers = workers ? workers : blockDim.x;
    sm.stop = 0;
  }
}

// barrier of the threads that call cta_malloc (named barrier 1 when a service
// warp runs beside them, which never joins it)
__device__ __forceinline__ void cta_sync(const cta_claim_smem &sm) {
  const uint32_t w = *(const volatile uint32_t *)&sm.workers;
  if (w == blockDim.x) {
    __syncthreads();
  } else {
    asm volatile("bar.sync 1, %0;" ::"r"(w) : "memory");
  }
}

// The service warp of a CTA-aggregated kernel: prepares the spare block of a
// slot whose block a claim of this CTA just replaced, off the claims' path.
// Returns when the workers set `stop` (or after a bounded number of polls).
GAL_DEVICE_COLD void cta_service(const state *s, cta_claim_smem &sm) {
  if (lane_id() != 0 || !s->use_spares) return;
  const uint64_t tid = thread_linear_id();
  for (uint32_t it = 0; it < (1u << 24); it++) {
    bool work = false;
    for (uint32_t t = 0; t < s->num_trees; t++) {
      const uint32_t si = atomicExch(&sm.refill[t], NOBLK);
      if (si == NOBLK) continue;
      work = true;
      if (ld_rlx(s->spares + si) != NOBLK) continue;
      const uint32_t nb = request_block(s, t, tid);
      if (nb == NOBLK) continue;
      __threadfence();
      if (atomicCAS(s->spares + si, NOBLK, nb) != NOBLK) retire_block(s, nb);
    }
    if (*(volatile uint32_t *)&sm.stop) return;
    if (!work) __nanosleep(256);
  }
}

// The workers' last call: after it the service warp returns.
__device__ __forceinline__ void cta_workers_done(cta_claim_smem &sm) {
  cta_sync(sm);
  if (threadIdx.x == 0) *(volatile uint32_t *)&sm.stop = 1u;
}

// Requests the CTA claim does not serve take the per-thread path, out of line
// so that it does not weigh on the claim loop's registers.
GAL_DEVICE_COLD void *malloc_fallback(const state *s, uint64_t size) { return gal::malloc(s, size); }

// Serves K requests per thread (request k of every thread of the CTA ranked
// together, one claim per class for all of them); out[k] = nullptr where
// has_request[k] is false.  More requests per call amortise the claim round
// trip and the CTA barriers over more allocations.
template <int K>
__device__ __forceinline__ void cta_malloc_n(const state *s, const uint64_t (&size)[K],
                                             const bool (&has_request)[K], cta_claim_smem &sm,
                                             void *(&out)[K]) {
  const uint32_t T = s->num_trees;
  if (threadIdx.x < GAL_MAX_TREES) sm.count[threadIdx.x] = 0;
  cta_sync(sm);
  int tree[K];
  uint32_t rank[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    tree[k] = -1;
    rank[k] = 0;
    if (has_request[k]) {
      int bits = ceil_log2(size[k]);
      int t = (size[k] >> s->min_shift) == 0 ? 0 : bits - (int)s->min_shift;
      if (t < (int)T) {
        tree[k] = t;
        rank[k] = atomicAdd(&sm.count[t], 1u);
      }
    }
  }
  cta_sync(sm);
  if (threadIdx.x < T && sm.count[threadIdx.x] > 0)
    cta_claim_class(s, threadIdx.x, sm.count[threadIdx.x], sm);
  cta_sync(sm);
#pragma unroll
  for (int k = 0; k < K; k++) {
    void *p = nullptr;
    bool fallback = has_request[k] && tree[k] < 0;
    if (tree[k] >= 0) {
      const int t = tree[k];
      uint32_t r = rank[k];
      fallback = true;
      for (uint32_t j = 0; j < sm.nruns[t]; j++) {
        uint32_t len = sm.run_len[t][j];
        if (r < len) {
          p = slice_ptr(s, sm.run_blk[t][j], sm.run_start[t][j] + r, (uint32_t)t);
          fallback = false;
          break;
        }
        r -= len;
      }
    }
    if (fallback) p = malloc_fallback(s, size[k]);  // clears its own bytes in calloc mode
    else if (p && s->zero_fill) zero_fill(p, size[k]);
    out[k] = p;
  }
  cta_sync(sm);
}

// Returns this thread's allocation (nullptr when has_request is false).
__device__ __forceinline__ void *cta_malloc(const state *s, uint64_t size, bool has_request,
                                            cta_claim_smem &sm) {
  const uint64_t sz[1] = {size};
  const bool has[1] = {has_request};
  void *out[1];
  cta_malloc_n<1>(s, sz, has, sm, out);
  return out[0];
}

// ------------------------------------------------------------ runs of slices
// The pinned block a CTA last claimed a run from, per class (claim_run).
struct run_cache {
  uint32_t blk[GAL_MAX_TREES];  // NOBLK: read the pinned slot
  uint32_t slot[GAL_MAX_TREES];
};

GAL_DEVICE_INLINE void run_cache_init(run_cache &c) {
  if (threadIdx.x < GAL_MAX_TREES) {
    c.blk[threadIdx.x] = NOBLK;
    c.slot[threadIdx.x] = 0;
  }
}

// One thread claims a run of up to `want` slices of class `tree` with one
// atomicAdd on the pinned block (the block of the CTA's last run while it
// lasts).  Returns the run's length (0: no block to be had), its block and
// first slice.  When the run crossed the end of its block and a spare block
// was swapped in, spare_slot receives the slot whose spare the caller should
// prepare again (after using the run), else NOBLK.
GAL_DEVICE_COLD uint32_t claim_run(const state *s, uint32_t tree, uint32_t want, run_cache &rc, uint32_t &run_blk,
                                   uint32_t &run_start, uint32_t &spare_slot) {
  const uint64_t tid = thread_linear_id();
  uint32_t blk = rc.blk[tree], slot = rc.slot[tree];
  spare_slot = NOBLK;
  for (int attempt = 0; attempt < CTA_CLAIM_ATTEMPTS; attempt++) {
    if (blk == NOBLK) {
      slot = pick_slot(s, tree, blk);
      if (blk == NOBLK) {
        backoff((uint32_t)attempt);
        continue;
      }
    }
    const unsigned long long old = atomicAdd(mword_ptr(s, blk), (unsigned long long)want);
    const uint64_t cnt = old & 0xFFFFFFFFull;
    if (cnt >= SLICES_PER_BLOCK) {  // exhausted: its crosser is installing the next one
      blk = NOBLK;
      __nanosleep(128);
      continue;
    }
    const uint32_t got = (uint32_t)min((uint64_t)want, (uint64_t)SLICES_PER_BLOCK - cnt);
    const bool crossed = cnt + want > SLICES_PER_BLOCK - 1;
    const bool mine = (uint32_t)(old >> 32) == tree;
    const uint32_t used = blk;
    if (!mine) {  // a block of another class (recycled since it was read): give the slices back
      credit_frees(s, blk, got);
      blk = NOBLK;
    }
    if (crossed && mine) {
      if (s->use_spares) {
        if (swap_spare(s, tree, slot, used, tid)) spare_slot = slot;
      } else {
        replace_block(s, tree, slot, used, tid);
      }
      blk = NOBLK;
    }
    rc.blk[tree] = blk;
    rc.slot[tree] = slot;
    if (mine) {
      run_blk = used;
      run_start = (uint32_t)cnt;
      return got;
    }
  }
  rc.blk[tree] = NOBLK;
  return 0;
}

template <int SLOTS>
struct cta_free_smem {
  uint32_t key[SLOTS];
  uint32_t cnt[SLOTS];
};

// Frees this thread's N pointers (nullptr = nothing); one free-counter atomic
// per distinct block per CTA.  SLOTS (a power of two) must be at least
// blockDim.x * N so the table cannot fill.
template <int SLOTS, int N>
__device__ __forceinline__ void cta_free(const state *s, void *const (&ptrs)[N], cta_free_smem<SLOTS> &sm) {
  for (int i = threadIdx.x; i < SLOTS; i += blockDim.x) {
    sm.key[i] = NOBLK;
    sm.cnt[i] = 0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) {
    void *ptr = ptrs[k];
    if (!ptr) continue;
    uint16_t tree;
    uint32_t blk = block_of(s, ptr, tree);
    bool placed = false;
    if (blk != NOBLK) {
      uint32_t h = (blk * 2654435761u) & (SLOTS - 1);
      for (int probe = 0; probe < SLOTS; probe++) {
        uint32_t prev = atomicCAS(&sm.key[h], NOBLK, blk);
        if (prev == NOBLK || prev == blk) {
          atomicAdd(&sm.cnt[h], 1u);
          placed = true;
          break;
        }
        h = (h + 1) & (SLOTS - 1);
      }
    }
    if (!placed) gal::free(s, ptr);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SLOTS; i += blockDim.x)
    if (sm.key[i] != NOBLK) credit_frees(s, sm.key[i], sm.cnt[i]);
  __syncthreads();
}

template <int SLOTS>
__device__ __forceinline__ void cta_free(const state *s, void *ptr, cta_free_smem<SLOTS> &sm) {
  void *const one[1] = {ptr};
  cta_free<SLOTS, 1>(s, one, sm);
}

}  // namespace gal
