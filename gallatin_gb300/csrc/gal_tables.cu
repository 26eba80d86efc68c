// gal_tables.cu — batched uneven instances: many chained hash tables served by
// the device allocator in one launch per phase (the workload of the reference's
// data_structs/chaining_table.cuh:114-327, which has no delete; the table here
// is this library's own).
//
// Table t holds n_t pairs of 64-bit keys and values.  Its bucket array (one
// 64-bit head word per bucket, bit 0 the bucket's lock) and every 128-byte
// node come from the allocator.  A node: next pointer, a 7-bit used mask and
// seven key/value pairs (8 + 8 + 7 x 16 = 128 B, the 128 B class).
//
// Phases, each one launch over all tables (ops flattened, table by binary
// search over the offsets held in shared memory):
//   insert every key; delete the keys whose coin is set (a node left empty is
//   unlinked and freed); look up every key (deleted ones must be absent);
//   reinsert the deleted keys; look up every key (all present, right value);
//   count the live pairs of every table; free every node and bucket array.
// Node allocation inside an insert: per thread under the bucket lock (plain
// form), or CTA-aggregated (batched form: threads that found no room ask
// together through gal::cta_malloc, then lock again and link the node, or
// free it when another thread made room meanwhile).
//
// Keys: a bijective 64-bit mix of (table << 32 | index) so the keys of a table
// are distinct and uniform; value = another mix of the key; coin = bit 0 of a
// third mix.  gallatin_gb300/tables.py restates them on the host.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"
#include "gal_batch.cuh"

extern "C" {
/* Result of gal_bench_tables (mirrored in gallatin_gb300/_abi.py). */
typedef struct gal_tables_result {
  float ms[6];                 /* insert, delete, lookup-after-delete, reinsert, lookup, teardown */
  uint64_t total_pairs;
  uint64_t inserted;           /* inserts that added a pair (phases 0 and 3) */
  uint64_t deleted;
  uint64_t nodes_allocated;
  uint64_t nodes_freed;        /* by deletes and teardown */
  uint64_t spare_nodes_freed;  /* batched form: claimed, then not needed */
  uint64_t malloc_failed;
  uint64_t lock_timeouts;
  uint64_t missing;            /* keys absent that should be present */
  uint64_t unexpected;         /* deleted keys still present */
  uint64_t wrong_value;
  uint64_t count_mismatch;     /* tables whose live pairs != expected */
  uint64_t error_word;
  uint64_t setup_failed;       /* bucket arrays the allocator refused */
} gal_tables_result;
}

namespace {

constexpr int TBT = 256;          // CTA size of the table kernels
constexpr int MAX_TABLES = 4096;  // offsets held in shared memory
constexpr uint32_t SLOTS = 7;
constexpr uint32_t FULL = (1u << SLOTS) - 1u;

struct node {
  unsigned long long next;
  uint32_t used;
  uint32_t pad;
  unsigned long long key[SLOTS];
  unsigned long long val[SLOTS];
};
static_assert(sizeof(node) == 128, "one 128 B slice per node");

struct table_desc {
  unsigned long long *heads;
  uint64_t nbuckets;  // a power of two
};

enum : int { S_INSERTED, S_DELETED, S_NODES, S_NODES_FREED, S_SPARE, S_MFAIL, S_LOCK, S_MISSING,
             S_UNEXPECTED, S_WRONG, S_COUNT_MISMATCH, S_SETUP_FAILED, S_N };

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser (a bijection)
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}
__device__ __forceinline__ uint64_t table_key(uint32_t t, uint64_t i, uint64_t seed) {
  return mix64((((uint64_t)t << 32) | i) + seed * 0x9E3779B97F4A7C15ull);
}
__device__ __forceinline__ uint64_t table_val(uint64_t key) { return mix64(key ^ 0x5851F42D4C957F2Dull); }
__device__ __forceinline__ bool table_coin(uint64_t key) { return mix64(key + 0x2545F4914F6CDD1Dull) & 1u; }
__device__ __forceinline__ uint64_t bucket_of(uint64_t key, uint64_t nb) {
  return mix64(key ^ 0x9E3779B97F4A7C15ull) & (nb - 1u);
}

// per-thread counters, summed per warp once at the end of a phase kernel
struct counters {
  uint32_t c[S_N];
};
__device__ __forceinline__ void count(counters &lc, int which, uint32_t n = 1) { lc.c[which] += n; }
__device__ __forceinline__ void count_global(unsigned long long *stats, int which, uint32_t n = 1) {
  if (n) atomicAdd(&stats[which], (unsigned long long)n);
}
// full warp
__device__ __forceinline__ void flush(unsigned long long *stats, const counters &lc) {
#pragma unroll
  for (int k = 0; k < S_N; k++) {
    uint32_t v = __reduce_add_sync(0xFFFFFFFFu, lc.c[k]);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&stats[k], (unsigned long long)v);
  }
}

// bucket lock: bit 0 of the head word; bounded wait
__device__ __forceinline__ bool lock_bucket(const gal::state *s, unsigned long long *hp,
                                            unsigned long long &head) {
  for (uint32_t i = 0; i < s->spin_limit; i++) {
    unsigned long long h = gal::ld_rlx((const uint64_t *)hp);
    if (!(h & 1ull) && atomicCAS(hp, h, h | 1ull) == h) {
      __threadfence();
      head = h;
      return true;
    }
    gal::backoff(i);
  }
  return false;
}
__device__ __forceinline__ void unlock_bucket(unsigned long long *hp, unsigned long long head) {
  __threadfence();
  atomicExch(hp, head & ~1ull);
}

// the table of flattened op i
__device__ __forceinline__ uint32_t table_of(const uint64_t *off, uint32_t ntab, uint64_t i) {
  uint32_t lo = 0, hi = ntab;  // off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Under the lock: the key's place, or a node with room.  found: key present
// (n, slot); else room: a node with a free slot (n, slot), or n == 0.
struct probe {
  node *n;
  uint32_t slot;
  bool found;
  node *prev;  // predecessor of a found key's node (0: the head)
};
__device__ __forceinline__ probe find(unsigned long long head, uint64_t key) {
  probe r{nullptr, 0, false, nullptr};
  node *room = nullptr;
  uint32_t room_slot = 0;
  node *prev = nullptr;
  for (node *n = (node *)(head & ~1ull); n; prev = n, n = (node *)__ldcg(&n->next)) {
    uint32_t used = __ldcg(&n->used);
    for (uint32_t m = used; m; m &= m - 1u) {
      uint32_t k = (uint32_t)__ffs(m) - 1u;
      if (__ldcg(&n->key[k]) == key) {
        r.n = n;
        r.slot = k;
        r.found = true;
        r.prev = prev;
        return r;
      }
    }
    if (!room && used != FULL) {
      room = n;
      room_slot = (uint32_t)__ffs(~used & FULL) - 1u;
    }
  }
  r.n = room;
  r.slot = room_slot;
  return r;
}

// node words are read past L1 (__ldcg): another SM may have written them
// under the same bucket lock since this SM last cached the line
__device__ __forceinline__ void put(node *n, uint32_t slot, uint64_t key, uint64_t val) {
  n->key[slot] = key;
  n->val[slot] = val;
  n->used = __ldcg(&n->used) | (1u << slot);
}

// Insert under the lock.  spare: a node the caller already holds (batched
// form) or null; returns true when spare was used.
__device__ bool insert_locked(const gal::state *s, unsigned long long *hp, unsigned long long &head,
                              uint64_t key, uint64_t val, node *spare, bool may_malloc,
                              counters &lc, bool &need) {
  need = false;
  probe p = find(head, key);
  if (p.found) {
    p.n->val[p.slot] = val;
    return false;
  }
  if (p.n) {
    put(p.n, p.slot, key, val);
    count(lc, S_INSERTED);
    return false;
  }
  node *n = spare;
  if (!n && may_malloc) {
    n = (node *)gal::malloc(s, sizeof(node));
    if (!n) {
      count(lc, S_MFAIL);
      return false;
    }
    count(lc, S_NODES);
  }
  if (!n) {
    need = true;
    return false;
  }
  n->next = head & ~1ull;
  n->used = 1u;
  n->key[0] = key;
  n->val[0] = val;
  head = (unsigned long long)n;
  count(lc, S_INSERTED);
  return n == spare;
}

// phase ops
enum : int { PH_INSERT = 0, PH_DELETE = 1, PH_CHECK_DELETED = 2, PH_REINSERT = 3, PH_CHECK_ALL = 4 };

__device__ void lookup_check(const table_desc &d, uint64_t key, bool expect, counters &lc) {
  unsigned long long head = __ldcg(&d.heads[bucket_of(key, d.nbuckets)]);
  probe p = find(head, key);
  if (expect && !p.found) count(lc, S_MISSING);
  if (!expect && p.found) count(lc, S_UNEXPECTED);
  if (expect && p.found && __ldcg(&p.n->val[p.slot]) != table_val(key)) count(lc, S_WRONG);
}

__device__ void delete_key(const gal::state *s, const table_desc &d, uint64_t key, counters &lc) {
  unsigned long long *hp = &d.heads[bucket_of(key, d.nbuckets)];
  unsigned long long head;
  if (!lock_bucket(s, hp, head)) {
    count(lc, S_LOCK);
    return;
  }
  probe p = find(head, key);
  node *dead = nullptr;
  if (p.found) {
    uint32_t used = __ldcg(&p.n->used) & ~(1u << p.slot);
    p.n->used = used;
    count(lc, S_DELETED);
    if (used == 0) {  // unlink and free the empty node
      unsigned long long nx = __ldcg(&p.n->next);
      if (p.prev) p.prev->next = nx;
      else head = nx;
      dead = p.n;
    }
  }
  unlock_bucket(hp, head);
  if (dead) {
    gal::free(s, dead);
    count(lc, S_NODES_FREED);
  }
}

__device__ void insert_plain(const gal::state *s, const table_desc &d, uint64_t key, counters &lc) {
  unsigned long long *hp = &d.heads[bucket_of(key, d.nbuckets)];
  unsigned long long head;
  if (!lock_bucket(s, hp, head)) {
    count(lc, S_LOCK);
    return;
  }
  bool need;
  insert_locked(s, hp, head, key, table_val(key), nullptr, true, lc, need);
  unlock_bucket(hp, head);
}

__global__ void __launch_bounds__(TBT)
    k_tables_phase(const gal::state *s, int phase, int batched, uint32_t ntab, const uint64_t *offsets,
                   const table_desc *desc, uint64_t seed, unsigned long long *stats) {
  __shared__ uint64_t off[MAX_TABLES + 1];
  __shared__ gal::cta_claim_smem cm;
  for (uint32_t i = threadIdx.x; i <= ntab; i += blockDim.x) off[i] = offsets[i];
  gal::cta_claim_init(cm);
  __syncthreads();
  counters lc = {};
  const uint64_t total = off[ntab];
  const uint64_t stride = (uint64_t)gridDim.x * TBT;
  // the batched insert needs every thread of the CTA at each cta_malloc: the
  // loop runs the same number of iterations in all of them
  for (uint64_t base = (uint64_t)blockIdx.x * TBT; base < total; base += stride) {
    const uint64_t i = base + threadIdx.x;
    const bool has = i < total;
    uint32_t t = 0;
    uint64_t key = 0;
    if (has) {
      t = table_of(off, ntab, i);
      key = table_key(t, i - off[t], seed);
    }
    const table_desc d = has ? desc[t] : table_desc{nullptr, 1};
    const bool ok = has && d.heads != nullptr;
    const bool coin = ok && table_coin(key);
    if (phase == PH_INSERT || phase == PH_REINSERT) {
      const bool mine = ok && (phase == PH_INSERT || coin);
      if (!batched) {
        if (mine) insert_plain(s, d, key, lc);
        continue;
      }
      // batched: try without allocating, then ask for nodes together
      bool need = false;
      unsigned long long *hp = mine ? &d.heads[bucket_of(key, d.nbuckets)] : nullptr;
      if (mine) {
        unsigned long long head;
        if (lock_bucket(s, hp, head)) {
          insert_locked(s, hp, head, key, table_val(key), nullptr, false, lc, need);
          unlock_bucket(hp, head);
        } else {
          count(lc, S_LOCK);
        }
      }
      node *spare = (node *)gal::cta_malloc(s, sizeof(node), need, cm);
      if (need && !spare) count(lc, S_MFAIL);
      if (spare) {
        count(lc, S_NODES);
        unsigned long long head;
        bool used = false;
        if (lock_bucket(s, hp, head)) {
          bool again;
          used = insert_locked(s, hp, head, key, table_val(key), spare, false, lc, again);
          unlock_bucket(hp, head);
        } else {
          count(lc, S_LOCK);
        }
        if (!used) {  // another thread made room meanwhile
          gal::free(s, spare);
          count(lc, S_SPARE);
        }
      }
    } else if (phase == PH_DELETE) {
      if (ok && coin) delete_key(s, d, key, lc);
    } else if (phase == PH_CHECK_DELETED) {
      if (ok) lookup_check(d, key, !coin, lc);
    } else {
      if (ok) lookup_check(d, key, true, lc);
    }
  }
  flush(stats, lc);  // every thread ran the same iterations: the warps are whole
}

// one CTA per table: its bucket array from the allocator, zeroed
__global__ void __launch_bounds__(TBT)
    k_tables_setup(const gal::state *s, const uint64_t *offsets, table_desc *desc,
                   unsigned long long *stats) {
  __shared__ unsigned long long *heads;
  const uint32_t t = blockIdx.x;
  const uint64_t n = offsets[t + 1] - offsets[t];
  uint64_t nb = 16;
  while (nb * 4 < n) nb <<= 1;  // ~4 pairs per bucket
  if (threadIdx.x == 0) {
    heads = (unsigned long long *)gal::malloc(s, nb * sizeof(unsigned long long));
    desc[t].heads = heads;
    desc[t].nbuckets = nb;
    if (!heads) count_global(stats, S_SETUP_FAILED);
  }
  __syncthreads();
  if (!heads) return;
  for (uint64_t b = threadIdx.x; b < nb; b += blockDim.x) heads[b] = 0ull;
}

// one CTA per table: live pairs, compared with the expected count
__global__ void __launch_bounds__(TBT)
    k_tables_count(const uint64_t *offsets, const table_desc *desc, unsigned long long *stats) {
  __shared__ unsigned long long live;
  const uint32_t t = blockIdx.x;
  const table_desc d = desc[t];
  if (threadIdx.x == 0) live = 0;
  __syncthreads();
  if (!d.heads) return;
  unsigned long long mine = 0;
  for (uint64_t b = threadIdx.x; b < d.nbuckets; b += blockDim.x)
    for (node *n = (node *)(__ldcg(&d.heads[b]) & ~1ull); n; n = (node *)__ldcg(&n->next))
      mine += (unsigned long long)__popc(__ldcg(&n->used));
  atomicAdd(&live, mine);
  __syncthreads();
  if (threadIdx.x == 0 && live != offsets[t + 1] - offsets[t]) count_global(stats, S_COUNT_MISMATCH);
}

// one CTA per table: (key, value) pairs of table `which` appended to out
__global__ void k_tables_dump(const table_desc *desc, uint32_t which, unsigned long long *keys,
                              unsigned long long *vals, uint64_t cap, unsigned long long *n_out) {
  const table_desc d = desc[which];
  if (!d.heads) return;
  for (uint64_t b = threadIdx.x; b < d.nbuckets; b += blockDim.x)
    for (node *n = (node *)(__ldcg(&d.heads[b]) & ~1ull); n; n = (node *)__ldcg(&n->next)) {
      uint32_t used = __ldcg(&n->used);
      for (uint32_t m = used; m; m &= m - 1u) {
        uint32_t k = (uint32_t)__ffs(m) - 1u;
        unsigned long long at = atomicAdd(n_out, 1ull);
        if (at < cap) {
          keys[at] = __ldcg(&n->key[k]);
          vals[at] = __ldcg(&n->val[k]);
        }
      }
    }
}

// one CTA per table: every node and the bucket array back to the allocator
__global__ void __launch_bounds__(TBT)
    k_tables_destroy(const gal::state *s, const table_desc *desc, unsigned long long *stats) {
  const table_desc d = desc[blockIdx.x];
  if (!d.heads) return;
  uint32_t freed = 0;
  for (uint64_t b = threadIdx.x; b < d.nbuckets; b += blockDim.x) {
    node *n = (node *)(__ldcg(&d.heads[b]) & ~1ull);
    while (n) {
      node *nx = (node *)__ldcg(&n->next);
      gal::free(s, n);
      freed++;
      n = nx;
    }
  }
  count_global(stats, S_NODES_FREED, freed);
  __syncthreads();
  if (threadIdx.x == 0) gal::free(s, d.heads);
}

}  // namespace

extern "C" {

/* The table workload on an allocator: n_tables tables, table t holding
 * offsets[t+1] - offsets[t] pairs (host array of n_tables + 1 prefix sums),
 * keys from `seed`; batched selects the CTA-aggregated node allocation.
 * Phases and checks as described at the top of this file.  When dump_keys is
 * not null, the pairs of table dump_table after the last lookup are copied
 * there (at most dump_cap; *dump_n receives the count). */
int gal_bench_tables(gal_handle *h, uint32_t n_tables, const uint64_t *offsets, uint64_t seed,
                     int batched, gal_tables_result *res, uint32_t dump_table, uint64_t *dump_keys,
                     uint64_t *dump_vals, uint64_t dump_cap, uint64_t *dump_n) {
  if (!h || !res || !offsets || n_tables == 0 || n_tables > MAX_TABLES) return GAL_ERR_ARGS;
  for (uint32_t t = 0; t < n_tables; t++)
    if (offsets[t + 1] < offsets[t] || offsets[t + 1] - offsets[t] >= (1ull << 32)) return GAL_ERR_ARGS;
  memset(res, 0, sizeof(*res));
  const gal::state *d = (const gal::state *)gal_device_state(h);
  int rc = GAL_OK;
  uint64_t *d_off = nullptr;
  table_desc *d_desc = nullptr;
  unsigned long long *stats = nullptr, *d_keys = nullptr, *d_vals = nullptr, *d_n = nullptr;
  cudaEvent_t ev[8] = {};  // phase boundaries 0-5, teardown 6-7
  unsigned long long hs[S_N];
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tables_phase, TBT, 0);
  const uint64_t total = offsets[n_tables];
  const uint64_t need_ctas = (total + TBT - 1) / TBT;
  const unsigned grid = (unsigned)std::min<uint64_t>(need_ctas ? need_ctas : 1,
                                                     (uint64_t)sms * (per_sm > 0 ? per_sm : 1));
#define TK(x)                        \
  do {                               \
    if ((x) != cudaSuccess) {        \
      rc = GAL_ERR_CUDA;             \
      goto done;                     \
    }                                \
  } while (0)
  TK(cudaMalloc(&d_off, (n_tables + 1) * sizeof(uint64_t)));
  TK(cudaMalloc(&d_desc, n_tables * sizeof(table_desc)));
  TK(cudaMalloc(&stats, sizeof(hs)));
  TK(cudaMemcpy(d_off, offsets, (n_tables + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
  TK(cudaMemset(stats, 0, sizeof(hs)));
  for (auto &e : ev) TK(cudaEventCreate(&e));
  k_tables_setup<<<n_tables, TBT>>>(d, d_off, d_desc, stats);
  TK(cudaGetLastError());
  TK(cudaEventRecord(ev[0]));
  {
    const int phases[5] = {PH_INSERT, PH_DELETE, PH_CHECK_DELETED, PH_REINSERT, PH_CHECK_ALL};
    for (int k = 0; k < 5; k++) {
      k_tables_phase<<<grid, TBT>>>(d, phases[k], batched, n_tables, d_off, d_desc, seed, stats);
      TK(cudaGetLastError());
      TK(cudaEventRecord(ev[k + 1]));
    }
  }
  k_tables_count<<<n_tables, TBT>>>(d_off, d_desc, stats);
  TK(cudaGetLastError());
  if (dump_keys && dump_vals && dump_n && dump_table < n_tables && dump_cap) {
    TK(cudaMalloc(&d_keys, dump_cap * 8));
    TK(cudaMalloc(&d_vals, dump_cap * 8));
    TK(cudaMalloc(&d_n, 8));
    TK(cudaMemset(d_n, 0, 8));
    k_tables_dump<<<1, TBT>>>(d_desc, dump_table, d_keys, d_vals, dump_cap, d_n);
    TK(cudaGetLastError());
    TK(cudaMemcpy(dump_n, d_n, 8, cudaMemcpyDeviceToHost));
    uint64_t got = *dump_n < dump_cap ? *dump_n : dump_cap;
    TK(cudaMemcpy(dump_keys, d_keys, got * 8, cudaMemcpyDeviceToHost));
    TK(cudaMemcpy(dump_vals, d_vals, got * 8, cudaMemcpyDeviceToHost));
  }
  TK(cudaEventRecord(ev[6]));
  k_tables_destroy<<<n_tables, TBT>>>(d, d_desc, stats);
  TK(cudaGetLastError());
  TK(cudaEventRecord(ev[7]));
  TK(cudaEventSynchronize(ev[7]));
  TK(cudaEventElapsedTime(&res->ms[5], ev[6], ev[7]));
  for (int k = 0; k < 5; k++) TK(cudaEventElapsedTime(&res->ms[k], ev[k], ev[k + 1]));
  TK(cudaMemcpy(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost));
  res->total_pairs = total;
  res->inserted = hs[S_INSERTED];
  res->deleted = hs[S_DELETED];
  res->nodes_allocated = hs[S_NODES];
  res->nodes_freed = hs[S_NODES_FREED];
  res->spare_nodes_freed = hs[S_SPARE];
  res->malloc_failed = hs[S_MFAIL];
  res->lock_timeouts = hs[S_LOCK];
  res->missing = hs[S_MISSING];
  res->unexpected = hs[S_UNEXPECTED];
  res->wrong_value = hs[S_WRONG];
  res->count_mismatch = hs[S_COUNT_MISMATCH];
  res->setup_failed = hs[S_SETUP_FAILED];
  {
    uint32_t w = 0;
    gal_last_error(h, &w);
    res->error_word = w;
  }
#undef TK
done:
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  if (d_off) cudaFree(d_off);
  if (d_desc) cudaFree(d_desc);
  if (stats) cudaFree(stats);
  if (d_keys) cudaFree(d_keys);
  if (d_vals) cudaFree(d_vals);
  if (d_n) cudaFree(d_n);
  return rc;
}

}  // extern "C"
