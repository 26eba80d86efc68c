// gal_device.cuh — device side of the GB300-native Gallatin-compatible allocator.
//
// Header-inline because device malloc/free run inside the caller's kernels.
// The host side (construction, teardown, stats, state export) is the C ABI in
// include/gallatin_gb300.h; the drop-in C++ API is include/gallatin/allocators/.
//
// Algorithm: the reference allocator (chillenzer/gallatin,
// include/gallatin/allocators/gallatin.cuh and friends), restated so a serial
// trace returns the reference's offsets byte for byte.  Layout and
// synchronisation are this library's own:
//   * all metadata in one device region addressed from one state struct
//     (no pointer chasing through per-structure objects);
//   * blocks, queue entries and pinned slots are 32-bit block ids, not Block*;
//   * the malloc word of a block is 64-bit: (tree << 32) | count, so stale
//     claims can never carry a count into the tree field (the reference packs
//     tree << 20 | count into 32 bits, block.cuh:53);
//   * a block's malloc and free counters share one 32-byte record (one L2
//     sector per block, gal_config.block_layout), so the pinned blocks that
//     different SMs claim from never share a sector; the dense layout (all
//     malloc words, then all free counters) remains selectable;
//   * each segment's count of blocks left carries a set-up generation, so a
//     reservation checks the segment's class before it subtracts and never
//     has to give back into a later owner's count;
//   * every class lock sits in a 32-byte sector of its own;
//   * every spin-wait is bounded by state::spin_limit and reports through the
//     error word instead of trapping (the reference traps, gallatin.cuh:87);
//   * a vEB remove re-checks the emptied child word after clearing its
//     summary bit, with acquire-release fences ordering each thread's word
//     and summary accesses, closing the race that hides a non-empty word;
//   * a failed contiguous-run search does not roll back bits it never took
//     (the reference's exit rollback, veb.cuh:447);
//   * a multi-segment free resets the segment's tree id before returning its
//     bits, so a concurrent claim never meets a stale id (gallatin.cuh:1283-1302
//     returns the bits first).
#pragma once

#include <stdint.h>

#include "../gallatin_gb300.h"

#ifndef GAL_DEVICE_INLINE
#define GAL_DEVICE_INLINE __device__ __forceinline__
#endif
// cold paths stay out of line (register pressure of the hot path); static so
// the header can be included by several translation units
#define GAL_DEVICE_COLD static __device__ __noinline__

namespace gal {

static constexpr uint32_t NOBLK = 0xFFFFFFFFu;
static constexpr uint64_t FAIL = ~0ULL;
static constexpr uint16_t FREE_TREE = 0xFFFF;
static constexpr uint32_t SLICES_PER_BLOCK = 4096;

// retry caps of the reference (gallatin.cuh:108-112, veb.cuh:59)
static constexpr int SLICE_ATTEMPTS = 500 * 10;
static constexpr int VEB_ATTEMPTS = 15;
static constexpr int GATHER_RETRIES = 8;
static constexpr int BLOCK_ATTEMPTS = 8;
static constexpr int SEGMENT_ATTEMPTS = 8;
static constexpr int SLOT_PROBE_LIMIT = 30;  // SHARED_BLOCK_COUNTER_CUTOFF

struct veb_shape {
  uint32_t layers;
  uint32_t words;                        // words of one tree, all layers
  uint32_t off[GAL_MAX_VEB_LAYERS];      // word offset of each layer (0 = top)
  uint32_t nwords[GAL_MAX_VEB_LAYERS];
  uint64_t items[GAL_MAX_VEB_LAYERS];    // universe of each layer
};

// Everything a kernel needs; lives in device memory (the object a
// Gallatin<>* points to) and may also be passed by value as a kernel param.
struct state {
  char *memory;
  uint64_t num_segments;
  uint64_t seed;
  uint32_t seg_shift;   // log2 bytes_per_segment
  uint32_t min_shift;   // log2 min_size
  uint32_t bps_shift;   // log2 table blocks per segment
  uint32_t num_trees;
  uint32_t policy;
  int32_t smid_override;
  uint32_t spin_limit;
  uint32_t total_slots;
  uint32_t gather_unlocked_below;  // see gal_config
  uint32_t gather_ahead;           // see gal_config
  uint32_t team_width;             // see gal_config (1..32, a power of two)
  uint32_t use_spares;             // see gal_config.spare_blocks
  uint32_t zero_fill;              // see gal_config.zero_fill
  uint32_t slot_base[GAL_MAX_TREES];
  uint32_t slot_count[GAL_MAX_TREES];
  veb_shape veb;
  uint64_t *seg_tree;            // [veb.words]
  uint64_t *sub_trees;           // [num_trees * veb.words]
  uint16_t *tree_ids;            // [S]
  uint32_t *qc;                  // [S] hand-out position
  uint32_t *qfc;                 // [S] return position
  uint32_t *fqfc;                // [S] finalised return position
  unsigned long long *act;       // [S] (generation << 32) | (blocks left - 1 + ACT_BIAS)
  unsigned long long *mwords;    // per block (tree << 32) | count, every mstride-th word
  uint32_t *fctr;                // per block frees counted, every fstride-th word
  uint32_t mstride;              // 4 with fstride 8: one 32-byte record per block
  uint32_t fstride;              // 1 with fstride 1: dense arrays (gal_config.block_layout)
  uint32_t *queues;              // [S << bps_shift] recycle ring (block ids)
  uint32_t *slots;               // [total_slots] pinned blocks
  uint32_t *spares;              // [total_slots] next block per slot, prepared ahead
                                 // (gal_config.spare_blocks; NOBLK: none)
  uint32_t *locks;               // lock word of tree t at t * LOCK_STRIDE; runs at num_trees
  uint32_t *error;               // GAL_DEV_ERR_* bits
};

// ------------------------------------------------------------------ layout
static constexpr uint32_t BLOCK_RECORD_BYTES = 32;  // block_layout 1: one sector per block
static constexpr uint32_t LOCK_STRIDE = 8;          // u32 words between lock words (32 B)
GAL_DEVICE_INLINE __host__ unsigned long long *mword_ptr(const state *s, uint32_t blk) {
  return s->mwords + (uint64_t)blk * s->mstride;
}
GAL_DEVICE_INLINE __host__ uint32_t *fctr_ptr(const state *s, uint32_t blk) {
  return s->fctr + (uint64_t)blk * s->fstride;
}
// A segment's count word: generation in the high half, the reference's
// active count (blocks left to hand out minus one; -1 when none is left or the
// segment is free) plus ACT_BIAS in the low half, so adding or subtracting one
// never carries into the generation.
static constexpr uint32_t ACT_BIAS = 0x80000000u;
GAL_DEVICE_INLINE __host__ int32_t act_unbias(uint32_t low) { return (int32_t)(low - ACT_BIAS); }
GAL_DEVICE_INLINE __host__ int32_t act_count(unsigned long long w) { return act_unbias((uint32_t)w); }
GAL_DEVICE_INLINE __host__ uint32_t act_gen(unsigned long long w) { return (uint32_t)(w >> 32); }
GAL_DEVICE_INLINE __host__ unsigned long long act_word(uint32_t gen, int32_t count) {
  return ((unsigned long long)gen << 32) | (uint32_t)((uint32_t)count + ACT_BIAS);
}

// ------------------------------------------------------------------ helpers
GAL_DEVICE_INLINE uint32_t lane_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
  return r;
}
// Mask of the lanes executing here.  Read through volatile asm: the
// __activemask() builtin may be re-evaluated by the compiler at a later,
// divergent use site, which splits a warp team across convergence groups.
GAL_DEVICE_INLINE uint32_t active_lanes() {
  uint32_t m;
  asm volatile("activemask.b32 %0;" : "=r"(m));
  return m;
}
GAL_DEVICE_INLINE uint32_t lanemask_lt() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}
// The lanes this lane may aggregate with: the whole warp (team_width 32, the
// reference's coalesced team) or its aligned group of team_width lanes.
GAL_DEVICE_INLINE uint32_t team_group(const state *s) {
  const uint32_t w = s->team_width;
  if (w >= 32) return 0xFFFFFFFFu;
  return ((1u << w) - 1u) << (lane_id() & ~(w - 1u));
}
GAL_DEVICE_INLINE uint32_t sm_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}
GAL_DEVICE_INLINE uint64_t ld_rlx(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
GAL_DEVICE_INLINE uint32_t ld_rlx(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
GAL_DEVICE_INLINE int32_t ld_rlx(const int32_t *p) {
  return (int32_t)ld_rlx((const uint32_t *)p);
}
GAL_DEVICE_INLINE unsigned long long ld_rlx(const unsigned long long *p) {
  return (unsigned long long)ld_rlx((const uint64_t *)p);
}
GAL_DEVICE_INLINE uint16_t ld_rlx(const uint16_t *p) {
  uint16_t v;
  asm volatile("ld.relaxed.gpu.global.u16 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
  return v;
}
// acquire-release fence at device scope: orders this thread's earlier and
// later memory accesses (lighter than __threadfence's sequentially
// consistent one)
GAL_DEVICE_INLINE void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
GAL_DEVICE_INLINE uint64_t amo_or(uint64_t *p, uint64_t v) {
  return atomicOr((unsigned long long *)p, (unsigned long long)v);
}
GAL_DEVICE_INLINE uint64_t amo_and(uint64_t *p, uint64_t v) {
  return atomicAnd((unsigned long long *)p, (unsigned long long)v);
}
GAL_DEVICE_INLINE uint16_t cas16(uint16_t *p, uint16_t cmp, uint16_t val) {
  return (uint16_t)atomicCAS((unsigned short *)p, (unsigned short)cmp, (unsigned short)val);
}
GAL_DEVICE_INLINE void set_error(const state *s, uint32_t bits) { atomicOr(s->error, bits); }
// error word plus the first error's site and two values (error[2..9] as 4 u64:
// site, a, b, taken) for gal_error_info
GAL_DEVICE_COLD void set_error_info(const state *s, uint32_t bits, uint64_t site, uint64_t a,
                                    uint64_t b) {
  atomicOr(s->error, bits);
  unsigned long long *info = (unsigned long long *)(s->error + 2);
  if (atomicCAS(&info[3], 0ull, 1ull) == 0ull) {
    info[0] = site;
    info[1] = a;
    info[2] = b;
    __threadfence();
  }
}
enum : uint64_t {
  SITE_RETURN_BAD_TREE = 1,
  SITE_FREE_OVERFLOW = 2,
  SITE_FREE_OUTSIDE = 3,
  SITE_FREE_FREE_SEGMENT = 4,
  SITE_FREE_RUN_TWICE = 5,
  SITE_REQUEST_LOCK = 6,   // request_block: the class lock stayed taken (a: class, b: spins)
  SITE_REQUEST_RETRY = 7,  // request_block: listed segments kept refusing a block (a: class, b: last segment)
  SITE_RUN_LOCK = 8,       // malloc_segment_run: the run lock stayed taken (a: segments wanted)
};
GAL_DEVICE_INLINE void backoff(uint32_t i) { __nanosleep(i < 8 ? 32u << i : 4096u); }

// ceil(log2(x)) for x > 0, 0 for x == 0 (alloc_utils.cuh:382-398)
GAL_DEVICE_INLINE int ceil_log2(uint64_t x) {
  return 63 - __clzll((long long)x) + (__popcll(x) != 1);
}

// MurmurHash64A (Austin Appleby, public domain) of one 8-byte key
GAL_DEVICE_INLINE uint64_t murmur64a_u64(uint64_t key, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ULL;
  uint64_t h = seed ^ (8ULL * m);
  uint64_t k = key * m;
  k ^= k >> 47;
  k *= m;
  h ^= k;
  h *= m;
  h ^= h >> 47;
  h *= m;
  h ^= h >> 47;
  return h;
}

GAL_DEVICE_INLINE uint64_t bitmask(int n) { return n >= 64 ? ~0ULL : ((1ULL << n) - 1ULL); }
GAL_DEVICE_INLINE uint32_t blocks_in_segment(const state *s, uint32_t tree) {
  return 1u << (s->bps_shift - tree);
}
GAL_DEVICE_INLINE uint64_t thread_linear_id() {
  return (uint64_t)(threadIdx.x + blockIdx.x * blockDim.x);  // 32-bit as veb.cuh:948
}

// ------------------------------------------------------------------ vEB
// Word layout of one tree: layer 0 (top) first; bit i of layer l word w is
// item 64*w + i of that layer (veb.cuh:109-526, 528-1228).
struct veb_ref {
  uint64_t *w;
  const veb_shape *sh;
  uint64_t seed;
  GAL_DEVICE_INLINE uint64_t *word(int layer, uint64_t high) const { return w + sh->off[layer] + high; }
};

GAL_DEVICE_INLINE int veb_find_next(const veb_ref &v, int layer, uint64_t high, int low) {
  if (high >= v.sh->items[layer]) return -1;  // layer::find_next, veb.cuh:250-275
  uint64_t b = ld_rlx(v.word(layer, high));
  if (low == -1) return __ffsll((long long)b) - 1;
  return __ffsll((long long)(b & ~bitmask(low + 1))) - 1;
}

GAL_DEVICE_INLINE bool veb_query(const veb_ref &v, uint64_t x) {
  return (ld_rlx(v.word(v.sh->layers - 1, x >> 6)) >> (x & 63)) & 1ULL;
}

// veb_tree::remove (veb.cuh:737-755) plus the child re-check.  A remove that
// empties a word clears the word's summary bit, then reads the word again: an
// insert that refilled it meanwhile set the word's bit before the summary's,
// and acquire-release fences on both sides order the two accesses of each
// thread (the insert's set of the summary publishes its set of the word), so
// either the insert's summary set lands after this clear or this re-read sees
// the refilled word.  Without them a clear could land after the insert's set
// while the re-read still saw the empty word, leaving a non-empty word behind
// a clear summary bit, where top-down searches never find its items.
GAL_DEVICE_INLINE bool veb_remove(const veb_ref &v, uint64_t x) {
  int layer = (int)v.sh->layers - 1;
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  uint64_t old = amo_and(v.word(layer, high), ~(1ULL << low));
  if (!(old & (1ULL << low))) return false;
  while (__popcll(old) == 1 && layer > 0) {
    uint64_t *child = v.word(layer, high);
    layer -= 1;
    low = (int)(high & 63);
    high >>= 6;
    fence_acq_rel();
    old = amo_and(v.word(layer, high), ~(1ULL << low));
    fence_acq_rel();
    if (ld_rlx(child) != 0) {  // an insert raced in: keep the summary bit
      amo_or(v.word(layer, high), 1ULL << low);
      break;
    }
  }
  return true;
}

// veb_tree::insert_force_update (veb.cuh:775-798); the fence orders each
// word's set before its summary's (see veb_remove)
GAL_DEVICE_INLINE bool veb_insert(const veb_ref &v, uint64_t x) {
  int layer = (int)v.sh->layers - 1;
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  uint64_t old = amo_or(v.word(layer, high), 1ULL << low);
  if (old & (1ULL << low)) return false;
  while (__popcll(old) == 0 && layer > 0) {
    layer -= 1;
    low = (int)(high & 63);
    high >>= 6;
    fence_acq_rel();
    old = amo_or(v.word(layer, high), 1ULL << low);
  }
  return true;
}

// veb_tree::successor_thorough (veb.cuh:878-916): smallest item > q
GAL_DEVICE_COLD uint64_t veb_successor(const veb_ref &v, uint64_t q) {
  const int bottom = (int)v.sh->layers - 1;
  uint64_t high = q >> 6;
  int low = (int)(q & 63);
  int layer = bottom;
  for (;;) {
    for (;;) {
      if (veb_find_next(v, layer, high, low) != -1) break;
      if (layer == 0) return FAIL;
      layer -= 1;
      low = (int)(high & 63);
      high >>= 6;
    }
    while (layer != bottom) {
      low = veb_find_next(v, layer, high, low);
      if (low == -1) break;
      layer += 1;
      high = (high << 6) + (uint64_t)low;
      low = -1;
    }
    low = veb_find_next(v, layer, high, low);
    // only a bottom-layer hit is an item; a summary word refilled by a racing
    // insert is searched again from the top of the loop
    if (low != -1 && layer == bottom) return (high << 6) + (uint64_t)low;
  }
}

// veb_tree::lock_offset (veb.cuh:918-937)
GAL_DEVICE_INLINE uint64_t veb_lock_offset(const veb_ref &v, uint64_t start) {
  if (veb_query(v, start) && veb_remove(v, start)) return start;
  for (;;) {
    start = veb_successor(v, start);
    if (start == FAIL) return FAIL;
    if (veb_remove(v, start)) return start;
  }
}

// veb_tree::malloc_first (veb.cuh:979-991)
GAL_DEVICE_COLD uint64_t veb_malloc_first(const veb_ref &v) {
  for (int a = 0; a < VEB_ATTEMPTS; a++) {
    uint64_t o = veb_lock_offset(v, 0);
    if (o != FAIL) return o;
  }
  return FAIL;
}

// veb_tree::find_random_valid_index (veb.cuh:946-977)
// A search that came back empty from `start` shows that no item lies in
// [start, U); later attempts starting at or above the lowest such start are
// answered from that without touching the tree (the result is the one the
// reference's repeated searches give when nothing is inserted meanwhile, and
// one of the outcomes its relaxed reads allow when something is).  A sparse
// tree whose items sit at low ids otherwise costs all 15 attempts.
GAL_DEVICE_COLD uint64_t veb_find_random(const veb_ref &v, uint64_t tid) {
  const uint64_t U = v.sh->items[v.sh->layers - 1];
  uint64_t h1 = murmur64a_u64(tid, v.seed);
  uint64_t h2 = murmur64a_u64(tid, h1);
  uint64_t empty_from = U;  // no item in [empty_from, U)
  for (uint64_t a = 0; a < (uint64_t)VEB_ATTEMPTS; a++) {
    uint64_t start = (h1 + a * h2) % U;
    if (start >= empty_from) continue;
    if (veb_query(v, start)) return start;
    uint64_t idx = veb_successor(v, start);
    if (idx != FAIL) return idx;
    empty_from = start;
  }
  return veb_successor(v, 0);
}

// veb_tree::find_first_valid_index (veb.cuh:940-944): smallest listed id
GAL_DEVICE_INLINE uint64_t veb_find_first(const veb_ref &v) {
  if (veb_query(v, 0)) return 0;
  return veb_successor(v, 0);
}

GAL_DEVICE_INLINE int cfc64(uint64_t b) {  // alloc_utils.cuh:440-453
  int p = __popcll(b);
  if (p == 0 || p == 64) return p;
  return __ffsll((long long)~b) - 1;
}

GAL_DEVICE_INLINE void veb_rollback(const veb_ref &v, uint64_t start_block, uint64_t nbits) {
  const int bottom = (int)v.sh->layers - 1;  // layer::rollback, veb.cuh:305-321
  while (nbits > 64) {
    amo_or(v.word(bottom, start_block), ~0ULL);
    nbits -= 64;
    start_block++;
  }
  amo_or(v.word(bottom, start_block), bitmask((int)nbits));
}

// layer::gather_multiple (veb.cuh:323-452) on the bottom layer: claims a run
// ending in the trailing ones of a word, scanning words from the top down.
GAL_DEVICE_COLD uint64_t veb_gather_run(const veb_ref &v, uint64_t needed) {
  const int bottom = (int)v.sh->layers - 1;
  uint64_t sb = v.sh->nwords[bottom] - 1;
  // every pass either moves down a word or retries one that changed under it;
  // bound the retries so heavy interference ends in a clean failure
  uint64_t budget = 8ull * v.sh->nwords[bottom] + 1024;
  while (sb != 0) {
    if (budget-- == 0) return FAIL;
    uint64_t n = needed;
    uint64_t *w = v.word(bottom, sb);
    int c = cfc64(ld_rlx(w));
    if (c == 0) {
      sb -= 1;
      continue;
    }
    if ((uint64_t)c >= n) {
      uint64_t acq = bitmask((int)n) << (c - (int)n);
      uint64_t got = amo_and(w, ~acq);
      if ((uint64_t)__popcll(got & acq) == n) return sb * 64 + (uint64_t)(c - (int)n);
      amo_or(w, acq & got);
      continue;
    }
    uint64_t got = amo_and(w, ~bitmask(c));
    if (__popcll(got & bitmask(c)) != c) {
      amo_or(w, got & bitmask(c));
      continue;
    }
    n -= (uint64_t)c;
    bool ok = true;
    while (n > 64) {
      if (sb == 0) {  // run would leave the arena (the reference indexes word -1):
        veb_rollback(v, sb, needed - n);  // give back words 0 .. the first one
        return FAIL;
      }
      sb--;
      uint64_t full = amo_and(v.word(bottom, sb), 0ULL);
      if (__popcll(full) != 64) {
        amo_or(v.word(bottom, sb), full);
        veb_rollback(v, sb + 1, needed - n);
        ok = false;
        break;
      }
      n -= 64;
    }
    if (!ok) continue;
    if (sb == 0) {  // the same: the words taken start at word 0
      veb_rollback(v, sb, needed - n);
      return FAIL;
    }
    sb--;
    uint64_t fmask = bitmask((int)n) << (64 - n);
    uint64_t fb = amo_and(v.word(bottom, sb), ~fmask);
    if ((uint64_t)__popcll(fb & fmask) == n) return sb * 64 + 64 - n;
    amo_or(v.word(bottom, sb), fmask & fb);
    veb_rollback(v, sb + 1, needed - n);
  }
  return FAIL;
}

// veb_tree::gather_multiple (veb.cuh:1160-1196)
GAL_DEVICE_COLD uint64_t veb_gather_multiple(const veb_ref &v, uint64_t n) {
  uint64_t found = veb_gather_run(v, n);
  if (found == FAIL) return FAIL;
  uint64_t lo = found;
  for (int i = (int)v.sh->layers - 2; i >= 0; i--) {
    uint64_t hi = (lo + n - 1) / 64 + 1;
    lo = lo / 64;
    n = hi - lo;
    for (uint64_t wb = lo; wb < lo + n; wb++) {
      if (ld_rlx(v.word(i + 1, wb)) != 0) continue;
      amo_and(v.word(i, wb / 64), ~(1ULL << (wb % 64)));
      fence_acq_rel();
      // an insert that refilled the word between the load and the clear found
      // the summary bit still set and left it: put it back, as veb_remove does
      if (ld_rlx(v.word(i + 1, wb)) != 0) amo_or(v.word(i, wb / 64), 1ULL << (wb % 64));
    }
  }
  return found;
}

// veb_tree::return_multiple (veb.cuh:1198-1218, layer form veb.cuh:495-523)
GAL_DEVICE_COLD void veb_return_multiple(const veb_ref &v, uint64_t start, uint64_t n) {
  const int bottom = (int)v.sh->layers - 1;
  uint64_t bi = start / 64;
  int bs = (int)(start % 64);
  uint64_t left = n;
  while (left + (uint64_t)bs > 64) {
    int add = 64 - bs;
    amo_or(v.word(bottom, bi), bitmask(add) << bs);
    bs = 0;
    bi++;
    left -= (uint64_t)add;
  }
  amo_or(v.word(bottom, bi), bitmask((int)left) << bs);
  // maybe_return_layer_bits (veb.cuh:1128-1154) lists a word only when it is
  // full; an edge word that the claim emptied comes back partly filled and
  // would stay unlisted (its segments unreachable by every single-item
  // search).  Every non-empty word is listed here; a listed word that a
  // racing remove empties again is skipped by veb_successor.
  uint64_t lo = start;
  for (int i = bottom - 1; i >= 0; i--) {
    uint64_t hi = (lo + n - 1) / 64 + 1;
    lo = lo / 64;
    n = hi - lo;
    fence_acq_rel();  // the words below are set before their summaries (see veb_remove)
    for (uint64_t wb = lo; wb < lo + n; wb++)
      if (ld_rlx(v.word(i + 1, wb)) != 0) amo_or(v.word(i, wb / 64), 1ULL << (wb % 64));
  }
}

GAL_DEVICE_INLINE veb_ref seg_tree(const state *s) { return veb_ref{s->seg_tree, &s->veb, s->seed}; }
GAL_DEVICE_INLINE veb_ref sub_tree(const state *s, uint32_t t) {
  return veb_ref{s->sub_trees + (uint64_t)t * s->veb.words, &s->veb, s->seed + t};
}

// ------------------------------------------------------------------ locks
// one lock word per class (and one for runs) in a 32-byte sector of its own;
// the reference keeps them as bits of one word (gallatin.cuh:1513-1519)
GAL_DEVICE_INLINE bool try_lock(const state *s, uint32_t bit) {
  return atomicExch(s->locks + bit * LOCK_STRIDE, 1u) == 0u;
}
GAL_DEVICE_INLINE void unlock(const state *s, uint32_t bit) {
  __threadfence();
  atomicExch(s->locks + bit * LOCK_STRIDE, 0u);
}

// ------------------------------------------------------------------ table
// alloc_table::setup_segment (memory_table.cuh:746-818)
GAL_DEVICE_COLD bool setup_segment(const state *s, uint64_t seg, uint32_t tree) {
  if (cas16(&s->tree_ids[seg], FREE_TREE, (uint16_t)tree) != FREE_TREE) return false;
  uint32_t nb = blocks_in_segment(s, tree);
  uint32_t *q = s->queues + (seg << s->bps_shift);
  for (uint32_t i = 0; i < nb; i++) q[i] = NOBLK;
  __threadfence();
  atomicExch(&s->qc[seg], 0u);
  atomicExch(&s->qfc[seg], 0u);
  atomicExch(&s->fqfc[seg], 0u);
  __threadfence();
  // count -1 -> nb - 1 and a new generation, by addition: a reservation
  // attempt still in flight from before the segment's release gives its one
  // back into this count, as it took it from the count it found
  atomicAdd(&s->act[seg], (1ull << 32) + nb);
  return true;
}

// Gallatin::gather_new_segment (gallatin.cuh:1465-1510)
GAL_DEVICE_COLD int64_t gather_new_segment(const state *s, uint32_t tree) {
  uint64_t seg = veb_malloc_first(seg_tree(s));
  if (seg == FAIL) return -1;
  if (!setup_segment(s, seg, tree)) {
    set_error(s, GAL_DEV_ERR_SEGMENT_SETUP);
    return -1;
  }
  __threadfence();
  veb_insert(sub_tree(s, tree), seg);
  __threadfence();
  return (int64_t)seg;
}

// Releases segment `seg` of class `tree` when its count word still reads
// `gen` with every block home (nb - 1): removes it from the class's tree,
// frees its class and lists it in the segment tree (the release steps of
// Gallatin::return_block, gallatin.cuh:1663-1722, finish_freeing_block,
// memory_table.cuh:1226-1241).
GAL_DEVICE_COLD void release_segment(const state *s, uint64_t seg, uint32_t tree, uint32_t gen, uint32_t nb) {
  const unsigned long long home = act_word(gen, (int32_t)nb - 1);
  if (atomicCAS(&s->act[seg], home, act_word(gen, -1)) != home) return;
  __threadfence();
  veb_remove(sub_tree(s, tree), seg);
  __threadfence();
  if (cas16(&s->tree_ids[seg], (uint16_t)tree, FREE_TREE) != (uint16_t)tree) set_error(s, GAL_DEV_ERR_SEGMENT_SETUP);
  __threadfence();
  veb_insert(seg_tree(s), seg);
}

// Gives back a reservation taken from segment `seg` that no block came of.
// While it was held the count stayed below every-block-home, so no release
// could run; if giving it back brings the count there and blocks were handed
// out in this generation (every one of them has come home, the last return
// having found the count one short), the segment is released here.  With no
// hand-out yet the segment is a fresh one whose gatherer takes its first
// block next, so it stays.
GAL_DEVICE_COLD void give_back_reservation(const state *s, uint64_t seg) {
  const unsigned long long old = atomicAdd(&s->act[seg], 1ull);
  __threadfence();
  const uint16_t tree = ld_rlx(&s->tree_ids[seg]);
  if (tree >= s->num_trees) return;
  const uint32_t nb = blocks_in_segment(s, tree);
  if (act_count(old) + 1 == (int32_t)nb - 1 && ld_rlx(&s->qc[seg]) != 0)
    release_segment(s, seg, tree, act_gen(old), nb);
}

// alloc_table::get_block (memory_table.cuh:915-993)
// The reference subtracts one from the segment's count and adds it back when
// the count went negative or the segment belongs to another class
// (memory_table.cuh:923-929, get_slot_in_segment / return_slot_to_segment).
// An add-back that lands after the segment was released and set up again
// raises the new owner's count above its blocks, and one that lands after the
// segment's last return leaves it unreleased.  Here the class is checked
// against the count's generation before the subtraction, a count already
// negative is not touched, and the subtraction carries into a new set-up (see
// setup_segment), so the only give-backs left are the rare ones of a race
// between the check and the subtraction, which give_back_reservation
// settles.
GAL_DEVICE_COLD uint32_t get_block(const state *s, uint64_t seg, uint32_t tree, bool &last) {
  last = false;
  const unsigned long long seen = ld_rlx(&s->act[seg]);
  if (act_count(seen) < 0) return NOBLK;  // nothing left (or a free segment)
  __threadfence();
  if (ld_rlx(&s->tree_ids[seg]) != (uint16_t)tree) return NOBLK;  // another class's segment
  const unsigned long long old = atomicAdd(&s->act[seg], ~0ull);  // minus one
  const int32_t ac = act_count(old);
  if (ac < 0) {  // the last block went to another thread meanwhile
    give_back_reservation(s, seg);
    return NOBLK;
  }
  __threadfence();
  if (act_gen(old) != act_gen(seen) && ld_rlx(&s->tree_ids[seg]) != (uint16_t)tree) {
    // released and set up for another class between the check and the
    // subtraction; the class read now is the generation's own, as the
    // reservation keeps it from being released
    give_back_reservation(s, seg);
    return NOBLK;
  }
  uint32_t nb = blocks_in_segment(s, tree);
  uint32_t pos = atomicAdd(&s->qc[seg], 1u);
  uint32_t blk;
  if (pos < nb) {
    blk = (uint32_t)(seg << s->bps_shift) + pos;
  } else {
    uint32_t *e = s->queues + (seg << s->bps_shift) + (pos % nb);
    blk = atomicExch(e, NOBLK);
    for (uint32_t i = 0; blk == NOBLK && i < s->spin_limit; i++) {  // a return still in flight
      backoff(i);
      blk = atomicExch(e, NOBLK);
    }
    if (blk == NOBLK) {
      set_error(s, GAL_DEV_ERR_NULL_QUEUE);
      return NOBLK;
    }
  }
  atomicExch(mword_ptr(s, blk), (unsigned long long)tree << 32);  // Block::init_malloc
  if (ac == 0) last = true;
  return blk;
}

// Gallatin::request_new_block_from_tree (gallatin.cuh:1525-1631)
GAL_DEVICE_COLD uint32_t request_block(const state *s, uint32_t tree, uint64_t tid) {
  uint32_t spins = 0;
  int gather_fails = 0;
  for (;;) {
    veb_ref sub = sub_tree(s, tree);
    uint64_t seg = s->policy == GAL_POLICY_LOWEST ? veb_find_first(sub) : veb_find_random(sub, tid);
    // classes with few blocks per segment need a segment per few requests:
    // the class lock only serialises them (serially the lock is always free)
    const bool unlocked = blocks_in_segment(s, tree) < s->gather_unlocked_below;
    if (seg == FAIL) {
      if (unlocked || try_lock(s, tree)) {
        int64_t got = gather_new_segment(s, tree);
        if (!unlocked) unlock(s, tree);
        if (got < 0) {
          // segment tree empty: nothing a retry by this thread alone changes
          if (++gather_fails >= GATHER_RETRIES) return NOBLK;
          backoff(gather_fails);
          continue;
        }
        seg = (uint64_t)got;
      } else {
        if (++spins > s->spin_limit) {
          set_error_info(s, GAL_DEV_ERR_TIMEOUT, SITE_REQUEST_LOCK, tree, spins);
          return NOBLK;
        }
        backoff(spins);
        continue;
      }
    }
    bool last = false;
    uint32_t blk = get_block(s, seg, tree, last);
    if (last) {
      veb_remove(sub, seg);
      if (s->gather_ahead && (unlocked || try_lock(s, tree))) {
        gather_new_segment(s, tree);
        if (!unlocked) unlock(s, tree);
      }
      __threadfence();
    }
    if (blk != NOBLK) return blk;
    if (++spins > s->spin_limit) {
      set_error_info(s, GAL_DEV_ERR_TIMEOUT, SITE_REQUEST_RETRY, tree, seg);
      return NOBLK;
    }
    backoff(spins);
  }
}

// Gallatin::return_block (gallatin.cuh:1637-1726) with reserve_segment_slot,
// finalize_free_queue and finish_freeing_block (memory_table.cuh:906-910,1158-1241)
GAL_DEVICE_COLD void return_block(const state *s, uint32_t blk) {
  uint64_t seg = blk >> s->bps_shift;
  uint16_t tree = ld_rlx(&s->tree_ids[seg]);
  if (tree >= s->num_trees) {
    set_error_info(s, GAL_DEV_ERR_BAD_FREE, SITE_RETURN_BAD_TREE, blk, tree);
    return;
  }
  uint32_t nb = blocks_in_segment(s, tree);
  uint32_t pos = atomicAdd(&s->qfc[seg], 1u);
  uint32_t live = pos % nb;
  atomicExch(s->queues + (seg << s->bps_shift) + live, blk);
  __threadfence();
  // The reference finalises returns in position order with a CAS spin
  // (memory_table.cuh:906-910) so a hand-out never meets an empty ring entry;
  // get_block here waits (bounded) for an entry still in flight instead, so a
  // return only counts itself, leaving the same counter value.
  atomicAdd(&s->fqfc[seg], 1u);
  // re-register at the 10% crossing (gallatin.cuh:1646): live/nb >= 0.1 and
  // (live-1)/nb < 0.1 in doubles; for the power-of-two nb used here that is
  // 10*live > nb >= 10*(live-1) with live-1 taken as unsigned (live 0 never).
  if (live != 0 && 10ull * live > nb && 10ull * (live - 1) < nb) {
    veb_insert(sub_tree(s, tree), seg);
    __threadfence();
  }
  const unsigned long long old = atomicAdd(&s->act[seg], 1ull);
  __threadfence();
  if ((uint32_t)(act_count(old) + 2) == nb)  // all_blocks_free: the count was nb - 2
    release_segment(s, seg, tree, act_gen(old), nb);
}

// Block::block_free_multiple + reset_free + free_block (block.cuh:87-98,200-212,
// gallatin.cuh:1732-1766)
GAL_DEVICE_INLINE void credit_done(const state *s, uint32_t blk, uint32_t old, uint32_t n);
GAL_DEVICE_INLINE void credit_frees(const state *s, uint32_t blk, uint32_t n) {
  credit_done(s, blk, atomicAdd(fctr_ptr(s, blk), n), n);
}
// the block's free counter was `old` before this thread added n
GAL_DEVICE_INLINE void credit_done(const state *s, uint32_t blk, uint32_t old, uint32_t n) {
  if (old + n == SLICES_PER_BLOCK) {
    atomicExch(fctr_ptr(s, blk), 0u);
    __threadfence();
    return_block(s, blk);
  } else if (old + n > SLICES_PER_BLOCK) {
    set_error_info(s, GAL_DEV_ERR_BAD_FREE, SITE_FREE_OVERFLOW, blk,
                   ((uint64_t)old << 32) | n);
  }
}

// Gives back a block this thread took for a slot or a spare and could not
// install: closes it to further claims (its count goes past the end) and
// credits the slices nobody claimed, so it returns to its segment now, or
// once the slices a claim did take (one that read the block in an earlier
// life and landed after its hand-out) are freed.  Crediting all 4,096 would
// return it under those live slices.
GAL_DEVICE_COLD void retire_block(const state *s, uint32_t blk) {
  const unsigned long long old = atomicAdd(mword_ptr(s, blk), (unsigned long long)SLICES_PER_BLOCK);
  const uint32_t handed_out = (uint32_t)old;
  if (handed_out < SLICES_PER_BLOCK) credit_frees(s, blk, SLICES_PER_BLOCK - handed_out);
}

// Gallatin::free_offset (gallatin.cuh:1774-1827): team by block, one atomic
GAL_DEVICE_INLINE void free_block_slices(const state *s, uint32_t blk) {
  uint32_t active = active_lanes();
  uint32_t team = __match_any_sync(active, blk) & team_group(s);
  if ((int)lane_id() == __ffs(team) - 1) credit_frees(s, blk, (uint32_t)__popc(team));
}

// ------------------------------------------------------------------ pinned slots
// per_size_pinned_blocks::get_valid_block_index (shared_block_storage.cuh:119-134)
// Returns the slot index; `blk` receives the block read from it (one read per
// probed slot, the last one doubling as the reference's get_my_block read).
GAL_DEVICE_INLINE uint32_t pick_slot(const state *s, uint32_t tree, uint32_t &blk) {
  const uint32_t n = s->slot_count[tree];
  const uint32_t *slots = s->slots + s->slot_base[tree];
  uint32_t smid = s->smid_override >= 0 ? (uint32_t)s->smid_override : sm_id();
  int my = (int)(smid % n);
  int original = my;
  int counter = 0;
  uint32_t v = ld_rlx(&slots[my]);
  while (v == NOBLK && my != original - 1) {
    my = (my + 1) % (int)n;
    v = ld_rlx(&slots[my]);
    if (++counter >= SLOT_PROBE_LIMIT) break;
  }
  blk = v;
  return (uint32_t)my;
}

// Gallatin::replace_block (gallatin.cuh:1083-1138)
GAL_DEVICE_COLD bool replace_block(const state *s, uint32_t tree, uint32_t slot, uint32_t blk,
                                   uint64_t tid) {
  uint32_t *sp = s->slots + s->slot_base[tree] + slot;
  if (atomicCAS(sp, blk, NOBLK) != blk) return true;
  __threadfence();
  uint32_t nb = request_block(s, tree, tid);
  if (nb == NOBLK) return false;
  __threadfence();
  if (atomicCAS(sp, NOBLK, nb) != NOBLK) {
    set_error(s, GAL_DEV_ERR_SLOT_SWAP);
    retire_block(s, nb);  // hand the block back
    return false;
  }
  return true;
}

// Spare blocks (gal_config.spare_blocks): the slot's prepared next block is
// swapped in with one CAS, so other warps see a fresh block at once instead of
// an empty slot for the length of a segment search; the search then refills
// the spare.  swap_spare returns whether the caller should refill (it falls
// back to replace_block when no spare was ready).
GAL_DEVICE_COLD bool swap_spare(const state *s, uint32_t tree, uint32_t slot, uint32_t blk, uint64_t tid) {
  const uint32_t si = s->slot_base[tree] + slot;
  const uint32_t nx = atomicExch(s->spares + si, NOBLK);
  if (nx == NOBLK) {
    replace_block(s, tree, slot, blk, tid);
  } else if (atomicCAS(s->slots + si, blk, nx) != blk) {
    retire_block(s, nx);  // the slot moved on: give the spare back
    return false;
  }
  return true;
}
GAL_DEVICE_COLD void refill_spare(const state *s, uint32_t tree, uint32_t slot, uint64_t tid) {
  const uint32_t si = s->slot_base[tree] + slot;
  if (ld_rlx(s->spares + si) != NOBLK) return;
  const uint32_t nb = request_block(s, tree, tid);
  if (nb == NOBLK) return;
  __threadfence();
  if (atomicCAS(s->spares + si, NOBLK, nb) != NOBLK) retire_block(s, nb);
}

// Gallatin::boot_block (gallatin.cuh:726-787)
GAL_DEVICE_COLD bool boot_block(const state *s, uint32_t tree, uint32_t slot, uint64_t tid) {
  if (slot >= s->slot_count[tree]) return false;
  uint32_t blk = request_block(s, tree, tid);
  if (blk == NOBLK) return false;
  if (ld_rlx(&s->tree_ids[blk >> s->bps_shift]) != tree) return false;
  return atomicCAS(s->slots + s->slot_base[tree] + slot, NOBLK, blk) == NOBLK;
}

// ------------------------------------------------------------------ addresses
GAL_DEVICE_INLINE char *slice_ptr(const state *s, uint32_t blk, uint64_t idx, uint32_t tree) {
  uint64_t seg = blk >> s->bps_shift;
  uint64_t q = blk & ((1u << s->bps_shift) - 1u);
  return s->memory + (seg << s->seg_shift) + (((q << 12) + idx) << (s->min_shift + tree));
}

// ------------------------------------------------------------------ malloc tiers
// Gallatin::malloc_slice_allocation (gallatin.cuh:865-1078): warp team per
// size class, one atomicAdd on the pinned block per team.  Two ways to know
// the team: as the reference does, the lanes executing each attempt together
// (NAMED = false: every attempt re-forms the teams from the active lanes, and
// a lane leaves the loop as soon as it has its slice); or named by the caller
// (NAMED = true: `pending`, the lanes that called together and ask for
// slices, shrinks as lanes get their slices, and every warp-wide step of an
// attempt names it, so a team holds every caller of its class even when the
// callers' earlier branches left them in separate groups).
// A CTA's copy of its SM's pinned blocks, in shared memory (gal::malloc_cached):
// per class the block last read from the class's pinned slot and that slot.
// A copy that has gone stale (its block exhausted or replaced) shows up in the
// claim itself -- the count comes back at or past the block's end, or with
// another class -- and is dropped, so the next team reads the slot again.
struct slot_cache {
  uint32_t blk[GAL_MAX_TREES];
  uint32_t slot[GAL_MAX_TREES];
};

// every thread of the CTA, followed by a __syncthreads()
GAL_DEVICE_INLINE void slot_cache_init(slot_cache &c) {
  if (threadIdx.x < GAL_MAX_TREES) {
    c.blk[threadIdx.x] = NOBLK;
    c.slot[threadIdx.x] = 0;
  }
}

// The rare part of a claim, out of line so the claim's common path keeps few
// values live across calls: credits the slices this lane gives back and, for
// the team's leader when the block must be replaced, swaps in the slot's spare
// (or replaces the block).  Returns whether the spare wants a refill.
GAL_DEVICE_COLD bool claim_slow_path(const state *s, uint32_t tree, uint32_t slot, uint32_t blk, uint32_t credit,
                                     bool lead, uint64_t tid) {
  if (credit) credit_frees(s, blk, credit);
  if (!lead) return false;
  if (s->use_spares) return swap_spare(s, tree, slot, blk, tid);
  replace_block(s, tree, slot, blk, tid);
  return false;
}

// A block is exhausted by exactly one claim -- the one that crosses slice
// 4095 -- and that claim's team replaces it in its pinned slot.  A team that
// claimed from a block it read some time before (a CTA's slot_cache, or a
// slow team) may cross a block that has since been recycled into another
// slot or a spare; its replace then finds its own slot holding something else
// and does nothing, and the slot that does hold the block keeps it exhausted.
// Every failed claim still adds to the block's count, so a block left
// exhausted in a slot soon reads far past its end: a team that reads its
// slot's block more than STUCK_MARGIN slices past the end replaces it itself
// (a compare-and-swap on the slot, so at most one replacement happens).  The
// rightful crosser swaps its block within a few claims of the end, so the
// margin keeps the teams out of each other's way.  One thread alone never
// meets an exhausted block in its slot, so serial offsets are unchanged.
static constexpr uint32_t STUCK_MARGIN = 1u << 12;
template <bool NAMED>
GAL_DEVICE_INLINE void *malloc_slices(const state *s, uint32_t tree, uint32_t count, uint32_t pending,
                                      slot_cache *cache = nullptr) {
  const uint32_t lane = lane_id();
  const uint64_t tid = thread_linear_id();
  for (int attempt = 0; attempt < SLICE_ATTEMPTS; attempt++) {
    const uint32_t active = NAMED ? pending : active_lanes();
    const uint32_t team = __match_any_sync(active, tree) & team_group(s);
    const int leader = __ffs(team) - 1;
    const int last = 31 - __clz(team);
    const uint32_t lt = lanemask_lt();
    // every lane of a team reads the same slot words in the same instruction
    // (one broadcast transaction), so the team needs no leader branch here
    uint32_t seen = NOBLK, slot = 0;
    if (cache) {
      seen = *(volatile uint32_t *)&cache->blk[tree];
      slot = *(volatile uint32_t *)&cache->slot[tree];
    }
    const bool fresh = seen == NOBLK;  // read from the pinned slot this attempt
    if (fresh) {
      slot = pick_slot(s, tree, seen);
      if (cache && seen != NOBLK) {  // every lane of the team writes the same values
        *(volatile uint32_t *)&cache->slot[tree] = slot;
        *(volatile uint32_t *)&cache->blk[tree] = seen;
      }
    }
    const uint32_t blk = __shfl_sync(active, seen, leader);
    // teams whose slot was empty retry; the rest carry on with mask `live`
    const uint32_t live = __ballot_sync(active, blk != NOBLK);
    if (!NAMED && blk == NOBLK) continue;
    void *result = nullptr;
    bool refill = false;
    if (blk != NOBLK) {
      uint32_t prefix, total;
      if (__all_sync(live, count == 1)) {
        prefix = (uint32_t)__popc(team & lt);
        total = (uint32_t)__popc(team);
      } else {  // big slices: counts are powers of two up to one block
        prefix = 0;
        total = 0;
        for (uint32_t c = 1; c <= SLICES_PER_BLOCK; c <<= 1) {
          uint32_t b = __ballot_sync(live, count == c) & team;
          prefix += c * (uint32_t)__popc(b & lt);
          total += c * (uint32_t)__popc(b);
        }
      }
      unsigned long long old = 0;
      if ((int)lane == last) old = atomicAdd(mword_ptr(s, blk), (unsigned long long)total);
      old = __shfl_sync(live, old, last);
      const uint64_t alloc = (old & 0xFFFFFFFFull) + prefix;
      const bool start_valid = alloc <= SLICES_PER_BLOCK - 1;
      const bool end_valid = alloc + count <= SLICES_PER_BLOCK;
      const bool should_replace = start_valid && alloc + count > SLICES_PER_BLOCK - 1;
      const bool foreign = (uint32_t)(old >> 32) != tree;
      const bool valid = start_valid && end_valid;
      if (valid && !foreign) result = slice_ptr(s, blk, alloc, tree);
      // slices this lane gives back: the rest of a run, or the part of it past
      // the block's end (block_correct_frees), and a claimed slice of a block
      // that serves another class now (Block::check_valid failed)
      const uint32_t credit = (start_valid ? (end_valid ? count - 1 : (uint32_t)(SLICES_PER_BLOCK - alloc)) : 0u) +
                              (valid && foreign ? 1u : 0u);
      uint32_t rep = __ballot_sync(live, should_replace) & team;
      const bool exhausted = !foreign && (__ballot_sync(live, start_valid) & team) == 0;
      if (cache) {  // exhausted, replaced or foreign: the next team reads the slot again
        if ((rep || exhausted || foreign) && (int)lane == leader) atomicCAS(&cache->blk[tree], blk, NOBLK);
      }
      if (exhausted && fresh && (old & 0xFFFFFFFFull) >= SLICES_PER_BLOCK + STUCK_MARGIN)
        rep = team;  // the slot has held an exhausted block for a while: replace it here
      const bool lead = rep && (int)lane == leader;
      if (credit || lead) refill = claim_slow_path(s, tree, slot, blk, credit, lead, tid);
      __syncwarp(live);
      if (!NAMED && refill) refill_spare(s, tree, slot, tid);  // the team's other lanes go on
    }
    if (NAMED) {
      pending = __ballot_sync(active, result == nullptr);
      if (refill) refill_spare(s, tree, slot, tid);  // the team's other lanes go on
    }
    if (result) return result;
  }
  return nullptr;
}

// Gallatin::malloc_block_allocation (gallatin.cuh:828-861), Block::malloc_fill_block
GAL_DEVICE_COLD void *malloc_whole_block(const state *s, uint32_t tree) {
  const uint64_t tid = thread_linear_id();
  for (int a = 0; a < BLOCK_ATTEMPTS; a++) {
    uint32_t blk = request_block(s, tree, tid);
    if (blk == NOBLK) return nullptr;
    unsigned long long old = atomicAdd(mword_ptr(s, blk), (unsigned long long)SLICES_PER_BLOCK);
    uint32_t old_count = (uint32_t)old;
    if ((uint32_t)(old >> 32) != tree) set_error(s, GAL_DEV_ERR_BLOCK_TREE);
    atomicAdd(fctr_ptr(s, blk), (SLICES_PER_BLOCK - 1) - old_count);
    if (old_count != 0) {
      credit_frees(s, blk, 1);
      continue;
    }
    return slice_ptr(s, blk, 0, tree);
  }
  return nullptr;
}

// Gallatin::malloc_segment_allocation (gallatin.cuh:790-826)
GAL_DEVICE_COLD void *malloc_segment_run(const state *s, uint32_t count) {
  for (int a = 0; a < SEGMENT_ATTEMPTS; a++) {
    uint32_t spins = 0;
    while (!try_lock(s, s->num_trees)) {
      if (++spins > s->spin_limit) {
        set_error_info(s, GAL_DEV_ERR_TIMEOUT, SITE_RUN_LOCK, count, spins);
        return nullptr;
      }
      backoff(spins);
    }
    uint64_t idx = veb_gather_multiple(seg_tree(s), count);
    if (idx != FAIL) {
      if (cas16(&s->tree_ids[idx], FREE_TREE, (uint16_t)(s->num_trees + 1 + count)) != FREE_TREE)
        set_error(s, GAL_DEV_ERR_SEGMENT_SETUP);
      unlock(s, s->num_trees);
      return s->memory + (idx << s->seg_shift);
    }
    unlock(s, s->num_trees);
  }
  return nullptr;
}

// calloc mode (gal_config.zero_fill): the requested bytes, rounded up to 16,
// are cleared by the allocating thread.  Every allocation starts on a 16-byte
// boundary and covers at least its request rounded up to 16 (slices are at
// least 16 B), so the stores stay inside it.
GAL_DEVICE_COLD void zero_fill(void *p, uint64_t size) {
  uint4 *q = (uint4 *)p;
  const uint64_t n = size ? (size + 15) >> 4 : 1;
  for (uint64_t i = 0; i < n; i++) q[i] = make_uint4(0u, 0u, 0u, 0u);
}
GAL_DEVICE_INLINE void *handed_out(const state *s, void *p, uint64_t size) {
  if (p && s->zero_fill) zero_fill(p, size);
  return p;
}

// the block and segment tiers of Gallatin::malloc (gallatin.cuh:1203-1258)
GAL_DEVICE_COLD void *malloc_large(const state *s, uint64_t size, int block_tree) {
  if (block_tree < (int)s->num_trees) return malloc_whole_block(s, (uint32_t)block_tree);
  return malloc_segment_run(s, (uint32_t)((size - 1) >> s->seg_shift) + 1);
}

// Gallatin::malloc (gallatin.cuh:1186-1276) called by the lanes in `callers`
// together.  Those that ask for slices reach malloc_slices on one path (the
// class and run length are selects, not branches), so single slices and runs
// of the same class share a team.
template <bool NAMED>
GAL_DEVICE_INLINE void *malloc_from(const state *s, uint64_t size, uint32_t callers, slot_cache *cache = nullptr) {
  const int T = (int)s->num_trees;
  const int bits = ceil_log2(size);
  const int t = (size >> s->min_shift) == 0 ? 0 : bits - (int)s->min_shift;
  const int block_tree = bits - (int)(s->min_shift + 12);
  const bool slices = t < T || block_tree < 0;
  const uint32_t members = __ballot_sync(callers, slices);
  if (!slices) return handed_out(s, malloc_large(s, size, block_tree), size);
  // big slices (4 KiB < size <= 32 KiB by default): runs of the last class
  const bool big = t >= T;
  const uint32_t count = 1u << (big ? t - (T - 1) : 0);
  const uint32_t tree = (uint32_t)(big ? T - 1 : t);
  return handed_out(s, malloc_slices<NAMED>(s, tree, count, members, cache), size);
}

// Gallatin::malloc as the reference calls it: each attempt's team is the lanes
// executing it together (its coalesced_threads(), gallatin.cuh:883).
GAL_DEVICE_INLINE void *malloc(const state *s, uint64_t size) {
  return malloc_from<false>(s, size, active_lanes());
}

// malloc for kernels whose CTAs serve many requests (persistent loops): the
// teams take the pinned block from the CTA's slot_cache in shared memory and
// read the pinned slot in global memory only when the copy has gone stale, so
// a team's claim costs one L2 round trip instead of two.  Same results
// contract as malloc.
GAL_DEVICE_INLINE void *malloc_cached(const state *s, uint64_t size, slot_cache &cache) {
  return malloc_from<false>(s, size, active_lanes(), &cache);
}

// malloc with the calling lanes named: every lane of `callers` calls with the
// same mask (the contract of the *_sync warp intrinsics), and the lanes asking
// for slices of one class form one team whatever grouping of diverged lanes
// the scheduler chose.
GAL_DEVICE_INLINE void *malloc_team(const state *s, uint64_t size, uint32_t callers) {
  return malloc_from<true>(s, size, callers);
}

// multi-segment free (gallatin.cuh:1394-1417, 1283-1302), id reset first
GAL_DEVICE_COLD void free_segment_run(const state *s, uint64_t seg, uint16_t tree) {
  uint32_t count = (uint32_t)tree - s->num_trees - 1;
  if (cas16(&s->tree_ids[seg], tree, FREE_TREE) != tree) {
    set_error_info(s, GAL_DEV_ERR_BAD_FREE, SITE_FREE_RUN_TWICE, seg, tree);
    return;
  }
  __threadfence();
  veb_return_multiple(seg_tree(s), seg, count);
}

// Gallatin::free (gallatin.cuh:1378-1461)
GAL_DEVICE_INLINE void free(const state *s, void *ptr) {
  uint64_t off = (uint64_t)((char *)ptr - s->memory);
  uint64_t seg = off >> s->seg_shift;
  if (seg >= s->num_segments) {
    set_error_info(s, GAL_DEV_ERR_BAD_FREE, SITE_FREE_OUTSIDE, off, 0);
    return;
  }
  uint16_t tree = ld_rlx(&s->tree_ids[seg]);
  if (tree >= s->num_trees) {
    if (tree == FREE_TREE || tree == s->num_trees) {
      set_error_info(s, GAL_DEV_ERR_BAD_FREE, SITE_FREE_FREE_SEGMENT, off, tree);
      return;
    }
    free_segment_run(s, seg, tree);
    return;
  }
  uint64_t in_seg = off & ((1ull << s->seg_shift) - 1ull);
  uint32_t blk = (uint32_t)(seg << s->bps_shift) + (uint32_t)(in_seg >> (s->min_shift + tree + 12));
  free_block_slices(s, blk);
}

// block id of a live pointer (slice or whole block), NOBLK for a segment run
GAL_DEVICE_INLINE uint32_t block_of(const state *s, const void *ptr, uint16_t &tree_out) {
  uint64_t off = (uint64_t)((const char *)ptr - s->memory);
  uint64_t seg = off >> s->seg_shift;
  uint16_t tree = seg < s->num_segments ? ld_rlx(&s->tree_ids[seg]) : FREE_TREE;
  tree_out = tree;
  if (tree >= s->num_trees) return NOBLK;
  uint64_t in_seg = off & ((1ull << s->seg_shift) - 1ull);
  return (uint32_t)(seg << s->bps_shift) + (uint32_t)(in_seg >> (s->min_shift + tree + 12));
}

// Frees the pointers p[k] with go[k] set, as N calls of free() would, but
// with their table lookups and their free-counter atomics each issued back to
// back so the round trips overlap.  Warp teams form per k, as in free().
// `classes`, when given, is a copy of tree_ids taken after every pointer
// passed was allocated (see stage_classes); a live pointer's segment keeps
// its class, so the copy answers the lookup without a trip to L2.
template <int N>
GAL_DEVICE_INLINE void free_n(const state *s, void *const (&p)[N], const bool (&go)[N],
                              const uint16_t *classes = nullptr) {
  uint16_t tree[N];
  uint64_t off[N];
#pragma unroll
  for (int k = 0; k < N; k++) {
    tree[k] = FREE_TREE;
    off[k] = go[k] ? (uint64_t)((char *)p[k] - s->memory) : 0;
    if (go[k] && (off[k] >> s->seg_shift) < s->num_segments)
      tree[k] = classes ? classes[off[k] >> s->seg_shift] : ld_rlx(&s->tree_ids[off[k] >> s->seg_shift]);
  }
  uint32_t blk[N], old[N], cnt[N];
  bool lead[N];
#pragma unroll
  for (int k = 0; k < N; k++) {
    lead[k] = false;
    blk[k] = NOBLK;
    if (!go[k]) continue;
    if (tree[k] >= s->num_trees) {  // segment runs and bad pointers: the scalar path
      gal::free(s, p[k]);
      continue;
    }
    uint64_t in_seg = off[k] & ((1ull << s->seg_shift) - 1ull);
    blk[k] = (uint32_t)((off[k] >> s->seg_shift) << s->bps_shift) +
             (uint32_t)(in_seg >> (s->min_shift + tree[k] + 12));
  }
#pragma unroll
  for (int k = 0; k < N; k++) {
    if (blk[k] == NOBLK) continue;
    const uint32_t active = active_lanes();
    const uint32_t team = __match_any_sync(active, blk[k]) & team_group(s);
    lead[k] = (int)lane_id() == __ffs(team) - 1;
    cnt[k] = (uint32_t)__popc(team);
    if (lead[k]) old[k] = atomicAdd(fctr_ptr(s, blk[k]), cnt[k]);
  }
#pragma unroll
  for (int k = 0; k < N; k++)
    if (lead[k]) credit_done(s, blk[k], old[k], cnt[k]);
}

// Segments whose classes fit in CLASS_STAGE_BYTES of shared memory can be
// staged for free_n: every thread of the CTA calls stage_classes, then
// __syncthreads().  Returns false (nothing staged) for larger arenas.
static constexpr uint32_t CLASS_STAGE_BYTES = 32768;
GAL_DEVICE_INLINE bool stage_classes(const state *s, uint16_t *smem) {
  if (s->num_segments * 2 > CLASS_STAGE_BYTES) return false;
  for (uint64_t g = threadIdx.x; g < s->num_segments; g += blockDim.x) smem[g] = ld_rlx(&s->tree_ids[g]);
  return true;
}

// a block's malloc word in the reference packing, (tree << 20) + count (block.cuh:53,220)
GAL_DEVICE_INLINE uint32_t export_mword(const state *s, uint32_t blk) {
  const unsigned long long w = *mword_ptr(s, blk);
  return (uint32_t)(((w >> 32) << 20) + (w & 0xFFFFFFFFull));
}

// bytes a request of `size` occupies (Gallatin::get_allocated_size, gallatin.cuh:1152-1183)
GAL_DEVICE_INLINE uint64_t allocated_size(const state *s, uint64_t size) {
  if (size < 16) size = 16;
  int bits = ceil_log2(size);
  int tree = bits - (int)s->min_shift;
  if (tree > (int)s->num_trees) {
    int block_tree = bits - (int)(s->min_shift + 12);
    if (block_tree > (int)s->num_trees) return (((size - 1) >> s->seg_shift) + 1) << s->seg_shift;
  }
  return 1ull << bits;
}

GAL_DEVICE_INLINE bool owns(const state *s, const void *p) {
  return (uint64_t)((const char *)p - s->memory) < (s->num_segments << s->seg_shift);
}

}  // namespace gal
