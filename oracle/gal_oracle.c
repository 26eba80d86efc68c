/*
 * gal_oracle.c — single-threaded CPU restatement of the reference allocator.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links it.
 *
 * Every function names the reference code it restates (paths inside the
 * chillenzer/gallatin project, include/gallatin/allocators/).  The model runs
 * one thread at a time, so each atomic of the reference is a plain
 * read-modify-write here and each warp team has one member.  Retry loops whose
 * repetition cannot change state when nothing else runs are executed once (the
 * comment at each says which).
 *
 * Parity is pinned against the reference's own CUDA build: oracle/ref_harness.cu
 * is compiled from the reference sources into oracle/_ref/ and run on a GB300;
 * tests/golden/ holds its outputs and tests/test_oracle_golden.py checks this
 * model against them.
 */
#include "gal_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXL GAL_MAX_VEB_LAYERS
#define MAXT GAL_MAX_TREES
#define NOBLK (-1)

static void orc_die(const char *msg) {
  fprintf(stderr, "gal_oracle: %s\n", msg);
  abort();
}

/* ------------------------------------------------------------------ bits */
static int popc64(uint64_t x) { return __builtin_popcountll(x); }
static int ffs64(uint64_t x) { return x ? __builtin_ctzll(x) + 1 : 0; } /* __ffsll */
static uint64_t bitmask(int n) { return n >= 64 ? ~0ULL : ((1ULL << n) - 1ULL); }

/* ceil(log2(x)) for x>0; 0 for x==0 (alloc_utils.cuh:382-398, device form) */
static int first_bit_bigger(uint64_t x) {
  if (x == 0) return 0;
  return 63 - __builtin_clzll(x) + (popc64(x) != 1);
}

/* count of contiguous ones from bit 0 (alloc_utils.cuh:440-453) */
static int cfc64(uint64_t bits) {
  int p = popc64(bits);
  if (p == 0 || p == 64) return p;
  return ffs64(~bits) - 1;
}

/* MurmurHash64A (Austin Appleby, public domain) of one 8-byte key, as used by
 * veb.cuh:950-956 through murmurhash.cuh:20-61. */
uint64_t orc_murmur64a_u64(uint64_t key, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ULL;
  const int r = 47;
  uint64_t h = seed ^ (8ULL * m);
  uint64_t k = key;
  k *= m;
  k ^= k >> r;
  k *= m;
  h ^= k;
  h *= m;
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

/* ------------------------------------------------------------------ vEB */
typedef struct {
  int L;
  uint64_t universe;
  uint64_t seed;
  uint64_t lu[MAXL];  /* items per layer, 0 = top */
  uint64_t nw[MAXL];  /* words per layer          */
  uint64_t off[MAXL]; /* word offset per layer    */
  uint64_t total;
  uint64_t *w;
} veb;

/* veb_tree::generate_on_device_nowait + layer init (veb.cuh:595-649,162-202,72-84) */
static void veb_init(veb *v, uint64_t universe, uint64_t seed) {
  memset(v, 0, sizeof(*v));
  int max_height = 64 - __builtin_clzll(universe);
  v->L = (max_height - 1) / 6 + 1;
  if (v->L > MAXL) orc_die("too many vEB layers");
  v->universe = universe;
  v->seed = seed;
  uint64_t u = universe;
  for (int i = 0; i < v->L; i++) {
    int layer = v->L - 1 - i;
    v->lu[layer] = u;
    v->nw[layer] = (u - 1) / 64 + 1;
    u = (u - 1) / 64 + 1;
  }
  uint64_t o = 0;
  for (int l = 0; l < v->L; l++) {
    v->off[l] = o;
    o += v->nw[l];
  }
  v->total = o;
  v->w = (uint64_t *)calloc(o, sizeof(uint64_t));
  for (int l = 0; l < v->L; l++)
    for (uint64_t i = 0; i < v->lu[l]; i++) v->w[v->off[l] + i / 64] |= 1ULL << (i % 64);
}

static uint64_t *vw(veb *v, int layer, uint64_t word) {
  if (word >= v->nw[layer]) orc_die("vEB word index out of range");
  return &v->w[v->off[layer] + word];
}

static int float_up(int *layer, uint64_t *high, int *low) { /* veb.cuh:697-704 */
  *layer -= 1;
  *low = (int)(*high & 63);
  *high = *high >> 6;
  return *layer >= 0;
}

static int float_down(veb *v, int *layer, uint64_t *high, int *low) { /* veb.cuh:706-712 */
  *layer += 1;
  *high = (*high << 6) + (uint64_t)*low;
  *low = -1;
  return *layer < v->L;
}

/* layer::find_next (veb.cuh:250-275) */
static int find_next(veb *v, int layer, uint64_t high, int low) {
  if (high >= v->lu[layer]) return -1;
  uint64_t b = *vw(v, layer, high);
  if (low == -1) return ffs64(b) - 1;
  return ffs64(b & ~bitmask(low + 1)) - 1;
}

/* veb_tree::remove (veb.cuh:737-755) */
static int veb_remove(veb *v, uint64_t x) {
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = v->L - 1;
  uint64_t *w = vw(v, layer, high);
  uint64_t old = *w;
  *w = old & ~(1ULL << low);
  if (!(old & (1ULL << low))) return 0;
  while (popc64(old) == 1 && float_up(&layer, &high, &low)) {
    w = vw(v, layer, high);
    old = *w;
    *w = old & ~(1ULL << low);
  }
  return 1;
}

/* veb_tree::insert_force_update (veb.cuh:775-798) */
static int veb_insert_force(veb *v, uint64_t x) {
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = v->L - 1;
  uint64_t *w = vw(v, layer, high);
  uint64_t old = *w;
  *w = old | (1ULL << low);
  if (old & (1ULL << low)) return 0;
  while (popc64(old) == 0 && float_up(&layer, &high, &low)) {
    w = vw(v, layer, high);
    old = *w;
    *w = old | (1ULL << low);
  }
  return 1;
}

/* veb_tree::query (veb.cuh:824-829) */
static int veb_query(veb *v, uint64_t x) {
  return (*vw(v, v->L - 1, x >> 6) >> (x & 63)) & 1;
}

/* veb_tree::successor_thorough (veb.cuh:878-916): strictly greater than q */
static uint64_t veb_successor(veb *v, uint64_t q) {
  uint64_t high = q >> 6;
  int low = (int)(q & 63);
  int layer = v->L - 1;
  for (;;) {
    for (;;) {
      int found = find_next(v, layer, high, low);
      if (found == -1) {
        if (layer == 0) return ORC_FAIL;
        float_up(&layer, &high, &low);
        continue;
      }
      break;
    }
    while (layer != v->L - 1) {
      low = find_next(v, layer, high, low);
      if (low == -1) break;
      float_down(v, &layer, &high, &low);
    }
    low = find_next(v, layer, high, low);
    if (low != -1) return (high << 6) + (uint64_t)low;
  }
}

/* veb_tree::lock_offset (veb.cuh:918-937) */
static uint64_t veb_lock_offset(veb *v, uint64_t start) {
  if (veb_query(v, start) && veb_remove(v, start)) return start;
  for (;;) {
    start = veb_successor(v, start);
    if (start == ORC_FAIL) return start;
    if (veb_remove(v, start)) return start;
  }
}

/* veb_tree::malloc_first (veb.cuh:979-991).  Its 15 attempts repeat an
 * identical search when one thread runs; one attempt is equivalent. */
static uint64_t veb_malloc_first(veb *v) { return veb_lock_offset(v, 0); }

/* veb_tree::find_random_valid_index (veb.cuh:946-977) */
static uint64_t veb_find_random(veb *v, uint64_t tid) {
  uint64_t hash1 = orc_murmur64a_u64(tid, v->seed);
  uint64_t hash2 = orc_murmur64a_u64(tid, hash1);
  for (uint64_t attempts = 0; attempts < 15; attempts++) {
    uint64_t start = (hash1 + attempts * hash2) % v->universe;
    if (veb_query(v, start)) return start;
    uint64_t idx = veb_successor(v, start);
    if (idx != ORC_FAIL) return idx;
  }
  return veb_successor(v, 0);
}

/* veb_tree::find_first_valid_index (veb.cuh:940-944): smallest listed id */
static uint64_t veb_find_first(veb *v) {
  if (veb_query(v, 0)) return 0;
  return veb_successor(v, 0);
}

/* layer::rollback (veb.cuh:305-321) on the bottom layer */
static void layer_rollback(veb *v, int layer, uint64_t start_block, uint64_t bits_to_set) {
  while (bits_to_set > 64) {
    *vw(v, layer, start_block) |= ~0ULL;
    bits_to_set -= 64;
    start_block++;
  }
  *vw(v, layer, start_block) |= bitmask((int)bits_to_set);
}

/* layer::gather_multiple (veb.cuh:323-452) on the bottom layer */
static uint64_t layer_gather_multiple(veb *v, uint64_t num_contiguous, uint32_t fix) {
  int layer = v->L - 1;
  uint64_t start_block = v->nw[layer] - 1;
  uint64_t num_needed = num_contiguous;
  while (start_block != 0) {
    num_contiguous = num_needed;
    uint64_t *w = vw(v, layer, start_block);
    int contig_start = cfc64(*w);
    if (contig_start == 0) {
      start_block -= 1;
      continue;
    }
    if ((uint64_t)contig_start >= num_contiguous) {
      uint64_t acq = bitmask((int)num_contiguous) << (contig_start - (int)num_contiguous);
      uint64_t got = *w;
      *w = got & ~acq;
      if ((uint64_t)popc64(got & acq) == num_contiguous)
        return start_block * 64 + (uint64_t)(contig_start - (int)num_contiguous);
      *w |= (acq & got);
      continue;
    }
    uint64_t got = *w;
    *w = got & ~bitmask(contig_start);
    int succeeded = 1;
    if (popc64(got & bitmask(contig_start)) == contig_start) {
      num_contiguous -= (uint64_t)contig_start;
      while (num_contiguous > 64) {
        if (start_block == 0 && (fix & ORC_FIX_RUN_BELOW_ARENA)) {
          layer_rollback(v, layer, 0, num_needed - num_contiguous);
          return ORC_FAIL;
        }
        start_block--;
        w = vw(v, layer, start_block);
        got = *w;
        *w = 0;
        if (popc64(got) != 64) {
          *w |= got;
          layer_rollback(v, layer, start_block + 1, num_needed - num_contiguous);
          succeeded = 0;
          break;
        }
        num_contiguous -= 64;
      }
      if (!succeeded) continue;
      if (start_block == 0 && (fix & ORC_FIX_RUN_BELOW_ARENA)) {
        layer_rollback(v, layer, 0, num_needed - num_contiguous);
        return ORC_FAIL;
      }
      start_block--;
      w = vw(v, layer, start_block);
      uint64_t fmask = bitmask((int)num_contiguous) << (64 - num_contiguous);
      uint64_t fbits = *w;
      *w = fbits & ~fmask;
      if ((uint64_t)popc64(fbits & fmask) == num_contiguous)
        return start_block * 64 + 64 - num_contiguous;
      *w |= (fmask & fbits);
      layer_rollback(v, layer, start_block + 1, num_needed - num_contiguous);
      continue;
    } else {
      *w |= (got & bitmask(contig_start));
      continue;
    }
  }
  /* veb.cuh:447: the reference rolls back (num_needed - num_contiguous) bits
   * at word 0 on exit although every failed try already restored its bits. */
  if (!(fix & ORC_FIX_GATHER_EXIT_ROLLBACK))
    layer_rollback(v, layer, 0, num_needed - num_contiguous);
  return ORC_FAIL;
}

/* layer::return_multiple (veb.cuh:495-523) */
static void layer_return_multiple(veb *v, int layer, uint64_t start, uint64_t n) {
  uint64_t block_index = start / 64;
  int block_start = (int)(start % 64);
  while (n + (uint64_t)block_start > 64) {
    int added = 64 - block_start;
    *vw(v, layer, block_index) |= bitmask(added) << block_start;
    block_start = 0;
    block_index += 1;
    n -= (uint64_t)added;
  }
  *vw(v, layer, block_index) |= bitmask((int)n) << block_start;
}

/* layer::remove / insert of one bit (veb.cuh:242-248) */
static void layer_remove_bit(veb *v, int layer, uint64_t high, int low) {
  *vw(v, layer, high) &= ~(1ULL << low);
}
static void layer_insert_bit(veb *v, int layer, uint64_t high, int low) {
  *vw(v, layer, high) |= (1ULL << low);
}

/* veb_tree::gather_multiple (veb.cuh:1160-1196) with
 * maybe_remove_layer_bits (veb.cuh:1100-1126) */
static uint64_t veb_gather_multiple(veb *v, uint64_t num_contiguous, uint32_t fix) {
  uint64_t found = layer_gather_multiple(v, num_contiguous, fix);
  uint64_t original = found;
  if (found == ORC_FAIL) return ORC_FAIL;
  for (int i = v->L - 2; i >= 0; i--) {
    uint64_t tread_high = (found + num_contiguous - 1) / 64 + 1;
    uint64_t tread_low = found / 64;
    found = tread_low;
    num_contiguous = tread_high - tread_low;
    for (uint64_t wb = found; wb < found + num_contiguous; wb++) {
      if (*vw(v, i + 1, wb) == 0) layer_remove_bit(v, i, wb / 64, (int)(wb % 64));
    }
  }
  return original;
}

/* veb_tree::return_multiple (veb.cuh:1198-1218) with
 * maybe_return_layer_bits (veb.cuh:1128-1154); ORC_FIX_RUN_RETURN_SUMMARY
 * lists every word the run made non-empty, not only the full ones */
static void veb_return_multiple(veb *v, uint64_t start_bit, uint64_t num_contiguous, uint32_t fix) {
  layer_return_multiple(v, v->L - 1, start_bit, num_contiguous);
  for (int i = v->L - 2; i >= 0; i--) {
    uint64_t tread_high = (start_bit + num_contiguous - 1) / 64 + 1;
    uint64_t tread_low = start_bit / 64;
    start_bit = tread_low;
    num_contiguous = tread_high - tread_low;
    for (uint64_t wb = start_bit; wb < start_bit + num_contiguous; wb++) {
      const uint64_t child = *vw(v, i + 1, wb);
      const int listed = (fix & ORC_FIX_RUN_RETURN_SUMMARY) ? child != 0 : popc64(child) == 64;
      if (listed) layer_insert_bit(v, i, wb / 64, (int)(wb % 64));
    }
  }
}

/* ------------------------------------------------------------ allocator */
struct orc_alloc {
  uint64_t seg_bytes, min_size, max_size;
  int smallest_bits;
  int num_trees;
  uint64_t S;   /* segments                         */
  uint64_t bps; /* table blocks per segment         */
  uint32_t fix;
  uint32_t policy;
  veb seg_tree;
  veb sub[MAXT];
  uint16_t *tree_ids;
  int32_t *active;
  uint32_t *qc, *qfc, *fqfc;
  uint32_t *mc, *fc;
  int32_t *queues;
  int nslots[MAXT];
  int32_t *slots[MAXT];
  int32_t *spares[MAXT]; /* the product's spare blocks (orc_set_spares) */
  int use_spares;
  uint32_t locks;
};

static uint64_t tree_alloc_size(orc_alloc *a, int tree) { return a->min_size << tree; }
/* alloc_table::get_blocks_per_segment (memory_table.cuh:1057-1061) */
static uint64_t blocks_per_segment_tree(orc_alloc *a, int tree) {
  return a->seg_bytes / (tree_alloc_size(a, tree) * 4096);
}
/* alloc_table::get_max_allocations_per_segment (memory_table.cuh:1065-1070) */
static uint64_t max_allocs_per_segment(orc_alloc *a) { return a->seg_bytes / a->min_size; }

/* Gallatin::generate_on_device minus the boot (gallatin.cuh:324-413),
 * alloc_table::generate_on_device_nowait (memory_table.cuh:471-647),
 * gallatin_init_counters_kernel (memory_table.cuh:173-201),
 * boot_segment_trees (gallatin.cuh:136-145),
 * pinned_shared_blocks::generate_on_device_nowait (shared_block_storage.cuh:251-274). */
orc_alloc *orc_create(uint64_t num_bytes, uint64_t seed, uint64_t seg_bytes, uint64_t min_size,
                      uint64_t max_size, uint32_t pinned_first, uint32_t pinned_min,
                      uint32_t fix_flags, uint32_t policy) {
  orc_alloc *a = (orc_alloc *)calloc(1, sizeof(orc_alloc));
  a->seg_bytes = seg_bytes;
  a->min_size = min_size;
  a->max_size = max_size;
  a->fix = fix_flags;
  a->policy = policy;
  a->S = num_bytes / seg_bytes;
  if (a->S == 0) orc_die("arena smaller than one segment");
  a->smallest_bits = first_bit_bigger(min_size);
  a->num_trees = first_bit_bigger(max_size) - first_bit_bigger(min_size) + 1;
  if (a->num_trees > MAXT) orc_die("too many trees");
  a->bps = seg_bytes / (min_size * 4096);
  veb_init(&a->seg_tree, a->S, seed);
  for (int i = 0; i < a->num_trees; i++) {
    veb_init(&a->sub[i], a->S, (uint64_t)i + seed);
    for (uint64_t s = 0; s < a->S; s++) veb_remove(&a->sub[i], s);
  }
  a->tree_ids = (uint16_t *)malloc(a->S * sizeof(uint16_t));
  memset(a->tree_ids, 0xFF, a->S * sizeof(uint16_t));
  a->active = (int32_t *)malloc(a->S * sizeof(int32_t));
  a->qc = (uint32_t *)calloc(a->S, sizeof(uint32_t));
  a->qfc = (uint32_t *)calloc(a->S, sizeof(uint32_t));
  a->fqfc = (uint32_t *)calloc(a->S, sizeof(uint32_t));
  for (uint64_t s = 0; s < a->S; s++) a->active[s] = -1;
  uint64_t nblocks = a->S * a->bps;
  a->mc = (uint32_t *)malloc(nblocks * sizeof(uint32_t));
  a->fc = (uint32_t *)calloc(nblocks, sizeof(uint32_t));
  a->queues = (int32_t *)malloc(nblocks * sizeof(int32_t));
  for (uint64_t b = 0; b < nblocks; b++) {
    a->mc[b] = 4097u; /* Block::init, block.cuh:64-68 */
    a->queues[b] = NOBLK;
  }
  uint64_t n = pinned_first;
  for (int t = 0; t < a->num_trees; t++) {
    uint64_t cnt = n == 0 ? 1 : n;
    a->nslots[t] = (int)cnt;
    a->slots[t] = (int32_t *)malloc(cnt * sizeof(int32_t));
    a->spares[t] = (int32_t *)malloc(cnt * sizeof(int32_t));
    for (uint64_t i = 0; i < cnt; i++) a->slots[t][i] = a->spares[t][i] = NOBLK;
    n = n / 2;
    if (n < pinned_min) n = pinned_min;
  }
  a->locks = 0;
  return a;
}

void orc_destroy(orc_alloc *a) {
  if (!a) return;
  free(a->seg_tree.w);
  for (int i = 0; i < a->num_trees; i++) {
    free(a->sub[i].w);
    free(a->slots[i]);
    free(a->spares[i]);
  }
  free(a->tree_ids);
  free(a->active);
  free(a->qc);
  free(a->qfc);
  free(a->fqfc);
  free(a->mc);
  free(a->fc);
  free(a->queues);
  free(a);
}

uint64_t orc_arena_bytes(orc_alloc *a) { return a->S * a->seg_bytes; }

/* alloc_table::setup_segment (memory_table.cuh:746-818) */
static int setup_segment(orc_alloc *a, uint64_t seg, int tree) {
  if (a->tree_ids[seg] != 0xFFFF) return 0;
  a->tree_ids[seg] = (uint16_t)tree;
  int nb = (int)blocks_per_segment_tree(a, tree);
  for (int i = 0; i < nb; i++) a->queues[seg * a->bps + (uint64_t)i] = NOBLK;
  a->qc[seg] = 0;
  a->qfc[seg] = 0;
  a->fqfc[seg] = 0;
  a->active[seg] = nb - 1;
  return 1;
}

/* Gallatin::gather_new_segment (gallatin.cuh:1465-1510) */
static int64_t gather_new_segment(orc_alloc *a, int tree) {
  uint64_t seg = veb_malloc_first(&a->seg_tree);
  if (seg == ORC_FAIL) return -1;
  if (!setup_segment(a, seg, tree)) orc_die("setup_segment failed (reference traps)");
  veb_insert_force(&a->sub[tree], seg);
  return (int64_t)seg;
}

/* alloc_table::get_block (memory_table.cuh:915-993) */
static int32_t get_block(orc_alloc *a, uint64_t seg, int tree, int *empty) {
  *empty = 0;
  int32_t active_count = a->active[seg]--;
  if (active_count < 0) {
    a->active[seg]++;
    return NOBLK;
  }
  if (a->tree_ids[seg] != (uint16_t)tree) {
    a->active[seg]++;
    return NOBLK;
  }
  uint64_t nb = blocks_per_segment_tree(a, tree);
  int queue_pos = (int)(a->qc[seg]++);
  int32_t blk;
  if ((uint64_t)(int64_t)queue_pos < nb) {
    blk = (int32_t)(seg * a->bps + (uint64_t)queue_pos);
  } else {
    uint64_t wrapped = (uint64_t)queue_pos % nb;
    blk = a->queues[seg * a->bps + wrapped];
    a->queues[seg * a->bps + wrapped] = NOBLK;
  }
  if (blk == NOBLK) orc_die("null block from recycle ring (reference traps)");
  a->mc[blk] = (uint32_t)tree << 20; /* Block::init_malloc, block.cuh:215-224 */
  if (active_count == 0) *empty = 1;
  return blk;
}

/* sub-tree choice: reference hashed start or smallest id */
static uint64_t subtree_pick(orc_alloc *a, int tree, uint64_t tid) {
  if (a->policy == GAL_POLICY_LOWEST) return veb_find_first(&a->sub[tree]);
  return veb_find_random(&a->sub[tree], tid);
}

/* Gallatin::request_new_block_from_tree (gallatin.cuh:1525-1631).  When one
 * thread runs, a failed gather leaves the state unchanged, so the reference's
 * 1000 identical retries are folded into one. */
static int32_t request_new_block(orc_alloc *a, int tree, uint64_t tid) {
  for (uint64_t guard = 0; guard < 1000000; guard++) {
    uint64_t seg = subtree_pick(a, tree, tid);
    if (seg == ORC_FAIL) {
      int64_t got = gather_new_segment(a, tree);
      if (got == -1) return NOBLK;
      seg = (uint64_t)got;
    }
    int last = 0;
    int32_t blk = get_block(a, seg, tree, &last);
    if (last) {
      veb_remove(&a->sub[tree], seg);
      gather_new_segment(a, tree);
    }
    if (blk != NOBLK) return blk;
  }
  orc_die("request_new_block did not settle");
  return NOBLK;
}

/* Gallatin::boot_block (gallatin.cuh:726-787) */
static int boot_block(orc_alloc *a, int tree, int smid, uint64_t tid) {
  if (smid >= a->nslots[tree]) return -1;
  int32_t blk = request_new_block(a, tree, tid);
  if (blk == NOBLK) return -2;
  if (a->tree_ids[(uint64_t)blk / a->bps] != tree) return -3;
  if (a->slots[tree][smid] != NOBLK) return -4;
  a->slots[tree][smid] = blk;
  return 0;
}

/* boot_shared_block_container_one_thread (gallatin.cuh:196-221): every slot
 * is tried even after one finds no block (the slot stays empty); the first
 * failure is reported */
int orc_boot_one_thread(orc_alloc *a) {
  int first = 0;
  for (int tree = 0; tree < a->num_trees; tree++)
    for (int i = 0; i < a->nslots[tree]; i++) {
      int r = boot_block(a, tree, i, 0);
      if (r && !first) first = r;
    }
  return first;
}

static void free_offset(orc_alloc *a, uint64_t offset);

/* Gallatin::return_block (gallatin.cuh:1637-1726) with
 * alloc_table::reserve_segment_slot / finish_freeing_block
 * (memory_table.cuh:1158-1241) */
static void return_block(orc_alloc *a, int32_t blk, uint64_t seg, int tree) {
  uint64_t num_blocks = blocks_per_segment_tree(a, tree);
  uint32_t pos = a->qfc[seg]++;
  uint32_t live = (uint32_t)(pos % num_blocks);
  a->queues[seg * a->bps + live] = blk;
  if (a->fqfc[seg] != pos) orc_die("free ring finalisation out of order");
  a->fqfc[seg] = pos + 1;
  uint32_t reserved_slot = live;
  if (1.0 * reserved_slot / num_blocks >= 0.1 &&
      (1.0 * (uint32_t)(reserved_slot - 1) / num_blocks) < 0.1) {
    veb_insert_force(&a->sub[tree], seg);
  }
  int32_t return_id = a->active[seg]++;
  int need_to_deregister = 0;
  if ((uint64_t)(int64_t)return_id == num_blocks - 2) {
    if (a->active[seg] == (int32_t)(num_blocks - 1)) {
      a->active[seg] = -1;
      need_to_deregister = 1;
    }
  }
  if (need_to_deregister) {
    veb_remove(&a->sub[tree], seg);
    if (a->tree_ids[seg] != (uint16_t)tree) orc_die("reset_tree_id failed (reference traps)");
    a->tree_ids[seg] = 0xFFFF;
    veb_insert_force(&a->seg_tree, seg);
  }
}

/* Gallatin::free_block (gallatin.cuh:1732-1766), non-calloc branch */
static void free_block(orc_alloc *a, int32_t blk) {
  uint64_t seg = (uint64_t)blk / a->bps;
  int tree = a->tree_ids[seg];
  return_block(a, blk, seg, tree);
}

/* Gallatin::free_offset (gallatin.cuh:1774-1827) with
 * Block::block_free_multiple / reset_free (block.cuh:87-98,200-212) */
static void free_offset(orc_alloc *a, uint64_t offset) {
  uint64_t blk = offset / 4096;
  uint32_t old = a->fc[blk];
  a->fc[blk] = old + 1;
  if (old + 1 == 4096) {
    a->fc[blk] = 0;
    free_block(a, (int32_t)blk);
  }
}

/* Trim (an addition of the product, gal_trim; the reference has none):
 * retire every pinned block in slot order, crediting the slices it never
 * handed out so that a block with nothing live goes back to its segment, then
 * boot the slots again in the one-thread order. */
int orc_trim(orc_alloc *a) {
  for (int pass = 0; pass < 2; pass++) /* spare blocks first, then the slots */
  for (int tree = 0; tree < a->num_trees; tree++)
    for (int i = 0; i < a->nslots[tree]; i++) {
      int32_t *cell = pass == 0 ? &a->spares[tree][i] : &a->slots[tree][i];
      int32_t blk = *cell;
      if (blk == NOBLK) continue;
      *cell = NOBLK;
      uint32_t merged = a->mc[blk];
      a->mc[blk] = merged + 4096u;
      uint32_t c = merged & 0xFFFFFu;
      if (c < 4096u) {
        a->fc[blk] += 4096u - c;
        if (a->fc[blk] == 4096u) {
          a->fc[blk] = 0;
          free_block(a, blk);
        }
      }
    }
  /* segments of a class none of whose blocks is out (those gathered ahead
   * when a class took the last block of its previous segment) go back too */
  for (uint64_t seg = 0; seg < a->S; seg++) {
    int tree = a->tree_ids[seg];
    if (tree >= a->num_trees) continue;
    if (a->active[seg] != (int32_t)(blocks_per_segment_tree(a, tree) - 1)) continue;
    a->active[seg] = -1;
    veb_remove(&a->sub[tree], seg);
    a->tree_ids[seg] = 0xFFFF;
    veb_insert_force(&a->seg_tree, seg);
  }
  return orc_boot_one_thread(a);
}

/* pinned slot choice (shared_block_storage.cuh:119-134) */
static int valid_block_index(orc_alloc *a, int tree, uint32_t smid) {
  int n = a->nslots[tree];
  int my = (int)((uint64_t)smid % (uint64_t)n);
  int original = my;
  int counter = 0;
  while (a->slots[tree][my] == NOBLK && my != (original - 1)) {
    my = (my + 1) % n;
    counter += 1;
    if (counter >= 30) break;
  }
  return my;
}

/* Gallatin::replace_block (gallatin.cuh:1083-1138) */
static int replace_block(orc_alloc *a, int tree, int slot, int32_t blk, uint64_t tid) {
  if (a->slots[tree][slot] == blk) {
    a->slots[tree][slot] = NOBLK;
    int32_t nb = request_new_block(a, tree, tid);
    if (nb == NOBLK) return 0;
    if (a->slots[tree][slot] != NOBLK) orc_die("slot refilled concurrently (reference traps)");
    a->slots[tree][slot] = nb;
  }
  return 1;
}

/* The product's spare blocks (gal_config.spare_blocks; no reference
 * counterpart): the crossing lane's team leader swaps the slot's prepared
 * block in instead of searching for one, falling back to replace_block when
 * none is ready, and then prepares the next one with its own thread id.  A
 * single thread always finds the slot still holding the exhausted block. */
static void replace_or_swap(orc_alloc *a, int tree, int slot, int32_t blk, uint64_t tid) {
  if (!a->use_spares) {
    replace_block(a, tree, slot, blk, tid);
    return;
  }
  int32_t nx = a->spares[tree][slot];
  a->spares[tree][slot] = NOBLK;
  if (nx == NOBLK) {
    replace_block(a, tree, slot, blk, tid);
  } else if (a->slots[tree][slot] != blk) {
    a->fc[nx] = 0; /* the slot moved on: all 4096 slices credited, the spare goes back */
    free_block(a, nx);
    return;
  } else {
    a->slots[tree][slot] = nx;
  }
  if (a->spares[tree][slot] == NOBLK) {
    int32_t nb = request_new_block(a, tree, tid);
    if (nb != NOBLK) a->spares[tree][slot] = nb;
  }
}

void orc_set_spares(orc_alloc *a, int on) { a->use_spares = on != 0; }

/* Gallatin::malloc_slice_allocation (gallatin.cuh:865-1078), team of one.
 * The reference's 500 attempts are kept: a failed attempt can replace the
 * pinned block, so a retry can succeed. */
static uint64_t malloc_slice(orc_alloc *a, int tree, uint32_t alloc_count, uint32_t smid,
                             uint64_t tid) {
  for (int attempts = 0; attempts < 500; attempts++) {
    int slot = valid_block_index(a, tree, smid);
    int32_t blk = a->slots[tree][slot];
    if (blk == NOBLK) continue;
    uint64_t gbid = (uint64_t)blk;
    uint32_t merged = a->mc[blk];
    a->mc[blk] = merged + alloc_count; /* block_malloc_tree_multi_size */
    uint64_t allocation = (uint64_t)(merged & 0xFFFFFu);
    int should_replace = (allocation <= 4095 && (allocation + alloc_count) > 4095);
    int start_valid = allocation <= 4095;
    int end_valid = allocation + alloc_count <= 4096;
    uint32_t leftover = (uint32_t)((start_valid && end_valid) * (uint64_t)(alloc_count - 1) +
                                   (start_valid && !end_valid) * (4096 - allocation));
    if (leftover > 0) { /* block_correct_frees */
      a->fc[blk] += leftover;
      if ((a->fix & ORC_FIX_LEFTOVER_COMPLETES) && a->fc[blk] == 4096) {
        a->fc[blk] = 0;
        free_block(a, blk);
      }
    }
    if (allocation + alloc_count > 4096) allocation = ORC_FAIL;
    if (should_replace) replace_or_swap(a, tree, slot, blk, tid);
    if (allocation != ORC_FAIL) {
      if ((merged >> 20) != (uint32_t)tree) { /* Block::check_valid */
        free_offset(a, allocation + gbid * 4096);
      } else {
        return allocation + gbid * 4096;
      }
    }
  }
  return ORC_FAIL;
}

/* Gallatin::malloc_slice_allocation (gallatin.cuh:865-1078) for one
 * convergent warp whose lanes in `pending` all ask for slices of `tree`
 * (counts[l] slices each: 1, or 2-8 for the big-slice sizes of the last tree),
 * i.e. one labeled_partition team.  Per attempt: the team's lowest lane picks
 * the slot; the exclusive scan of the counts in lane order gives each lane its
 * place after the one atomicAdd of the team's total, which the team's last
 * lane issues (Block::block_malloc_tree_multi_size, block.cuh:245-264); the
 * leftover slices are credited as one sum (block_correct_frees, :267-281);
 * the lowest lane replaces the block when some lane crossed slice 4095, with
 * its own thread id as the sub-tree seed.  Lanes that got a slice leave the
 * team; the rest form the next attempt's team.  The reference's 10 x 500
 * attempts are one loop of 5,000: a failing attempt leaves no other state. */
static void malloc_slice_team(orc_alloc *a, int tree, const uint32_t *counts, uint32_t pending,
                              uint32_t smid, uint64_t tid0, uint64_t *res) {
  for (int attempts = 0; attempts < 5000 && pending; attempts++) {
    int leader = __builtin_ctz(pending);
    int slot = valid_block_index(a, tree, smid);
    int32_t blk = a->slots[tree][slot];
    if (blk == NOBLK) continue;
    uint32_t merged = a->mc[blk];
    uint32_t total = 0;
    for (int l = 0; l < 32; l++)
      if ((pending >> l) & 1u) total += counts[l];
    a->mc[blk] = merged + total;
    uint64_t alloc[32];
    uint32_t prefix = 0, leftover = 0;
    int should_replace = 0;
    for (int l = 0; l < 32; l++) {
      if (!((pending >> l) & 1u)) continue;
      uint64_t al = (uint64_t)(merged & 0xFFFFFu) + prefix;
      uint32_t c = counts[l];
      prefix += c;
      int start_valid = al <= 4095, end_valid = al + c <= 4096;
      if (start_valid && al + c > 4095) should_replace = 1;
      leftover += start_valid ? (end_valid ? c - 1 : (uint32_t)(4096 - al)) : 0;
      alloc[l] = end_valid ? al : ORC_FAIL;
    }
    if (leftover > 0) {
      a->fc[blk] += leftover;
      if ((a->fix & ORC_FIX_LEFTOVER_COMPLETES) && a->fc[blk] == 4096) {
        a->fc[blk] = 0;
        free_block(a, blk);
      }
    }
    if (should_replace) replace_or_swap(a, tree, slot, blk, tid0 + (uint64_t)leader);
    for (int l = 0; l < 32; l++) {
      if (!((pending >> l) & 1u) || alloc[l] == ORC_FAIL) continue;
      uint64_t off = alloc[l] + (uint64_t)blk * 4096;
      if ((merged >> 20) != (uint32_t)tree) { /* Block::check_valid */
        free_offset(a, off);
      } else {
        res[l] = off;
        pending &= ~(1u << l);
      }
    }
  }
}

/* Gallatin::malloc_block_allocation (gallatin.cuh:828-861) with
 * Block::malloc_fill_block (block.cuh:288-340) */
static uint64_t malloc_block(orc_alloc *a, int tree, uint64_t tid) {
  int32_t blk = request_new_block(a, tree, tid);
  if (blk == NOBLK) return ORC_FAIL;
  uint64_t gbid = (uint64_t)blk;
  uint32_t old_merged = a->mc[blk];
  a->mc[blk] = old_merged + 4096;
  uint32_t old_count = old_merged & 0xFFFFFu;
  if ((old_merged >> 20) != (uint32_t)tree) orc_die("whole-block fill on foreign block (reference traps)");
  a->fc[blk] += 4095u - old_count;
  if (old_count != 0) {
    free_offset(a, gbid * 4096);
    return ORC_FAIL;
  }
  return gbid * 4096;
}

/* Gallatin::malloc_segment_allocation (gallatin.cuh:790-826) */
static uint64_t malloc_segments(orc_alloc *a, uint32_t count) {
  uint64_t idx = veb_gather_multiple(&a->seg_tree, count, a->fix);
  if (idx == ORC_FAIL) return ORC_FAIL;
  if (a->tree_ids[idx] != 0xFFFF) orc_die("set_tree_id failed (reference traps)");
  a->tree_ids[idx] = (uint16_t)(a->num_trees + 1 + count);
  return idx * a->bps * 4096;
}

/* alloc_table::offset_to_allocation (memory_table.cuh:1072-1086), as a byte
 * offset from the arena base */
static uint64_t offset_to_bytes(orc_alloc *a, uint64_t offset, int tree) {
  uint64_t per = max_allocs_per_segment(a);
  uint64_t seg = offset / per;
  uint64_t rel = offset % per;
  return seg * a->seg_bytes + rel * tree_alloc_size(a, tree);
}

/* Gallatin::malloc (gallatin.cuh:1186-1276) */
uint64_t orc_malloc(orc_alloc *a, uint64_t size, uint32_t smid, uint64_t tid) {
  int tree = size < a->min_size ? 0 : first_bit_bigger(size) - a->smallest_bits;
  uint32_t alloc_count = 1;
  if (tree >= a->num_trees) {
    int smallest_tree_bits = first_bit_bigger(a->min_size * 4096);
    int block_tree = first_bit_bigger(size) - smallest_tree_bits;
    if (block_tree < 0) {
      alloc_count = 1u << (tree - (a->num_trees - 1));
      tree = a->num_trees - 1;
    } else if (block_tree < a->num_trees) {
      /* 500 attempts: a failed attempt with one thread leaves no state to
       * retry against except the whole-block collision, which cannot occur */
      uint64_t off = malloc_block(a, block_tree, tid);
      if (off == ORC_FAIL) return ORC_FAIL;
      return offset_to_bytes(a, off, block_tree);
    } else {
      uint32_t count = (uint32_t)((size - 1) / a->seg_bytes + 1);
      uint64_t off = malloc_segments(a, count);
      if (off == ORC_FAIL) return ORC_FAIL;
      return offset_to_bytes(a, off, 0);
    }
  }
  for (int attempt = 0; attempt < 10; attempt++) {
    uint64_t off = malloc_slice(a, tree, alloc_count, smid, tid);
    if (off != ORC_FAIL) return offset_to_bytes(a, off, tree);
  }
  return ORC_FAIL;
}

/* Gallatin::free (gallatin.cuh:1378-1461) with
 * alloc_table::allocation_to_offset (memory_table.cuh:1090-1127) and
 * submit_segment_for_free (gallatin.cuh:1283-1302) */
void orc_free(orc_alloc *a, uint64_t byte_offset) {
  uint64_t seg = byte_offset / a->seg_bytes;
  if (seg >= a->S) orc_die("free outside the arena");
  uint16_t tree = a->tree_ids[seg];
  if (tree == 0xFFFF || tree == (uint16_t)a->num_trees) orc_die("free into a free segment");
  if (tree > a->num_trees) {
    uint16_t count = (uint16_t)(tree - a->num_trees - 1);
    veb_return_multiple(&a->seg_tree, seg, count, a->fix);
    a->tree_ids[seg] = 0xFFFF;
    return;
  }
  uint64_t seg_off = byte_offset - seg * a->seg_bytes;
  uint64_t offset = seg_off / tree_alloc_size(a, tree) + seg * max_allocs_per_segment(a);
  free_offset(a, offset);
}

int orc_replay(orc_alloc *a, const uint64_t *ops, uint64_t nops, uint32_t smid, uint64_t tid,
               uint64_t *out) {
  for (uint64_t i = 0; i < nops; i++) {
    uint64_t op = ops[i];
    if (op >> 63) {
      uint64_t target = op & ~(1ULL << 63);
      if (target >= i) return -1;
      if (out[target] != ORC_FAIL) orc_free(a, out[target]);
      out[i] = ORC_FAIL;
    } else {
      out[i] = orc_malloc(a, op, smid, tid);
    }
  }
  return 0;
}

/* A trace of warp-wide calls, replayed by one warp (lanes 0-31 of thread ids
 * tid0..tid0+31).  Step i is 33 words: word 0 = kind << 32 | lane mask, then
 * one word per lane.  Kind 0: the masked lanes call malloc together with the
 * lane's size (all sizes of one step in the same slice class); kind 1: the
 * masked lanes free, one lane at a time in lane order, the result of the
 * earlier call whose index (step * 32 + lane) the lane's word holds.  out has
 * 32 words per step: byte offsets of kind-0 results, ORC_FAIL elsewhere.
 * A free of a failed call is skipped.  Returns 0, or -1 for a malformed step
 * (mixed classes, a tier other than slices, a free of a later call). */
int orc_replay_warp(orc_alloc *a, const uint64_t *steps, uint64_t nsteps, uint32_t smid,
                    uint64_t tid0, uint64_t *out) {
  for (uint64_t i = 0; i < nsteps; i++) {
    const uint64_t *w = steps + i * 33;
    uint32_t kind = (uint32_t)(w[0] >> 32), mask = (uint32_t)w[0];
    uint64_t *o = out + i * 32;
    for (int l = 0; l < 32; l++) o[l] = ORC_FAIL;
    if (kind == 1) {
      for (int l = 0; l < 32; l++) {
        if (!((mask >> l) & 1u)) continue;
        uint64_t target = w[1 + l];
        if (target >= i * 32) return -1;
        if (out[target] != ORC_FAIL) orc_free(a, out[target]);
      }
      continue;
    }
    if (kind != 0) return -1;
    int tree = -1;
    uint32_t counts[32] = {0};
    for (int l = 0; l < 32; l++) {
      if (!((mask >> l) & 1u)) continue;
      uint64_t size = w[1 + l];
      int t = size < a->min_size ? 0 : first_bit_bigger(size) - a->smallest_bits;
      uint32_t c = 1;
      if (t >= a->num_trees) {
        int block_tree = first_bit_bigger(size) - first_bit_bigger(a->min_size * 4096);
        if (block_tree >= 0) return -1;
        c = 1u << (t - (a->num_trees - 1));
        t = a->num_trees - 1;
      }
      if (tree >= 0 && t != tree) return -1;
      tree = t;
      counts[l] = c;
    }
    if (tree < 0) continue;
    uint64_t res[32];
    for (int l = 0; l < 32; l++) res[l] = ORC_FAIL;
    malloc_slice_team(a, tree, counts, mask, smid, tid0, res);
    for (int l = 0; l < 32; l++)
      if (res[l] != ORC_FAIL) o[l] = offset_to_bytes(a, res[l], tree);
  }
  return 0;
}

/* ------------------------------------------------------------ state view */
int orc_dims(orc_alloc *a, gal_state_dims *d) {
  memset(d, 0, sizeof(*d));
  d->num_segments = a->S;
  d->num_trees = (uint32_t)a->num_trees;
  d->blocks_per_segment = (uint32_t)a->bps;
  d->veb_layers = (uint32_t)a->seg_tree.L;
  d->veb_words = (uint32_t)a->seg_tree.total;
  uint32_t tot = 0;
  for (int t = 0; t < a->num_trees; t++) {
    d->slot_counts[t] = (uint32_t)a->nslots[t];
    tot += (uint32_t)a->nslots[t];
  }
  d->total_slots = tot;
  return 0;
}

int orc_export(orc_alloc *a, const gal_state_view *v) {
  uint64_t W = a->seg_tree.total, nb = a->S * a->bps;
  memcpy(v->seg_tree_words, a->seg_tree.w, W * 8);
  for (int t = 0; t < a->num_trees; t++) memcpy(v->sub_tree_words + (uint64_t)t * W, a->sub[t].w, W * 8);
  memcpy(v->tree_ids, a->tree_ids, a->S * 2);
  memcpy(v->active_counts, a->active, a->S * 4);
  memcpy(v->queue_counters, a->qc, a->S * 4);
  memcpy(v->queue_free_counters, a->qfc, a->S * 4);
  memcpy(v->final_queue_free_counters, a->fqfc, a->S * 4);
  memcpy(v->malloc_counters, a->mc, nb * 4);
  memcpy(v->free_counters, a->fc, nb * 4);
  memcpy(v->queues, a->queues, nb * 4);
  uint64_t o = 0;
  for (int t = 0; t < a->num_trees; t++) {
    memcpy(v->slots + o, a->slots[t], (uint64_t)a->nslots[t] * 4);
    o += (uint64_t)a->nslots[t];
  }
  ((gal_state_view *)v)->locks = a->locks;
  ((gal_state_view *)v)->error_word = 0;
  return 0;
}

int orc_import(orc_alloc *a, const gal_state_view *v) {
  uint64_t W = a->seg_tree.total, nb = a->S * a->bps;
  memcpy(a->seg_tree.w, v->seg_tree_words, W * 8);
  for (int t = 0; t < a->num_trees; t++) memcpy(a->sub[t].w, v->sub_tree_words + (uint64_t)t * W, W * 8);
  memcpy(a->tree_ids, v->tree_ids, a->S * 2);
  memcpy(a->active, v->active_counts, a->S * 4);
  memcpy(a->qc, v->queue_counters, a->S * 4);
  memcpy(a->qfc, v->queue_free_counters, a->S * 4);
  memcpy(a->fqfc, v->final_queue_free_counters, a->S * 4);
  memcpy(a->mc, v->malloc_counters, nb * 4);
  memcpy(a->fc, v->free_counters, nb * 4);
  memcpy(a->queues, v->queues, nb * 4);
  uint64_t o = 0;
  for (int t = 0; t < a->num_trees; t++) {
    memcpy(a->slots[t], v->slots + o, (uint64_t)a->nslots[t] * 4);
    for (int i = 0; i < a->nslots[t]; i++) a->spares[t][i] = NOBLK; /* the view holds none */
    o += (uint64_t)a->nslots[t];
  }
  a->locks = v->locks;
  return 0;
}

/* ------------------------------------------------------------ traces */
static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* Serial trace: each op draws r; if r % 100 < malloc_pct or nothing is live
 * it is a malloc of size_quantum * (1 + next % size_steps), else a free of a
 * uniformly chosen live malloc (swap-remove from the live list). */
int orc_gen_serial_trace(uint64_t seed, uint64_t nops, uint32_t malloc_pct, uint64_t size_quantum,
                         uint64_t size_steps, uint64_t *ops) {
  uint64_t s = seed;
  uint64_t *live = (uint64_t *)malloc((nops + 1) * sizeof(uint64_t));
  uint64_t nlive = 0;
  for (uint64_t i = 0; i < nops; i++) {
    uint64_t r = splitmix64(&s);
    if ((r % 100) < malloc_pct || nlive == 0) {
      uint64_t size = size_quantum * (1 + splitmix64(&s) % size_steps);
      ops[i] = size;
      live[nlive++] = i;
    } else {
      uint64_t j = splitmix64(&s) % nlive;
      ops[i] = (1ULL << 63) | live[j];
      live[j] = live[--nlive];
    }
  }
  free(live);
  return 0;
}

/* Trace with log-uniform sizes: k uniform in [lo_bits, hi_bits], size uniform
 * in [2^(k-1)+1, 2^k] (k == lo_bits: [1, 2^k]); malloc/free choice as above. */
int orc_gen_trace_log(uint64_t seed, uint64_t nops, uint32_t malloc_pct, uint32_t lo_bits,
                      uint32_t hi_bits, uint64_t *ops) {
  uint64_t s = seed;
  uint64_t *live = (uint64_t *)malloc((nops + 1) * sizeof(uint64_t));
  uint64_t nlive = 0;
  for (uint64_t i = 0; i < nops; i++) {
    uint64_t r = splitmix64(&s);
    if ((r % 100) < malloc_pct || nlive == 0) {
      uint32_t k = lo_bits + (uint32_t)(splitmix64(&s) % (uint64_t)(hi_bits - lo_bits + 1));
      uint64_t lo = (k == lo_bits) ? 1 : (1ULL << (k - 1)) + 1;
      uint64_t hi = 1ULL << k;
      ops[i] = lo + splitmix64(&s) % (hi - lo + 1);
      live[nlive++] = i;
    } else {
      uint64_t j = splitmix64(&s) % nlive;
      ops[i] = (1ULL << 63) | live[j];
      live[j] = live[--nlive];
    }
  }
  free(live);
  return 0;
}
