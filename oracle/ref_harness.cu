// ref_harness.cu — drives the reference allocator's OWN device code
// (chillenzer/gallatin, include/gallatin/allocators/gallatin.cuh) on a GPU.
//
// TEST INFRASTRUCTURE ONLY.  Compiled in this container from the reference
// sources into oracle/_ref/ref_harness.cubin (see oracle/Makefile); run on the
// GPU by oracle/ref_loader.c.  Nothing in the product includes or loads it.
//
// The reference's host constructor (Gallatin::generate_on_device,
// gallatin.cuh:324-421) cannot be compiled for the Arm GPU host here, so
// ref_build restates its steps on the device with one thread, field by field,
// from a caller-provided scratch buffer:
//   segment tree + 9 sub-trees      veb.cuh:595-649, layer init veb.cuh:162-202,72-84
//   sub-tree clearing               boot_segment_trees, gallatin.cuh:136-145
//   pinned slots (128 halving to 4) shared_block_storage.cuh:251-274,36-42
//   alloc table + counters          memory_table.cuh:471-647,173-201
// after which every malloc/free call below is the reference's unmodified code.
#include <gallatin/allocators/gallatin.cuh>

#include "../gallatin_gb300/csrc/churn.cuh"

using namespace gallatin::allocators;

#ifndef REF_SEGMENT_BYTES
#define REF_SEGMENT_BYTES (16ULL * 1024 * 1024)
#endif
#ifndef REF_MIN_SIZE
#define REF_MIN_SIZE 16ULL
#endif
#ifndef REF_MAX_SIZE
#define REF_MAX_SIZE 4096ULL
#endif

using ref_type = Gallatin<REF_SEGMENT_BYTES, REF_MIN_SIZE, REF_MAX_SIZE>;

// the template arguments this cubin was built with (read by ref_loader.c)
extern "C" __device__ uint64_t ref_geometry[3] = {REF_SEGMENT_BYTES, REF_MIN_SIZE, REF_MAX_SIZE};
using table_type = alloc_table<REF_SEGMENT_BYTES, REF_MIN_SIZE>;
using pinned_type = pinned_shared_blocks<REF_MIN_SIZE, REF_MAX_SIZE>;

struct bump {
  char *base;
  uint64_t used, cap;
  bool ok;
  __device__ void *take(uint64_t n) {
    uint64_t start = (used + 255) & ~255ULL;
    if (start + n > cap) {
      ok = false;
      return nullptr;
    }
    used = start + n;
    return base + start;
  }
};

__device__ static veb_tree *build_veb(bump &b, uint64_t universe, uint64_t seed) {
  veb_tree *t = (veb_tree *)b.take(sizeof(veb_tree));
  if (!t) return nullptr;
  int max_height = 64 - __clzll(universe);
  int L = (max_height - 1) / 6 + 1;
  layer **layers = (layer **)b.take(L * sizeof(layer *));
  if (!layers) return nullptr;
  uint64_t u = universe;
  for (int i = 0; i < L; i++) {
    layer *ly = (layer *)b.take(sizeof(layer));
    if (!ly) return nullptr;
    uint64_t nw = (u - 1) / 64 + 1;
    uint64_t *bits = (uint64_t *)b.take(nw * sizeof(uint64_t));
    if (!bits) return nullptr;
    for (uint64_t w = 0; w < nw; w++) bits[w] = 0;
    for (uint64_t x = 0; x < u; x++) bits[x / 64] |= 1ULL << (x % 64);
    ly->universe_size = u;
    ly->num_blocks = nw;
    ly->bits = bits;
    layers[L - 1 - i] = ly;
    u = (u - 1) / 64 + 1;
  }
  t->num_layers = L;
  t->original_num_layers = L;
  t->layers = layers;
  t->seed = seed;
  t->total_universe = universe;
  return t;
}

// status[0]: 0 ok, 1 scratch too small; status[1]: scratch bytes used
extern "C" __global__ void ref_build(char *scratch, uint64_t scratch_bytes, char *arena,
                                    uint64_t num_bytes, uint64_t seed, ref_type **out_alloc,
                                    uint64_t *status) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  bump b{scratch, 0, scratch_bytes, true};
  uint64_t S = num_bytes / REF_SEGMENT_BYTES;
  ref_type *a = (ref_type *)b.take(sizeof(ref_type));
  if (!a) goto fail;
  a->segment_tree = build_veb(b, S, seed);
  if (!a->segment_tree) goto fail;
  {
    int num_trees = ref_type::get_num_trees();
    a->num_trees = num_trees;
    a->smallest_bits = gallatin::utils::get_first_bit_bigger(REF_MIN_SIZE);
    a->is_calloc = false;
    a->locks = 0;
    // pinned slots
    pinned_type *pb = (pinned_type *)b.take(sizeof(pinned_type));
    per_size_pinned_blocks **containers =
        (per_size_pinned_blocks **)b.take(num_trees * sizeof(per_size_pinned_blocks *));
    if (!pb || !containers) goto fail;
    uint64_t n = 128;
    for (int t = 0; t < num_trees; t++) {
      uint64_t cnt = n == 0 ? 1 : n;
      per_size_pinned_blocks *c = (per_size_pinned_blocks *)b.take(sizeof(per_size_pinned_blocks));
      uint64_t nu = (cnt - 1) / 64 + 1;
      uint64_t *bm = (uint64_t *)b.take(nu * sizeof(uint64_t));
      Block **blks = (Block **)b.take(cnt * sizeof(Block *));
      if (!c || !bm || !blks) goto fail;
      for (uint64_t i = 0; i < nu; i++) bm[i] = 0;
      for (uint64_t i = 0; i < cnt; i++) blks[i] = nullptr;
      c->num_blocks = cnt;
      c->block_bitmap = bm;
      c->blocks = blks;
      containers[t] = c;
      n = n / 2;
      if (n < MIN_PINNED_CUTOFF) n = MIN_PINNED_CUTOFF;
    }
    pb->block_containers = containers;
    a->local_blocks = pb;
    // sub trees, then cleared
    veb_tree **subs = (veb_tree **)b.take(num_trees * sizeof(veb_tree *));
    if (!subs) goto fail;
    for (int t = 0; t < num_trees; t++) {
      subs[t] = build_veb(b, S, (uint64_t)t + seed);
      if (!subs[t]) goto fail;
    }
    a->sub_trees = subs;
    for (uint64_t s = 0; s < S; s++)
      for (int t = 0; t < num_trees; t++) subs[t]->remove(s);
    // table
    table_type *tb = (table_type *)b.take(sizeof(table_type));
    if (!tb) goto fail;
    uint64_t bps = REF_SEGMENT_BYTES / (REF_MIN_SIZE * 4096);
    tb->chunk_ids = (uint16_t *)b.take(S * sizeof(uint16_t));
    tb->blocks = (Block *)b.take(S * bps * sizeof(Block));
    tb->queues = (Block **)b.take(S * bps * sizeof(Block *));
    tb->queue_counters = (uint *)b.take(S * sizeof(uint));
    tb->queue_free_counters = (uint *)b.take(S * sizeof(uint));
    tb->final_queue_free_counters = (uint *)b.take(S * sizeof(uint));
    tb->active_counts = (int *)b.take(S * sizeof(int));
    if (!b.ok) goto fail;
    tb->memory = arena;
    tb->num_segments = S;
    tb->blocks_per_segment = bps;
    tb->memory_control = device_only;
    tb->calloc_mode = false;
    tb->calloc_counters = nullptr;
    tb->calloc_enqueue_position = nullptr;
    tb->calloc_clear_counters = nullptr;
    tb->calloc_enqueue_finished = nullptr;
    tb->calloc_queues = nullptr;
    for (uint64_t s = 0; s < S; s++) {
      tb->chunk_ids[s] = 0xFFFF;
      tb->active_counts[s] = -1;
      tb->queue_counters[s] = 0;
      tb->queue_free_counters[s] = 0;
      tb->final_queue_free_counters[s] = 0;
    }
    for (uint64_t i = 0; i < S * bps; i++) {
      tb->blocks[i].init();
      tb->queues[i] = nullptr;
    }
    a->table = tb;
  }
  __threadfence();
  *out_alloc = a;
  status[0] = 0;
  status[1] = b.used;
  return;
fail:
  status[0] = 1;
  status[1] = b.used;
}

// boot_shared_block_container_one_thread (gallatin.cuh:196-221), <<<1,1>>>
extern "C" __global__ void ref_boot_one_thread(ref_type *a) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  int max_smid = 128;
  for (uint16_t tree = 0; tree < a->num_trees; tree++) {
    for (int i = 0; i < max_smid; i++) a->boot_block(tree, i);
    max_smid = max_smid / 2;
    if (max_smid < MIN_PINNED_CUTOFF) max_smid = MIN_PINNED_CUTOFF;
  }
}

// boot_shared_block_container (gallatin.cuh:171-191), launched <<<1,128>>>
// exactly as generate_on_device does (gallatin.cuh:415).
extern "C" __global__ void ref_boot_racy(ref_type *a) {
  uint64_t tid = gallatin::utils::get_tid();
  int max_smid = 128;
  uint16_t tree_id = 0;
  while (tree_id < a->num_trees) {
    if (tid >= (uint64_t)max_smid) return;
    a->boot_block(tree_id, (int)tid);
    max_smid = max_smid / 2;
    if (max_smid < MIN_PINNED_CUTOFF) max_smid = MIN_PINNED_CUTOFF;
    tree_id += 1;
  }
}

// serial trace, one thread (tests/src/gallatin_single_thread.cu:38-93 generalised)
extern "C" __global__ void ref_replay(ref_type *a, const uint64_t *ops, uint64_t nops,
                                     uint64_t *out, uint32_t *out_smid) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  out_smid[0] = gallatin::utils::get_smid();
  char *base = a->table->memory;
  for (uint64_t i = 0; i < nops; i++) {
    uint64_t op = ops[i];
    if (op >> 63) {
      uint64_t target = op & ~(1ULL << 63);
      if (target < i && out[target] != ~0ULL) a->free(base + out[target]);
      out[i] = ~0ULL;
    } else {
      void *p = a->malloc(op);
      out[i] = p ? (uint64_t)((char *)p - base) : ~0ULL;
    }
    __threadfence();
  }
}

// warp trace, one warp (step encoding of gal_replay_warp_trace: 33 words per
// step, word 0 = kind << 32 | lane mask; kind 0: the masked lanes call malloc
// together; kind 1: the masked lanes free, one at a time in lane order, the
// result of call step * 32 + lane named by the lane's word)
extern "C" __global__ void ref_replay_warp(ref_type *a, const uint64_t *steps, uint64_t nsteps,
                                           uint64_t *out, uint32_t *out_smid) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const uint32_t lane = threadIdx.x;
  if (lane == 0) out_smid[0] = gallatin::utils::get_smid();
  char *base = a->table->memory;
  for (uint64_t i = 0; i < nsteps; i++) {
    const uint64_t *w = steps + i * 33;
    const uint32_t kind = (uint32_t)(w[0] >> 32), mask = (uint32_t)w[0];
    uint64_t res = ~0ULL;
    __syncwarp();
    if (kind == 0) {
      if ((mask >> lane) & 1u) {
        void *p = a->malloc(w[1 + lane]);
        res = p ? (uint64_t)((char *)p - base) : ~0ULL;
      }
    } else {
      for (uint32_t l = 0; l < 32; l++) {
        if (((mask >> l) & 1u) && lane == l) {
          const uint64_t t = w[1 + l];
          if (t < i * 32 && out[t] != ~0ULL) a->free(base + out[t]);
        }
        __syncwarp();
      }
    }
    out[i * 32 + lane] = res;
    __threadfence();
    __syncwarp();
  }
}

struct export_ptrs {
  uint64_t *seg_tree_words;
  uint64_t *sub_tree_words;
  uint16_t *tree_ids;
  int32_t *active_counts;
  uint32_t *queue_counters, *queue_free_counters, *final_queue_free_counters;
  uint32_t *malloc_counters, *free_counters;
  int32_t *queues;
  int32_t *slots;
  uint32_t *locks;
  uint64_t veb_words;
};

__device__ static void export_veb(veb_tree *t, uint64_t *dst) {
  uint64_t o = 0;
  for (int l = 0; l < t->num_layers; l++) {
    layer *ly = t->layers[l];
    for (uint64_t w = 0; w < ly->num_blocks; w++) dst[o++] = ly->bits[w];
  }
}

// state in the layout-neutral view of include/gallatin_gb300.h; grid-stride
extern "C" __global__ void ref_export(ref_type *a, export_ptrs p) {
  uint64_t tid = gallatin::utils::get_tid();
  uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  table_type *tb = a->table;
  uint64_t S = tb->num_segments, bps = tb->blocks_per_segment;
  for (uint64_t i = tid; i < S * bps; i += nthreads) {
    p.malloc_counters[i] = tb->blocks[i].malloc_counter;
    p.free_counters[i] = tb->blocks[i].free_counter;
    Block *q = tb->queues[i];
    p.queues[i] = q ? (int32_t)(q - tb->blocks) : -1;
  }
  for (uint64_t s = tid; s < S; s += nthreads) {
    p.tree_ids[s] = tb->chunk_ids[s];
    p.active_counts[s] = tb->active_counts[s];
    p.queue_counters[s] = tb->queue_counters[s];
    p.queue_free_counters[s] = tb->queue_free_counters[s];
    p.final_queue_free_counters[s] = tb->final_queue_free_counters[s];
  }
  if (tid == 0) {
    export_veb(a->segment_tree, p.seg_tree_words);
    for (int t = 0; t < a->num_trees; t++) export_veb(a->sub_trees[t], p.sub_tree_words + t * p.veb_words);
    uint64_t o = 0;
    for (int t = 0; t < a->num_trees; t++) {
      per_size_pinned_blocks *c = a->local_blocks->block_containers[t];
      for (uint64_t i = 0; i < c->num_blocks; i++) {
        Block *b = c->blocks[i];
        p.slots[o++] = b ? (int32_t)(b - tb->blocks) : -1;
      }
    }
    p.locks[0] = a->locks;
  }
}

// ---- mixed-size churn through the reference's per-thread malloc/free ----
extern "C" __global__ void ref_churn_malloc(ref_type *a, void **ptrs, uint32_t *live, uint64_t base,
                                           uint64_t n, uint32_t seed, unsigned long long *stats) {
  galwl::churn_malloc_body(a, ptrs, live, base, n, seed, stats);
}

// persistent grid of 256-thread CTAs (ref_loader.c sizes it by occupancy)
extern "C" __global__ void __launch_bounds__(256)
    ref_churn_free(ref_type *a, void **ptrs, uint32_t *live, uint64_t nslots, uint32_t round,
                   uint32_t seed, int all, unsigned long long *stats) {
  __shared__ uint16_t lists[256 / 32][galwl::WARP_SLOTS];
  galwl::churn_free_warps(a, ptrs, live, nslots, round, seed, all != 0, stats, lists[threadIdx.x >> 5]);
}

// 1,048,576 threads x global_malloc(16) + tid stamp (tests/src/global_test.cu:34-118)
extern "C" __global__ void ref_stamp_malloc(ref_type *a, uint64_t n, uint64_t size, uint64_t **ptrs,
                                           unsigned long long *stats) {
  uint64_t tid = gallatin::utils::get_tid();
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)a->malloc(size);
  if (p) p[0] = tid;
  ptrs[tid] = p;
  galwl::warp_count(stats, 0, p != nullptr);
  galwl::warp_count(stats, 1, p == nullptr);
}

extern "C" __global__ void ref_stamp_free(ref_type *a, uint64_t n, uint64_t **ptrs,
                                         unsigned long long *stats) {
  uint64_t tid = gallatin::utils::get_tid();
  if (tid >= n) return;
  uint64_t *p = ptrs[tid];
  bool bad = false;
  if (p) {
    bad = p[0] != tid;
    a->free(p);
    ptrs[tid] = nullptr;
  }
  galwl::warp_count(stats, 2, bad);
  galwl::warp_count(stats, 3, p != nullptr);
}

// one thread per request through the reference's per-thread malloc / free
// (global_malloc / global_free, global_allocator.cuh:72-82, on a handle)
extern "C" __global__ void ref_malloc_sizes(ref_type *a, const uint64_t *sizes, uint64_t n, void **out) {
  uint64_t tid = gallatin::utils::get_tid();
  if (tid >= n) return;
  out[tid] = a->malloc(sizes[tid]);
}

extern "C" __global__ void ref_free_ptrs(ref_type *a, void *const *ptrs, uint64_t n) {
  uint64_t tid = gallatin::utils::get_tid();
  if (tid >= n) return;
  void *p = ptrs[tid];
  if (p) a->free(p);
}
