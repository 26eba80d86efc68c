// gal_lib.cu — host side of the allocator behind the C ABI of
// include/gallatin_gb300.h, plus the kernels the library launches itself
// (initialisation, boot, state export/import, statistics, serial replay,
// per-thread and batched malloc/free).
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <unordered_map>
#include <vector>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"
#include "gal_batch.cuh"
#include "gal_internal.h"

struct gal_handle {
  int device = 0;
  gal_config cfg{};
  uint64_t num_bytes = 0, seed = 0;
  gal::state st{};             // host copy of the device-resident state
  gal::state *d_state = nullptr;
  char *meta = nullptr;
  size_t meta_bytes = 0;
  char *arena = nullptr;
  uint64_t arena_bytes = 0;
  gal_state_dims dims{};
  int grid_free = 0;  // persistent grid of the batched free kernel (0: not yet known)
};

namespace {

std::mutex g_mu;
std::unordered_map<const void *, gal_handle *> g_by_state;
gal_handle *g_global = nullptr;
gal_handle *g_global_host = nullptr;  // gal_init_host

#define CUDA_TRY(x)                                                                   \
  do {                                                                                \
    cudaError_t _e = (x);                                                             \
    if (_e != cudaSuccess) {                                                          \
      fprintf(stderr, "gallatin_gb300: %s failed: %s\n", #x, cudaGetErrorString(_e)); \
      return GAL_ERR_CUDA;                                                            \
    }                                                                                 \
  } while (0)

bool is_pow2(uint64_t x) { return x && !(x & (x - 1)); }
uint32_t log2u(uint64_t x) { return 63 - __builtin_clzll(x); }

size_t align_up(size_t x, size_t a) { return (x + a - 1) & ~(a - 1); }

// ---------------------------------------------------------------- kernels
// malloc words 4097 (Block::init), every segment's count -1 in generation 0,
// the segment tree full; everything else was zeroed
__global__ void k_init_words(gal::state st, uint64_t nblocks) {
  uint64_t *seg_tree = st.seg_tree;
  const gal::veb_shape &sh = st.veb;
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = i; b < nblocks; b += stride) *gal::mword_ptr(&st, (uint32_t)b) = 4097ull;
  for (uint64_t g = i; g < st.num_segments; g += stride) st.act[g] = gal::act_word(0, -1);
  for (uint32_t l = 0; l < sh.layers; l++) {
    uint64_t items = sh.items[l];
    for (uint64_t w = i; w < sh.nwords[l]; w += stride) {
      uint64_t lo = w * 64;
      uint64_t n = items > lo ? items - lo : 0;
      seg_tree[sh.off[l] + w] = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
    }
  }
}

// boot_shared_block_container_one_thread order (gallatin.cuh:196-221)
__global__ void k_boot(const gal::state *s) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  for (uint32_t t = 0; t < s->num_trees; t++)
    for (uint32_t i = 0; i < s->slot_count[t]; i++)
      if (!gal::boot_block(s, t, i, 0)) gal::set_error(s, GAL_DEV_ERR_BOOT);
}

// gal_trim: retire every pinned block (slot order, one thread), crediting the
// slices it never handed out so that a block with nothing live goes back to
// its segment now (and one with live slices when the last is freed), then
// boot the slots again in the one-thread order.
__global__ void k_trim(const gal::state *s) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  for (uint32_t i = 0; i < s->total_slots; i++) {  // spare blocks
    uint32_t blk = atomicExch(s->spares + i, gal::NOBLK);
    if (blk != gal::NOBLK) gal::retire_block(s, blk);
  }
  for (uint32_t t = 0; t < s->num_trees; t++)
    for (uint32_t i = 0; i < s->slot_count[t]; i++) {
      uint32_t blk = atomicExch(s->slots + s->slot_base[t] + i, gal::NOBLK);
      if (blk != gal::NOBLK) gal::retire_block(s, blk);
    }
  // segments of a class none of whose blocks is out (those gathered ahead when
  // a class took the last block of its previous segment) go back too
  for (uint64_t seg = 0; seg < s->num_segments; seg++) {
    uint16_t tree = s->tree_ids[seg];
    if (tree >= s->num_trees) continue;
    const uint32_t nb = gal::blocks_in_segment(s, tree);
    const unsigned long long w = s->act[seg];
    if (gal::act_count(w) != (int32_t)nb - 1) continue;
    gal::release_segment(s, seg, tree, gal::act_gen(w), nb);
  }
  for (uint32_t t = 0; t < s->num_trees; t++)
    for (uint32_t i = 0; i < s->slot_count[t]; i++)
      if (!gal::boot_block(s, t, i, 0)) gal::set_error(s, GAL_DEV_ERR_BOOT);
}

__global__ void k_export_blocks(const gal::state *s, uint32_t *mc, uint64_t nblocks) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = i; b < nblocks; b += stride) mc[b] = gal::export_mword(s, (uint32_t)b);
}

__global__ void k_import_blocks(const gal::state *s, const uint32_t *mc, uint64_t nblocks) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = i; b < nblocks; b += stride)
    *gal::mword_ptr(s, (uint32_t)b) = ((unsigned long long)(mc[b] >> 20) << 32) | (mc[b] & 0xFFFFFu);
}

__global__ void k_stats(const gal::state *s, gal_stats *out) {
  __shared__ unsigned long long acc[3 + 3 * GAL_MAX_TREES];
  const uint32_t T = s->num_trees;
  for (int i = threadIdx.x; i < 3 + 3 * GAL_MAX_TREES; i += blockDim.x) acc[i] = 0;
  __syncthreads();
  const uint32_t bottom = s->veb.layers - 1;
  const uint64_t nw = s->veb.nwords[bottom];
  for (uint64_t w = threadIdx.x; w < nw; w += blockDim.x) {
    atomicAdd(&acc[0], (unsigned long long)__popcll(s->seg_tree[s->veb.off[bottom] + w]));
    for (uint32_t t = 0; t < T; t++)
      atomicAdd(&acc[3 + GAL_MAX_TREES + t],
                (unsigned long long)__popcll(
                    s->sub_trees[(uint64_t)t * s->veb.words + s->veb.off[bottom] + w]));
  }
  for (uint64_t g = threadIdx.x; g < s->num_segments; g += blockDim.x) {
    uint16_t id = s->tree_ids[g];
    if (id < T) {
      atomicAdd(&acc[3 + id], 1ull);
      int handed = (int)gal::blocks_in_segment(s, id) - 1 - gal::act_count(s->act[g]);
      if (handed > 0) atomicAdd(&acc[3 + 2 * GAL_MAX_TREES + id], (unsigned long long)handed);
    } else if (id != 0xFFFF && id > T) {
      atomicAdd(&acc[1], 1ull);
      atomicAdd(&acc[2], (unsigned long long)(id - T - 1));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // longest run of free segments in the bottom layer of the segment tree
    uint64_t best = 0, cur = 0;
    for (uint64_t g = 0; g < s->num_segments; g++) {
      bool f = (s->seg_tree[s->veb.off[bottom] + (g >> 6)] >> (g & 63)) & 1ull;
      cur = f ? cur + 1 : 0;
      if (cur > best) best = cur;
    }
    out->num_segments = s->num_segments;
    out->free_segments = acc[0];
    out->largest_free_run = best;
    out->num_trees = T;
    out->error_word = *s->error;
    for (uint32_t t = 0; t < GAL_MAX_TREES; t++) {
      out->tree_segments[t] = t < T ? acc[3 + t] : 0;
      out->tree_listed[t] = t < T ? acc[3 + GAL_MAX_TREES + t] : 0;
      out->tree_live_blocks[t] = t < T ? acc[3 + 2 * GAL_MAX_TREES + t] : 0;
    }
    out->multi_segment_allocs = acc[1];
    out->multi_segment_segments = acc[2];
  }
}

// one device thread replays a trace (gallatin_single_thread.cu generalised)
__global__ void k_replay(const gal::state *s, const uint64_t *ops, uint64_t nops, uint64_t *out,
                         uint32_t *out_smid) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  out_smid[0] = gal::sm_id();
  for (uint64_t i = 0; i < nops; i++) {
    uint64_t op = ops[i];
    if (op >> 63) {
      uint64_t target = op & ~(1ull << 63);
      if (target < i && out[target] != gal::FAIL) gal::free(s, s->memory + out[target]);
      out[i] = gal::FAIL;
    } else {
      void *p = gal::malloc(s, op);
      out[i] = p ? (uint64_t)((char *)p - s->memory) : gal::FAIL;
    }
  }
}

// warp-wide calls by one warp (gal_replay_warp_trace)
__global__ void k_replay_warp(const gal::state *s, const uint64_t *steps, uint64_t nsteps,
                              uint64_t *out, uint32_t *out_smid) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const uint32_t lane = threadIdx.x;
  if (lane == 0) out_smid[0] = gal::sm_id();
  for (uint64_t i = 0; i < nsteps; i++) {
    const uint64_t *w = steps + i * 33;
    const uint32_t kind = (uint32_t)(w[0] >> 32), mask = (uint32_t)w[0];
    uint64_t res = gal::FAIL;
    __syncwarp();
    if (kind == 0) {
      if ((mask >> lane) & 1u) {  // the step's lanes call together: one team per class
        void *p = gal::malloc_team(s, w[1 + lane], mask);
        res = p ? (uint64_t)((char *)p - s->memory) : gal::FAIL;
      }
    } else {
      for (uint32_t l = 0; l < 32; l++) {
        if (((mask >> l) & 1u) && lane == l) {
          const uint64_t t = w[1 + l];
          if (t < i * 32 && out[t] != gal::FAIL) gal::free(s, s->memory + out[t]);
        }
        __syncwarp();
      }
    }
    out[i * 32 + lane] = res;
    __threadfence();
    __syncwarp();
  }
}

__global__ void k_malloc_per_thread(const gal::state *s, const uint64_t *sizes, uint64_t n,
                                    void **out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = gal::malloc(s, sizes[i]);
}

__global__ void k_free_per_thread(const gal::state *s, void *const *ptrs, uint64_t n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  void *p = ptrs[i];
  if (p) gal::free(s, p);
}

constexpr int BATCH_THREADS = 512;

// Batched malloc: one thread per request, warp teams claiming with one
// atomicAdd per team on their SM's pinned block (gal::malloc), compiled for
// four CTAs of 256 threads per SM (64 registers).  On the mixed 16 B-4 KiB
// churn's requests this served 64 Mi mallocs in 2.2 ms per step, against
// 2.6 ms for the same kernel without a register bound and for a persistent
// grid keeping the pinned blocks in shared memory (gal::malloc_cached).
constexpr int MALLOC_THREADS = 256;

__global__ void __launch_bounds__(MALLOC_THREADS, 4)
    k_malloc_batched(const gal::state *s, const uint64_t *sizes, uint64_t n, void **out) {
  for (uint64_t i = (uint64_t)blockIdx.x * MALLOC_THREADS + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * MALLOC_THREADS)
    out[i] = gal::malloc(s, sizes[i]);
}

// Batched free: each thread takes FREE_PER_THREAD entries per pass of a
// persistent grid and frees them with gal::free_n (table lookups and
// free-counter atomics issued back to back, warp teams per block).  The list
// holds n entries, or *d_count when that is given and smaller (a count that
// an earlier kernel on the stream wrote).
constexpr int FREE_PER_THREAD = 4;

__global__ void __launch_bounds__(BATCH_THREADS)
    k_free_batched(const gal::state *s, void *const *ptrs, uint64_t n,
                   const unsigned long long *d_count, int stage) {
  // the pointers were allocated before this call, and a live pointer's
  // segment keeps its class: a copy of the classes staged now serves them
  extern __shared__ uint16_t classes[];
  const bool staged = stage && gal::stage_classes(s, classes);
  __syncthreads();
  if (d_count && *d_count < n) n = *d_count;
  // a warp takes 32 x FREE_PER_THREAD consecutive entries; lane l holds entries
  // l, l + 32, ... so neighbouring lanes hold neighbouring entries (which share
  // blocks) in each of the FREE_PER_THREAD team formations
  const uint64_t per_warp = 32ull * FREE_PER_THREAD;
  const uint64_t warp = ((uint64_t)blockIdx.x * BATCH_THREADS + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * BATCH_THREADS) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  for (uint64_t w0 = warp * per_warp; w0 < n; w0 += nwarps * per_warp) {
    void *p[FREE_PER_THREAD];
    bool go[FREE_PER_THREAD];
#pragma unroll
    for (int k = 0; k < FREE_PER_THREAD; k++) {
      const uint64_t i = w0 + (uint64_t)k * 32u + lane;
      p[k] = i < n ? ptrs[i] : nullptr;
      go[k] = p[k] != nullptr;
    }
    gal::free_n<FREE_PER_THREAD>(s, p, go, staged ? classes : nullptr);
  }
}

template <class K>
int persistent_grid(int device, K kernel, int threads, size_t dyn_smem = 0) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn_smem);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

void free_handle(gal_handle *h) {
  if (!h) return;
  if (h->meta) cudaFree(h->meta);
  if (h->arena) {
    if (h->cfg.arena_kind == GAL_ARENA_HOST) cudaFreeHost(h->arena);
    else cudaFree(h->arena);  // device and managed arenas
  }
  delete h;
}

// the arena: device memory, pinned host memory mapped for the device (with
// unified addressing its device address is the host address), or managed
cudaError_t alloc_arena(gal_handle *h) {
  switch (h->cfg.arena_kind) {
    case GAL_ARENA_HOST: {
      cudaError_t e = cudaHostAlloc((void **)&h->arena, h->arena_bytes, cudaHostAllocMapped);
      if (e != cudaSuccess) return e;
      void *dp = nullptr;
      e = cudaHostGetDevicePointer(&dp, h->arena, 0);
      if (e == cudaSuccess && dp != (void *)h->arena) e = cudaErrorInvalidValue;
      return e;
    }
    case GAL_ARENA_MANAGED:
      return cudaMallocManaged((void **)&h->arena, h->arena_bytes, cudaMemAttachGlobal);
    default:
      return cudaMalloc((void **)&h->arena, h->arena_bytes);
  }
}

int build(uint64_t num_bytes, uint64_t seed, const gal_config *cfg_in, bool boot, gal_handle **out) {
  if (!out) return GAL_ERR_ARGS;
  *out = nullptr;
  gal_config cfg;
  if (cfg_in)
    cfg = *cfg_in;
  else
    gal_config_default(&cfg);
  if (!is_pow2(cfg.bytes_per_segment) || !is_pow2(cfg.min_size) || !is_pow2(cfg.max_size))
    return GAL_ERR_ARGS;
  if (cfg.max_size < cfg.min_size || cfg.bytes_per_segment < cfg.max_size * 4096) return GAL_ERR_ARGS;
  if (cfg.subtree_policy > GAL_POLICY_LOWEST) return GAL_ERR_ARGS;
  if (cfg.team_width > 32 || (cfg.team_width & (cfg.team_width - 1))) return GAL_ERR_ARGS;
  if (cfg.arena_kind > GAL_ARENA_MANAGED) return GAL_ERR_ARGS;
  if (cfg.spare_blocks > 1 || cfg.zero_fill > 1 || cfg.block_layout > 1) return GAL_ERR_ARGS;
  if (cfg.l2_fetch_bytes != 0 && cfg.l2_fetch_bytes != 32 && cfg.l2_fetch_bytes != 64 &&
      cfg.l2_fetch_bytes != 128)
    return GAL_ERR_ARGS;
  if (cfg.gather_ahead > 1) return GAL_ERR_ARGS;
  const uint32_t T = log2u(cfg.max_size) - log2u(cfg.min_size) + 1;
  const uint64_t S = num_bytes / cfg.bytes_per_segment;
  if (T > GAL_MAX_TREES || S == 0 || S + T + 1 >= 0xFFFF) return GAL_ERR_ARGS;
  const uint32_t bps_shift = log2u(cfg.bytes_per_segment) - log2u(cfg.min_size) - 12;
  const uint64_t nblocks = S << bps_shift;
  if (nblocks >= 0xFFFFFFFFull) return GAL_ERR_ARGS;
  if (cfg.l2_fetch_bytes) {  // a hint for the current device's whole context
    cudaError_t e = cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, cfg.l2_fetch_bytes);
    if (e != cudaSuccess) {
      fprintf(stderr, "gallatin_gb300: setting the L2 fetch granularity failed: %s\n", cudaGetErrorString(e));
      return GAL_ERR_CUDA;
    }
  }

  gal_handle *h = new gal_handle();
  h->cfg = cfg;
  h->num_bytes = num_bytes;
  h->seed = seed;
  cudaGetDevice(&h->device);
  gal::state &st = h->st;
  st.num_segments = S;
  st.seed = seed;
  st.seg_shift = log2u(cfg.bytes_per_segment);
  st.min_shift = log2u(cfg.min_size);
  st.bps_shift = bps_shift;
  st.num_trees = T;
  st.policy = cfg.subtree_policy;
  st.smid_override = cfg.smid_override;
  st.spin_limit = cfg.spin_limit ? cfg.spin_limit : (1u << 16);
  st.gather_unlocked_below = cfg.gather_unlocked_below;
  st.gather_ahead = cfg.gather_ahead;
  st.team_width = cfg.team_width ? cfg.team_width : 32;
  st.use_spares = cfg.spare_blocks ? 1u : 0u;
  st.zero_fill = cfg.zero_fill;
  // pinned slots: first, halving per tree, floored (shared_block_storage.cuh:260-267);
  // pinned_slots_first == 0 asks for one slot per SM in every size class
  if (cfg.pinned_slots_first == 0) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    cfg.pinned_slots_first = cfg.pinned_slots_min = (uint32_t)(sms > 0 ? sms : 1);
    h->cfg = cfg;
  }
  uint64_t n = cfg.pinned_slots_first, total = 0;
  for (uint32_t t = 0; t < T; t++) {
    uint64_t c = n == 0 ? 1 : n;
    st.slot_base[t] = (uint32_t)total;
    st.slot_count[t] = (uint32_t)c;
    total += c;
    n = n / 2;
    if (n < cfg.pinned_slots_min) n = cfg.pinned_slots_min;
  }
  st.total_slots = (uint32_t)total;
  // vEB shape over S items (veb.cuh:595-649)
  int max_height = 64 - __builtin_clzll(S);
  st.veb.layers = (uint32_t)((max_height - 1) / 6 + 1);
  {
    uint64_t u = S;
    for (uint32_t i = 0; i < st.veb.layers; i++) {
      uint32_t l = st.veb.layers - 1 - i;
      st.veb.items[l] = u;
      st.veb.nwords[l] = (uint32_t)((u - 1) / 64 + 1);
      u = (u - 1) / 64 + 1;
    }
    uint32_t o = 0;
    for (uint32_t l = 0; l < st.veb.layers; l++) {
      st.veb.off[l] = o;
      o += st.veb.nwords[l];
    }
    st.veb.words = o;
  }
  // one metadata region
  const size_t A = 256;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, A);
    return o;
  };
  size_t o_state = carve(sizeof(gal::state));
  size_t o_seg = carve((size_t)st.veb.words * 8);
  size_t o_sub = carve((size_t)T * st.veb.words * 8);
  size_t o_ids = carve(S * 2);
  size_t o_act = carve(S * 8), o_qc = carve(S * 4), o_qfc = carve(S * 4), o_fqfc = carve(S * 4);
  // block counters: one 32-byte record per block, or two dense arrays
  const bool records = cfg.block_layout == GAL_BLOCK_LAYOUT_RECORD;
  size_t o_mw = carve(nblocks * (records ? gal::BLOCK_RECORD_BYTES : 8));
  size_t o_fc = records ? o_mw + 8 : carve(nblocks * 4);
  size_t o_q = carve(nblocks * 4);
  size_t o_slots = carve(total * 4);
  size_t o_spares = carve(total * 4);
  size_t o_locks = carve((size_t)(T + 1) * gal::LOCK_STRIDE * 4), o_err = carve(128);
  h->meta_bytes = off;
  if (cudaMalloc(&h->meta, h->meta_bytes) != cudaSuccess) {
    free_handle(h);
    return GAL_ERR_OOM;
  }
  h->arena_bytes = S * cfg.bytes_per_segment;
  if (alloc_arena(h) != cudaSuccess) {
    cudaGetLastError();
    free_handle(h);
    return GAL_ERR_OOM;
  }
  char *m = h->meta;
  st.memory = h->arena;
  st.seg_tree = (uint64_t *)(m + o_seg);
  st.sub_trees = (uint64_t *)(m + o_sub);
  st.tree_ids = (uint16_t *)(m + o_ids);
  st.act = (unsigned long long *)(m + o_act);
  st.qc = (uint32_t *)(m + o_qc);
  st.qfc = (uint32_t *)(m + o_qfc);
  st.fqfc = (uint32_t *)(m + o_fqfc);
  st.mwords = (unsigned long long *)(m + o_mw);
  st.fctr = (uint32_t *)(m + o_fc);
  st.mstride = records ? gal::BLOCK_RECORD_BYTES / 8 : 1;
  st.fstride = records ? gal::BLOCK_RECORD_BYTES / 4 : 1;
  st.queues = (uint32_t *)(m + o_q);
  st.slots = (uint32_t *)(m + o_slots);
  st.spares = (uint32_t *)(m + o_spares);
  st.locks = (uint32_t *)(m + o_locks);
  st.error = (uint32_t *)(m + o_err);
  h->d_state = (gal::state *)(m + o_state);

  int rc = GAL_OK;
  do {
    // everything zero, then the non-zero patterns
    if (cudaMemset(h->meta, 0, h->meta_bytes) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cudaMemset(st.tree_ids, 0xFF, S * 2) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cudaMemset(st.queues, 0xFF, nblocks * 4) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cudaMemset(st.slots, 0xFF, total * 4) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cudaMemset(st.spares, 0xFF, total * 4) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    k_init_words<<<1024, 256>>>(st, nblocks);
    if (cudaGetLastError() != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cfg.zero_arena && cudaMemset(h->arena, 0, h->arena_bytes) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (cudaMemcpy(h->d_state, &st, sizeof(st), cudaMemcpyHostToDevice) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (boot) {
      k_boot<<<1, 1>>>(h->d_state);
      if (cudaGetLastError() != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    // the allocation-free export's fixed array and stream, placed now so that
    // the export itself never loads or allocates anything
    if (gal_noalloc_setup(h->device) != GAL_OK) { rc = GAL_ERR_CUDA; break; }
    uint32_t err = 0;
    if (cudaMemcpy(&err, st.error, 4, cudaMemcpyDeviceToHost) != cudaSuccess) { rc = GAL_ERR_CUDA; break; }
    if (err) { rc = GAL_ERR_DEVICE; break; }
  } while (0);
  if (rc != GAL_OK) {
    free_handle(h);
    return rc;
  }
  // dims of the state view
  h->dims.num_segments = S;
  h->dims.num_trees = T;
  h->dims.blocks_per_segment = 1u << bps_shift;
  h->dims.veb_layers = st.veb.layers;
  h->dims.veb_words = st.veb.words;
  h->dims.total_slots = (uint32_t)total;
  for (uint32_t t = 0; t < T; t++) h->dims.slot_counts[t] = st.slot_count[t];
  {
    std::lock_guard<std::mutex> g(g_mu);
    g_by_state[h->d_state] = h;
  }
  *out = h;
  return GAL_OK;
}

// makes h the process-wide instance unless another thread installed one while
// h was being built (the check before building is only a fast path)
int install_global(gal_handle **slot, gal_handle *h) {
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (!*slot) {
      *slot = h;
      return GAL_OK;
    }
    g_by_state.erase(h->d_state);
  }
  free_handle(h);
  return GAL_ERR_STATE;
}

int push_state(gal_handle *h) {
  CUDA_TRY(cudaMemcpy(h->d_state, &h->st, sizeof(h->st), cudaMemcpyHostToDevice));
  return GAL_OK;
}

unsigned grid_for(uint64_t n, unsigned block) {
  uint64_t g = (n + block - 1) / block;
  if (g == 0) g = 1;
  if (g > 0x7FFFFFFFull) g = 0x7FFFFFFFull;
  return (unsigned)g;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

int gal_config_default(gal_config *cfg) {
  if (!cfg) return GAL_ERR_ARGS;
  cfg->bytes_per_segment = 16ull << 20;
  cfg->min_size = 16;
  cfg->max_size = 4096;
  cfg->smid_override = -1;
  cfg->subtree_policy = GAL_POLICY_REFERENCE;
  cfg->pinned_slots_first = 128;
  cfg->pinned_slots_min = 4;
  cfg->zero_arena = 1;
  cfg->spin_limit = 1u << 16;  // x backoff capped at 4 us: ~0.27 s per wait at most
  cfg->gather_unlocked_below = 16;  // serially the lock is always free: same offsets
  cfg->team_width = 32;
  cfg->arena_kind = GAL_ARENA_DEVICE;
  cfg->spare_blocks = 0;
  cfg->zero_fill = 0;
  cfg->block_layout = GAL_BLOCK_LAYOUT_RECORD;
  cfg->l2_fetch_bytes = 0;
  cfg->gather_ahead = 1;
  return GAL_OK;
}

int gal_create(uint64_t num_bytes, uint64_t seed, const gal_config *cfg, gal_handle **out) {
  return build(num_bytes, seed, cfg, true, out);
}

int gal_create_unbooted(uint64_t num_bytes, uint64_t seed, const gal_config *cfg, gal_handle **out) {
  return build(num_bytes, seed, cfg, false, out);
}

int gal_destroy(gal_handle *h) {
  if (!h) return GAL_ERR_ARGS;
  cudaDeviceSynchronize();
  {
    std::lock_guard<std::mutex> g(g_mu);
    g_by_state.erase(h->d_state);
    if (g_global == h) g_global = nullptr;
    if (g_global_host == h) g_global_host = nullptr;
  }
  free_handle(h);
  return GAL_OK;
}

gal_handle *gal_handle_of(const void *device_state) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_by_state.find(device_state);
  return it == g_by_state.end() ? nullptr : it->second;
}

void *gal_device_state(gal_handle *h) { return h ? (void *)h->d_state : nullptr; }
void *gal_arena_base(gal_handle *h) { return h ? (void *)h->arena : nullptr; }
uint64_t gal_arena_bytes(gal_handle *h) { return h ? h->arena_bytes : 0; }

int gal_get_stats(gal_handle *h, gal_stats *out) {
  if (!h || !out) return GAL_ERR_ARGS;
  gal_stats *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, sizeof(gal_stats)));
  k_stats<<<1, 1024>>>(h->d_state, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof(gal_stats), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return GAL_ERR_CUDA;
  out->metadata_bytes = h->meta_bytes;
  return GAL_OK;
}

int gal_print_stats(gal_handle *h) {
  gal_stats s;
  int rc = gal_get_stats(h, &s);
  if (rc) return rc;
  printf("\nGallatin (GB300) usage stats:\n");
  printf("Segment tree sees %llu/%llu segments available, largest free run %llu\n",
         (unsigned long long)s.free_segments, (unsigned long long)s.num_segments,
         (unsigned long long)s.largest_free_run);
  for (uint32_t t = 0; t < s.num_trees; t++)
    printf("Tree %u: size %llu, owns %llu segments, lists %llu, %llu blocks handed out\n", t,
           (unsigned long long)(h->cfg.min_size << t), (unsigned long long)s.tree_segments[t],
           (unsigned long long)s.tree_listed[t], (unsigned long long)s.tree_live_blocks[t]);
  printf("Multi-segment allocations: %llu covering %llu segments\n",
         (unsigned long long)s.multi_segment_allocs, (unsigned long long)s.multi_segment_segments);
  printf("Allocator is using %llu bytes of metadata, error word 0x%x\n",
         (unsigned long long)s.metadata_bytes, s.error_word);
  return GAL_OK;
}

int gal_last_error(gal_handle *h, uint32_t *bits) {
  if (!h || !bits) return GAL_ERR_ARGS;
  CUDA_TRY(cudaMemcpy(bits, h->st.error, 4, cudaMemcpyDeviceToHost));
  return GAL_OK;
}

int gal_clear_error(gal_handle *h) {
  if (!h) return GAL_ERR_ARGS;
  CUDA_TRY(cudaMemset(h->st.error, 0, 8 + 4 * sizeof(uint64_t)));
  return GAL_OK;
}

int gal_error_info(gal_handle *h, uint64_t *out4) {
  if (!h || !out4) return GAL_ERR_ARGS;
  CUDA_TRY(cudaMemcpy(out4, h->st.error + 2, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return GAL_OK;
}

int gal_state_dims_get(gal_handle *h, gal_state_dims *out) {
  if (!h || !out) return GAL_ERR_ARGS;
  *out = h->dims;
  return GAL_OK;
}

int gal_export_state(gal_handle *h, gal_state_view *v) {
  if (!h || !v) return GAL_ERR_ARGS;
  const gal::state &st = h->st;
  const uint64_t S = st.num_segments, nb = S << st.bps_shift, W = st.veb.words, T = st.num_trees;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  CUDA_TRY(cudaDeviceSynchronize());
  const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
  CUDA_TRY(cudaMemcpy(v->seg_tree_words, st.seg_tree, W * 8, D2H));
  CUDA_TRY(cudaMemcpy(v->sub_tree_words, st.sub_trees, T * W * 8, D2H));
  CUDA_TRY(cudaMemcpy(v->tree_ids, st.tree_ids, S * 2, D2H));
  CUDA_TRY(cudaMemcpy2D(v->active_counts, 4, st.act, 8, 4, S, D2H));  // low halves: biased counts
  CUDA_TRY(cudaMemcpy(v->queue_counters, st.qc, S * 4, D2H));
  CUDA_TRY(cudaMemcpy(v->queue_free_counters, st.qfc, S * 4, D2H));
  CUDA_TRY(cudaMemcpy(v->final_queue_free_counters, st.fqfc, S * 4, D2H));
  CUDA_TRY(cudaMemcpy2D(v->free_counters, 4, st.fctr, (size_t)st.fstride * 4, 4, nb, D2H));
  CUDA_TRY(cudaMemcpy(v->queues, st.queues, nb * 4, D2H));
  CUDA_TRY(cudaMemcpy(v->slots, st.slots, (uint64_t)st.total_slots * 4, D2H));
  uint32_t *d_mc = nullptr;
  CUDA_TRY(cudaMalloc(&d_mc, nb * 4));
  k_export_blocks<<<1024, 256>>>(h->d_state, d_mc, nb);
  cudaError_t e = cudaMemcpy(v->malloc_counters, d_mc, nb * 4, D2H);
  cudaFree(d_mc);
  if (e != cudaSuccess) return GAL_ERR_CUDA;
  uint32_t locks[GAL_MAX_TREES + 1] = {}, err = 0;
  CUDA_TRY(cudaMemcpy2D(locks, 4, st.locks, gal::LOCK_STRIDE * 4, 4, T + 1, D2H));
  CUDA_TRY(cudaMemcpy(&err, st.error, 4, D2H));
  for (uint64_t i = 0; i < S; i++) v->active_counts[i] = gal::act_unbias((uint32_t)v->active_counts[i]);
  uint32_t bits = 0;
  for (uint32_t t = 0; t <= T; t++) bits |= locks[t] ? 1u << t : 0u;
  v->locks = bits;
  v->error_word = err;
  return GAL_OK;
}

int gal_import_state(gal_handle *h, const gal_state_view *v) {
  if (!h || !v) return GAL_ERR_ARGS;
  const gal::state &st = h->st;
  const uint64_t S = st.num_segments, nb = S << st.bps_shift, W = st.veb.words, T = st.num_trees;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  CUDA_TRY(cudaDeviceSynchronize());
  const cudaMemcpyKind H2D = cudaMemcpyHostToDevice;
  CUDA_TRY(cudaMemcpy(st.seg_tree, v->seg_tree_words, W * 8, H2D));
  CUDA_TRY(cudaMemcpy(st.sub_trees, v->sub_tree_words, T * W * 8, H2D));
  CUDA_TRY(cudaMemcpy(st.tree_ids, v->tree_ids, S * 2, H2D));
  {
    std::vector<unsigned long long> act(S);  // generation 0, the view's counts
    for (uint64_t i = 0; i < S; i++) act[i] = gal::act_word(0, v->active_counts[i]);
    CUDA_TRY(cudaMemcpy(st.act, act.data(), S * 8, H2D));
  }
  CUDA_TRY(cudaMemcpy(st.qc, v->queue_counters, S * 4, H2D));
  CUDA_TRY(cudaMemcpy(st.qfc, v->queue_free_counters, S * 4, H2D));
  CUDA_TRY(cudaMemcpy(st.fqfc, v->final_queue_free_counters, S * 4, H2D));
  CUDA_TRY(cudaMemcpy2D(st.fctr, (size_t)st.fstride * 4, v->free_counters, 4, 4, nb, H2D));
  CUDA_TRY(cudaMemcpy(st.queues, v->queues, nb * 4, H2D));
  CUDA_TRY(cudaMemcpy(st.slots, v->slots, (uint64_t)st.total_slots * 4, H2D));
  CUDA_TRY(cudaMemset(st.spares, 0xFF, (uint64_t)st.total_slots * 4));  // the view holds none
  uint32_t *d_mc = nullptr;
  CUDA_TRY(cudaMalloc(&d_mc, nb * 4));
  cudaError_t e = cudaMemcpy(d_mc, v->malloc_counters, nb * 4, H2D);
  if (e == cudaSuccess) {
    k_import_blocks<<<1024, 256>>>(h->d_state, d_mc, nb);
    e = cudaDeviceSynchronize();
  }
  cudaFree(d_mc);
  if (e != cudaSuccess) return GAL_ERR_CUDA;
  uint32_t locks[GAL_MAX_TREES + 1];
  for (uint32_t t = 0; t <= T; t++) locks[t] = (v->locks >> t) & 1u;
  CUDA_TRY(cudaMemcpy2D(st.locks, gal::LOCK_STRIDE * 4, locks, 4, 4, T + 1, H2D));
  return GAL_OK;
}

int gal_set_smid_override(gal_handle *h, int32_t smid) {
  if (!h) return GAL_ERR_ARGS;
  h->st.smid_override = smid;
  h->cfg.smid_override = smid;
  return push_state(h);
}

int gal_set_policy(gal_handle *h, uint32_t policy) {
  if (!h || policy > GAL_POLICY_LOWEST) return GAL_ERR_ARGS;
  h->st.policy = policy;
  h->cfg.subtree_policy = policy;
  return push_state(h);
}

int gal_init(uint64_t num_bytes, uint64_t seed, const gal_config *cfg) {
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (g_global) return GAL_ERR_STATE;
  }
  gal_handle *h = nullptr;
  int rc = gal_create(num_bytes, seed, cfg, &h);
  if (rc) return rc;
  return install_global(&g_global, h);
}

int gal_teardown(void) {
  gal_handle *h;
  {
    std::lock_guard<std::mutex> g(g_mu);
    h = g_global;
  }
  if (!h) return GAL_ERR_STATE;
  return gal_destroy(h);
}

gal_handle *gal_global(void) {
  std::lock_guard<std::mutex> g(g_mu);
  return g_global;
}

int gal_init_host(uint64_t num_bytes, uint64_t seed, const gal_config *cfg) {
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (g_global_host) return GAL_ERR_STATE;
  }
  gal_config c;
  if (cfg) c = *cfg;
  else gal_config_default(&c);
  c.arena_kind = GAL_ARENA_HOST;
  gal_handle *h = nullptr;
  int rc = gal_create(num_bytes, seed, &c, &h);
  if (rc) return rc;
  return install_global(&g_global_host, h);
}

int gal_teardown_host(void) {
  gal_handle *h;
  {
    std::lock_guard<std::mutex> g(g_mu);
    h = g_global_host;
  }
  if (!h) return GAL_ERR_STATE;
  return gal_destroy(h);
}

gal_handle *gal_global_host(void) {
  std::lock_guard<std::mutex> g(g_mu);
  return g_global_host;
}

int gal_replay_trace(gal_handle *h, const uint64_t *ops, uint64_t nops, uint64_t *out_offsets,
                     uint32_t *out_smid, void *stream) {
  if (!h || !ops || !out_offsets || !out_smid) return GAL_ERR_ARGS;
  k_replay<<<1, 1, 0, (cudaStream_t)stream>>>(h->d_state, ops, nops, out_offsets, out_smid);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_replay_warp_trace(gal_handle *h, const uint64_t *steps, uint64_t nsteps,
                          uint64_t *out_offsets, uint32_t *out_smid, void *stream) {
  if (!h || (nsteps && (!steps || !out_offsets)) || !out_smid) return GAL_ERR_ARGS;
  k_replay_warp<<<1, 32, 0, (cudaStream_t)stream>>>(h->d_state, steps, nsteps, out_offsets, out_smid);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_malloc_per_thread(gal_handle *h, const uint64_t *sizes, uint64_t n, void **out, void *stream) {
  if (!h || (n && (!sizes || !out))) return GAL_ERR_ARGS;
  if (!n) return GAL_OK;
  gal_device_guard on_dev(h->device);  // the handle's device, whatever the caller's current one
  CUDA_TRY(on_dev.err);
  k_malloc_per_thread<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(h->d_state, sizes, n, out);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_free_per_thread(gal_handle *h, void *const *ptrs, uint64_t n, void *stream) {
  if (!h || (n && !ptrs)) return GAL_ERR_ARGS;
  if (!n) return GAL_OK;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  k_free_per_thread<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(h->d_state, ptrs, n);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_trim(gal_handle *h, void *stream) {
  if (!h) return GAL_ERR_ARGS;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  k_trim<<<1, 1, 0, (cudaStream_t)stream>>>(h->d_state);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_malloc_batched(gal_handle *h, const uint64_t *sizes, uint64_t n, void **out, void *stream) {
  if (!h || (n && (!sizes || !out))) return GAL_ERR_ARGS;
  if (!n) return GAL_OK;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  k_malloc_batched<<<grid_for(n, MALLOC_THREADS), MALLOC_THREADS, 0, (cudaStream_t)stream>>>(h->d_state, sizes,
                                                                                          n, out);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

int gal_free_batched(gal_handle *h, void *const *ptrs, uint64_t n, void *stream) {
  return gal_free_batched_n(h, ptrs, nullptr, n, stream);
}

int gal_free_batched_n(gal_handle *h, void *const *ptrs, const unsigned long long *d_count,
                       uint64_t max_n, void *stream) {
  if (!h || (max_n && !ptrs)) return GAL_ERR_ARGS;
  if (!max_n) return GAL_OK;
  gal_device_guard on_dev(h->device);
  CUDA_TRY(on_dev.err);
  unsigned g = grid_for((max_n + FREE_PER_THREAD - 1) / FREE_PER_THREAD, BATCH_THREADS);
  const size_t stage = h->st.num_segments * 2 <= gal::CLASS_STAGE_BYTES ? h->st.num_segments * 2 : 0;
  if (!h->grid_free) h->grid_free = persistent_grid(h->device, k_free_batched, BATCH_THREADS, stage);
  unsigned p = (unsigned)h->grid_free;
  k_free_batched<<<g < p ? g : p, BATCH_THREADS, stage, (cudaStream_t)stream>>>(h->d_state, ptrs, max_n,
                                                                                d_count, stage > 0);
  CUDA_TRY(cudaGetLastError());
  return GAL_OK;
}

}  // extern "C"

int gal_internal_device(const gal_handle *h) { return h->device; }
const gal::state *gal_internal_host_state(const gal_handle *h) { return &h->st; }
