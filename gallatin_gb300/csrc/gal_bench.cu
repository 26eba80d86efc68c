// gal_bench.cu — workload kernels used by bench.py and the GPU tests:
//   * mixed-size churn (16 B–4 KiB, 50% random frees per round, uint32
//     payload written and checked), plain per-thread or CTA-batched, stream
//     launches or one captured CUDA graph per step;
//   * the same churn end to end through the public entry points
//     (gal_malloc_batched / gal_free_batched) with request sizes copied from
//     pinned host memory every round;
//   * n threads x malloc(size) with a thread-id stamp (the reference's
//     tests/src/global_test.cu workload);
//   * an L2 atomic throughput probe giving the roofline denominator.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"
#include "churn.cuh"
#include "gal_batch.cuh"

extern "C" {
typedef struct gal_churn_result {
  double ms_total;           /* sum over timed steps (CUDA events)               */
  double ms_malloc_kernels;  /* malloc-phase kernels, summed over timed steps    */
  double ms_free_kernels;    /* free-phase kernels (incl. drain)                 */
  uint64_t mallocs_ok, mallocs_failed, payload_mismatch, frees;
  uint64_t malloc_launches, free_launches, other_launches;
  uint64_t h2d_bytes, d2h_bytes; /* per timed step (e2e only)                   */
  uint32_t error_word;
} gal_churn_result;
}

namespace {

struct plain_alloc {
  const gal::state *s;
  const uint16_t *classes;  // staged segment classes (gal::stage_classes) or nullptr
  __device__ void *malloc(uint64_t n) { return gal::malloc(s, n); }
  __device__ void free(void *p) { gal::free(s, p); }
};

}  // namespace

// this library frees a thread's pointers with overlapped lookups and atomics
template <>
struct galwl::free_many<plain_alloc> {
  static __device__ __forceinline__ void run(plain_alloc *a, void *const (&p)[galwl::FREE_SLOTS],
                                             const bool (&go)[galwl::FREE_SLOTS]) {
    gal::free_n<galwl::FREE_SLOTS>(a->s, p, go, a->classes);
  }
};

namespace {

constexpr int BT = 512;  // batched CTA size

// one thread per request; MINB: CTAs of 256 threads per SM its registers must
// allow (1: no bound, 94 registers; 3: 85; 4: 64)
constexpr int PLAIN_BT = 256;
template <bool PAYLOAD, int MINB>
__global__ void __launch_bounds__(PLAIN_BT, MINB)
    k_churn_malloc_plain(const gal::state *s, void **ptrs, uint32_t *live, uint64_t base,
                         uint64_t n, uint32_t seed, unsigned long long *stats) {
  plain_alloc a{s, nullptr};
  galwl::churn_malloc_body<plain_alloc, PAYLOAD>(&a, ptrs, live, base, n, seed, stats);
}

constexpr int FREE_BT = 256;  // free phase CTA size (persistent grid)

// The free phase; with dynamic shared memory of 2 bytes per segment the
// segments' classes are staged first (every pointer freed here was allocated
// by an earlier kernel, and a live pointer's segment keeps its class).
// MINB: CTAs per SM the registers must allow (1: no bound, 80 registers; 4: 64).
template <bool PAYLOAD, int MINB>
__global__ void __launch_bounds__(FREE_BT, MINB)
    k_churn_free_plain(const gal::state *s, void **ptrs, uint32_t *live, uint64_t nslots,
                       uint32_t round, uint32_t seed, int all, int stage, unsigned long long *stats) {
  __shared__ uint16_t lists[FREE_BT / 32][galwl::WARP_SLOTS];
  extern __shared__ uint16_t classes[];
  const bool staged = stage && gal::stage_classes(s, classes);
  __syncthreads();
  plain_alloc a{s, staged ? classes : nullptr};
  galwl::churn_free_warps<plain_alloc, PAYLOAD>(&a, ptrs, live, nslots, round, seed, all != 0, stats,
                                                lists[threadIdx.x >> 5]);
}

// persistent malloc phase of one round with the pinned blocks cached per CTA
// (gal::malloc_cached): each thread serves slots c + threadIdx.x of the CTA's
// chunks, so a warp's lanes keep 32 consecutive slots for the liveness words.
// MINB: CTAs per SM the registers must allow (64 registers at 4).
constexpr int CACHED_BT = 256;
template <bool PAYLOAD, int MINB>
__global__ void __launch_bounds__(CACHED_BT, MINB)
    k_churn_malloc_cached(const gal::state *s, void **ptrs, uint32_t *live, uint64_t base, uint64_t n,
                          uint32_t seed, unsigned long long *stats) {
  __shared__ gal::slot_cache cache;
  gal::slot_cache_init(cache);
  __syncthreads();
  for (uint64_t c = (uint64_t)blockIdx.x * CACHED_BT; c < n; c += (uint64_t)gridDim.x * CACHED_BT) {
    const uint64_t t = c + threadIdx.x;
    if (t >= n) break;  // whole warps: n is a multiple of SLOT_ALIGN
    const uint64_t slot = base + t;
    void *p = gal::malloc_cached(s, galwl::mixed_size(slot, seed), cache);
    if (PAYLOAD && p) *(volatile uint32_t *)p = galwl::payload(slot, seed);
    ptrs[slot] = p;
    galwl::publish_live(live, slot, p != nullptr);
    galwl::warp_count(stats, 0, p != nullptr);
    galwl::warp_count(stats, 1, p == nullptr);
  }
}

// persistent, CTA-aggregated malloc phase of one round: BW worker threads and
// one service warp (spare blocks) per CTA; each iteration of the workers serves
// K x BW requests (request k of worker t is slot c + k*BW + t, so a warp's lanes
// keep 32 consecutive slots for the liveness words)
constexpr int BW = BT - 32;
template <int K>
__global__ void __launch_bounds__(BT)
    k_churn_malloc_batched(const gal::state *s, void **ptrs, uint32_t *live, uint64_t base,
                           uint64_t n, uint32_t seed, unsigned long long *stats) {
  __shared__ gal::cta_claim_smem sm;
  gal::cta_claim_init(sm, BW);
  __syncthreads();
  if (threadIdx.x >= BW) {
    gal::cta_service(s, sm);
    return;
  }
  for (uint64_t c = (uint64_t)blockIdx.x * BW * K; c < n; c += (uint64_t)gridDim.x * BW * K) {
    uint64_t size[K];
    bool has[K];
    void *p[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint64_t t = c + (uint64_t)k * BW + threadIdx.x;
      has[k] = t < n;  // whole warps: n is a multiple of SLOT_ALIGN
      size[k] = has[k] ? galwl::mixed_size(base + t, seed) : 0;
    }
    gal::cta_malloc_n<K>(s, size, has, sm, p);
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (!has[k]) continue;
      const uint64_t slot = base + c + (uint64_t)k * BW + threadIdx.x;
      if (p[k]) *(volatile uint32_t *)p[k] = galwl::payload(slot, seed);
      ptrs[slot] = p[k];
      galwl::publish_live(live, slot, p[k] != nullptr);
      galwl::warp_count(stats, 0, p[k] != nullptr);
      galwl::warp_count(stats, 1, p[k] == nullptr);
    }
  }
  gal::cta_workers_done(sm);
}

// persistent, CTA-aggregated free phase (coin flips, or everything when all)
__global__ void __launch_bounds__(BT)
    k_churn_free_batched(const gal::state *s, void **ptrs, uint32_t *live, uint64_t nslots,
                         uint32_t round, uint32_t seed, int all, unsigned long long *stats) {
  constexpr int F = galwl::FREE_SLOTS;
  __shared__ gal::cta_free_smem<2 * BT * F> sm;
  for (uint64_t c = (uint64_t)blockIdx.x * BT * F; c < nslots; c += (uint64_t)gridDim.x * BT * F) {
    uint64_t i0 = c + (uint64_t)threadIdx.x * F;
    const bool valid = i0 < nslots;  // whole warps: nslots is a multiple of SLOT_ALIGN
    const uint32_t word = valid ? live[i0 >> 5] : 0u;
    const uint32_t sel = galwl::select_frees(word, i0, round, seed, all != 0);
    void *p[F];
    if (sel) {
      galwl::load_slots(ptrs, i0, nslots, p);
    } else {
#pragma unroll
      for (int k = 0; k < F; k++) p[k] = nullptr;
    }
    uint32_t nbad = 0, ngo = 0;
#pragma unroll
    for (int k = 0; k < F; k++) {
      if (((sel >> k) & 1u) && p[k] != nullptr) {
        nbad += *(const uint32_t *)p[k] != galwl::payload(i0 + k, seed);
        ngo++;
      } else {
        p[k] = nullptr;
      }
    }
    gal::cta_free<2 * BT * F, F>(s, p, sm);
    if (valid) galwl::clear_live(live, i0, word, sel);
    galwl::warp_add(stats, 2, nbad);
    galwl::warp_add(stats, 3, ngo);
  }
}

// end-to-end helpers: user-side kernels around the public batched entry points
__global__ void k_stamp_payload(void **ptrs, uint32_t *live, uint64_t base, uint64_t n, uint32_t seed,
                                unsigned long long *stats) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;  // whole warps: n is a multiple of SLOT_ALIGN
  void *p = ptrs[base + t];
  if (p) *(volatile uint32_t *)p = galwl::payload(base + t, seed);
  galwl::publish_live(live, base + t, p != nullptr);
  galwl::warp_count(stats, 0, p != nullptr);
  galwl::warp_count(stats, 1, p == nullptr);
}

// Appends the pointers this round frees to freelist (*count entries so far)
// and checks their payloads; persistent grid, one warp per 1,024 slots.
__global__ void __launch_bounds__(FREE_BT)
    k_select_free_list(void **ptrs, uint32_t *live, void **freelist, unsigned long long *count,
                       uint64_t lo, uint64_t nslots, uint32_t round, uint32_t seed, int all,
                       unsigned long long *stats) {
  __shared__ uint16_t lists[FREE_BT / 32][galwl::WARP_SLOTS];
  galwl::churn_select_warps(ptrs, live, lo, nslots, round, seed, all != 0, stats, lists[threadIdx.x >> 5],
                            freelist, count);
}

// n threads x malloc(size) + thread-id stamp, then check + free (global_test.cu)
__global__ void k_stamp_malloc(const gal::state *s, uint64_t n, uint64_t size, uint64_t **ptrs,
                               unsigned long long *stats) {
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)gal::malloc(s, size);
  if (p) p[0] = tid;
  ptrs[tid] = p;
  galwl::warp_count(stats, 0, p != nullptr);
  galwl::warp_count(stats, 1, p == nullptr);
}

__global__ void k_stamp_free(const gal::state *s, uint64_t n, uint64_t **ptrs,
                             unsigned long long *stats) {
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  uint64_t *p = ptrs[tid];
  bool bad = false;
  if (p) {
    bad = p[0] != tid;
    gal::free(s, p);
  }
  galwl::warp_count(stats, 2, bad);
  galwl::warp_count(stats, 3, p != nullptr);
}

// per-request latency: clock64() around each malloc / free of one churn round
__global__ void k_lat_malloc_plain(const gal::state *s, void **ptrs, uint64_t base, uint64_t n,
                                   uint32_t seed, uint32_t *cycles) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint64_t size = galwl::mixed_size(base + t, seed);
  long long c0 = clock64();
  void *p = gal::malloc(s, size);
  long long c1 = clock64();
  if (p) *(volatile uint32_t *)p = galwl::payload(base + t, seed);
  ptrs[base + t] = p;
  cycles[t] = (uint32_t)min(c1 - c0, 0xFFFFFFFFll);
}

__global__ void k_lat_free_plain(const gal::state *s, void **ptrs, uint64_t base, uint64_t n,
                                 uint32_t *cycles) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  void *p = ptrs[base + t];
  long long c0 = clock64();
  if (p) gal::free(s, p);
  long long c1 = clock64();
  ptrs[base + t] = nullptr;
  cycles[t] = (uint32_t)min(c1 - c0, 0xFFFFFFFFll);
}

__global__ void __launch_bounds__(BT)
    k_lat_malloc_batched(const gal::state *s, void **ptrs, uint64_t base, uint64_t n, uint32_t seed,
                         uint32_t *cycles) {
  __shared__ gal::cta_claim_smem sm;
  gal::cta_claim_init(sm, BW);
  __syncthreads();
  if (threadIdx.x >= BW) {
    gal::cta_service(s, sm);
    return;
  }
  for (uint64_t c = (uint64_t)blockIdx.x * BW; c < n; c += (uint64_t)gridDim.x * BW) {
    uint64_t t = c + threadIdx.x;
    bool has = t < n;
    uint64_t size = has ? galwl::mixed_size(base + t, seed) : 0;
    long long c0 = clock64();
    void *p = gal::cta_malloc(s, size, has, sm);
    long long c1 = clock64();
    if (has) {
      if (p) *(volatile uint32_t *)p = galwl::payload(base + t, seed);
      ptrs[base + t] = p;
      cycles[t] = (uint32_t)min(c1 - c0, 0xFFFFFFFFll);
    }
  }
  gal::cta_workers_done(sm);
}

__global__ void __launch_bounds__(CACHED_BT)
    k_lat_malloc_cached(const gal::state *s, void **ptrs, uint64_t base, uint64_t n, uint32_t seed,
                        uint32_t *cycles) {
  __shared__ gal::slot_cache cache;
  gal::slot_cache_init(cache);
  __syncthreads();
  for (uint64_t c = (uint64_t)blockIdx.x * CACHED_BT; c < n; c += (uint64_t)gridDim.x * CACHED_BT) {
    const uint64_t t = c + threadIdx.x;
    if (t >= n) break;
    const uint64_t size = galwl::mixed_size(base + t, seed);
    long long c0 = clock64();
    void *p = gal::malloc_cached(s, size, cache);
    long long c1 = clock64();
    if (p) *(volatile uint32_t *)p = galwl::payload(base + t, seed);
    ptrs[base + t] = p;
    cycles[t] = (uint32_t)min(c1 - c0, 0xFFFFFFFFll);
  }
}

// the batched free path (gal_free_batched): warp teams per block through
// gal::free_n, here one pointer per thread so each free is timed alone
__global__ void __launch_bounds__(BT)
    k_lat_free_batched(const gal::state *s, void **ptrs, uint64_t base, uint64_t n, uint32_t *cycles) {
  for (uint64_t c = (uint64_t)blockIdx.x * BT; c < n; c += (uint64_t)gridDim.x * BT) {
    uint64_t t = c + threadIdx.x;
    void *const p[1] = {t < n ? ptrs[base + t] : nullptr};
    const bool go[1] = {p[0] != nullptr};
    long long c0 = clock64();
    gal::free_n<1>(s, p, go);
    long long c1 = clock64();
    if (t < n) {
      ptrs[base + t] = nullptr;
      cycles[t] = (uint32_t)min(c1 - c0, 0xFFFFFFFFll);
    }
  }
}

// the four counters of a sharded stats buffer (churn.cuh), summed; one warp
__global__ void k_stat_reduce(const unsigned long long *stats, unsigned long long *out4) {
  for (int which = 0; which < 4; which++) {
    unsigned long long t = 0;
    for (int sh = threadIdx.x; sh < galwl::STAT_SHARDS; sh += 32) t += stats[(sh * 4 + which) * 4];
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    if (threadIdx.x == 0) out4[which] = t;
  }
}

// L2 atomic probe: each thread does `iters` atomicAdd (with return) on
// distinct words of a buffer that fits in L2 (stride keeps a warp's lanes on
// different 32-byte sectors), or on one shared word when same_address.
__global__ void k_atomic_probe(uint32_t *buf, uint64_t words, int iters, int same_address,
                               uint32_t *sink) {
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  uint32_t acc = 0;
  for (int k = 0; k < iters; k++) {
    uint64_t idx = same_address ? 0 : ((tid * 8 + (uint64_t)k * nthreads * 8) % words);
    acc += atomicAdd(&buf[idx], 1u);
  }
  if (acc == 0xFFFFFFFFu) sink[0] = acc;
}

// Hot-word layout probe: `hot` counters of 8 bytes, `per_sector` of them in
// each 32-byte sector (1 = one counter per sector, 4 = densely packed); warp w
// of the grid adds to counter w % hot with one lane, `iters` times, so every
// counter is hit by its own warps only, as a pinned block's malloc word is hit
// by the claims of its SM.
__global__ void k_sector_probe(unsigned long long *buf, uint32_t hot, uint32_t per_sector, int iters,
                               unsigned long long *sink) {
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if ((threadIdx.x & 31) != 0) return;
  const uint32_t w = (uint32_t)(warp % hot);
  unsigned long long *p = buf + (uint64_t)(w / per_sector) * 4 + (w % per_sector);
  unsigned long long acc = 0;
  for (int k = 0; k < iters; k++) acc += atomicAdd(p, 1ull);
  if (acc == ~0ull) sink[0] = acc;
}

struct churn_ctx {
  gal_handle *h;
  const gal::state *d;
  uint64_t N;
  uint32_t R, seed;
  int batched;
  bool payload;   // false: the allocator-only form (no payload written or checked)
  int minb;       // CTAs per SM the malloc kernel's registers allow (2: the default; 3 or 4)
  int free_minb;  // the same for the free kernel (1: no bound; 4)
  int grid_c;     // persistent grid of the cached malloc
  size_t stage_bytes;  // dynamic shared memory of the free phase: staged segment classes (0: none)
  void **ptrs;
  uint32_t *live;  // slot liveness bits (churn.cuh)
  unsigned long long *stats;
  int k_shift;  // batched malloc: 2^k_shift requests per thread per iteration
  int grid_b;   // persistent grids: batched malloc/free, warp free phase
  int grid_f;
  std::vector<cudaEvent_t> ev;  // [2 per kernel]
  int nk = 0;
  std::vector<int> kind;        // 0 malloc, 1 free
};

void enqueue_step(churn_ctx &c, cudaStream_t st, bool capturing) {
  const uint64_t nslots = c.N * c.R;
  int k = 0;
  auto mark = [&](int kind, bool begin) {
    cudaEvent_t e = c.ev[2 * k + (begin ? 0 : 1)];
    if (capturing)
      cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else
      cudaEventRecord(e, st);
    if (!begin) {
      c.kind[k] = kind;
      k++;
    }
  };
  for (uint32_t r = 0; r <= c.R; r++) {
    bool drain = r == c.R;
    if (r > 0) {
      uint64_t nscan = drain ? nslots : c.N * r;
      mark(1, true);
      if (c.batched & 2) {
        const uint64_t chunk = (uint64_t)BT * galwl::FREE_SLOTS;
        unsigned g = (unsigned)std::min<uint64_t>((nscan + chunk - 1) / chunk, (uint64_t)c.grid_b);
        k_churn_free_batched<<<g, BT, 0, st>>>(c.d, c.ptrs, c.live, nscan, r, c.seed, drain ? 1 : 0,
                                               c.stats);
      } else {
        const uint64_t chunk = (uint64_t)(FREE_BT / 32) * galwl::WARP_SLOTS;
        unsigned g = (unsigned)std::min<uint64_t>((nscan + chunk - 1) / chunk, (uint64_t)c.grid_f);
        auto launch = [&](auto kern) {
          kern<<<g, FREE_BT, c.stage_bytes, st>>>(c.d, c.ptrs, c.live, nscan, r, c.seed, drain ? 1 : 0,
                                                  c.stage_bytes > 0, c.stats);
        };
        if (c.free_minb == 4)
          c.payload ? launch(k_churn_free_plain<true, 4>) : launch(k_churn_free_plain<false, 4>);
        else
          c.payload ? launch(k_churn_free_plain<true, 1>) : launch(k_churn_free_plain<false, 1>);
      }
      mark(1, false);
    }
    if (drain) break;
    uint64_t base = c.N * r;
    mark(0, true);
    if (c.batched & 4) {
      const unsigned gc = (unsigned)std::min<uint64_t>((c.N + CACHED_BT - 1) / CACHED_BT, (uint64_t)c.grid_c);
      auto launch = [&](auto kern) { kern<<<gc, CACHED_BT, 0, st>>>(c.d, c.ptrs, c.live, base, c.N, c.seed, c.stats); };
      if (c.minb == 4)
        c.payload ? launch(k_churn_malloc_cached<true, 4>) : launch(k_churn_malloc_cached<false, 4>);
      else if (c.minb == 3)
        c.payload ? launch(k_churn_malloc_cached<true, 3>) : launch(k_churn_malloc_cached<false, 3>);
      else
        c.payload ? launch(k_churn_malloc_cached<true, 2>) : launch(k_churn_malloc_cached<false, 2>);
    } else if (c.batched & 1) {
      const int per = 1 << c.k_shift;  // requests per thread per iteration
      unsigned gk = (unsigned)std::min<uint64_t>((c.N + (uint64_t)BW * per - 1) / ((uint64_t)BW * per),
                                                 (uint64_t)c.grid_b);
      if (c.k_shift == 2)
        k_churn_malloc_batched<4><<<gk, BT, 0, st>>>(c.d, c.ptrs, c.live, base, c.N, c.seed, c.stats);
      else if (c.k_shift == 1)
        k_churn_malloc_batched<2><<<gk, BT, 0, st>>>(c.d, c.ptrs, c.live, base, c.N, c.seed, c.stats);
      else
        k_churn_malloc_batched<1><<<gk, BT, 0, st>>>(c.d, c.ptrs, c.live, base, c.N, c.seed, c.stats);
    } else {
      const unsigned gp = (unsigned)((c.N + PLAIN_BT - 1) / PLAIN_BT);
      auto launch = [&](auto kern) { kern<<<gp, PLAIN_BT, 0, st>>>(c.d, c.ptrs, c.live, base, c.N, c.seed, c.stats); };
      if (c.minb == 4)
        c.payload ? launch(k_churn_malloc_plain<true, 4>) : launch(k_churn_malloc_plain<false, 4>);
      else if (c.minb == 3)
        c.payload ? launch(k_churn_malloc_plain<true, 3>) : launch(k_churn_malloc_plain<false, 3>);
      else
        c.payload ? launch(k_churn_malloc_plain<true, 1>) : launch(k_churn_malloc_plain<false, 1>);
    }
    mark(0, false);
  }
  c.nk = k;
}

#define CK(x)                                                                       \
  do {                                                                              \
    cudaError_t _e = (x);                                                           \
    if (_e != cudaSuccess) {                                                        \
      fprintf(stderr, "gallatin_gb300 bench: %s: %s\n", #x, cudaGetErrorString(_e)); \
      rc = GAL_ERR_CUDA;                                                            \
      goto done;                                                                    \
    }                                                                               \
  } while (0)

}  // namespace

extern "C" {

/* Mixed-size churn.  One step = `rounds` x (coin frees of the live slots before
 * every round but the first, then threads_per_round mallocs), then a drain of
 * all live slots; every step serves the same requests.  batched: bit 0 CTA-aggregated
 * malloc, bit 1 CTA-aggregated free (else per-thread with warp teams), bit 2
 * malloc in persistent CTAs that cache their SM's pinned blocks
 * (gal::malloc_cached; takes precedence over bit 0), bit 3 the allocator-only
 * form (no payload written or checked), bits 4-5: log2 of the requests each
 * thread of the CTA-aggregated malloc serves per iteration (0-2), bit 6: the
 * free phase looks segment classes up in global memory instead of a copy
 * staged in shared memory, bit 7: the cached or per-thread malloc kernel
 * compiled for 4 CTAs of 256 threads per SM (64 registers), bit 8: for 3 CTAs
 * (85 registers) -- without either, the cached kernel is compiled for 2 and
 * the per-thread kernel has no register bound; bit 9: the free kernel
 * compiled for 4 CTAs of 256 threads per SM (64 registers; else no bound);
 * higher bits are refused;
 * use_graph: the step is one captured CUDA graph.
 * step_ms[i]: duration of timed step i (CUDA events on the launching stream). */
int gal_bench_churn(gal_handle *h, uint64_t threads_per_round, uint32_t rounds, uint32_t seed,
                    int batched, int use_graph, int warmup, int steps, float *step_ms,
                    gal_churn_result *res) {
  if (!h || !res || !threads_per_round || !rounds || steps < 0 || warmup < 0) return GAL_ERR_ARGS;
  if (threads_per_round % galwl::SLOT_ALIGN) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  churn_ctx c;
  c.h = h;
  c.d = (const gal::state *)gal_device_state(h);
  c.N = threads_per_round;
  c.R = rounds;
  c.seed = seed;
  c.batched = batched & 7;
  c.payload = !(batched & 8);
  c.minb = (batched & 128) ? 4 : (batched & 256) ? 3 : 2;
  c.free_minb = (batched & 512) ? 4 : 1;
  if (batched & ~0x3FF) return GAL_ERR_ARGS;
  c.k_shift = (batched >> 4) & 3;
  if (c.k_shift > 2) return GAL_ERR_ARGS;
  c.ptrs = nullptr;
  c.live = nullptr;
  c.stats = nullptr;
  int dev = 0, sms = 0, per_sm = 0;
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const int nkern = 2 * (int)rounds + 1;
  memset(res, 0, sizeof(*res));
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_malloc_batched<1>, BT, 0);
  c.grid_b = sms * (per_sm > 0 ? per_sm : 1);
  per_sm = 0;
  {
    gal_state_dims dims;
    gal_state_dims_get(h, &dims);
    c.stage_bytes = dims.num_segments * 2 <= gal::CLASS_STAGE_BYTES && !(batched & 64) ? dims.num_segments * 2 : 0;
  }
  if (c.free_minb == 4)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_free_plain<true, 4>, FREE_BT, c.stage_bytes);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_free_plain<true, 1>, FREE_BT, c.stage_bytes);
  c.grid_f = sms * (per_sm > 0 ? per_sm : 1);
  per_sm = 0;
  if (c.minb == 4)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_malloc_cached<true, 4>, CACHED_BT, 0);
  else if (c.minb == 3)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_malloc_cached<true, 3>, CACHED_BT, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_churn_malloc_cached<true, 2>, CACHED_BT, 0);
  c.grid_c = sms * (per_sm > 0 ? per_sm : 1);
  c.ev.resize(2 * nkern);
  c.kind.resize(nkern);
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  for (auto &e : c.ev) CK(cudaEventCreate(&e));
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaMalloc(&c.ptrs, threads_per_round * rounds * sizeof(void *)));
  CK(cudaMemsetAsync(c.ptrs, 0, threads_per_round * rounds * sizeof(void *), st));
  CK(cudaMalloc(&c.live, threads_per_round * rounds / 8));
  CK(cudaMemsetAsync(c.live, 0, threads_per_round * rounds / 8, st));
  CK(cudaMalloc(&c.stats, galwl::STAT_WORDS * sizeof(unsigned long long)));
  if (use_graph) {
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    enqueue_step(c, st, true);
    CK(cudaStreamEndCapture(st, &graph));
    CK(cudaGraphInstantiate(&exec, graph, 0));
  }
  for (int s = 0; s < warmup + steps; s++) {
    CK(cudaMemsetAsync(c.stats, 0, galwl::STAT_WORDS * sizeof(unsigned long long), st));
    CK(cudaStreamSynchronize(st));
    CK(cudaEventRecord(e0, st));
    if (use_graph)
      CK(cudaGraphLaunch(exec, st));
    else
      enqueue_step(c, st, false);
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    CK(cudaGetLastError());
    if (s >= warmup) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (step_ms) step_ms[s - warmup] = ms;
      res->ms_total += ms;
      for (int k = 0; k < c.nk; k++) {
        float km = 0;
        CK(cudaEventElapsedTime(&km, c.ev[2 * k], c.ev[2 * k + 1]));
        if (c.kind[k] == 0) {
          res->ms_malloc_kernels += km;
          res->malloc_launches++;
        } else {
          res->ms_free_kernels += km;
          res->free_launches++;
        }
      }
      std::vector<unsigned long long> sv(galwl::STAT_WORDS);
      CK(cudaMemcpy(sv.data(), c.stats, sv.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      res->mallocs_ok += galwl::stat_total(sv.data(), 0);
      res->mallocs_failed += galwl::stat_total(sv.data(), 1);
      res->payload_mismatch += galwl::stat_total(sv.data(), 2);
      res->frees += galwl::stat_total(sv.data(), 3);
    }
  }
  gal_last_error(h, &res->error_word);
done:
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (auto &e : c.ev)
    if (e) cudaEventDestroy(e);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (c.ptrs) cudaFree(c.ptrs);
  if (c.live) cudaFree(c.live);
  if (c.stats) cudaFree(c.stats);
  if (st) cudaStreamDestroy(st);
  return rc;
}

/* The churn end to end through the public entry points: every round the
 * request sizes are copied from pinned host memory (host_sizes, rounds x
 * threads_per_round, same sizes as the device-generated workload) on a copy
 * stream, two rounds ahead into two alternating buffers, and served by
 * gal_malloc_batched; a user kernel stamps the payloads; frees are selected by
 * a user kernel that compacts them into a list whose length stays on the
 * device, served by gal_free_batched_n; the step's counters are read back.
 * The selection runs on a third stream in two parts: the slots of the older
 * rounds as soon as the previous selection is done (overlapping the previous
 * round's free, malloc and stamp), the slots of the round just stamped after
 * its stamp; each part's frees are served as soon as it is selected (the first
 * part's while the second is selected), from lists that alternate between
 * rounds.  Each round still frees before it allocates.  use_graph: the step (all three streams, copies
 * included) is captured once as a CUDA graph, as a user replaying the same
 * step would. */
int gal_bench_churn_e2e(gal_handle *h, const uint64_t *host_sizes, uint64_t threads_per_round,
                        uint32_t rounds, uint32_t seed, int warmup, int steps, float *step_ms,
                        gal_churn_result *res, int use_graph) {
  if (!h || !res || !host_sizes || !threads_per_round || !rounds) return GAL_ERR_ARGS;
  if (threads_per_round % galwl::SLOT_ALIGN) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  const uint64_t N = threads_per_round, nslots = N * rounds;
  void **ptrs = nullptr, **freelist[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  uint32_t *live = nullptr;
  uint64_t *d_sizes[2] = {nullptr, nullptr};
  unsigned long long *stats = nullptr, *total4 = nullptr, *hst = nullptr;
  unsigned long long *count[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaStream_t st = nullptr, cp = nullptr, sl = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr, copied[2] = {nullptr, nullptr},
              consumed[2] = {nullptr, nullptr}, stamped = nullptr, selected[2] = {nullptr, nullptr};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int dev = 0, sms = 0, per_sm = 0;
  memset(res, 0, sizeof(*res));
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_select_free_list, FREE_BT, 0);
  const uint64_t grid_sel = (uint64_t)sms * (per_sm > 0 ? per_sm : 1);
  auto sel_grid = [&](uint64_t nscan) {
    const uint64_t chunk = (uint64_t)(FREE_BT / 32) * galwl::WARP_SLOTS;
    return (unsigned)std::min<uint64_t>((nscan + chunk - 1) / chunk, grid_sel);
  };
  auto enqueue = [&]() -> int {
    if (cudaMemsetAsync(stats, 0, galwl::STAT_WORDS * sizeof(unsigned long long), st) != cudaSuccess) return GAL_ERR_CUDA;
    if (cudaEventRecord(fork, st) != cudaSuccess || cudaStreamWaitEvent(cp, fork, 0) != cudaSuccess ||
        cudaStreamWaitEvent(sl, fork, 0) != cudaSuccess)
      return GAL_ERR_CUDA;
    for (uint32_t r = 0; r < rounds && r < 2; r++) {
      if (cudaMemcpyAsync(d_sizes[r], host_sizes + (uint64_t)r * N, N * sizeof(uint64_t),
                          cudaMemcpyHostToDevice, cp) != cudaSuccess ||
          cudaEventRecord(copied[r], cp) != cudaSuccess)
        return GAL_ERR_CUDA;
    }
    for (uint32_t r = 0; r <= rounds; r++) {
      const bool drain = r == rounds;
      if (r > 0) {
        // part 0: the older rounds' slots, selected without waiting for the
        // round just stamped and freed while part 1 (that round's slots) is
        // still being selected
        const int q = (int)(r & 1u);
        const uint64_t mid = (uint64_t)(r - 1) * N, hi = drain ? nslots : N * r;
        const uint64_t lo_of[2] = {0, mid}, hi_of[2] = {mid, hi};
        for (int part = 0; part < 2; part++) {
          if (part == 1 && cudaStreamWaitEvent(sl, stamped, 0) != cudaSuccess) return GAL_ERR_CUDA;
          if (hi_of[part] == lo_of[part]) continue;
          if (cudaMemsetAsync(count[q][part], 0, sizeof(unsigned long long), sl) != cudaSuccess)
            return GAL_ERR_CUDA;
          k_select_free_list<<<sel_grid(hi_of[part] - lo_of[part]), FREE_BT, 0, sl>>>(
              ptrs, live, freelist[q][part], count[q][part], lo_of[part], hi_of[part], r, seed,
              drain ? 1 : 0, stats);
          if (cudaEventRecord(selected[part], sl) != cudaSuccess ||
              cudaStreamWaitEvent(st, selected[part], 0) != cudaSuccess)
            return GAL_ERR_CUDA;
          int e = gal_free_batched_n(h, freelist[q][part], count[q][part], hi_of[part] - lo_of[part], st);
          if (e) return e;
        }
      }
      if (drain) break;
      const int b = (int)(r & 1u);
      if (cudaStreamWaitEvent(st, copied[b], 0) != cudaSuccess) return GAL_ERR_CUDA;
      int e = gal_malloc_batched(h, d_sizes[b], N, ptrs + (uint64_t)r * N, st);
      if (e) return e;
      if (cudaEventRecord(consumed[b], st) != cudaSuccess) return GAL_ERR_CUDA;
      if (r + 2 < rounds) {
        if (cudaStreamWaitEvent(cp, consumed[b], 0) != cudaSuccess ||
            cudaMemcpyAsync(d_sizes[b], host_sizes + (uint64_t)(r + 2) * N, N * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, cp) != cudaSuccess ||
            cudaEventRecord(copied[b], cp) != cudaSuccess)
          return GAL_ERR_CUDA;
      }
      k_stamp_payload<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(ptrs, live, (uint64_t)r * N, N,
                                                                   seed, stats);
      if (cudaEventRecord(stamped, st) != cudaSuccess) return GAL_ERR_CUDA;
    }
    k_stat_reduce<<<1, 32, 0, st>>>(stats, total4);  // the step's four counters, then read back
    if (cudaMemcpyAsync(hst, total4, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st) !=
        cudaSuccess)
      return GAL_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? GAL_OK : GAL_ERR_CUDA;
  };
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&cp, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&sl, cudaStreamNonBlocking));
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&stamped, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&selected[0], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&selected[1], cudaEventDisableTiming));
  for (int b = 0; b < 2; b++) {
    CK(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&consumed[b], cudaEventDisableTiming));
    CK(cudaMalloc(&d_sizes[b], N * sizeof(uint64_t)));
    for (int part = 0; part < 2; part++) {
      CK(cudaMalloc(&freelist[b][part], nslots * sizeof(void *)));
      CK(cudaMalloc(&count[b][part], sizeof(unsigned long long)));
    }
  }
  CK(cudaMalloc(&ptrs, nslots * sizeof(void *)));
  CK(cudaMalloc(&live, nslots / 8));
  CK(cudaMalloc(&stats, galwl::STAT_WORDS * sizeof(unsigned long long)));
  CK(cudaMalloc(&total4, 4 * sizeof(unsigned long long)));
  CK(cudaMallocHost(&hst, 4 * sizeof(unsigned long long)));
  CK(cudaMemsetAsync(ptrs, 0, nslots * sizeof(void *), st));
  CK(cudaMemsetAsync(live, 0, nslots / 8, st));
  CK(cudaStreamSynchronize(st));
  if (use_graph) {
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    int e = enqueue();
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (e) { rc = e; goto done; }
    CK(ce);
    CK(cudaGraphInstantiate(&exec, graph, 0));
  }
  for (int s = 0; s < warmup + steps; s++) {
    CK(cudaStreamSynchronize(st));
    CK(cudaEventRecord(e0, st));
    if (use_graph) {
      CK(cudaGraphLaunch(exec, st));
    } else {
      int e = enqueue();
      if (e) { rc = e; goto done; }
    }
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    CK(cudaGetLastError());
    if (s >= warmup) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (step_ms) step_ms[s - warmup] = ms;
      res->ms_total += ms;
      res->mallocs_ok += hst[0];
      res->mallocs_failed += hst[1];
      res->payload_mismatch += hst[2];
      res->frees += hst[3];
      res->malloc_launches += rounds;
      res->free_launches += rounds;
      res->other_launches += 3 * rounds + 1;  // two selection parts and the stamp a round, the count
    }
  }
  res->h2d_bytes = nslots * sizeof(uint64_t);
  res->d2h_bytes = 4 * sizeof(unsigned long long);
  gal_last_error(h, &res->error_word);
done:
  if (st) cudaStreamSynchronize(st);
  if (cp) cudaStreamSynchronize(cp);
  if (sl) cudaStreamSynchronize(sl);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (fork) cudaEventDestroy(fork);
  if (stamped) cudaEventDestroy(stamped);
  for (int part = 0; part < 2; part++)
    if (selected[part]) cudaEventDestroy(selected[part]);
  for (int b = 0; b < 2; b++) {
    if (copied[b]) cudaEventDestroy(copied[b]);
    if (consumed[b]) cudaEventDestroy(consumed[b]);
    if (d_sizes[b]) cudaFree(d_sizes[b]);
    for (int part = 0; part < 2; part++) {
      if (freelist[b][part]) cudaFree(freelist[b][part]);
      if (count[b][part]) cudaFree(count[b][part]);
    }
  }
  if (ptrs) cudaFree(ptrs);
  if (live) cudaFree(live);
  if (stats) cudaFree(stats);
  if (total4) cudaFree(total4);
  if (hst) cudaFreeHost(hst);
  if (st) cudaStreamDestroy(st);
  if (cp) cudaStreamDestroy(cp);
  if (sl) cudaStreamDestroy(sl);
  return rc;
}

/* Per-request latency in SM cycles (clock64) of one churn round of n mixed
 * requests at full concurrency: malloc_cycles[i], then free_cycles[i] when the
 * same allocations are freed.  One unmeasured round first.  Host buffers.
 * batched: 0 per-thread calls, 1 CTA-aggregated claims and batched frees,
 * 2 persistent CTAs with cached pinned blocks and batched frees. */
int gal_bench_latency(gal_handle *h, uint64_t n, uint32_t seed, int batched,
                      uint32_t *malloc_cycles, uint32_t *free_cycles) {
  if (!h || !n || !malloc_cycles || !free_cycles) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  void **ptrs = nullptr;
  uint32_t *cm = nullptr, *cf = nullptr;
  const gal::state *d = (const gal::state *)gal_device_state(h);
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lat_malloc_batched, BT, 0);
  unsigned gb = (unsigned)std::min<uint64_t>((n + BW - 1) / BW, (uint64_t)sms * (per_sm > 0 ? per_sm : 1));
  per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lat_malloc_cached, CACHED_BT, 0);
  unsigned gr = (unsigned)std::min<uint64_t>((n + CACHED_BT - 1) / CACHED_BT, (uint64_t)sms * (per_sm > 0 ? per_sm : 1));
  unsigned gp = (unsigned)((n + 255) / 256);
  CK(cudaMalloc(&ptrs, n * sizeof(void *)));
  CK(cudaMalloc(&cm, n * 4));
  CK(cudaMalloc(&cf, n * 4));
  for (int r = 0; r < 2; r++) {
    if (batched == 2) {
      k_lat_malloc_cached<<<gr, CACHED_BT>>>(d, ptrs, 0, n, seed + r, cm);
      k_lat_free_batched<<<gb, BT>>>(d, ptrs, 0, n, cf);
    } else if (batched) {
      k_lat_malloc_batched<<<gb, BT>>>(d, ptrs, 0, n, seed + r, cm);
      k_lat_free_batched<<<gb, BT>>>(d, ptrs, 0, n, cf);
    } else {
      k_lat_malloc_plain<<<gp, 256>>>(d, ptrs, 0, n, seed + r, cm);
      k_lat_free_plain<<<gp, 256>>>(d, ptrs, 0, n, cf);
    }
    CK(cudaDeviceSynchronize());
  }
  CK(cudaMemcpy(malloc_cycles, cm, n * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(free_cycles, cf, n * 4, cudaMemcpyDeviceToHost));
done:
  if (ptrs) cudaFree(ptrs);
  if (cm) cudaFree(cm);
  if (cf) cudaFree(cf);
  return rc;
}

/* Request sizes of the churn workload, computed on the host (for e2e). */
int gal_churn_sizes(uint64_t base_slot, uint64_t n, uint32_t seed, uint64_t *out) {
  if (!out) return GAL_ERR_ARGS;
  for (uint64_t i = 0; i < n; i++) out[i] = galwl::mixed_size(base_slot + i, seed);
  return GAL_OK;
}

/* n threads x malloc(size) with a thread-id stamp, then check and free, for
 * `rounds` rounds.  ms[0]: malloc kernels, ms[1]: free kernels (summed).
 * stats: [0] ok [1] failed [2] stamp mismatches [3] frees. */
int gal_bench_stamp(gal_handle *h, uint64_t n, uint64_t size, int rounds, float *ms,
                    uint64_t *stats_out) {
  if (!h || !ms || !stats_out || !n) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  uint64_t **ptrs = nullptr;
  unsigned long long *stats = nullptr;
  cudaEvent_t a = nullptr, b = nullptr, c = nullptr;
  const gal::state *d = (const gal::state *)gal_device_state(h);
  unsigned grid = (unsigned)((n + 255) / 256);
  ms[0] = ms[1] = 0;
  CK(cudaMalloc(&ptrs, n * sizeof(void *)));
  CK(cudaMalloc(&stats, galwl::STAT_WORDS * sizeof(unsigned long long)));
  CK(cudaMemset(stats, 0, galwl::STAT_WORDS * sizeof(unsigned long long)));
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventCreate(&c));
  for (int r = 0; r < rounds; r++) {
    CK(cudaEventRecord(a));
    k_stamp_malloc<<<grid, 256>>>(d, n, size, ptrs, stats);
    CK(cudaEventRecord(b));
    k_stamp_free<<<grid, 256>>>(d, n, ptrs, stats);
    CK(cudaEventRecord(c));
    CK(cudaEventSynchronize(c));
    CK(cudaGetLastError());
    float x = 0, y = 0;
    CK(cudaEventElapsedTime(&x, a, b));
    CK(cudaEventElapsedTime(&y, b, c));
    ms[0] += x;
    ms[1] += y;
  }
  {
    std::vector<unsigned long long> sv(galwl::STAT_WORDS);
    CK(cudaMemcpy(sv.data(), stats, sv.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 4; i++) stats_out[i] = galwl::stat_total(sv.data(), i);
  }
done:
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (c) cudaEventDestroy(c);
  if (ptrs) cudaFree(ptrs);
  if (stats) cudaFree(stats);
  return rc;
}

/* Atomics per second on `hot` 8-byte counters packed `per_sector` to a
 * 32-byte sector (1, 2 or 4), each counter hit by warps of its own
 * (k_sector_probe): how the packing of concurrently claimed malloc words
 * changes the L2 atomic rate. */
int gal_bench_sector_probe(uint32_t hot, uint32_t per_sector, double *atomics_per_s) {
  if (!atomics_per_s || !hot || !per_sector || per_sector > 4) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  unsigned long long *buf = nullptr, *sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned block = 256, grid = (unsigned)sms * 4;
  const int iters = 512;
  const uint64_t words = ((uint64_t)hot / per_sector + 1) * 4;
  CK(cudaMalloc(&buf, words * 8));
  CK(cudaMalloc(&sink, 8));
  CK(cudaMemset(buf, 0, words * 8));
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  {
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
      CK(cudaEventRecord(a));
      k_sector_probe<<<grid, block>>>(buf, hot, per_sector, iters, sink);
      CK(cudaEventRecord(b));
      CK(cudaEventSynchronize(b));
      CK(cudaGetLastError());
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0 && ms < best) best = ms;
    }
    *atomics_per_s = (double)grid * (block / 32) * iters / (best * 1e-3);
  }
done:
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (buf) cudaFree(buf);
  if (sink) cudaFree(sink);
  return rc;
}

/* L2 atomic throughput (atomicAdd.u32 with return) in atomics per second, on
 * distinct words of a 32 MiB buffer (resident in L2) and on one word. */
int gal_bench_atomic_peak(double *distinct_per_s, double *same_addr_per_s) {
  if (!distinct_per_s || !same_addr_per_s) return GAL_ERR_ARGS;
  int rc = GAL_OK;
  uint32_t *buf = nullptr, *sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  const uint64_t words = (32ull << 20) / 4;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)sms * 8, block = 256;
  const int iters = 256;
  CK(cudaMalloc(&buf, words * 4));
  CK(cudaMalloc(&sink, 4));
  CK(cudaMemset(buf, 0, words * 4));
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  for (int same = 0; same < 2; same++) {
    int it = same ? 16 : iters;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
      CK(cudaEventRecord(a));
      k_atomic_probe<<<grid, block>>>(buf, words, it, same, sink);
      CK(cudaEventRecord(b));
      CK(cudaEventSynchronize(b));
      CK(cudaGetLastError());
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0 && ms < best) best = ms;
    }
    double n = (double)grid * block * it;
    (same ? *same_addr_per_s : *distinct_per_s) = n / (best * 1e-3);
  }
done:
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (buf) cudaFree(buf);
  if (sink) cudaFree(sink);
  return rc;
}

}  // extern "C"
