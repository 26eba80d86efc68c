/*
 * gallatin_gb300.h — C ABI of the GB300-native Gallatin-compatible device allocator.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (GAL_OK == 0, otherwise one of the GAL_ERR_* codes below).  Device buffers are
 * raw CUDA device pointers; `stream` is a cudaStream_t passed as void* (NULL =
 * legacy default stream).  No C++ or torch types appear in these signatures.
 *
 * The reference (chillenzer/gallatin) is a header-only CUDA C++ library with no
 * FFI of its own.  Each function below names the reference interface it stands
 * in for (path:line inside the reference project).  The device-side malloc/free
 * stay header-inline (include/gallatin_gb300/gal_device.cuh and the drop-in
 * headers under include/gallatin/allocators/) because a device function cannot
 * cross a C ABI.
 */
#ifndef GALLATIN_GB300_H
#define GALLATIN_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GAL_OK               0
#define GAL_ERR_ARGS         1   /* invalid argument / size out of range            */
#define GAL_ERR_CUDA         2   /* a CUDA runtime call failed                       */
#define GAL_ERR_OOM          3   /* device memory for arena/metadata not available   */
#define GAL_ERR_STATE        4   /* handle not initialised / already initialised     */
#define GAL_ERR_DEVICE       5   /* the device error word is non-zero (see below)    */

/* ---- device error word bits (gal_last_error) ----------------------------- */
#define GAL_DEV_ERR_TIMEOUT        0x1u  /* a bounded spin-wait gave up             */
#define GAL_DEV_ERR_BAD_FREE       0x2u  /* free of a pointer in a free segment      */
#define GAL_DEV_ERR_NULL_QUEUE     0x4u  /* recycle ring slot empty on hand-out      */
#define GAL_DEV_ERR_SEGMENT_SETUP  0x8u  /* segment tree id claim failed             */
#define GAL_DEV_ERR_SLOT_SWAP      0x10u /* pinned slot swap-in found a block        */
#define GAL_DEV_ERR_BLOCK_TREE     0x20u /* whole-block fill saw a foreign tree id   */
#define GAL_DEV_ERR_BOOT           0x40u /* boot could not fill a pinned slot        */

/* ---- sub-tree (size class) segment choice --------------------------------- */
#define GAL_POLICY_REFERENCE 0u  /* Murmur-hashed start, as gallatin veb.cuh:946-977 */
#define GAL_POLICY_LOWEST    1u  /* always the smallest segment id with free blocks */

/* ---- limits --------------------------------------------------------------- */
#define GAL_MAX_TREES        16
#define GAL_MAX_VEB_LAYERS   8

/* Runtime configuration.  The three geometry fields are the reference's
 * template parameters Gallatin<bytes_per_segment, smallest, biggest>
 * (gallatin.cuh:292); all three must be powers of two and
 * bytes_per_segment >= max_size*4096 (gallatin.cuh:300). */
typedef struct gal_config {
  uint64_t bytes_per_segment;   /* default 16 MiB                                  */
  uint64_t min_size;            /* default 16 B                                    */
  uint64_t max_size;            /* default 4096 B                                  */
  int32_t  smid_override;       /* -1: pinned slot from %smid; >=0: fixed value   */
  uint32_t subtree_policy;      /* GAL_POLICY_*                                    */
  uint32_t pinned_slots_first;  /* pinned slots of tree 0 (reference: 128);
                                   0 = one slot per SM in every size class        */
  uint32_t pinned_slots_min;    /* floor when halving per tree (reference: 4)     */
  uint32_t zero_arena;          /* 1: memset the arena at init (reference does)   */
  uint32_t spin_limit;          /* iteration cap for every device spin-wait       */
  uint32_t gather_unlocked_below; /* size classes with fewer blocks per segment
                                   gather segments without the class lock
                                   (default 16; 0 = always lock, as
                                   gallatin.cuh:1538).  One thread alone always
                                   finds the lock free, so serial offsets are
                                   the reference's either way; concurrently,
                                   classes whose blocks fill a segment in a few
                                   replacements stop queueing on the lock.     */
  uint32_t team_width;          /* aggregation width of per-thread claims and
                                   frees: lanes that share one atomic come from
                                   aligned groups of this many (1..32, a power
                                   of two; 32 or 0 = the whole warp, as the
                                   reference's coalesced teams)                  */
  uint32_t arena_kind;          /* GAL_ARENA_*: where the arena lives; metadata
                                   is always device memory                       */
  uint32_t spare_blocks;        /* 1: every pinned slot keeps its next block
                                   prepared, so a block running out is replaced
                                   by one swap instead of a search of the
                                   class's segments on the claim's path (the
                                   CTA-aggregated kernels refill spares from a
                                   service warp, per-thread calls from the lane
                                   that swapped, after its team has gone on).
                                   Costs one block per slot held in reserve;
                                   serial offsets then differ from the
                                   reference's.  0 = the reference's behaviour. */
  uint32_t zero_fill;           /* 1: calloc mode (the reference's running_calloc):
                                   the requested bytes of every allocation are
                                   zero when handed out.  The reference keeps
                                   returned blocks and segment runs zero by
                                   clearing them in child kernels (dynamic
                                   parallelism); here the allocating thread
                                   clears its own bytes.  Default 0.            */
  uint32_t block_layout;        /* GAL_BLOCK_LAYOUT_*: where each block's malloc
                                   and free counters live.  RECORD (default):
                                   both in one 32-byte record, one L2 sector per
                                   block, so the blocks that different SMs claim
                                   from at the same time never share a sector.
                                   DENSE: all malloc words in one array (8 B
                                   each), all free counters in another (4 B).
                                   The reference's Block is the dense 8-byte
                                   pair (block.cuh:59); offsets are the same
                                   either way.                                   */
  uint32_t l2_fetch_bytes;      /* 0 (default): leave the context as it is; 32,
                                   64 or 128: gal_create sets
                                   cudaLimitMaxL2FetchGranularity to it on the
                                   allocator's device.  A hint for the whole
                                   context (every kernel of the process on
                                   that device, until changed).  Scattered
                                   small reads of allocations, such as a
                                   payload check before each free, then fetch
                                   32 B instead of a whole line: the mixed
                                   churn's free phase read 2.8x fewer DRAM
                                   bytes at 32.                                 */
  uint32_t gather_ahead;        /* 1 (default): a request that takes the last
                                   block of a class's segment also gathers the
                                   class's next segment, as the reference does
                                   (gallatin.cuh:1598-1612).  0: segments are
                                   gathered only by requests that find their
                                   class without one (slower on the mixed
                                   churn: those requests wait for the
                                   gather).  0 changes serial results.        */
} gal_config;

/* Block counter layouts (gal_config.block_layout). */
#define GAL_BLOCK_LAYOUT_DENSE 0u
#define GAL_BLOCK_LAYOUT_RECORD 1u

/* Arena backing (gal_config.arena_kind). */
#define GAL_ARENA_DEVICE 0u  /* cudaMalloc (generate_on_device, gallatin.cuh:324)  */
#define GAL_ARENA_HOST 1u    /* pinned host memory mapped into the device's
                                address space (generate_on_device_host,
                                gallatin.cuh:427)                                  */
#define GAL_ARENA_MANAGED 2u /* cudaMallocManaged (generate_on_device_managed,
                                gallatin.cuh:531)                                  */

/* Aggregate statistics (stands in for Gallatin::print_info, gallatin.cuh:1855). */
typedef struct gal_stats {
  uint64_t num_segments;
  uint64_t free_segments;                 /* set bits of the segment tree        */
  uint64_t largest_free_run;              /* longest run of free segments        */
  uint32_t num_trees;
  uint32_t error_word;
  uint64_t tree_segments[GAL_MAX_TREES];  /* segments owned (table tree id)      */
  uint64_t tree_listed[GAL_MAX_TREES];    /* set bits of each size-class tree    */
  uint64_t tree_live_blocks[GAL_MAX_TREES];
  uint64_t multi_segment_allocs;          /* live multi-segment allocations     */
  uint64_t multi_segment_segments;        /* segments they cover                 */
  uint64_t metadata_bytes;                /* device bytes of allocator metadata  */
} gal_stats;

/* Dimensions of the host-side state view (sizes of the arrays below). */
typedef struct gal_state_dims {
  uint64_t num_segments;        /* S                                              */
  uint32_t num_trees;           /* T                                              */
  uint32_t blocks_per_segment;  /* table stride: bytes_per_segment/(min*4096)     */
  uint32_t veb_layers;          /* layers of every vEB tree (universe S)          */
  uint32_t veb_words;           /* 64-bit words of one tree, all layers           */
  uint32_t total_slots;         /* pinned slots summed over trees                 */
  uint32_t slot_counts[GAL_MAX_TREES];
} gal_state_dims;

/* Host-side, layout-neutral copy of the whole allocator state, in the
 * reference's value conventions so that states from the reference build, the
 * CPU oracle and this library compare word for word:
 *   - vEB words: per tree, layer 0 (top) first, each layer ceil(u/64) words;
 *   - malloc_counters: (tree << 20) | count, as gallatin block.cuh:53,220;
 *   - queues / slots: global block id, or -1 for an empty entry (nullptr).
 * The caller owns every buffer; sizes follow gal_state_dims. */
typedef struct gal_state_view {
  uint64_t *seg_tree_words;             /* [veb_words]                     */
  uint64_t *sub_tree_words;             /* [num_trees * veb_words]         */
  uint16_t *tree_ids;                   /* [S], 0xFFFF = free              */
  int32_t  *active_counts;              /* [S]                             */
  uint32_t *queue_counters;             /* [S]                             */
  uint32_t *queue_free_counters;        /* [S]                             */
  uint32_t *final_queue_free_counters;  /* [S]                             */
  uint32_t *malloc_counters;            /* [S * blocks_per_segment]        */
  uint32_t *free_counters;              /* [S * blocks_per_segment]        */
  int32_t  *queues;                     /* [S * blocks_per_segment]        */
  int32_t  *slots;                      /* [total_slots]                   */
  uint32_t  locks;
  uint32_t  error_word;
} gal_state_view;

typedef struct gal_handle gal_handle;

/* Fill *cfg with the reference defaults: <16 MiB, 16, 4096>, 128/4 pinned
 * slots, reference sub-tree policy, hardware %smid, zeroed arena. */
int gal_config_default(gal_config *cfg);

/* Build an allocator over `num_bytes` of device memory on the current device.
 * Replaces Gallatin<>::generate_on_device (gallatin.cuh:324-421).  The pinned
 * slots are booted deterministically in the order of the reference's
 * boot_shared_block_container_one_thread (gallatin.cuh:196-221).  The calls
 * that launch work for a handle (batched and per-thread malloc/free, trim,
 * the exports) run it on the handle's device, whichever device is current,
 * and leave the caller's current device as it was; the stream passed must
 * belong to that device. */
int gal_create(uint64_t num_bytes, uint64_t seed, const gal_config *cfg, gal_handle **out);

/* Same as gal_create without the boot (pinned slots empty); for state import. */
int gal_create_unbooted(uint64_t num_bytes, uint64_t seed, const gal_config *cfg, gal_handle **out);

/* Release arena and metadata.  Replaces Gallatin<>::free_on_device
 * (gallatin.cuh:643-668).  Pointers handed out become invalid. */
int gal_destroy(gal_handle *h);

/* Device pointer to the allocator object (what a Gallatin<>* points to). */
void *gal_device_state(gal_handle *h);
/* Host handle that owns a device allocator object (NULL if none). */
gal_handle *gal_handle_of(const void *device_state);
/* Device pointer to the first byte of the arena (alloc_table::memory,
 * memory_table.cuh:255). */
void *gal_arena_base(gal_handle *h);
/* Bytes covered by the arena (num_segments * bytes_per_segment). */
uint64_t gal_arena_bytes(gal_handle *h);

/* Replaces print_global_stats / Gallatin::print_info
 * (global_allocator.cuh:86-97, gallatin.cuh:1855-1897). */
int gal_get_stats(gal_handle *h, gal_stats *out);
int gal_print_stats(gal_handle *h);

/* Device error word (GAL_DEV_ERR_* bits); replaces the reference's `trap`
 * on invariant breaks (gallatin.cuh:87). */
int gal_last_error(gal_handle *h, uint32_t *out_bits);
int gal_clear_error(gal_handle *h);
/* First recorded error: out4 = {site, value a, value b, recorded flag}.
 * Sites: 1 a block returned to a segment of no class (a: block, b: tree id);
 * 2-5 frees (overflowing a block's count, outside the arena, into a free
 * segment, of a segment run twice); 6 a block request whose class lock
 * stayed taken past spin_limit (a: class, b: spins); 7 a block request whose
 * listed segments kept refusing a block (a: class, b: last segment); 8 a
 * segment-run request whose lock stayed taken (a: segments wanted). */
int gal_error_info(gal_handle *h, uint64_t *out4);

/* State view export/import (no reference counterpart: a snapshot of every
 * metadata array, for parity tests and drain checks). */
int gal_state_dims_get(gal_handle *h, gal_state_dims *out);
int gal_export_state(gal_handle *h, gal_state_view *view);
int gal_import_state(gal_handle *h, const gal_state_view *view);

/* Same result as gal_export_state, without allocating device memory and
 * without waiting for the whole device: for callers that cannot
 * cudaMalloc/cudaFree at this point (a caching allocator already holds the
 * device's memory, or the device-memory budget is fixed) and for monitors
 * that snapshot while other streams keep running.  No counterpart in the
 * reference.  Stages the block counters in a fixed 1 MiB device array
 * (GAL_NOALLOC_MAX_BLOCKS counters) that every GPU loading the library keeps
 * until exit; larger allocators get GAL_ERR_ARGS.  Runs on a stream of its
 * own and waits for that stream only, on the handle's device.  gal_create
 * sets the array and the stream up on its device, so the call itself loads
 * and allocates nothing; a first call on a device that was never set up does
 * the set-up then and should come before any stream capture.  Calls share the
 * array, so calls that overlap on the GPU race.  While device malloc/free run
 * on other streams the copy is not a consistent cut (each word holds some
 * value it had during the call). */
#define GAL_NOALLOC_MAX_BLOCKS (1u << 18)
int gal_export_state_noalloc(gal_handle *h, gal_state_view *view);

/* Change the pinned-slot smid override after creation (-1 = hardware). */
int gal_set_smid_override(gal_handle *h, int32_t smid);
/* Change the sub-tree policy after creation (GAL_POLICY_*). */
int gal_set_policy(gal_handle *h, uint32_t policy);

/* ---- process-global instance (drop-in init/teardown) ---------------------- */
/* Replaces init_global_allocator (global_allocator.cuh:48-56). */
int gal_init(uint64_t num_bytes, uint64_t seed, const gal_config *cfg);
/* Replaces free_global_allocator (global_allocator.cuh:59-70). */
int gal_teardown(void);
/* The global handle (NULL before gal_init). */
gal_handle *gal_global(void);
/* The second process-global instance, with its arena in host memory: replaces
 * init_global_allocator_host / free_global_allocator_host
 * (global_allocator.cuh:100-123); cfg->arena_kind is forced to GAL_ARENA_HOST. */
int gal_init_host(uint64_t num_bytes, uint64_t seed, const gal_config *cfg);
int gal_teardown_host(void);
gal_handle *gal_global_host(void);

/* ---- device work launched by the library ---------------------------------- */

/* Serial replay of an op trace by one device thread, the single-thread test of
 * the reference (tests/src/gallatin_single_thread.cu:38-93) generalised.
 * ops[i]: bit 63 clear → malloc(ops[i]); bit 63 set → free of the pointer
 * returned by op (ops[i] & ~bit63).  out_offsets[i] = pointer - arena base for
 * a malloc (UINT64_MAX for nullptr), UINT64_MAX for a free.  out_smid[0] =
 * %smid the thread ran on.  All buffers are device pointers. */
int gal_replay_trace(gal_handle *h, const uint64_t *ops, uint64_t nops,
                     uint64_t *out_offsets, uint32_t *out_smid, void *stream);

/* Replay of a trace of warp-wide calls by one warp (thread ids 0-31): the
 * warp-aggregated slice claim of Gallatin::malloc_slice_allocation
 * (gallatin.cuh:865-1078) with lanes joining one team.  Step i is 33 words:
 * steps[33 i] = kind << 32 | lane mask, then one word per lane.  Kind 0: the
 * masked lanes call malloc together as one set of callers (the device
 * malloc_team with the step's mask, so the teams do not depend on how the
 * scheduler regroups diverged lanes), lane l with size steps[33 i + 1 + l];
 * kind 1: the masked lanes free, one lane at a time in lane order, the
 * result of earlier call steps[33 i + 1 + l] (an index step * 32 + lane;
 * failed calls and later indices are skipped).  out_offsets[32 i + l] =
 * pointer - arena base of a kind-0 result, UINT64_MAX otherwise.  Device
 * pointers. */
int gal_replay_warp_trace(gal_handle *h, const uint64_t *steps, uint64_t nsteps,
                          uint64_t *out_offsets, uint32_t *out_smid, void *stream);

/* One device thread per request: out_ptrs[i] = malloc(sizes[i]) (per-thread
 * global_malloc, global_allocator.cuh:72-76). */
int gal_malloc_per_thread(gal_handle *h, const uint64_t *sizes, uint64_t n,
                          void **out_ptrs, void *stream);
/* One device thread per pointer: free(ptrs[i]) unless NULL
 * (global_free, global_allocator.cuh:78-82). */
int gal_free_per_thread(gal_handle *h, void *const *ptrs, uint64_t n, void *stream);

/* Give back what the pinned slots hold (no counterpart in the reference; the
 * host-side analogue of malloc_trim).  Call with no device malloc/free in
 * flight.  Every pinned block is retired: the slices it never handed out are
 * credited to its free counter, so a block with nothing live returns to its
 * segment (and one with live slices when the last of them is freed), and
 * emptied segments return to the segment tree.  The slots are then booted
 * again in the one-thread order, so with nothing live the trees, segment
 * classes and slots equal those of a freshly created allocator. */
int gal_trim(gal_handle *h, void *stream);

/* Batched form: the same results contract as gal_malloc_per_thread /
 * gal_free_per_thread.  Mallocs run one request per thread in a kernel
 * compiled for four CTAs of 256 threads per SM, warp teams claiming with one
 * atomicAdd per team; frees take four entries per thread on a persistent
 * grid, look the segment classes up in a copy staged in shared memory, and
 * form warp teams per block (one free-counter atomic per team). */
int gal_malloc_batched(gal_handle *h, const uint64_t *sizes, uint64_t n,
                       void **out_ptrs, void *stream);
int gal_free_batched(gal_handle *h, void *const *ptrs, uint64_t n, void *stream);
/* gal_free_batched over the first *d_count entries of ptrs (at most max_n),
 * where d_count is device memory written by earlier work on the same stream:
 * a kernel that compacts the pointers it wants freed need not send the count
 * back to the host first. */
int gal_free_batched_n(gal_handle *h, void *const *ptrs, const unsigned long long *d_count,
                       uint64_t max_n, void *stream);

/* ---- served jobs (request loop, gallatin_gb300/serve.py) -------------------
 * One job = a grid of gal_job_ctas(kind, n) CTAs launched on `stream` that
 * allocate through the device allocator: GAL_JOB_VECTOR grows device vectors
 * of uint32 by capacity doubling (the reference's
 * data_structs/single_vector.cuh:86-143 growth), CTA b of G over elements
 * [b n / G, (b + 1) n / G); GAL_JOB_QUEUE runs n enqueue/dequeue operations
 * on queues of 32 B nodes.  result (device u64[3], zeroed by the caller):
 * checksum, mallocs+frees, failed mallocs.  hist (device
 * u64[2 * GAL_JOB_LAT_BINS] or NULL): the job adds the latency of each of its
 * mallocs (bins 0..GAL_JOB_LAT_BINS-1) and frees (the next GAL_JOB_LAT_BINS),
 * in SM cycles measured with clock64 around the call; c cycles fall in bin c
 * for c < 4, else in bin 4 floor(log2 c) + ((c >> (floor(log2 c) - 2)) & 3),
 * the last bin taking everything above. */
#define GAL_JOB_VECTOR 0u
#define GAL_JOB_QUEUE 1u
#define GAL_JOB_LAT_BINS 160
uint32_t gal_job_ctas(uint32_t kind, uint64_t n);
int gal_job_launch(gal_handle *h, uint32_t kind, uint64_t job_id, uint64_t n,
                   unsigned long long *result, unsigned long long *hist, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GALLATIN_GB300_H */
