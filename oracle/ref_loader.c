/*
 * ref_loader.c — host side of the reference harness (TEST INFRASTRUCTURE ONLY).
 *
 * Loads oracle/_ref/ref_harness*.cubin (the reference's own device code compiled
 * from its sources, one cubin per segment size) through the CUDA driver API and
 * exposes a small C ABI used by oracle/refgpu.py: build + boot an instance,
 * replay a serial trace, export the state in the gal_state_view layout, serve
 * request batches, and time the churn / stamp workloads.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gallatin_gb300.h"

#define CK(x)                                                              \
  do {                                                                     \
    CUresult _r = (x);                                                     \
    if (_r != CUDA_SUCCESS) {                                              \
      const char *_s = NULL;                                               \
      cuGetErrorString(_r, &_s);                                           \
      fprintf(stderr, "ref_loader: %s failed: %s\n", #x, _s ? _s : "?");   \
      return -(int)_r - 1000;                                              \
    }                                                                      \
  } while (0)

static CUcontext g_ctx;
static int g_init = 0;

/* the churn's counters, four of them each in STAT_SHARDS copies one sector
 * apart (the layout of galwl::stat_word in gallatin_gb300/csrc/churn.cuh) */
#define STAT_SHARDS 64
#define STAT_BYTES (STAT_SHARDS * 4 * 4 * 8)
static void stat_totals(const unsigned long long *buf, unsigned long long *out4) {
  for (int which = 0; which < 4; which++) {
    unsigned long long t = 0;
    for (int sh = 0; sh < STAT_SHARDS; sh++) t += buf[(sh * 4 + which) * 4];
    out4[which] = t;
  }
}

/* one loaded cubin: the reference built for one Gallatin<seg, min, max> */
typedef struct {
  char path[1024];
  CUmodule mod;
  unsigned free_grid; /* persistent grid of ref_churn_free: SMs x resident CTAs */
  uint64_t seg_bytes, min_size, max_size;
  CUfunction f_build, f_boot1, f_bootr, f_replay, f_replay_warp, f_export, f_cmalloc, f_cfree, f_smalloc,
      f_sfree, f_malloc_n, f_free_n;
} ref_mod;

#define MAX_MODS 4
static ref_mod g_mods[MAX_MODS];
static int g_nmods = 0;

typedef struct {
  const ref_mod *m;
  CUdeviceptr arena, scratch, alloc_ptr_buf, status;
  uint64_t num_bytes, scratch_bytes;
  CUdeviceptr alloc; /* device address of the Gallatin object */
} ref_inst;

/* Loads a harness cubin (once per path); returns its module id (>= 0) or a
 * negative error. */
int ref_open(const char *cubin) {
  for (int i = 0; i < g_nmods; i++)
    if (strcmp(g_mods[i].path, cubin) == 0) return i;
  if (g_nmods == MAX_MODS || strlen(cubin) >= sizeof(g_mods[0].path)) return -1;
  CUdevice d;
  if (!g_init) {
    CK(cuInit(0));
    CK(cuDeviceGet(&d, 0));
    CK(cuDevicePrimaryCtxRetain(&g_ctx, d));
    g_init = 1;
  }
  CK(cuCtxSetCurrent(g_ctx));
  CK(cuDeviceGet(&d, 0));
  ref_mod *m = &g_mods[g_nmods];
  memset(m, 0, sizeof(*m));
  strcpy(m->path, cubin);
  CK(cuModuleLoad(&m->mod, cubin));
  CK(cuModuleGetFunction(&m->f_build, m->mod, "ref_build"));
  CK(cuModuleGetFunction(&m->f_boot1, m->mod, "ref_boot_one_thread"));
  CK(cuModuleGetFunction(&m->f_bootr, m->mod, "ref_boot_racy"));
  CK(cuModuleGetFunction(&m->f_replay, m->mod, "ref_replay"));
  CK(cuModuleGetFunction(&m->f_replay_warp, m->mod, "ref_replay_warp"));
  CK(cuModuleGetFunction(&m->f_export, m->mod, "ref_export"));
  CK(cuModuleGetFunction(&m->f_cmalloc, m->mod, "ref_churn_malloc"));
  CK(cuModuleGetFunction(&m->f_cfree, m->mod, "ref_churn_free"));
  CK(cuModuleGetFunction(&m->f_smalloc, m->mod, "ref_stamp_malloc"));
  CK(cuModuleGetFunction(&m->f_sfree, m->mod, "ref_stamp_free"));
  CK(cuModuleGetFunction(&m->f_malloc_n, m->mod, "ref_malloc_sizes"));
  CK(cuModuleGetFunction(&m->f_free_n, m->mod, "ref_free_ptrs"));
  {
    CUdeviceptr gp;
    size_t gb = 0;
    uint64_t geo[3];
    CK(cuModuleGetGlobal(&gp, &gb, m->mod, "ref_geometry"));
    if (gb != sizeof(geo)) return -2;
    CK(cuMemcpyDtoH(geo, gp, sizeof(geo)));
    m->seg_bytes = geo[0];
    m->min_size = geo[1];
    m->max_size = geo[2];
  }
  {
    int sms = 0, per_sm = 0;
    CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, d));
    CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, m->f_cfree, 256, 0));
    m->free_grid = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
  }
  return g_nmods++;
}

/* the geometry a module was built for: bytes per segment, min and max slice */
int ref_module_geometry(int mod, uint64_t *out3) {
  if (mod < 0 || mod >= g_nmods || !out3) return -1;
  out3[0] = g_mods[mod].seg_bytes;
  out3[1] = g_mods[mod].min_size;
  out3[2] = g_mods[mod].max_size;
  return 0;
}

static int launch(CUfunction f, unsigned grid, unsigned block, void **args) {
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, 0, args, NULL));
  return 0;
}

/* boot_mode: 0 none, 1 one-thread order, 2 the reference's racy <<<1,128>>> */
int ref_create(int mod, uint64_t num_bytes, uint64_t seed, int boot_mode, void **out) {
  if (mod < 0 || mod >= g_nmods) return -1;
  const ref_mod *m = &g_mods[mod];
  CK(cuCtxSetCurrent(g_ctx));
  uint64_t S = num_bytes / m->seg_bytes;
  if (S == 0) return -2;
  const uint64_t bps = m->seg_bytes / (m->min_size * 4096);
  ref_inst *r = (ref_inst *)calloc(1, sizeof(ref_inst));
  r->m = m;
  r->num_bytes = num_bytes;
  /* Block (8 B) and queue entry (8 B) per block, plus trees and slots */
  r->scratch_bytes = S * bps * 16 + (8ULL << 20);
  CK(cuMemAlloc(&r->arena, S * m->seg_bytes));
  CK(cuMemsetD8(r->arena, 0, S * m->seg_bytes));
  CK(cuMemAlloc(&r->scratch, r->scratch_bytes));
  CK(cuMemAlloc(&r->alloc_ptr_buf, 8));
  CK(cuMemAlloc(&r->status, 16));
  void *args[] = {&r->scratch, &r->scratch_bytes, &r->arena, &num_bytes, &seed, &r->alloc_ptr_buf,
                  &r->status};
  int e = launch(m->f_build, 1, 1, args);
  if (e) return e;
  CK(cuCtxSynchronize());
  uint64_t st[2];
  CK(cuMemcpyDtoH(st, r->status, 16));
  if (st[0] != 0) {
    fprintf(stderr, "ref_loader: scratch too small (%llu used)\n", (unsigned long long)st[1]);
    return -3;
  }
  CK(cuMemcpyDtoH(&r->alloc, r->alloc_ptr_buf, 8));
  if (boot_mode == 1) {
    void *a2[] = {&r->alloc};
    e = launch(m->f_boot1, 1, 1, a2);
    if (e) return e;
  } else if (boot_mode == 2) {
    void *a2[] = {&r->alloc};
    e = launch(m->f_bootr, 1, 128, a2);
    if (e) return e;
  }
  CK(cuCtxSynchronize());
  *out = r;
  return 0;
}

uint64_t ref_arena_base(void *h) { return (uint64_t)((ref_inst *)h)->arena; }

int ref_destroy(void *h) {
  ref_inst *r = (ref_inst *)h;
  if (!r) return 0;
  CK(cuCtxSynchronize());
  CK(cuMemFree(r->arena));
  CK(cuMemFree(r->scratch));
  CK(cuMemFree(r->alloc_ptr_buf));
  CK(cuMemFree(r->status));
  free(r);
  return 0;
}

int ref_replay(void *h, const uint64_t *ops, uint64_t n, uint64_t *out, uint32_t *smid) {
  ref_inst *r = (ref_inst *)h;
  CUdeviceptr d_ops, d_out, d_smid;
  CK(cuMemAlloc(&d_ops, n * 8 + 8));
  CK(cuMemAlloc(&d_out, n * 8 + 8));
  CK(cuMemAlloc(&d_smid, 8));
  CK(cuMemcpyHtoD(d_ops, ops, n * 8));
  CK(cuMemsetD8(d_out, 0xFF, n * 8));
  void *args[] = {&r->alloc, &d_ops, &n, &d_out, &d_smid};
  int e = launch(r->m->f_replay, 1, 1, args);
  if (e) return e;
  CK(cuCtxSynchronize());
  CK(cuMemcpyDtoH(out, d_out, n * 8));
  CK(cuMemcpyDtoH(smid, d_smid, 4));
  CK(cuMemFree(d_ops));
  CK(cuMemFree(d_out));
  CK(cuMemFree(d_smid));
  return 0;
}

/* warp trace: nsteps x 33 words in, nsteps x 32 offsets out, one warp */
int ref_replay_warp(void *h, const uint64_t *steps, uint64_t nsteps, uint64_t *out, uint32_t *smid) {
  ref_inst *r = (ref_inst *)h;
  CUdeviceptr d_steps, d_out, d_smid;
  CK(cuMemAlloc(&d_steps, nsteps * 33 * 8 + 8));
  CK(cuMemAlloc(&d_out, nsteps * 32 * 8 + 8));
  CK(cuMemAlloc(&d_smid, 8));
  CK(cuMemcpyHtoD(d_steps, steps, nsteps * 33 * 8));
  CK(cuMemsetD8(d_out, 0xFF, nsteps * 32 * 8));
  void *args[] = {&r->alloc, &d_steps, &nsteps, &d_out, &d_smid};
  int e = launch(r->m->f_replay_warp, 1, 32, args);
  if (e) return e;
  CK(cuCtxSynchronize());
  CK(cuMemcpyDtoH(out, d_out, nsteps * 32 * 8));
  CK(cuMemcpyDtoH(smid, d_smid, 4));
  CK(cuMemFree(d_steps));
  CK(cuMemFree(d_out));
  CK(cuMemFree(d_smid));
  return 0;
}

struct export_ptrs {
  CUdeviceptr seg_tree_words, sub_tree_words, tree_ids, active_counts, queue_counters,
      queue_free_counters, final_queue_free_counters, malloc_counters, free_counters, queues, slots,
      locks;
  uint64_t veb_words;
};

int ref_export(void *h, const gal_state_dims *d, gal_state_view *v) {
  ref_inst *r = (ref_inst *)h;
  uint64_t S = d->num_segments, nb = S * d->blocks_per_segment, W = d->veb_words,
           T = d->num_trees;
  struct export_ptrs p;
  memset(&p, 0, sizeof(p));
  CK(cuMemAlloc(&p.seg_tree_words, W * 8));
  CK(cuMemAlloc(&p.sub_tree_words, T * W * 8));
  CK(cuMemAlloc(&p.tree_ids, S * 2 + 8));
  CK(cuMemAlloc(&p.active_counts, S * 4));
  CK(cuMemAlloc(&p.queue_counters, S * 4));
  CK(cuMemAlloc(&p.queue_free_counters, S * 4));
  CK(cuMemAlloc(&p.final_queue_free_counters, S * 4));
  CK(cuMemAlloc(&p.malloc_counters, nb * 4));
  CK(cuMemAlloc(&p.free_counters, nb * 4));
  CK(cuMemAlloc(&p.queues, nb * 4));
  CK(cuMemAlloc(&p.slots, (uint64_t)d->total_slots * 4 + 4));
  CK(cuMemAlloc(&p.locks, 8));
  p.veb_words = W;
  void *args[] = {&r->alloc, &p};
  int e = launch(r->m->f_export, 152, 256, args);
  if (e) return e;
  CK(cuCtxSynchronize());
  CK(cuMemcpyDtoH(v->seg_tree_words, p.seg_tree_words, W * 8));
  CK(cuMemcpyDtoH(v->sub_tree_words, p.sub_tree_words, T * W * 8));
  CK(cuMemcpyDtoH(v->tree_ids, p.tree_ids, S * 2));
  CK(cuMemcpyDtoH(v->active_counts, p.active_counts, S * 4));
  CK(cuMemcpyDtoH(v->queue_counters, p.queue_counters, S * 4));
  CK(cuMemcpyDtoH(v->queue_free_counters, p.queue_free_counters, S * 4));
  CK(cuMemcpyDtoH(v->final_queue_free_counters, p.final_queue_free_counters, S * 4));
  CK(cuMemcpyDtoH(v->malloc_counters, p.malloc_counters, nb * 4));
  CK(cuMemcpyDtoH(v->free_counters, p.free_counters, nb * 4));
  CK(cuMemcpyDtoH(v->queues, p.queues, nb * 4));
  CK(cuMemcpyDtoH(v->slots, p.slots, (uint64_t)d->total_slots * 4));
  uint32_t locks;
  CK(cuMemcpyDtoH(&locks, p.locks, 4));
  v->locks = locks;
  v->error_word = 0;
  CUdeviceptr *all = &p.seg_tree_words;
  for (int i = 0; i < 12; i++) CK(cuMemFree(all[i]));
  return 0;
}

/* the free phase is persistent: one warp per 1,024 slots at a time (churn.cuh) */
static unsigned free_grid(const ref_mod *m, uint64_t nscan) {
  uint64_t need = (nscan + 8 * 1024 - 1) / (8 * 1024);
  return (unsigned)(need < m->free_grid ? need : m->free_grid);
}

/* Mixed-size churn, `steps` timed steps after `warmup` untimed ones.  One step:
 * rounds x (50% coin frees of live slots before every round but the first,
 * then threads_per_round mallocs), then a drain of every live slot.
 * out_ms[i] = duration of timed step i; stats (4 x u64) summed over timed steps. */
int ref_churn(void *h, uint64_t threads_per_round, uint32_t rounds, uint32_t seed, int warmup,
              int steps, float *out_ms, unsigned long long *stats_out) {
  ref_inst *r = (ref_inst *)h;
  uint64_t nslots = threads_per_round * rounds;
  /* rounds are whole warps of liveness words and coin groups (churn.cuh SLOT_ALIGN) */
  if (threads_per_round % 128) return -2;
  CUdeviceptr ptrs, live, stats;
  CK(cuMemAlloc(&ptrs, nslots * 8));
  CK(cuMemsetD8(ptrs, 0, nslots * 8));
  CK(cuMemAlloc(&live, nslots / 8));
  CK(cuMemsetD8(live, 0, nslots / 8));
  CK(cuMemAlloc(&stats, STAT_BYTES));
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  unsigned block = 256;
  memset(stats_out, 0, 4 * sizeof(unsigned long long));
  unsigned long long *hbuf = (unsigned long long *)malloc(STAT_BYTES);
  for (int s = 0; s < warmup + steps; s++) {
    CK(cuMemsetD8(stats, 0, STAT_BYTES));
    CK(cuCtxSynchronize());
    CK(cuEventRecord(e0, 0));
    for (uint32_t rd = 0; rd < rounds; rd++) {
      if (rd > 0) {
        uint64_t nscan = threads_per_round * rd;
        int all = 0;
        void *fa[] = {&r->alloc, &ptrs, &live, &nscan, &rd, &seed, &all, &stats};
        int e = launch(r->m->f_cfree, free_grid(r->m, nscan), block, fa);
        if (e) return e;
      }
      uint64_t base = threads_per_round * rd;
      void *ma[] = {&r->alloc, &ptrs, &live, &base, &threads_per_round, &seed, &stats};
      int e = launch(r->m->f_cmalloc, (unsigned)((threads_per_round + block - 1) / block), block, ma);
      if (e) return e;
    }
    {
      int all = 1;
      uint32_t rd = rounds;
      void *fa[] = {&r->alloc, &ptrs, &live, &nslots, &rd, &seed, &all, &stats};
      int e = launch(r->m->f_cfree, free_grid(r->m, nslots), block, fa);
      if (e) return e;
    }
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float ms = 0;
    CK(cuEventElapsedTime(&ms, e0, e1));
    if (s >= warmup) {
      out_ms[s - warmup] = ms;
      unsigned long long st[4];
      CK(cuMemcpyDtoH(hbuf, stats, STAT_BYTES));
      stat_totals(hbuf, st);
      for (int i = 0; i < 4; i++) stats_out[i] += st[i];
    }
  }
  free(hbuf);
  CK(cuEventDestroy(e0));
  CK(cuEventDestroy(e1));
  CK(cuMemFree(ptrs));
  CK(cuMemFree(live));
  CK(cuMemFree(stats));
  return 0;
}

/* n threads x malloc(size) with a tid stamp, then check + free (global_test.cu).
 * out_ms[0] malloc kernel, out_ms[1] free kernel; stats as ref_churn. */
int ref_stamp(void *h, uint64_t n, uint64_t size, int rounds, float *out_ms,
              unsigned long long *stats_out) {
  ref_inst *r = (ref_inst *)h;
  CUdeviceptr ptrs, stats;
  CK(cuMemAlloc(&ptrs, n * 8));
  CK(cuMemsetD8(ptrs, 0, n * 8));
  CK(cuMemAlloc(&stats, STAT_BYTES));
  CK(cuMemsetD8(stats, 0, STAT_BYTES));
  CUevent e0, e1, e2;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e2, CU_EVENT_DEFAULT));
  unsigned block = 256;
  unsigned grid = (unsigned)((n + block - 1) / block);
  out_ms[0] = out_ms[1] = 0;
  for (int i = 0; i < rounds; i++) {
    void *ma[] = {&r->alloc, &n, &size, &ptrs, &stats};
    void *fa[] = {&r->alloc, &n, &ptrs, &stats};
    CK(cuEventRecord(e0, 0));
    int e = launch(r->m->f_smalloc, grid, block, ma);
    if (e) return e;
    CK(cuEventRecord(e1, 0));
    e = launch(r->m->f_sfree, grid, block, fa);
    if (e) return e;
    CK(cuEventRecord(e2, 0));
    CK(cuEventSynchronize(e2));
    float a = 0, b = 0;
    CK(cuEventElapsedTime(&a, e0, e1));
    CK(cuEventElapsedTime(&b, e1, e2));
    out_ms[0] += a;
    out_ms[1] += b;
  }
  {
    unsigned long long *hbuf = (unsigned long long *)malloc(STAT_BYTES);
    CK(cuMemcpyDtoH(hbuf, stats, STAT_BYTES));
    stat_totals(hbuf, stats_out);
    free(hbuf);
  }
  CK(cuMemFree(ptrs));
  CK(cuMemFree(stats));
  return 0;
}

/* One device thread per request: out[i] = malloc(sizes[i]) through the
 * reference's per-thread malloc; host arrays in and out.  *ms: kernel time
 * (CUDA events around the launch). */
int ref_malloc_sizes(void *h, const uint64_t *sizes, uint64_t n, uint64_t *out, float *ms) {
  ref_inst *r = (ref_inst *)h;
  if (!n) return 0;
  CUdeviceptr d_sizes, d_out;
  CK(cuMemAlloc(&d_sizes, n * 8));
  CK(cuMemAlloc(&d_out, n * 8));
  CK(cuMemcpyHtoD(d_sizes, sizes, n * 8));
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  void *args[] = {&r->alloc, &d_sizes, &n, &d_out};
  CK(cuEventRecord(e0, 0));
  int e = launch(r->m->f_malloc_n, (unsigned)((n + 255) / 256), 256, args);
  if (e) return e;
  CK(cuEventRecord(e1, 0));
  CK(cuEventSynchronize(e1));
  CK(cuEventElapsedTime(ms, e0, e1));
  CK(cuMemcpyDtoH(out, d_out, n * 8));
  CK(cuEventDestroy(e0));
  CK(cuEventDestroy(e1));
  CK(cuMemFree(d_sizes));
  CK(cuMemFree(d_out));
  return 0;
}

/* One device thread per pointer: free(ptrs[i]) unless 0; host array in. */
int ref_free_ptrs(void *h, const uint64_t *ptrs, uint64_t n, float *ms) {
  ref_inst *r = (ref_inst *)h;
  if (!n) return 0;
  CUdeviceptr d_ptrs;
  CK(cuMemAlloc(&d_ptrs, n * 8));
  CK(cuMemcpyHtoD(d_ptrs, ptrs, n * 8));
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  void *args[] = {&r->alloc, &d_ptrs, &n};
  CK(cuEventRecord(e0, 0));
  int e = launch(r->m->f_free_n, (unsigned)((n + 255) / 256), 256, args);
  if (e) return e;
  CK(cuEventRecord(e1, 0));
  CK(cuEventSynchronize(e1));
  CK(cuEventElapsedTime(ms, e0, e1));
  CK(cuEventDestroy(e0));
  CK(cuEventDestroy(e1));
  CK(cuMemFree(d_ptrs));
  return 0;
}
