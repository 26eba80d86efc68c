/*
 * ref_loader.c — host side of the reference harness (TEST INFRASTRUCTURE ONLY).
 *
 * Loads oracle/_ref/ref_harness.cubin (the reference's own device code compiled
 * from its sources) through the CUDA driver API and exposes a small C ABI used
 * by oracle/refgpu.py: build + boot an instance, replay a serial trace, export
 * the state in the gal_state_view layout, and time the churn / stamp workloads.
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
static CUmodule g_mod;
static unsigned g_free_grid; /* persistent grid of ref_churn_free: SMs x resident CTAs */
static CUfunction f_build, f_boot1, f_bootr, f_replay, f_replay_warp, f_export, f_cmalloc, f_cfree, f_smalloc, f_sfree;
static int g_open = 0;

typedef struct {
  CUdeviceptr arena, scratch, alloc_ptr_buf, status;
  uint64_t num_bytes, scratch_bytes;
  CUdeviceptr alloc; /* device address of the Gallatin object */
} ref_inst;

int ref_open(const char *cubin) {
  if (g_open) return 0;
  CUdevice d;
  CK(cuInit(0));
  CK(cuDeviceGet(&d, 0));
  CK(cuDevicePrimaryCtxRetain(&g_ctx, d));
  CK(cuCtxSetCurrent(g_ctx));
  CK(cuModuleLoad(&g_mod, cubin));
  CK(cuModuleGetFunction(&f_build, g_mod, "ref_build"));
  CK(cuModuleGetFunction(&f_boot1, g_mod, "ref_boot_one_thread"));
  CK(cuModuleGetFunction(&f_bootr, g_mod, "ref_boot_racy"));
  CK(cuModuleGetFunction(&f_replay, g_mod, "ref_replay"));
  CK(cuModuleGetFunction(&f_replay_warp, g_mod, "ref_replay_warp"));
  CK(cuModuleGetFunction(&f_export, g_mod, "ref_export"));
  CK(cuModuleGetFunction(&f_cmalloc, g_mod, "ref_churn_malloc"));
  CK(cuModuleGetFunction(&f_cfree, g_mod, "ref_churn_free"));
  CK(cuModuleGetFunction(&f_smalloc, g_mod, "ref_stamp_malloc"));
  CK(cuModuleGetFunction(&f_sfree, g_mod, "ref_stamp_free"));
  {
    int sms = 0, per_sm = 0;
    CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, d));
    CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f_cfree, 256, 0));
    g_free_grid = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
  }
  g_open = 1;
  return 0;
}

static int launch(CUfunction f, unsigned grid, unsigned block, void **args) {
  CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, 0, args, NULL));
  return 0;
}

/* boot_mode: 0 none, 1 one-thread order, 2 the reference's racy <<<1,128>>> */
int ref_create(uint64_t num_bytes, uint64_t seed, int boot_mode, void **out) {
  if (!g_open) return -1;
  ref_inst *r = (ref_inst *)calloc(1, sizeof(ref_inst));
  uint64_t S = num_bytes / (16ULL << 20);
  if (S == 0) return -2;
  r->num_bytes = num_bytes;
  r->scratch_bytes = S * 256 * 16 + (8ULL << 20);
  CK(cuMemAlloc(&r->arena, S * (16ULL << 20)));
  CK(cuMemsetD8(r->arena, 0, S * (16ULL << 20)));
  CK(cuMemAlloc(&r->scratch, r->scratch_bytes));
  CK(cuMemAlloc(&r->alloc_ptr_buf, 8));
  CK(cuMemAlloc(&r->status, 16));
  void *args[] = {&r->scratch, &r->scratch_bytes, &r->arena, &num_bytes, &seed, &r->alloc_ptr_buf,
                  &r->status};
  int e = launch(f_build, 1, 1, args);
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
    e = launch(f_boot1, 1, 1, a2);
    if (e) return e;
  } else if (boot_mode == 2) {
    void *a2[] = {&r->alloc};
    e = launch(f_bootr, 1, 128, a2);
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
  int e = launch(f_replay, 1, 1, args);
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
  int e = launch(f_replay_warp, 1, 32, args);
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
  int e = launch(f_export, 152, 256, args);
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
static unsigned free_grid(uint64_t nscan) {
  uint64_t need = (nscan + 8 * 1024 - 1) / (8 * 1024);
  return (unsigned)(need < g_free_grid ? need : g_free_grid);
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
  CK(cuMemAlloc(&stats, 32));
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  unsigned block = 256;
  memset(stats_out, 0, 4 * sizeof(unsigned long long));
  for (int s = 0; s < warmup + steps; s++) {
    CK(cuMemsetD8(stats, 0, 32));
    CK(cuCtxSynchronize());
    CK(cuEventRecord(e0, 0));
    for (uint32_t rd = 0; rd < rounds; rd++) {
      if (rd > 0) {
        uint64_t nscan = threads_per_round * rd;
        int all = 0;
        void *fa[] = {&r->alloc, &ptrs, &live, &nscan, &rd, &seed, &all, &stats};
        int e = launch(f_cfree, free_grid(nscan), block, fa);
        if (e) return e;
      }
      uint64_t base = threads_per_round * rd;
      void *ma[] = {&r->alloc, &ptrs, &live, &base, &threads_per_round, &seed, &stats};
      int e = launch(f_cmalloc, (unsigned)((threads_per_round + block - 1) / block), block, ma);
      if (e) return e;
    }
    {
      int all = 1;
      uint32_t rd = rounds;
      void *fa[] = {&r->alloc, &ptrs, &live, &nslots, &rd, &seed, &all, &stats};
      int e = launch(f_cfree, free_grid(nslots), block, fa);
      if (e) return e;
    }
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float ms = 0;
    CK(cuEventElapsedTime(&ms, e0, e1));
    if (s >= warmup) {
      out_ms[s - warmup] = ms;
      unsigned long long st[4];
      CK(cuMemcpyDtoH(st, stats, 32));
      for (int i = 0; i < 4; i++) stats_out[i] += st[i];
    }
  }
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
  CK(cuMemAlloc(&stats, 32));
  CK(cuMemsetD8(stats, 0, 32));
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
    int e = launch(f_smalloc, grid, block, ma);
    if (e) return e;
    CK(cuEventRecord(e1, 0));
    e = launch(f_sfree, grid, block, fa);
    if (e) return e;
    CK(cuEventRecord(e2, 0));
    CK(cuEventSynchronize(e2));
    float a = 0, b = 0;
    CK(cuEventElapsedTime(&a, e0, e1));
    CK(cuEventElapsedTime(&b, e1, e2));
    out_ms[0] += a;
    out_ms[1] += b;
  }
  CK(cuMemcpyDtoH(stats_out, stats, 32));
  CK(cuMemFree(ptrs));
  CK(cuMemFree(stats));
  return 0;
}
