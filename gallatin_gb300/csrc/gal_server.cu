// gal_server.cu — the resident allocator server under load: several producer
// streams of uneven request sizes, counts and lifetimes, served through the
// request rings of gal_server.cuh by server CTAs of the same cooperative
// launch, one launch per step (optionally captured as a CUDA graph).  The
// same producers calling the per-thread malloc directly (no server CTAs) give
// the comparison at the same allocator settings.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "../../include/gallatin_gb300.h"
#include "gal_server.cuh"
#include "workload.cuh"

extern "C" {
/* One producer stream: `requests` mallocs of sizes drawn uniformly from
 * [lo, hi] bytes (log-uniformly when log_uniform), each allocation freed
 * `keep` requests of the same lane later (0..4). */
typedef struct gal_server_stream {
  uint64_t requests;
  uint32_t lo, hi;
  uint32_t log_uniform;
  uint32_t keep;
} gal_server_stream;

typedef struct gal_server_result {
  double ms_total;                       /* sum over timed steps (CUDA events) */
  uint64_t mallocs_ok, mallocs_failed, stamp_mismatch, frees, misaligned;
  uint64_t not_zeroed;                   /* zero-fill allocators: first or last word not zero */
  uint32_t status;                       /* SERVER_ERR_* bits seen           */
  uint32_t error_word;                   /* the allocator's device error word */
  uint32_t grid, server_ctas, block;
  int graph;                             /* 1 when the steps ran as a CUDA graph */
} gal_server_result;
}

namespace {

constexpr int MAX_STREAMS = 4;
constexpr int SRV_BT = 256;
constexpr int KEEP_MAX = 4;

// Producer CTAs [begin[i], begin[i + 1]) of the producers serve stream i:
// each stream's share is in proportion to its requests (at least one CTA), as
// a producer kernel per stream would be sized for its own work.  (An equal
// share left the largest stream's lanes with the most requests each, and they
// alone set the step's length.)
struct streams_param {
  gal_server_stream s[MAX_STREAMS];
  uint32_t begin[MAX_STREAMS + 1];
  uint32_t n;
};

__device__ __forceinline__ uint64_t stream_size(const gal_server_stream &st, uint64_t r, uint32_t which) {
  galwl::u32x4 c = {{(uint32_t)r, (uint32_t)(r >> 32), which, 0x5E7Eu}};
  galwl::u32x4 x = galwl::philox4x32_10(c, 0x5EEDu, 0xA11Cu);
  if (st.log_uniform) {  // 2^(log2 lo + u (log2 hi - log2 lo)), u from 24 bits
    const float u = (float)(x.v[0] >> 8) * (1.0f / 16777216.0f);
    const float l0 = __log2f((float)st.lo), l1 = __log2f((float)st.hi);
    uint64_t v = (uint64_t)exp2f(l0 + u * (l1 - l0));
    return v < st.lo ? st.lo : v > st.hi ? st.hi : v;
  }
  return st.lo + (uint64_t)(x.v[0] % (st.hi - st.lo + 1));
}

// stats: [0] mallocs ok [1] failed [2] stamp mismatches [3] frees [4] misaligned
// [5] not zeroed
__device__ __forceinline__ void count(unsigned long long *c, uint32_t v) {
  if (v) atomicAdd(c, (unsigned long long)v);
}

__device__ __forceinline__ bool stamps_ok(const void *p, uint64_t size, uint64_t id) {
  const uint64_t *q = (const uint64_t *)p;
  return q[0] == id && *(const uint64_t *)((const char *)p + ((size - 8) & ~7ull)) == id;
}

__global__ void __launch_bounds__(SRV_BT)
    k_server_step(const gal::state *s, gal::server_rings r, streams_param sp, uint32_t server_ctas, int direct,
                  unsigned long long *stats) {
  __shared__ gal::server_smem sm;
  const uint64_t t0 = gal::global_ns();
  if (blockIdx.x < server_ctas) {
    if (!direct) gal::server_loop(s, r, sm, t0);
    return;
  }
  const uint32_t pc = blockIdx.x - server_ctas;
  uint32_t p = 0;
  while (p + 1 < sp.n && pc >= sp.begin[p + 1]) p++;
  const gal_server_stream st = sp.s[p];
  const uint32_t q = pc - sp.begin[p], cp = sp.begin[p + 1] - sp.begin[p];  // this CTA among its stream's
  const uint32_t wpc = SRV_BT / 32, warp = threadIdx.x / 32, lane = threadIdx.x & 31u;
  const uint64_t slot = (uint64_t)blockIdx.x * SRV_BT + threadIdx.x;  // this lane's reply slot
  const uint64_t chunks = (st.requests + 31) / 32;
  const uint32_t keep = st.keep < KEEP_MAX ? st.keep : KEEP_MAX;
  // the lane's live allocations, oldest at `head`: up to `keep` of them plus
  // the one just made
  constexpr uint32_t RING = KEEP_MAX + 1;
  void *kept[RING];
  uint64_t kept_id[RING], kept_size[RING];
  uint32_t nkept = 0, head = 0;
  uint32_t ok = 0, failed = 0, bad = 0, frees = 0, misaligned = 0, not_zeroed = 0;
  for (uint64_t ch = (uint64_t)q * wpc + warp; ch < chunks; ch += (uint64_t)cp * wpc) {
    const uint64_t rq = ch * 32 + lane;
    if (rq >= st.requests) break;
    const uint64_t size = stream_size(st, rq, p);
    const uint64_t id = ((uint64_t)(p + 1) << 48) | rq;
    void *ptr = direct ? gal::malloc(s, size) : gal::server_malloc(s, r, size, slot, t0);
    if (ptr) {
      ok++;
      // a slice sits on a multiple of its class size, a run of the largest
      // slices on a multiple of the largest slice (streams stay below whole blocks)
      const int bits = gal::ceil_log2(size);
      const uint64_t cls = 1ull << (bits < (int)s->min_shift ? s->min_shift : bits);
      const uint64_t largest = 1ull << (s->min_shift + s->num_trees - 1);
      misaligned += ((uint64_t)((char *)ptr - s->memory) % (cls < largest ? cls : largest)) != 0;
      uint64_t *last = (uint64_t *)((char *)ptr + ((size - 8) & ~7ull));
      if (s->zero_fill) not_zeroed += ((uint64_t *)ptr)[0] != 0ull || *last != 0ull;
      ((uint64_t *)ptr)[0] = id;
      *last = id;
      kept[(head + nkept) % RING] = ptr;
      kept_id[(head + nkept) % RING] = id;
      kept_size[(head + nkept) % RING] = size;
      nkept++;
    } else {
      failed++;
    }
    while (nkept > keep) {  // the lane's oldest allocation goes
      bad += !stamps_ok(kept[head], kept_size[head], kept_id[head]);
      gal::free(s, kept[head]);
      frees++;
      head = (head + 1) % RING;
      nkept--;
    }
  }
  while (nkept) {
    bad += !stamps_ok(kept[head], kept_size[head], kept_id[head]);
    gal::free(s, kept[head]);
    frees++;
    head = (head + 1) % RING;
    nkept--;
  }
  count(&stats[0], ok);
  count(&stats[1], failed);
  count(&stats[2], bad);
  count(&stats[3], frees);
  count(&stats[4], misaligned);
  count(&stats[5], not_zeroed);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicSub(r.producers_left, 1u);
  }
}

__global__ void k_set_u32(uint32_t *p, uint32_t v) { *p = v; }

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t _e = (x);                                                            \
    if (_e != cudaSuccess) {                                                         \
      fprintf(stderr, "gallatin_gb300 server: %s: %s\n", #x, cudaGetErrorString(_e)); \
      rc = GAL_ERR_CUDA;                                                             \
      goto done;                                                                     \
    }                                                                                \
  } while (0)

}  // namespace

extern "C" {

/* Steps of the served workload: every step is one cooperative launch of
 * grid = SMs x resident CTAs, server_pct percent of them (at least one)
 * serving the rings unless `direct`, in which case every CTA is a producer
 * calling the per-thread malloc.  use_graph: the step is captured once as a
 * CUDA graph (falls back to plain launches when the capture is refused, and
 * says so in res->graph).  Every wait inside ends within deadline_ms. */
int gal_bench_server(gal_handle *h, const gal_server_stream *streams, uint32_t nstreams, uint32_t server_pct,
                     int direct, int use_graph, int warmup, int steps, uint32_t deadline_ms, float *step_ms,
                     gal_server_result *res) {
  if (!h || !streams || !res || nstreams == 0 || nstreams > MAX_STREAMS || server_pct > 90 || steps < 0 ||
      warmup < 0)
    return GAL_ERR_ARGS;
  for (uint32_t i = 0; i < nstreams; i++)  // slices and runs of slices only, stamped at both ends
    if (streams[i].lo < 16 || streams[i].hi < streams[i].lo || streams[i].hi > 32768 ||
        streams[i].keep > KEEP_MAX)
      return GAL_ERR_ARGS;
  int rc = GAL_OK;
  memset(res, 0, sizeof(*res));
  const gal::state *d = (const gal::state *)gal_device_state(h);
  gal::state hs;
  streams_param sp;
  memset(&sp, 0, sizeof(sp));
  memcpy(sp.s, streams, nstreams * sizeof(gal_server_stream));
  sp.n = nstreams;
  gal::server_rings r;
  memset(&r, 0, sizeof(r));
  unsigned long long *stats = nullptr, *counters = nullptr;
  uint32_t *flags = nullptr;
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  uint32_t grid = 0, nsrv = 0, prod = 0;
  cudaGetDevice(&dev);
  CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return GAL_ERR_STATE;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_server_step, SRV_BT, 0));
  if (per_sm < 1) return GAL_ERR_STATE;
  grid = (uint32_t)(sms * per_sm);
  nsrv = direct ? 0u : (grid * server_pct + 99) / 100;
  if (!direct && nsrv < 1) nsrv = 1;
  if (nsrv >= grid) return GAL_ERR_ARGS;
  prod = grid - nsrv;
  if (prod < nstreams) return GAL_ERR_ARGS;
  {  // each stream one CTA, the rest in proportion to the requests (largest remainders)
    uint64_t total = 0;
    for (uint32_t i = 0; i < nstreams; i++) total += streams[i].requests;
    uint32_t cnt[MAX_STREAMS], given = 0;
    for (uint32_t i = 0; i < nstreams; i++) {
      cnt[i] = 1u + (uint32_t)(total ? (uint64_t)(prod - nstreams) * streams[i].requests / total : 0);
      given += cnt[i];
    }
    while (given < prod) {  // fewer than nstreams left: to the most requests per CTA
      uint32_t best = 0;
      for (uint32_t i = 1; i < nstreams; i++)
        if ((double)streams[i].requests / cnt[i] > (double)streams[best].requests / cnt[best]) best = i;
      cnt[best]++;
      given++;
    }
    sp.begin[0] = 0;
    for (uint32_t i = 0; i < nstreams; i++) sp.begin[i + 1] = sp.begin[i] + cnt[i];
  }
  CK(cudaMemcpy(&hs, d, sizeof(hs), cudaMemcpyDeviceToHost));
  r.cap_shift = 18;
  // Every producer team's reservation and every server's take hits the
  // classes' tail and taken counters.  One 32-byte sector apart, all 18 fit
  // in five 128-byte lines, so a few L2 slices took all of that traffic: the
  // step ran at 9.6-11.4 ms on three allocators of four, against 7.0-7.9 ms
  // on seven in a row with the counters 4 KiB apart.
  r.ctr_stride = 512u;
  r.deadline_ns = (uint64_t)(deadline_ms ? deadline_ms : 5000) * 1000000ull;
  CK(cudaMalloc(&r.entries, ((uint64_t)hs.num_trees << r.cap_shift) * 8));
  CK(cudaMemset(r.entries, 0, ((uint64_t)hs.num_trees << r.cap_shift) * 8));
  CK(cudaMalloc(&counters, (uint64_t)hs.num_trees * r.ctr_stride * 8 * 2));
  CK(cudaMemset(counters, 0, (uint64_t)hs.num_trees * r.ctr_stride * 8 * 2));
  r.tail = counters;
  r.taken = counters + (uint64_t)hs.num_trees * r.ctr_stride;
  CK(cudaMalloc(&r.reply, (uint64_t)grid * SRV_BT * 8));
  CK(cudaMalloc(&flags, 64));
  CK(cudaMemset(flags, 0, 64));
  r.producers_left = flags;
  r.status = flags + 8;
  CK(cudaMalloc(&stats, 8 * sizeof(unsigned long long)));
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  res->grid = grid;
  res->server_ctas = nsrv;
  res->block = SRV_BT;
  {
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(SRV_BT);
    lc.stream = st;
    lc.attrs = &attr;
    lc.numAttrs = 1;
    int direct_arg = direct;
    auto enqueue = [&]() -> cudaError_t {
      cudaError_t e = cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), st);
      if (e == cudaSuccess) {
        k_set_u32<<<1, 1, 0, st>>>(r.producers_left, prod);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaLaunchKernelEx(&lc, k_server_step, d, r, sp, nsrv, direct_arg, stats);
      return e;
    };
    if (use_graph) {
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t le = enqueue();
        e = cudaStreamEndCapture(st, &graph);
        if (le != cudaSuccess) e = le;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (e != cudaSuccess) {  // the capture was refused: plain launches
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        graph = nullptr;
        exec = nullptr;
      }
    }
    res->graph = exec != nullptr;
    for (int i = 0; i < warmup + steps; i++) {
      CK(cudaStreamSynchronize(st));
      CK(cudaEventRecord(e0, st));
      if (exec)
        CK(cudaGraphLaunch(exec, st));
      else
        CK(enqueue());
      CK(cudaEventRecord(e1, st));
      CK(cudaEventSynchronize(e1));
      CK(cudaGetLastError());
      uint32_t status = 0;
      CK(cudaMemcpy(&status, r.status, 4, cudaMemcpyDeviceToHost));
      res->status |= status;
      if (i >= warmup) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (step_ms) step_ms[i - warmup] = ms;
        res->ms_total += ms;
        unsigned long long sv[8];
        CK(cudaMemcpy(sv, stats, sizeof(sv), cudaMemcpyDeviceToHost));
        res->mallocs_ok += sv[0];
        res->mallocs_failed += sv[1];
        res->stamp_mismatch += sv[2];
        res->frees += sv[3];
        res->misaligned += sv[4];
        res->not_zeroed += sv[5];
      }
      if (status) break;  // a wait ran out: rings may hold unserved entries
    }
  }
  gal_last_error(h, &res->error_word);
done:
  if (st) cudaStreamSynchronize(st);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (r.entries) cudaFree(r.entries);
  if (counters) cudaFree(counters);
  if (r.reply) cudaFree(r.reply);
  if (flags) cudaFree(flags);
  if (stats) cudaFree(stats);
  if (st) cudaStreamDestroy(st);
  return rc;
}

}  // extern "C"
