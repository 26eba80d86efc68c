// gal_noalloc.cu — state export that allocates no device memory.
//
// gal_export_state() stages the per-block malloc counters through a device
// buffer it gets from cudaMalloc and gives back with cudaFree, and waits for
// the whole device first.  Some callers cannot do either: a framework whose
// caching allocator has already reserved the device's memory (a fresh
// cudaMalloc can fail even though the allocator's own state is readable), a
// monitor that snapshots the allocator while other streams keep running
// (cudaFree and cudaDeviceSynchronize wait for all of them), or code with a
// fixed device-memory budget.  gal_export_state_noalloc() does the same
// export with its staging area in a fixed array that is part of this
// library's device image, on a stream of its own, and waits for that stream
// only.
//
// Limits and sharing:
//   * the array holds GAL_NOALLOC_MAX_BLOCKS block counters (1 MiB); larger
//     allocators are rejected with GAL_ERR_ARGS and a message;
//   * every GPU that loads the library keeps this 1 MiB until the process exits;
//   * set-up, once per device with that device current: the array's device
//     address is looked up (which loads this file's module, placing the array
//     on the device) and the export's stream is created.  gal_create does it
//     for the device it builds on, so the export itself allocates nothing; a
//     handle's first export on a device that was never set up does it then,
//     and that call should come before any stream capture;
//   * all calls share the one array and it keeps the last call's contents;
//     each call writes every entry it reads back, so nothing needs clearing,
//     but calls that overlap on the GPU (for example from two host threads at
//     once) race on it;
//   * the copies run while other streams may still be changing the state, so
//     a snapshot taken during device malloc/free is not a consistent cut: each
//     word holds some value it had during the call.  With no device work on
//     the allocator in flight it equals gal_export_state's result.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "gal_internal.h"

namespace {

constexpr uint64_t kMaxBlocks = GAL_NOALLOC_MAX_BLOCKS;

static __device__ __align__(256) uint32_t g_export_scratch[kMaxBlocks];

constexpr int kMaxDevices = 64;
struct per_device {
  uint32_t *scratch = nullptr;   // device address of g_export_scratch
  cudaStream_t stream = nullptr; // the export's own non-blocking stream
};
std::mutex g_mu;
per_device g_dev[kMaxDevices];

// per-block malloc counters in the reference packing, written into `out`
__global__ void k_export_blocks_fixed(const gal::state *s, uint32_t *out, uint64_t nblocks) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = i; b < nblocks; b += stride) out[b] = gal::export_mword(s, (uint32_t)b);
}

// set-up for `dev`, which must be current; the caller holds g_mu
int setup_locked(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return GAL_ERR_CUDA;
  per_device &d = g_dev[dev];
  if (!d.scratch) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_export_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "gallatin_gb300: cudaGetSymbolAddress of the export scratch failed: %s\n",
              cudaGetErrorString(e));
      return GAL_ERR_CUDA;
    }
    d.scratch = (uint32_t *)p;
  }
  if (!d.stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      fprintf(stderr, "gallatin_gb300: creating the export stream failed: %s\n", cudaGetErrorString(e));
      d.stream = nullptr;
      return GAL_ERR_CUDA;
    }
  }
  return GAL_OK;
}

#define TRY(x)                                                                         \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if (_e != cudaSuccess) {                                                           \
      fprintf(stderr, "gallatin_gb300: %s failed: %s\n", #x, cudaGetErrorString(_e));  \
      return GAL_ERR_CUDA;                                                             \
    }                                                                                  \
  } while (0)

}  // namespace

int gal_noalloc_setup(int device) {
  std::lock_guard<std::mutex> g(g_mu);
  return setup_locked(device);
}

extern "C" int gal_export_state_noalloc(gal_handle *h, gal_state_view *v) {
  if (!h || !v) return GAL_ERR_ARGS;
  const gal::state &st = *gal_internal_host_state(h);
  const uint64_t S = st.num_segments, nb = S << st.bps_shift, W = st.veb.words, T = st.num_trees;
  if (nb > kMaxBlocks) {
    fprintf(stderr,
            "gallatin_gb300: gal_export_state_noalloc handles at most %llu blocks "
            "(this allocator has %llu); use gal_export_state\n",
            (unsigned long long)kMaxBlocks, (unsigned long long)nb);
    return GAL_ERR_ARGS;
  }
  const int dev = gal_internal_device(h);
  gal_device_guard on_dev(dev);  // the handle's device, whatever the caller's current one
  TRY(on_dev.err);
  per_device d;
  {
    std::lock_guard<std::mutex> g(g_mu);
    int rc = setup_locked(dev);
    if (rc != GAL_OK) return rc;
    d = g_dev[dev];
  }
  const gal::state *d_state = (const gal::state *)gal_device_state(h);
  cudaStream_t s = d.stream;
  const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
  TRY(cudaMemcpyAsync(v->seg_tree_words, st.seg_tree, W * 8, D2H, s));
  TRY(cudaMemcpyAsync(v->sub_tree_words, st.sub_trees, T * W * 8, D2H, s));
  TRY(cudaMemcpyAsync(v->tree_ids, st.tree_ids, S * 2, D2H, s));
  // the low half of each segment's count word (its biased count), then unbiased below
  TRY(cudaMemcpy2DAsync(v->active_counts, 4, st.act, 8, 4, S, D2H, s));
  TRY(cudaMemcpyAsync(v->queue_counters, st.qc, S * 4, D2H, s));
  TRY(cudaMemcpyAsync(v->queue_free_counters, st.qfc, S * 4, D2H, s));
  TRY(cudaMemcpyAsync(v->final_queue_free_counters, st.fqfc, S * 4, D2H, s));
  TRY(cudaMemcpy2DAsync(v->free_counters, 4, st.fctr, (size_t)st.fstride * 4, 4, nb, D2H, s));
  TRY(cudaMemcpyAsync(v->queues, st.queues, nb * 4, D2H, s));
  TRY(cudaMemcpyAsync(v->slots, st.slots, (uint64_t)st.total_slots * 4, D2H, s));
  k_export_blocks_fixed<<<1024, 256, 0, s>>>(d_state, d.scratch, nb);
  TRY(cudaGetLastError());
  TRY(cudaMemcpyAsync(v->malloc_counters, d.scratch, nb * 4, D2H, s));
  uint32_t locks[GAL_MAX_TREES + 1] = {}, err = 0;
  TRY(cudaMemcpy2DAsync(locks, 4, st.locks, gal::LOCK_STRIDE * 4, 4, T + 1, D2H, s));
  TRY(cudaMemcpyAsync(&err, st.error, 4, D2H, s));
  TRY(cudaStreamSynchronize(s));
  for (uint64_t i = 0; i < S; i++) v->active_counts[i] = gal::act_unbias((uint32_t)v->active_counts[i]);
  uint32_t bits = 0;
  for (uint32_t t = 0; t <= T; t++) bits |= locks[t] ? 1u << t : 0u;
  v->locks = bits;
  v->error_word = err;
  return GAL_OK;
}
