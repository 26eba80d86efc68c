// gal_noalloc.cu — state export that allocates no device memory.
//
// gal_export_state() stages the per-block malloc counters through a device
// buffer it gets from cudaMalloc and gives back with cudaFree.  Some callers
// cannot do that: a framework whose caching allocator has already reserved the
// device's memory (a fresh cudaMalloc can fail even though the allocator's own
// state is readable), a monitor that snapshots the allocator while other
// streams keep running (cudaFree waits for the whole device), or code with a
// fixed device-memory budget.  gal_export_state_noalloc() does the same export
// with its staging area in a fixed array that is part of this library's
// device image.
//
// Limits and sharing:
//   * the array holds GAL_NOALLOC_MAX_BLOCKS block counters (1 MiB); larger
//     allocators are rejected with GAL_ERR_ARGS and a message;
//   * every GPU that loads the library keeps this 1 MiB until the process exits;
//   * the first call on a device looks up the array's device address (with
//     that device current) and caches it; make that first call before any
//     stream capture;
//   * all calls share the one array and it keeps the last call's contents;
//     each call writes every entry it reads back, so nothing needs clearing,
//     but calls that overlap on the GPU (for example from two host threads at
//     once) race on it.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"

namespace {

constexpr uint64_t kMaxBlocks = GAL_NOALLOC_MAX_BLOCKS;

static __device__ __align__(256) uint32_t g_export_scratch[kMaxBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t *g_scratch_addr[kMaxDevices] = {};

// per-block malloc counters in the reference packing, written into `out`
__global__ void k_export_blocks_fixed(const gal::state *s, uint32_t *out, uint64_t nblocks) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = i; b < nblocks; b += stride) {
    unsigned long long w = s->mwords[b];
    out[b] = (uint32_t)(((w >> 32) << 20) + (w & 0xFFFFFFFFull));
  }
}

// device address of the scratch array on the current device (looked up once)
int scratch_for_current_device(uint32_t **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GAL_ERR_CUDA;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_export_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "gallatin_gb300: cudaGetSymbolAddress of the export scratch failed: %s\n",
              cudaGetErrorString(e));
      return GAL_ERR_CUDA;
    }
    g_scratch_addr[dev] = (uint32_t *)p;
  }
  *out = g_scratch_addr[dev];
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

extern "C" int gal_export_state_noalloc(gal_handle *h, const gal_state_view *v) {
  if (!h || !v) return GAL_ERR_ARGS;
  gal_state_dims d;
  if (gal_state_dims_get(h, &d) != GAL_OK) return GAL_ERR_ARGS;
  const uint64_t S = d.num_segments, nb = S * d.blocks_per_segment, W = d.veb_words, T = d.num_trees;
  if (nb > kMaxBlocks) {
    fprintf(stderr,
            "gallatin_gb300: gal_export_state_noalloc handles at most %llu blocks "
            "(this allocator has %llu); use gal_export_state\n",
            (unsigned long long)kMaxBlocks, (unsigned long long)nb);
    return GAL_ERR_ARGS;
  }
  uint32_t *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != GAL_OK) return rc;
  const gal::state *d_state = (const gal::state *)gal_device_state(h);
  gal::state st;  // host copy of the device-resident state: array addresses
  TRY(cudaDeviceSynchronize());
  TRY(cudaMemcpy(&st, d_state, sizeof(st), cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->seg_tree_words, st.seg_tree, W * 8, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->sub_tree_words, st.sub_trees, T * W * 8, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->tree_ids, st.tree_ids, S * 2, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->active_counts, st.active, S * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->queue_counters, st.qc, S * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->queue_free_counters, st.qfc, S * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->final_queue_free_counters, st.fqfc, S * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->free_counters, st.fctr, nb * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->queues, st.queues, nb * 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(v->slots, st.slots, (uint64_t)st.total_slots * 4, cudaMemcpyDeviceToHost));
  k_export_blocks_fixed<<<1024, 256>>>(d_state, scratch, nb);
  TRY(cudaGetLastError());
  TRY(cudaMemcpy(v->malloc_counters, scratch, nb * 4, cudaMemcpyDeviceToHost));
  uint32_t locks = 0, err = 0;
  TRY(cudaMemcpy(&locks, st.locks, 4, cudaMemcpyDeviceToHost));
  TRY(cudaMemcpy(&err, st.error, 4, cudaMemcpyDeviceToHost));
  ((gal_state_view *)v)->locks = locks;
  ((gal_state_view *)v)->error_word = err;
  return GAL_OK;
}
