// gallatin/allocators/global_allocator.cuh — drop-in for the reference's
// global allocator API (chillenzer/gallatin
// include/gallatin/allocators/global_allocator.cuh:41-357): global_gallatin,
// init_global_allocator, free_global_allocator, global_malloc, global_free,
// print_global_stats; the host-backed instance (global_host_gallatin and its
// *_host functions), the combined and fused (device first, then host) entry
// points, and the poisoned-allocation debug API, in namespace
// gallatin::allocators.
//
// The reference declares `__device__ inline global_gallatin`, which nvcc 13
// accepts only with -rdc=true.  Here the handle is a per-translation-unit
// `static __device__` unless GALLATIN_GLOBAL_RDC is defined (then it is the
// reference's `__device__ inline` and needs -rdc=true).  With the default,
// call init_global_allocator in the translation unit whose kernels use
// global_malloc/global_free.  The instance itself is the process-global one
// of the C ABI (gal_init / gal_teardown).
//
// A handle that was never set in this translation unit, or was cleared by
// free_global_allocator, is null: global_malloc then returns nullptr (the
// reference's failure value, global_allocator.cuh:72-76) and global_free does
// nothing, instead of dereferencing the null handle.
#pragma once

#include "gallatin.cuh"

namespace gallatin {
namespace allocators {

using global_allocator_type = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;

#ifdef GALLATIN_GLOBAL_RDC
__device__ inline global_allocator_type *global_gallatin;
__device__ inline global_allocator_type *global_host_gallatin;
#else
static __device__ global_allocator_type *global_gallatin;
static __device__ global_allocator_type *global_host_gallatin;
#endif

__host__ inline void init_global_allocator(uint64_t num_bytes, uint64_t seed, bool print_info = true,
                                           bool running_calloc = false) {
  gal_config cfg = global_allocator_type::config();
  cfg.zero_fill = running_calloc ? 1u : 0u;  // calloc mode: allocations handed out zeroed
  int rc = gal_init(num_bytes, seed, &cfg);
  if (rc != GAL_OK) {
    fprintf(stderr, "Gallatin: init_global_allocator failed with status %d\n", rc);
    return;
  }
  global_allocator_type *local_copy = (global_allocator_type *)gal_device_state(gal_global());
  cudaMemcpyToSymbol(global_gallatin, &local_copy, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (print_info)
    printf("Booted Gallatin with %d trees in range 16-4096 and %f GB of memory %llu segments\n",
           global_allocator_type::get_num_trees(), 1.0 * num_bytes / 1024 / 1024 / 1024,
           (unsigned long long)(num_bytes >> 24));
}

__host__ inline void free_global_allocator() {
  global_allocator_type *null_copy = nullptr;
  cudaDeviceSynchronize();
  gal_teardown();
  cudaMemcpyToSymbol(global_gallatin, &null_copy, sizeof(global_allocator_type *));
}

__device__ __forceinline__ void *global_malloc(uint64_t num_bytes) {
  global_allocator_type *a = global_gallatin;
  return a ? a->malloc(num_bytes) : nullptr;
}

__device__ __forceinline__ void global_free(void *ptr) {
  global_allocator_type *a = global_gallatin;
  if (a) a->free(ptr);
}

__host__ inline void print_global_stats() {
  gal_handle *h = gal_global();
  if (h) gal_print_stats(h);
}

// ---- the host-backed instance (global_allocator.cuh:100-150): its arena is
// pinned host memory mapped into the device's address space

__host__ inline void init_global_allocator_host(uint64_t num_bytes, uint64_t seed, bool print_info = true,
                                                bool running_calloc = false) {
  gal_config cfg = global_allocator_type::config();
  cfg.zero_fill = running_calloc ? 1u : 0u;  // calloc mode: allocations handed out zeroed
  int rc = gal_init_host(num_bytes, seed, &cfg);
  if (rc != GAL_OK) {
    fprintf(stderr, "Gallatin: init_global_allocator_host failed with status %d\n", rc);
    return;
  }
  global_allocator_type *local_copy = (global_allocator_type *)gal_device_state(gal_global_host());
  cudaMemcpyToSymbol(global_host_gallatin, &local_copy, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (print_info)
    printf("Booted Gallatin with %d trees in range 16-4096 and %f GB of host memory %llu segments\n",
           global_allocator_type::get_num_trees(), 1.0 * num_bytes / 1024 / 1024 / 1024,
           (unsigned long long)(num_bytes >> 24));
}

__host__ inline void free_global_allocator_host() {
  global_allocator_type *null_copy = nullptr;
  cudaDeviceSynchronize();
  gal_teardown_host();
  cudaMemcpyToSymbol(global_host_gallatin, &null_copy, sizeof(global_allocator_type *));
}

__device__ __forceinline__ void *global_malloc_host(uint64_t num_bytes) {
  global_allocator_type *a = global_host_gallatin;
  return a ? a->malloc(num_bytes) : nullptr;
}

__device__ __forceinline__ void global_free_host(void *ptr) {
  global_allocator_type *a = global_host_gallatin;
  if (a) a->free(ptr);
}

__host__ inline void print_global_stats_host() {
  gal_handle *h = gal_global_host();
  if (h) gal_print_stats(h);
}

// ---- both instances (global_allocator.cuh:152-232)

__host__ inline void init_global_allocator_combined(uint64_t num_bytes, uint64_t host_bytes, uint64_t seed,
                                                    bool print_info = true, bool running_calloc = false) {
  init_global_allocator(num_bytes, seed, print_info, running_calloc);
  init_global_allocator_host(host_bytes, seed, print_info, running_calloc);
}

__host__ inline void free_global_allocator_combined() {
  free_global_allocator();
  free_global_allocator_host();
}

__device__ __forceinline__ void *global_malloc_combined(uint64_t num_bytes, bool on_host = false) {
  return on_host ? global_malloc_host(num_bytes) : global_malloc(num_bytes);
}

__device__ __forceinline__ void global_free_combined(void *ptr, bool on_host = false) {
  if (on_host) global_free_host(ptr);
  else global_free(ptr);
}

// device memory first, host memory when the device arena cannot serve the
// request; pointers stay where they were placed until freed
__device__ __forceinline__ void *global_malloc_fused(uint64_t num_bytes) {
  void *p = global_malloc(num_bytes);
  return p ? p : global_malloc_host(num_bytes);
}

__device__ __forceinline__ void global_free_fused(void *ptr) {
  global_allocator_type *a = global_gallatin;
  if (a && a->owns_allocation(ptr)) global_free(ptr);
  else global_free_host(ptr);
}

__host__ inline void print_global_stats_combined() {
  printf("Device Allocator:\n");
  print_global_stats();
  printf("Host Allocator:\n");
  print_global_stats_host();
}

// ---- poisoned allocations (global_allocator.cuh:236-357): the 16 bytes
// before the user region record (bytes requested, padding); the padding after
// the region holds 0, 1, 2, ... and the 16 bytes after it repeat the record.

__device__ inline void *global_malloc_poison(uint64_t bytes_needed) {
  global_allocator_type *a = global_gallatin;
  if (!a) return nullptr;
  const uint64_t total = a->get_allocated_size(bytes_needed + 32);
  const uint64_t extra = total - (bytes_needed + 32);
  char *base = (char *)a->malloc(bytes_needed + 32);
  if (!base) return nullptr;
  uint64_t *head = (uint64_t *)base;
  uint64_t *tail = (uint64_t *)(base + 16 + bytes_needed + extra);
  char *pad = base + 16 + bytes_needed;
  for (uint64_t i = 0; i < extra; i++) pad[i] = (char)i;
  atomicExch((unsigned long long *)&head[0], (unsigned long long)bytes_needed);
  atomicExch((unsigned long long *)&head[1], (unsigned long long)extra);
  atomicExch((unsigned long long *)&tail[0], (unsigned long long)bytes_needed);
  atomicExch((unsigned long long *)&tail[1], (unsigned long long)extra);
  return base + 16;
}

// true when both records agree and the padding is intact
__device__ inline bool global_check_poison(void *allocation) {
  if (allocation == nullptr) return false;
  const char *user = (const char *)allocation;
  const uint64_t *head = (const uint64_t *)(user - 16);
  const uint64_t bytes_needed = head[0], extra = head[1];
  if ((bytes_needed + extra) % 16 != 0) return false;
  const uint64_t *tail = (const uint64_t *)(user + bytes_needed + extra);
  if (tail[0] != bytes_needed || tail[1] != extra) return false;
  const char *pad = user + bytes_needed;
  for (uint64_t i = 0; i < extra; i++)
    if (pad[i] != (char)i) return false;
  return true;
}

__device__ inline void global_free_poison(void *allocation) {
  if (!global_check_poison(allocation)) printf("Gallatin: poison violated at %p\n", allocation);
  global_free((char *)allocation - 16);
}

}  // namespace allocators
}  // namespace gallatin
