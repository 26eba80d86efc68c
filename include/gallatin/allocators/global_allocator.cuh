// gallatin/allocators/global_allocator.cuh — drop-in for the reference's
// global allocator API (chillenzer/gallatin
// include/gallatin/allocators/global_allocator.cuh:41-97): global_gallatin,
// init_global_allocator, free_global_allocator, global_malloc, global_free,
// print_global_stats, in namespace gallatin::allocators.
//
// The reference declares `__device__ inline global_gallatin`, which nvcc 13
// accepts only with -rdc=true.  Here the handle is a per-translation-unit
// `static __device__` unless GALLATIN_GLOBAL_RDC is defined (then it is the
// reference's `__device__ inline` and needs -rdc=true).  With the default,
// call init_global_allocator in the translation unit whose kernels use
// global_malloc/global_free.  The instance itself is the process-global one
// of the C ABI (gal_init / gal_teardown).
#pragma once

#include "gallatin.cuh"

namespace gallatin {
namespace allocators {

using global_allocator_type = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;

#ifdef GALLATIN_GLOBAL_RDC
__device__ inline global_allocator_type *global_gallatin;
#else
static __device__ global_allocator_type *global_gallatin;
#endif

__host__ inline void init_global_allocator(uint64_t num_bytes, uint64_t seed, bool print_info = true,
                                           bool running_calloc = false) {
  if (running_calloc) {
    fprintf(stderr, "Gallatin: calloc mode (dynamic parallelism) is not provided\n");
    return;
  }
  gal_config cfg = global_allocator_type::config();
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

__device__ __forceinline__ void *global_malloc(uint64_t num_bytes) { return global_gallatin->malloc(num_bytes); }

__device__ __forceinline__ void global_free(void *ptr) { global_gallatin->free(ptr); }

__host__ inline void print_global_stats() {
  gal_handle *h = gal_global();
  if (h) gal_print_stats(h);
}

}  // namespace allocators
}  // namespace gallatin
