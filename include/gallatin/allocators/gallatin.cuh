// gallatin/allocators/gallatin.cuh — drop-in for the reference's
// gallatin::allocators::Gallatin<bytes_per_segment, smallest, biggest>
// (chillenzer/gallatin include/gallatin/allocators/gallatin.cuh:292-2035).
//
// Same namespace, type name, template parameters and member names; the object
// the returned pointer designates is this library's allocator state (device
// memory), built and destroyed through the C ABI of gallatin_gb300.h, so link
// with libgallatin_gb300.so.  Device malloc/free are header-inline.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../gallatin_gb300.h"
#include "../../gallatin_gb300/gal_device.cuh"

namespace gallatin {
namespace allocators {

namespace detail {
__host__ __device__ constexpr bool is_pow2(uint64_t x) { return x && !(x & (x - 1)); }
__host__ __device__ constexpr int log2_exact(uint64_t x) { return x <= 1 ? 0 : 1 + log2_exact(x >> 1); }
}  // namespace detail

template <uint64_t bytes_per_segment, uint64_t smallest, uint64_t biggest>
struct Gallatin {
  using my_type = Gallatin<bytes_per_segment, smallest, biggest>;
  static_assert(bytes_per_segment >= biggest * 4096, "segment must hold one block of the largest slice");
  static_assert(detail::is_pow2(bytes_per_segment) && detail::is_pow2(smallest) && detail::is_pow2(biggest),
                "geometry must be powers of two");
  static_assert(biggest >= smallest, "biggest < smallest");

  gal::state st;  // device-resident allocator state

  static __host__ gal_config config() {
    gal_config cfg;
    gal_config_default(&cfg);
    cfg.bytes_per_segment = bytes_per_segment;
    cfg.min_size = smallest;
    cfg.max_size = biggest;
    return cfg;
  }

  // gallatin.cuh:324.  Returns nullptr (and prints why) if construction fails.
  static __host__ my_type *generate_on_device(uint64_t max_bytes, uint64_t seed, bool print_info = true,
                                              bool running_calloc = false) {
    return generate_with_arena(max_bytes, seed, print_info, running_calloc, GAL_ARENA_DEVICE);
  }

  // gallatin.cuh:427: the arena in pinned host memory mapped into the device's
  // address space; the allocator's metadata stays in device memory
  static __host__ my_type *generate_on_device_host(uint64_t max_bytes, uint64_t seed, bool print_info = true,
                                                   bool running_calloc = false) {
    return generate_with_arena(max_bytes, seed, print_info, running_calloc, GAL_ARENA_HOST);
  }

  // gallatin.cuh:531: the arena in managed memory
  static __host__ my_type *generate_on_device_managed(uint64_t max_bytes, uint64_t seed,
                                                      bool print_info = true, bool running_calloc = false) {
    return generate_with_arena(max_bytes, seed, print_info, running_calloc, GAL_ARENA_MANAGED);
  }

  static __host__ my_type *generate_with_arena(uint64_t max_bytes, uint64_t seed, bool print_info,
                                               bool running_calloc, uint32_t arena_kind) {
    gal_config cfg = config();
    cfg.arena_kind = arena_kind;
    cfg.zero_fill = running_calloc ? 1u : 0u;  // calloc mode: allocations handed out zeroed
    gal_handle *h = nullptr;
    int rc = gal_create(max_bytes, seed, &cfg, &h);
    if (rc != GAL_OK) {
      fprintf(stderr, "Gallatin: construction failed with status %d\n", rc);
      return nullptr;
    }
    if (print_info)
      printf("Booted Gallatin with %d trees in range %llu-%llu and %f GB of memory %llu segments\n",
             get_num_trees(), (unsigned long long)smallest, (unsigned long long)biggest,
             1.0 * max_bytes / 1024 / 1024 / 1024, (unsigned long long)(max_bytes / bytes_per_segment));
    return (my_type *)gal_device_state(h);
  }

  // gallatin.cuh:643
  static __host__ void free_on_device(my_type *dev_version) {
    gal_handle *h = gal_handle_of(dev_version);
    if (h) gal_destroy(h);
  }

  static __host__ __device__ int get_num_trees() {
    return detail::log2_exact(biggest) - detail::log2_exact(smallest) + 1;
  }

  // gallatin.cuh:1186 / :1378
  __device__ __forceinline__ void *malloc(uint64_t size) { return gal::malloc(&st, size); }
  __device__ __forceinline__ void free(void *ptr) { gal::free(&st, ptr); }

  // gallatin.cuh:1152, :2027
  __device__ __forceinline__ uint64_t get_allocated_size(uint64_t bytes_needed) {
    return gal::allocated_size(&st, bytes_needed);
  }
  __device__ __forceinline__ bool owns_allocation(void *alloc) { return gal::owns(&st, alloc); }

  // gallatin.cuh:1855 (called on the device pointer from the host)
  __host__ void print_info() {
    gal_handle *h = gal_handle_of(this);
    if (h) gal_print_stats(h);
  }
};

}  // namespace allocators
}  // namespace gallatin
