// Drop-in check: user code written against the reference's API
// (#include <gallatin/allocators/global_allocator.cuh>, global_malloc /
// global_free in kernels, Gallatin<...>::generate_on_device with ->malloc /
// ->free through a handle), compiled unchanged against this library's headers
// and linked with libgallatin_gb300.so.  The kernels follow the reference's
// tests/src/global_test.cu and gallatin_test.cu: every thread allocates,
// stamps its id into the allocation, a second kernel checks the stamp and frees.
#include <gallatin/allocators/global_allocator.cuh>

using namespace gallatin::allocators;

__global__ void insert_one_size(uint64_t num_inserts, uint64_t size, uint64_t **bitarray,
                                unsigned long long *misses) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= num_inserts) return;
  uint64_t *p = (uint64_t *)global_malloc(size);
  bitarray[tid] = p;
  if (p == nullptr) {
    atomicAdd(misses, 1ull);
    return;
  }
  p[0] = tid;
}

__global__ void free_one_size(uint64_t num_allocs, uint64_t **bitarray, unsigned long long *errors) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= num_allocs) return;
  uint64_t *p = bitarray[tid];
  if (p == nullptr) return;
  if (p[0] != tid) atomicAdd(errors, 1ull);
  global_free(p);
}

template <typename allocator_type>
__global__ void handle_malloc(allocator_type *alloc, uint64_t n, uint64_t size, uint64_t **bitarray,
                              unsigned long long *misses) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)alloc->malloc(size);
  bitarray[tid] = p;
  if (p == nullptr) {
    atomicAdd(misses, 1ull);
    return;
  }
  if (!alloc->owns_allocation(p)) atomicAdd(misses + 2, 1ull);
  p[0] = tid;
}

template <typename allocator_type>
__global__ void handle_free(allocator_type *alloc, uint64_t n, uint64_t **bitarray, unsigned long long *errors) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = bitarray[tid];
  if (p == nullptr) return;
  if (p[0] != tid) atomicAdd(errors, 1ull);
  alloc->free(p);
}

// out[0] misses, out[1] stamp errors, out[2] foreign pointers, out[3] device error word
extern "C" int dropin_global_test(uint64_t num_bytes, uint64_t n, uint64_t size, int rounds, uint64_t *out) {
  init_global_allocator(num_bytes, 42, false);
  uint64_t **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(uint64_t *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 511) / 512);
  for (int r = 0; r < rounds; r++) {
    insert_one_size<<<grid, 512>>>(n, size, bits, c);
    free_one_size<<<grid, 512>>>(n, bits, c + 1);
  }
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global(), &err);
  cudaFree(bits);
  cudaFree(c);
  free_global_allocator();
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

extern "C" int dropin_handle_test(uint64_t num_bytes, uint64_t n, uint64_t size, int rounds, uint64_t *out) {
  using gallatin_type = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;
  gallatin_type *alloc = gallatin_type::generate_on_device(num_bytes, 42, false);
  if (!alloc) return 2;
  uint64_t **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(uint64_t *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 511) / 512);
  for (int r = 0; r < rounds; r++) {
    handle_malloc<gallatin_type><<<grid, 512>>>(alloc, n, size, bits, c);
    handle_free<gallatin_type><<<grid, 512>>>(alloc, n, bits, c + 1);
  }
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_handle_of(alloc), &err);
  alloc->print_info();
  cudaFree(bits);
  cudaFree(c);
  gallatin_type::free_on_device(alloc);
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}
