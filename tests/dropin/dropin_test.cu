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

// ---- host-backed, managed, fused and poisoned allocations
// (global_allocator.cuh:100-357, gallatin.cuh:427-630)

__global__ void host_malloc_stamp(uint64_t n, uint64_t size, uint64_t **bits, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)global_malloc_host(size);
  bits[tid] = p;
  if (!p) {
    atomicAdd(&c[0], 1ull);
    return;
  }
  p[0] = tid;
}

__global__ void host_check_free(uint64_t n, uint64_t **bits, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = bits[tid];
  if (!p) return;
  if (p[0] != tid) atomicAdd(&c[1], 1ull);
  global_free_host(p);
}

// out[0] misses, [1] stamp errors seen on the device, [2] stamps the host read
// wrong through the same pointers, [3] device error word
extern "C" int dropin_host_test(uint64_t host_bytes, uint64_t n, uint64_t size, uint64_t *out) {
  init_global_allocator_host(host_bytes, 42, false);
  if (!gal_global_host()) return 2;
  uint64_t **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(uint64_t *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 255) / 256);
  host_malloc_stamp<<<grid, 256>>>(n, size, bits, c);
  cudaError_t e = cudaDeviceSynchronize();
  // the allocations live in host memory: the host reads the stamps directly
  uint64_t **hb = (uint64_t **)malloc(n * sizeof(uint64_t *));
  cudaMemcpy(hb, bits, n * sizeof(uint64_t *), cudaMemcpyDeviceToHost);
  uint64_t host_bad = 0;
  for (uint64_t i = 0; i < n; i++)
    if (hb[i] && hb[i][0] != i) host_bad++;
  free(hb);
  host_check_free<<<grid, 256>>>(n, bits, c);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global_host(), &err);
  print_global_stats_host();
  cudaFree(bits);
  cudaFree(c);
  free_global_allocator_host();
  out[0] = h[0];
  out[1] = h[1];
  out[2] = host_bad;
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

// managed arena through the handle API; out as dropin_host_test
extern "C" int dropin_managed_test(uint64_t bytes, uint64_t n, uint64_t size, uint64_t *out) {
  using gallatin_type = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;
  gallatin_type *alloc = gallatin_type::generate_on_device_managed(bytes, 42, false);
  if (!alloc) return 2;
  uint64_t **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(uint64_t *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 255) / 256);
  handle_malloc<gallatin_type><<<grid, 256>>>(alloc, n, size, bits, c);
  cudaError_t e = cudaDeviceSynchronize();
  uint64_t **hb = (uint64_t **)malloc(n * sizeof(uint64_t *));
  cudaMemcpy(hb, bits, n * sizeof(uint64_t *), cudaMemcpyDeviceToHost);
  uint64_t host_bad = 0;
  for (uint64_t i = 0; i < n; i++)
    if (hb[i] && hb[i][0] != i) host_bad++;
  free(hb);
  handle_free<gallatin_type><<<grid, 256>>>(alloc, n, bits, c + 1);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_handle_of(alloc), &err);
  cudaFree(bits);
  cudaFree(c);
  gallatin_type::free_on_device(alloc);
  out[0] = h[0];
  out[1] = h[1];
  out[2] = host_bad + h[2];
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

__global__ void fused_malloc(uint64_t n, uint64_t size, uint64_t **bits, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)global_malloc_fused(size);
  bits[tid] = p;
  if (!p) {
    atomicAdd(&c[0], 1ull);
    return;
  }
  if (!global_gallatin->owns_allocation(p)) atomicAdd(&c[2], 1ull);  // served from host memory
  p[0] = tid;
}

__global__ void fused_free(uint64_t n, uint64_t **bits, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = bits[tid];
  if (!p) return;
  if (p[0] != tid) atomicAdd(&c[1], 1ull);
  global_free_fused(p);
}

// device arena too small for all requests: the rest come from host memory.
// out[0] misses, [1] stamp errors, [2] served from host, [3] error words (OR)
extern "C" int dropin_fused_test(uint64_t dev_bytes, uint64_t host_bytes, uint64_t n, uint64_t size,
                                 uint64_t *out) {
  init_global_allocator_combined(dev_bytes, host_bytes, 42, false);
  if (!gal_global() || !gal_global_host()) return 2;
  uint64_t **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(uint64_t *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 255) / 256);
  fused_malloc<<<grid, 256>>>(n, size, bits, c);
  fused_free<<<grid, 256>>>(n, bits, c);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0, err2 = 0;
  gal_last_error(gal_global(), &err);
  gal_last_error(gal_global_host(), &err2);
  print_global_stats_combined();
  cudaFree(bits);
  cudaFree(c);
  free_global_allocator_combined();
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = err | err2;
  return e == cudaSuccess ? 0 : 1;
}

// c[0] poisoned allocations failed, c[1] intact ones reported violated,
// c[2] padding changes not reported, c[3] user-region checks failed
__global__ void poison_roundtrip(uint64_t n, uint64_t bytes, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  char *p = (char *)global_malloc_poison(bytes);
  if (!p) {
    atomicAdd(&c[0], 1ull);
    return;
  }
  for (uint64_t i = 0; i < bytes; i++) p[i] = (char)(tid + i);  // the user region only
  if (!global_check_poison(p)) atomicAdd(&c[1], 1ull);
  // one byte past the user region: inside the allocation's padding
  const uint64_t extra = global_gallatin->get_allocated_size(bytes + 32) - (bytes + 32);
  if (extra > 0) {
    char keep = p[bytes];
    p[bytes] = (char)(keep ^ 0x5A);
    if (global_check_poison(p)) atomicAdd(&c[2], 1ull);
    p[bytes] = keep;
  }
  for (uint64_t i = 0; i < bytes; i++)
    if (p[i] != (char)(tid + i)) {
      atomicAdd(&c[3], 1ull);
      break;
    }
  global_free_poison(p);
}

// out[0..3] as above, out[4] device error word
extern "C" int dropin_poison_test(uint64_t num_bytes, uint64_t n, uint64_t bytes, uint64_t *out) {
  init_global_allocator(num_bytes, 42, false);
  unsigned long long *c = nullptr;
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  poison_roundtrip<<<(unsigned)((n + 255) / 256), 256>>>(n, bytes, c);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global(), &err);
  cudaFree(c);
  free_global_allocator();
  for (int i = 0; i < 4; i++) out[i] = h[i];
  out[4] = err;
  return e == cudaSuccess ? 0 : 1;
}

// ---- divergent calls in data-dependent loops (the reference's threading
// contract: any subset of a warp's lanes may call malloc/free, in loops)

__device__ __forceinline__ uint64_t mixbits(uint64_t z) {
  z ^= z >> 31;
  z *= 0x7FB5D329728EA185ull;
  z ^= z >> 27;
  return z;
}

// thread t runs (h % 7) iterations; in each it allocates a size drawn from h,
// stamps it, and frees the previous allocation on odd draws (so lanes of a
// warp call malloc and free at different times, some exiting early).  The
// live allocations at the end stay in bits[t * 8 + j] with their sizes.
__global__ void divergent_loops(uint64_t n, uint64_t **bits, uint64_t *sizes, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t h = mixbits(tid * 0x9E3779B97F4A7C15ull + 1);
  if ((h & 15) == 0) return;  // some lanes never call
  const int iters = (int)(h % 7);
  uint64_t *prev = nullptr;
  int kept = 0;
  for (int i = 0; i < iters; i++) {
    h = mixbits(h + i);
    uint64_t size = 16ull << (h % 9);  // 16 B .. 4 KiB
    if (h & 32) size += (h >> 8) % 17;  // and some in between
    uint64_t *p = (uint64_t *)global_malloc(size);
    if (!p) continue;
    atomicAdd(&c[0], 1ull);
    p[0] = tid;
    p[(size / 8) - 1 > 0 ? (size / 8) - 1 : 0] = ~tid;
    if ((h & 1) && prev) {
      if (prev[0] != tid) atomicAdd(&c[1], 1ull);
      global_free(prev);
      prev = nullptr;
    }
    if (prev && kept < 8) {  // keep it for the host's overlap check
      bits[tid * 8 + kept] = prev;
      sizes[tid * 8 + kept] = 0;  // filled below
      kept++;
    }
    prev = p;
    if (kept < 8) sizes[tid * 8 + kept] = size;
  }
  if (prev && kept < 8) bits[tid * 8 + kept] = prev;
}

__global__ void divergent_check_free(uint64_t n, uint64_t **bits, unsigned long long *c) {
  uint64_t i = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (i >= n * 8) return;
  uint64_t *p = bits[i];
  if (!p) return;
  if (p[0] != i / 8) atomicAdd(&c[1], 1ull);
  global_free(p);
}

// out[0] successful mallocs, [1] stamp mismatches, [2] overlapping live
// allocations (checked on the host), [3] device error word
extern "C" int dropin_divergent_test(uint64_t num_bytes, uint64_t n, int rounds, uint64_t *out) {
  init_global_allocator(num_bytes, 42, false);
  uint64_t **bits = nullptr;
  uint64_t *sizes = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * 8 * sizeof(uint64_t *));
  cudaMalloc(&sizes, n * 8 * sizeof(uint64_t));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  uint64_t overlaps = 0;
  cudaError_t e = cudaSuccess;
  for (int r = 0; r < rounds && e == cudaSuccess; r++) {
    cudaMemset(bits, 0, n * 8 * sizeof(uint64_t *));
    cudaMemset(sizes, 0, n * 8 * sizeof(uint64_t));
    divergent_loops<<<(unsigned)((n + 255) / 256), 256>>>(n, bits, sizes, c);
    e = cudaDeviceSynchronize();
    // live ranges [p, p + 16) at least: no two live pointers may coincide
    uint64_t *hb = (uint64_t *)malloc(n * 8 * sizeof(uint64_t));
    cudaMemcpy(hb, bits, n * 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    uint64_t m = 0;
    for (uint64_t i = 0; i < n * 8; i++)
      if (hb[i]) hb[m++] = hb[i];
    qsort(hb, m, sizeof(uint64_t), [](const void *a, const void *b) {
      uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
      return x < y ? -1 : (x > y ? 1 : 0);
    });
    for (uint64_t i = 1; i < m; i++)
      if (hb[i] < hb[i - 1] + 16) overlaps++;
    free(hb);
    divergent_check_free<<<(unsigned)((n * 8 + 255) / 256), 256>>>(n, bits, c);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global(), &err);
  cudaFree(bits);
  cudaFree(sizes);
  cudaFree(c);
  free_global_allocator();
  out[0] = h[0];
  out[1] = h[1];
  out[2] = overlaps;
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

// The reference's pointer churn (tests/src/global_churn.cu:184-245): every
// thread loops: malloc of a hashed size, exchange its id into the first word
// (the old word must be 0: the arena starts zeroed and every user clears the
// word before freeing), exchange 0 back (the word must still hold the id),
// free.  A shared allocation shows up as a non-zero old word or a changed id.
// Sizes span [min_size, max_size) here; the reference's host passes the two
// swapped (global_churn.cu:295 vs :185), so every request there was max_size.
__device__ uint64_t churn_mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void pointer_churn(uint64_t n, int rounds, uint64_t min_size, uint64_t max_size,
                              unsigned long long *c) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  const unsigned long long me = tid + 1;
  uint64_t h = tid;
  for (int i = 0; i < rounds; i++) {
    h = churn_mix(h ^ (uint64_t)i);
    const uint64_t size = min_size + h % (max_size - min_size);
    unsigned long long *p = (unsigned long long *)global_malloc(size);
    for (int retry = 0; p == nullptr && retry < 10; retry++) p = (unsigned long long *)global_malloc(size);
    if (p == nullptr) {
      atomicAdd(&c[0], 1ull);
      continue;
    }
    if (atomicExch(p, me) != 0ull) atomicAdd(&c[1], 1ull);
    if (atomicExch(p, 0ull) != me) atomicAdd(&c[2], 1ull);
    global_free(p);
  }
}

extern "C" int dropin_churn_test(uint64_t num_bytes, uint64_t n, int rounds, uint64_t min_size,
                                 uint64_t max_size, uint64_t *out) {
  if (max_size <= min_size || min_size < 8) return 3;
  init_global_allocator(num_bytes, 111, false);
  unsigned long long *c = nullptr;
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  pointer_churn<<<(unsigned)((n + 255) / 256), 256>>>(n, rounds, min_size, max_size, c);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global(), &err);
  cudaFree(c);
  free_global_allocator();
  out[0] = h[0];  // requests that failed 11 times
  out[1] = h[1];  // allocation already held another thread's id
  out[2] = h[2];  // id changed while held
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

// calloc mode (init_global_allocator(..., running_calloc = true)): every
// allocation reads zero over its requested bytes, also when its memory was
// written by an earlier allocation and came back through a free.  Half the
// requests are whole blocks (32-64 KiB), which a free returns to their
// segment for the next round to reuse; the rest are slices.
__global__ void calloc_round(uint64_t n, int round, unsigned char **bits, unsigned long long *c) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  const uint64_t h = churn_mix(tid * 0x100000001B3ull + (uint64_t)round);
  const uint64_t size = (h & 1) ? 32769 + (h >> 1) % 32768 : 16 + (h >> 1) % 4081;
  unsigned char *p = (unsigned char *)global_malloc(size);
  bits[tid] = p;
  if (p == nullptr) {
    atomicAdd(&c[0], 1ull);
    return;
  }
  bool dirty = false;
  const uint32_t *w = (const uint32_t *)p;  // allocations start 16-byte aligned
  for (uint64_t i = 0; i < size / 4; i++) dirty |= w[i] != 0u;
  for (uint64_t i = size & ~3ull; i < size; i++) dirty |= p[i] != 0;
  if (dirty) atomicAdd(&c[1], 1ull);
  for (uint64_t i = 0; i < size; i++) p[i] = 0xA5;  // leave the memory dirty
}

__global__ void calloc_free(uint64_t n, unsigned char **bits) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid < n && bits[tid]) global_free(bits[tid]);
}

extern "C" int dropin_calloc_test(uint64_t num_bytes, uint64_t n, int rounds, int calloc_mode, uint64_t *out) {
  init_global_allocator(num_bytes, 42, false, calloc_mode != 0);
  if (!gal_global()) return 2;
  unsigned char **bits = nullptr;
  unsigned long long *c = nullptr;
  cudaMalloc(&bits, n * sizeof(unsigned char *));
  cudaMalloc(&c, 4 * sizeof(unsigned long long));
  cudaMemset(c, 0, 4 * sizeof(unsigned long long));
  for (int r = 0; r < rounds; r++) {
    calloc_round<<<(unsigned)((n + 255) / 256), 256>>>(n, r, bits, c);
    calloc_free<<<(unsigned)((n + 255) / 256), 256>>>(n, bits);
  }
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  uint32_t err = 0;
  gal_last_error(gal_global(), &err);
  cudaFree(bits);
  cudaFree(c);
  free_global_allocator();
  out[0] = h[0];  // failed requests
  out[1] = h[1];  // allocations that did not read zero
  out[2] = 0;
  out[3] = err;
  return e == cudaSuccess ? 0 : 1;
}

// ---- a global handle that is not set: global_malloc returns nullptr and
// global_free does nothing (the reference's failure contract,
// global_allocator.cuh:72-82), in a translation unit that never called
// init_global_allocator or after free_global_allocator cleared the handle

__global__ void null_handle_calls(uint64_t n, uint64_t size, void *stale, unsigned long long *c) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  void *p = global_malloc(size);
  void *q = global_malloc_host(size);
  if (p != nullptr) atomicAdd(c, 1ull);
  if (q != nullptr) atomicAdd(c + 1, 1ull);
  global_free(stale);       // no instance: nothing to give it back to
  global_free_host(stale);
  if (global_malloc_poison(size) != nullptr) atomicAdd(c + 2, 1ull);
}

__global__ void one_malloc(uint64_t size, void **out) { out[0] = global_malloc(size); }

// out[0] non-null results before any init, out[1] non-null host results,
// out[2] non-null poison results, out[3] whether the initialised instance
// served (1), out[4] non-null results after free_global_allocator
extern "C" int dropin_null_handle_test(uint64_t n, uint64_t *out) {
  unsigned long long *c = nullptr;
  void **slot = nullptr;
  cudaMalloc(&c, 3 * sizeof(unsigned long long));
  cudaMalloc(&slot, sizeof(void *));
  cudaMemset(c, 0, 3 * sizeof(unsigned long long));
  unsigned grid = (unsigned)((n + 255) / 256);
  null_handle_calls<<<grid, 256>>>(n, 64, nullptr, c);
  cudaError_t e = cudaDeviceSynchronize();
  unsigned long long h[3] = {0, 0, 0};
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  init_global_allocator(1ull << 30, 42, false);
  one_malloc<<<1, 1>>>(64, slot);
  void *served = nullptr;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaMemcpy(&served, slot, sizeof(void *), cudaMemcpyDeviceToHost);
  out[3] = served != nullptr;
  free_global_allocator();
  cudaMemset(c, 0, 3 * sizeof(unsigned long long));
  null_handle_calls<<<grid, 256>>>(n, 64, served, c);  // `served` now dangles: the free ignores it
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaMemcpy(h, c, sizeof(h), cudaMemcpyDeviceToHost);
  out[4] = h[0] + h[1] + h[2];
  cudaFree(c);
  cudaFree(slot);
  return e == cudaSuccess ? 0 : 1;
}
