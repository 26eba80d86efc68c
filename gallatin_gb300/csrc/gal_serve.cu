// gal_serve.cu — device jobs of the served request loop (gallatin_gb300/serve.py).
//
// Two job kinds, each a grid of gal_job_ctas(kind, n) CTAs allocating through
// the device allocator while other jobs run on other streams:
//   * vector: n uint32 values pushed back into device vectors whose capacity
//     starts at 1,024 elements and doubles through malloc / copy / free (the
//     growth of the reference's data_structs/single_vector.cuh:86-143); CTA b
//     of G grows its own vector over elements [b n / G, (b + 1) n / G), so a
//     large job crosses 4 KiB slices, 8-32 KiB slice runs, whole blocks and
//     multi-segment runs;
//   * queue (CTAs of QUEUE_THREADS): n enqueue/dequeue operations on
//     per-thread FIFO queues of 32 B nodes (malloc on enqueue, free on
//     dequeue), drained at the end.
// result[0] = checksum (sum of the vector's values / of every dequeued value),
// which depends only on the job's id and size; result[1] = mallocs + frees;
// result[2] = failed mallocs.  hist (optional) receives the latency of every
// malloc and free the job makes, in SM cycles (clock64 around the call),
// binned by lat_bin: each CTA counts in shared memory (one shared atomic per
// call) and adds its non-zero bins to hist at the end.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"

namespace {

constexpr int JOB_THREADS = 256;
constexpr int BINS = GAL_JOB_LAT_BINS;

__device__ __forceinline__ uint32_t job_value(uint64_t job, uint64_t j) {
  uint64_t x = job * 0x9E3779B97F4A7C15ull + j * 0xBF58476D1CE4E5B9ull + 0x94D049BB133111EBull;
  x ^= x >> 31;
  x *= 0xD6E8FEB86659FD93ull;
  return (uint32_t)(x >> 32);
}

// c for c < 4, else 4 floor(log2 c) + the two bits below the leading one:
// four bins per power of two (bin edges within 19% of each other)
__device__ __forceinline__ uint32_t lat_bin(long long cycles) {
  const uint64_t c = cycles > 0 ? (uint64_t)cycles : 0;
  if (c < 4) return (uint32_t)c;
  const uint32_t e = 63u - (uint32_t)__clzll((long long)c);
  const uint32_t b = 4u * e + (uint32_t)((c >> (e - 2)) & 3u);
  return b < (uint32_t)BINS ? b : (uint32_t)BINS - 1u;
}

struct job_hist {
  uint32_t n[2 * BINS];  // mallocs, then frees
};

__device__ __forceinline__ void hist_init(job_hist &h) {
  for (int i = threadIdx.x; i < 2 * BINS; i += blockDim.x) h.n[i] = 0;
}
__device__ __forceinline__ void hist_add(job_hist &h, int which, long long cycles) {
  atomicAdd(&h.n[which * BINS + lat_bin(cycles)], 1u);
}
__device__ __forceinline__ void hist_flush(const job_hist &h, unsigned long long *out) {
  if (!out) return;
  for (int i = threadIdx.x; i < 2 * BINS; i += blockDim.x)
    if (h.n[i]) atomicAdd(&out[i], (unsigned long long)h.n[i]);
}

__global__ void __launch_bounds__(JOB_THREADS)
    k_job_vector(const gal::state *s, uint64_t job, uint64_t n, unsigned long long *result,
                 unsigned long long *hist) {
  __shared__ uint32_t *buf;
  __shared__ uint32_t *next;
  __shared__ uint64_t cap;
  __shared__ int failed;
  __shared__ unsigned long long ops;
  __shared__ job_hist lh;
  const int t = threadIdx.x;
  // this CTA's share of the job's elements
  const uint64_t lo = n * blockIdx.x / gridDim.x, hi = n * (blockIdx.x + 1) / gridDim.x;
  const uint64_t m = hi - lo;
  hist_init(lh);
  __syncthreads();
  if (t == 0) {
    long long c0 = clock64();
    buf = (uint32_t *)gal::malloc(s, 1024 * sizeof(uint32_t));
    hist_add(lh, 0, clock64() - c0);
    cap = 1024;
    failed = buf == nullptr;
    ops = 1;
  }
  __syncthreads();
  uint64_t size = 0;
  for (uint64_t base = 0; base < m && !failed; base += JOB_THREADS) {
    if (base + JOB_THREADS > cap) {  // grow: malloc 2x, copy, free the old buffer
      if (t == 0) {
        long long c0 = clock64();
        next = (uint32_t *)gal::malloc(s, 2 * cap * sizeof(uint32_t));
        hist_add(lh, 0, clock64() - c0);
        ops++;
        failed = next == nullptr;
      }
      __syncthreads();
      if (failed) break;
      for (uint64_t j = t; j < size; j += JOB_THREADS) next[j] = buf[j];
      __syncthreads();
      if (t == 0) {
        long long c0 = clock64();
        gal::free(s, buf);
        hist_add(lh, 1, clock64() - c0);
        ops++;
        buf = next;
        cap *= 2;
      }
      __syncthreads();
    }
    uint64_t j = base + t;
    if (j < m) buf[j] = job_value(job, lo + j);
    size = min(m, base + JOB_THREADS);
  }
  __syncthreads();
  unsigned long long sum = 0;
  if (!failed)
    for (uint64_t j = t; j < m; j += JOB_THREADS) sum += buf[j];
  if (sum) atomicAdd(&result[0], sum);  // 64-bit partial sums: no carry is lost
  __syncthreads();
  if (t == 0) {
    if (buf) {
      long long c0 = clock64();
      gal::free(s, buf);
      hist_add(lh, 1, clock64() - c0);
      ops++;
    }
    atomicAdd(&result[1], ops);
    atomicAdd(&result[2], (unsigned long long)failed);
  }
  __syncthreads();
  hist_flush(lh, hist);
}

struct qnode {
  qnode *next;
  uint64_t value;
  uint64_t pad[2];  // a 32 B node
};

constexpr int QUEUE_THREADS = 1024;

__global__ void __launch_bounds__(QUEUE_THREADS)
    k_job_queue(const gal::state *s, uint64_t job, uint64_t n, unsigned long long *result,
                unsigned long long *hist) {
  __shared__ job_hist lh;
  hist_init(lh);
  __syncthreads();
  // thread t of the whole grid runs its share of the n operations
  const uint64_t t = (uint64_t)blockIdx.x * QUEUE_THREADS + threadIdx.x;
  const uint64_t nt = (uint64_t)gridDim.x * QUEUE_THREADS;
  const uint64_t mine = n / nt + (t < n % nt ? 1 : 0);
  qnode *head = nullptr, *tail = nullptr;
  unsigned long long sum = 0, ops = 0, failed = 0;
  for (uint64_t o = 0; o < mine; o++) {
    uint64_t key = (t << 40) ^ o;
    uint32_t h = job_value(job, key);
    if (head == nullptr || h % 10 < 6) {  // enqueue
      long long c0 = clock64();
      qnode *q = (qnode *)gal::malloc(s, sizeof(qnode));
      hist_add(lh, 0, clock64() - c0);
      ops++;
      if (!q) {
        failed++;
        continue;
      }
      q->next = nullptr;
      q->value = h;
      if (tail)
        tail->next = q;
      else
        head = q;
      tail = q;
    } else {  // dequeue
      qnode *q = head;
      head = q->next;
      if (!head) tail = nullptr;
      sum += q->value;
      long long c0 = clock64();
      gal::free(s, q);
      hist_add(lh, 1, clock64() - c0);
      ops++;
    }
  }
  while (head) {  // drain
    qnode *q = head;
    head = q->next;
    sum += q->value;
    long long c0 = clock64();
    gal::free(s, q);
    hist_add(lh, 1, clock64() - c0);
    ops++;
  }
  atomicAdd(&result[0], sum);
  atomicAdd(&result[1], ops);
  if (failed) atomicAdd(&result[2], failed);
  __syncthreads();
  hist_flush(lh, hist);
}

}  // namespace

extern "C" uint32_t gal_job_ctas(uint32_t kind, uint64_t n) {
  const uint64_t g = kind == GAL_JOB_VECTOR ? n >> 20 : n >> 18;
  return g < 1 ? 1u : g > 8 ? 8u : (uint32_t)g;
}

extern "C" int gal_job_launch(gal_handle *h, uint32_t kind, uint64_t job_id, uint64_t n,
                              unsigned long long *result, unsigned long long *hist, void *stream) {
  if (!h || !result || kind > GAL_JOB_QUEUE) return GAL_ERR_ARGS;
  const gal::state *d = (const gal::state *)gal_device_state(h);
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned g = gal_job_ctas(kind, n);
  if (kind == GAL_JOB_VECTOR)
    k_job_vector<<<g, JOB_THREADS, 0, st>>>(d, job_id, n, result, hist);
  else
    k_job_queue<<<g, QUEUE_THREADS, 0, st>>>(d, job_id, n, result, hist);
  return cudaGetLastError() == cudaSuccess ? GAL_OK : GAL_ERR_CUDA;
}
