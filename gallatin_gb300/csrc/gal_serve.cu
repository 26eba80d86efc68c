// gal_serve.cu — device jobs of the served request loop (gallatin_gb300/serve.py).
//
// Two job kinds, each one CTA of JOB_THREADS threads allocating through the
// device allocator while other jobs run on other streams:
//   * vector: n uint32 values pushed back into a device vector whose capacity
//     starts at 1,024 elements and doubles through malloc / copy / free (the
//     growth of the reference's data_structs/single_vector.cuh:86-143), so a
//     large job crosses 4 KiB slices, 8-32 KiB slice runs, whole blocks and
//     multi-segment runs;
//   * queue (one CTA of QUEUE_THREADS): n enqueue/dequeue operations on
//     per-thread FIFO queues of 32 B nodes (malloc on enqueue, free on
//     dequeue), drained at the end.
// result[0] = checksum (sum of the vector's values / of every dequeued value),
// which depends only on the job's id and size; result[1] = mallocs + frees;
// result[2] = failed mallocs.  lat[0..63] / lat[64..127] receive the cycles
// (clock64) of the first 64 mallocs / frees of thread 0.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"

namespace {

constexpr int JOB_THREADS = 256;
constexpr int LAT = GAL_JOB_LAT_SAMPLES;

__device__ __forceinline__ uint32_t job_value(uint64_t job, uint64_t j) {
  uint64_t x = job * 0x9E3779B97F4A7C15ull + j * 0xBF58476D1CE4E5B9ull + 0x94D049BB133111EBull;
  x ^= x >> 31;
  x *= 0xD6E8FEB86659FD93ull;
  return (uint32_t)(x >> 32);
}

__global__ void __launch_bounds__(JOB_THREADS)
    k_job_vector(const gal::state *s, uint64_t job, uint64_t n, unsigned long long *result,
                 uint32_t *lat) {
  __shared__ uint32_t *buf;
  __shared__ uint32_t *next;
  __shared__ uint64_t cap;
  __shared__ int failed;
  __shared__ unsigned long long ops;
  __shared__ int nm, nf;
  const int t = threadIdx.x;
  if (t == 0) {
    long long c0 = clock64();
    buf = (uint32_t *)gal::malloc(s, 1024 * sizeof(uint32_t));
    if (lat) lat[0] = (uint32_t)(clock64() - c0);
    nm = 1;
    nf = 0;
    cap = 1024;
    failed = buf == nullptr;
    ops = 1;
  }
  __syncthreads();
  uint64_t size = 0;
  for (uint64_t base = 0; base < n && !failed; base += JOB_THREADS) {
    if (base + JOB_THREADS > cap) {  // grow: malloc 2x, copy, free the old buffer
      if (t == 0) {
        long long c0 = clock64();
        next = (uint32_t *)gal::malloc(s, 2 * cap * sizeof(uint32_t));
        if (lat && nm < LAT) lat[nm] = (uint32_t)(clock64() - c0);
        nm++;
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
        if (lat && nf < LAT) lat[LAT + nf] = (uint32_t)(clock64() - c0);
        nf++;
        ops++;
        buf = next;
        cap *= 2;
      }
      __syncthreads();
    }
    uint64_t j = base + t;
    if (j < n) buf[j] = job_value(job, j);
    size = min(n, base + JOB_THREADS);
  }
  __syncthreads();
  unsigned long long sum = 0;
  if (!failed)
    for (uint64_t j = t; j < n; j += JOB_THREADS) sum += buf[j];
  if (sum) atomicAdd(&result[0], sum);  // 64-bit partial sums: no carry is lost
  __syncthreads();
  if (t == 0) {
    if (buf) {
      long long c0 = clock64();
      gal::free(s, buf);
      if (lat && nf < LAT) lat[LAT + nf] = (uint32_t)(clock64() - c0);
      ops++;
    }
    atomicAdd(&result[1], ops);
    atomicAdd(&result[2], (unsigned long long)failed);
  }
}

struct qnode {
  qnode *next;
  uint64_t value;
  uint64_t pad[2];  // a 32 B node
};

constexpr int QUEUE_THREADS = 1024;

__global__ void __launch_bounds__(QUEUE_THREADS)
    k_job_queue(const gal::state *s, uint64_t job, uint64_t n, unsigned long long *result,
                uint32_t *lat) {
  const int t = threadIdx.x;
  const uint64_t mine = n / QUEUE_THREADS + ((uint64_t)t < n % QUEUE_THREADS ? 1 : 0);
  qnode *head = nullptr, *tail = nullptr;
  unsigned long long sum = 0, ops = 0, failed = 0;
  int nm = 0, nf = 0;
  for (uint64_t o = 0; o < mine; o++) {
    uint64_t key = ((uint64_t)t << 40) ^ o;
    uint32_t h = job_value(job, key);
    if (head == nullptr || h % 10 < 6) {  // enqueue
      long long c0 = clock64();
      qnode *q = (qnode *)gal::malloc(s, sizeof(qnode));
      if (lat && t == 0 && nm < LAT) lat[nm++] = (uint32_t)(clock64() - c0);
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
      if (lat && t == 0 && nf < LAT) lat[LAT + nf++] = (uint32_t)(clock64() - c0);
      ops++;
    }
  }
  while (head) {  // drain
    qnode *q = head;
    head = q->next;
    sum += q->value;
    gal::free(s, q);
    ops++;
  }
  atomicAdd(&result[0], sum);
  atomicAdd(&result[1], ops);
  if (failed) atomicAdd(&result[2], failed);
}

}  // namespace

extern "C" int gal_job_launch(gal_handle *h, uint32_t kind, uint64_t job_id, uint64_t n,
                              unsigned long long *result, uint32_t *lat, void *stream) {
  if (!h || !result || kind > GAL_JOB_QUEUE) return GAL_ERR_ARGS;
  const gal::state *d = (const gal::state *)gal_device_state(h);
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == GAL_JOB_VECTOR)
    k_job_vector<<<1, JOB_THREADS, 0, st>>>(d, job_id, n, result, lat);
  else
    k_job_queue<<<1, QUEUE_THREADS, 0, st>>>(d, job_id, n, result, lat);
  return cudaGetLastError() == cudaSuccess ? GAL_OK : GAL_ERR_CUDA;
}
