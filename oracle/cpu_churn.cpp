// cpu_churn.cpp — CPU baselines of the mixed-size churn workload
// (TEST/BENCH INFRASTRUCTURE ONLY; bench.py's cpu_baseline leg).
//
//   orc_churn_oracle: the oracle (the reference allocator's algorithm restated
//     for one CPU thread) serving a bounded sample of the workload;
//   orc_churn_glibc: glibc malloc/free on `threads` host threads, each serving
//     a disjoint share of every round, payload written and checked.
// Both serve the same requests as the GPU churn (gallatin_gb300/csrc/workload.cuh).
#include <stdint.h>

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../gallatin_gb300/csrc/workload.cuh"
#include "gal_oracle.h"

extern "C" {

// ops_out[0] mallocs ok, [1] mallocs failed, [2] frees; returns seconds.
// Gallatin<segment_bytes, 16, 4096> with the reference's pinned slots.
double orc_churn_oracle(uint64_t arena_bytes, uint64_t segment_bytes, uint64_t threads_per_round,
                        uint32_t rounds, uint32_t seed, uint64_t *ops_out) {
  orc_alloc *a = orc_create(arena_bytes, 42, segment_bytes, 16, 4096, 128, 4,
                            ORC_FIX_GATHER_EXIT_ROLLBACK | ORC_FIX_LEFTOVER_COMPLETES | ORC_FIX_RUN_BELOW_ARENA |
                                ORC_FIX_RUN_RETURN_SUMMARY, 0);
  orc_boot_one_thread(a);
  const uint64_t nslots = threads_per_round * rounds;
  std::vector<uint64_t> live(nslots, ~0ull);
  uint64_t ok = 0, fail = 0, frees = 0;
  auto t0 = std::chrono::steady_clock::now();
  for (uint32_t r = 0; r <= rounds; r++) {
    bool drain = r == rounds;
    if (r > 0) {
      uint64_t n = drain ? nslots : threads_per_round * r;
      for (uint64_t i = 0; i < n; i++) {
        if (live[i] == ~0ull) continue;
        if (!drain && !galwl::free_coin(i, r, seed)) continue;
        orc_free(a, live[i]);
        live[i] = ~0ull;
        frees++;
      }
    }
    if (drain) break;
    for (uint64_t t = 0; t < threads_per_round; t++) {
      uint64_t slot = threads_per_round * r + t;
      uint64_t off = orc_malloc(a, galwl::mixed_size(slot, seed), (uint32_t)(t / 2048), t);
      live[slot] = off;
      if (off == ~0ull)
        fail++;
      else
        ok++;
    }
  }
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  orc_destroy(a);
  ops_out[0] = ok;
  ops_out[1] = fail;
  ops_out[2] = frees;
  return s;
}

// ops_out[0] mallocs ok, [1] failed, [2] frees, [3] payload mismatches; returns seconds
double orc_churn_glibc(uint64_t threads_per_round, uint32_t rounds, uint32_t seed, int threads,
                       uint64_t *ops_out) {
  const uint64_t nslots = threads_per_round * rounds;
  std::vector<void *> ptrs(nslots, nullptr);
  std::vector<uint64_t> counts(4 * (size_t)threads, 0);
  auto worker = [&](int w, uint32_t r, bool malloc_phase) {
    uint64_t *c = &counts[4 * (size_t)w];
    if (malloc_phase) {
      uint64_t lo = threads_per_round * w / threads, hi = threads_per_round * (w + 1) / threads;
      for (uint64_t t = lo; t < hi; t++) {
        uint64_t slot = threads_per_round * r + t;
        void *p = std::malloc(galwl::mixed_size(slot, seed));
        if (p) {
          *(volatile uint32_t *)p = galwl::payload(slot, seed);
          c[0]++;
        } else {
          c[1]++;
        }
        ptrs[slot] = p;
      }
    } else {
      bool drain = r == rounds;
      uint64_t n = drain ? nslots : threads_per_round * r;
      uint64_t lo = n * w / threads, hi = n * (w + 1) / threads;
      for (uint64_t i = lo; i < hi; i++) {
        void *p = ptrs[i];
        if (!p || (!drain && !galwl::free_coin(i, r, seed))) continue;
        if (*(volatile uint32_t *)p != galwl::payload(i, seed)) c[3]++;
        std::free(p);
        ptrs[i] = nullptr;
        c[2]++;
      }
    }
  };
  auto t0 = std::chrono::steady_clock::now();
  for (uint32_t r = 0; r <= rounds; r++) {
    for (int phase = 0; phase < 2; phase++) {
      bool malloc_phase = phase == 1;
      if (!malloc_phase && r == 0) continue;
      if (malloc_phase && r == rounds) continue;
      std::vector<std::thread> ts;
      for (int w = 0; w < threads; w++) ts.emplace_back(worker, w, r, malloc_phase);
      for (auto &t : ts) t.join();
    }
  }
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < 4; i++) {
    ops_out[i] = 0;
    for (int w = 0; w < threads; w++) ops_out[i] += counts[4 * (size_t)w + i];
  }
  return s;
}

}  // extern "C"
