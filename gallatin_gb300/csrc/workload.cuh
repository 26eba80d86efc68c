// workload.cuh — seeded synthetic request streams shared by the benchmark
// kernels, the CPU baseline and the reference-side harness, so that every
// implementation serves exactly the same requests.
//
// Counter-based generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011), restated from the
// paper: ten rounds of two 32x32->64 multiplies with the published constants,
// key bumped by the published Weyl increments between rounds.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GAL_HD __host__ __device__ __forceinline__
#else
#define GAL_HD static inline
#endif

namespace galwl {

struct u32x4 {
  uint32_t v[4];
};

GAL_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

GAL_HD u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; r++) {
    if (r) {
      k0 += W0;
      k1 += W1;
    }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, ctr.v[0], hi0, lo0);
    mulhilo32(M1, ctr.v[2], hi1, lo1);
    u32x4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
  }
  return ctr;
}

// Request size of slot `slot`: log-uniform over [16 B, 4 KiB] rounded up to a
// power of two means the size class (ceil log2) is uniform over 32..4096.
// The request itself is uniform inside (2^(c-1), 2^c] so the allocator sees
// non-power-of-two sizes and does the rounding.
GAL_HD uint64_t mixed_size(uint64_t slot, uint32_t seed) {
  u32x4 c = {{(uint32_t)slot, (uint32_t)(slot >> 32), 0xA110Cu, 0u}};
  u32x4 r = philox4x32_10(c, seed, 0x51CE5u);
  uint32_t x = r.v[0];
  uint32_t cls = 5u + (x >> 29);           // 5..12
  uint32_t half = 1u << (cls - 1);         // 16..2048
  return (uint64_t)half + 1u + (r.v[1] & (half - 1u));
}

// Payload stamped into an allocation (first 4 bytes).
GAL_HD uint32_t payload(uint64_t slot, uint32_t seed) {
  return (uint32_t)(slot * 0x9E3779B97F4A7C15ull >> 32) ^ seed ^ 0x5EEDu;
}

// Fair coins of 128 consecutive slots (group = slot / 128) in round `round`:
// one Philox call, one bit per slot.  Decides the 50% free.
GAL_HD u32x4 free_coin_group(uint64_t group, uint32_t round, uint32_t seed) {
  u32x4 c = {{(uint32_t)group, (uint32_t)(group >> 32), round, 0xF4EEu}};
  return philox4x32_10(c, seed, 0xC01Du);
}
GAL_HD bool coin_bit(const u32x4 &g, uint64_t slot) {
  return (g.v[(slot >> 5) & 3u] >> (slot & 31u)) & 1u;
}
GAL_HD bool free_coin(uint64_t slot, uint32_t round, uint32_t seed) {
  return coin_bit(free_coin_group(slot >> 7, round, seed), slot);
}

}  // namespace galwl
