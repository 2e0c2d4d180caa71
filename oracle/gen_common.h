/* gen_common.h -- hashing shared by the oracle's seeded graph generators
 * (test infrastructure, not the product). */
#ifndef KAMSTA_ORACLE_GEN_COMMON_H
#define KAMSTA_ORACLE_GEN_COMMON_H
#include <stdint.h>

namespace gen {

/* SplitMix64's output function (Steele, Lea, Flood 2014). */
inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* High 64 bits of the 128-bit product a * b. */
inline uint64_t hi64(uint64_t a, uint64_t b) {
  return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
}

/* Edge weight of the generators: 1 + hi64(mix64(wseed ^ (lo << 32 | hi)) *
 * max_weight), lo < hi the endpoints. */
inline uint32_t weight(uint64_t wseed, uint64_t lo, uint64_t hi, uint32_t max_weight) {
  return 1u + static_cast<uint32_t>(hi64(mix64(wseed ^ ((lo << 32) | hi)), max_weight));
}

constexpr uint64_t kWeightSalt = 0x6a09e667f3bcc909ull;

/* floor(sqrt(x)), by bisection on 64-bit integers. */
inline uint64_t isqrt(uint64_t x) {
  uint64_t lo = 0, hi = 0xffffffffull;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo + 1) / 2;
    if (mid * mid <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

/* Weight of a geometric edge with squared distance d2 <= R2 under distance
 * rule `mode` (0 random: weight(); 1 Euclidean: 1 + floor((max_weight-1)
 * sqrt(d2 / R2)) computed as 1 + isqrt(floor((max_weight-1)^2 d2 / R2));
 * 2 squared Euclidean: 1 + floor((max_weight-1) d2 / R2)). */
inline uint32_t geo_weight(uint32_t mode, uint64_t d2, uint64_t R2, uint64_t wseed, uint64_t lo,
                           uint64_t hi, uint32_t max_weight) {
  if (mode == 0) return weight(wseed, lo, hi, max_weight);
  if (R2 == 0) return 1u;
  const unsigned __int128 k = max_weight - 1ull;
  if (mode == 2) return 1u + static_cast<uint32_t>(d2 * k / R2);
  return 1u + static_cast<uint32_t>(isqrt(static_cast<uint64_t>(d2 * k * k / R2)));
}

}  // namespace gen
#endif
