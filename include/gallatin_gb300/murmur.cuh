// MurmurHash64A (Austin Appleby's published 64-bit MurmurHash2 variant),
// specialised to the single 8-byte key the vEB random start hashes
// (reference murmurhash.cuh:20-61, called with len = 8 from veb.cuh:950-956).
#ifndef GALLATIN_GB300_MURMUR_CUH
#define GALLATIN_GB300_MURMUR_CUH

#include <stdint.h>

namespace gal {

__host__ __device__ __forceinline__ uint64_t murmur64a_u64(uint64_t key, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ull;
  const int r = 47;
  uint64_t h = seed ^ (8ull * m);
  uint64_t k = key * m;
  k ^= k >> r;
  k *= m;
  h ^= k;
  h *= m;
  // len & 7 == 0: no tail bytes
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

}  // namespace gal

#endif  // GALLATIN_GB300_MURMUR_CUH
