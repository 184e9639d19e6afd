// std_hash.h -- the partition hash of the reference, for host and device.
//
// The reference buckets a row by std::hash<std::string> of one cell modulo
// n_partitions (core/components/data_mngr.h:157, 187).  With libstdc++ on a
// 64-bit target that is _Hash_bytes(data, len, 0xc70f6907): a byte-string
// hash in the MurmurHash2 64-bit family (Austin Appleby's MurmurHash64A
// mixing with multiplier 0xc6a4a7935bd1e995 and a 47-bit shift).  Restated:
//   h = seed ^ (len * M)
//   for each whole 8-byte little-endian word w:
//       w = mix(w * M) * M;  h = (h ^ w) * M          mix(v) = v ^ (v >> 47)
//   if 1-7 bytes remain: t = those bytes as a little-endian integer;
//       h = (h ^ t) * M
//   h = mix(mix(h) * M)
// Equality with the host's own std::hash is checked by the tests on every
// machine they run on (x86-64 and aarch64 load words little-endian alike).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define HBX_HD __host__ __device__ __forceinline__
#else
#define HBX_HD inline
#endif

namespace hbx {

constexpr uint64_t kStdHashSeed = 0xc70f6907ull;
constexpr uint64_t kStdHashMul = 0xc6a4a7935bd1e995ull;

HBX_HD uint64_t std_hash_mix(uint64_t v) { return v ^ (v >> 47); }

// Little-endian value of bytes p[0 .. n), n <= 8, byte by byte (no alignment
// needed).
HBX_HD uint64_t load_le(const uint8_t* p, uint32_t n) {
  uint64_t v = 0;
  for (uint32_t k = n; k > 0; k--) v = (v << 8) | p[k - 1];
  return v;
}

// The same hash with another seed (the dictionaries rehash with a fresh seed
// when two distinct cells share a hash).
HBX_HD uint64_t hash_bytes_seeded(const uint8_t* p, uint64_t len, uint64_t seed) {
  uint64_t h = seed ^ (len * kStdHashMul);
  const uint64_t whole = len & ~7ull;
  for (uint64_t i = 0; i < whole; i += 8) {
    const uint64_t w = std_hash_mix(load_le(p + i, 8) * kStdHashMul) * kStdHashMul;
    h = (h ^ w) * kStdHashMul;
  }
  if (len & 7) h = (h ^ load_le(p + whole, (uint32_t)(len & 7))) * kStdHashMul;
  return std_hash_mix(std_hash_mix(h) * kStdHashMul);
}

HBX_HD uint64_t std_hash_bytes(const uint8_t* p, uint64_t len) {
  return hash_bytes_seeded(p, len, kStdHashSeed);
}

}  // namespace hbx
