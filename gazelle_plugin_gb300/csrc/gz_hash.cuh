// Spark Murmur3_x86_32 hash chain and divide-free pmod, shared by the hash kernels.
//
// Reference: HashSplitter::ComputeAndCountPartitionId, native-sql-engine/cpp/src/shuffle/splitter.cc:1440-1470
// (hash chain seeded with 42, a null key passes the seed through, pmod of the result).
#pragma once
#include <stdint.h>

namespace gz {
namespace hash {

// Spark Murmur3_x86_32 (hashInt / hashLong), seed chained, nulls pass the seed through.
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return __funnelshift_l(x, x, r); }
__device__ __forceinline__ uint32_t mix_k1(uint32_t k1) {
  k1 *= 0xcc9e2d51u;
  k1 = rotl32(k1, 15);
  return k1 * 0x1b873593u;
}
__device__ __forceinline__ uint32_t mix_h1(uint32_t h1, uint32_t k1) {
  h1 ^= k1;
  h1 = rotl32(h1, 13);
  return h1 * 5u + 0xe6546b64u;
}
__device__ __forceinline__ uint32_t fmix32(uint32_t h1, uint32_t len) {
  h1 ^= len;
  h1 ^= h1 >> 16;
  h1 *= 0x85ebca6bu;
  h1 ^= h1 >> 13;
  h1 *= 0xc2b2ae35u;
  h1 ^= h1 >> 16;
  return h1;
}
__device__ __forceinline__ int32_t hash_int(int32_t v, int32_t seed) {
  return (int32_t)fmix32(mix_h1((uint32_t)seed, mix_k1((uint32_t)v)), 4);
}
__device__ __forceinline__ int32_t hash_long(int64_t v, int32_t seed) {
  uint64_t u = (uint64_t)v;
  uint32_t h1 = mix_h1((uint32_t)seed, mix_k1((uint32_t)u));
  h1 = mix_h1(h1, mix_k1((uint32_t)(u >> 32)));
  return (int32_t)fmix32(h1, 8);
}

// Spark Murmur3_x86_32.hashUnsafeBytes (the utf8 key hash): 4-byte little-endian blocks, then
// every remaining byte, sign-extended, as a block of its own; finalised with the byte length.
// The blocks are funnel-shifted out of aligned words; the second word of a pair always holds a
// byte of the string, so no word past the string's last aligned word is read.
__device__ __forceinline__ int32_t hash_bytes(const uint8_t* p, int32_t len, int32_t seed) {
  uint32_t h1 = (uint32_t)seed;
  const int32_t aligned = len & ~3;
  const uint32_t* base = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(p) & ~uintptr_t(3));
  const uint32_t sh = (uint32_t)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
  for (int32_t i = 0; i < aligned; i += 4) {
    const uint32_t k = sh ? __funnelshift_r(base[i >> 2], base[(i >> 2) + 1], sh) : base[i >> 2];
    h1 = mix_h1(h1, mix_k1(k));
  }
  for (int32_t i = aligned; i < len; i++) h1 = mix_h1(h1, mix_k1((uint32_t)(int32_t)(int8_t)p[i]));
  return (int32_t)fmix32(h1, (uint32_t)len);
}

// Spark pmod(h, P) without a hardware divide: Lemire, Kaser & Kurz, "Faster remainder by
// direct computation" (2019): a mod d = hi64((M * a) mod 2^64 * d) with M = floor(2^64-1 / d) + 1.
__device__ __forceinline__ uint32_t fastmod_u32(uint32_t a, uint32_t d, unsigned long long M) {
  const unsigned long long low = M * (unsigned long long)a;
  return (uint32_t)__umul64hi(low, (unsigned long long)d);
}
__device__ __forceinline__ uint32_t fast_pmod(int32_t h, uint32_t P, unsigned long long M) {
  if (P == 1) return 0;
  if (h >= 0) return fastmod_u32((uint32_t)h, P, M);
  const uint32_t r = fastmod_u32(0u - (uint32_t)h, P, M);
  return r == 0 ? 0 : P - r;
}

__device__ __forceinline__ bool get_bit(const uint8_t* bits, uint32_t i) {
  return (bits[i >> 3] >> (i & 7)) & 1;
}

}  // namespace hash
}  // namespace gz
