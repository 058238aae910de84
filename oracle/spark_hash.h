/*
 * Oracle (test infrastructure only): a CPU restatement of the Spark-compatible
 * Murmur3 hash that the reference hash partitioner evaluates per row.
 *
 * The reference builds the chain  h = f_k(key_k, ... f_1(key_1, 42))  in
 * HashSplitter::CreateProjector (native-sql-engine/cpp/src/shuffle/splitter.cc:1402-1438)
 * and evaluates it with gandiva functions whose bodies live in the un-vendored
 * Arrow fork oap-project/arrow@arrow-4.0.0-oap (declarations only:
 * native-sql-engine/cpp/src/third_party/gandiva/types.h:82-99).  Their published
 * semantics are Spark's Murmur3_x86_32:
 *   - hashInt(v, seed): one 4-byte block, length 4          (int8/16/32, bool, date32, float32 bits)
 *   - hashLong(v, seed): low 32 bits then high 32 bits, length 8 (int64, float64 bits)
 *     == native-sql-engine/cpp/src/third_party/murmurhash/murmurhash32.h:74-108
 *   - a null value returns the seed unchanged (the is_valid argument, types.h:88-97).
 * Floating-point keys are hashed by their raw IEEE bits (no NaN / -0.0 canonicalisation).
 * The partition id is Spark's pmod (splitter.cc:1456-1466).
 *
 * Only tests/, the smoke check and bench.py's CPU baseline use this file.
 */
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
extern "C++" {
namespace gzoracle {

static inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

static inline uint32_t mix_k1(uint32_t k1) {
  k1 *= 0xcc9e2d51u;
  k1 = rotl32(k1, 15);
  k1 *= 0x1b873593u;
  return k1;
}

static inline uint32_t mix_h1(uint32_t h1, uint32_t k1) {
  h1 ^= k1;
  h1 = rotl32(h1, 13);
  h1 = h1 * 5u + 0xe6546b64u;
  return h1;
}

static inline uint32_t fmix32(uint32_t h1, uint32_t length) {
  h1 ^= length;
  h1 ^= h1 >> 16;
  h1 *= 0x85ebca6bu;
  h1 ^= h1 >> 13;
  h1 *= 0xc2b2ae35u;
  h1 ^= h1 >> 16;
  return h1;
}

/* Spark Murmur3_x86_32.hashInt */
static inline int32_t spark_hash_int(int32_t v, int32_t seed) {
  uint32_t h1 = mix_h1((uint32_t)seed, mix_k1((uint32_t)v));
  return (int32_t)fmix32(h1, 4);
}

/* Spark Murmur3_x86_32.hashLong */
static inline int32_t spark_hash_long(int64_t v, int32_t seed) {
  uint64_t u = (uint64_t)v;
  uint32_t h1 = mix_h1((uint32_t)seed, mix_k1((uint32_t)(u & 0xffffffffu)));
  h1 = mix_h1(h1, mix_k1((uint32_t)(u >> 32)));
  return (int32_t)fmix32(h1, 8);
}

/* Generic MurmurHash3_x86_32 over a byte string (Austin Appleby's published algorithm,
 * little-endian blocks).  Used only to self-check hashInt/hashLong: for 4- and 8-byte
 * keys the two must agree. */
static inline uint32_t murmur3_x86_32(const void* key, int len, uint32_t seed) {
  const uint8_t* data = (const uint8_t*)key;
  const int nblocks = len / 4;
  uint32_t h1 = seed;
  for (int i = 0; i < nblocks; i++) {
    uint32_t k1;
    memcpy(&k1, data + 4 * i, 4);
    h1 = mix_h1(h1, mix_k1(k1));
  }
  const uint8_t* tail = data + nblocks * 4;
  uint32_t k1 = 0;
  switch (len & 3) {
    case 3: k1 ^= (uint32_t)tail[2] << 16; /* fall through */
    case 2: k1 ^= (uint32_t)tail[1] << 8;  /* fall through */
    case 1:
      k1 ^= tail[0];
      h1 ^= mix_k1(k1);
  }
  return fmix32(h1, (uint32_t)len);
}

/* Spark pmod(h, P) with P > 0 */
static inline int32_t spark_pmod(int32_t h, int32_t p) {
  int32_t r = h % p;
  return r < 0 ? r + p : r;
}

}  // namespace gzoracle
}
#endif
