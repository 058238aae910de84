// Small helpers shared by the splitter's translation units (splitter.cc, splitter_nested.cc).
#pragma once
#include <stdint.h>
#include <string.h>

#include <stddef.h>

#include "../../include/gz_split.h"

namespace gz {

inline int64_t BytesForBits(int64_t n) { return (n + 7) >> 3; }
inline size_t AlignUp(size_t x, size_t a) { return (x + a - 1) / a * a; }

inline int ByteWidth(int t) {
  switch (t) {
    case GZ_TYPE_INT8: case GZ_TYPE_UINT8: return 1;
    case GZ_TYPE_INT16: case GZ_TYPE_UINT16: case GZ_TYPE_HALF_FLOAT: return 2;
    case GZ_TYPE_INT32: case GZ_TYPE_UINT32: case GZ_TYPE_FLOAT32: case GZ_TYPE_DATE32:
    case GZ_TYPE_TIME32: return 4;
    case GZ_TYPE_INT64: case GZ_TYPE_UINT64: case GZ_TYPE_FLOAT64: case GZ_TYPE_DATE64:
    case GZ_TYPE_TIME64: case GZ_TYPE_TIMESTAMP: return 8;
    case GZ_TYPE_DECIMAL128: return 16;
    default: return 0;
  }
}
inline bool IsBinary(int t) {
  return t == GZ_TYPE_STRING || t == GZ_TYPE_BINARY || t == GZ_TYPE_LARGE_STRING || t == GZ_TYPE_LARGE_BINARY;
}
// Bytes of one offset of a binary column: int32, or int64 for LargeBinary / LargeString
// (splitter.cc:480-516, 626-629, 1291-1299)
inline int OffW(int t) { return t == GZ_TYPE_LARGE_STRING || t == GZ_TYPE_LARGE_BINARY ? 8 : 4; }
// Offset r of an offsets buffer of width w, as int64
inline int64_t OffAt(const uint8_t* off, int w, size_t r) {
  if (w == 8) {
    int64_t v;
    memcpy(&v, off + r * 8, 8);
    return v;
  }
  int32_t v;
  memcpy(&v, off + r * 4, 4);
  return v;
}

// Copies `nbits` bits from src (starting at bit `sbit`) to dst (starting at bit `dbit`);
// dst bits outside the range are left as they are.
inline void CopyBits(const uint8_t* src, uint64_t sbit, uint8_t* dst, uint64_t dbit, uint64_t nbits) {
  for (uint64_t i = 0; i < nbits; i++) {
    const uint64_t s = sbit + i, d = dbit + i;
    const uint8_t b = (src[s >> 3] >> (s & 7)) & 1;
    if (b) dst[d >> 3] |= (uint8_t)(1u << (d & 7));
    else dst[d >> 3] &= (uint8_t)~(1u << (d & 7));
  }
}

inline int64_t CountZeros(const uint8_t* bits, int64_t n) {
  int64_t ones = 0;
  int64_t full = n >> 3;
  for (int64_t i = 0; i < full; i++) ones += __builtin_popcount(bits[i]);
  for (int64_t i = full * 8; i < n; i++) ones += (bits[i >> 3] >> (i & 7)) & 1;
  return n - ones;
}

}  // namespace gz
