/*
 * ORACLE - test infrastructure only.
 *
 * A CPU restatement of the decoding side of the LZ4 frame format (the codec the reference's
 * LZ4_FRAME shuffle compression writes through Arrow's Lz4FrameCodec, splitter.cc:311-327,
 * 586-600) and of the IPC body compression around it: each compressed body buffer is an int64
 * little-endian uncompressed length followed by one LZ4 frame (length -1: the bytes follow
 * uncompressed).  Written from the published LZ4 frame and block format descriptions and the
 * published xxHash32 algorithm (the frame header checksum); pinned against the LZ4 library that
 * pyarrow ships in the CPU tests.  Used to check the CUDA compressor's output.
 *
 * Only tests/ and bench.py's CPU leg use this file.
 */
#include <stdint.h>
#include <string.h>

namespace {

inline uint32_t Rotl(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
inline uint32_t Le32(const uint8_t* p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }

constexpr uint32_t P1 = 2654435761u, P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;

uint32_t Xxh32(const uint8_t* p, size_t n, uint32_t seed) {
  const uint8_t* end = p + n;
  uint32_t h;
  if (n >= 16) {
    uint32_t v1 = seed + P1 + P2, v2 = seed + P2, v3 = seed, v4 = seed - P1;
    const uint8_t* limit = end - 16;
    do {
      v1 = Rotl(v1 + Le32(p) * P2, 13) * P1;
      v2 = Rotl(v2 + Le32(p + 4) * P2, 13) * P1;
      v3 = Rotl(v3 + Le32(p + 8) * P2, 13) * P1;
      v4 = Rotl(v4 + Le32(p + 12) * P2, 13) * P1;
      p += 16;
    } while (p <= limit);
    h = Rotl(v1, 1) + Rotl(v2, 7) + Rotl(v3, 12) + Rotl(v4, 18);
  } else {
    h = seed + P5;
  }
  h += (uint32_t)n;
  for (; p + 4 <= end; p += 4) h = Rotl(h + Le32(p) * P3, 17) * P4;
  for (; p < end; p++) h = Rotl(h + (*p) * P5, 11) * P1;
  h ^= h >> 15;
  h *= P2;
  h ^= h >> 13;
  h *= P3;
  h ^= h >> 16;
  return h;
}

// One LZ4 block (sequences of token, literals, offset, match) appended at out[*op]; matches may
// reach back into earlier blocks of the same output (linked blocks).  false on malformed input.
bool DecodeBlock(const uint8_t* ip, size_t n, uint8_t* out, size_t cap, size_t* op) {
  const uint8_t* iend = ip + n;
  size_t o = *op;
  while (ip < iend) {
    const uint8_t token = *ip++;
    size_t lit = token >> 4;
    if (lit == 15) {
      uint8_t b;
      do {
        if (ip >= iend) return false;
        b = *ip++;
        lit += b;
      } while (b == 255);
    }
    if ((size_t)(iend - ip) < lit || cap - o < lit) return false;
    memcpy(out + o, ip, lit);
    ip += lit;
    o += lit;
    if (ip == iend) break;  // the last sequence ends with its literals
    if (iend - ip < 2) return false;
    const size_t off = (size_t)ip[0] | (size_t)ip[1] << 8;
    ip += 2;
    if (off == 0 || off > o) return false;
    size_t ml = token & 15;
    if (ml == 15) {
      uint8_t b;
      do {
        if (ip >= iend) return false;
        b = *ip++;
        ml += b;
      } while (b == 255);
    }
    ml += 4;
    if (cap - o < ml) return false;
    for (size_t i = 0; i < ml; i++) out[o + i] = out[o - off + i];  // may overlap
    o += ml;
  }
  *op = o;
  return true;
}

}  // namespace

extern "C" {

uint32_t gzo_xxh32(const uint8_t* p, int64_t n, uint32_t seed) { return Xxh32(p, (size_t)n, seed); }

/* Decodes one LZ4 frame of `n` bytes into dst (capacity cap); returns the decoded size, or -1
 * when the frame is malformed (bad magic, header checksum, block or content checksum). */
int64_t gzo_lz4f_decompress(const uint8_t* src, int64_t n, uint8_t* dst, int64_t cap) {
  if (n < 7 || Le32(src) != 0x184D2204u) return -1;
  const uint8_t flg = src[4], bd = src[5];
  if ((flg >> 6) != 1 || (bd & 0x8F) != 0) return -1;
  const bool block_checksum = flg & 0x10, content_size = flg & 0x08, content_checksum = flg & 0x04,
             dict_id = flg & 0x01;
  size_t pos = 6 + (content_size ? 8 : 0) + (dict_id ? 4 : 0);
  if ((size_t)n < pos + 1) return -1;
  if (src[pos] != (uint8_t)((Xxh32(src + 4, pos - 4, 0) >> 8) & 0xFF)) return -1;
  pos++;
  size_t o = 0;
  for (;;) {
    if ((size_t)n < pos + 4) return -1;
    const uint32_t bs = Le32(src + pos);
    pos += 4;
    if (bs == 0) break;  // end mark
    const size_t sz = bs & 0x7FFFFFFFu;
    if ((size_t)n < pos + sz + (block_checksum ? 4 : 0)) return -1;
    if (block_checksum && Le32(src + pos + sz) != Xxh32(src + pos, sz, 0)) return -1;
    if (bs & 0x80000000u) {  // stored uncompressed
      if ((size_t)cap - o < sz) return -1;
      memcpy(dst + o, src + pos, sz);
      o += sz;
    } else if (!DecodeBlock(src + pos, sz, dst, (size_t)cap, &o)) {
      return -1;
    }
    pos += sz + (block_checksum ? 4 : 0);
  }
  if (content_checksum) {
    if ((size_t)n < pos + 4 || Le32(src + pos) != Xxh32(dst, o, 0)) return -1;
    pos += 4;
  }
  if (content_size) {
    uint64_t cs;
    memcpy(&cs, src + 6, 8);
    if (cs != o) return -1;
  }
  return (int64_t)o;
}

}  // extern "C"
