// sm_103a kernels of the LZ4_FRAME shuffle codec: block compression (the map side, emitted
// record-batch buffers) and frame decoding (the reduce side).
//
// The reference compresses each body buffer of an emitted record batch with Arrow's
// Lz4FrameCodec (splitter.cc:311-327, 586-600) through the LZ4 library on one CPU core; the
// buffer is written as an int64 uncompressed length followed by one LZ4 frame.  Here the
// buffers are cut into chunks of at most 8 KiB, each staged in shared memory and compressed by
// one warp into one LZ4 block (greedy single-candidate matching, hash table in shared memory:
// every read of the match search is a shared-memory read; 12 KiB of shared memory per warp, 16
// warps per SM), and the host strings the blocks of a buffer into a frame (independent blocks,
// 64 KiB maximum block size in the descriptor, no checksums).  The search is bound by its
// dependent instruction chains, so its speed follows the warps per SM and the latency of its
// reads: against 64 KiB blocks searched in global memory, the Stop compression of the wide
// fact-table bodies runs 2.1x faster, for 1.9% more output (an 8 KiB history); 16 KiB blocks (8
// warps per SM) were 1.0x, 8 KiB blocks with a 4096-entry table (12 warps) 1.5x.  The output is
// a valid frame for any LZ4 frame decoder; it is not the same byte string the LZ4 library would
// produce (the codec's output is not unique).
//
// Formats (published LZ4 block / frame descriptions):
//   block    sequences of [token: literal length << 4 | match length - 4][literal length
//            bytes when >= 15][literals][offset, 2 bytes LE][match length bytes when >= 15];
//            the last sequence has literals only; a match starts at least 12 bytes before the
//            end of the block and the last 5 bytes are literals
//   frame    magic 0x184D2204, FLG, BD, header checksum, blocks [size (bit 31: stored)]
//            [payload], end mark 0
#include <cuda_runtime.h>
#include <stdint.h>

#include "lz4_kernels.h"

namespace gz {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 4;  // warps per CTA
constexpr int kHashLog = 11;
constexpr int kCWarps = 2;                       // warps per CTA of the compressor
constexpr uint32_t kStage = kLz4MaxBlock + 16;   // a warp's staged chunk (and a zero-padded word)
constexpr size_t kCompressSmem = (size_t)kCWarps * (kStage + (2u << kHashLog));
constexpr uint16_t kEmpty = 0xffff;  // no position (position 65535 never starts a match)

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// Little-endian 4 bytes at chunk position q: two aligned words of the source funnel-shifted.
// Both words hold bytes of the same source buffer (q + 4 <= len).
__device__ __forceinline__ uint32_t read32(const uint32_t* base, uint32_t sh0, uint32_t q) {
  const uint32_t i = sh0 + q;
  const uint32_t w0 = __ldg(base + (i >> 2));
  if ((i & 3) == 0) return w0;
  const uint32_t w1 = __ldg(base + (i >> 2) + 1);
  return __funnelshift_r(w0, w1, (i & 3) * 8);
}

__device__ __forceinline__ uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashLog); }

// Length bytes of a literal or match length field >= 15: (x - 15) as 255s and a last byte < 255.
__device__ __forceinline__ uint32_t ext_bytes(uint32_t x) { return x >= 15 ? (x - 15) / 255 + 1 : 0; }
__device__ __forceinline__ void put_ext(uint8_t* p, uint32_t x, uint32_t nb) {
  for (uint32_t i = lane_id(); i < nb; i += 32) p[i] = i + 1 < nb ? 255 : (uint8_t)((x - 15) - 255 * (nb - 1));
}

// One sequence at dst + o: literals src[anchor, anchor + lit) then (when off != 0) a match of
// mlen bytes at distance off.  Returns the new output position (the same in every lane).
__device__ uint32_t emit(uint8_t* dst, uint32_t o, const uint8_t* src, uint32_t anchor, uint32_t lit,
                         uint32_t off, uint32_t mlen) {
  const uint32_t ml = off ? mlen - 4 : 0;
  if (lane_id() == 0) dst[o] = (uint8_t)(((lit < 15 ? lit : 15) << 4) | (ml < 15 ? ml : 15));
  const uint32_t nl = ext_bytes(lit);
  put_ext(dst + o + 1, lit, nl);
  o += 1 + nl;
  for (uint32_t i = lane_id(); i < lit; i += 32) dst[o + i] = src[anchor + i];
  o += lit;
  if (off) {
    if (lane_id() == 0) {
      dst[o] = (uint8_t)(off & 255);
      dst[o + 1] = (uint8_t)(off >> 8);
    }
    const uint32_t nm = ext_bytes(ml);
    put_ext(dst + o + 2, ml, nm);
    o += 2 + nm;
  }
  return o;
}

// Compresses src[0, n) (n <= 65536) into dst (room for n + n / 255 + 16 bytes); returns the
// block's size.  Positions are scanned 32 at a time: every lane hashes its position's 4 bytes and
// looks up the last earlier position with that hash; the first lane whose candidate matches
// starts the match, which the warp then extends 32 bytes at a time.  Table entries come only from
// earlier windows (inserted after the lookups), so a candidate always precedes its position.
// Little-endian 4 bytes at position q of a staged (word-aligned, shared-memory) chunk.
__device__ __forceinline__ uint32_t read32_s(const uint32_t* sw, uint32_t q) {
  const uint32_t w0 = sw[q >> 2];
  return (q & 3) == 0 ? w0 : __funnelshift_r(w0, sw[(q >> 2) + 1], (q & 3) * 8);
}

__device__ uint32_t compress_block(const uint8_t* src, uint32_t n, uint16_t* table, uint8_t* dst) {
  const uint32_t lane = lane_id();
  const uint32_t* sw = reinterpret_cast<const uint32_t*>(src);  // the staged chunk (word aligned)
  uint32_t o = 0, anchor = 0, p = 0;
  uint32_t misses = 0;  // windows in a row without a match
  if (n >= 13) {
    for (uint32_t i = lane; i < (1u << kHashLog); i += 32) table[i] = kEmpty;
    __syncwarp();
    while (p + 12 <= n) {
      const uint32_t q = p + lane;
      const bool valid = q + 12 <= n;
      uint32_t v = 0, h = 0, cand = kEmpty;
      if (valid) {
        v = read32_s(sw, q);
        h = hash4(v);
        cand = table[h];
      }
      const bool ok = valid && cand != kEmpty && cand < q && read32_s(sw, cand) == v;
      const unsigned m = __ballot_sync(kFull, ok);
      __syncwarp();
      if (m == 0) {
        if (valid) table[h] = (uint16_t)q;
        __syncwarp();
        // acceleration (as LZ4's fast mode): the longer no match turns up, the further the next
        // window jumps, the positions in between staying literals; incompressible data costs a
        // fraction of a full scan
        misses++;
        p += 32u << min(misses >> 3, 4u);
        continue;
      }
      misses = 0;
      const uint32_t f = __ffs(m) - 1;
      if (valid && lane <= f) table[h] = (uint16_t)q;  // positions up to the match start only
      const uint32_t mq = p + f;
      const uint32_t mc = __shfl_sync(kFull, cand, f);
      __syncwarp();
      uint32_t len = 4;
      for (;;) {  // the match may end at n - 5 at the latest
        const uint32_t a = mq + len + lane;
        const bool eq = a + 5 < n && src[a] == src[mc + len + lane];
        const unsigned ne = __ballot_sync(kFull, !eq);
        if (ne == 0) {
          len += 32;
          continue;
        }
        len += __ffs(ne) - 1;
        break;
      }
      o = emit(dst, o, src, anchor, mq - anchor, mq - mc, len);
      p = mq + len;
      anchor = p;
    }
  }
  o = emit(dst, o, src, anchor, n - anchor, 0, 0);
  return o;
}

__global__ void __launch_bounds__(kCWarps * 32, 8)
k_lz4_compress(const Lz4Chunk* __restrict__ chunks, uint32_t n_chunks, uint32_t* next, uint8_t* scratch,
               uint8_t* out, unsigned long long* out_used, unsigned long long out_cap, Lz4Block* res,
               int32_t* err) {
  extern __shared__ __align__(16) uint8_t csm[];
  const uint32_t warp = threadIdx.x >> 5;
  uint8_t* sbuf = csm + (size_t)warp * (kStage + (2u << kHashLog));
  uint16_t* table = reinterpret_cast<uint16_t*>(sbuf + kStage);
  uint8_t* slot = scratch + (size_t)(blockIdx.x * kCWarps + warp) * kLz4Slot;
  for (;;) {
    uint32_t c = 0;
    if (lane_id() == 0) c = atomicAdd(next, 1u);
    c = __shfl_sync(kFull, c, 0);
    if (c >= n_chunks) return;
    const Lz4Chunk ch = chunks[c];
    const uint32_t n = ch.raw || ch.len <= kLz4MaxBlock ? ch.len : 0;  // the host cuts blocks to 64 KiB
    uint32_t size = n;
    if (!ch.raw) {
      // the chunk into this warp's shared buffer (then zeros up to two words past its end)
      const uintptr_t a = reinterpret_cast<uintptr_t>(ch.src);
      if ((a & 15) == 0) {
        const uint32_t nv = n >> 4;
        for (uint32_t i = lane_id(); i < nv; i += 32)
          reinterpret_cast<uint4*>(sbuf)[i] = __ldg(reinterpret_cast<const uint4*>(ch.src) + i);
        for (uint32_t i = (nv << 4) + lane_id(); i < n; i += 32) sbuf[i] = __ldg(ch.src + i);
      } else {
        for (uint32_t i = lane_id(); i < n; i += 32) sbuf[i] = __ldg(ch.src + i);
      }
      if (lane_id() < 8) sbuf[n + lane_id()] = 0;
      __syncwarp();
      size = compress_block(sbuf, n, table, slot);
      __syncwarp();
    }
    const bool stored = size >= n;  // a plain copy, or no gain: the block is stored as it is
    if (stored) size = n;
    unsigned long long pos = 0;
    if (lane_id() == 0) pos = atomicAdd(out_used, (unsigned long long)((size + 15) & ~15u));
    pos = __shfl_sync(kFull, pos, 0);
    if (pos + size > out_cap) {
      if (lane_id() == 0) {
        atomicOr(err, 1);
        res[c] = Lz4Block{0, 0, 0};
      }
      continue;
    }
    uint8_t* d = out + pos;  // 16-byte aligned, like the slot
    if (stored) {
      const uintptr_t a = reinterpret_cast<uintptr_t>(ch.src);
      if ((a & 15) == 0) {
        const uint32_t nv = n >> 4;
        for (uint32_t i = lane_id(); i < nv; i += 32)
          reinterpret_cast<uint4*>(d)[i] = __ldg(reinterpret_cast<const uint4*>(ch.src) + i);
        for (uint32_t i = (nv << 4) + lane_id(); i < n; i += 32) d[i] = __ldg(ch.src + i);
      } else if ((a & 3) == 0) {
        const uint32_t nv = n >> 2;
        for (uint32_t i = lane_id(); i < nv; i += 32)
          reinterpret_cast<uint32_t*>(d)[i] = __ldg(reinterpret_cast<const uint32_t*>(ch.src) + i);
        for (uint32_t i = (nv << 2) + lane_id(); i < n; i += 32) d[i] = __ldg(ch.src + i);
      } else {
        // unaligned source: aligned destination words, each a funnel shift of two aligned source
        // words (both hold bytes of the chunk), then the last bytes one by one
        const uint32_t* base = reinterpret_cast<const uint32_t*>(a & ~uintptr_t(3));
        const uint32_t sh = (uint32_t)(a & 3) * 8;
        const uint32_t nv = n >> 2;
        for (uint32_t i = lane_id(); i < nv; i += 32)
          reinterpret_cast<uint32_t*>(d)[i] = __funnelshift_r(__ldg(base + i), __ldg(base + i + 1), sh);
        for (uint32_t i = (nv << 2) + lane_id(); i < n; i += 32) d[i] = __ldg(ch.src + i);
      }
    } else {
      const uint32_t nv = size >> 4;
      for (uint32_t i = lane_id(); i < nv; i += 32)
        reinterpret_cast<uint4*>(d)[i] = reinterpret_cast<const uint4*>(slot)[i];
      for (uint32_t i = (nv << 4) + lane_id(); i < size; i += 32) d[i] = slot[i];
    }
    if (lane_id() == 0) res[c] = Lz4Block{pos, size, stored ? 1u : 0u};
    __syncwarp();
  }
}

// ---- decoding ---------------------------------------------------------------------------

// xxHash32 of a few bytes (the frame descriptor), seed 0: the published algorithm's path for
// inputs shorter than 16 bytes.
__device__ uint32_t xxh32_short(const uint8_t* p, uint32_t n) {
  constexpr uint32_t P1 = 2654435761u, P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;
  uint32_t h = P5 + n;
  uint32_t i = 0;
  for (; i + 4 <= n; i += 4) {
    const uint32_t w = (uint32_t)p[i] | (uint32_t)p[i + 1] << 8 | (uint32_t)p[i + 2] << 16 | (uint32_t)p[i + 3] << 24;
    h += w * P3;
    h = ((h << 17) | (h >> 15)) * P4;
  }
  for (; i < n; i++) {
    h += p[i] * P5;
    h = ((h << 11) | (h >> 21)) * P1;
  }
  h ^= h >> 15;
  h *= P2;
  h ^= h >> 13;
  h *= P3;
  h ^= h >> 16;
  return h;
}

__device__ __forceinline__ uint32_t le32(const uint8_t* p) {
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}

// Decodes one LZ4 block src[0, n) into dst at *op (capacity cap); matches may reach back into the
// frame's earlier blocks.  Every read and write is checked; false on malformed input.
__device__ bool decode_block(const uint8_t* src, uint32_t n, uint8_t* dst, uint64_t cap, uint64_t* op) {
  uint64_t o = *op;
  uint32_t ip = 0;
  while (ip < n) {
    const uint32_t token = src[ip++];
    uint32_t lit = token >> 4;
    if (lit == 15) {
      uint32_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        lit += b;
      } while (b == 255);
    }
    if (lit > n - ip || lit > cap - o) return false;
    for (uint32_t i = lane_id(); i < lit; i += 32) dst[o + i] = src[ip + i];
    ip += lit;
    o += lit;
    if (ip == n) break;
    if (n - ip < 2) return false;
    const uint32_t off = (uint32_t)src[ip] | (uint32_t)src[ip + 1] << 8;
    ip += 2;
    if (off == 0 || off > o) return false;
    uint32_t ml = token & 15;
    if (ml == 15) {
      uint32_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        ml += b;
      } while (b == 255);
    }
    ml += 4;
    if (ml > cap - o) return false;
    __syncwarp();  // the bytes a match copies are written
    // byte i of a match repeats byte i mod off of its source run, so overlapping copies read
    // only bytes written before the match
    for (uint32_t i = lane_id(); i < ml; i += 32) dst[o + i] = dst[o - off + (i % off)];
    __syncwarp();
    o += ml;
  }
  *op = o;
  return true;
}

__global__ void __launch_bounds__(kWarps * 32) k_lz4_decode(const Lz4Frame* __restrict__ frames, uint32_t n_frames,
                                                            int32_t* err) {
  const uint32_t warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
  for (uint32_t fi = warp; fi < n_frames; fi += gridDim.x * kWarps) {
    const Lz4Frame fr = frames[fi];
    const uint8_t* s = fr.src;
    const uint64_t n = fr.src_len;
    bool ok = n >= 7 && le32(s) == 0x184D2204u;
    uint64_t pos = 0, o = 0;
    bool block_sum = false, content_sum = false;
    if (ok) {
      const uint8_t flg = s[4], bd = s[5];
      block_sum = flg & 0x10;
      content_sum = flg & 0x04;
      pos = 6 + ((flg & 0x08) ? 8 : 0) + ((flg & 0x01) ? 4 : 0);
      ok = (flg >> 6) == 1 && (bd & 0x8F) == 0 && n > pos &&
           s[pos] == (uint8_t)((xxh32_short(s + 4, (uint32_t)(pos - 4)) >> 8) & 0xFF);
      pos++;
    }
    while (ok) {
      if (n - pos < 4) {
        ok = false;
        break;
      }
      const uint32_t bs = le32(s + pos);
      pos += 4;
      if (bs == 0) break;  // end mark
      const uint32_t sz = bs & 0x7FFFFFFFu;
      if (sz > n - pos || (block_sum && n - pos - sz < 4)) {
        ok = false;
        break;
      }
      if (bs & 0x80000000u) {  // stored
        if (sz > fr.dst_len - o) {
          ok = false;
          break;
        }
        for (uint32_t i = lane_id(); i < sz; i += 32) fr.dst[o + i] = s[pos + i];
        o += sz;
      } else {
        ok = decode_block(s + pos, sz, fr.dst, fr.dst_len, &o);
      }
      pos += sz + (block_sum ? 4 : 0);
      __syncwarp();
    }
    // (content checksums are skipped, not verified)
    if (ok && content_sum && n - pos < 4) ok = false;
    if (!(ok && o == fr.dst_len) && lane_id() == 0) atomicOr(err, 1);
    __syncwarp();
  }
}

int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  }
  return sms;
}

}  // namespace

uint32_t lz4_compress_warps() { return (uint32_t)sm_count() * 8 * kCWarps; }

cudaError_t launch_lz4_compress(const Lz4Chunk* chunks, uint32_t n_chunks, uint32_t* next, uint8_t* scratch,
                                uint8_t* out, unsigned long long* out_used, unsigned long long out_cap,
                                Lz4Block* res, int32_t* err, cudaStream_t st) {
  if (n_chunks == 0) return cudaSuccess;
  const uint32_t grid = lz4_compress_warps() / kCWarps;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_lz4_compress, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCompressSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_lz4_compress<<<grid, kCWarps * 32, kCompressSmem, st>>>(chunks, n_chunks, next, scratch, out, out_used, out_cap, res, err);
  return cudaGetLastError();
}

cudaError_t launch_lz4_decode(const Lz4Frame* frames, uint32_t n_frames, int32_t* err, cudaStream_t st) {
  if (n_frames == 0) return cudaSuccess;
  const uint32_t need = (n_frames + kWarps - 1) / kWarps;
  const uint32_t cap = (uint32_t)sm_count() * 16;
  k_lz4_decode<<<need < cap ? need : cap, kWarps * 32, 0, st>>>(frames, n_frames, err);
  return cudaGetLastError();
}

}  // namespace gz
