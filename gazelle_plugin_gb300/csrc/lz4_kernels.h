// LZ4_FRAME codec kernels (lz4_kernels.cu): block compression of buffer chunks and frame decoding.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gz {

constexpr uint32_t kLz4MaxBlock = 8192;  // bytes of input per block (at most the frame's 64 KiB block size)
// worst-case compressed block (all literals: token, length bytes) rounded to 16 bytes
constexpr uint32_t kLz4Slot = ((kLz4MaxBlock + kLz4MaxBlock / 255 + 16) + 15) & ~15u;

struct Lz4Chunk {  // one block's input: 1 .. kLz4MaxBlock bytes (raw: any length, copied as it is)
  const uint8_t* src;
  uint32_t len;
  uint32_t raw;
};

struct Lz4Block {  // where a chunk's block landed in the output arena
  uint64_t pos;      // 16-byte aligned
  uint32_t size;     // payload bytes
  uint32_t stored;   // 1: the payload is the input itself (the frame marks it uncompressed)
};

struct Lz4Frame {  // one frame to decode: src_len bytes into exactly dst_len bytes
  const uint8_t* src;
  uint64_t src_len;
  uint8_t* dst;
  uint64_t dst_len;
};

// Warps of the compression grid (each needs kLz4Slot bytes of scratch).
uint32_t lz4_compress_warps();

// Compresses every chunk into the arena `out` (out_cap bytes; *out_used is the bump counter,
// *next the work counter, both zero at launch); res[c] tells where chunk c went.  *err gets bit
// 0 when the arena ran out.
cudaError_t launch_lz4_compress(const Lz4Chunk* chunks, uint32_t n_chunks, uint32_t* next, uint8_t* scratch,
                                uint8_t* out, unsigned long long* out_used, unsigned long long out_cap,
                                Lz4Block* res, int32_t* err, cudaStream_t st);

// Decodes every frame; *err gets bit 0 for a malformed frame or a size that differs.
cudaError_t launch_lz4_decode(const Lz4Frame* frames, uint32_t n_frames, int32_t* err, cudaStream_t st);

}  // namespace gz
