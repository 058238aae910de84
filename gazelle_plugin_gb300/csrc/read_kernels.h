// Job lists of the reduce-side read kernels (read_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gz {

struct ByteJob {  // bytes [src, src + bytes) to dst
  const uint8_t* src;
  uint8_t* dst;
  uint64_t bytes;
};

struct OffsetJob {  // dst[i] = src[i] + add, i < n; int32 offsets, or int64 when wide
  const void* src;
  void* dst;
  uint32_t n;
  uint32_t wide;
  int64_t add;
};

struct BitJob {  // bits [src_bit, src_bit + nbits) of src (all ones when src is null) ORed into dst at dst_bit
  const uint32_t* src;
  uint32_t* dst;
  uint64_t src_bit;
  uint64_t dst_bit;
  uint64_t nbits;
};

// out[i] = *src[i] for n device addresses (host arrays; waits for nothing but the copies it
// enqueues: the caller synchronises `st` before reading out).
cudaError_t gather_words(const int32_t* const* src, int32_t* out, size_t n, cudaStream_t st);

// Runs the three job lists on `st` (the job arrays in device memory).
cudaError_t launch_read_jobs(const ByteJob* bytes, uint32_t n_bytes, const OffsetJob* offs, uint32_t n_offs,
                             const BitJob* bits, uint32_t n_bits, cudaStream_t st);

}  // namespace gz
