// sm_103a kernels of the reduce-side read (PartitionReader): the record batches of a partition's
// IPC streams, already in HBM, concatenated into one set of Arrow columns.  Three job lists, each
// job at most a few hundred KB so that one CTA per job keeps every SM busy:
//   byte jobs   values of fixed-width columns and characters of binary columns, copied
//   offset jobs binary offsets (int32, or int64 of the large types) rebased:
//               out[i] = in[i] - in[0] + (the batch's first character)
//   bit jobs    validity / bool bits moved to their row in the output (OR into zeroed words;
//               a batch without a validity buffer contributes ones)
#include <cuda_runtime.h>
#include <stdint.h>

#include "read_kernels.h"

namespace gz {

namespace {

constexpr int kThreads = 256;

template <typename V>
__device__ __forceinline__ void copy_words(const uint8_t* src, uint8_t* dst, uint64_t n) {
  constexpr uint32_t W = sizeof(V);
  const uint64_t lead = (W - (reinterpret_cast<uintptr_t>(src) & (W - 1))) & (W - 1);
  const uint64_t head = n < lead ? n : lead;
  if (threadIdx.x < head) dst[threadIdx.x] = src[threadIdx.x];
  const uint64_t nv = (n - head) / W;
  const V* sv = reinterpret_cast<const V*>(src + head);
  V* dv = reinterpret_cast<V*>(dst + head);
  for (uint64_t i = threadIdx.x; i < nv; i += kThreads) dv[i] = sv[i];
  for (uint64_t j = head + nv * W + threadIdx.x; j < n; j += kThreads) dst[j] = src[j];
}

__global__ void __launch_bounds__(kThreads) k_read_bytes(const ByteJob* __restrict__ jobs, uint32_t n_jobs) {
  for (uint32_t b = blockIdx.x; b < n_jobs; b += gridDim.x) {
    const ByteJob job = jobs[b];
    const uintptr_t phase = reinterpret_cast<uintptr_t>(job.src) ^ reinterpret_cast<uintptr_t>(job.dst);
    if ((phase & 15) == 0) copy_words<uint4>(job.src, job.dst, job.bytes);
    else if ((phase & 7) == 0) copy_words<uint2>(job.src, job.dst, job.bytes);
    else if ((phase & 3) == 0) copy_words<uint32_t>(job.src, job.dst, job.bytes);
    else
      for (uint64_t j = threadIdx.x; j < job.bytes; j += kThreads) job.dst[j] = job.src[j];
  }
}

__global__ void __launch_bounds__(kThreads) k_read_offsets(const OffsetJob* __restrict__ jobs, uint32_t n_jobs) {
  for (uint32_t b = blockIdx.x; b < n_jobs; b += gridDim.x) {
    const OffsetJob job = jobs[b];
    if (job.wide) {
      const int64_t* src = static_cast<const int64_t*>(job.src);
      int64_t* dst = static_cast<int64_t*>(job.dst);
      for (uint32_t i = threadIdx.x; i < job.n; i += kThreads) dst[i] = src[i] + job.add;
    } else {
      const int32_t* src = static_cast<const int32_t*>(job.src);
      int32_t* dst = static_cast<int32_t*>(job.dst);
      const int32_t add = (int32_t)job.add;
      for (uint32_t i = threadIdx.x; i < job.n; i += kThreads) dst[i] = src[i] + add;
    }
  }
}

// Bits [start, start + len) of `src` (len <= 32) as the low bits of a word.  Reads only the 4-byte
// words that hold those bits.
__device__ __forceinline__ uint32_t extract_bits(const uint32_t* src, uint64_t start, uint32_t len) {
  const uint64_t w = start >> 5;
  const uint32_t sh = (uint32_t)(start & 31);
  uint32_t v = src[w] >> sh;
  if (sh + len > 32) v |= src[w + 1] << (32 - sh);
  return len == 32 ? v : v & ((1u << len) - 1);
}

__global__ void __launch_bounds__(kThreads) k_read_bits(const BitJob* __restrict__ jobs, uint32_t n_jobs) {
  for (uint32_t b = blockIdx.x; b < n_jobs; b += gridDim.x) {
    const BitJob job = jobs[b];
    if (job.nbits == 0) continue;
    const uint64_t d0 = job.dst_bit, d1 = job.dst_bit + job.nbits;
    const uint64_t w0 = d0 >> 5, w1 = (d1 - 1) >> 5;
    for (uint64_t w = w0 + threadIdx.x; w <= w1; w += kThreads) {
      const uint64_t lo = w * 32 > d0 ? w * 32 : d0;
      const uint64_t hi = w * 32 + 32 < d1 ? w * 32 + 32 : d1;
      const uint32_t len = (uint32_t)(hi - lo);
      const uint32_t bits = job.src ? extract_bits(job.src, job.src_bit + (lo - d0), len)
                                    : (len == 32 ? 0xffffffffu : (1u << len) - 1);
      if (bits) atomicOr(job.dst + w, bits << (uint32_t)(lo - w * 32));
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_read_words(const int32_t* const* __restrict__ src, int32_t* out, size_t n) {
  for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kThreads) out[i] = *src[i];
}

unsigned grid_for(uint32_t n_jobs) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  }
  const uint32_t cap = 8u * (uint32_t)sms;
  return n_jobs < cap ? n_jobs : cap;
}

}  // namespace

cudaError_t gather_words(const int32_t* const* src, int32_t* out, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  uint8_t* d = nullptr;
  const size_t pb = (n * sizeof(void*) + 255) / 256 * 256;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d), pb + n * sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(d, src, n * sizeof(void*), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    const size_t blocks = (n + kThreads - 1) / kThreads;
    k_read_words<<<blocks < 1024 ? (unsigned)blocks : 1024u, kThreads, 0, st>>>(
        reinterpret_cast<const int32_t* const*>(d), reinterpret_cast<int32_t*>(d + pb), n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + pb, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  return e;
}

cudaError_t launch_read_jobs(const ByteJob* bytes, uint32_t n_bytes, const OffsetJob* offs, uint32_t n_offs,
                             const BitJob* bits, uint32_t n_bits, cudaStream_t st) {
  if (n_bytes) k_read_bytes<<<grid_for(n_bytes), kThreads, 0, st>>>(bytes, n_bytes);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (n_offs) k_read_offsets<<<grid_for(n_offs), kThreads, 0, st>>>(offs, n_offs);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (n_bits) k_read_bits<<<grid_for(n_bits), kThreads, 0, st>>>(bits, n_bits);
  return cudaGetLastError();
}

}  // namespace gz
