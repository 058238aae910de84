// Partition ids of one device-resident batch, computed without allocating device memory
// (C entry point gz_hash_partition_static).
//
// The hash chain and pmod are the splitter's (k_hash_count, restating
// HashSplitter::ComputeAndCountPartitionId, native-sql-engine/cpp/src/shuffle/splitter.cc:1440-1470).
// k_hash_count counts rows per (tile, partition) in memory the splitter allocates for each
// device pass; here those per-tile counts live in one file-scope device array of fixed size, so
// that callers which may not allocate device memory can run the kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "gz_engine.cuh"
#include "gz_hash.cuh"
#include "hash_static.h"

namespace gz {
namespace {

using namespace hash;

constexpr uint32_t kTile = 1024;     // rows per CTA
constexpr uint32_t kThreads = 256;
constexpr uint32_t kSmemHistMaxP = 12288;  // a tile's histogram stays in shared memory (48 KB)

// Per-tile row counts, [tile][partition], of the most recent call on this device.  Every call
// shares it and it keeps the last call's contents: each CTA clears the row it owns before it
// counts.  Host code reaches it only through the address cudaGetSymbolAddress returns.
static __device__ __align__(256) uint32_t g_tile_counts[kStaticScratchWords];

struct KeySet {
  const uint8_t* validity[kMaxKeys];
  const uint8_t* values[kMaxKeys];
  int32_t kind[kMaxKeys];
  int32_t n;
};

// One CTA per 1024-row tile: partition id of every row, and the tile's row count per partition
// into row blockIdx.x of `tile_counts`.
__global__ void __launch_bounds__(kThreads)
k_hash_count_static(const KeySet keys, uint32_t nrows, uint32_t P, unsigned long long M,
                    int hist_in_smem, uint16_t* __restrict__ pids, uint32_t* __restrict__ tile_counts) {
  extern __shared__ uint32_t smem[];
  const uint32_t row0 = blockIdx.x * kTile;
  const uint32_t n = min(kTile, nrows - row0);
  uint32_t* row = tile_counts + (size_t)blockIdx.x * P;
  uint32_t* H = hist_in_smem ? smem : row;
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) H[i] = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint32_t r = row0 + i;
    int32_t h = 42;
    for (int k = 0; k < keys.n; k++) {
      const uint8_t* valid = keys.validity[k];
      if (valid != nullptr && !get_bit(valid, r)) continue;  // null: the seed passes through
      const uint8_t* v = keys.values[k];
      switch (keys.kind[k]) {
        case KEY_I32: h = hash_int(reinterpret_cast<const int32_t*>(v)[r], h); break;
        case KEY_I64: h = hash_long(reinterpret_cast<const int64_t*>(v)[r], h); break;
        case KEY_I8: h = hash_int(reinterpret_cast<const int8_t*>(v)[r], h); break;
        case KEY_I16: h = hash_int(reinterpret_cast<const int16_t*>(v)[r], h); break;
        default: h = hash_int(get_bit(v, r) ? 1 : 0, h); break;
      }
    }
    const uint32_t p = fast_pmod(h, P, M);
    pids[r] = (uint16_t)p;
    atomicAdd(&H[p], 1u);
  }
  if (hist_in_smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) row[i] = H[i];
  }
}

// counts[p] = sum over tiles of tile_counts[t][p].  Block (32, 32): x picks the partition,
// y strides over the tiles; the 32 partial sums of a partition are added in shared memory.
__global__ void __launch_bounds__(1024)
k_sum_tile_counts(const uint32_t* __restrict__ tile_counts, uint32_t n_tiles, uint32_t P,
                  int64_t* __restrict__ counts) {
  __shared__ unsigned long long part[32][33];
  const uint32_t p = blockIdx.x * 32 + threadIdx.x;
  unsigned long long s = 0;
  if (p < P)
    for (uint32_t t = threadIdx.y; t < n_tiles; t += 32) s += tile_counts[(size_t)t * P + p];
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && p < P) {
    unsigned long long tot = 0;
    for (int y = 0; y < 32; y++) tot += part[y][threadIdx.x];
    counts[p] = (int64_t)tot;
  }
}

std::mutex g_mu;
// device address of g_tile_counts, per device ordinal, in that device's primary context (the
// one the runtime API uses; other contexts are not supported)
std::vector<uint32_t*> g_addr;

// Looks up (once per device, with `device` current) the device address of g_tile_counts.
cudaError_t ScratchAddress(int device, uint32_t** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_addr.size() <= device) g_addr.resize(device + 1, nullptr);
  if (g_addr[device] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_tile_counts);
    if (e != cudaSuccess) return e;
    g_addr[device] = static_cast<uint32_t*>(p);
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace

GzStatus HashPartitionStatic(int32_t device, int32_t P, const GzKeyColumn* keys, int32_t n_keys,
                             int32_t num_rows, uint16_t* pids, int64_t* counts, cudaStream_t stream,
                             std::string* msg) {
  if (P < 1 || P > 65536) {
    *msg = "num_partitions must be in [1, 65536], got " + std::to_string(P);
    return GZ_INVALID;
  }
  if (keys == nullptr || n_keys < 1 || n_keys > kMaxKeys) {
    *msg = "need 1 to " + std::to_string(kMaxKeys) + " key columns";
    return GZ_INVALID;
  }
  if (num_rows < 0 || counts == nullptr || (num_rows > 0 && pids == nullptr)) {
    *msg = "num_rows must be >= 0 and the output pointers non-null";
    return GZ_INVALID;
  }
  // A null-type key has no hash function and leaves the chain unchanged (the NullType case of
  // HashSplitter::CreateProjector, splitter.cc:1407-1408): it takes no slot of the key list.
  KeySet ks{};
  ks.n = 0;
  for (int k = 0; k < n_keys; k++) {
    if (keys[k].type == GZ_TYPE_NULL) continue;
    int kind;
    switch (keys[k].type) {
      case GZ_TYPE_BOOL: kind = KEY_BOOL; break;
      case GZ_TYPE_INT8: kind = KEY_I8; break;
      case GZ_TYPE_INT16: kind = KEY_I16; break;
      case GZ_TYPE_INT32: case GZ_TYPE_FLOAT32: case GZ_TYPE_DATE32: kind = KEY_I32; break;
      case GZ_TYPE_INT64: case GZ_TYPE_FLOAT64: kind = KEY_I64; break;
      default:
        *msg = "key " + std::to_string(k) + ": type " + std::to_string(keys[k].type) +
               " has no Spark-compatible hash here";
        return GZ_NOT_IMPLEMENTED;
    }
    if (num_rows > 0 && keys[k].values == nullptr) {
      *msg = "key " + std::to_string(k) + ": null values pointer";
      return GZ_INVALID;
    }
    ks.kind[ks.n] = kind;
    ks.validity[ks.n] = keys[k].validity;
    ks.values[ks.n] = keys[k].values;
    ks.n++;
  }
  const uint64_t n_tiles = ((uint64_t)num_rows + kTile - 1) / kTile;
  if (n_tiles * (uint64_t)P > kStaticScratchWords) {
    *msg = std::to_string(num_rows) + " rows x " + std::to_string(P) + " partitions need " +
           std::to_string(n_tiles * (uint64_t)P) + " per-tile counters; the static scratch holds " +
           std::to_string(kStaticScratchWords) + " (16 MiB): split the batch into smaller calls";
    return GZ_INVALID;
  }

  // An error already pending on this thread came from the caller's earlier work, not from this
  // call: report it as such (and leave it pending) instead of taking it for a launch failure.
  {
    const cudaError_t before = cudaPeekAtLastError();
    if (before != cudaSuccess) {
      *msg = std::string("a CUDA error from earlier work on this thread is pending (nothing was "
                         "launched): ") + cudaGetErrorString(before);
      return GZ_CUDA;
    }
  }
  int prev = -1;
  cudaError_t e = cudaGetDevice(&prev);
  if (e == cudaSuccess) e = cudaSetDevice(device);
  uint32_t* scratch = nullptr;
  if (e == cudaSuccess) {
    e = ScratchAddress(device, &scratch);
    if (e == cudaErrorMemoryAllocation) {
      // with lazy module loading the array is reserved here, on the first call on a device
      cudaGetLastError();
      if (prev >= 0 && prev != device) cudaSetDevice(prev);
      *msg = "out of device memory reserving the library's 16 MiB static scratch array on device " +
             std::to_string(device) + ": make the first call on each device before reserving its free memory";
      return GZ_OOM;
    }
  }
  if (e == cudaSuccess && n_tiles > 0) {
    const int smem_hist = P <= (int32_t)kSmemHistMaxP;
    const size_t sm = smem_hist ? sizeof(uint32_t) * P : 0;
    const unsigned long long M = P > 1 ? UINT64_MAX / (uint64_t)P + 1 : 0;
    k_hash_count_static<<<(unsigned)n_tiles, kThreads, sm, stream>>>(ks, (uint32_t)num_rows, (uint32_t)P,
                                                                      M, smem_hist, pids, scratch);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_sum_tile_counts<<<(P + 31) / 32, dim3(32, 32), 0, stream>>>(scratch, (uint32_t)n_tiles,
                                                                  (uint32_t)P, counts);
    e = cudaGetLastError();
  }
  if (prev >= 0 && prev != device) {
    cudaError_t e2 = cudaSetDevice(prev);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) {
    *msg = std::string("CUDA error: ") + cudaGetErrorString(e);
    return GZ_CUDA;
  }
  return GZ_OK;
}

}  // namespace gz
