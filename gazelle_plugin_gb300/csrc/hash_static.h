// Host side of the no-allocation partition-id entry point (hash_static.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

#include "../../include/gz_split.h"

namespace gz {

// Size of the file-scope per-tile count array: 4,194,304 32-bit counters (16 MiB).
constexpr size_t kStaticScratchWords = size_t(4) << 20;

// Enqueues the partition ids and per-partition row counts of one batch on `stream`; no device
// allocation.  On failure returns the status and sets *msg.
GzStatus HashPartitionStatic(int32_t device, int32_t P, const GzKeyColumn* keys, int32_t n_keys,
                             int32_t num_rows, uint16_t* pids, int64_t* counts, cudaStream_t stream,
                             std::string* msg);

}  // namespace gz
