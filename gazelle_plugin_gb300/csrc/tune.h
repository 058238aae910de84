// gz::tune — pass options chosen by measurement, cached per schema signature.
//
// The device pass has two run-time knobs: its size (flush_bytes: input gathered before one pass)
// and the length of the segments k_hash_count and the plan work on (seg_tiles).  Small passes
// start sooner and overlap more with the host reads; large ones spread the per-pass plan and
// launch costs over more rows; long segments shrink the plan for many partitions.  gz_autotune
// times candidate settings on sample batches of a schema and keeps the fastest under the
// schema's signature (field types, key columns, partitions); a splitter made with flush_bytes 0
// and seg_tiles 0 takes the cached choice.  The cache lives in the process and can be saved to /
// loaded from a text file (one line per signature), and is read from $GZ_TUNE_CACHE on first use.
// Tile size, rows per warp and staging depth are compile-time constants of k_scatter.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "splitter.h"

namespace gz {

struct TuneChoice {
  int64_t flush_bytes = 0;
  int32_t seg_tiles = 0;
  double gbs = 0;  // input GB/s of the sample at this choice
};

// Cache key of a split: field types, key columns and partition count; partitioners other than
// "hash" are named in front and their keys dropped (they take none).
std::string SchemaSignature(const std::string& short_name, const std::vector<Field>& fields,
                            const std::vector<int32_t>& keys, int32_t P);
bool TuneLookup(const std::string& signature, TuneChoice* out);
void TuneStore(const std::string& signature, const TuneChoice& choice);
Status TuneSave(const std::string& path);
Status TuneLoad(const std::string& path);

}  // namespace gz
