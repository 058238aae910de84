// Shared host/device definitions of the GB300 hash-split engine.
//
// One "flush" is a device pass over a group of consecutive input batches:
//   k_hash_count : the partition id of every row (Spark Murmur3 chain + pmod, the running
//                  round-robin selection, or the range partitioner's id column), per-segment
//                  partition histograms (rows, and bytes of every utf8 column), null counts
//   k_plan       : per-partition walk over the flush's batches that restates the reference
//                  buffer policy (allocate / emit / reuse, validity presence) and turns the
//                  histograms into destination offsets; then scans over partitions
//   k_scatter    : per 1024-row tile, a stable counting sort by partition id in shared memory,
//                  then a coalesced scatter of every column into partition-contiguous output
// A segment is up to seg_tiles consecutive tiles of one batch (a batch is cut into equal
// segments): the unit of k_hash_count and of the plan's offsets.  k_hash_count also records, for every tile after the first of its
// segment, how many rows and bytes each partition received from the segment's earlier tiles, so
// each k_scatter CTA (one tile) finds its destinations without the others.
// Output of a flush, per array column, is partition-major: all rows of partition 0 in input
// order, then partition 1, ...  An emitted record batch (reference CacheRecordBatch) is a
// contiguous row range of one partition, possibly continued from the previous flush.
#pragma once
#include <stdint.h>

namespace gz {

constexpr int kMaxKeys = 8;
constexpr int kMaxCols = 64;    // array columns (fixed + bool + binary)
constexpr int kMaxSchemaCols = 256;
constexpr int kTileRows = 1024; // rows per k_scatter tile
constexpr int kMaxSegTiles = 32;  // tiles per segment
constexpr size_t kHistSmemBytes = 96 * 1024;  // k_hash_count's histograms in shared memory up to this
constexpr int kScatterThreads = 256;
constexpr int kPlanThreads = 1024;
constexpr int kMaxBatchesPerFlush = 4096;

enum KeyKind : int32_t { KEY_I32 = 0, KEY_I64 = 1, KEY_I8 = 2, KEY_I16 = 3, KEY_BOOL = 4, KEY_STR = 5 };
// Splitter::Make short names (native-sql-engine/cpp/src/shuffle/splitter.cc:190-208):
// "hash" (HashSplitter), "rr" and "single" (RoundRobinSplitter, single = 1 partition),
// "range" (FallbackRangeSplitter: int32 ids in schema field 0, key_col[0] = 0)
enum Partitioner : int32_t { PART_HASH = 0, PART_RR = 1, PART_RANGE = 2 };
enum ColKind : int32_t { COL_FIXED = 0, COL_BOOL = 1, COL_BINARY = 2 };

// Static description of the split, copied to the device once at make.
struct SchemaDesc {
  int32_t P;
  int32_t n_cols;      // schema fields, including null-type fields
  int32_t n_array;     // array columns: fixed (incl. bool) first, then binary (splitter.cc:246-269)
  int32_t n_fixed;     // fixed_width_col_cnt_
  int32_t n_str;       // binary columns
  int32_t n_keys;
  int32_t prefer_spill;
  int32_t partitioner;  // Partitioner
  uint64_t quirk_mask;  // array columns a with array_idx_[a] < fixed_width_col_cnt_ (splitter.cc:878-886)
  uint64_t pmod_magic;  // floor((2^64 - 1) / P) + 1, for the pmod without a divide
  int32_t key_col[kMaxKeys];
  int32_t key_kind[kMaxKeys];
  int32_t arr_col[kMaxCols];    // schema index of array column a
  int32_t arr_kind[kMaxCols];   // ColKind
  int32_t arr_width[kMaxCols];  // value bytes of a fixed column; offset bytes (4 / 8) of a binary one
  int32_t arr_str[kMaxCols];    // binary ordinal k of a binary column, -1 otherwise
  int32_t order[kMaxCols];      // order in which k_scatter processes the array columns
  // list columns (binary-like, after the binary ones): their "characters" are the element
  // values, a row's byte length is its element count << arr_shift, and a null row has none
  int32_t arr_shift[kMaxCols];
  uint64_t list_mask;           // array columns that are lists
  uint64_t listbit_mask;        // lists of bool elements: one bit each; their "characters" are the
                                // element indices and out_chars is a bit region (0xff-filled)
  uint64_t nopay_mask;          // list-like columns whose elements carry no values (struct entries:
                                // their element validity only; also in listbit_mask)
};

// Device addresses of one input column of one batch.  offsets only for binary columns (int32,
// or int64 for large binary columns: arr_width 8); validity == nullptr means an empty validity
// buffer (no nulls).
struct ColPtr {
  const uint8_t* validity;
  const int32_t* offsets;
  const uint8_t* values;
  uint64_t values_bytes;  // readable bytes at `values` (binary columns: offsets are checked)
  const uint8_t* child_validity;  // list: the elements' validity bitmap; nullptr: none
};

// One input buffer the device copies out of host memory (a coherent host-device link lets
// kernels read host addresses): `bytes` from `src` (host) to `dst` (device staging).
struct HostCopy {
  const uint8_t* src;
  uint8_t* dst;
  uint64_t bytes;
};

// bits of FlushDesc::err
constexpr int32_t kErrEmitOverflow = 1;
constexpr int32_t kErrBadOffsets = 2;
constexpr int32_t kErrTimeout = 4;  // a bounded wait in a kernel gave up
constexpr int32_t kErrBadPid = 8;   // a range partition id is negative or >= P
constexpr int32_t kErrNestSpan = 16;  // a null entry inside a nested column holds elements

// One array k_nest_prep computes for a batch of a nested column.
//   compose: out[r] = off[depth-1][ ... off[1][off[0][r]] ... ] for r < n (int32 out; every index
//            checked against the entries of the array it reads, lim[d]);
//   lengths: out[i] = valid(i) ? off[0][i + 1] - off[0][i] : 0 for i < n; with `inner` a null
//            entry holding elements is an error (kErrNestSpan).
constexpr int kMaxNestChain = 6;
struct NestJob {
  uint32_t kind;   // 0 compose, 1 lengths
  uint32_t n;
  uint32_t depth;
  uint32_t inner;
  const void* off[kMaxNestChain];
  uint64_t lim[kMaxNestChain];   // readable entries of off[d]; lengths: lim[1] validity bits
  uint32_t wide[kMaxNestChain];  // 1: int64 offsets
  const uint8_t* validity;       // lengths: the entries' validity (nullptr: all valid)
  int32_t* out;
};

struct BatchDesc {
  uint32_t nrows;
  uint32_t seg0;        // first segment
  uint32_t nsegs;
  uint32_t split_size;  // CalculateSplitBatchSize for this batch (splitter.cc:800-853)
};

struct TileDesc {
  uint32_t batch;
  uint32_t row0;   // first row inside the batch
  uint32_t nrows;
  uint32_t frow0;  // first row inside the flush (index into pids)
  uint32_t seg;    // its segment
  uint32_t tseg;   // its index inside the segment (0: no earlier tiles)
  uint32_t pad[2];
};

struct SegDesc {
  uint32_t batch;
  uint32_t row0;   // first row inside the batch (a multiple of kTileRows)
  uint32_t nrows;
  uint32_t frow0;  // first row inside the flush (index into pids)
  uint32_t tile0;  // first tile inside the flush (index into crange)
  uint32_t pad[3];
};

// Emission record written by k_plan: [p, frow_end, rows, hv_lo, hv_hi, fb_end[n_str]]
constexpr int kEmitFixedWords = 5;

struct FlushDesc {
  uint32_t n_batches;
  uint32_t n_segs;
  uint32_t n_rows;
  uint32_t hist_in_smem;  // 1: k_hash_count histograms in shared memory
  uint32_t n_tiles;
  uint32_t seg_tiles;     // tiles per segment (1 when the running counts do not fit)

  const BatchDesc* batches;  // [n_batches]
  const SegDesc* segs;       // [n_segs]
  const TileDesc* tiles;     // [n_tiles]
  const ColPtr* cols;        // [n_batches][n_cols]

  // scratch (two buffers, used by alternate flushes)
  uint16_t* pids;     // [n_rows]
  uint32_t* cnt;      // [n_segs][P] rows; rewritten by k_plan to the flush-local row offset
  uint32_t* bcnt;     // [n_segs][n_str][P] bytes; rewritten to the flush-local byte offset
  uint32_t* vpos;     // [n_segs][P] validity bit offset (pieces start on 64-bit boundaries)
  uint32_t* sbyte;    // [n_segs][n_str][P] byte offset inside the partition's emitted batch
  uint32_t* nullcnt;  // [n_batches][n_array]
  int2* crange;       // [n_tiles][n_str] offsets of the tile's first and one-past-last row
  uint32_t* tilepre;  // [n_tiles][P] rows from the segment's earlier tiles (seg_tiles > 1)
  uint32_t* tilebpre; // [n_tiles][n_str][P] bytes from the segment's earlier tiles

  // per-partition results of this flush
  uint32_t* rows_f;   // [P]
  uint32_t* vbits_f;  // [P]
  uint32_t* bytes_f;  // [n_str][P]
  uint32_t* pstart;   // [P]   exclusive scans over partitions
  uint32_t* vstart;   // [P]
  uint32_t* cstart;   // [n_str][P]

  uint32_t* emit;        // [emit_cap][kEmitFixedWords + n_str]
  uint32_t* emit_count;  // [1]
  uint32_t emit_cap;
  uint32_t rr_base;      // round-robin selection at the pass's first row (pid_selection_)
  uint32_t spin_limit;   // polls of k_scatter's waits for data / free slots; 0: the default
  uint32_t* call_flags;  // [n_batches] 1 when some partition ran CalculateSplitBatchSize
  uint32_t* rec_idx;     // [n_batches][P] 1 + emission record index when a segment was cut
  unsigned long long* hn;   // [n_batches] columns with nulls in the batch
  unsigned long long* ihn;  // [n_batches] input_has_null_ after the batch

  // outputs of this flush, indexed by array column
  uint8_t* out_values[kMaxCols];   // fixed: n_rows * width; binary: n_rows end offsets (arr_width bytes)
  uint32_t* out_bits[kMaxCols];    // bool values, same bit layout as validity
  uint32_t* out_valid[kMaxCols];   // validity words, 0xff-filled; nullptr: no nulls in flush
  uint8_t* out_chars[kMaxCols];    // binary bytes (list: element values)
  uint32_t* out_cvalid[kMaxCols];  // list: element validity bits at the element's position in
                                   // out_chars, 0xff-filled; nullptr: no element nulls in flush

  // persistent partition state (the reference's per-pid buffer bookkeeping)
  uint32_t* st_cap;               // partition_buffer_size_
  uint32_t* st_base;              // partition_buffer_idx_base_
  unsigned long long* st_hv;      // validity buffer present, per array column
  uint32_t* st_sb;                // [n_str][P] bytes in the open segment
  unsigned long long* st_ihn;     // [1] input_has_null_ (sticky)
  int32_t* err;                   // device error word
};

}  // namespace gz
