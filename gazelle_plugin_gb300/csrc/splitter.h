// gz::Splitter — the host side of the GB300 hash split, keeping the reference Splitter's
// interface (native-sql-engine/cpp/src/shuffle/splitter.h:55-126): Make / Split / Stop /
// SpillFixedSize / SetCompressType / CompressedSize and the metric getters.
//
// Split() only gathers the batch: host inputs are read before it returns, as the JNI contract
// requires, either by the GPU itself over a coherent host link (k_gather into device staging,
// where the device can read pageable host memory through the host page tables) or by a CPU
// copy into pinned staging; every `flush_bytes` of input one device pass runs the kernels on
// the splitter's streams (see the pass schedule below).  Emission decisions are made on the
// device by k_plan, so Split never waits for the GPU.  Stop() finishes the device work,
// assembles every emitted partition batch from the flush outputs and writes the Arrow IPC
// data file in partition order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/gz_split.h"
#include "gz_engine.cuh"
#include "host_util.h"
#include "ipc.h"
#include "schema_ipc.h"

namespace gz {

struct Status {
  GzStatus code = GZ_OK;
  std::string msg;
  bool ok() const { return code == GZ_OK; }
  static Status OK() { return Status(); }
  static Status Error(GzStatus c, std::string m) {
    Status s;
    s.code = c;
    s.msg = std::move(m);
    return s;
  }
};

// Entries of a nested field in a batch's flat buffer list (MakeArrayData's depth-first order).
int NestedBufferCount(const Field& f);

class Splitter {
  friend Status SyncGroup(const std::vector<Splitter*>& tasks, int* failed);

 public:
  static Status Make(const std::string& short_name, std::vector<Field> fields, int32_t P,
                     std::vector<int32_t> keys, const GzSplitOptions& opts,
                     std::unique_ptr<Splitter>* out);
  ~Splitter();

  // One batch; host inputs are fully read when it returns.
  Status Split(int32_t num_rows, const int64_t* addrs, const int64_t* sizes, int32_t n);
  // Split(rows[i], addrs + i * n, sizes + i * n, n) for every batch; host inputs are fully
  // read when it returns (also on error).
  Status SplitBatches(int32_t n_batches, const int32_t* rows, const int64_t* addrs,
                      const int64_t* sizes, int32_t n);
  // SplitBatches without waiting for the host reads: the caller calls StartHostReads and then
  // WaitHostReads before it releases the buffers (SplitGroup below).
  Status SplitMany(int32_t n_batches, const int32_t* rows, const int64_t* addrs, const int64_t* sizes,
                   int32_t n);
  Status StartHostReads();
  Status WaitHostReads();
  Status CompressedSize(int32_t num_rows, const int64_t* addrs, const int64_t* sizes, int32_t n,
                        int64_t* out);
  Status Stop();
  Status SpillFixedSize(int64_t size, int64_t* actual);
  Status SetCompressType(int32_t codec);
  Status LastPids(uint16_t* out, int32_t n);
  Status KernelTimes(double* out4);
  // Polls of k_scatter's bounded waits for data and free slots in later passes (0: default).
  void SetSpinLimit(uint32_t polls) { spin_limit_ = polls; }
  // Runs the pending device pass and waits for all device work of the batches split so far.
  Status Sync();
  void Stats(int64_t* out8) const;
  // [0] local-dir files written, [1] their bytes, [2] files present now
  void DiskSpillStats(int64_t* out3) const;

  int64_t TotalBytesWritten() const { return total_bytes_written_; }
  int64_t TotalBytesSpilled() const { return total_bytes_spilled_; }
  int64_t TotalWriteTime() const { return total_write_time_; }
  int64_t TotalSpillTime() const { return total_spill_time_; }
  int64_t TotalCompressTime() const { return total_compress_time_; }
  int64_t TotalComputePidTime() const { return total_compute_pid_time_; }
  const std::vector<int64_t>& PartitionLengths() const { return partition_lengths_; }
  const std::vector<int64_t>& RawPartitionLengths() const { return raw_partition_lengths_; }
  const std::vector<uint8_t>& DataBytes() const { return data_bytes_; }
  int32_t num_partitions() const { return P_; }
  bool stopped() const { return stopped_; }

 private:
  struct PendingBatch {
    uint32_t nrows;
    uint32_t split_size;
    uint64_t validity_mask;  // array columns with a validity buffer
    uint64_t cvalid_mask;    // list columns with an element validity buffer
  };

  // Nested columns (list / large_list / map / struct other than a list of fixed-width or bool
  // elements, list_array_idx_ in the reference).  A top-level row selects one contiguous range
  // of entries at every node of the column's type tree: the rows themselves at the top and
  // under structs, the children's entries [offsets[lo], offsets[hi]) under a list or map.  Each
  // node's entries reach the device as a "stream": a list-like array column (after the binary
  // and simple list ones) whose row offsets are those ranges (the node's offsets composed along
  // its path, computed by k_nest_prep; the rows themselves through an identity array), whose
  // element validity is the node's validity and whose elements carry the node's payload: fixed
  // width values, bool bits, the entries' lengths (binary, list and map nodes: their offsets are
  // rebuilt from them at Stop) or nothing (struct).  A binary node's characters are one more
  // stream.  A top-level list or map is merged with its child's stream (its own validity and
  // offsets are that stream's row validity and offsets), as simple lists are.
 public:
  enum StreamPayload { PAY_VALUES = 0, PAY_BITS = 1, PAY_LENGTHS = 2, PAY_NONE = 3 };
  struct NestNode {
    int type = 0;
    int width = 0;          // element bytes of a fixed-width leaf
    int buf = 0;            // its first buffer in the batch's flat list
    int parent = -1;
    std::vector<int> kids;  // node indices (pre-order)
    bool ident = false;     // its entries are the rows
    bool inner = false;     // below a list or map: a null entry must hold no elements
    int mask = -1;          // node whose validity empties the rows of its streams (a list / map
                            // whose entries are rows)
    std::vector<int> chain; // nodes whose offsets compose its row ranges, outermost first
    int stream = -1;        // array column of its entries (-1: none, e.g. a map's entries struct)
    int chars = -1;         // binary node: array column of its characters
  };
  struct NestPlan {
    int field = -1;
    std::vector<NestNode> nodes;  // pre-order; nodes[0] is the field
    bool root_list = false;       // nodes[0] (list / large_list / map) shares its child's stream
  };
  struct Stream {  // one array column of a nested field
    int plan = 0, node = 0;
    bool chars = false;  // the node's characters
    int payload = PAY_NONE;
    int slot = 0;        // its ColPtr slot
  };
  // an array computed on the device per batch (k_nest_prep) and pointed at from a ColPtr
  struct PendingDerived {
    uint32_t batch;
    int slot;
    bool values;    // the slot's values (lengths) rather than its offsets (composed ranges)
    NestJob job;    // out filled at Flush
    size_t bytes;
    int same_as;    // >= 0: the slot points at that earlier entry's array (same composed ranges)
  };

 private:
  struct Need {
    const uint8_t* src;
    size_t bytes;
  };

  // One device pass and what Stop needs from it.
  struct FlushRec {
    uint32_t n_rows = 0;
    uint32_t n_batches = 0;
    uint8_t* d_out = nullptr;           // device outputs (nullptr once moved to host)
    size_t out_bytes = 0;
    uint8_t* h_out = nullptr;           // pinned host copy of the outputs (in host_chunks_), or
                                        // the read-only mapping of its local-dir file
    bool on_host = false;
    bool on_file = false;               // h_out maps spill_path (past host_budget)
    std::string spill_path;
    std::vector<size_t> off_values, off_bits, off_valid, off_chars;  // per array column, SIZE_MAX: none
    std::vector<size_t> off_cvalid;  // list columns: element validity bits (in the bit regions)
    uint32_t* h_meta = nullptr;         // pinned: rows_f, pstart, vstart, bytes_f, cstart, count, emit
    size_t bits_begin = 0, bits_end = 0;  // the bit regions (validity, bool values) in the output
    uint8_t* h_bits = nullptr;          // pinned copy of just the bit regions (compressed Stop)
    size_t meta_words = 0;
    uint32_t emit_cap = 0;
    // [0] k_hash_count start, [1] its end (hstream_); [4] k_scatter start, [3] its end (stream_); [5]
    // plan start, [2] its end, [6] the end of the pass's work on pstream_ (plan + metadata copies)
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool launched = false;              // its k_scatter is queued (ev[3] recorded)
    int scratch = 0;                    // which scratch buffer the pass used
    const uint32_t* rows_f() const { return h_meta; }
    const uint32_t* pstart(int P) const { return h_meta + P; }
    const uint32_t* vstart(int P) const { return h_meta + 2 * (size_t)P; }
    const uint32_t* bytes_f(int P) const { return h_meta + 3 * (size_t)P; }
    const uint32_t* cstart(int P, int nstr) const { return h_meta + (3 + (size_t)nstr) * P; }
    uint32_t emit_count(int P, int nstr) const { return h_meta[(3 + 2 * (size_t)nstr) * P]; }
    const uint32_t* emits(int P, int nstr) const { return h_meta + (3 + 2 * (size_t)nstr) * P + 1; }
  };

  struct Piece {
    int32_t flush;
    uint32_t frow0, frow1;  // flush-local rows of the partition
    uint32_t vpos0;         // flush-local validity bit of frow0
    std::vector<uint32_t> fb0, fb1;  // flush-local byte range per binary column
  };

  struct Segment {  // one emitted record batch of one partition
    uint32_t rows = 0;
    uint64_t hv = 0;
    bool at_stop = false;
    bool spilled = false;
    int64_t body_length = -1;
    int64_t message_bytes = -1;
    // rows [0, valid_wipe_rows) read as valid in every column: SpillPartition refills the
    // validity buffers of the partition's open buffers with 0xff (splitter.cc:765-773)
    uint32_t valid_wipe_rows = 0;
    std::vector<Piece> pieces;
  };

  Splitter() = default;
  Status Init(const std::string& short_name, std::vector<Field> fields, int32_t P,
              std::vector<int32_t> keys, const GzSplitOptions& opts);
  Status Cuda(cudaError_t e, const char* what);
  Status EnsureScratch(size_t bytes_needed, bool* fresh);
  Status EnsureStaging(size_t bytes);
  void ReleaseStaging();
  uint8_t* HostAlloc(size_t bytes);
  void ReleaseHost();
  Status SplitOne(int32_t num_rows, const int64_t* addrs, const int64_t* sizes, int32_t n);
  Status LaunchGather();
  Status FinishHostReads();
  bool reads_marked_ = false;  // gather_ev_ marks host reads not yet waited for
  Status PinnedMeta(size_t bytes, uint32_t** out);
  Status Flush();
  Status SyncAndCheck();
  Status MoveFlushToHost(FlushRec& f);
  Status ProcessFlushes();
  // One emitted record batch ready to write: IPC metadata and the byte ranges of its body.
  struct SegMsg {
    std::vector<uint8_t> header;
    std::vector<Chunk> pieces;  // the body in order, padding included
    std::vector<std::vector<uint8_t>> temps;  // bitmaps assembled for it
    int64_t bytes = 0;  // header + body
    int64_t body = 0;
    int64_t raw = 0;    // its raw buffer bytes (batch_nbytes)
    uint32_t rows = 0;
    std::vector<FieldNodeMeta> nodes;
    std::vector<ChunkedBuffer> bufs;  // device view: the body buffers before compression
  };
  // `device_view`: body ranges point at the pass outputs where they are (HBM, or pinned host
  // memory the device reads; Chunk::dev set) for the device to compress or copy, bit regions at
  // their host copies (h_bits); otherwise everything points at the host copies (h_out).
  Status BuildSegment(int p, const Segment& s, SegMsg* msg, bool device_view = false) const;
  // Compressed Stop: body ranges of every record batch through the device (LZ4 blocks for
  // batches above batch_compress_threshold rows, plain copies for the others) into one arena,
  // which is then copied to pinned host memory; fills every message's header and pieces.
  Status CompressBodies(std::vector<std::vector<SegMsg>>* msgs);
  uint32_t SplitBatchSize(int32_t num_rows, const std::vector<const uint8_t*>& host_offsets,
                          bool* complete);

  // nested columns
  Status PlanNested();
  void PlanNode(NestPlan& np, const Field& f, int parent, int* buf);
  Status StageNested(uint32_t nr, const int64_t* addrs, const int64_t* sizes, const uint8_t* const* dptr,
                     ColPtr* cols, bool host_in);
  Status EnsureIota(uint32_t rows);
  // Stop: the nested field's nodes and body buffers of one record batch
  void BuildNested(int p, const Segment& s, const NestPlan& np, int node, std::vector<FieldNodeMeta>* nodes,
                   std::vector<ChunkedBuffer>* bufs, std::vector<std::vector<uint8_t>>* temps, bool device_view,
                   int64_t* raw) const;
  void NestedBodyBuffers(const NestPlan& np, int node, int64_t off, int64_t len, const int64_t* addrs,
                         const int64_t* sizes, std::vector<std::pair<const uint8_t*, int64_t>>* bufs,
                         std::vector<std::vector<uint8_t>>* temps) const;
  std::vector<NestPlan> nest_;
  std::vector<Stream> streams_;  // streams_[a - first_stream_] for array column a
  int first_stream_ = 0;
  int n_slots_ = 0;              // ColPtr slots per batch: the fields, then one per stream
  uint64_t lenpay_mask_ = 0;     // streams whose elements are lengths (kept with the bit regions)
  std::vector<PendingDerived> pending_derived_;
  std::vector<const uint8_t*> dptr_;  // per-call scratch: device address of every input buffer
  int32_t* d_iota_ = nullptr;    // 0, 1, 2, ...: the row ranges of streams whose entries are rows
  uint32_t iota_cap_ = 0;
  std::vector<int32_t*> old_iota_;

  // schema
  std::vector<Field> fields_;  // the input schema (the range partitioner's id field included)
  int32_t P_ = 0;
  std::vector<int32_t> keys_;
  std::string short_name_;
  int32_t partitioner_ = PART_HASH;
  int32_t pid_field_ = -1;  // range: the partition id field (0), not an output column
  uint32_t rr_sel_ = 0;     // round-robin selection at the next pass's first row
  uint32_t spin_limit_ = 0; // k_scatter wait limit (0: the kernel's default)
  int32_t codec_ = 0;       // GzCodec of the emitted record batches
  std::vector<PinnedBlock> arena_blocks_;  // pinned host copies of compressed bodies (Stop)
  // input field index minus this = output schema index
  int32_t out_shift() const { return pid_field_ >= 0 ? 1 : 0; }
  GzSplitOptions opts_{};
  std::string data_file_;
  SchemaDesc sd_{};
  std::vector<int32_t> array_idx_;  // schema index per array column
  std::vector<int32_t> field_array_;  // array column per schema field (-1 for null type)
  std::vector<int32_t> field_buf0_;   // index of the field's first buffer in the flat list
  int32_t n_bufs_expected_ = 0;
  // array columns: fixed [0, fixed_cnt_), binary [fixed_cnt_, n_policy_) - the reference's
  // array_idx_, which the buffer policy reads - then list [n_policy_, n_array_); n_str_: binary
  // and list columns (the device's string-like columns), n_bin_: binary ones
  int32_t fixed_cnt_ = 0, n_str_ = 0, n_array_ = 0, n_bin_ = 0, n_policy_ = 0;
  uint32_t seg_tiles_ = 1;  // tiles per k_scatter segment
  std::vector<uint64_t> empirical_;  // binary_array_empirical_size_

  // device
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  uint8_t* d_state_ = nullptr;      // persistent partition state
  uint32_t* st_cap_ = nullptr;
  uint32_t* st_base_ = nullptr;
  unsigned long long* st_hv_ = nullptr;
  uint32_t* st_sb_ = nullptr;
  unsigned long long* st_ihn_ = nullptr;
  int32_t* d_err_ = nullptr;
  uint32_t* d_call_ = nullptr;
  // The pass schedule: k_hash_count (with its pass's table copies and clears) on hstream_, the
  // plan kernels on pstream_, k_scatter on stream_.  With device-resident inputs a pass's
  // k_scatter is queued only when the next pass is (or at a sync), after that pass's k_hash_count
  // and plan; with host inputs (bound by the host link) it is queued right after its own plan.
  // The per-pass scratch has three buffers (scr_cur_: the buffer of the next pass), so a pass's
  // k_hash_count waits only for the k_scatter two passes back (scr_ev_) and is ready while the
  // previous pass's k_scatter runs: stream priorities (k_gather, then the plan, then k_scatter,
  // then k_hash_count) let its blocks take the SMs that k_scatter's last wave leaves idle.
  static constexpr int kScratchBufs = 3;
  cudaStream_t pstream_ = nullptr;
  cudaStream_t hstream_ = nullptr;
  cudaEvent_t hwait_ev_ = nullptr;                 // stream_'s work so far (a scratch buffer allocated)
  cudaEvent_t scr_ev_[kScratchBufs] = {};          // the last k_scatter that read each buffer
  bool scr_used_[kScratchBufs] = {};
  uint8_t* d_scratch_[kScratchBufs] = {};
  size_t scratch_cap_[kScratchBufs] = {};
  int scr_cur_ = 0;
  struct PendingScatter {
    bool valid = false;
    FlushDesc fd;
    size_t flush = 0;  // index in flushes_
    int stage = 0;     // staging buffer the pass reads (host inputs)
    bool host_in = false;
  };
  PendingScatter pend_;
  Status LaunchPendingScatter();
  Status Drain();  // Flush, then queue the pending k_scatter
  Status MoveOutputs();
  // Past host_budget, the oldest passes in pinned host memory go to local-dir files.
  Status KeepHostBudget();
  Status MoveFlushToFile(FlushRec& f);
  std::string NextSpillPath();
  std::vector<std::string> spill_dirs_;  // local_dirs, split at commas
  std::vector<int> sub_dir_sel_;         // next sub-directory of each dir
  int dir_sel_ = 0;
  size_t host_resident_ = 0;             // pinned host bytes of moved passes
  int64_t disk_files_ = 0, disk_bytes_ = 0, disk_files_now_ = 0;

  // staging (host inputs): double-buffered device buffers, filled by k_gather (direct_) or
  // by H2D copies of pinned host twins
  bool direct_ = false;              // the device reads pageable host memory (coherent link)
  cudaStream_t cstream_ = nullptr;   // k_gather
  cudaStream_t ostream_ = nullptr;   // partition data to host
  cudaEvent_t gather_ev_ = nullptr;
  HostCopy* h_jobs_ = nullptr;       // pinned ring of k_gather descriptors
  size_t h_jobs_bytes_ = 0;
  size_t jobs_cap_ = 0, jobs_begin_ = 0, jobs_end_ = 0;
  size_t gather_pending_bytes_ = 0;
  uint8_t* h_stage_[2] = {nullptr, nullptr};
  size_t h_stage_cap_ = 0;
  uint8_t* d_stage_[2] = {nullptr, nullptr};
  size_t stage_cap_ = 0;
  cudaEvent_t stage_ev_[2] = {nullptr, nullptr};
  bool stage_busy_[2] = {false, false};
  int cur_ = 0;
  size_t used_ = 0;
  // pinned pass tables (device-retained and device-read host inputs): a ring, so that reusing a
  // buffer waits for a table copy kTabBufs passes back, which stream_ has long passed
  static constexpr int kTabBufs = 8;
  uint8_t* h_tables_[kTabBufs] = {};
  size_t tables_cap_[kTabBufs] = {};
  cudaEvent_t tab_ev_[kTabBufs] = {};
  bool tab_busy_[kTabBufs] = {};
  int tab_cur_ = 0;
  std::vector<PinnedBlock> meta_chunks_;
  std::vector<PinnedBlock> host_chunks_;  // pinned host partition data of moved passes
  size_t meta_chunk_cap_ = 0, meta_used_ = 0;
  std::vector<std::vector<uint8_t>> dev_off_;  // offset ends read from device inputs (offset-width bytes)
  bool seen_rows_ = false;

  std::vector<PendingBatch> pending_;
  std::vector<ColPtr> pending_cols_;      // [batch][field]
  std::vector<uint64_t> pending_chars_;   // [batch][binary column] bytes the output may need
  uint64_t pending_bytes_ = 0;
  size_t pending_tiles_ = 0;
  std::vector<Need> need_;                // per-call scratch
  std::vector<const uint8_t*> host_off_;  // offsets of each binary column readable on the host
  std::vector<uint64_t> char_scratch_;
  std::vector<CopyJob> jobs_;
  size_t spilled_to_host_bytes_ = 0;
  int64_t stat_input_bytes_ = 0, stat_h2d_bytes_ = 0, stat_batches_ = 0, stat_rows_ = 0;
  int64_t stat_emitted_ = -1;
  std::vector<FlushRec> flushes_;
  size_t processed_flushes_ = 0;
  size_t resident_bytes_ = 0;

  // per-partition emitted segments (host view, built from the flush metadata)
  std::vector<std::vector<Segment>> segments_;
  std::vector<Segment> open_;  // open segment per partition
  uint32_t last_batch_rows_ = 0;

  bool stopped_ = false;
  int64_t total_bytes_written_ = 0, total_bytes_spilled_ = 0, total_write_time_ = 0;
  int64_t total_spill_time_ = 0, total_compress_time_ = 0, total_compute_pid_time_ = 0;
  double kernel_ms_[4] = {0, 0, 0, 0};
  size_t timed_flushes_ = 0;
  std::vector<int64_t> partition_lengths_, raw_partition_lengths_;
  std::vector<uint8_t> data_bytes_;
};

// Split calls of several tasks at once (task i: n_batches[i] batches of n_bufs[i] buffers, its
// rows / addresses / sizes following the previous task's): every task's host reads are started
// before any is waited for.  *failed: the first task whose call failed.
Status SplitGroup(const std::vector<Splitter*>& tasks, const int32_t* n_batches, const int32_t* rows,
                  const int64_t* addrs, const int64_t* sizes, const int32_t* n_bufs, int* failed);
// Sync of several tasks: every task's pending pass is queued before any is waited for.
Status SyncGroup(const std::vector<Splitter*>& tasks, int* failed);

}  // namespace gz
