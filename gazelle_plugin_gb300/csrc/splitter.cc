// Host engine of the GB300 hash split (see splitter.h).
#include "splitter.h"

#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/uio.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <numeric>

#include "gz_kernels.h"
#include "lz4_kernels.h"
#include "host_util.h"
#include "split_util.h"
#include "tune.h"

namespace gz {

namespace {

constexpr int64_t kMapWriteBytes = 256ll << 20;  // data files from this size are written through a mapping
inline int64_t NowNs() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

}  // namespace

Status Splitter::Cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status::OK();
  cudaGetLastError();
  return Status::Error(e == cudaErrorMemoryAllocation ? GZ_OOM : GZ_CUDA,
                       std::string(what) + ": " + cudaGetErrorString(e));
}

Status Splitter::Make(const std::string& short_name, std::vector<Field> fields, int32_t P,
                      std::vector<int32_t> keys, const GzSplitOptions& opts,
                      std::unique_ptr<Splitter>* out) {
  std::unique_ptr<Splitter> s(new Splitter());
  Status st = s->Init(short_name, std::move(fields), P, std::move(keys), opts);
  if (!st.ok()) return st;
  *out = std::move(s);
  return Status::OK();
}

Status Splitter::Init(const std::string& short_name, std::vector<Field> fields, int32_t P,
                      std::vector<int32_t> keys, const GzSplitOptions& opts) {
  // Splitter::Make (splitter.cc:190-208): "single" is round-robin over one partition; the
  // round-robin and range partitioners take no key expressions
  if (short_name == "hash") {
    partitioner_ = PART_HASH;
  } else if (short_name == "rr" || short_name == "single") {
    partitioner_ = PART_RR;
    if (short_name == "single") P = 1;
    keys.clear();
  } else if (short_name == "range") {
    // FallbackRangeSplitter::Init (splitter.cc:1486-1490): field 0 holds the partition ids and
    // the output schema is the input schema without it
    partitioner_ = PART_RANGE;
    if (fields.empty()) return Status::Error(GZ_INVALID, "range partitioning needs a partition id field");
    pid_field_ = 0;
    keys.assign(1, 0);
  } else {
    return Status::Error(GZ_NOT_IMPLEMENTED, "Partitioning " + short_name + " not supported yet.");
  }
  short_name_ = short_name;
  if (P <= 0 || P > 64 * 1024) return Status::Error(GZ_INVALID, "num_partitions must be in [1, 65536]");
  opts_ = opts;
  if (opts_.buffer_size <= 0) opts_.buffer_size = 4096;
  if (opts_.buffer_size > 32 * 1024) return Status::Error(GZ_INVALID, "buffer_size must be <= 32768");
  if (opts_.compression == GZ_CODEC_LZ4_FRAME) codec_ = GZ_CODEC_LZ4_FRAME;
  else if (opts_.compression != GZ_CODEC_UNCOMPRESSED)
    return Status::Error(GZ_NOT_IMPLEMENTED, "codec " + std::to_string(opts_.compression) + " is not implemented");
  data_file_ = opts.data_file ? opts.data_file : "";
  // spill dirs (the JNI's localDirs, the reference's NATIVESQL_SPARK_LOCAL_DIRS): comma
  // separated, empty entries skipped (GetConfiguredLocalDirs, utils.h:64-88)
  if (opts.local_dirs) {
    std::string all = opts.local_dirs;
    size_t at = 0;
    while (at <= all.size()) {
      const size_t comma = std::min(all.find(',', at), all.size());
      if (comma > at) spill_dirs_.push_back(all.substr(at, comma - at));
      at = comma + 1;
    }
  }
  sub_dir_sel_.assign(spill_dirs_.size(), 0);
  if (opts_.num_sub_dirs <= 0) opts_.num_sub_dirs = 64;
  if (opts_.host_budget < 0) return Status::Error(GZ_INVALID, "host_budget must be >= 0");
  if (opts_.host_budget > 0 && spill_dirs_.empty())
    return Status::Error(GZ_INVALID, "host_budget needs local_dirs to spill to");
  opts_.data_file = nullptr;
  opts_.local_dirs = nullptr;
  if ((int)fields.size() > kMaxSchemaCols) return Status::Error(GZ_NOT_IMPLEMENTED, "too many fields");
  fields_ = std::move(fields);
  P_ = P;
  keys_ = std::move(keys);
  // pass size and segment length: given, else the autotuner's choice for this schema
  if (opts_.flush_bytes <= 0 || opts_.seg_tiles <= 0) {
    TuneChoice tc;
    if (TuneLookup(SchemaSignature(short_name_, fields_, keys_, P_), &tc)) {
      if (opts_.flush_bytes <= 0) opts_.flush_bytes = tc.flush_bytes;
      if (opts_.seg_tiles <= 0) opts_.seg_tiles = tc.seg_tiles;
    }
  }
  // partition data of host inputs goes back to the host as passes finish (overlapping the
  // split); of device-resident inputs it stays in HBM until Stop
  // (with a codec it stays: the device compresses it at Stop)
  if (opts_.keep_output_on_device < 0)
    opts_.keep_output_on_device = opts_.input_kind == GZ_INPUT_HOST && codec_ == GZ_CODEC_UNCOMPRESSED ? 0 : 1;
  if (opts_.flush_bytes <= 0) opts_.flush_bytes = 512ll << 20;
  if (opts_.flush_bytes > (1ll << 30)) opts_.flush_bytes = 1ll << 30;
  if (opts_.seg_tiles > kMaxSegTiles) opts_.seg_tiles = kMaxSegTiles;

  // Splitter::Init column classification (splitter.cc:246-269); list columns
  // (list_array_idx_, :254-258) follow the binary ones here, outside the buffer policy's columns
  std::vector<int32_t> bin, lists;
  field_array_.assign(fields_.size(), -1);
  for (size_t i = 0; i < fields_.size(); i++) {
    const int t = fields_[i].type;
    if ((int)i == pid_field_) continue;  // not an output column
    if (IsBinary(t)) bin.push_back((int32_t)i);
    else if (t == GZ_TYPE_NULL) continue;
    else if (fields_[i].nested() || t == GZ_TYPE_LARGE_LIST || t == GZ_TYPE_STRUCT || t == GZ_TYPE_MAP) {
      if (!fields_[i].nested()) return Status::Error(GZ_INVALID, "nested field without child fields");
      continue;  // streams, planned below
    } else if (t == GZ_TYPE_LIST) {
      if (ByteWidth(fields_[i].elem) <= 0 && fields_[i].elem != GZ_TYPE_BOOL)
        return Status::Error(GZ_NOT_IMPLEMENTED, "list columns of fixed-width or bool elements only");
      lists.push_back((int32_t)i);
    } else if (t == GZ_TYPE_BOOL || ByteWidth(t) > 0) array_idx_.push_back((int32_t)i);
    else return Status::Error(GZ_NOT_IMPLEMENTED, "field type not implemented in ColumnarShuffle");
  }
  fixed_cnt_ = (int32_t)array_idx_.size();
  array_idx_.insert(array_idx_.end(), bin.begin(), bin.end());
  n_bin_ = (int32_t)bin.size();
  n_policy_ = (int32_t)array_idx_.size();
  array_idx_.insert(array_idx_.end(), lists.begin(), lists.end());
  first_stream_ = (int32_t)array_idx_.size();
  n_slots_ = (int32_t)fields_.size();
  {
    Status ps = PlanNested();  // appends the nested columns' streams to array_idx_
    if (!ps.ok()) return ps;
  }
  n_array_ = (int32_t)array_idx_.size();
  n_str_ = (int32_t)(bin.size() + lists.size() + streams_.size());
  if (n_array_ == 0) return Status::Error(GZ_NOT_IMPLEMENTED, "schema without data columns");
  if (n_array_ > kMaxCols) return Status::Error(GZ_NOT_IMPLEMENTED, "more than 64 data columns");
  if (n_str_ > max_str_columns()) return Status::Error(GZ_NOT_IMPLEMENTED, "more than 64 binary, list and nested-stream columns");
  if ((int)keys_.size() > kMaxKeys) return Status::Error(GZ_NOT_IMPLEMENTED, "more than 8 hash keys");

  memset(&sd_, 0, sizeof(sd_));
  sd_.P = P_;
  sd_.n_cols = n_slots_;
  sd_.n_array = n_array_;
  sd_.n_fixed = fixed_cnt_;
  sd_.n_str = n_str_;
  sd_.n_keys = (int32_t)keys_.size();
  sd_.prefer_spill = opts_.prefer_spill ? 1 : 0;
  sd_.partitioner = partitioner_;
  sd_.pmod_magic = P_ > 1 ? UINT64_MAX / (uint64_t)P_ + 1 : 0;
  for (int a = 0; a < n_array_; a++) {
    const int ci = array_idx_[a];
    if (a >= first_stream_) {  // a nested column's stream: list-like, rows from its slot
      const Stream& sm = streams_[a - first_stream_];
      if (field_array_[ci] < 0) field_array_[ci] = a;
      sd_.arr_col[a] = sm.slot;
      sd_.arr_kind[a] = COL_BINARY;
      sd_.arr_width[a] = 4;
      sd_.arr_str[a] = a - fixed_cnt_;
      sd_.list_mask |= 1ull << a;
      const NestNode& nd = nest_[sm.plan].nodes[sm.node];
      int sh = 0;
      if (sm.chars) {
        sh = 0;
      } else if (sm.payload == PAY_VALUES) {
        while ((1 << sh) < nd.width) sh++;
      } else if (sm.payload == PAY_LENGTHS) {
        sh = 2;
        lenpay_mask_ |= 1ull << a;
      } else {
        sd_.listbit_mask |= 1ull << a;
        if (sm.payload == PAY_NONE) sd_.nopay_mask |= 1ull << a;
      }
      sd_.arr_shift[a] = sh;
      continue;
    }
    field_array_[ci] = a;
    const int t = fields_[ci].type;
    sd_.arr_col[a] = ci;
    const bool list = t == GZ_TYPE_LIST;
    sd_.arr_kind[a] = IsBinary(t) || list ? COL_BINARY : t == GZ_TYPE_BOOL ? COL_BOOL : COL_FIXED;
    sd_.arr_width[a] = IsBinary(t) ? OffW(t) : list ? 4 : ByteWidth(t);  // binary / list: offset bytes
    sd_.arr_str[a] = a >= fixed_cnt_ ? a - fixed_cnt_ : -1;
    if (list) {
      int sh = 0;
      while ((1 << sh) < ByteWidth(fields_[ci].elem)) sh++;
      sd_.arr_shift[a] = sh;
      sd_.list_mask |= 1ull << a;
      if (fields_[ci].elem == GZ_TYPE_BOOL) sd_.listbit_mask |= 1ull << a;
    }
    // compared as an index of the output schema (the range partitioner's ids are not in it)
    if (a < n_policy_ && ci - out_shift() < fixed_cnt_) sd_.quirk_mask |= 1ull << a;
  }
  // k_scatter processing order: binary columns spread evenly among the fixed ones, so the
  // characters of the next binary column stream in while fixed columns are scattered
  {
    std::vector<int32_t> fixed, binary;
    for (int a = 0; a < n_array_; a++) (sd_.arr_kind[a] == COL_BINARY ? binary : fixed).push_back(a);
    size_t fi = 0, bi = 0;
    for (int i = 0; i < n_array_; i++) {
      // binary column bi goes to position floor(bi * n_array / n_binary)
      const bool take_binary =
          bi < binary.size() && (fi == fixed.size() || (int64_t)i >= (int64_t)bi * n_array_ / (int64_t)binary.size());
      sd_.order[i] = take_binary ? binary[bi++] : fixed[fi++];
    }
  }
  // The plan works on segments of several tiles when k_hash_count keeps the running rows and
  // bytes of every partition in shared memory (it then records each tile's prefix).  Its work
  // grows with segments x partitions: from 1024 partitions on, segments are as long as they go
  // (32 tiles; on 32768-row batches with 2000 / 8000 partitions that was 17% / 19% faster per
  // split than 8 / 31 tiles), below that 4 tiles keep k_hash_count's grid wide.
  if ((size_t)(1 + n_str_) * P_ * 4 > kHistSmemBytes) seg_tiles_ = 1;
  else if (opts_.seg_tiles > 0) seg_tiles_ = (uint32_t)opts_.seg_tiles;
  else seg_tiles_ = P_ >= 1024 ? (uint32_t)kMaxSegTiles : 4u;
  // hash chain (HashSplitter::CreateProjector, splitter.cc:1402-1438); the range partitioner's
  // one "key" is its id column, read as int32 values (a wrong type fails every Split)
  // A null-type key has no hash function and leaves the chain unchanged (the NullType case,
  // splitter.cc:1407-1408), so it takes no slot of the device key list.
  int nk = 0;
  for (size_t k = 0; k < keys_.size(); k++) {
    const int ci = keys_[k];
    if (ci < 0 || ci >= (int)fields_.size()) return Status::Error(GZ_INVALID, "key column out of range");
    if (partitioner_ != PART_RANGE && fields_[ci].type == GZ_TYPE_NULL) continue;
    int kind;
    switch (partitioner_ == PART_RANGE ? GZ_TYPE_INT32 : fields_[ci].type) {
      case GZ_TYPE_BOOL: kind = KEY_BOOL; break;
      case GZ_TYPE_INT8: kind = KEY_I8; break;
      case GZ_TYPE_INT16: kind = KEY_I16; break;
      case GZ_TYPE_INT32: case GZ_TYPE_FLOAT32: case GZ_TYPE_DATE32: kind = KEY_I32; break;
      case GZ_TYPE_INT64: case GZ_TYPE_FLOAT64: kind = KEY_I64; break;
      case GZ_TYPE_STRING: kind = KEY_STR; break;  // hashbuf_spark (splitter.cc:1424-1427)
      default:
        return Status::Error(GZ_NOT_IMPLEMENTED,
                             "hash key type has no Spark-compatible hash in the GPU splitter");
    }
    sd_.key_col[nk] = ci;
    sd_.key_kind[nk] = kind;
    nk++;
  }
  sd_.n_keys = nk;
  // JNI buffer layout (jni_common.h:186-382): [validity, (offsets), values] per field, nested
  // fields depth first
  field_buf0_.resize(fields_.size());
  int nb = 0;
  for (size_t i = 0; i < fields_.size(); i++) {
    field_buf0_[i] = nb;
    nb += fields_[i].nested() ? NestedBufferCount(fields_[i])
          : fields_[i].type == GZ_TYPE_LIST ? 4 : IsBinary(fields_[i].type) ? 3 : 2;
  }
  n_bufs_expected_ = nb;
  for (NestPlan& np : nest_)
    for (NestNode& nd : np.nodes) nd.buf += field_buf0_[np.field];
  dptr_.assign(n_bufs_expected_ + 1, nullptr);
  empirical_.assign(n_bin_, 0);

  device_ = opts_.device;
  GzStatus dummy;
  (void)dummy;
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  {
    // host reads, then the plan kernels, get the higher priorities: their few CTAs are
    // scheduled ahead of the remaining CTAs of a running k_scatter; k_hash_count gets the lowest,
    // so it takes the SMs k_scatter leaves idle instead of delaying it
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    st = Cuda(cudaStreamCreateWithPriority(&cstream_, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    if (!st.ok()) return st;
    st = Cuda(cudaStreamCreateWithPriority(&pstream_, cudaStreamNonBlocking, std::min(greatest + 1, least)),
              "cudaStreamCreate");
    if (!st.ok()) return st;
    st = Cuda(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, std::min(greatest + 2, least)),
              "cudaStreamCreate");
    if (!st.ok()) return st;
    st = Cuda(cudaStreamCreateWithPriority(&hstream_, cudaStreamNonBlocking, least), "cudaStreamCreate");
    if (!st.ok()) return st;
  }
  st = Cuda(cudaEventCreateWithFlags(&hwait_ev_, cudaEventDisableTiming), "cudaEventCreate");
  if (!st.ok()) return st;
  for (auto& e : scr_ev_) {
    st = Cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    if (!st.ok()) return st;
  }
  st = Cuda(cudaStreamCreateWithFlags(&ostream_, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!st.ok()) return st;
  st = Cuda(cudaEventCreateWithFlags(&gather_ev_, cudaEventDisableTiming), "cudaEventCreate");
  if (!st.ok()) return st;
  if (opts_.input_kind == GZ_INPUT_HOST && opts_.host_read == GZ_HOST_READ_AUTO) {
    // kernels may dereference any host address when the device walks the host page tables
    // (a coherent CPU-GPU link): host inputs are then read by k_gather, no CPU copy
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device_);
    direct_ = pageable != 0 && host_tables != 0;
  }
  if (direct_) {
    jobs_cap_ = size_t(1) << 20;  // 24 MiB of descriptors: a refill waits for the device
    const PinnedBlock b = PinnedAcquire(jobs_cap_ * sizeof(HostCopy));
    if (!b.ptr) return Status::Error(GZ_OOM, "pinned host memory for the gather descriptors");
    h_jobs_ = reinterpret_cast<HostCopy*>(b.ptr);
    h_jobs_bytes_ = b.cap;
  }
  {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device_) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  // persistent partition state
  const size_t state_bytes = AlignUp(sizeof(uint32_t) * P_, 256) * 2 +
                             AlignUp(sizeof(unsigned long long) * P_, 256) +
                             AlignUp(sizeof(uint32_t) * (size_t)std::max(n_str_, 1) * P_, 256) +
                             256 * 3;
  st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d_state_), state_bytes, stream_), "cudaMallocAsync(state)");
  if (!st.ok()) return st;
  st = Cuda(cudaMemsetAsync(d_state_, 0, state_bytes, stream_), "cudaMemset(state)");
  if (!st.ok()) return st;
  uint8_t* q = d_state_;
  st_cap_ = reinterpret_cast<uint32_t*>(q); q += AlignUp(sizeof(uint32_t) * P_, 256);
  st_base_ = reinterpret_cast<uint32_t*>(q); q += AlignUp(sizeof(uint32_t) * P_, 256);
  st_hv_ = reinterpret_cast<unsigned long long*>(q); q += AlignUp(sizeof(unsigned long long) * P_, 256);
  st_sb_ = reinterpret_cast<uint32_t*>(q); q += AlignUp(sizeof(uint32_t) * (size_t)std::max(n_str_, 1) * P_, 256);
  st_ihn_ = reinterpret_cast<unsigned long long*>(q); q += 256;
  d_err_ = reinterpret_cast<int32_t*>(q); q += 256;
  d_call_ = reinterpret_cast<uint32_t*>(q);
  for (int i = 0; i < 2; i++) {
    st = Cuda(cudaEventCreateWithFlags(&stage_ev_[i], cudaEventDisableTiming), "cudaEventCreate");
    if (!st.ok()) return st;
  }
  for (int i = 0; i < kTabBufs; i++) {
    st = Cuda(cudaEventCreateWithFlags(&tab_ev_[i], cudaEventDisableTiming), "cudaEventCreate");
    if (!st.ok()) return st;
  }
  dev_off_.resize(n_str_);
  need_.assign(n_bufs_expected_ + 1, Need{nullptr, 0});
  host_off_.assign(n_str_, nullptr);
  char_scratch_.assign(std::max(n_str_, 1), 0);

  partition_lengths_.assign(P_, 0);
  raw_partition_lengths_.assign(P_, 0);
  segments_.assign(P_, {});
  open_.assign(P_, Segment());
  return Status::OK();
}

Splitter::~Splitter() {
  if (cstream_) cudaStreamSynchronize(cstream_);
  if (hstream_) cudaStreamSynchronize(hstream_);
  if (stream_) cudaStreamSynchronize(stream_);
  if (pstream_) cudaStreamSynchronize(pstream_);
  if (ostream_) cudaStreamSynchronize(ostream_);
  for (auto& f : flushes_) {
    if (f.d_out) cudaFreeAsync(f.d_out, stream_);
    for (auto& e : f.ev)
      if (e) cudaEventDestroy(e);
  }
  ReleaseHost();
  for (auto& c : meta_chunks_) PinnedRelease(c);
  for (int i = 0; i < kTabBufs; i++) {
    PinnedRelease(PinnedBlock{h_tables_[i], tables_cap_[i]});
    if (tab_ev_[i]) cudaEventDestroy(tab_ev_[i]);
  }
  for (int i = 0; i < 2; i++) {
    PinnedRelease(PinnedBlock{h_stage_[i], h_stage_cap_});
    if (d_stage_[i]) cudaFreeAsync(d_stage_[i], stream_);
    if (stage_ev_[i]) cudaEventDestroy(stage_ev_[i]);
  }
  for (int i = 0; i < kScratchBufs; i++) {
    if (d_scratch_[i]) cudaFreeAsync(d_scratch_[i], stream_);
    if (scr_ev_[i]) cudaEventDestroy(scr_ev_[i]);
  }
  if (d_state_) cudaFreeAsync(d_state_, stream_);
  if (d_iota_ || !old_iota_.empty()) {
    if (stream_) cudaStreamSynchronize(stream_);
    if (d_iota_) cudaFree(d_iota_);
    for (int32_t* o : old_iota_) cudaFree(o);
  }
  PinnedRelease(PinnedBlock{reinterpret_cast<uint8_t*>(h_jobs_), h_jobs_bytes_});
  if (gather_ev_) cudaEventDestroy(gather_ev_);
  if (pstream_) cudaStreamDestroy(pstream_);
  if (hstream_) cudaStreamDestroy(hstream_);
  if (hwait_ev_) cudaEventDestroy(hwait_ev_);
  if (cstream_) cudaStreamDestroy(cstream_);
  if (ostream_) cudaStreamDestroy(ostream_);
  if (stream_) cudaStreamDestroy(stream_);
}

// CalculateSplitBatchSize (splitter.cc:800-853).  `host_offsets` (may hold nullptr) are the
// batch's offset buffers per binary column, readable on the host.
uint32_t Splitter::SplitBatchSize(int32_t num_rows, const std::vector<const uint8_t*>& host_offsets,
                                  bool* complete) {
  for (int k = 0; k < n_bin_; k++) {
    if (empirical_[k] == 0 && host_offsets[k] != nullptr && num_rows > 0) {
      // the character bytes of the batch: int32 offsets subtract as int32, int64 as int64
      const int w = sd_.arr_width[fixed_cnt_ + k];
      const int64_t d = OffAt(host_offsets[k], w, (size_t)num_rows) - OffAt(host_offsets[k], w, 0);
      const uint64_t len = w == 8 ? (uint64_t)d : (uint64_t)(uint32_t)(int32_t)d;
      empirical_[k] = len % num_rows == 0 ? len / num_rows : len / num_rows + 1;
    }
  }
  *complete = true;
  for (int k = 0; k < n_bin_; k++)
    if (empirical_[k] == 0) *complete = false;
  uint32_t size_per_row = 0;
  for (int k = 0; k < n_bin_; k++) size_per_row += (uint32_t)empirical_[k];
  for (int a = 0; a < n_policy_; a++) {
    const int ci = array_idx_[a];
    if (ci - out_shift() < fixed_cnt_) {  // an index of the output schema, as in the reference
      const int t = fields_[ci].type;
      size_per_row += t == GZ_TYPE_BOOL ? 0 : ByteWidth(t);
    }
  }
  int64_t rows = opts_.offheap_per_task > 0 && size_per_row > 0
                     ? (opts_.offheap_per_task / size_per_row / P_) >> 2
                     : opts_.buffer_size;
  rows = std::min<int64_t>(rows, opts_.buffer_size);
  return (uint32_t)rows;
}

Status Splitter::EnsureStaging(size_t bytes) {
  if (bytes <= stage_cap_) return Status::OK();
  // the old buffers go: the last pass's k_scatter, which reads them, is queued first
  Status st = LaunchPendingScatter();
  if (!st.ok()) return st;
  st = FinishHostReads();
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(hstream_), "sync");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(stream_), "sync");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(pstream_), "sync");
  if (!st.ok()) return st;
  size_t cap = AlignUp(std::max<size_t>(bytes, (size_t)opts_.flush_bytes + (8u << 20)), 1 << 20);
  for (int i = 0; i < 2; i++) {
    PinnedRelease(PinnedBlock{h_stage_[i], h_stage_cap_});
    if (d_stage_[i]) cudaFreeAsync(d_stage_[i], stream_);
    h_stage_[i] = nullptr;
    d_stage_[i] = nullptr;
    if (!direct_) {
      const PinnedBlock b = PinnedAcquire(cap);
      if (!b.ptr) return Status::Error(GZ_OOM, "pinned host memory for staging");
      h_stage_[i] = b.ptr;
      h_stage_cap_ = b.cap;
    }
    st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d_stage_[i]), cap, stream_), "cudaMallocAsync(stage)");
    if (!st.ok()) return st;
    stage_busy_[i] = false;
  }
  stage_cap_ = cap;
  // the staging is written on cstream_ (k_gather): its allocation on stream_ must be complete
  return Cuda(cudaStreamSynchronize(stream_), "sync");
}

Status Splitter::Split(int32_t num_rows, const int64_t* addrs, const int64_t* sizes, int32_t n) {
  Status st = SplitOne(num_rows, addrs, sizes, n);
  Status fin = FinishHostReads();
  return st.ok() ? fin : st;
}

Status Splitter::SplitBatches(int32_t n_batches, const int32_t* rows, const int64_t* addrs,
                              const int64_t* sizes, int32_t n) {
  Status st = SplitMany(n_batches, rows, addrs, sizes, n);
  Status fin = FinishHostReads();
  return st.ok() ? fin : st;
}

Status Splitter::SplitMany(int32_t n_batches, const int32_t* rows, const int64_t* addrs, const int64_t* sizes,
                           int32_t n) {
  Status st;
  for (int32_t i = 0; i < n_batches && st.ok(); i++)
    st = SplitOne(rows[i], addrs + (size_t)i * n, sizes + (size_t)i * n, n);
  return st;
}

// Launches k_gather over the descriptors queued since the last launch.
Status Splitter::LaunchGather() {
  const size_t n = jobs_end_ - jobs_begin_;
  if (n == 0) return Status::OK();
  Status st = Cuda(launch_gather(h_jobs_ + jobs_begin_, (uint32_t)n, cstream_), "k_gather");
  jobs_begin_ = jobs_end_;
  gather_pending_bytes_ = 0;
  return st;
}

// Waits until every queued host read has landed in device staging; afterwards the caller's
// host buffers are no longer needed and the descriptor ring starts over.
Status Splitter::FinishHostReads() {
  Status st = StartHostReads();
  return st.ok() ? WaitHostReads() : st;
}

// Launches the queued host reads and marks their end; WaitHostReads waits for that mark.
Status Splitter::StartHostReads() {
  if (!direct_ || jobs_end_ == 0) return Status::OK();
  Status st = LaunchGather();
  if (!st.ok()) return st;
  st = Cuda(cudaEventRecord(gather_ev_, cstream_), "event");
  if (!st.ok()) return st;
  reads_marked_ = true;
  return Status::OK();
}

Status Splitter::WaitHostReads() {
  if (!reads_marked_) return Status::OK();
  reads_marked_ = false;
  Status st = Cuda(cudaEventSynchronize(gather_ev_), "host reads");
  if (!st.ok()) return st;
  jobs_begin_ = jobs_end_ = 0;
  return Status::OK();
}

Status SplitGroup(const std::vector<Splitter*>& tasks, const int32_t* n_batches, const int32_t* rows,
                  const int64_t* addrs, const int64_t* sizes, const int32_t* n_bufs, int* failed) {
  // every task's batches are gathered and its host reads started before any task waits, so the
  // tasks' reads are in flight together
  std::vector<Status> st(tasks.size());
  size_t r = 0, a = 0;
  for (size_t i = 0; i < tasks.size(); i++) {
    st[i] = tasks[i]->SplitMany(n_batches[i], rows + r, addrs + a, sizes + a, n_bufs[i]);
    if (st[i].ok()) st[i] = tasks[i]->StartHostReads();
    r += (size_t)n_batches[i];
    a += (size_t)n_batches[i] * (size_t)n_bufs[i];
  }
  for (size_t i = 0; i < tasks.size(); i++) {
    Status w = tasks[i]->WaitHostReads();
    if (st[i].ok()) st[i] = w;
  }
  for (size_t i = 0; i < tasks.size(); i++)
    if (!st[i].ok()) {
      *failed = (int)i;
      return st[i];
    }
  return Status::OK();
}

Status Splitter::SplitOne(int32_t num_rows, const int64_t* addrs, const int64_t* sizes, int32_t n) {
  if (stopped_) return Status::Error(GZ_INVALID, "split after stop");
  if (n < n_bufs_expected_) return Status::Error(GZ_INVALID, "insufficient number of in_buf_addrs");
  if (num_rows < 0) return Status::Error(GZ_INVALID, "negative num_rows");
  if (num_rows == 0) return Status::OK();  // an empty batch changes no splitter state
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  const bool host_in = opts_.input_kind == GZ_INPUT_HOST;
  const uint32_t nr = (uint32_t)num_rows;
  const size_t C = (size_t)n_slots_;  // ColPtr slots: the fields, then the nested streams
  const size_t nf = fields_.size();

  // validate and size every buffer that is read
  uint64_t validity_mask = 0, cvalid_mask = 0;
  size_t batch_bytes = 0;
  for (int k = 0; k < n_str_; k++) host_off_[k] = nullptr;
  for (size_t f = 0; f < nf; f++) {
    const int b0 = field_buf0_[f];
    need_[b0] = Need{nullptr, 0};
    need_[b0 + 1] = Need{nullptr, 0};
    if ((int)f == pid_field_) {
      // FallbackRangeSplitter::ComputeAndCountPartitionId (splitter.cc:1499-1516): int32 ids,
      // validity not read
      if (fields_[f].type != GZ_TYPE_INT32)
        return Status::Error(GZ_INVALID, "RecordBatch field 0 should be int32");
      const size_t vbytes = (size_t)nr * 4;
      if (addrs[b0 + 1] == 0 || (size_t)sizes[b0 + 1] < vbytes)
        return Status::Error(GZ_INVALID, "partition id buffer too small");
      need_[b0 + 1] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 1]), vbytes};
      continue;
    }
    const int a = field_array_[f];
    if (a < 0) continue;  // null type: buffers ignored
    const int t = fields_[f].type;
    if (fields_[f].nested()) {
      // every buffer of the field goes to the device whole; its streams' validity buffers (their
      // row masks and element validity) decide which bit regions the pass allocates
      const int nb = NestedBufferCount(fields_[f]);
      for (int j = b0; j < b0 + nb; j++)
        need_[j] = addrs[j] != 0 && sizes[j] > 0 ? Need{reinterpret_cast<const uint8_t*>(addrs[j]), (size_t)sizes[j]}
                                                 : Need{nullptr, 0};
      for (size_t si = 0; si < streams_.size(); si++) {
        const Stream& sm = streams_[si];
        const NestPlan& np = nest_[sm.plan];
        if (np.field != (int)f) continue;
        const NestNode& nd = np.nodes[sm.node];
        const int maskn = sm.chars ? (nd.ident ? sm.node : nd.mask) : nd.mask;
        const bool entries = nd.parent >= 0 && np.nodes[nd.parent].type == GZ_TYPE_MAP;
        if (maskn >= 0 && need_[np.nodes[maskn].buf].bytes) validity_mask |= 1ull << (first_stream_ + si);
        if (!sm.chars && !entries && need_[nd.buf].bytes) cvalid_mask |= 1ull << (first_stream_ + si);
      }
      continue;
    }
    if (addrs[b0] != 0 && sizes[b0] > 0) {
      const size_t vb = (size_t)BytesForBits(nr);
      if ((size_t)sizes[b0] < vb) return Status::Error(GZ_INVALID, "validity buffer too small");
      need_[b0] = Need{reinterpret_cast<const uint8_t*>(addrs[b0]), vb};
      validity_mask |= 1ull << a;
    }
    if (IsBinary(t)) {
      const int vi = b0 + 2;
      need_[vi] = Need{nullptr, 0};
      const int ow = OffW(t);
      const size_t ob = (size_t)(nr + 1) * ow;
      if (addrs[b0 + 1] == 0 || (size_t)sizes[b0 + 1] < ob)
        return Status::Error(GZ_INVALID, "offsets buffer too small");
      need_[b0 + 1] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 1]), ob};
      const int k = a - fixed_cnt_;
      size_t cb = (size_t)std::max<int64_t>(sizes[vi], 0);
      // the device engine keeps byte positions in 32 bits: a 64-bit-offset column's batch may
      // not address more characters than a 32-bit one can
      if (ow == 8 && sizes[vi] > (int64_t)INT32_MAX)
        return Status::Error(GZ_NOT_IMPLEMENTED, "a large binary column batch with more than 2^31 - 1 character bytes");
      if (host_in) {
        const uint8_t* off = reinterpret_cast<const uint8_t*>(addrs[b0 + 1]);
        host_off_[k] = off;
        const int64_t o0 = OffAt(off, ow, 0), o1 = OffAt(off, ow, nr);
        if (o1 < o0 || o0 < 0 || o1 > sizes[vi])
          return Status::Error(GZ_INVALID, "offsets exceed the value buffer");
        cb = (size_t)o1;
        char_scratch_[k] = (uint64_t)(o1 - o0);
      } else {
        char_scratch_[k] = (uint64_t)cb;
      }
      if (cb > 0) need_[vi] = Need{reinterpret_cast<const uint8_t*>(addrs[vi]), cb};
    } else if (t == GZ_TYPE_LIST) {
      // [validity, int32 offsets, element validity, element values] (jni_common.h:190-226)
      need_[b0 + 2] = Need{nullptr, 0};
      need_[b0 + 3] = Need{nullptr, 0};
      const size_t ob = (size_t)(nr + 1) * 4;
      if (addrs[b0 + 1] == 0 || (size_t)sizes[b0 + 1] < ob)
        return Status::Error(GZ_INVALID, "list offsets buffer too small");
      need_[b0 + 1] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 1]), ob};
      const int k = a - fixed_cnt_;
      const int w = ByteWidth(fields_[f].elem);  // 0: bool elements, one bit each
      const int64_t vsz = std::max<int64_t>(sizes[b0 + 3], 0);
      if (vsz > (int64_t)INT32_MAX)
        return Status::Error(GZ_NOT_IMPLEMENTED, "a list column batch with more than 2^31 - 1 element bytes");
      size_t vb = (size_t)vsz, eb = (size_t)std::max<int64_t>(sizes[b0 + 2], 0);
      if (host_in) {
        const int32_t* off = reinterpret_cast<const int32_t*>(addrs[b0 + 1]);
        const int64_t o0 = off[0], o1 = off[nr];
        if (o1 < o0 || o0 < 0 || (w ? o1 * w : BytesForBits(o1)) > vsz)
          return Status::Error(GZ_INVALID, "list offsets exceed the element values");
        if (addrs[b0 + 2] != 0 && eb > 0 && (int64_t)eb < BytesForBits(o1))
          return Status::Error(GZ_INVALID, "element validity buffer too small");
        vb = (size_t)(w ? o1 * w : BytesForBits(o1));
        eb = eb > 0 ? (size_t)BytesForBits(o1) : 0;
        char_scratch_[k] = (uint64_t)((o1 - o0) * std::max(w, 1));  // bool elements: one "byte" each
      } else {
        char_scratch_[k] = (uint64_t)(w ? vb : vb * 8);
      }
      if (addrs[b0 + 2] != 0 && eb > 0) {
        need_[b0 + 2] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 2]), eb};
        cvalid_mask |= 1ull << a;
      }
      if (vb > 0) need_[b0 + 3] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 3]), vb};
    } else {
      const size_t vbytes = t == GZ_TYPE_BOOL ? (size_t)BytesForBits(nr) : (size_t)nr * ByteWidth(t);
      if (addrs[b0 + 1] == 0 || (size_t)sizes[b0 + 1] < vbytes)
        return Status::Error(GZ_INVALID, "value buffer too small");
      need_[b0 + 1] = Need{reinterpret_cast<const uint8_t*>(addrs[b0 + 1]), vbytes};
    }
  }
  for (int i = 0; i < n_bufs_expected_; i++) batch_bytes += AlignUp(need_[i].bytes, 64);
  // staging room for buffers kept at their source's 16-byte phase (k_gather)
  const size_t phase_slack = direct_ ? (size_t)64 * n_bufs_expected_ : 0;

  // CalculateSplitBatchSize.  Its row count depends on the empirical binary sizes only when
  // offheap_per_task > 0; those sizes are learned from the first batch with rows (where every
  // partition allocates, so the reference always computes them) and, while one is still 0,
  // from each later batch in which some partition reaches the function (splitter.cc:804-835).
  bool probe_call = false;
  std::vector<uint64_t> empirical_before;
  if (opts_.offheap_per_task > 0 && n_bin_ > 0) {
    bool missing = false;
    for (int k = 0; k < n_bin_; k++) missing |= empirical_[k] == 0;
    if (missing && !host_in) {
      st = Cuda(cudaStreamSynchronize(stream_), "sync");
      if (!st.ok()) return st;
      for (int k = 0; k < n_bin_; k++) {
        const int f = array_idx_[fixed_cnt_ + k];
        const int ow = sd_.arr_width[fixed_cnt_ + k];
        const uint8_t* doff = reinterpret_cast<const uint8_t*>(addrs[field_buf0_[f] + 1]);
        dev_off_[k].assign((size_t)(nr + 1) * ow, 0);
        st = Cuda(cudaMemcpy(&dev_off_[k][0], doff, ow, cudaMemcpyDeviceToHost), "read offsets");
        if (!st.ok()) return st;
        st = Cuda(cudaMemcpy(&dev_off_[k][(size_t)nr * ow], doff + (size_t)nr * ow, ow, cudaMemcpyDeviceToHost),
                  "read offsets");
        if (!st.ok()) return st;
        host_off_[k] = dev_off_[k].data();
      }
    }
    probe_call = missing && seen_rows_;
    if (probe_call) empirical_before = empirical_;
  }
  bool complete = true;
  const uint32_t split_size = SplitBatchSize(num_rows, host_off_, &complete);
  seen_rows_ = true;
  last_batch_rows_ = nr;
  const uint32_t ntiles = (nr + kTileRows - 1) / kTileRows;

  // make room in the current flush group
  const size_t NB1 = pending_.size() + 1;
  const size_t jobs_one = sizeof(NestJob) * 2 * streams_.size();  // derived arrays of a batch, at most
  const size_t tables_need = AlignUp(sizeof(BatchDesc) * NB1, 256) +
                             2 * AlignUp(sizeof(TileDesc) * (pending_tiles_ + ntiles), 256) +
                             AlignUp(sizeof(ColPtr) * NB1 * C, 256) + AlignUp(jobs_one * NB1, 256) + 256;
  // (a batch whose call flag is read back has to be alone in its device pass: the earlier
  // batches go first, before this one is staged, so each pass reads its own staging buffer)
  if (!pending_.empty() &&
      (probe_call || pending_bytes_ + batch_bytes > (uint64_t)opts_.flush_bytes ||
       NB1 > (size_t)kMaxBatchesPerFlush ||
       (host_in && used_ + batch_bytes + (direct_ ? phase_slack : tables_need) > stage_cap_))) {
    st = Flush();
    if (!st.ok()) return st;
  }
  ColPtr* cols = nullptr;
  {
    const size_t b = pending_.size();
    pending_cols_.resize((b + 1) * C);
    pending_chars_.resize((b + 1) * std::max(n_str_, 1));
    cols = &pending_cols_[b * C];
    for (int k = 0; k < n_str_; k++) pending_chars_[b * n_str_ + k] = char_scratch_[k];
  }
  if (host_in) {
    const size_t tables_one = AlignUp(sizeof(BatchDesc), 256) + 2 * AlignUp(sizeof(TileDesc) * ntiles, 256) +
                              AlignUp(sizeof(ColPtr) * C, 256) + AlignUp(jobs_one, 256) + 256;
    st = EnsureStaging(batch_bytes + (direct_ ? phase_slack : tables_one));
    if (!st.ok()) return st;
    if (pending_.empty() && stage_busy_[cur_]) {
      // the device pass that last read this staging buffer must be done before it is refilled
      if (direct_) st = Cuda(cudaStreamWaitEvent(cstream_, stage_ev_[cur_], 0), "stage wait");
      else st = Cuda(cudaEventSynchronize(stage_ev_[cur_]), "stage wait");
      if (!st.ok()) return st;
      stage_busy_[cur_] = false;
    }
    if (direct_ && jobs_end_ + (size_t)n_bufs_expected_ > jobs_cap_) {
      st = FinishHostReads();
      if (!st.ok()) return st;
    }
    // the batch goes to device staging: read there by k_gather (direct_) or copied by the CPU
    // into the pinned twin; device addresses point into the device buffer
    jobs_.clear();
    size_t copy_bytes = 0;
    for (size_t f = 0; f < C; f++) {
      ColPtr cp{nullptr, nullptr, nullptr, 0, nullptr};
      const int a = f < nf ? field_array_[f] : -1;
      if (a >= 0 || (int)f == pid_field_) {
        const int t = fields_[f].type;
        const int b0 = field_buf0_[f];
        const bool nested = fields_[f].nested();
        const bool list = t == GZ_TYPE_LIST && !nested;
        const int nbuf = nested ? NestedBufferCount(fields_[f]) : list ? 4 : IsBinary(t) ? 3 : 2;
        for (int j = 0; j < nbuf; j++) {
          const Need& nd = need_[b0 + j];
          if (nested) dptr_[b0 + j] = nullptr;
          if (nd.bytes == 0) continue;
          size_t phase = 0;
          if (direct_) {
            // same 16-byte phase as the source when that keeps the elements aligned (a nested
            // field's buffers stay 64-byte aligned: their element widths vary by node)
            const uintptr_t sp = reinterpret_cast<uintptr_t>(nd.src);
            const uintptr_t elem = j == 0 ? 1
                                 : list ? (j == 1 ? 4 : j == 2 ? 1 : (uintptr_t)std::max(1, ByteWidth(fields_[f].elem)))
                                 : IsBinary(t) ? (j == 1 ? (uintptr_t)OffW(t) : 1)
                                 : t == GZ_TYPE_BOOL ? 1 : (uintptr_t)ByteWidth(t);
            if (!nested && sp % elem == 0) phase = sp & 15;
            h_jobs_[jobs_end_++] = HostCopy{nd.src, d_stage_[cur_] + used_ + phase, nd.bytes};
          } else {
            jobs_.push_back(CopyJob{h_stage_[cur_] + used_, nd.src, nd.bytes});
          }
          copy_bytes += nd.bytes;
          const uint8_t* dptr = d_stage_[cur_] + used_ + phase;
          used_ += AlignUp(phase + nd.bytes, 64);
          if (nested) {  // read through the field's streams (StageNested)
            dptr_[b0 + j] = dptr;
            continue;
          }
          if (j == 0) cp.validity = dptr;
          else if ((IsBinary(t) || list) && j == 1) cp.offsets = reinterpret_cast<const int32_t*>(dptr);
          else if (list && j == 2) cp.child_validity = dptr;
          else {
            cp.values = dptr;
            cp.values_bytes = nd.bytes;
          }
        }
        if ((IsBinary(t) || list) && cp.values == nullptr) cp.values = d_stage_[cur_];  // all empty
      }
      cols[f] = cp;
    }
    if (direct_) {
      stat_h2d_bytes_ += (int64_t)copy_bytes;
      gather_pending_bytes_ += copy_bytes;
      if (gather_pending_bytes_ >= (32u << 20)) {
        st = LaunchGather();
        if (!st.ok()) return st;
      }
    } else {
      ParallelCopy(jobs_, copy_bytes);
    }
  } else {
    for (size_t f = 0; f < C; f++) {
      ColPtr cp{nullptr, nullptr, nullptr, 0, nullptr};
      const int a = f < nf ? field_array_[f] : -1;
      if (a >= 0 || (int)f == pid_field_) {
        const int t = fields_[f].type;
        const int b0 = field_buf0_[f];
        if (fields_[f].nested()) {  // read through the field's streams (StageNested)
          const int nb = NestedBufferCount(fields_[f]);
          for (int j = b0; j < b0 + nb; j++) dptr_[j] = need_[j].bytes ? need_[j].src : nullptr;
          cols[f] = cp;
          continue;
        }
        if (need_[b0].bytes) cp.validity = need_[b0].src;
        if (IsBinary(t)) {
          cp.offsets = reinterpret_cast<const int32_t*>(addrs[b0 + 1]);
          cp.values = reinterpret_cast<const uint8_t*>(addrs[b0 + 2]);
          cp.values_bytes = (uint64_t)std::max<int64_t>(sizes[b0 + 2], 0);
          if (reinterpret_cast<uintptr_t>(cp.offsets) % (uintptr_t)OffW(t))
            return Status::Error(GZ_INVALID, "device offsets buffer must be aligned to its offset width");
        } else if (t == GZ_TYPE_LIST) {
          cp.offsets = reinterpret_cast<const int32_t*>(addrs[b0 + 1]);
          if (addrs[b0 + 2] != 0 && sizes[b0 + 2] > 0) cp.child_validity = reinterpret_cast<const uint8_t*>(addrs[b0 + 2]);
          cp.values = reinterpret_cast<const uint8_t*>(addrs[b0 + 3]);
          cp.values_bytes = (uint64_t)std::max<int64_t>(sizes[b0 + 3], 0);
          if (reinterpret_cast<uintptr_t>(cp.offsets) % 4 ||
              reinterpret_cast<uintptr_t>(cp.values) % (uintptr_t)std::max(1, ByteWidth(fields_[f].elem)))
            return Status::Error(GZ_INVALID, "device list buffers must be aligned to their widths");
          if (cp.values == nullptr) cp.values = reinterpret_cast<const uint8_t*>(addrs[b0 + 1]);  // no elements
        } else {
          cp.values = need_[b0 + 1].src;
          const int w = t == GZ_TYPE_BOOL ? 1 : ByteWidth(t);
          if (reinterpret_cast<uintptr_t>(cp.values) % (uintptr_t)w)
            return Status::Error(GZ_INVALID, "device value buffer is not aligned to its width");
        }
      }
      cols[f] = cp;
    }
  }
  if (!streams_.empty()) {
    st = StageNested(nr, addrs, sizes, dptr_.data(), cols, host_in);
    if (!st.ok()) return st;
    const size_t b = pending_.size();
    for (size_t si = 0; si < streams_.size(); si++) {
      const int k = first_stream_ + (int)si - fixed_cnt_;
      pending_chars_[b * n_str_ + k] = char_scratch_[k];
    }
  }
  pending_bytes_ += batch_bytes;
  pending_tiles_ += ntiles;
  stat_input_bytes_ += (int64_t)batch_bytes;
  stat_batches_++;
  stat_rows_ += nr;
  pending_.push_back(PendingBatch{nr, split_size, validity_mask, cvalid_mask});
  if (probe_call) {
    st = Flush();
    if (!st.ok()) return st;
    uint32_t called = 0;
    st = Cuda(cudaMemcpyAsync(&called, d_call_, 4, cudaMemcpyDeviceToHost, pstream_), "read call flag");
    if (!st.ok()) return st;
    st = Cuda(cudaStreamSynchronize(pstream_), "sync");
    if (!st.ok()) return st;
    if (!called) empirical_ = empirical_before;  // nobody recomputed the sizes in this batch
  }
  return Status::OK();
}

// Small pinned blocks for per-flush metadata, carved from 4 MiB chunks kept until destruction.
Status Splitter::PinnedMeta(size_t bytes, uint32_t** out) {
  bytes = AlignUp(bytes, 256);
  if (meta_chunks_.empty() || meta_used_ + bytes > meta_chunk_cap_) {
    const PinnedBlock c = PinnedAcquire(std::max<size_t>(bytes, 4u << 20));
    if (!c.ptr) return Status::Error(GZ_OOM, "pinned host memory for pass metadata");
    meta_chunks_.push_back(c);
    meta_chunk_cap_ = c.cap;
    meta_used_ = 0;
  }
  *out = reinterpret_cast<uint32_t*>(meta_chunks_.back().ptr + meta_used_);
  meta_used_ += bytes;
  return Status::OK();
}

Status Splitter::EnsureScratch(size_t bytes, bool* fresh) {
  const int i = scr_cur_;
  *fresh = false;
  if (bytes <= scratch_cap_[i]) return Status::OK();
  *fresh = true;
  // stream-ordered (no wait for the whole device, which other splitters may be using): the old
  // buffer is freed on stream_, which already waits for the last k_scatter that read it
  if (d_scratch_[i]) {
    Status st = Cuda(cudaFreeAsync(d_scratch_[i], stream_), "cudaFreeAsync(scratch)");
    if (!st.ok()) return st;
    d_scratch_[i] = nullptr;
  }
  size_t cap = AlignUp(bytes + bytes / 4, 1 << 20);
  Status st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d_scratch_[i]), cap, stream_), "cudaMallocAsync(scratch)");
  if (!st.ok()) return st;
  scratch_cap_[i] = cap;
  return Status::OK();
}

Status Splitter::Flush() {
  if (pending_.empty()) return Status::OK();
  const bool host_in = opts_.input_kind == GZ_INPUT_HOST;
  const uint32_t NB = (uint32_t)pending_.size();
  const size_t C = (size_t)n_slots_;
  const int P = P_;
  const int nstr = n_str_;
  const int A = n_array_;

  // tables
  std::vector<BatchDesc> batches(NB);
  std::vector<SegDesc> segs;
  std::vector<TileDesc> tiles;
  uint64_t R = 0;
  uint64_t emit_bound_a = 0;
  uint32_t smin = UINT32_MAX, capmax = (uint32_t)opts_.buffer_size;
  uint32_t NT = 0;  // tiles
  segs.reserve(pending_tiles_);
  tiles.reserve(pending_tiles_);
  for (uint32_t b = 0; b < NB; b++) {
    const PendingBatch& pb = pending_[b];
    // as few segments as seg_tiles allows, of equal length (no short last segment)
    const uint32_t bt = (pb.nrows + kTileRows - 1) / kTileRows;
    const uint32_t ns = (bt + seg_tiles_ - 1) / seg_tiles_;
    const uint32_t seg_rows = ns ? (bt + ns - 1) / ns * (uint32_t)kTileRows : (uint32_t)kTileRows;
    batches[b] = BatchDesc{pb.nrows, (uint32_t)segs.size(), ns, pb.split_size};
    for (uint32_t g = 0; g < ns; g++) {
      const uint32_t r0 = g * seg_rows;
      const uint32_t nr = std::min<uint32_t>(seg_rows, pb.nrows - r0);
      segs.push_back(SegDesc{b, r0, nr, (uint32_t)(R + r0), NT, {0, 0, 0}});
      for (uint32_t q = 0; q * kTileRows < nr; q++) {
        const uint32_t tr0 = r0 + q * kTileRows;
        tiles.push_back(TileDesc{b, tr0, std::min<uint32_t>(kTileRows, pb.nrows - tr0), (uint32_t)(R + tr0),
                                 (uint32_t)segs.size() - 1, q, {0, 0}});
      }
      NT = (uint32_t)tiles.size();
    }
    R += pb.nrows;
    emit_bound_a += std::min<uint64_t>((uint64_t)P, pb.nrows);
    smin = std::min(smin, pb.split_size);
    capmax = std::max(capmax, pb.nrows);
  }
  if (R >= (1ull << 31)) return Status::Error(GZ_INVALID, "flush too large");
  const uint32_t T = (uint32_t)segs.size();
  const uint64_t emit_bound_b =
      2 * (R + (uint64_t)P * capmax) / std::max<uint32_t>(smin, 1) + 2 * (uint64_t)P + 16;
  const uint32_t emit_cap = (uint32_t)std::min(emit_bound_a, emit_bound_b) + 1;
  const uint64_t pieces_max = (uint64_t)P + emit_cap;
  const uint64_t vbits_max = R + 64 * pieces_max;
  const size_t vwords_bytes = AlignUp((size_t)((vbits_max + 31) / 32) * 4, 256);

  // output layout
  FlushRec fr;
  fr.n_rows = (uint32_t)R;
  fr.n_batches = NB;
  fr.emit_cap = emit_cap;
  fr.off_values.assign(A, SIZE_MAX);
  fr.off_bits.assign(A, SIZE_MAX);
  fr.off_valid.assign(A, SIZE_MAX);
  fr.off_chars.assign(A, SIZE_MAX);
  fr.off_cvalid.assign(A, SIZE_MAX);
  uint64_t any_valid = 0, any_cvalid = 0;
  for (auto& pb : pending_) {
    any_valid |= pb.validity_mask;
    any_cvalid |= pb.cvalid_mask;
  }
  size_t o = 0;
  for (int a = 0; a < A; a++) {
    const int kind = sd_.arr_kind[a];
    if (kind == COL_FIXED) {
      fr.off_values[a] = o;
      o += AlignUp((size_t)R * sd_.arr_width[a], 256);
    } else if (kind == COL_BINARY) {
      fr.off_values[a] = o;
      o += AlignUp((size_t)R * sd_.arr_width[a], 256);  // end offsets, 4 or 8 bytes
      if ((sd_.listbit_mask >> a) & 1ull) continue;     // bool elements: a bit region, below
      if ((lenpay_mask_ >> a) & 1ull) continue;         // lengths: beside the bit regions, below
      uint64_t cb = 0;
      for (uint32_t b = 0; b < NB; b++) cb += pending_chars_[(size_t)b * n_str_ + sd_.arr_str[a]];
      fr.off_chars[a] = o;
      o += AlignUp((size_t)cb + 16, 256);
    }
  }
  const size_t bits_begin = o;
  for (int a = 0; a < A; a++) {
    if (sd_.arr_kind[a] == COL_BOOL) {
      fr.off_bits[a] = o;
      o += vwords_bytes;
    }
    if (any_valid & (1ull << a)) {
      fr.off_valid[a] = o;
      o += vwords_bytes;
    }
    if ((lenpay_mask_ >> a) & 1ull) {  // entries' lengths: read on the host at Stop, as bits are
      uint64_t cb = 0;
      for (uint32_t b = 0; b < NB; b++) cb += pending_chars_[(size_t)b * n_str_ + sd_.arr_str[a]];
      fr.off_chars[a] = o;
      o += AlignUp((size_t)cb + 16, 256);
    }
    if (((sd_.listbit_mask & ~sd_.nopay_mask) >> a) & 1ull) {  // a list of bool elements: one bit per element
      uint64_t cb = 0;
      for (uint32_t b = 0; b < NB; b++) cb += pending_chars_[(size_t)b * n_str_ + sd_.arr_str[a]];
      fr.off_chars[a] = o;
      o += AlignUp((size_t)((cb + 31) / 32 * 4) + 8, 256);
    }
    if (any_cvalid & (1ull << a)) {  // one bit per element byte group of the column's characters
      uint64_t cb = 0;
      for (uint32_t b = 0; b < NB; b++) cb += pending_chars_[(size_t)b * n_str_ + sd_.arr_str[a]];
      fr.off_cvalid[a] = o;
      o += AlignUp((size_t)(((cb >> sd_.arr_shift[a]) + 31) / 32 * 4) + 8, 256);
    }
  }
  const size_t bits_end = o;
  fr.bits_begin = bits_begin;
  fr.bits_end = bits_end;
  fr.out_bytes = std::max<size_t>(o, 256);
  Status st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&fr.d_out), fr.out_bytes, stream_),
                   "cudaMallocAsync(flush output)");
  if (!st.ok()) return st;
  if (bits_end > bits_begin) {
    st = Cuda(cudaMemsetAsync(fr.d_out + bits_begin, 0xff, bits_end - bits_begin, stream_), "memset bits");
    if (!st.ok()) return st;
  }

  // scratch layout
  const size_t TP = (size_t)T * P;
  size_t so = 0;
  auto take = [&](size_t bytes) {
    size_t at = so;
    so += AlignUp(bytes, 256);
    return at;
  };
  const size_t s_pids = take(R * 2);
  const size_t s_cnt = take(TP * 4);
  const size_t s_vpos = take(TP * 4);
  const size_t s_bcnt = take(TP * nstr * 4 + 4);
  const size_t s_sbyte = take(TP * nstr * 4 + 4);
  const size_t s_null = take((size_t)NB * A * 4);
  const size_t s_crange = take((size_t)NT * std::max(nstr, 1) * 8);
  const bool tile_prefix = seg_tiles_ > 1;
  const size_t s_tpre = tile_prefix ? take((size_t)NT * P * 4) : 0;
  const size_t s_tbpre = tile_prefix ? take((size_t)NT * std::max(nstr, 1) * P * 4) : 0;
  const size_t s_call = take((size_t)NB * 4);
  const size_t s_rec = take((size_t)NB * P * 4);
  const size_t s_hn = take((size_t)NB * 8);
  const size_t s_ihn = take((size_t)NB * 8);
  const size_t s_vbits = take((size_t)P * 4);
  const size_t meta_words = (3 + 2 * (size_t)nstr) * P + 1 + (size_t)emit_cap * (kEmitFixedWords + nstr);
  const size_t s_meta = take(meta_words * 4);  // rows_f, pstart, vstart, bytes_f, cstart, count, emits
  // nested columns' derived arrays (k_nest_prep) and their jobs
  std::vector<size_t> der_at(pending_derived_.size(), 0);
  size_t der_bytes = 0, n_jobs = 0;
  for (size_t i = 0; i < pending_derived_.size(); i++) {
    if (pending_derived_[i].same_as >= 0) continue;
    der_at[i] = der_bytes;
    der_bytes += AlignUp(pending_derived_[i].bytes, 256);
    n_jobs++;
  }
  const size_t s_der = der_bytes ? take(der_bytes) : 0;
  const size_t tb_batches = AlignUp(sizeof(BatchDesc) * NB, 256);
  const size_t tb_tiles = AlignUp(sizeof(SegDesc) * T, 256);
  const size_t tb_cols = AlignUp(sizeof(ColPtr) * NB * C, 256);
  const size_t tb_tdesc = AlignUp(sizeof(TileDesc) * NT, 256);
  const size_t tb_jobs = AlignUp(sizeof(NestJob) * n_jobs, 256);
  const size_t tb_total = tb_batches + tb_tiles + tb_cols + tb_tdesc + tb_jobs;
  const bool staged_tables = host_in && !direct_;  // tables travel with the pinned staging copy
  const size_t s_tab = staged_tables ? 0 : take(tb_total);
  // this pass's scratch buffer: stream_ already holds the k_scatter that last read it (queued by
  // an earlier Flush); this pass's work on hstream_ starts after that k_scatter, or after all of
  // stream_'s work so far when the buffer was (re)allocated there
  bool fresh = false;
  st = EnsureScratch(so, &fresh);
  if (!st.ok()) return st;
  uint8_t* S = d_scratch_[scr_cur_];
  if (fresh) {
    st = Cuda(cudaEventRecord(hwait_ev_, stream_), "event");
    if (st.ok()) st = Cuda(cudaStreamWaitEvent(hstream_, hwait_ev_, 0), "wait stream");
  } else if (scr_used_[scr_cur_]) {
    st = Cuda(cudaStreamWaitEvent(hstream_, scr_ev_[scr_cur_], 0), "wait scratch");
  }
  if (!st.ok()) return st;

  FlushDesc fd;
  memset(&fd, 0, sizeof(fd));
  fd.n_batches = NB;
  fd.n_segs = T;
  fd.n_tiles = NT;
  fd.seg_tiles = seg_tiles_;
  fd.n_rows = (uint32_t)R;
  fd.hist_in_smem = (size_t)P * (1 + nstr) * 4 <= kHistSmemBytes ? 1 : 0;
  fd.pids = reinterpret_cast<uint16_t*>(S + s_pids);
  fd.cnt = reinterpret_cast<uint32_t*>(S + s_cnt);
  fd.vpos = reinterpret_cast<uint32_t*>(S + s_vpos);
  fd.bcnt = reinterpret_cast<uint32_t*>(S + s_bcnt);
  fd.sbyte = reinterpret_cast<uint32_t*>(S + s_sbyte);
  fd.nullcnt = reinterpret_cast<uint32_t*>(S + s_null);
  fd.crange = reinterpret_cast<int2*>(S + s_crange);
  fd.tilepre = tile_prefix ? reinterpret_cast<uint32_t*>(S + s_tpre) : nullptr;
  fd.tilebpre = tile_prefix ? reinterpret_cast<uint32_t*>(S + s_tbpre) : nullptr;
  fd.call_flags = reinterpret_cast<uint32_t*>(S + s_call);
  fd.rec_idx = reinterpret_cast<uint32_t*>(S + s_rec);
  fd.hn = reinterpret_cast<unsigned long long*>(S + s_hn);
  fd.ihn = reinterpret_cast<unsigned long long*>(S + s_ihn);
  fd.vbits_f = reinterpret_cast<uint32_t*>(S + s_vbits);
  uint32_t* meta = reinterpret_cast<uint32_t*>(S + s_meta);
  fd.rows_f = meta;
  fd.pstart = meta + P;
  fd.vstart = meta + 2 * (size_t)P;
  fd.bytes_f = meta + 3 * (size_t)P;
  fd.cstart = meta + (3 + (size_t)nstr) * P;
  fd.emit_count = meta + (3 + 2 * (size_t)nstr) * P;
  fd.emit = fd.emit_count + 1;
  fd.emit_cap = emit_cap;
  for (int a = 0; a < A; a++) {
    if (fr.off_values[a] != SIZE_MAX) fd.out_values[a] = fr.d_out + fr.off_values[a];
    if (fr.off_bits[a] != SIZE_MAX) fd.out_bits[a] = reinterpret_cast<uint32_t*>(fr.d_out + fr.off_bits[a]);
    if (fr.off_valid[a] != SIZE_MAX) fd.out_valid[a] = reinterpret_cast<uint32_t*>(fr.d_out + fr.off_valid[a]);
    if (fr.off_chars[a] != SIZE_MAX) fd.out_chars[a] = fr.d_out + fr.off_chars[a];
    if (fr.off_cvalid[a] != SIZE_MAX) fd.out_cvalid[a] = reinterpret_cast<uint32_t*>(fr.d_out + fr.off_cvalid[a]);
  }
  fd.st_cap = st_cap_;
  fd.st_base = st_base_;
  fd.st_hv = st_hv_;
  fd.st_sb = st_sb_;
  fd.st_ihn = st_ihn_;
  fd.err = d_err_;
  fd.rr_base = rr_sel_;
  fd.spin_limit = spin_limit_;
  rr_sel_ = (uint32_t)((rr_sel_ + R) % (uint64_t)P);

  // tables into staging (host inputs) or a pinned table buffer
  uint8_t* htab;
  uint8_t* dtab;
  if (staged_tables) {
    used_ = AlignUp(used_, 256);
    if (used_ + tb_total > stage_cap_) return Status::Error(GZ_INVALID, "staging overflow");
    htab = h_stage_[cur_] + used_;
    dtab = d_stage_[cur_] + used_;
    used_ += tb_total;
  } else {
    // a ring of pinned table buffers; wait only for the copy that last used this one
    const int ti = tab_cur_;
    if (tab_busy_[ti]) {
      st = Cuda(cudaEventSynchronize(tab_ev_[ti]), "table wait");
      if (!st.ok()) return st;
      tab_busy_[ti] = false;
    }
    if (tb_total > tables_cap_[ti]) {
      PinnedRelease(PinnedBlock{h_tables_[ti], tables_cap_[ti]});
      h_tables_[ti] = nullptr;
      const PinnedBlock b = PinnedAcquire(AlignUp(tb_total * 2, 1 << 20));
      if (!b.ptr) return Status::Error(GZ_OOM, "pinned host memory for the pass tables");
      h_tables_[ti] = b.ptr;
      tables_cap_[ti] = b.cap;
      if (!st.ok()) return st;
    }
    htab = h_tables_[ti];
    dtab = nullptr;
  }
  // derived arrays: in this pass's scratch, pointed at from their slots; jobs after the tiles
  {
    NestJob* hj = reinterpret_cast<NestJob*>(htab + tb_batches + tb_tiles + tb_cols + tb_tdesc);
    size_t j = 0;
    for (size_t i = 0; i < pending_derived_.size(); i++) {
      PendingDerived& pd = pending_derived_[i];
      const size_t src = pd.same_as >= 0 ? (size_t)pd.same_as : i;
      int32_t* arr = reinterpret_cast<int32_t*>(S + s_der + der_at[src]);
      ColPtr& cp = pending_cols_[(size_t)pd.batch * C + pd.slot];
      if (pd.values) cp.values = reinterpret_cast<const uint8_t*>(arr);
      else cp.offsets = arr;
      if (pd.same_as >= 0) continue;
      pd.job.out = arr;
      hj[j++] = pd.job;
    }
  }
  memcpy(htab, batches.data(), sizeof(BatchDesc) * NB);
  memcpy(htab + tb_batches, segs.data(), sizeof(SegDesc) * T);
  ColPtr* hc = reinterpret_cast<ColPtr*>(htab + tb_batches + tb_tiles);
  memcpy(hc, pending_cols_.data(), sizeof(ColPtr) * NB * C);
  memcpy(htab + tb_batches + tb_tiles + tb_cols, tiles.data(), sizeof(TileDesc) * NT);
  if (staged_tables) {
    st = Cuda(cudaMemcpyAsync(d_stage_[cur_], h_stage_[cur_], used_, cudaMemcpyHostToDevice, hstream_), "H2D");
    stat_h2d_bytes_ += (int64_t)used_;
    if (!st.ok()) return st;
  } else {
    if (direct_) {  // the pass reads what k_gather wrote
      st = LaunchGather();
      if (!st.ok()) return st;
      st = Cuda(cudaEventRecord(gather_ev_, cstream_), "event");
      if (!st.ok()) return st;
      st = Cuda(cudaStreamWaitEvent(hstream_, gather_ev_, 0), "wait gather");
      if (!st.ok()) return st;
    }
    dtab = S + s_tab;
    st = Cuda(cudaMemcpyAsync(dtab, htab, tb_total, cudaMemcpyHostToDevice, hstream_), "H2D tables");
    if (!st.ok()) return st;
    st = Cuda(cudaEventRecord(tab_ev_[tab_cur_], hstream_), "event");
    if (!st.ok()) return st;
    tab_busy_[tab_cur_] = true;
    tab_cur_ = (tab_cur_ + 1) % kTabBufs;
  }
  fd.batches = reinterpret_cast<const BatchDesc*>(dtab);
  fd.segs = reinterpret_cast<const SegDesc*>(dtab + tb_batches);
  fd.cols = reinterpret_cast<const ColPtr*>(dtab + tb_batches + tb_tiles);
  fd.tiles = reinterpret_cast<const TileDesc*>(dtab + tb_batches + tb_tiles + tb_cols);

  st = Cuda(cudaMemsetAsync(S + s_null, 0, (size_t)NB * A * 4, hstream_), "memset");
  if (!st.ok()) return st;
  st = Cuda(cudaMemsetAsync(S + s_call, 0, (size_t)NB * 4, hstream_), "memset");
  if (!st.ok()) return st;
  st = Cuda(cudaMemsetAsync(fd.emit_count, 0, 4, hstream_), "memset");
  if (!st.ok()) return st;
  if (!fd.hist_in_smem) {
    st = Cuda(cudaMemsetAsync(S + s_cnt, 0, TP * 4, hstream_), "memset");
    if (!st.ok()) return st;
    if (nstr) {
      st = Cuda(cudaMemsetAsync(S + s_bcnt, 0, TP * nstr * 4, hstream_), "memset");
      if (!st.ok()) return st;
    }
  }
  for (auto& e : fr.ev) {
    st = Cuda(cudaEventCreate(&e), "cudaEventCreate");
    if (!st.ok()) return st;
  }
  if (n_jobs) {  // the nested columns' row ranges and lengths, before anything reads them
    st = Cuda(launch_nest_prep(reinterpret_cast<const NestJob*>(dtab + tb_batches + tb_tiles + tb_cols + tb_tdesc),
                               (uint32_t)n_jobs, d_err_, hstream_),
              "k_nest_prep");
    if (!st.ok()) return st;
  }
  cudaEventRecord(fr.ev[0], hstream_);
  st = Cuda(launch_hash_count(sd_, fd, hstream_), "k_hash_count");
  if (!st.ok()) return st;
  cudaEventRecord(fr.ev[1], hstream_);
  // the plan on pstream_, after this pass's k_hash_count (and the previous pass's plan)
  st = Cuda(cudaStreamWaitEvent(pstream_, fr.ev[1], 0), "wait k_hash_count");
  if (!st.ok()) return st;
  cudaEventRecord(fr.ev[5], pstream_);
  st = Cuda(launch_plan(sd_, fd, pstream_), "k_plan");
  if (!st.ok()) return st;
  cudaEventRecord(fr.ev[2], pstream_);
  // the last batch's call flag, for the empirical-size bookkeeping
  st = Cuda(cudaMemcpyAsync(d_call_, fd.call_flags + (NB - 1), 4, cudaMemcpyDeviceToDevice, pstream_), "D2D");
  if (!st.ok()) return st;
  // flush metadata to pinned host memory
  fr.meta_words = meta_words;
  st = PinnedMeta(meta_words * 4, &fr.h_meta);
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpyAsync(fr.h_meta, meta, meta_words * 4, cudaMemcpyDeviceToHost, pstream_), "D2H meta");
  if (!st.ok()) return st;
  cudaEventRecord(fr.ev[6], pstream_);
  // the previous pass's k_scatter goes behind this k_hash_count; this pass's waits for the next
  st = LaunchPendingScatter();
  if (!st.ok()) return st;
  pend_.valid = true;
  pend_.fd = fd;
  pend_.flush = flushes_.size();
  pend_.stage = cur_;
  pend_.host_in = host_in;
  fr.scratch = scr_cur_;
  scr_cur_ = (scr_cur_ + 1) % kScratchBufs;
  // host inputs: the pass is bound by the host link, not by the device; its k_scatter goes
  // right away so its partition data can start back to the host sooner.  So does the first
  // pass's: the device has nothing else to do while the host gathers the next pass.
  const bool scatter_now = host_in || flushes_.empty();

  resident_bytes_ += fr.out_bytes;
  flushes_.push_back(std::move(fr));
  if (scatter_now) {
    st = LaunchPendingScatter();
    if (!st.ok()) return st;
  }
  pending_.clear();
  pending_cols_.clear();
  pending_chars_.clear();
  pending_derived_.clear();
  pending_bytes_ = 0;
  pending_tiles_ = 0;
  if (host_in) {
    cur_ ^= 1;
    used_ = 0;
  }
  return MoveOutputs();
}

// Keeps HBM use under the budget (or moves every finished pass out when asked to): passes whose
// k_scatter is queued go to pinned host memory, oldest first.
Status Splitter::MoveOutputs() {
  const size_t budget = opts_.device_budget > 0 ? (size_t)opts_.device_budget : (64ull << 30);
  for (auto& f : flushes_) {
    if (!(opts_.keep_output_on_device == 0 || resident_bytes_ > budget)) break;
    if (!f.on_host && f.launched) {
      Status st = MoveFlushToHost(f);
      if (!st.ok()) return st;
    }
  }
  return KeepHostBudget();
}

// Queues the k_scatter of the last flushed pass on stream_, after that pass's plan and metadata
// copies; the pass's staging is free again once it has run.
Status Splitter::LaunchPendingScatter() {
  if (!pend_.valid) return Status::OK();
  pend_.valid = false;
  FlushRec& f = flushes_[pend_.flush];
  Status st = Cuda(cudaStreamWaitEvent(stream_, f.ev[6], 0), "wait plan");
  if (!st.ok()) return st;
  cudaEventRecord(f.ev[4], stream_);
  st = Cuda(launch_scatter(sd_, pend_.fd, stream_), "k_scatter");
  if (!st.ok()) return st;
  cudaEventRecord(f.ev[3], stream_);
  f.launched = true;
  st = Cuda(cudaEventRecord(scr_ev_[f.scratch], stream_), "event");
  if (!st.ok()) return st;
  scr_used_[f.scratch] = true;
  if (pend_.host_in) {
    st = Cuda(cudaEventRecord(stage_ev_[pend_.stage], stream_), "event");
    if (!st.ok()) return st;
    stage_busy_[pend_.stage] = true;
  }
  return Status::OK();
}

Status Splitter::Drain() {
  Status st = Flush();
  if (!st.ok()) return st;
  st = LaunchPendingScatter();
  if (!st.ok()) return st;
  return MoveOutputs();
}

// Copies a flush's outputs into a pinned host block and releases the HBM copy (both stream
// ordered); the host bytes are valid once the stream has reached this point.
Status Splitter::MoveFlushToHost(FlushRec& f) {
  if (f.on_host) return Status::OK();
  f.h_out = HostAlloc(f.out_bytes);
  if (!f.h_out) return Status::Error(GZ_OOM, "pinned host memory for partition data");
  // on its own stream, after the pass's kernels, so the copy overlaps the next pass
  if (!f.launched) return Status::Error(GZ_CUDA, "partition data of a pass whose k_scatter is not queued");
  Status st = Cuda(cudaStreamWaitEvent(ostream_, f.ev[3], 0), "wait pass");
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpyAsync(f.h_out, f.d_out, f.out_bytes, cudaMemcpyDeviceToHost, ostream_),
            "D2H out");
  if (!st.ok()) return st;
  st = Cuda(cudaFreeAsync(f.d_out, ostream_), "cudaFreeAsync");
  if (!st.ok()) return st;
  f.d_out = nullptr;
  f.on_host = true;
  resident_bytes_ -= f.out_bytes;
  spilled_to_host_bytes_ += f.out_bytes;
  host_resident_ += f.out_bytes;
  return Status::OK();
}

// A spill file: temp_shuffle_<32 hex digits> in <local dir>/<sub dir as 2 hex digits>, the dirs
// and each dir's sub-directories taken in turn (NextSpilledFileDir, splitter.cc:1346-1353;
// GetSpilledShuffleFileDir / CreateTempShuffleFile, utils.h:55-62, 90-115).
std::string Splitter::NextSpillPath() {
  const std::string& dir = spill_dirs_[dir_sel_];
  char sub[16];
  snprintf(sub, sizeof(sub), "%02x", sub_dir_sel_[dir_sel_]);
  sub_dir_sel_[dir_sel_] = (sub_dir_sel_[dir_sel_] + 1) % opts_.num_sub_dirs;
  dir_sel_ = (dir_sel_ + 1) % (int)spill_dirs_.size();
  const std::string d = dir + "/" + sub;
  mkdir(dir.c_str(), 0777);  // existing dirs are fine; a real failure shows at open
  mkdir(d.c_str(), 0777);
  static std::atomic<uint64_t> seq{0};
  const uint64_t a = (uint64_t)NowNs() ^ ((uint64_t)getpid() << 32), b = seq.fetch_add(1) * 0x9E3779B97F4A7C15ull;
  char name[64];
  snprintf(name, sizeof(name), "temp_shuffle_%016llx%016llx", (unsigned long long)a, (unsigned long long)b);
  return d + "/" + name;
}

// Writes a moved pass's bytes to a new local-dir file, maps it read-only in place of the pinned
// block and gives the block back to the pool; Stop reads the pass through the mapping.
Status Splitter::MoveFlushToFile(FlushRec& f) {
  Status st = Cuda(cudaStreamSynchronize(ostream_), "D2H partition data");  // the bytes have landed
  if (!st.ok()) return st;
  std::string path;
  int fd = -1;
  for (int tries = 0; tries < 8 && fd < 0; tries++) {
    path = NextSpillPath();
    fd = open(path.c_str(), O_RDWR | O_CREAT | O_EXCL | O_CLOEXEC, 0600);
  }
  if (fd < 0) return Status::Error(GZ_IO, "cannot create spill file " + path + ": " + strerror(errno));
  constexpr size_t kPiece = 64u << 20;
  const size_t pieces = (f.out_bytes + kPiece - 1) / kPiece;
  std::atomic<int> err{0};
  ParallelFor(pieces, [&](size_t i) {
    size_t off = i * kPiece;
    const size_t end = std::min(off + kPiece, f.out_bytes);
    while (off < end && err.load() == 0) {
      const ssize_t w = pwrite(fd, f.h_out + off, end - off, (off_t)off);
      if (w <= 0) {
        if (w < 0 && errno == EINTR) continue;
        err.store(w < 0 ? errno : EIO);
        break;
      }
      off += (size_t)w;
    }
  });
  void* m = MAP_FAILED;
  if (err.load() == 0 && f.out_bytes > 0) m = mmap(nullptr, f.out_bytes, PROT_READ, MAP_SHARED, fd, 0);
  const int e = err.load() ? err.load() : errno;
  close(fd);
  if (m == MAP_FAILED) {
    unlink(path.c_str());
    return Status::Error(GZ_IO, "spill file " + path + ": " + strerror(e));
  }
  for (size_t i = 0; i < host_chunks_.size(); i++) {
    if (host_chunks_[i].ptr == f.h_out) {
      PinnedRelease(host_chunks_[i]);
      host_chunks_.erase(host_chunks_.begin() + (long)i);
      break;
    }
  }
  f.h_out = static_cast<uint8_t*>(m);
  f.on_file = true;
  f.spill_path = path;
  host_resident_ -= f.out_bytes;
  disk_files_++;
  disk_files_now_++;
  disk_bytes_ += (int64_t)f.out_bytes;
  return Status::OK();
}

Status Splitter::KeepHostBudget() {
  if (opts_.host_budget <= 0) return Status::OK();
  for (auto& f : flushes_) {
    if (host_resident_ <= (size_t)opts_.host_budget) break;
    if (f.on_host && !f.on_file && f.h_out != nullptr && f.out_bytes > 0) {
      Status st = MoveFlushToFile(f);
      if (!st.ok()) return st;
    }
  }
  return Status::OK();
}

void Splitter::DiskSpillStats(int64_t* out3) const {
  out3[0] = disk_files_;
  out3[1] = disk_bytes_;
  out3[2] = disk_files_now_;
}

Status Splitter::SyncAndCheck() {
  Status st = Cuda(cudaStreamSynchronize(cstream_), "host reads");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(hstream_), "device work");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(stream_), "device work");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(pstream_), "device work");
  if (!st.ok()) return st;
  st = Cuda(cudaStreamSynchronize(ostream_), "partition data to host");
  if (!st.ok()) return st;
  int32_t err = 0;
  st = Cuda(cudaMemcpy(&err, d_err_, 4, cudaMemcpyDeviceToHost), "read error word");
  if (!st.ok()) return st;
  if (err & kErrTimeout) return Status::Error(GZ_TIMEOUT, "a device-side wait timed out");
  if (err & kErrBadOffsets)
    return Status::Error(GZ_INVALID, "binary offsets are decreasing or exceed the value buffer");
  if (err & kErrBadPid)
    return Status::Error(GZ_INVALID, "a partition id is negative or not less than num_partitions");
  if (err & kErrNestSpan)
    return Status::Error(GZ_NOT_IMPLEMENTED,
                         "a null list, map or string entry inside a nested column holds elements");
  if (err) return Status::Error(GZ_CUDA, "device emission list overflow");
  for (; timed_flushes_ < flushes_.size() && flushes_[timed_flushes_].launched; timed_flushes_++) {
    FlushRec& f = flushes_[timed_flushes_];
    float ms[3] = {0, 0, 0};
    cudaEventElapsedTime(&ms[0], f.ev[0], f.ev[1]);
    cudaEventElapsedTime(&ms[1], f.ev[5], f.ev[2]);
    cudaEventElapsedTime(&ms[2], f.ev[4], f.ev[3]);
    kernel_ms_[0] += ms[0];
    kernel_ms_[1] += ms[1];
    kernel_ms_[2] += ms[2];
    kernel_ms_[3] += ms[0] + ms[1] + ms[2];
    total_compute_pid_time_ += (int64_t)(ms[0] * 1e6);
  }
  return Status::OK();
}

// Turns the emission records of finished flushes into per-partition segments.
Status Splitter::ProcessFlushes() {
  const int P = P_;
  const int nstr = n_str_;
  const int words = kEmitFixedWords + nstr;
  for (; processed_flushes_ < flushes_.size(); processed_flushes_++) {
    const int32_t fi = (int32_t)processed_flushes_;
    const FlushRec& f = flushes_[fi];
    const uint32_t ne = f.emit_count(P, nstr);
    if (ne > f.emit_cap) return Status::Error(GZ_CUDA, "emission list overflow");
    const uint32_t* recs = f.emits(P, nstr);
    std::vector<std::vector<const uint32_t*>> by_p(P);
    for (uint32_t i = 0; i < ne; i++) {
      const uint32_t* r = recs + (size_t)i * words;
      if (r[0] >= (uint32_t)P) return Status::Error(GZ_CUDA, "bad emission record");
      by_p[r[0]].push_back(r);
    }
    const uint32_t* rows_f = f.rows_f();
    const uint32_t* bytes_f = f.bytes_f(P);
    for (int p = 0; p < P; p++) {
      auto& v = by_p[p];
      std::sort(v.begin(), v.end(), [](const uint32_t* x, const uint32_t* y) { return x[1] < y[1]; });
      uint32_t frow0 = 0, vpos0 = 0;
      std::vector<uint32_t> fb0(nstr, 0);
      Segment& open = open_[p];
      for (const uint32_t* r : v) {
        const uint32_t frow1 = r[1];
        std::vector<uint32_t> fb1(r + kEmitFixedWords, r + kEmitFixedWords + nstr);
        if (frow1 > frow0) open.pieces.push_back(Piece{fi, frow0, frow1, vpos0, fb0, fb1});
        vpos0 += (frow1 - frow0 + 63u) & ~63u;
        frow0 = frow1;
        fb0 = fb1;
        open.rows = r[2];
        open.hv = (uint64_t)r[3] | ((uint64_t)r[4] << 32);
        open.at_stop = false;
        open.spilled = opts_.prefer_spill != 0;
        uint32_t got = 0;
        for (auto& pc : open.pieces) got += pc.frow1 - pc.frow0;
        if (got != open.rows) return Status::Error(GZ_CUDA, "segment rows do not add up");
        segments_[p].push_back(std::move(open));
        open = Segment();
      }
      if (rows_f[p] > frow0) {
        std::vector<uint32_t> fb1(nstr);
        for (int k = 0; k < nstr; k++) fb1[k] = bytes_f[(size_t)k * P + p];
        open.pieces.push_back(Piece{fi, frow0, rows_f[p], vpos0, fb0, fb1});
      }
    }
  }
  return Status::OK();
}

// Assembles the record batch of segment `s` of partition `p` from the host copies of the
// flush outputs (CacheRecordBatch): its IPC metadata and the byte ranges of its body, padding
// included, ready to be written (WriteIpcPayload).  Reads only, so partitions can be built in
// parallel.
Status Splitter::BuildSegment(int p, const Segment& s, SegMsg* msg, bool device_view) const {
  const int P = P_;
  const int nstr = n_str_;
  const uint32_t n = s.rows;
  // where a pass's body bytes and bit regions are read from
  auto body_base = [&](const FlushRec& f, bool* dev) -> const uint8_t* {
    *dev = device_view;
    return device_view && !f.on_host ? f.d_out : f.h_out;
  };
  auto bit_base = [&](const FlushRec& f, size_t off) -> const uint8_t* {
    return f.on_host ? f.h_out + off : f.h_bits + (off - f.bits_begin);
  };
  std::vector<FieldNodeMeta> nodes;
  std::vector<ChunkedBuffer> bufs;
  std::vector<std::vector<uint8_t>>& temps = msg->temps;
  temps.clear();
  temps.reserve(2 * fields_.size());
  static const uint8_t kZero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int64_t rawb = 0;

  // bits of a per-flush bit region (validity or bool values) for this segment
  auto gather_bits = [&](const std::vector<size_t> FlushRec::*offs, int a, bool* all_ones) -> const uint8_t* {
    const int64_t nb = BytesForBits(n);
    if (s.pieces.size() == 1) {
      const Piece& pc = s.pieces[0];
      const FlushRec& f = flushes_[pc.flush];
      const size_t off = (f.*offs)[a];
      if (off == SIZE_MAX) {
        *all_ones = true;
        return nullptr;
      }
      *all_ones = false;
      const uint64_t bit0 = (uint64_t)f.vstart(P)[p] + pc.vpos0;  // multiple of 64
      return bit_base(f, off) + bit0 / 8;
    }
    temps.emplace_back(nb, 0xff);
    uint8_t* dst = temps.back().data();
    uint64_t drow = 0;
    bool any = false;
    for (const Piece& pc : s.pieces) {
      const FlushRec& f = flushes_[pc.flush];
      const size_t off = (f.*offs)[a];
      const uint32_t len = pc.frow1 - pc.frow0;
      if (off != SIZE_MAX) {
        const uint64_t bit0 = (uint64_t)f.vstart(P)[p] + pc.vpos0;
        CopyBits(bit_base(f, off), bit0, dst, drow, len);
        any = true;
      }
      drow += len;
    }
    *all_ones = !any;
    return any ? dst : nullptr;
  };

  for (size_t fi = 0; fi < fields_.size(); fi++) {
    if ((int)fi == pid_field_) continue;  // not in the output schema
    const int a = field_array_[fi];
    if (a < 0) {
      nodes.push_back(FieldNodeMeta{n, n});
      continue;
    }
    if (fields_[fi].nested()) {  // its builder's output (splitter.cc:532-545), rebuilt from its streams
      for (const NestPlan& np : nest_)
        if (np.field == (int)fi) BuildNested(p, s, np, 0, &nodes, &bufs, &temps, device_view, &rawb);
      continue;
    }
    if ((sd_.list_mask >> a) & 1ull) {
      // a list column, as its partition's ListBuilder finishes it (CacheRecordBatch,
      // splitter.cc:532-545): list node and buffers [validity, offsets], then the element node
      // and [validity, values]; each bitmap zero-padded and written only when it holds a null
      const int k = sd_.arr_str[a];
      const int sh = sd_.arr_shift[a];
      int64_t lnulls = 0;
      ChunkedBuffer lvb;
      {
        bool ones = true;
        const uint8_t* bits = gather_bits(&FlushRec::off_valid, a, &ones);
        if (!ones && (lnulls = CountZeros(bits, n)) > 0) {
          temps.emplace_back(bits, bits + BytesForBits(n));
          if (n & 7) temps.back().back() &= (uint8_t)((1u << (n & 7)) - 1);
          lvb.push_back(Chunk{temps.back().data(), BytesForBits(n)});
        }
      }
      ChunkedBuffer offs, vals;
      offs.push_back(Chunk{kZero8, 4});
      uint64_t elems = 0;
      for (const Piece& pc : s.pieces) elems += (pc.fb1[k] - pc.fb0[k]) >> sh;
      temps.emplace_back((size_t)BytesForBits((int64_t)elems), 0);
      uint8_t* ev = temps.back().data();
      const bool bitvals = (sd_.listbit_mask >> a) & 1ull;  // bool elements: gathered bits
      uint8_t* bv = nullptr;
      if (bitvals) {
        temps.emplace_back((size_t)BytesForBits((int64_t)elems), 0);
        bv = temps.back().data();
      }
      uint64_t erow = 0;
      for (const Piece& pc : s.pieces) {
        const FlushRec& f = flushes_[pc.flush];
        bool dev;
        const uint8_t* fb = body_base(f, &dev);
        offs.push_back(Chunk{fb + f.off_values[a] + ((size_t)f.pstart(P)[p] + pc.frow0) * 4,
                             (int64_t)(pc.frow1 - pc.frow0) * 4, dev});
        const uint32_t c0 = pc.fb0[k], c1 = pc.fb1[k];
        const size_t cb = (size_t)f.cstart(P, nstr)[(size_t)k * P + p] + c0;
        const uint64_t m = (c1 - c0) >> sh;
        if (bitvals) CopyBits(bit_base(f, f.off_chars[a]), cb, bv, erow, m);
        else if (c1 > c0) vals.push_back(Chunk{fb + f.off_chars[a] + cb, (int64_t)(c1 - c0), dev});
        if (f.off_cvalid[a] != SIZE_MAX) {
          CopyBits(bit_base(f, f.off_cvalid[a]), cb >> sh, ev, erow, m);
        } else {
          for (uint64_t i = erow; i < erow + m; i++) ev[i >> 3] |= (uint8_t)(1u << (i & 7));
        }
        erow += m;
      }
      if (bitvals) vals.push_back(Chunk{bv, BytesForBits((int64_t)elems)});
      const int64_t cnulls = CountZeros(ev, (int64_t)elems);
      ChunkedBuffer cvb;
      if (cnulls > 0) cvb.push_back(Chunk{ev, BytesForBits((int64_t)elems)});
      nodes.push_back(FieldNodeMeta{n, lnulls});
      nodes.push_back(FieldNodeMeta{(int64_t)elems, cnulls});
      bufs.push_back(lvb);
      bufs.push_back(offs);
      bufs.push_back(cvb);
      bufs.push_back(vals);
      // batch_nbytes: the list's own buffers (splitter.cc:438-453)
      rawb += (lnulls > 0 ? BytesForBits(n) : 0) + (int64_t)(n + 1) * 4;
      continue;
    }
    const int kind = sd_.arr_kind[a];
    int64_t nulls = 0;
    ChunkedBuffer vb;
    if (s.hv & (1ull << a)) {
      rawb += BytesForBits(n);
      bool ones = true;
      const uint8_t* bits = gather_bits(&FlushRec::off_valid, a, &ones);
      if (!ones && s.valid_wipe_rows > 0) {
        temps.emplace_back(bits, bits + BytesForBits(n));
        uint8_t* w = temps.back().data();
        for (uint32_t r = 0; r < s.valid_wipe_rows && r < n; r++) w[r >> 3] |= (uint8_t)(1u << (r & 7));
        bits = w;
      }
      if (!ones) {
        nulls = CountZeros(bits, n);
        if (nulls > 0) vb.push_back(Chunk{bits, BytesForBits(n)});
      }
    }
    nodes.push_back(FieldNodeMeta{n, nulls});
    bufs.push_back(vb);
    if (kind == COL_FIXED) {
      const int w = sd_.arr_width[a];
      ChunkedBuffer vals;
      for (const Piece& pc : s.pieces) {
        const FlushRec& f = flushes_[pc.flush];
        bool dev;
        const uint8_t* base = body_base(f, &dev) + f.off_values[a];
        vals.push_back(Chunk{base + ((size_t)f.pstart(P)[p] + pc.frow0) * w,
                             (int64_t)(pc.frow1 - pc.frow0) * w, dev});
      }
      rawb += (int64_t)n * w;
      bufs.push_back(vals);
    } else if (kind == COL_BOOL) {
      bool ones = true;
      const uint8_t* bits = gather_bits(&FlushRec::off_bits, a, &ones);
      if (ones) {
        temps.emplace_back(BytesForBits(n), 0xff);
        bits = temps.back().data();
      }
      rawb += BytesForBits(n);
      bufs.push_back(ChunkedBuffer{Chunk{bits, BytesForBits(n)}});
    } else {
      const int k = sd_.arr_str[a];
      ChunkedBuffer offs, chars;
      const int ow = sd_.arr_width[a];  // offset bytes
      offs.push_back(Chunk{kZero8, ow});
      int64_t clen = 0;
      for (const Piece& pc : s.pieces) {
        const FlushRec& f = flushes_[pc.flush];
        bool dev;
        const uint8_t* fb = body_base(f, &dev);
        const uint8_t* ob = fb + f.off_values[a];
        offs.push_back(Chunk{ob + ((size_t)f.pstart(P)[p] + pc.frow0) * ow, (int64_t)(pc.frow1 - pc.frow0) * ow, dev});
        const uint8_t* cb = fb + f.off_chars[a];
        const uint32_t c0 = pc.fb0[k], c1 = pc.fb1[k];
        if (c1 > c0)
          chars.push_back(Chunk{cb + (size_t)f.cstart(P, nstr)[(size_t)k * P + p] + c0, (int64_t)(c1 - c0), dev});
        clen += c1 - c0;
      }
      rawb += (int64_t)(n + 1) * ow + clen;
      bufs.push_back(offs);
      bufs.push_back(chars);
    }
  }
  msg->raw = rawb;
  msg->rows = n;
  if (device_view) {  // the body is encoded after the device has compressed / copied it
    msg->nodes = std::move(nodes);
    msg->bufs = std::move(bufs);
    return Status::OK();
  }
  std::vector<int64_t> lens(bufs.size(), 0);
  for (size_t i = 0; i < bufs.size(); i++)
    for (const Chunk& c : bufs[i]) lens[i] += c.len;
  RecordBatchHeader(n, nodes, lens, &msg->header, &msg->body);
  // the body: every buffer's chunks, then zeros up to its 8-byte boundary
  msg->pieces.clear();
  for (size_t i = 0; i < bufs.size(); i++) {
    for (const Chunk& c : bufs[i])
      if (c.len > 0) msg->pieces.push_back(c);
    const int64_t pad = ((lens[i] + 7) & ~int64_t(7)) - lens[i];
    if (pad) msg->pieces.push_back(Chunk{kZero8, pad});
  }
  msg->bytes = (int64_t)msg->header.size() + msg->body;
  return Status::OK();
}

namespace {

// Gathers byte ranges and writes them at consecutive offsets of a file (pwritev, at most
// IOV_MAX ranges a call) or copies them into memory.
class RangeWriter {
 public:
  RangeWriter(int fd, uint8_t* mem, int64_t offset) : fd_(fd), mem_(mem), off_(offset) {}
  bool Add(const void* p, int64_t n) {
    if (n <= 0) return true;
    if (mem_) {
      memcpy(mem_ + off_, p, (size_t)n);
      off_ += n;
      return true;
    }
    iov_.push_back(iovec{const_cast<void*>(p), (size_t)n});
    pending_ += n;
    return iov_.size() < kMaxIov || Flush();
  }
  bool Flush() {
    size_t i = 0;
    while (i < iov_.size()) {
      const int cnt = (int)std::min(iov_.size() - i, kMaxIov);
      const ssize_t w = pwritev(fd_, iov_.data() + i, cnt, off_);
      if (w < 0) {
        if (errno == EINTR) continue;
        return false;
      }
      off_ += w;
      // drop the ranges written in full; shorten a range written in part
      size_t left = (size_t)w;
      while (i < iov_.size() && left >= iov_[i].iov_len) left -= iov_[i++].iov_len;
      if (left) {
        iov_[i].iov_base = static_cast<uint8_t*>(iov_[i].iov_base) + left;
        iov_[i].iov_len -= left;
      }
    }
    iov_.clear();
    pending_ = 0;
    return true;
  }

 private:
  static constexpr size_t kMaxIov = 1024;
  int fd_;
  uint8_t* mem_;
  int64_t off_;
  int64_t pending_ = 0;
  std::vector<iovec> iov_;
};

}  // namespace

Status Splitter::Stop() {
  if (stopped_) return Status::Error(GZ_INVALID, "splitter already stopped");
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  st = Drain();
  if (!st.ok()) return st;
  st = SyncAndCheck();
  if (!st.ok()) return st;
  st = ProcessFlushes();
  if (!st.ok()) return st;
  // the open buffer of every partition is emitted at Stop (CacheRecordBatch(pid, true))
  std::vector<uint32_t> base(P_);
  std::vector<unsigned long long> hv(P_);
  st = Cuda(cudaMemcpy(base.data(), st_base_, 4 * (size_t)P_, cudaMemcpyDeviceToHost), "D2H state");
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpy(hv.data(), st_hv_, 8 * (size_t)P_, cudaMemcpyDeviceToHost), "D2H state");
  if (!st.ok()) return st;
  for (int p = 0; p < P_; p++) {
    Segment& open = open_[p];
    if (base[p] > 0) {
      open.rows = base[p];
      open.hv = hv[p];
      open.at_stop = true;
      uint32_t got = 0;
      for (auto& pc : open.pieces) got += pc.frow1 - pc.frow0;
      if (got != open.rows) return Status::Error(GZ_CUDA, "open segment rows do not add up");
      segments_[p].push_back(std::move(open));
    }
    open = Segment();
  }
  const bool compressed = codec_ != GZ_CODEC_UNCOMPRESSED;
  const int64_t m0 = NowNs();
  for (auto& f : flushes_) {
    if (!compressed) {
      st = MoveFlushToHost(f);
    } else if (!f.on_host && f.bits_end > f.bits_begin) {
      // the device compresses the bodies where they are; only the bit regions (null counts,
      // bitmaps assembled on the host) come over now
      f.h_bits = HostAlloc(f.bits_end - f.bits_begin);
      if (!f.h_bits) return Status::Error(GZ_OOM, "pinned host memory for validity bits");
      st = Cuda(cudaMemcpyAsync(f.h_bits, f.d_out + f.bits_begin, f.bits_end - f.bits_begin,
                                cudaMemcpyDeviceToHost, ostream_), "D2H bits");
    }
    if (!st.ok()) return st;
  }
  st = Cuda(cudaStreamSynchronize(ostream_), "D2H partition data");
  if (!st.ok()) return st;
  total_spill_time_ += NowNs() - m0;

  // Stop (splitter.cc:395-437): partitions in order, each [schema message if write_schema] +
  // its record batches + EOS when it has rows, else nothing.  Partitions are independent: their
  // messages are built in parallel, which gives every partition's length and so its offset in
  // the data file; then they are written in parallel at those offsets.
  const int64_t c0 = NowNs();
  std::vector<Field> out_fields = fields_;
  if (pid_field_ >= 0) out_fields.erase(out_fields.begin() + pid_field_);
  const std::vector<uint8_t> schema_msg = opts_.write_schema ? EncodeSchemaMessage(out_fields) : std::vector<uint8_t>();
  std::vector<std::vector<SegMsg>> msgs(P_);
  std::vector<Status> pst(P_);
  ParallelFor((size_t)P_, [&](size_t pi) {
    const int p = (int)pi;
    const auto& segs = segments_[p];
    msgs[p].resize(segs.size());
    for (size_t i = 0; i < segs.size(); i++) {
      Status b = BuildSegment(p, segs[i], &msgs[p][i], compressed);
      if (!b.ok()) {
        pst[p] = b;
        return;
      }
    }
  });
  for (int p = 0; p < P_; p++)
    if (!pst[p].ok()) return pst[p];
  if (compressed) {
    st = CompressBodies(&msgs);
    if (!st.ok()) return st;
  }
  for (int p = 0; p < P_; p++) {
    if (msgs[p].empty()) {
      partition_lengths_[p] = 0;
      continue;
    }
    int64_t len = (int64_t)schema_msg.size() + 8;  // + EOS
    for (const SegMsg& m : msgs[p]) {
      len += m.bytes;
      raw_partition_lengths_[p] += m.raw;
    }
    partition_lengths_[p] = len;
  }
  std::vector<int64_t> start(P_ + 1, 0);
  for (int p = 0; p < P_; p++) {
    start[p + 1] = start[p] + partition_lengths_[p];
    for (size_t i = 0; i < segments_[p].size(); i++) {
      segments_[p][i].message_bytes = msgs[p][i].bytes;
      segments_[p][i].body_length = msgs[p][i].body;
      if (segments_[p][i].spilled) total_bytes_spilled_ += msgs[p][i].bytes;
    }
  }
  const int64_t total = start[P_];
  total_compress_time_ += NowNs() - c0;

  const int64_t t0 = NowNs();
  int fd = -1;
  uint8_t* mem = nullptr;
  void* mapped = nullptr;
  if (data_file_.empty()) {
    data_bytes_.assign((size_t)total, 0);
    mem = data_bytes_.data();
  } else {
    fd = open(data_file_.c_str(), O_RDWR | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return Status::Error(GZ_IO, "cannot open data file " + data_file_ + ": " + strerror(errno));
    struct stat sb;
    const bool regular = fstat(fd, &sb) == 0 && S_ISREG(sb.st_mode);  // not e.g. /dev/null
    if (regular && total > 0 && ftruncate(fd, total) != 0) {
      const std::string why = strerror(errno);
      close(fd);
      return Status::Error(GZ_IO, "cannot size data file " + data_file_ + ": " + why);
    }
    // Writes to one file serialise on the file's lock; a large file is mapped instead, so that
    // the partitions are copied into it in parallel.
    if (regular && total >= kMapWriteBytes) {
      mapped = mmap(nullptr, (size_t)total, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
      if (mapped == MAP_FAILED) mapped = nullptr;
      else mem = static_cast<uint8_t*>(mapped);
    }
  }
  static const uint32_t kEos[2] = {0xFFFFFFFFu, 0u};  // WriteEOS (splitter.cc:166-172)
  std::vector<char> wrote(P_, 1);
  ParallelFor((size_t)P_, [&](size_t pi) {
    const int p = (int)pi;
    if (msgs[p].empty()) return;
    RangeWriter w(fd, mem, start[p]);
    bool ok = w.Add(schema_msg.data(), (int64_t)schema_msg.size());
    for (const SegMsg& m : msgs[p]) {
      ok = ok && w.Add(m.header.data(), (int64_t)m.header.size());
      for (const Chunk& c : m.pieces) ok = ok && w.Add(c.data, c.len);
    }
    ok = ok && w.Add(kEos, 8) && w.Flush();
    wrote[p] = ok;
  });
  bool ok = true;
  for (int p = 0; p < P_; p++) ok = ok && wrote[p];
  if (mapped && munmap(mapped, (size_t)total) != 0) ok = false;
  if (fd >= 0 && close(fd) != 0) ok = false;
  if (!ok) return Status::Error(GZ_IO, "writing the data file failed: " + data_file_);
  total_bytes_written_ += total;
  stat_emitted_ = 0;
  for (auto& v : segments_) stat_emitted_ += (int64_t)v.size();
  total_write_time_ += NowNs() - t0;
  stopped_ = true;
  // the pinned copies are no longer needed
  ReleaseHost();
  ReleaseStaging();
  return Status::OK();
}

Status Splitter::CompressBodies(std::vector<std::vector<SegMsg>>* msgs_p) {
  auto& msgs = *msgs_p;
  const int64_t threshold = opts_.batch_compress_threshold;
  auto lz4 = [&](const SegMsg& m) { return codec_ == GZ_CODEC_LZ4_FRAME && (int64_t)m.rows > threshold; };
  // 1. the device work: every device-readable body range, cut into chunks (LZ4 blocks of at
  //    most kLz4MaxBlock bytes for compressed batches, plain copies of at most 1 MiB for the others)
  constexpr uint32_t kCopyChunk = 1u << 20;
  std::vector<Lz4Chunk> chunks;
  std::vector<std::vector<uint32_t>> first(P_);  // first chunk of each message
  uint64_t arena_bytes = 0;
  for (int p = 0; p < P_; p++) {
    first[p].resize(msgs[p].size());
    for (size_t i = 0; i < msgs[p].size(); i++) {
      const SegMsg& m = msgs[p][i];
      first[p][i] = (uint32_t)chunks.size();
      const uint32_t step = lz4(m) ? kLz4MaxBlock : kCopyChunk;
      for (const ChunkedBuffer& b : m.bufs)
        for (const Chunk& c : b) {
          if (!c.dev) continue;
          for (int64_t x = 0; x < c.len; x += step) {
            const uint32_t len = (uint32_t)std::min<int64_t>(step, c.len - x);
            chunks.push_back(Lz4Chunk{c.data + x, len, lz4(m) ? 0u : 1u});
            arena_bytes += AlignUp(len, 16);
          }
        }
    }
  }
  std::vector<Lz4Block> res(chunks.size());
  uint8_t* arena = nullptr;
  if (!chunks.empty()) {
    const size_t n = chunks.size();
    const size_t scratch = (size_t)lz4_compress_warps() * kLz4Slot;
    const size_t tab = AlignUp(sizeof(Lz4Chunk) * n, 256), rb = AlignUp(sizeof(Lz4Block) * n, 256);
    uint8_t* d = nullptr;
    Status st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d), tab + rb + 256 + scratch + arena_bytes, stream_),
                     "cudaMallocAsync(compression)");
    if (!st.ok()) return st;
    Lz4Chunk* d_chunks = reinterpret_cast<Lz4Chunk*>(d);
    Lz4Block* d_res = reinterpret_cast<Lz4Block*>(d + tab);
    unsigned long long* d_used = reinterpret_cast<unsigned long long*>(d + tab + rb);
    uint32_t* d_next = reinterpret_cast<uint32_t*>(d + tab + rb + 8);
    int32_t* d_err = reinterpret_cast<int32_t*>(d + tab + rb + 16);
    uint8_t* d_scratch = d + tab + rb + 256;
    uint8_t* d_arena = d_scratch + scratch;
    unsigned long long used = 0;
    int32_t err = 0;
    st = Cuda(cudaMemcpyAsync(d_chunks, chunks.data(), sizeof(Lz4Chunk) * n, cudaMemcpyHostToDevice, stream_), "H2D chunks");
    if (st.ok()) st = Cuda(cudaMemsetAsync(d + tab + rb, 0, 256, stream_), "memset");
    const int64_t c0 = NowNs();
    if (st.ok())
      st = Cuda(launch_lz4_compress(d_chunks, (uint32_t)n, d_next, d_scratch, d_arena, d_used, arena_bytes, d_res,
                                    d_err, stream_), "k_lz4_compress");
    if (st.ok()) st = Cuda(cudaMemcpyAsync(res.data(), d_res, sizeof(Lz4Block) * n, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (st.ok()) st = Cuda(cudaMemcpyAsync(&used, d_used, 8, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (st.ok()) st = Cuda(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (st.ok()) st = Cuda(cudaStreamSynchronize(stream_), "k_lz4_compress");
    total_compress_time_ += NowNs() - c0;
    if (st.ok() && (err || used > arena_bytes)) st = Status::Error(GZ_CUDA, "compression arena overflow");
    if (st.ok() && used > 0) {  // only the bytes the blocks took come to the host
      arena = HostAlloc(used);
      if (!arena) st = Status::Error(GZ_OOM, "pinned host memory for compressed bodies");
      if (st.ok()) st = Cuda(cudaMemcpyAsync(arena, d_arena, used, cudaMemcpyDeviceToHost, stream_), "D2H bodies");
      if (st.ok()) st = Cuda(cudaStreamSynchronize(stream_), "D2H bodies");
    }
    cudaFreeAsync(d, stream_);
    if (!st.ok()) return st;
  }
  // 2. the messages: compressed buffers as uncompressed length + LZ4 frame of the chunks' blocks
  //    (host-side ranges, e.g. assembled bitmaps, as stored blocks); the rest as plain bytes
  static const uint8_t kZero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  ParallelFor((size_t)P_, [&](size_t pi) {
    const int p = (int)pi;
    for (size_t i = 0; i < msgs[p].size(); i++) {
      SegMsg& m = msgs[p][i];
      const bool z = lz4(m);
      uint32_t k = first[p][i];
      std::vector<int64_t> lens(m.bufs.size(), 0);
      std::vector<Chunk> body;
      for (size_t b = 0; b < m.bufs.size(); b++) {
        int64_t raw_len = 0;
        for (const Chunk& c : m.bufs[b]) raw_len += c.len;
        if (raw_len == 0) continue;  // an empty buffer stays empty
        const size_t at = body.size();
        if (z) {
          std::vector<Lz4BlockRef> blocks;
          for (const Chunk& c : m.bufs[b]) {
            for (int64_t x = 0; x < c.len; x += kLz4MaxBlock) {
              const uint32_t len = (uint32_t)std::min<int64_t>(kLz4MaxBlock, c.len - x);
              if (c.dev) {
                const Lz4Block& r = res[k++];
                blocks.push_back(Lz4BlockRef{arena + r.pos, r.size, r.stored != 0});
              } else {
                blocks.push_back(Lz4BlockRef{c.data + x, len, true});
              }
            }
          }
          lens[b] = AppendLz4Buffer(raw_len, blocks, &body, &m.temps);
        } else {
          for (const Chunk& c : m.bufs[b]) {
            if (!c.dev) {
              body.push_back(c);
              continue;
            }
            for (int64_t x = 0; x < c.len; x += kCopyChunk) {
              const Lz4Block& r = res[k++];
              body.push_back(Chunk{arena + r.pos, (int64_t)r.size});
            }
          }
          lens[b] = raw_len;
        }
        (void)at;
        const int64_t pad = ((lens[b] + 7) & ~int64_t(7)) - lens[b];
        if (pad) body.push_back(Chunk{kZero8, pad});
      }
      if (z) CompressedRecordBatchHeader(m.rows, m.nodes, lens, &m.header, &m.body);
      else RecordBatchHeader(m.rows, m.nodes, lens, &m.header, &m.body);
      m.pieces = std::move(body);
      m.bytes = (int64_t)m.header.size() + m.body;
    }
  });
  return Status::OK();
}

// Pinned host space for one pass's partition data, from the process-wide pool; everything goes
// back at Stop.
uint8_t* Splitter::HostAlloc(size_t bytes) {
  PinnedBlock b = PinnedAcquire(bytes);
  if (!b.ptr) return nullptr;
  host_chunks_.push_back(b);
  return b.ptr;
}

void Splitter::ReleaseHost() {
  for (auto& b : host_chunks_) PinnedRelease(b);
  host_chunks_.clear();
  for (auto& f : flushes_) {
    if (f.on_file) {  // the pass's local-dir file: unmapped and deleted
      munmap(f.h_out, f.out_bytes);
      unlink(f.spill_path.c_str());
      f.on_file = false;
      disk_files_now_--;
    }
    f.h_out = nullptr;
  }
  host_resident_ = 0;
}

// After Stop nothing more is split: staging and scratch go back (all streams are idle).
void Splitter::ReleaseStaging() {
  for (int i = 0; i < 2; i++) {
    PinnedRelease(PinnedBlock{h_stage_[i], h_stage_cap_});
    if (d_stage_[i]) cudaFreeAsync(d_stage_[i], stream_);
    h_stage_[i] = nullptr;
    d_stage_[i] = nullptr;
    stage_busy_[i] = false;
  }
  stage_cap_ = 0;
  for (int i = 0; i < kScratchBufs; i++) {
    if (d_scratch_[i]) cudaFreeAsync(d_scratch_[i], stream_);
    d_scratch_[i] = nullptr;
    scratch_cap_[i] = 0;
  }
}

Status Splitter::SpillFixedSize(int64_t size, int64_t* actual) {
  *actual = 0;
  if (opts_.prefer_spill) return Status::OK();  // every emitted batch was spilled already
  // cached batches exist only without prefer_spill: make them visible on the host
  Status st = Drain();
  if (!st.ok()) return st;
  st = SyncAndCheck();
  if (!st.ok()) return st;
  st = ProcessFlushes();
  if (!st.ok()) return st;
  for (auto& f : flushes_) {
    st = MoveFlushToHost(f);
    if (!st.ok()) return st;
  }
  st = Cuda(cudaStreamSynchronize(ostream_), "D2H partition data");
  if (!st.ok()) return st;
  st = KeepHostBudget();
  if (!st.ok()) return st;
  // SpillLargestPartition up to 5 times (splitter.cc:741-799): largest cached body bytes
  int64_t cur = 0;
  int tries = 0;
  while (cur < size && tries < 5) {
    tries++;
    int64_t best = 0;
    int pick = -1;
    for (int p = 0; p < P_; p++) {
      int64_t cached = 0;
      for (Segment& s : segments_[p]) {
        if (s.spilled) continue;
        if (s.body_length < 0) {
          SegMsg m;
          st = BuildSegment(p, s, &m);
          if (!st.ok()) return st;
          s.body_length = m.body;
          s.message_bytes = m.bytes;
        }
        cached += s.body_length;
      }
      if (cached > best) {
        best = cached;
        pick = p;
      }
    }
    if (pick < 0) break;
    for (Segment& s : segments_[pick]) s.spilled = true;
    // SpillPartition also refills the validity of the open buffers, pending rows included
    uint32_t open_rows = 0;
    for (const Piece& pc : open_[pick].pieces) open_rows += pc.frow1 - pc.frow0;
    open_[pick].valid_wipe_rows = std::max(open_[pick].valid_wipe_rows, open_rows);
    cur += best;
  }
  *actual = cur;
  return Status::OK();
}

Status Splitter::SetCompressType(int32_t codec) {
  if (codec != GZ_CODEC_UNCOMPRESSED && codec != GZ_CODEC_LZ4_FRAME)
    return Status::Error(GZ_NOT_IMPLEMENTED, "codec " + std::to_string(codec) + " is not implemented");
  codec_ = codec;
  return Status::OK();
}

// IPC body length of the input batch (Splitter::CompressedSize, splitter.cc:358-369).
Status Splitter::CompressedSize(int32_t num_rows, const int64_t* addrs, const int64_t* sizes,
                                int32_t n, int64_t* out) {
  if (n < n_bufs_expected_) return Status::Error(GZ_INVALID, "insufficient number of in_buf_addrs");
  if (opts_.input_kind != GZ_INPUT_HOST)
    return Status::Error(GZ_NOT_IMPLEMENTED, "CompressedSize reads host buffers");
  const uint32_t nr = (uint32_t)std::max(num_rows, 0);
  auto pad8 = [](int64_t x) { return (x + 7) & ~int64_t(7); };
  // the body buffers as the IPC writer lays them out (validity only with nulls)
  std::vector<std::pair<const uint8_t*, int64_t>> bufs;
  std::vector<std::vector<uint8_t>> temps;
  for (size_t f = 0; f < fields_.size(); f++) {
    const int t = fields_[f].type;
    if (t == GZ_TYPE_NULL) continue;
    const int b0 = field_buf0_[f];
    if (fields_[f].nested()) {
      for (const NestPlan& np : nest_)
        if (np.field == (int)f) NestedBodyBuffers(np, 0, 0, nr, addrs, sizes, &bufs, &temps);
      continue;
    }
    const uint8_t* vb = reinterpret_cast<const uint8_t*>(addrs[b0]);
    bufs.push_back({vb, addrs[b0] != 0 && sizes[b0] > 0 && nr > 0 && CountZeros(vb, nr) > 0 ? BytesForBits(nr) : 0});
    if (t == GZ_TYPE_LIST) {  // offsets, then the element array (validity only with nulls)
      const int32_t* off = reinterpret_cast<const int32_t*>(addrs[b0 + 1]);
      bufs.push_back({reinterpret_cast<const uint8_t*>(off), (int64_t)(nr + 1) * 4});
      const int64_t e0 = nr > 0 && off ? off[0] : 0, e1 = nr > 0 && off ? off[nr] : 0;
      const uint8_t* ev = reinterpret_cast<const uint8_t*>(addrs[b0 + 2]);
      bool enull = false;
      if (ev && sizes[b0 + 2] > 0)
        for (int64_t e = e0; e < e1 && !enull; e++) enull = !((ev[e >> 3] >> (e & 7)) & 1);
      bufs.push_back({ev, enull ? BytesForBits(e1 - e0) : 0});
      const int w = ByteWidth(fields_[f].elem);
      if (w == 0) bufs.push_back({reinterpret_cast<const uint8_t*>(addrs[b0 + 3]) + e0 / 8, BytesForBits(e1 - e0)});
      else bufs.push_back({reinterpret_cast<const uint8_t*>(addrs[b0 + 3]) + e0 * w, (e1 - e0) * w});
      continue;
    }
    if (IsBinary(t)) {
      const int ow = OffW(t);
      const uint8_t* off = reinterpret_cast<const uint8_t*>(addrs[b0 + 1]);
      bufs.push_back({off, (int64_t)(nr + 1) * ow});
      const int64_t c0 = nr > 0 && off ? OffAt(off, ow, 0) : 0, c1 = nr > 0 && off ? OffAt(off, ow, nr) : 0;
      bufs.push_back({reinterpret_cast<const uint8_t*>(addrs[b0 + 2]) + c0, c1 - c0});
    } else {
      bufs.push_back({reinterpret_cast<const uint8_t*>(addrs[b0 + 1]),
                      t == GZ_TYPE_BOOL ? BytesForBits(nr) : (int64_t)nr * ByteWidth(t)});
    }
  }
  int64_t body = 0;
  if (codec_ == GZ_CODEC_UNCOMPRESSED || nr == 0) {
    for (auto& b : bufs) body += pad8(b.second);
    *out = body;
    return Status::OK();
  }
  // LZ4_FRAME (GetRecordBatchPayload with the codec, splitter.cc:358-369): the buffers compressed
  // by the device; each non-empty one costs its uncompressed length (8 bytes), the frame header
  // (7), a size word per block and the end mark (4)
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  int64_t total = 0;
  for (auto& b : bufs) total += (int64_t)AlignUp((size_t)b.second, 16);
  std::vector<Lz4Chunk> chunks;
  const size_t scratch = (size_t)lz4_compress_warps() * kLz4Slot;
  uint8_t* d = nullptr;
  const size_t nch = (size_t)(total / kLz4MaxBlock) + bufs.size() + 1;
  const size_t tab = AlignUp(sizeof(Lz4Chunk) * nch, 256), rb = AlignUp(sizeof(Lz4Block) * nch, 256);
  st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d), tab + rb + 256 + scratch + 2 * (size_t)total + 256, stream_),
            "cudaMallocAsync(compressed size)");
  if (!st.ok()) return st;
  uint8_t* d_in = d + tab + rb + 256 + scratch;
  uint8_t* d_arena = d_in + total;
  int64_t at = 0;
  for (auto& b : bufs) {
    if (b.second <= 0) continue;
    if (st.ok()) st = Cuda(cudaMemcpyAsync(d_in + at, b.first, (size_t)b.second, cudaMemcpyHostToDevice, stream_), "H2D");
    for (int64_t x = 0; x < b.second; x += kLz4MaxBlock)
      chunks.push_back(Lz4Chunk{d_in + at + x, (uint32_t)std::min<int64_t>(kLz4MaxBlock, b.second - x), 0u});
    at += (int64_t)AlignUp((size_t)b.second, 16);
  }
  std::vector<Lz4Block> res(chunks.size());
  int32_t err = 0;
  if (st.ok()) st = Cuda(cudaMemcpyAsync(d, chunks.data(), sizeof(Lz4Chunk) * chunks.size(), cudaMemcpyHostToDevice, stream_), "H2D");
  if (st.ok()) st = Cuda(cudaMemsetAsync(d + tab + rb, 0, 256, stream_), "memset");
  if (st.ok())
    st = Cuda(launch_lz4_compress(reinterpret_cast<Lz4Chunk*>(d), (uint32_t)chunks.size(),
                                  reinterpret_cast<uint32_t*>(d + tab + rb + 8), d + tab + rb + 256, d_arena,
                                  reinterpret_cast<unsigned long long*>(d + tab + rb), (unsigned long long)total + 256,
                                  reinterpret_cast<Lz4Block*>(d + tab), reinterpret_cast<int32_t*>(d + tab + rb + 16), stream_),
              "k_lz4_compress");
  if (st.ok()) st = Cuda(cudaMemcpyAsync(res.data(), d + tab, sizeof(Lz4Block) * res.size(), cudaMemcpyDeviceToHost, stream_), "D2H");
  if (st.ok()) st = Cuda(cudaMemcpyAsync(&err, d + tab + rb + 16, 4, cudaMemcpyDeviceToHost, stream_), "D2H");
  if (st.ok()) st = Cuda(cudaStreamSynchronize(stream_), "k_lz4_compress");
  cudaFreeAsync(d, stream_);
  if (!st.ok()) return st;
  if (err) return Status::Error(GZ_CUDA, "compression arena overflow");
  size_t k = 0;
  for (auto& b : bufs) {
    if (b.second <= 0) continue;
    int64_t len = 8 + 7 + 4;
    for (int64_t x = 0; x < b.second; x += kLz4MaxBlock) len += 4 + res[k++].size;
    body += pad8(len);
  }
  *out = body;
  return Status::OK();
}

Status Splitter::LastPids(uint16_t* out, int32_t n) {
  Status st = Drain();
  if (!st.ok()) return st;
  st = SyncAndCheck();
  if (!st.ok()) return st;
  if (flushes_.empty() || (uint32_t)n != last_batch_rows_ || d_scratch_[flushes_.back().scratch] == nullptr)
    return Status::Error(GZ_INVALID, "no batch of that size was split last (or the splitter stopped)");
  const FlushRec& f = flushes_.back();
  // the pids of the last flush sit at the start of its scratch; the last batch is at their end
  const uint16_t* pids = reinterpret_cast<const uint16_t*>(d_scratch_[f.scratch]);
  return Cuda(cudaMemcpy(out, pids + (f.n_rows - (uint32_t)n), 2 * (size_t)n, cudaMemcpyDeviceToHost),
              "D2H pids");
}

void Splitter::Stats(int64_t* o) const {
  o[0] = (int64_t)flushes_.size();
  o[1] = stat_input_bytes_;
  o[2] = stat_h2d_bytes_;
  o[3] = (int64_t)spilled_to_host_bytes_;
  o[4] = (int64_t)resident_bytes_;
  o[5] = stat_batches_;
  o[6] = stat_rows_;
  o[7] = stat_emitted_;
}

Status Splitter::Sync() {
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  st = Drain();
  if (!st.ok()) return st;
  return SyncAndCheck();
}

Status SyncGroup(const std::vector<Splitter*>& tasks, int* failed) {
  // every task's last pass is queued before any task is waited for, so their tails overlap
  for (size_t i = 0; i < tasks.size(); i++) {
    Status st = tasks[i]->Cuda(cudaSetDevice(tasks[i]->device_), "cudaSetDevice");
    if (st.ok()) st = tasks[i]->Drain();
    if (!st.ok()) {
      *failed = (int)i;
      return st;
    }
  }
  for (size_t i = 0; i < tasks.size(); i++) {
    Status st = tasks[i]->SyncAndCheck();
    if (!st.ok()) {
      *failed = (int)i;
      return st;
    }
  }
  return Status::OK();
}

Status Splitter::KernelTimes(double* out4) {
  Status st = SyncAndCheck();
  if (!st.ok()) return st;
  for (int i = 0; i < 4; i++) out4[i] = kernel_ms_[i];
  return Status::OK();
}

}  // namespace gz
