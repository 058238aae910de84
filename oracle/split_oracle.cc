/*
 * ORACLE — test infrastructure only.  A plain, row-at-a-time CPU restatement of the
 * reference Splitter (native-sql-engine/cpp/src/shuffle/splitter.{h,cc}), used by
 * tests/, the smoke check and bench.py's CPU-baseline leg to check the CUDA product.
 * It is never linked into, loaded by or called from the product library.
 *
 * What it restates (reference file:line in native-sql-engine/cpp/src/shuffle/):
 *   Init: column classification fixed-then-binary, P <= 64K, buffer_size <= 32K  splitter.cc:216-335
 *   Splitter::Make partitioners hash / rr / single / range                      splitter.cc:190-208
 *   hash chain (seed 42, Spark Murmur3, nulls pass the seed) + pmod + histogram  splitter.cc:1402-1470
 *   round-robin pid_selection_ carried across batches (single = rr over 1)      splitter.cc:1379-1387
 *   range: int32 partition ids in input field 0, which leaves the output schema splitter.cc:1486-1519
 *   DoSplit: sticky input_has_null_ quirk, per-pid prepare/emit/spill policy     splitter.cc:855-938
 *   CalculateSplitBatchSize (empirical binary sizes, offheap rule)               splitter.cc:800-853
 *   AllocatePartitionBuffers (validity iff input_has_null_, 0xff fill)           splitter.cc:610-713
 *   Split{FixedWidthValue,Validity,Binary}Buffer / SplitBoolType                 splitter.cc:939-1303
 *   CacheRecordBatch (slice, raw size, IPC payload)                              splitter.cc:438-608
 *   SpillPartition / SpillLargestPartition / SpillFixedSize                      splitter.cc:741-799
 *   nested columns (list / large_list / map / struct) through Arrow builders       splitter.cc:1322-1344
 *   Stop / WriteCachedRecordBatchAndClose / EOS                                  splitter.cc:84-172,395-437
 * Arrow IPC framing restates the Arrow C++ writer (continuation token, int32 metadata
 * length padded to 8, flatbuffer Message{RecordBatch}, 8-byte padded body; a validity
 * buffer is written only when the slice has nulls) with a small FlatBufferBuilder that
 * follows the published flatbuffers build algorithm (back-to-front, vtable dedup).
 *
 * Spilled payloads are kept in host memory ("spill files" are byte vectors); the bytes of a
 * partition do not depend on when it was spilled (splitter.cc:75-143).
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <functional>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "spark_hash.h"

namespace {

using namespace gzoracle;

// Type codes shared with include/gz_split.h (GZ_TYPE_*).
enum TypeCode {
  T_NULL = 0, T_BOOL = 1, T_INT8 = 2, T_UINT8 = 3, T_INT16 = 4, T_UINT16 = 5,
  T_HALF_FLOAT = 6, T_INT32 = 7, T_UINT32 = 8, T_FLOAT32 = 9, T_DATE32 = 10,
  T_TIME32 = 11, T_INT64 = 12, T_UINT64 = 13, T_FLOAT64 = 14, T_DATE64 = 15,
  T_TIME64 = 16, T_TIMESTAMP = 17, T_DECIMAL128 = 18, T_STRING = 19, T_BINARY = 20,
  T_LARGE_STRING = 21, T_LARGE_BINARY = 22, T_LIST = 23, T_LARGE_LIST = 24, T_STRUCT = 25,
  T_MAP = 26,
};
bool IsNested(int t) { return t == T_LIST || t == T_LARGE_LIST || t == T_STRUCT || t == T_MAP; }

int ByteWidth(int t) {
  switch (t) {
    case T_INT8: case T_UINT8: return 1;
    case T_INT16: case T_UINT16: case T_HALF_FLOAT: return 2;
    case T_INT32: case T_UINT32: case T_FLOAT32: case T_DATE32: case T_TIME32: return 4;
    case T_INT64: case T_UINT64: case T_FLOAT64: case T_DATE64: case T_TIME64:
    case T_TIMESTAMP: return 8;
    case T_DECIMAL128: return 16;
    default: return 0;
  }
}
bool IsBinary(int t) { return t == T_STRING || t == T_BINARY || t == T_LARGE_STRING || t == T_LARGE_BINARY; }
// Bytes of one offset: int32 (BinaryType / StringType) or int64 (LargeBinaryType /
// LargeStringType, SplitBinaryType<int64_t>, splitter.cc:1291-1299).
int OffW(int t) { return t == T_LARGE_STRING || t == T_LARGE_BINARY ? 8 : 4; }
int64_t OffAt(const uint8_t* off, int w, int64_t r) {
  return w == 8 ? reinterpret_cast<const int64_t*>(off)[r] : (int64_t)reinterpret_cast<const int32_t*>(off)[r];
}

int64_t BytesForBits(int64_t n) { return (n + 7) / 8; }
int64_t Pad8(int64_t n) { return (n + 7) & ~int64_t(7); }
bool GetBit(const uint8_t* b, int64_t i) { return (b[i >> 3] >> (i & 7)) & 1; }
void ClearBit(uint8_t* b, int64_t i) { b[i >> 3] &= (uint8_t)~(1u << (i & 7)); }

// ---------------------------------------------------------------------------------------
// Minimal FlatBufferBuilder: the published flatbuffers algorithm (buffer grows toward the
// front; offsets are distances from the end; tables end with a vtable that is shared when an
// identical one was written before).
class FlatBuilder {
 public:
  uint32_t Size() const { return (uint32_t)buf_.size(); }
  void Pad(size_t n) { buf_.insert(buf_.begin(), n, 0); }
  void Align(size_t a) {
    minalign_ = std::max(minalign_, a);
    Pad((~buf_.size() + 1) & (a - 1));
  }
  void PreAlign(size_t len, size_t a) {
    if (len == 0) return;
    minalign_ = std::max(minalign_, a);
    Pad((~(buf_.size() + len) + 1) & (a - 1));
  }
  template <typename T>
  uint32_t Push(T v) {
    Align(sizeof(T));
    uint8_t tmp[sizeof(T)];
    memcpy(tmp, &v, sizeof(T));
    buf_.insert(buf_.begin(), tmp, tmp + sizeof(T));
    return Size();
  }
  void PushBytes(const uint8_t* p, size_t n) { buf_.insert(buf_.begin(), p, p + n); }
  uint32_t ReferTo(uint32_t off) {
    Align(4);
    return Size() - off + 4;
  }
  // vector of 16-byte structs made of two int64 (FieldNode / Buffer)
  uint32_t StructVector16(const std::vector<std::pair<int64_t, int64_t>>& v) {
    PreAlign(v.size() * 16, 4);
    PreAlign(v.size() * 16, 8);
    std::vector<uint8_t> raw(v.size() * 16);
    for (size_t i = 0; i < v.size(); i++) {
      memcpy(&raw[i * 16], &v[i].first, 8);
      memcpy(&raw[i * 16 + 8], &v[i].second, 8);
    }
    PushBytes(raw.data(), raw.size());
    return Push<uint32_t>((uint32_t)v.size());
  }
  void StartTable() {
    fields_.clear();
    table_start_ = Size();
  }
  template <typename T>
  void AddScalar(uint16_t voff, T v, T def) {
    if (v == def) return;
    fields_.push_back({voff, Push<T>(v)});
  }
  void AddOffset(uint16_t voff, uint32_t off) {
    if (off == 0) return;
    fields_.push_back({voff, Push<uint32_t>(ReferTo(off))});
  }
  uint32_t EndTable() {
    uint32_t loc = Push<int32_t>(0);
    uint16_t maxv = 4;
    for (auto& f : fields_) maxv = std::max<uint16_t>(maxv, f.first + 2);
    std::vector<uint16_t> vt(maxv / 2, 0);
    vt[0] = maxv;
    vt[1] = (uint16_t)(loc - table_start_);
    for (auto& f : fields_) vt[f.first / 2] = (uint16_t)(loc - f.second);
    std::vector<uint8_t> vtb(maxv);
    memcpy(vtb.data(), vt.data(), maxv);
    uint32_t use = 0;
    for (uint32_t prev : vtables_) {
      const uint8_t* p = &buf_[buf_.size() - prev];
      uint16_t sz;
      memcpy(&sz, p, 2);
      if (sz == maxv && memcmp(p, vtb.data(), maxv) == 0) {
        use = prev;
        break;
      }
    }
    if (use == 0) {
      PushBytes(vtb.data(), vtb.size());
      use = Size();
      vtables_.push_back(use);
    }
    int32_t soff = (int32_t)use - (int32_t)loc;
    memcpy(&buf_[buf_.size() - loc], &soff, 4);
    return loc;
  }
  std::vector<uint8_t> Finish(uint32_t root) {
    PreAlign(4, minalign_);
    Push<uint32_t>(ReferTo(root));
    return buf_;
  }

 private:
  std::vector<uint8_t> buf_;
  size_t minalign_ = 1;
  uint32_t table_start_ = 0;
  std::vector<std::pair<uint16_t, uint32_t>> fields_;
  std::vector<uint32_t> vtables_;
};

// A body buffer of an IPC record batch; `len == 0` is an empty (placeholder) buffer.
struct BodyBuf {
  const uint8_t* data;
  int64_t len;
};

// Arrow IPC encapsulated message for one record batch (MetadataVersion V5, no codec).
std::vector<uint8_t> EncodeRecordBatch(int64_t length,
                                       const std::vector<std::pair<int64_t, int64_t>>& nodes,
                                       const std::vector<BodyBuf>& body, int64_t* body_len) {
  std::vector<std::pair<int64_t, int64_t>> bufmeta;
  int64_t off = 0;
  for (auto& b : body) {
    bufmeta.push_back({off, b.len});
    off += Pad8(b.len);
  }
  *body_len = off;
  FlatBuilder fb;
  uint32_t fnodes = fb.StructVector16(nodes);
  uint32_t fbufs = fb.StructVector16(bufmeta);
  fb.StartTable();  // RecordBatch: length(0) nodes(1) buffers(2) compression(3) variadic(4)
  fb.AddScalar<int64_t>(4, length, 0);
  fb.AddOffset(8, fbufs);
  fb.AddOffset(6, fnodes);
  uint32_t rb = fb.EndTable();
  fb.StartTable();  // Message: version(0) header_type(1) header(2) bodyLength(3) custom_metadata(4)
  fb.AddScalar<int64_t>(10, off, 0);
  fb.AddOffset(8, rb);
  fb.AddScalar<int16_t>(4, 4 /*V5*/, 0);
  fb.AddScalar<uint8_t>(6, 3 /*RecordBatch*/, 0);
  uint32_t msg = fb.EndTable();
  std::vector<uint8_t> meta = fb.Finish(msg);
  int64_t padded = Pad8(meta.size() + 8);
  std::vector<uint8_t> out;
  out.reserve(padded + off);
  uint32_t cont = 0xFFFFFFFFu;
  int32_t mlen = (int32_t)(padded - 8);
  out.insert(out.end(), (uint8_t*)&cont, (uint8_t*)&cont + 4);
  out.insert(out.end(), (uint8_t*)&mlen, (uint8_t*)&mlen + 4);
  out.insert(out.end(), meta.begin(), meta.end());
  out.resize(padded, 0);
  for (auto& b : body) {
    if (b.len > 0) out.insert(out.end(), b.data, b.data + b.len);
    out.resize(out.size() + (Pad8(b.len) - b.len), 0);
  }
  return out;
}

// A schema field; nested types carry their children: list / large_list one (the element),
// map one (the entries struct of key and value), struct its fields.
struct Field {
  int type;
  std::string name;
  std::vector<Field> kids;
};

// One input array (jni_common.h:186-300 MakeArrayData): buffers of the node, children below.
struct InNode {
  const uint8_t* validity = nullptr;  // nullptr when the validity buffer is empty
  const uint8_t* offsets = nullptr;   // binary / list / map
  const uint8_t* values = nullptr;    // fixed width, bool bits, binary characters
  int64_t null_count = 0;             // top level: counted; children: unused
  std::vector<InNode> kids;
};
using InCol = InNode;

inline void PutBit(std::vector<uint8_t>& v, int64_t i, bool b) {
  if ((int64_t)v.size() * 8 <= i) v.resize((size_t)(i / 8 + 1), 0);
  if (b) v[(size_t)(i >> 3)] |= (uint8_t)(1u << (i & 7));
}

// One partition's builder of a nested column (partition_list_builders_, splitter.cc:292-296,
// 664-674), filled by AppendArraySlice one row at a time (AppendList, splitter.cc:1335-1344)
// with the Arrow builders' semantics:
//   list / large_list / map: a null entry appends no elements, a valid one its slice;
//   struct: every child appends the same slice, null entries included;
//   binary: a null entry appends no bytes; fixed width and bool: values copied under nulls.
// A map's entries struct is all valid (its builder is sized from the keys).  Finish writes the
// nodes in pre-order with [validity, (offsets), (values)] each, a bitmap only when it holds a
// null, zero-padded like an Arrow builder's.
struct NodeBuf {
  std::vector<uint8_t> valid, data;
  std::vector<int64_t> offs{0};
  int64_t len = 0, nulls = 0, nbits = 0;
  std::vector<NodeBuf> kids;
};

void InitNode(const Field& t, NodeBuf* b) {
  *b = NodeBuf();
  b->kids.resize(t.kids.size());
  for (size_t i = 0; i < t.kids.size(); i++) InitNode(t.kids[i], &b->kids[i]);
}

void AppendValidity(NodeBuf* b, const uint8_t* validity, int64_t off, int64_t len) {
  for (int64_t i = 0; i < len; i++) {
    const bool v = validity == nullptr || GetBit(validity, off + i);
    PutBit(b->valid, b->len + i, v);
    b->nulls += !v;
  }
}

void AppendSlice(const Field& t, NodeBuf* b, const InNode& in, int64_t off, int64_t len) {
  if (t.type == T_STRUCT) {
    for (size_t k = 0; k < t.kids.size(); k++) AppendSlice(t.kids[k], &b->kids[k], in.kids[k], off, len);
    AppendValidity(b, in.validity, off, len);
    b->len += len;
    return;
  }
  if (t.type == T_LIST || t.type == T_LARGE_LIST || t.type == T_MAP) {
    const int ow = t.type == T_LARGE_LIST ? 8 : 4;
    for (int64_t r = off; r < off + len; r++) {
      const bool v = in.validity == nullptr || GetBit(in.validity, r);
      PutBit(b->valid, b->len, v);
      b->nulls += !v;
      b->len++;
      int64_t size = 0;
      if (v) {
        const int64_t o0 = OffAt(in.offsets, ow, r);
        size = OffAt(in.offsets, ow, r + 1) - o0;
        if (t.type == T_MAP) {  // MapBuilder: keys and items, the entries struct sized after them
          const Field& e = t.kids[0];
          NodeBuf& eb = b->kids[0];
          AppendSlice(e.kids[0], &eb.kids[0], in.kids[0].kids[0], o0, size);
          AppendSlice(e.kids[1], &eb.kids[1], in.kids[0].kids[1], o0, size);
          AppendValidity(&eb, nullptr, 0, size);
          eb.len += size;
        } else {
          AppendSlice(t.kids[0], &b->kids[0], in.kids[0], o0, size);
        }
      }
      b->offs.push_back(b->offs.back() + size);
    }
    return;
  }
  if (IsBinary(t.type)) {
    const int ow = OffW(t.type);
    for (int64_t r = off; r < off + len; r++) {
      const bool v = in.validity == nullptr || GetBit(in.validity, r);
      PutBit(b->valid, b->len, v);
      b->nulls += !v;
      b->len++;
      if (v) {
        const int64_t o0 = OffAt(in.offsets, ow, r), o1 = OffAt(in.offsets, ow, r + 1);
        b->data.insert(b->data.end(), in.values + o0, in.values + o1);
      }
      b->offs.push_back((int64_t)b->data.size());
    }
    return;
  }
  AppendValidity(b, in.validity, off, len);
  if (t.type == T_BOOL) {
    for (int64_t i = 0; i < len; i++) PutBit(b->data, b->nbits++, GetBit(in.values, off + i));
  } else {
    const int w = ByteWidth(t.type);
    b->data.insert(b->data.end(), in.values + off * w, in.values + (off + len) * w);
  }
  b->len += len;
}

// Builder Finish: nodes and body buffers in pre-order; `keep` holds the assembled buffers.
void FinishNode(const Field& t, NodeBuf* b, std::vector<std::pair<int64_t, int64_t>>* nodes,
                std::vector<std::pair<const uint8_t*, int64_t>>* body, std::vector<std::vector<uint8_t>>* keep) {
  const int64_t n = b->len;
  b->valid.resize((size_t)BytesForBits(n), 0);
  nodes->push_back({n, b->nulls});
  body->push_back(b->nulls > 0 ? std::make_pair((const uint8_t*)b->valid.data(), BytesForBits(n))
                               : std::make_pair((const uint8_t*)nullptr, (int64_t)0));
  const bool offs = t.type == T_LIST || t.type == T_LARGE_LIST || t.type == T_MAP || IsBinary(t.type);
  if (offs) {
    const int ow = t.type == T_LARGE_LIST || t.type == T_LARGE_STRING || t.type == T_LARGE_BINARY ? 8 : 4;
    keep->emplace_back((size_t)(n + 1) * ow);
    uint8_t* o = keep->back().data();
    for (int64_t i = 0; i <= n; i++) {
      if (ow == 8) {
        memcpy(o + i * 8, &b->offs[i], 8);
      } else {
        const int32_t v = (int32_t)b->offs[i];
        memcpy(o + i * 4, &v, 4);
      }
    }
    body->push_back({o, (int64_t)(n + 1) * ow});
  }
  if (IsBinary(t.type) || ByteWidth(t.type) > 0) {
    body->push_back({b->data.data(), (int64_t)b->data.size()});
  } else if (t.type == T_BOOL) {
    b->data.resize((size_t)BytesForBits(n), 0);
    body->push_back({b->data.data(), BytesForBits(n)});
  }
  for (size_t k = 0; k < t.kids.size(); k++) FinishNode(t.kids[k], &b->kids[k], nodes, body, keep);
}

// batch_nbytes (splitter.cc:438-453): the top-level array's own buffers only.
int64_t OwnBytes(const Field& t, const NodeBuf& b) {
  const int64_t n = b.len;
  int64_t r = b.nulls > 0 ? BytesForBits(n) : 0;
  if (t.type == T_LIST || t.type == T_MAP) r += (n + 1) * 4;
  if (t.type == T_LARGE_LIST) r += (n + 1) * 8;
  return r;
}

// Types a nested column may hold (anything but null below the top).
bool NestedSupported(const Field& t) {
  if (t.type == T_NULL) return false;
  if (t.type == T_MAP && (t.kids.size() != 1 || t.kids[0].type != T_STRUCT || t.kids[0].kids.size() != 2))
    return false;
  if ((t.type == T_LIST || t.type == T_LARGE_LIST) && t.kids.size() != 1) return false;
  if (t.type == T_STRUCT && t.kids.empty()) return false;
  if (!IsNested(t.type) && !t.kids.empty()) return false;
  if (!IsNested(t.type) && !IsBinary(t.type) && t.type != T_BOOL && ByteWidth(t.type) == 0) return false;
  for (const Field& k : t.kids)
    if (!NestedSupported(k)) return false;
  return true;
}

// MakeArrayData (jni_common.h:186-300): one array from the flat buffer list at *idx.
std::string ParseNode(const Field& t, const int64_t* addrs, const int64_t* sizes, int nbuf, int* idx,
                      InNode* out) {
  auto take = [&](bool* empty) -> const uint8_t* {
    const int i = (*idx)++;
    *empty = sizes[i] == 0 || addrs[i] == 0;
    return (const uint8_t*)addrs[i];
  };
  bool empty;
  if (*idx >= nbuf) return "insufficient number of buffers";
  const uint8_t* v = take(&empty);
  out->validity = empty ? nullptr : v;
  if (t.type == T_LIST || t.type == T_LARGE_LIST || t.type == T_MAP || IsBinary(t.type)) {
    if (*idx >= nbuf) return "insufficient number of buffers";
    out->offsets = take(&empty);
  }
  if (t.type == T_STRUCT || t.type == T_LIST || t.type == T_LARGE_LIST || t.type == T_MAP) {
    out->kids.resize(t.kids.size());
    for (size_t k = 0; k < t.kids.size(); k++) {
      std::string e = ParseNode(t.kids[k], addrs, sizes, nbuf, idx, &out->kids[k]);
      if (!e.empty()) return e;
    }
    // the map's entries struct: its validity is dropped (jni_common.h:284-288)
    if (t.type == T_MAP) out->kids[0].validity = nullptr;
    return "";
  }
  if (*idx >= nbuf) return "insufficient number of buffers";
  out->values = take(&empty);
  return "";
}

// Splitter::Make short names (splitter.cc:190-208); "single" is round-robin over one partition.
enum Mode { M_HASH = 0, M_RR = 1, M_RANGE = 2 };

struct Options {
  int mode = M_HASH;
  int64_t offheap_per_task = 0;
  int32_t buffer_size = 4096;
  int32_t batch_compress_threshold = 256;
  bool prefer_spill = true;
  bool write_schema = false;
};

// Per (array column, partition) buffers, mirroring partition_buffers_ (splitter.h:242-244).
struct PartBufs {
  bool has_validity = false;
  std::vector<uint8_t> validity;  // capacity bytes, 0xff filled
  std::vector<uint8_t> values;    // fixed: cap * width; bool: bitmap
  std::vector<int64_t> offsets;   // binary: cap + 1 (written out at the column's offset width)
  std::vector<uint8_t> chars;     // binary values (grows)
  int64_t chars_used = 0;
};

class OracleSplitter {
 public:
  OracleSplitter(std::vector<Field> fields, int P, std::vector<int> keys, Options o)
      : fields_(std::move(fields)), P_(P), keys_(std::move(keys)), opt_(o) {}

  std::string Init() {
    if (opt_.mode == M_RANGE) {
      // FallbackRangeSplitter::Init: the output schema is the input schema without field 0
      // (splitter.cc:1486-1490); field 0 holds the partition ids
      if (fields_.empty()) return "range partitioning needs a partition id field";
      in_type0_ = fields_[0].type;
      fields_.erase(fields_.begin());
    }
    if (opt_.mode != M_HASH) keys_.clear();  // rr / range take no key expressions
    if (P_ <= 0 || P_ > 65536) return "num_partitions must be in [1, 65536]";
    if (opt_.buffer_size > 32768) return "buffer_size must be <= 32768";
    std::vector<int> bin;
    for (int i = 0; i < (int)fields_.size(); i++) {
      int t = fields_[i].type;
      if (IsBinary(t)) bin.push_back(i);
      else if (t == T_NULL) continue;
      else if (IsNested(t)) {  // list_array_idx_ (splitter.cc:254-258)
        if (!NestedSupported(fields_[i])) return "nested type not supported";
        list_idx_.push_back(i);
      }
      else if (t == T_BOOL || ByteWidth(t) > 0) array_idx_.push_back(i);
      else return "unsupported field type";
    }
    fixed_cnt_ = (int)array_idx_.size();
    array_idx_.insert(array_idx_.end(), bin.begin(), bin.end());
    for (int k : keys_) {
      if (k < 0 || k >= (int)fields_.size()) return "key column out of range";
      int t = fields_[k].type;
      // a null-type key adds nothing to the chain (CreateProjector's NullType case,
      // splitter.cc:1407-1408)
      if (!(t == T_NULL || t == T_BOOL || t == T_INT8 || t == T_INT16 || t == T_INT32 || t == T_DATE32 ||
            t == T_FLOAT32 || t == T_INT64 || t == T_FLOAT64 || t == T_STRING))
        return "key type has no Spark hash";
    }
    int A = (int)array_idx_.size();
    bufs_.assign(A, std::vector<PartBufs>(P_));
    lists_.assign(list_idx_.size(), std::vector<NodeBuf>(P_));
    for (size_t li = 0; li < list_idx_.size(); li++)
      for (int p = 0; p < P_; p++) InitNode(fields_[list_idx_[li]], &lists_[li][p]);
    input_has_null_.assign(A, false);
    empirical_.assign(A - fixed_cnt_, 0);
    cap_.assign(P_, 0);
    base_.assign(P_, 0);
    cached_.assign(P_, {});
    cached_size_.assign(P_, 0);
    spilled_.assign(P_, {});
    writer_.assign(P_, false);
    spill_opened_.assign(P_, false);
    partition_lengths_.assign(P_, 0);
    raw_lengths_.assign(P_, 0);
    return "";
  }

  // buffers: flat list in schema order [validity, (offsets), values] per field; a null-type
  // field takes two ignored buffers (jni_common.h:308-343 generic branch)
  std::string Split(int32_t n, const int64_t* addrs, const int64_t* sizes, int nbuf) {
    std::vector<InCol> cols(fields_.size());
    int idx = 0;
    range_pids_ = nullptr;
    if (opt_.mode == M_RANGE) {
      // FallbackRangeSplitter::ComputeAndCountPartitionId (splitter.cc:1499-1519): field 0 must
      // be int32; its values (validity ignored) are the partition ids
      const int nb0 = IsBinary(in_type0_) ? 3 : 2;
      if (nbuf < nb0) return "insufficient number of buffers";
      if (in_type0_ != T_INT32) return "RecordBatch field 0 should be int32";
      range_pids_ = (const int32_t*)addrs[1];
      addrs += nb0;
      sizes += nb0;
      nbuf -= nb0;
    }
    for (size_t f = 0; f < fields_.size(); f++) {
      if (fields_[f].type == T_NULL) {
        if (idx + 2 > nbuf) return "insufficient number of buffers";
        idx += 2;
        continue;
      }
      InCol c;
      std::string pe = ParseNode(fields_[f], addrs, sizes, nbuf, &idx, &c);
      if (!pe.empty()) return pe;
      if (c.validity) {
        int64_t valid = 0;
        for (int64_t i = 0; i < n; i++) valid += GetBit(c.validity, i);
        c.null_count = n - valid;
      }
      cols[f] = c;
    }
    auto t0 = std::chrono::steady_clock::now();
    std::string e = ComputePid(n, cols);
    if (!e.empty()) return e;
    compute_pid_ns_ += std::chrono::duration_cast<std::chrono::nanoseconds>(
                           std::chrono::steady_clock::now() - t0).count();
    return DoSplit(n, cols);
  }

  // SpillFixedSize (splitter.cc:741-756)
  int64_t SpillFixedSize(int64_t size) {
    int64_t cur = 0;
    int tries = 0;
    while (cur < size && tries < 5) {
      tries++;
      int64_t got;
      if (SpillLargest(&got) < 0) break;
      cur += got;
    }
    return cur;
  }

  // The encapsulated IPC Schema message GetSchemaPayload + WriteIpcPayload give for the schema
  // (splitter.cc:145-151, 1355-1364); the caller serialises it with Arrow itself.
  void SetSchemaMessage(const uint8_t* p, size_t n) {
    opt_.write_schema = true;
    schema_msg_.assign(p, p + n);
  }

  // With a data file, each partition is written as soon as it is assembled, as the reference's
  // partition writers append to the data file (WriteCachedRecordBatchAndClose, splitter.cc:84-109);
  // without one the bytes are kept in *file_bytes.
  std::string Stop(const char* data_file, std::vector<uint8_t>* file_bytes) {
    std::vector<uint8_t> out;
    FILE* f = nullptr;
    if (data_file && data_file[0]) {
      f = fopen(data_file, "wb");
      if (!f) return std::string("cannot open data file ") + data_file;
    }
    for (int p = 0; p < P_; p++) {
      CacheRecordBatch(p, true);
      if (cached_size_[p] > 0) writer_[p] = true;
      if (writer_[p]) {
        if (f) out.clear();
        size_t before = out.size();
        // WriteSchemaPayload before the partition's batches when write_schema (splitter.cc:88-90)
        if (opt_.write_schema) out.insert(out.end(), schema_msg_.begin(), schema_msg_.end());
        if (!spill_opened_[p] && cached_size_[p] == 0) return "Partition writer got empty partition";
        if (spill_opened_[p]) {
          out.insert(out.end(), spilled_[p].begin(), spilled_[p].end());
          bytes_spilled_ += (int64_t)spilled_[p].size();
          std::vector<uint8_t>().swap(spilled_[p]);
        }
        for (auto& m : cached_[p]) out.insert(out.end(), m.begin(), m.end());
        cached_[p].clear();
        cached_size_[p] = 0;
        uint32_t eos[2] = {0xFFFFFFFFu, 0};
        out.insert(out.end(), (uint8_t*)eos, (uint8_t*)eos + 8);
        partition_lengths_[p] = (int64_t)(out.size() - before);
        bytes_written_ += partition_lengths_[p];
        if (f && fwrite(out.data(), 1, out.size(), f) != out.size()) {
          fclose(f);
          return "short write";
        }
      } else {
        partition_lengths_[p] = 0;
      }
    }
    if (f) {
      if (fclose(f) != 0) return "closing the data file failed";
      out.clear();
    }
    if (file_bytes) *file_bytes = std::move(out);
    return "";
  }

  const std::vector<int64_t>& partition_lengths() const { return partition_lengths_; }
  const std::vector<int64_t>& raw_lengths() const { return raw_lengths_; }
  int64_t bytes_written() const { return bytes_written_; }
  int64_t bytes_spilled() const { return bytes_spilled_; }
  int64_t compute_pid_ns() const { return compute_pid_ns_; }
  const std::vector<uint16_t>& last_pids() const { return pid_; }

 private:
  // ComputeAndCountPartitionId of the three partitioners
  std::string ComputePid(int32_t n, const std::vector<InCol>& cols) {
    pid_.assign(n, 0);
    cnt_.assign(P_, 0);
    if (opt_.mode == M_RR) {
      // RoundRobinSplitter (splitter.cc:1379-1387): the selection wraps at P and carries over
      // to the next batch
      for (int32_t r = 0; r < n; r++) {
        pid_[r] = (uint16_t)rr_sel_;
        cnt_[rr_sel_]++;
        rr_sel_ = rr_sel_ + 1 == P_ ? 0 : rr_sel_ + 1;
      }
      return "";
    }
    if (opt_.mode == M_RANGE) {
      // FallbackRangeSplitter (splitter.cc:1508-1516).  An id >= P fails the batch; a negative
      // id (undefined in the reference, which indexes its counters with it) fails it too
      for (int32_t r = 0; r < n; r++) {
        const int32_t p = range_pids_[r];
        if (p >= P_) return "Partition id " + std::to_string(p) + " is equal or greater than " + std::to_string(P_);
        if (p < 0) return "Partition id " + std::to_string(p) + " is negative";
        pid_[r] = (uint16_t)p;
        cnt_[p]++;
      }
      return "";
    }
    // HashSplitter::ComputeAndCountPartitionId (splitter.cc:1440-1470)
    for (int32_t r = 0; r < n; r++) {
      int32_t h = 42;
      for (int k : keys_) {
        if (fields_[k].type == T_NULL) continue;  // no hash function (splitter.cc:1407-1408)
        const InCol& c = cols[k];
        if (c.validity && !GetBit(c.validity, r)) continue;  // null: seed passes through
        switch (fields_[k].type) {
          case T_BOOL: h = spark_hash_int(GetBit(c.values, r) ? 1 : 0, h); break;
          case T_INT8: h = spark_hash_int(((const int8_t*)c.values)[r], h); break;
          case T_INT16: h = spark_hash_int(((const int16_t*)c.values)[r], h); break;
          case T_INT32: case T_DATE32: case T_FLOAT32:
            h = spark_hash_int(((const int32_t*)c.values)[r], h);
            break;
          case T_INT64: case T_FLOAT64:
            h = spark_hash_long(((const int64_t*)c.values)[r], h);
            break;
          case T_STRING: {
            const int32_t* off = (const int32_t*)c.offsets;
            h = SparkHashBytes(c.values + off[r], off[r + 1] - off[r], h);
            break;
          }
        }
      }
      int32_t p = spark_pmod(h, P_);
      pid_[r] = (uint16_t)p;
      cnt_[p]++;
    }
    return "";
  }

  static int32_t SparkHashBytes(const uint8_t* p, int32_t len, int32_t seed) {
    uint32_t h1 = (uint32_t)seed;
    int32_t aligned = len - len % 4;
    for (int32_t i = 0; i < aligned; i += 4) {
      uint32_t k;
      memcpy(&k, p + i, 4);
      h1 = mix_h1(h1, mix_k1(k));
    }
    for (int32_t i = aligned; i < len; i++) h1 = mix_h1(h1, mix_k1((uint32_t)(int32_t)(int8_t)p[i]));
    return (int32_t)fmix32(h1, (uint32_t)len);
  }

  // CalculateSplitBatchSize (splitter.cc:800-853)
  uint32_t SplitBatchSize(int32_t n, const std::vector<InCol>& cols) {
    int A = (int)array_idx_.size();
    for (int a = fixed_cnt_; a < A; a++) {
      uint64_t& e = empirical_[a - fixed_cnt_];
      if (e == 0) {
        const InCol& c = cols[array_idx_[a]];
        if (c.offsets) {
          const int w = OffW(fields_[array_idx_[a]].type);
          const uint64_t len = w == 8 ? (uint64_t)(OffAt(c.offsets, 8, n) - OffAt(c.offsets, 8, 0))
                                      : (uint64_t)(uint32_t)(int32_t)(OffAt(c.offsets, 4, n) - OffAt(c.offsets, 4, 0));
          e = len % n == 0 ? len / n : len / n + 1;
        }
      }
    }
    uint32_t size_per_row = 0;
    for (auto e : empirical_) size_per_row += (uint32_t)e;
    for (int a = 0; a < A; a++) {
      int ci = array_idx_[a];
      if (ci < fixed_cnt_) {
        int t = fields_[ci].type;
        size_per_row += t == T_BOOL ? 0 : ByteWidth(t);
      }
    }
    int64_t rows = opt_.offheap_per_task > 0 && size_per_row > 0
                       ? (opt_.offheap_per_task / size_per_row / P_) >> 2
                       : opt_.buffer_size;
    rows = std::min<int64_t>(rows, opt_.buffer_size);
    return (uint32_t)rows;
  }

  // AllocatePartitionBuffers (splitter.cc:610-713); capacities are logical.
  void Allocate(int p, uint32_t new_size) {
    int A = (int)array_idx_.size();
    for (int a = 0; a < A; a++) {
      PartBufs& b = bufs_[a][p];
      int t = fields_[array_idx_[a]].type;
      b = PartBufs();
      if (IsBinary(t)) {
        b.offsets.assign(new_size + 1, 0);
      } else if (t == T_BOOL) {
        b.values.assign(BytesForBits(new_size), 0xff);
      } else {
        b.values.assign((size_t)new_size * ByteWidth(t), 0);
      }
      if (input_has_null_[a]) {
        b.has_validity = true;
        b.validity.assign(BytesForBits(new_size), 0xff);
      }
    }
    cap_[p] = new_size;
  }

  // CacheRecordBatch (splitter.cc:462-608)
  void CacheRecordBatch(int p, bool reset) {
    uint32_t n = base_[p];
    if (n == 0) return;
    std::vector<std::pair<int64_t, int64_t>> nodes;
    std::vector<BodyBuf> body;
    std::vector<std::vector<uint8_t>> keep;
    int64_t raw = 0;
    int fixed_i = 0, bin_i = 0, list_i = 0;
    for (size_t f = 0; f < fields_.size(); f++) {
      int t = fields_[f].type;
      if (t == T_NULL) {
        nodes.push_back({n, n});
        continue;
      }
      if (IsNested(t)) {  // builder->Finish (splitter.cc:532-545)
        NodeBuf& b = lists_[list_i++][p];
        std::vector<std::pair<const uint8_t*, int64_t>> bb;
        FinishNode(fields_[f], &b, &nodes, &bb, &keep);
        for (auto& x : bb) body.push_back(BodyBuf{x.first, x.second});
        raw += OwnBytes(fields_[f], b);  // batch_nbytes: the column's own buffers
        continue;
      }
      int a = IsBinary(t) ? fixed_cnt_ + bin_i++ : fixed_i++;
      PartBufs& b = bufs_[a][p];
      int64_t nulls = 0;
      if (b.has_validity) {
        for (uint32_t i = 0; i < n; i++) nulls += !GetBit(b.validity.data(), i);
        raw += BytesForBits(n);
      }
      nodes.push_back({n, nulls});
      body.push_back(nulls > 0 ? BodyBuf{b.validity.data(), BytesForBits(n)} : BodyBuf{nullptr, 0});
      if (IsBinary(t)) {
        int64_t vlen = b.offsets[n];
        const int w = OffW(t);
        keep.emplace_back((size_t)(n + 1) * w);
        uint8_t* ob = keep.back().data();
        for (uint32_t i = 0; i <= n; i++) {
          if (w == 8) {
            memcpy(ob + (size_t)i * 8, &b.offsets[i], 8);
          } else {
            const int32_t o = (int32_t)b.offsets[i];
            memcpy(ob + (size_t)i * 4, &o, 4);
          }
        }
        body.push_back({ob, (int64_t)(n + 1) * w});
        body.push_back({b.chars.data(), vlen});
        raw += (int64_t)(n + 1) * w + vlen;
      } else {
        int64_t vlen = t == T_BOOL ? BytesForBits(n) : (int64_t)n * ByteWidth(t);
        body.push_back({b.values.data(), vlen});
        raw += vlen;
      }
    }
    int64_t body_len;
    auto msg = EncodeRecordBatch(n, nodes, body, &body_len);
    raw_lengths_[p] += raw;
    cached_size_[p] += body_len;
    cached_[p].push_back(std::move(msg));
    base_[p] = 0;
    for (size_t li = 0; li < list_idx_.size(); li++) InitNode(fields_[list_idx_[li]], &lists_[li][p]);
    int A = (int)array_idx_.size();
    for (int a = 0; a < A; a++) {
      PartBufs& b = bufs_[a][p];
      if (reset) {
        b = PartBufs();
      } else if (IsBinary(fields_[array_idx_[a]].type)) {
        b.chars_used = 0;
      }
    }
  }

  // SpillPartition (splitter.cc:758-776): payloads to the partition's spill bytes, then
  // every present validity buffer of the partition is refilled with 0xff.
  void SpillPartition(int p) {
    writer_[p] = true;
    spill_opened_[p] = true;
    for (auto& m : cached_[p]) spilled_[p].insert(spilled_[p].end(), m.begin(), m.end());
    cached_[p].clear();
    cached_size_[p] = 0;
    for (auto& col : bufs_) {
      if (col[p].has_validity) std::fill(col[p].validity.begin(), col[p].validity.end(), 0xff);
    }
  }

  int SpillLargest(int64_t* size) {
    int64_t max_size = 0;
    int pick = -1;
    for (int p = 0; p < P_; p++) {
      if (cached_size_[p] > max_size) {
        max_size = cached_size_[p];
        pick = p;
      }
    }
    *size = 0;
    if (pick >= 0) {
      SpillPartition(pick);
      *size = max_size;
    }
    return pick;
  }

  // DoSplit (splitter.cc:855-938)
  std::string DoSplit(int32_t n, const std::vector<InCol>& cols) {
    int A = (int)array_idx_.size();
    for (int a = 0; a < A; a++) {
      int ci = array_idx_[a];
      if (ci < fixed_cnt_ && !input_has_null_[a] && cols[ci].null_count != 0)
        input_has_null_[a] = true;
    }
    for (int p = 0; p < P_; p++) {
      uint32_t c = cnt_[p];
      if (c == 0) continue;
      if (cap_[p] == 0) {
        Allocate(p, std::max(SplitBatchSize(n, cols), c));
      } else if (base_[p] + c > cap_[p]) {
        uint32_t ns = std::max(SplitBatchSize(n, cols), c);
        if (opt_.prefer_spill) {
          if (ns > cap_[p]) {
            CacheRecordBatch(p, true);
            SpillPartition(p);
            Allocate(p, ns);
          } else {
            CacheRecordBatch(p, false);
            SpillPartition(p);
          }
        } else {
          CacheRecordBatch(p, true);
          Allocate(p, ns);
        }
      }
    }
    // stable scatter: rows in input order land at base + running rank
    std::vector<uint32_t> pos(base_.begin(), base_.end());
    std::vector<uint32_t> run(P_, 0);
    for (int a = 0; a < A; a++) {
      int ci = array_idx_[a];
      int t = fields_[ci].type;
      const InCol& c = cols[ci];
      // lazy validity (SplitValidityBuffer, splitter.cc:1179-1207)
      if (c.null_count > 0) {
        for (int p = 0; p < P_; p++) {
          if (cnt_[p] > 0 && !bufs_[a][p].has_validity) {
            bufs_[a][p].has_validity = true;
            uint32_t bits = std::max<uint32_t>(cnt_[p], (uint32_t)opt_.buffer_size);
            bufs_[a][p].validity.assign(BytesForBits(std::max<uint32_t>(bits, cap_[p])), 0xff);
          }
        }
      }
      std::fill(run.begin(), run.end(), 0);
      for (int32_t r = 0; r < n; r++) {
        int p = pid_[r];
        uint32_t d = pos[p] + run[p]++;
        PartBufs& b = bufs_[a][p];
        if (c.null_count > 0 && !GetBit(c.validity, r)) ClearBit(b.validity.data(), d);
        if (IsBinary(t)) {
          const int w = OffW(t);
          const int64_t o0 = OffAt(c.offsets, w, r);
          const int64_t len = OffAt(c.offsets, w, r + 1) - o0;
          if ((int64_t)b.chars.size() < b.chars_used + len)
            b.chars.resize(std::max<int64_t>(b.chars_used + len, b.chars.size() * 3 / 2 + 64));
          memcpy(b.chars.data() + b.chars_used, c.values + o0, len);
          b.chars_used += len;
          b.offsets[d + 1] = w == 8 ? b.chars_used : (int64_t)(int32_t)b.chars_used;
        } else if (t == T_BOOL) {
          if (!GetBit(c.values, r)) ClearBit(b.values.data(), d);
          else b.values[d >> 3] |= (uint8_t)(1u << (d & 7));
        } else {
          int w = ByteWidth(t);
          memcpy(b.values.data() + (size_t)d * w, c.values + (size_t)r * w, w);
        }
      }
      if (t == T_BOOL) {
        // SplitBoolType writes the last touched byte as 0xff & bits (splitter.cc:1162-1173):
        // bits above a partition's last row in that byte are 1.
        for (int p = 0; p < P_; p++) {
          if (cnt_[p] == 0) continue;
          uint32_t end = pos[p] + cnt_[p];
          for (uint32_t d = end; d & 7; d++) bufs_[a][p].values[d >> 3] |= (uint8_t)(1u << (d & 7));
        }
      }
    }
    // SplitListArray (splitter.cc:1322-1333): every row to its partition's builder
    for (size_t li = 0; li < list_idx_.size(); li++) {
      const InCol& c = cols[list_idx_[li]];
      const Field& t = fields_[list_idx_[li]];
      for (int32_t r = 0; r < n; r++) AppendSlice(t, &lists_[li][pid_[r]], c, r, 1);
    }
    for (int p = 0; p < P_; p++) base_[p] += cnt_[p];
    return "";
  }

  std::vector<Field> fields_;
  int P_;
  std::vector<int> keys_;
  Options opt_;
  std::vector<uint8_t> schema_msg_;
  std::vector<int> array_idx_;
  std::vector<int> list_idx_;
  std::vector<std::vector<NodeBuf>> lists_;  // [nested column][partition]
  int fixed_cnt_ = 0;
  std::vector<std::vector<PartBufs>> bufs_;
  std::vector<bool> input_has_null_;
  std::vector<uint64_t> empirical_;
  std::vector<uint32_t> cap_, base_;
  std::vector<std::vector<std::vector<uint8_t>>> cached_;
  std::vector<int64_t> cached_size_;
  std::vector<std::vector<uint8_t>> spilled_;
  std::vector<bool> writer_, spill_opened_;
  std::vector<int64_t> partition_lengths_, raw_lengths_;
  std::vector<uint16_t> pid_;
  int32_t rr_sel_ = 0;                   // RoundRobinSplitter::pid_selection_
  int in_type0_ = T_NULL;                // range: type of input field 0
  const int32_t* range_pids_ = nullptr;  // range: partition ids of the batch being split
  std::vector<uint32_t> cnt_;
  int64_t bytes_written_ = 0, bytes_spilled_ = 0, compute_pid_ns_ = 0;
};

}  // namespace

extern "C" void gzo_set_schema_message(void* hp, const uint8_t* msg, int64_t len);

namespace {

struct Handle {
  std::unique_ptr<OracleSplitter> s;
  std::string err;
  std::vector<uint8_t> file;
};

}  // namespace

extern "C" {

/* mode: "hash", "rr", "single" or "range" (Splitter::Make); fields: types[nf] (GZ_TYPE_*
 * codes, the input schema); keys: column indices (hash only); opts: see Options. */
void* gzo_make(const char* mode, const int32_t* types, int32_t nf, int32_t num_partitions,
               const int32_t* keys, int32_t n_keys, int64_t offheap_per_task, int32_t buffer_size,
               int32_t prefer_spill, char* err, int errlen) {
  // types: the fields in pre-order, each code with its child count above the low byte
  std::vector<Field> fields;
  int at = 0;
  std::function<Field(std::string)> node = [&](std::string name) {
    Field f{types[at] & 0xff, std::move(name), {}};
    const int nk = (types[at++] >> 8) & 0xff;
    for (int k = 0; k < nk; k++) f.kids.push_back(node("c" + std::to_string(k)));
    return f;
  };
  for (int i = 0; i < nf; i++) fields.push_back(node("f" + std::to_string(i)));
  Options o;
  const std::string m = mode ? mode : "hash";
  if (m == "hash") o.mode = M_HASH;
  else if (m == "rr") o.mode = M_RR;
  else if (m == "single") o.mode = M_RR, num_partitions = 1;
  else if (m == "range") o.mode = M_RANGE;
  else {
    if (err) snprintf(err, errlen, "Partitioning %s not supported yet.", m.c_str());
    return nullptr;
  }
  o.offheap_per_task = offheap_per_task;
  if (buffer_size > 0) o.buffer_size = buffer_size;
  o.prefer_spill = prefer_spill != 0;
  auto h = new Handle;
  h->s.reset(new OracleSplitter(fields, num_partitions, std::vector<int>(keys, keys + n_keys), o));
  std::string e = h->s->Init();
  if (!e.empty()) {
    if (err) snprintf(err, errlen, "%s", e.c_str());
    delete h;
    return nullptr;
  }
  return h;
}

void gzo_set_schema_message(void* hp, const uint8_t* msg, int64_t len) {
  ((Handle*)hp)->s->SetSchemaMessage(msg, (size_t)len);
}

int gzo_split(void* hp, int32_t num_rows, const int64_t* addrs, const int64_t* sizes,
              int32_t n, char* err, int errlen) {
  auto* h = (Handle*)hp;
  std::string e = h->s->Split(num_rows, addrs, sizes, n);
  if (!e.empty()) {
    if (err) snprintf(err, errlen, "%s", e.c_str());
    return 1;
  }
  return 0;
}

/* partition ids of the last Split call (uint16 per row) */
void gzo_last_pids(void* hp, uint16_t* out) {
  auto* h = (Handle*)hp;
  auto& v = h->s->last_pids();
  memcpy(out, v.data(), v.size() * 2);
}

int64_t gzo_spill(void* hp, int64_t size) { return ((Handle*)hp)->s->SpillFixedSize(size); }

/* metrics: [bytes_written, bytes_spilled, compute_pid_ns]; returns data size or -1 */
int64_t gzo_stop(void* hp, const char* data_file, int64_t* lengths, int64_t* raw_lengths,
                 int64_t* metrics, char* err, int errlen) {
  auto* h = (Handle*)hp;
  std::string e = h->s->Stop(data_file, &h->file);
  if (!e.empty()) {
    if (err) snprintf(err, errlen, "%s", e.c_str());
    return -1;
  }
  auto& pl = h->s->partition_lengths();
  auto& rl = h->s->raw_lengths();
  for (size_t i = 0; i < pl.size(); i++) {
    lengths[i] = pl[i];
    raw_lengths[i] = rl[i];
  }
  metrics[0] = h->s->bytes_written();
  metrics[1] = h->s->bytes_spilled();
  metrics[2] = h->s->compute_pid_ns();
  return (int64_t)h->file.size();
}

/* copies the data-file bytes produced by the last gzo_stop */
void gzo_file_bytes(void* hp, uint8_t* out) {
  auto* h = (Handle*)hp;
  memcpy(out, h->file.data(), h->file.size());
}

void gzo_close(void* hp) { delete (Handle*)hp; }

/* hash pins */
int32_t gzo_hash_int(int32_t v, int32_t seed) { return spark_hash_int(v, seed); }
int32_t gzo_hash_long(int64_t v, int32_t seed) { return spark_hash_long(v, seed); }
uint32_t gzo_murmur3_bytes(const uint8_t* p, int32_t len, uint32_t seed) {
  return murmur3_x86_32(p, len, seed);
}
int32_t gzo_pmod(int32_t h, int32_t p) { return spark_pmod(h, p); }

}  // extern "C"
