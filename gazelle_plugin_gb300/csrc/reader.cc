// Reduce-side read on the GPU (see reader.h).
#include "reader.h"

#include <string.h>

#include <algorithm>
#include <functional>

#include "flatbuf.h"
#include "gz_kernels.h"
#include "host_util.h"
#include "lz4_kernels.h"
#include "read_kernels.h"

namespace gz {

namespace {

inline int64_t Pad8(int64_t n) { return (n + 7) & ~int64_t(7); }
inline size_t AlignUp(size_t x, size_t a) { return (x + a - 1) / a * a; }

bool IsLargeBinaryType(int t) { return t == GZ_TYPE_LARGE_STRING || t == GZ_TYPE_LARGE_BINARY; }
bool IsBinaryType(int t) { return t == GZ_TYPE_STRING || t == GZ_TYPE_BINARY || IsLargeBinaryType(t); }
int OffsetWidth(int t) { return IsLargeBinaryType(t) ? 8 : 4; }
// Types whose batches carry int32 / int64 offsets: binary ones and lists (int32 element offsets)
bool HasOffsets(int t) { return IsBinaryType(t) || t == GZ_TYPE_LIST; }
// Offset r of a little-endian offsets buffer of width w
int64_t ReadOffset(const uint8_t* p, int w, int64_t r) {
  if (w == 8) {
    int64_t v;
    memcpy(&v, p + 8 * r, 8);
    return v;
  }
  int32_t v;
  memcpy(&v, p + 4 * r, 4);
  return v;
}

int FixedWidth(int t) {
  switch (t) {
    case GZ_TYPE_INT8: case GZ_TYPE_UINT8: return 1;
    case GZ_TYPE_INT16: case GZ_TYPE_UINT16: case GZ_TYPE_HALF_FLOAT: return 2;
    case GZ_TYPE_INT32: case GZ_TYPE_UINT32: case GZ_TYPE_FLOAT32: case GZ_TYPE_DATE32:
    case GZ_TYPE_TIME32: return 4;
    case GZ_TYPE_INT64: case GZ_TYPE_UINT64: case GZ_TYPE_FLOAT64: case GZ_TYPE_DATE64:
    case GZ_TYPE_TIME64: case GZ_TYPE_TIMESTAMP: return 8;
    case GZ_TYPE_DECIMAL128: return 16;
    default: return 0;
  }
}

bool ListLikeType(int t) { return t == GZ_TYPE_LIST || t == GZ_TYPE_LARGE_LIST || t == GZ_TYPE_MAP; }
bool NestedField(const Field& f) {
  return f.nested() || f.type == GZ_TYPE_LARGE_LIST || f.type == GZ_TYPE_STRUCT || f.type == GZ_TYPE_MAP;
}
// offset bytes of a node with offsets
int NodeOffsetWidth(int t) { return t == GZ_TYPE_LARGE_LIST || IsLargeBinaryType(t) ? 8 : 4; }
// the body buffers of one node: [validity] + offsets (list / map / binary) + values (leaves)
int NodeBuffers(int t) { return t == GZ_TYPE_STRUCT ? 1 : ListLikeType(t) ? 2 : IsBinaryType(t) ? 3 : 2; }

// Arrow IPC metadata (Message.fbs / Schema.fbs): Message {version, header_type, header,
// bodyLength}; RecordBatch {length, nodes: [FieldNode{length, null_count}], buffers:
// [Buffer{offset, length}], compression: BodyCompression{codec, method}}.
constexpr uint8_t kHeaderSchema = 1, kHeaderRecordBatch = 3;

}  // namespace

Status PartitionReader::Cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status::OK();
  cudaGetLastError();
  return Status::Error(e == cudaErrorMemoryAllocation ? GZ_OOM : GZ_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

Status PartitionReader::Make(std::vector<Field> fields, int device, std::unique_ptr<PartitionReader>* out) {
  std::unique_ptr<PartitionReader> r(new PartitionReader());
  r->tree_.assign(fields.size(), {});
  for (size_t i = 0; i < fields.size(); i++) {
    const Field& f = fields[i];
    if (NestedField(f)) {
      if (!f.nested()) return Status::Error(GZ_INVALID, "nested field without child fields");
      // pre-order type tree; a simple list below becomes a list node and its element leaf
      std::vector<RNode>& tree = r->tree_[i];
      bool ok = true;
      std::function<void(const Field&, int)> add = [&](const Field& g, int parent) {
        const int idx = (int)tree.size();
        tree.push_back(RNode{g.type, FixedWidth(g.type), parent, {}});
        if (parent >= 0) tree[parent].kids.push_back(idx);
        if (g.type == GZ_TYPE_LIST && !g.nested()) {
          Field e;
          e.type = g.elem;
          add(e, idx);
          return;
        }
        const bool leaf_ok = IsBinaryType(g.type) || g.type == GZ_TYPE_BOOL || FixedWidth(g.type) > 0;
        if (g.children.empty() ? !leaf_ok : !(ListLikeType(g.type) || g.type == GZ_TYPE_STRUCT)) ok = false;
        for (const Field& c : g.children) add(c, idx);
      };
      add(f, -1);
      if (!ok) return Status::Error(GZ_NOT_IMPLEMENTED, "nested field type not implemented by the reader");
      continue;
    }
    if (f.type == GZ_TYPE_LIST ? FixedWidth(f.elem) == 0 && f.elem != GZ_TYPE_BOOL
                               : f.type != GZ_TYPE_NULL && f.type != GZ_TYPE_BOOL && !IsBinaryType(f.type) &&
                                     FixedWidth(f.type) == 0)
      return Status::Error(GZ_NOT_IMPLEMENTED, "field type not implemented by the reader");
  }
  r->fields_ = std::move(fields);
  r->device_ = device;
  Status st = r->Cuda(cudaSetDevice(device), "cudaSetDevice");
  if (!st.ok()) return st;
  st = r->Cuda(cudaStreamCreateWithFlags(&r->stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!st.ok()) return st;
  int pageable = 0, host_tables = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
  cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
  r->direct_ = pageable != 0 && host_tables != 0;
  r->out_.assign(r->fields_.size(), OutCol());
  *out = std::move(r);
  return Status::OK();
}

PartitionReader::~PartitionReader() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (uint8_t* p : images_)
    if (p) cudaFreeAsync(p, stream_);
  for (uint8_t* p : arena_mem_)
    if (p) cudaFreeAsync(p, stream_);
  if (out_mem_) cudaFreeAsync(out_mem_, stream_);
  if (stream_) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
  PinnedRelease(PinnedBlock{reinterpret_cast<uint8_t*>(jobs_), jobs_bytes_});
}

// Walks the messages of one stream: an optional schema message, record batches, then the
// end-of-stream marker (or the end of the bytes).  Buffer ranges are recorded relative to the
// stream start, where the device copy keeps them.
Status PartitionReader::ParseStream(const uint8_t* data, int64_t len, int stream, std::vector<Batch>* out,
                                    std::vector<FrameRef>* frames, int64_t* arena_bytes) {
  int64_t pos = 0;
  while (pos < len) {
    if (len - pos < 4) return Status::Error(GZ_INVALID, "truncated IPC stream");
    uint32_t first;
    memcpy(&first, data + pos, 4);
    int32_t meta_len;
    int64_t meta_pos;
    if (first == 0xFFFFFFFFu) {  // continuation token, then the metadata length
      if (len - pos < 8) return Status::Error(GZ_INVALID, "truncated IPC stream");
      memcpy(&meta_len, data + pos + 4, 4);
      meta_pos = pos + 8;
    } else {  // legacy framing: the length alone
      meta_len = (int32_t)first;
      meta_pos = pos + 4;
    }
    if (meta_len == 0) break;  // end of stream
    if (meta_len < 0 || meta_pos + meta_len > len) return Status::Error(GZ_INVALID, "bad IPC message length");
    FlatReader r(data + meta_pos, meta_len);
    uint32_t root;
    if (!r.Get(0, &root)) return Status::Error(GZ_INVALID, "bad IPC message");
    const int64_t msg = root;
    const uint8_t header_type = r.Scalar<uint8_t>(msg, 1, 0);
    const int64_t body_len = r.Scalar<int64_t>(msg, 3, 0);
    const int64_t body_pos = meta_pos + meta_len;
    if (body_len < 0 || body_pos + body_len > len) return Status::Error(GZ_INVALID, "IPC message body exceeds the stream");
    if (body_pos & 7) return Status::Error(GZ_NOT_IMPLEMENTED, "IPC message body not on an 8-byte boundary");
    if (header_type == kHeaderSchema) {
      std::vector<Field> fs;
      std::string err;
      if (!ParseSchemaIpc(data + pos, body_pos - pos, &fs, &err))
        return Status::Error(GZ_INVALID, "schema message in the stream: " + err);
      if (fs.size() != fields_.size()) return Status::Error(GZ_INVALID, "stream schema differs from the reader's");
      for (size_t i = 0; i < fs.size(); i++)
        if (fs[i].type != fields_[i].type) return Status::Error(GZ_INVALID, "stream schema differs from the reader's");
    } else if (header_type == kHeaderRecordBatch) {
      const int64_t rb = r.Table(msg, 2);
      if (rb < 0) return Status::Error(GZ_INVALID, "record batch without header");
      // BodyCompression {codec, method}: LZ4_FRAME (0) and BUFFER (0) are the defaults
      const int64_t comp = r.Table(rb, 3);
      const bool compressed = comp >= 0;
      if (compressed && (r.Scalar<int8_t>(comp, 0, 0) != 0 || r.Scalar<int8_t>(comp, 1, 0) != 0))
        return Status::Error(GZ_NOT_IMPLEMENTED, "body compression other than LZ4_FRAME per buffer");
      Batch b;
      b.stream = stream;
      b.rows = r.Scalar<int64_t>(rb, 0, 0);
      const int64_t nodes = r.Table(rb, 1), bufs = r.Table(rb, 2);
      uint32_t n_nodes = 0, n_bufs = 0;
      if (nodes < 0 || bufs < 0 || !r.Get(nodes, &n_nodes) || !r.Get(bufs, &n_bufs))
        return Status::Error(GZ_INVALID, "record batch without nodes or buffers");
      uint32_t node = 0, buf = 0;
      auto next_buf = [&](BufRef* out_ref) -> bool {
        int64_t off, l;
        if (buf >= n_bufs || !r.Get(bufs + 4 + 16 * (int64_t)buf, &off) || !r.Get(bufs + 4 + 16 * (int64_t)buf + 8, &l))
          return false;
        buf++;
        if (off < 0 || l < 0 || off + l > body_len || (off & 7)) return false;
        out_ref->offset = body_pos + off;
        out_ref->length = l;
        out_ref->decoded = false;
        if (compressed && l > 0) {
          // an int64 uncompressed length, then one LZ4 frame (-1: the bytes follow as they are)
          if (l < 8) return false;
          int64_t ul;
          memcpy(&ul, data + body_pos + off, 8);
          if (ul == -1) {
            out_ref->offset += 8;
            out_ref->length = l - 8;
          } else {
            if (ul < 0) return false;
            frames->push_back(FrameRef{body_pos + off + 8, l - 8, *arena_bytes, ul});
            out_ref->offset = *arena_bytes;
            out_ref->length = ul;
            out_ref->decoded = true;
            *arena_bytes += Pad8(ul);
          }
        }
        return true;
      };
      b.cols.resize(fields_.size());
      for (size_t f = 0; f < fields_.size(); f++) {
        int64_t nl, nn;
        if (node >= n_nodes || !r.Get(nodes + 4 + 16 * (int64_t)node, &nl) ||
            !r.Get(nodes + 4 + 16 * (int64_t)node + 8, &nn))
          return Status::Error(GZ_INVALID, "record batch has too few field nodes");
        node++;
        if (nl != b.rows) return Status::Error(GZ_INVALID, "field length differs from the batch length");
        ColRef& c = b.cols[f];
        c.null_count = nn;
        const int t = fields_[f].type;
        if (t == GZ_TYPE_NULL) continue;  // no buffers
        if (!tree_[f].empty()) {  // a nested field: every node in pre-order with its buffers
          const std::vector<RNode>& tree = tree_[f];
          c.nodes.resize(tree.size());
          for (size_t q = 0; q < tree.size(); q++) {
            NodeRef& nr = c.nodes[q];
            if (q == 0) {
              nr.length = nl;
              nr.null_count = nn;
            } else {
              if (node >= n_nodes || !r.Get(nodes + 4 + 16 * (int64_t)node, &nr.length) ||
                  !r.Get(nodes + 4 + 16 * (int64_t)node + 8, &nr.null_count))
                return Status::Error(GZ_INVALID, "record batch has too few field nodes");
              node++;
            }
            const int qt = tree[q].type;
            bool ok = next_buf(&nr.validity);
            if (ListLikeType(qt) || IsBinaryType(qt)) ok = ok && next_buf(&nr.offsets);
            if (qt != GZ_TYPE_STRUCT && !ListLikeType(qt)) ok = ok && next_buf(&nr.values);
            if (!ok) return Status::Error(GZ_INVALID, "bad buffer list in a record batch");
            if (nr.length < 0 || nr.null_count < 0 || nr.null_count > nr.length || nr.length >= (1ll << 31))
              return Status::Error(GZ_INVALID, "bad field node");
            if (nr.null_count > 0 && nr.validity.length < (nr.length + 7) / 8)
              return Status::Error(GZ_INVALID, "validity buffer too short");
            if (nr.null_count == 0) nr.validity.length = 0;
            if (ListLikeType(qt) || IsBinaryType(qt)) {
              const int ow = NodeOffsetWidth(qt);
              if (nr.offsets.length < (nr.length + 1) * ow) return Status::Error(GZ_INVALID, "offsets buffer too short");
              if (!nr.offsets.decoded) {  // decoded offsets are read after decoding
                nr.o0 = ReadOffset(data + nr.offsets.offset, ow, 0);
                nr.o1 = ReadOffset(data + nr.offsets.offset, ow, nr.length);
              }
            } else if (qt != GZ_TYPE_STRUCT) {
              const int64_t need = qt == GZ_TYPE_BOOL ? (nr.length + 7) / 8 : nr.length * tree[q].width;
              if (nr.values.length < need) return Status::Error(GZ_INVALID, "value buffer too short");
            }
          }
          continue;
        }
        if (t == GZ_TYPE_LIST) {
          // the element node follows the list's; buffers [validity, offsets, element validity, values]
          int64_t cl, cn;
          if (node >= n_nodes || !r.Get(nodes + 4 + 16 * (int64_t)node, &cl) ||
              !r.Get(nodes + 4 + 16 * (int64_t)node + 8, &cn))
            return Status::Error(GZ_INVALID, "list without an element node");
          node++;
          c.child_nulls = cn;
          if (!(next_buf(&c.validity) && next_buf(&c.offsets) && next_buf(&c.cvalidity) && next_buf(&c.values)))
            return Status::Error(GZ_INVALID, "bad buffer list in a record batch");
          if ((nn > 0 && c.validity.length < (b.rows + 7) / 8) || (cn > 0 && c.cvalidity.length < (cl + 7) / 8))
            return Status::Error(GZ_INVALID, "validity buffer too short");
          if (nn == 0) c.validity.length = 0;
          if (cn == 0) c.cvalidity.length = 0;
          if (c.offsets.length < (b.rows + 1) * 4) return Status::Error(GZ_INVALID, "offsets buffer too short");
          const int w = FixedWidth(fields_[f].elem);  // 0: bool elements (bits)
          if (!c.offsets.decoded) {
            c.o0 = ReadOffset(data + c.offsets.offset, 4, 0);
            c.o1 = ReadOffset(data + c.offsets.offset, 4, b.rows);
            if (c.o0 < 0 || c.o1 < c.o0 || (w ? c.o1 * w : (c.o1 + 7) / 8) > c.values.length || c.o1 - c.o0 != cl)
              return Status::Error(GZ_INVALID, "list offsets exceed the elements");
          }
          continue;
        }
        bool ok = next_buf(&c.validity);
        if (IsBinaryType(t)) ok = ok && next_buf(&c.offsets);
        ok = ok && next_buf(&c.values);
        if (!ok) return Status::Error(GZ_INVALID, "bad buffer list in a record batch");
        if (nn > 0 && c.validity.length < (b.rows + 7) / 8) return Status::Error(GZ_INVALID, "validity buffer too short");
        if (nn == 0) c.validity.length = 0;
        const int64_t need = t == GZ_TYPE_BOOL ? (b.rows + 7) / 8
                             : IsBinaryType(t) ? 0 : b.rows * FixedWidth(t);
        if (c.values.length < need) return Status::Error(GZ_INVALID, "value buffer too short");
        if (IsBinaryType(t)) {
          const int ow = OffsetWidth(t);
          if (c.offsets.length < (b.rows + 1) * ow) return Status::Error(GZ_INVALID, "offsets buffer too short");
          if (!c.offsets.decoded) {  // decoded offsets are read after decoding
            c.o0 = ReadOffset(data + c.offsets.offset, ow, 0);
            c.o1 = ReadOffset(data + c.offsets.offset, ow, b.rows);
            if (c.o0 < 0 || c.o1 < c.o0 || c.o1 > c.values.length)
              return Status::Error(GZ_INVALID, "offsets exceed the characters");
          }
        }
      }
      if (b.rows > 0) out->push_back(std::move(b));
    } else {
      return Status::Error(GZ_NOT_IMPLEMENTED, "IPC message type " + std::to_string(header_type) + " in a shuffle stream");
    }
    pos = body_pos + Pad8(body_len);
  }
  return Status::OK();
}

Status PartitionReader::AddStream(const uint8_t* data, int64_t len) {
  if (finished_) return Status::Error(GZ_INVALID, "reader already finished");
  if (len < 0 || (len > 0 && data == nullptr)) return Status::Error(GZ_INVALID, "null stream");
  std::vector<Batch> bs;
  std::vector<FrameRef> frames;
  int64_t arena_bytes = 0;
  const int idx = (int)images_.size();
  Status st = ParseStream(data, len, idx, &bs, &frames, &arena_bytes);
  if (!st.ok()) return st;
  st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  uint8_t* d = nullptr;
  uint8_t* arena = nullptr;
  if (!bs.empty()) {
    st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&d), AlignUp((size_t)len, 256), stream_), "cudaMallocAsync(stream)");
    if (!st.ok()) return st;
    // the caller's bytes are read before the call returns: by the device itself where it walks
    // the host page tables (many CTAs reading 256 KiB pieces over the coherent link), else by a copy
    if (direct_) {
      const size_t piece = 256u << 10;
      const size_t n = ((size_t)len + piece - 1) / piece;
      if (jobs_cap_ < n) {
        PinnedRelease(PinnedBlock{reinterpret_cast<uint8_t*>(jobs_), jobs_bytes_});
        const PinnedBlock b = PinnedAcquire(sizeof(HostCopy) * n);
        if (!b.ptr) return Status::Error(GZ_OOM, "pinned host memory for copy descriptors");
        jobs_ = reinterpret_cast<HostCopy*>(b.ptr);
        jobs_bytes_ = b.cap;
        jobs_cap_ = b.cap / sizeof(HostCopy);
      }
      for (size_t i = 0; i < n; i++)
        jobs_[i] = HostCopy{data + i * piece, d + i * piece, std::min<uint64_t>(piece, (uint64_t)len - i * piece)};
      st = Cuda(launch_gather(jobs_, (uint32_t)n, stream_), "k_gather");
    } else {
      st = Cuda(cudaMemcpyAsync(d, data, (size_t)len, cudaMemcpyHostToDevice, stream_), "H2D stream");
    }
    if (!st.ok()) return st;
  }
  images_.push_back(d);
  arenas_.push_back(nullptr);
  if (!frames.empty()) {
    // compressed buffers: every LZ4 frame decoded by the device into the stream's arena
    std::vector<Lz4Frame> jobs;
    for (const FrameRef& f : frames)
      jobs.push_back(Lz4Frame{nullptr, (uint64_t)f.src_len, nullptr, (uint64_t)f.dst_len});
    const size_t jb = AlignUp(sizeof(Lz4Frame) * jobs.size(), 256);
    st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&arena), jb + 256 + AlignUp((size_t)arena_bytes, 256), stream_),
              "cudaMallocAsync(decode)");
    if (!st.ok()) return st;
    arenas_.back() = arena + jb + 256;
    for (size_t i = 0; i < jobs.size(); i++) {
      jobs[i].src = d + frames[i].src;
      jobs[i].dst = arenas_.back() + frames[i].dst;
    }
    int32_t* d_err = reinterpret_cast<int32_t*>(arena + jb);
    int32_t err = 0;
    st = Cuda(cudaMemcpyAsync(arena, jobs.data(), sizeof(Lz4Frame) * jobs.size(), cudaMemcpyHostToDevice, stream_), "H2D");
    if (st.ok()) st = Cuda(cudaMemsetAsync(d_err, 0, 4, stream_), "memset");
    if (st.ok()) st = Cuda(launch_lz4_decode(reinterpret_cast<const Lz4Frame*>(arena), (uint32_t)jobs.size(), d_err, stream_),
                           "k_lz4_decode");
    if (st.ok()) st = Cuda(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, stream_), "D2H");
    // the decoded offsets bound each batch's characters (and a nested node's child entries): for
    // each, the 4-byte words of its first and last offset (low word, then high word of a 64-bit one)
    std::vector<const int32_t*> where;
    std::vector<std::pair<size_t, size_t>> which;  // (batch, field)
    std::vector<std::pair<NodeRef*, int>> nested;  // a nested node and its offset width
    auto queue_ends = [&](const int32_t* o, int64_t n, int ow) {
      for (int end = 0; end < 2; end++) {
        const int64_t at = end ? n : 0;
        where.push_back(o + at * (ow / 4));
        if (ow == 8) where.push_back(o + at * 2 + 1);
      }
    };
    for (size_t bi = 0; bi < bs.size(); bi++)
      for (size_t f = 0; f < fields_.size(); f++) {
        ColRef& c = bs[bi].cols[f];
        if (!tree_[f].empty()) continue;
        if (!HasOffsets(fields_[f].type) || !c.offsets.decoded) continue;
        const int32_t* o = reinterpret_cast<const int32_t*>(arenas_.back() + c.offsets.offset);
        queue_ends(o, bs[bi].rows, IsLargeBinaryType(fields_[f].type) ? 8 : 4);
        which.push_back({bi, f});
      }
    for (size_t bi = 0; bi < bs.size(); bi++)
      for (size_t f = 0; f < fields_.size(); f++)
        for (size_t q = 0; q < tree_[f].size(); q++) {
          NodeRef& nr = bs[bi].cols[f].nodes[q];
          if (!nr.offsets.decoded) continue;
          const int ow = NodeOffsetWidth(tree_[f][q].type);
          queue_ends(reinterpret_cast<const int32_t*>(arenas_.back() + nr.offsets.offset), nr.length, ow);
          nested.push_back({&nr, ow});
        }
    std::vector<int32_t> ends(where.size());
    if (st.ok() && !where.empty()) st = Cuda(gather_words(where.data(), ends.data(), where.size(), stream_), "offsets");
    if (st.ok()) st = Cuda(cudaStreamSynchronize(stream_), "k_lz4_decode");
    if (!st.ok()) return st;
    if (err) return Status::Error(GZ_INVALID, "a compressed buffer is not a valid LZ4 frame of its stated length");
    size_t e = 0;
    auto word = [&](int ow) -> int64_t {
      const int64_t v = ow == 8 ? (int64_t)((uint64_t)(uint32_t)ends[e] | (uint64_t)(uint32_t)ends[e + 1] << 32)
                                : (int64_t)ends[e];
      e += ow / 4;
      return v;
    };
    for (size_t i = 0; i < which.size(); i++) {
      ColRef& c = bs[which[i].first].cols[which[i].second];
      const int ow = IsLargeBinaryType(fields_[which[i].second].type) ? 8 : 4;
      c.o0 = word(ow);
      c.o1 = word(ow);
      const int64_t w = fields_[which[i].second].type == GZ_TYPE_LIST ? FixedWidth(fields_[which[i].second].elem) : 1;
      if (c.o0 < 0 || c.o1 < c.o0 || (w ? c.o1 * w : (c.o1 + 7) / 8) > c.values.length)
        return Status::Error(GZ_INVALID, "offsets exceed the characters");
    }
    for (auto& x : nested) {
      x.first->o0 = word(x.second);
      x.first->o1 = word(x.second);
    }
    arena_mem_.push_back(arena);
  } else {
    st = Cuda(cudaStreamSynchronize(stream_), "H2D stream");
    if (!st.ok()) return st;
  }
  // nested fields: list / map children hold exactly the parent's entries from 0 (as Arrow's
  // builders and IPC writer leave them), struct children the struct's, characters lie inside
  // their buffer
  for (const Batch& b : bs)
    for (size_t f = 0; f < fields_.size(); f++)
      for (size_t q = 0; q < tree_[f].size(); q++) {
        const RNode& tn = tree_[f][q];
        const NodeRef& nr = b.cols[f].nodes[q];
        if (ListLikeType(tn.type)) {
          if (nr.o0 != 0 || nr.o1 != b.cols[f].nodes[tn.kids[0]].length)
            return Status::Error(GZ_NOT_IMPLEMENTED, "nested offsets that do not span their child from 0");
        } else if (IsBinaryType(tn.type)) {
          if (nr.o0 < 0 || nr.o1 < nr.o0 || nr.o1 > nr.values.length)
            return Status::Error(GZ_INVALID, "offsets exceed the characters");
        } else if (tn.type == GZ_TYPE_STRUCT) {
          for (int k : tn.kids)
            if (b.cols[f].nodes[k].length != nr.length)
              return Status::Error(GZ_INVALID, "struct child length differs from the struct's");
        }
      }
  for (Batch& b : bs) batches_.push_back(std::move(b));
  return Status::OK();
}

Status PartitionReader::Finish(int64_t* rows, int32_t* n_batches) {
  if (finished_) return Status::Error(GZ_INVALID, "reader already finished");
  Status st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  const size_t F = fields_.size();
  int64_t R = 0;
  for (const Batch& b : batches_) R += b.rows;
  if (R >= (1ll << 31)) return Status::Error(GZ_INVALID, "more than 2^31 - 1 rows in one partition");
  // output layout: per field validity (when some batch has nulls), offsets, values / characters
  std::vector<size_t> o_valid(F, SIZE_MAX), o_off(F, SIZE_MAX), o_val(F, SIZE_MAX), o_cvalid(F, SIZE_MAX);
  std::vector<int64_t> chars(F, 0);  // binary: characters; list: elements
  size_t total = 0;
  const size_t bit_bytes = AlignUp((size_t)((R + 31) / 32) * 4, 256);
  // nested fields, per node: entries, nulls, characters (binary) and where its buffers go
  struct NodeLayout {
    int64_t length = 0, nulls = 0, chars = 0;
    size_t valid = SIZE_MAX, off = SIZE_MAX, val = SIZE_MAX;
  };
  std::vector<std::vector<NodeLayout>> nl(F);
  for (size_t f = 0; f < F; f++) {
    const std::vector<RNode>& tree = tree_[f];
    if (tree.empty()) continue;
    nl[f].resize(tree.size());
    for (const Batch& b : batches_)
      for (size_t q = 0; q < tree.size(); q++) {
        const NodeRef& nr = b.cols[f].nodes[q];
        nl[f][q].length += nr.length;
        nl[f][q].nulls += nr.null_count;
        if (IsBinaryType(tree[q].type)) nl[f][q].chars += nr.o1 - nr.o0;
      }
    for (size_t q = 0; q < tree.size(); q++) {
      NodeLayout& L = nl[f][q];
      const int t = tree[q].type;
      if (L.length >= (1ll << 31) || (L.chars >= (1ll << 31) && !IsLargeBinaryType(t)))
        return Status::Error(GZ_INVALID, "more than 2^31 - 1 entries in one nested node");
      if (L.nulls > 0) {
        L.valid = total;
        total += AlignUp((size_t)((L.length + 31) / 32) * 4, 256);
      }
      if (ListLikeType(t) || IsBinaryType(t)) {
        L.off = total;
        total += AlignUp((size_t)(L.length + 1) * NodeOffsetWidth(t), 256);
      }
      if (IsBinaryType(t)) {
        L.val = total;
        total += AlignUp((size_t)L.chars + 16, 256);
      } else if (t == GZ_TYPE_BOOL) {
        L.val = total;
        total += AlignUp((size_t)((L.length + 31) / 32) * 4, 256);
      } else if (t != GZ_TYPE_STRUCT && !ListLikeType(t)) {
        L.val = total;
        total += AlignUp((size_t)L.length * tree[q].width, 256);
      }
    }
  }
  for (size_t f = 0; f < F; f++) {
    const int t = fields_[f].type;
    OutCol& oc = out_[f];
    oc = OutCol();
    if (!tree_[f].empty()) continue;
    if (t == GZ_TYPE_NULL) {
      oc.null_count = R;
      continue;
    }
    for (const Batch& b : batches_) {
      oc.null_count += b.cols[f].null_count;
      oc.child_null_count += b.cols[f].child_nulls;
      if (HasOffsets(t)) chars[f] += b.cols[f].o1 - b.cols[f].o0;
    }
    if (chars[f] >= (1ll << 31) && !IsLargeBinaryType(t))
      return Status::Error(GZ_INVALID, "more than 2^31 - 1 characters in one column");
    if (oc.null_count > 0) {
      o_valid[f] = total;
      total += bit_bytes;
    }
    if (HasOffsets(t)) {
      o_off[f] = total;
      total += AlignUp((size_t)(R + 1) * OffsetWidth(t), 256);
    }
    if (t == GZ_TYPE_LIST && oc.child_null_count > 0) {
      o_cvalid[f] = total;
      total += AlignUp((size_t)((chars[f] + 31) / 32) * 4, 256);
    }
    o_val[f] = total;
    total += t == GZ_TYPE_BOOL ? bit_bytes
             : IsBinaryType(t) ? AlignUp((size_t)chars[f] + 16, 256)
             : t == GZ_TYPE_LIST ? (fields_[f].elem == GZ_TYPE_BOOL ? AlignUp((size_t)((chars[f] + 31) / 32) * 4, 256)
                                                                    : AlignUp((size_t)chars[f] * FixedWidth(fields_[f].elem), 256))
                                 : AlignUp((size_t)R * FixedWidth(t), 256);
  }
  total = std::max<size_t>(total, 256);
  st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&out_mem_), total, stream_), "cudaMallocAsync(columns)");
  if (!st.ok()) return st;
  st = Cuda(cudaMemsetAsync(out_mem_, 0, total, stream_), "memset(columns)");
  if (!st.ok()) return st;

  // job lists, built on the host and copied to the device in one piece
  std::vector<ByteJob> bj;
  std::vector<OffsetJob> oj;
  std::vector<BitJob> tj;
  constexpr uint64_t kChunk = 256u << 10;   // bytes per byte job
  constexpr uint64_t kBitChunk = 1u << 20;  // bits per bit job
  auto add_bytes = [&](const uint8_t* src, uint8_t* dst, uint64_t n) {
    for (uint64_t x = 0; x < n; x += kChunk) bj.push_back(ByteJob{src + x, dst + x, std::min(kChunk, n - x)});
  };
  auto add_bits = [&](const uint8_t* src, uint32_t* dst, uint64_t dst_bit, uint64_t n) {
    for (uint64_t x = 0; x < n; x += kBitChunk)
      tj.push_back(BitJob{reinterpret_cast<const uint32_t*>(src), dst, src ? x : 0, dst_bit + x, std::min(kBitChunk, n - x)});
  };
  std::vector<int64_t> char_pos(F, 0);
  std::vector<std::vector<int64_t>> npos(F), ncpos(F);  // nested: entries / characters so far per node
  for (size_t f = 0; f < F; f++) {
    npos[f].assign(tree_[f].size(), 0);
    ncpos[f].assign(tree_[f].size(), 0);
  }
  int64_t row = 0;
  for (size_t bi = 0; bi < batches_.size(); bi++) {
    const Batch& b = batches_[bi];
    const bool last = bi + 1 == batches_.size();
    for (size_t f = 0; f < F; f++) {
      const int t = fields_[f].type;
      if (t == GZ_TYPE_NULL) continue;
      const ColRef& c = b.cols[f];
      if (!tree_[f].empty()) {
        // every node: validity bits at its entries so far, offsets rebased onto its child's
        // entries (or characters) so far, values / bits / characters appended
        const std::vector<RNode>& tree = tree_[f];
        for (size_t q = 0; q < tree.size(); q++) {
          const NodeRef& nr = c.nodes[q];
          const NodeLayout& L = nl[f][q];
          const int qt = tree[q].type;
          const uint64_t at = (uint64_t)npos[f][q];
          if (L.valid != SIZE_MAX && nr.length > 0)
            add_bits(nr.validity.length ? Base(nr.validity, b.stream) : nullptr,
                     reinterpret_cast<uint32_t*>(out_mem_ + L.valid), at, (uint64_t)nr.length);
          if (ListLikeType(qt) || IsBinaryType(qt)) {
            const int ow = NodeOffsetWidth(qt);
            const int64_t base = IsBinaryType(qt) ? ncpos[f][q] : npos[f][tree[q].kids[0]];
            const uint8_t* src_off = Base(nr.offsets, b.stream);
            uint8_t* dst_off = out_mem_ + L.off + at * ow;
            const uint64_t n = (uint64_t)nr.length + (last ? 1 : 0);
            for (uint64_t x = 0; x < n; x += kChunk / 4)
              oj.push_back(OffsetJob{src_off + x * ow, dst_off + x * ow, (uint32_t)std::min<uint64_t>(kChunk / 4, n - x),
                                     ow == 8 ? 1u : 0u, base - nr.o0});
          }
          if (IsBinaryType(qt)) {
            add_bytes(Base(nr.values, b.stream) + nr.o0, out_mem_ + L.val + ncpos[f][q], (uint64_t)(nr.o1 - nr.o0));
            ncpos[f][q] += nr.o1 - nr.o0;
          } else if (qt == GZ_TYPE_BOOL) {
            if (nr.length > 0)
              add_bits(Base(nr.values, b.stream), reinterpret_cast<uint32_t*>(out_mem_ + L.val), at, (uint64_t)nr.length);
          } else if (qt != GZ_TYPE_STRUCT && !ListLikeType(qt)) {
            add_bytes(Base(nr.values, b.stream), out_mem_ + L.val + at * tree[q].width,
                      (uint64_t)nr.length * tree[q].width);
          }
        }
        for (size_t q = 0; q < tree.size(); q++) npos[f][q] += c.nodes[q].length;
        continue;
      }
      if (o_valid[f] != SIZE_MAX)
        add_bits(c.validity.length ? Base(c.validity, b.stream) : nullptr,
                 reinterpret_cast<uint32_t*>(out_mem_ + o_valid[f]), (uint64_t)row, (uint64_t)b.rows);
      if (t == GZ_TYPE_BOOL) {
        add_bits(Base(c.values, b.stream), reinterpret_cast<uint32_t*>(out_mem_ + o_val[f]), (uint64_t)row,
                 (uint64_t)b.rows);
      } else if (IsBinaryType(t)) {
        // offsets rebased onto the characters of the earlier batches; the last batch also writes
        // the final offset
        const int ow = OffsetWidth(t);
        const uint8_t* src_off = Base(c.offsets, b.stream);
        uint8_t* dst_off = out_mem_ + o_off[f] + (size_t)row * ow;
        const int64_t add = char_pos[f] - c.o0;
        const uint64_t n = (uint64_t)b.rows + (last ? 1 : 0);
        for (uint64_t x = 0; x < n; x += kChunk / 4)
          oj.push_back(OffsetJob{src_off + x * ow, dst_off + x * ow, (uint32_t)std::min<uint64_t>(kChunk / 4, n - x),
                                 ow == 8 ? 1u : 0u, add});
        add_bytes(Base(c.values, b.stream) + c.o0, out_mem_ + o_val[f] + char_pos[f], (uint64_t)(c.o1 - c.o0));
        char_pos[f] += c.o1 - c.o0;
      } else if (t == GZ_TYPE_LIST) {
        // offsets rebased onto the elements of the earlier batches; the elements' values and
        // validity bits moved to their position (a batch without element nulls adds ones)
        const uint8_t* src_off = Base(c.offsets, b.stream);
        uint8_t* dst_off = out_mem_ + o_off[f] + (size_t)row * 4;
        const uint64_t n = (uint64_t)b.rows + (last ? 1 : 0);
        for (uint64_t x = 0; x < n; x += kChunk / 4)
          oj.push_back(OffsetJob{src_off + x * 4, dst_off + x * 4, (uint32_t)std::min<uint64_t>(kChunk / 4, n - x), 0u,
                                 char_pos[f] - c.o0});
        const int w = FixedWidth(fields_[f].elem);
        if (w == 0) {  // bool elements: bits [o0, o1) to bit char_pos
          for (uint64_t x = 0; x < (uint64_t)(c.o1 - c.o0); x += kBitChunk)
            tj.push_back(BitJob{reinterpret_cast<const uint32_t*>(Base(c.values, b.stream)),
                                reinterpret_cast<uint32_t*>(out_mem_ + o_val[f]), (uint64_t)c.o0 + x,
                                (uint64_t)char_pos[f] + x, std::min<uint64_t>(kBitChunk, (uint64_t)(c.o1 - c.o0) - x)});
        } else {
          add_bytes(Base(c.values, b.stream) + c.o0 * w, out_mem_ + o_val[f] + char_pos[f] * w,
                    (uint64_t)(c.o1 - c.o0) * w);
        }
        if (o_cvalid[f] != SIZE_MAX && c.o1 > c.o0) {
          const uint8_t* cv = c.cvalidity.length ? Base(c.cvalidity, b.stream) : nullptr;
          for (uint64_t x = 0; x < (uint64_t)(c.o1 - c.o0); x += kBitChunk)
            tj.push_back(BitJob{reinterpret_cast<const uint32_t*>(cv), reinterpret_cast<uint32_t*>(out_mem_ + o_cvalid[f]),
                                cv ? (uint64_t)c.o0 + x : 0, (uint64_t)char_pos[f] + x,
                                std::min<uint64_t>(kBitChunk, (uint64_t)(c.o1 - c.o0) - x)});
        }
        char_pos[f] += c.o1 - c.o0;
      } else {
        const int w = FixedWidth(t);
        add_bytes(Base(c.values, b.stream), out_mem_ + o_val[f] + (size_t)row * w, (uint64_t)b.rows * w);
      }
    }
    row += b.rows;
  }
  const size_t jb = AlignUp(sizeof(ByteJob) * bj.size(), 256), jo = AlignUp(sizeof(OffsetJob) * oj.size(), 256),
               jt = AlignUp(sizeof(BitJob) * tj.size(), 256);
  std::vector<uint8_t> hj(std::max<size_t>(jb + jo + jt, 256), 0);
  if (!bj.empty()) memcpy(hj.data(), bj.data(), sizeof(ByteJob) * bj.size());
  if (!oj.empty()) memcpy(hj.data() + jb, oj.data(), sizeof(OffsetJob) * oj.size());
  if (!tj.empty()) memcpy(hj.data() + jb + jo, tj.data(), sizeof(BitJob) * tj.size());
  uint8_t* dj = nullptr;
  st = Cuda(cudaMallocAsync(reinterpret_cast<void**>(&dj), hj.size(), stream_), "cudaMallocAsync(jobs)");
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpyAsync(dj, hj.data(), hj.size(), cudaMemcpyHostToDevice, stream_), "H2D jobs");
  if (st.ok())
    st = Cuda(launch_read_jobs(reinterpret_cast<const ByteJob*>(dj), (uint32_t)bj.size(),
                               reinterpret_cast<const OffsetJob*>(dj + jb), (uint32_t)oj.size(),
                               reinterpret_cast<const BitJob*>(dj + jb + jo), (uint32_t)tj.size(), stream_),
              "reader kernels");
  cudaFreeAsync(dj, stream_);
  if (!st.ok()) return st;
  // the stream images and decoded buffers are no longer needed
  for (uint8_t*& p : images_) {
    if (p) cudaFreeAsync(p, stream_);
    p = nullptr;
  }
  for (uint8_t*& p : arena_mem_) {
    if (p) cudaFreeAsync(p, stream_);
    p = nullptr;
  }
  st = Cuda(cudaStreamSynchronize(stream_), "reader kernels");
  if (!st.ok()) return st;
  out_nodes_.assign(F, {});
  for (size_t f = 0; f < F; f++) {
    for (size_t q = 0; q < tree_[f].size(); q++) {
      const NodeLayout& L = nl[f][q];
      const int qt = tree_[f][q].type;
      OutNode on;
      on.type = qt;
      on.length = L.length;
      on.null_count = L.nulls;
      if (L.valid != SIZE_MAX) on.validity = out_mem_ + L.valid;
      if (L.off != SIZE_MAX) on.offsets = out_mem_ + L.off;
      if (L.val != SIZE_MAX) on.values = out_mem_ + L.val;
      on.values_bytes = IsBinaryType(qt) ? L.chars : qt == GZ_TYPE_BOOL ? (L.length + 7) / 8
                        : L.val != SIZE_MAX ? L.length * tree_[f][q].width : 0;
      out_nodes_[f].push_back(on);
    }
  }
  for (size_t f = 0; f < F; f++) {
    OutCol& oc = out_[f];
    const int t = fields_[f].type;
    if (t == GZ_TYPE_NULL || !tree_[f].empty()) continue;
    if (o_valid[f] != SIZE_MAX) oc.validity = out_mem_ + o_valid[f];
    if (o_off[f] != SIZE_MAX) oc.offsets = out_mem_ + o_off[f];
    oc.values = out_mem_ + o_val[f];
    oc.values_bytes = t == GZ_TYPE_BOOL ? (R + 7) / 8 : IsBinaryType(t) ? chars[f]
                      : t == GZ_TYPE_LIST ? (fields_[f].elem == GZ_TYPE_BOOL ? (chars[f] + 7) / 8
                                                                             : chars[f] * FixedWidth(fields_[f].elem))
                                          : R * FixedWidth(t);
    if (t == GZ_TYPE_LIST) {
      oc.child_length = chars[f];
      if (o_cvalid[f] != SIZE_MAX) oc.child_validity = out_mem_ + o_cvalid[f];
    }
  }
  rows_ = R;
  finished_ = true;
  if (rows) *rows = R;
  if (n_batches) *n_batches = (int32_t)batches_.size();
  return Status::OK();
}

Status PartitionReader::Column(int field, GzDeviceColumn* out) const {
  if (!finished_) return Status::Error(GZ_INVALID, "reader not finished");
  if (field < 0 || field >= (int)fields_.size()) return Status::Error(GZ_INVALID, "field out of range");
  if (!tree_[field].empty()) return Node(field, 0, out);
  const OutCol& c = out_[field];
  out->type = fields_[field].type;
  out->reserved = 0;
  out->length = rows_;
  out->null_count = c.null_count;
  out->validity = c.validity;
  out->offsets = c.offsets;
  out->values = c.values;
  out->values_bytes = c.values_bytes;
  out->child_validity = c.child_validity;
  out->child_length = c.child_length;
  out->child_null_count = c.child_null_count;
  return Status::OK();
}

int PartitionReader::NodeCount(int field) const {
  if (field < 0 || field >= (int)fields_.size()) return 0;
  if (!tree_[field].empty()) return (int)tree_[field].size();
  return fields_[field].type == GZ_TYPE_LIST ? 2 : 1;
}

Status PartitionReader::Node(int field, int node, GzDeviceColumn* out) const {
  if (!finished_) return Status::Error(GZ_INVALID, "reader not finished");
  if (field < 0 || field >= (int)fields_.size()) return Status::Error(GZ_INVALID, "field out of range");
  if (node < 0 || node >= NodeCount(field)) return Status::Error(GZ_INVALID, "node out of range");
  memset(out, 0, sizeof(*out));
  if (!tree_[field].empty()) {
    const OutNode& n = out_nodes_[field][node];
    out->type = n.type;
    out->length = n.length;
    out->null_count = n.null_count;
    out->validity = n.validity;
    out->offsets = n.offsets;
    out->values = n.values;
    out->values_bytes = n.values_bytes;
    return Status::OK();
  }
  if (node == 0) {
    Status st = Column(field, out);
    if (st.ok() && fields_[field].type == GZ_TYPE_LIST) out->values = nullptr, out->values_bytes = 0;
    return st;
  }
  // a simple list's elements
  const OutCol& c = out_[field];
  out->type = fields_[field].elem;
  out->length = c.child_length;
  out->null_count = c.child_null_count;
  out->validity = c.child_validity;
  out->values = c.values;
  out->values_bytes = c.values_bytes;
  return Status::OK();
}

Status PartitionReader::NodeToHost(int field, int node, uint8_t* validity, void* offsets, uint8_t* values) {
  GzDeviceColumn c;
  Status st = Node(field, node, &c);
  if (!st.ok()) return st;
  st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  if (validity && c.validity) {
    st = Cuda(cudaMemcpyAsync(validity, c.validity, (size_t)(c.length + 7) / 8, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (!st.ok()) return st;
  }
  if (offsets && c.offsets) {
    st = Cuda(cudaMemcpyAsync(offsets, c.offsets, (size_t)(c.length + 1) * NodeOffsetWidth(c.type), cudaMemcpyDeviceToHost,
                              stream_), "D2H");
    if (!st.ok()) return st;
  }
  if (values && c.values && c.values_bytes > 0) {
    st = Cuda(cudaMemcpyAsync(values, c.values, (size_t)c.values_bytes, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (!st.ok()) return st;
  }
  return Cuda(cudaStreamSynchronize(stream_), "D2H");
}

Status PartitionReader::ElemValidityToHost(int field, uint8_t* out) {
  GzDeviceColumn c;
  Status st = Column(field, &c);
  if (!st.ok()) return st;
  if (!out || !c.child_validity) return Status::OK();
  st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpyAsync(out, c.child_validity, (size_t)(c.child_length + 7) / 8, cudaMemcpyDeviceToHost, stream_),
            "D2H");
  if (!st.ok()) return st;
  return Cuda(cudaStreamSynchronize(stream_), "D2H");
}

Status PartitionReader::ColumnToHost(int field, uint8_t* validity, void* offsets, uint8_t* values) {
  GzDeviceColumn c;
  Status st = Column(field, &c);
  if (!st.ok()) return st;
  st = Cuda(cudaSetDevice(device_), "cudaSetDevice");
  if (!st.ok()) return st;
  if (validity && c.validity) {
    st = Cuda(cudaMemcpyAsync(validity, c.validity, (size_t)(c.length + 7) / 8, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (!st.ok()) return st;
  }
  if (offsets && c.offsets) {
    st = Cuda(cudaMemcpyAsync(offsets, c.offsets, (size_t)(c.length + 1) * NodeOffsetWidth(c.type), cudaMemcpyDeviceToHost,
                              stream_), "D2H");
    if (!st.ok()) return st;
  }
  if (values && c.values && c.values_bytes > 0) {
    st = Cuda(cudaMemcpyAsync(values, c.values, (size_t)c.values_bytes, cudaMemcpyDeviceToHost, stream_), "D2H");
    if (!st.ok()) return st;
  }
  return Cuda(cudaStreamSynchronize(stream_), "D2H");
}

}  // namespace gz
