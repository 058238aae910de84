// Arrow IPC RecordBatch message encoder.
//
// The flatbuffer that Arrow C++ builds for Message{header: RecordBatch} with no codec, no
// custom metadata and no variadic buffer counts has one fixed shape, so it is written here
// directly rather than through a flatbuffer builder.  With L field nodes and M buffers the
// flatbuffer is 88 + 16 * (L + M) bytes (always a multiple of 8, so no padding follows it):
//
//   [0]     u32 root table offset = 20        [4]  4 zero bytes (root alignment)
//   [8]     Message vtable {12, 22, 6, 5, 8, 12}
//   [20]    Message table: i32 vtable distance 12, pad, u8 header_type 3 (RecordBatch),
//           i16 version 4 (V5), u32 header offset 24 (-> 52), i64 bodyLength at [32]
//   [40]    2 pad bytes, RecordBatch vtable {10, 24, 12, 4, 8}
//   [52]    RecordBatch table: i32 vtable distance 10, u32 nodes offset 16M+28,
//           u32 buffers offset 16, i64 length at [64], 4 pad bytes
//   [76]    u32 M, M x {i64 offset, i64 length}, 4 pad bytes, u32 L, L x {i64 length, i64 nulls}
//
// Field order and padding follow the flatbuffers build algorithm as Arrow drives it
// (CreateVectorOfStructs for nodes then buffers, CreateRecordBatch, CreateMessage, Finish);
// the tests compare it against the Arrow C++ writer's bytes.
#include "ipc.h"

#include <stdio.h>
#include <string.h>

namespace gz {

namespace {
inline int64_t Pad8(int64_t n) { return (n + 7) & ~int64_t(7); }
const uint8_t kZeros[64] = {0};

template <typename T>
void Put(uint8_t* p, T v) {
  memcpy(p, &v, sizeof(T));
}

bool WriteZeros(ByteSink* sink, int64_t n) {
  while (n > 0) {
    int64_t k = n < 64 ? n : 64;
    if (!sink->Write(kZeros, k)) return false;
    n -= k;
  }
  return true;
}
}  // namespace

bool MemorySink::Write(const void* p, int64_t n) {
  const uint8_t* b = static_cast<const uint8_t*>(p);
  buf_.insert(buf_.end(), b, b + n);
  return true;
}

FileSink::FileSink(const std::string& path) {
  f_ = fopen(path.c_str(), "wb");
  buf_.reserve(1 << 22);
}

FileSink::~FileSink() { Close(); }

bool FileSink::FlushBuf() {
  if (!f_ || buf_.empty()) return f_ != nullptr;
  bool ok = fwrite(buf_.data(), 1, buf_.size(), static_cast<FILE*>(f_)) == buf_.size();
  buf_.clear();
  return ok;
}

bool FileSink::Write(const void* p, int64_t n) {
  if (!f_) return false;
  pos_ += n;
  if ((int64_t)buf_.size() + n > (int64_t)buf_.capacity()) {
    if (!FlushBuf()) return false;
    if (n >= (int64_t)buf_.capacity()) {
      return fwrite(p, 1, n, static_cast<FILE*>(f_)) == (size_t)n;
    }
  }
  const uint8_t* b = static_cast<const uint8_t*>(p);
  buf_.insert(buf_.end(), b, b + n);
  return true;
}

bool FileSink::Close() {
  if (!f_) return true;
  bool ok = FlushBuf();
  ok = fclose(static_cast<FILE*>(f_)) == 0 && ok;
  f_ = nullptr;
  return ok;
}

int64_t RecordBatchMessageSize(int64_t n_nodes, const std::vector<int64_t>& buffer_lengths,
                               int64_t* body_length) {
  int64_t body = 0;
  for (int64_t l : buffer_lengths) body += Pad8(l);
  *body_length = body;
  return 8 + 88 + 16 * (n_nodes + (int64_t)buffer_lengths.size()) + body;
}

// With body compression the RecordBatch table gains its fourth field, an offset to an empty
// BodyCompression table (codec LZ4_FRAME and method BUFFER are the schema's defaults, so neither
// is stored), and each vector's length is padded so that its 16-byte structs stay 8-byte aligned:
//
//   [0..40) as above        [40] RecordBatch vtable {12, 28, 12, 4, 8, 20}
//   [52]    RecordBatch table: i32 vtable distance 12, u32 nodes offset 16M+36, u32 buffers
//           offset 24, i64 length at [64], u32 compression offset 16(M+L)+28 at [72], 4 pad bytes
//   [80]    4 pad bytes, u32 M, M x {offset, length}; 4 pad bytes, u32 L, L x {length, nulls}
//   [96+16(M+L)] BodyCompression vtable {4, 4}, table: i32 vtable distance 4
// for a flatbuffer of 104 + 16 * (L + M) bytes.
void CompressedRecordBatchHeader(int64_t length, const std::vector<FieldNodeMeta>& nodes,
                                 const std::vector<int64_t>& lens, std::vector<uint8_t>* out,
                                 int64_t* body_length) {
  const int64_t L = (int64_t)nodes.size();
  const int64_t M = (int64_t)lens.size();
  int64_t body = 0;
  const int64_t fb_size = 104 + 16 * (L + M);
  std::vector<uint8_t> meta(8 + fb_size, 0);
  uint8_t* h = meta.data();
  Put<uint32_t>(h, 0xFFFFFFFFu);
  Put<int32_t>(h + 4, (int32_t)fb_size);
  uint8_t* f = h + 8;
  Put<uint32_t>(f + 0, 20);
  const uint16_t msg_vt[6] = {12, 22, 6, 5, 8, 12};
  memcpy(f + 8, msg_vt, sizeof(msg_vt));
  Put<int32_t>(f + 20, 12);
  f[25] = 3;
  Put<int16_t>(f + 26, 4);
  Put<uint32_t>(f + 28, 24);
  const uint16_t rb_vt[6] = {12, 28, 12, 4, 8, 20};
  memcpy(f + 40, rb_vt, sizeof(rb_vt));
  Put<int32_t>(f + 52, 12);
  Put<uint32_t>(f + 56, (uint32_t)(16 * M + 36));
  Put<uint32_t>(f + 60, 24);
  Put<int64_t>(f + 64, length);
  Put<uint32_t>(f + 72, (uint32_t)(16 * (M + L) + 28));
  Put<uint32_t>(f + 84, (uint32_t)M);
  uint8_t* bm = f + 88;
  for (int64_t i = 0; i < M; i++) {
    Put<int64_t>(bm + 16 * i, body);
    Put<int64_t>(bm + 16 * i + 8, lens[i]);
    body += Pad8(lens[i]);
  }
  Put<int64_t>(f + 32, body);
  uint8_t* nm = f + 92 + 16 * M;
  Put<uint32_t>(nm, (uint32_t)L);
  for (int64_t i = 0; i < L; i++) {
    Put<int64_t>(nm + 4 + 16 * i, nodes[i].length);
    Put<int64_t>(nm + 4 + 16 * i + 8, nodes[i].null_count);
  }
  uint8_t* bc = f + 96 + 16 * (M + L);
  const uint16_t bc_vt[2] = {4, 4};
  memcpy(bc, bc_vt, sizeof(bc_vt));
  Put<int32_t>(bc + 4, 4);
  *body_length = body;
  *out = std::move(meta);
}

uint8_t Lz4FrameHeaderChecksum(const uint8_t* desc, int n) {
  // xxHash32 (seed 0) of the frame descriptor, its second byte: the published algorithm's path
  // for inputs shorter than 16 bytes
  constexpr uint32_t P1 = 2654435761u, P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;
  uint32_t x = P5 + (uint32_t)n;
  int i = 0;
  for (; i + 4 <= n; i += 4) {
    uint32_t w;
    memcpy(&w, desc + i, 4);
    x += w * P3;
    x = ((x << 17) | (x >> 15)) * P4;
  }
  for (; i < n; i++) {
    x += desc[i] * P5;
    x = ((x << 11) | (x >> 21)) * P1;
  }
  x ^= x >> 15;
  x *= P2;
  x ^= x >> 13;
  x *= P3;
  x ^= x >> 16;
  return (uint8_t)((x >> 8) & 0xFF);
}

int64_t AppendLz4Buffer(int64_t uncompressed_len, const std::vector<Lz4BlockRef>& blocks,
                        std::vector<Chunk>* pieces, std::vector<std::vector<uint8_t>>* temps) {
  const size_t nb = blocks.size();
  temps->emplace_back(8 + 7 + 4 * nb + 4, 0);
  uint8_t* m = temps->back().data();
  Put<int64_t>(m, uncompressed_len);
  Put<uint32_t>(m + 8, 0x184D2204u);
  m[12] = kLz4Flg;
  m[13] = kLz4Bd;
  m[14] = Lz4FrameHeaderChecksum(m + 12, 2);
  pieces->push_back(Chunk{m, 15});
  int64_t total = 15;
  for (size_t i = 0; i < nb; i++) {
    uint8_t* w = m + 15 + 4 * i;
    Put<uint32_t>(w, blocks[i].size | (blocks[i].stored ? 0x80000000u : 0u));
    pieces->push_back(Chunk{w, 4});
    if (blocks[i].size) pieces->push_back(Chunk{blocks[i].data, (int64_t)blocks[i].size});
    total += 4 + blocks[i].size;
  }
  pieces->push_back(Chunk{m + 15 + 4 * nb, 4});  // end mark (zeros)
  return total + 4;
}

void RecordBatchHeader(int64_t length, const std::vector<FieldNodeMeta>& nodes,
                       const std::vector<int64_t>& lens, std::vector<uint8_t>* out,
                       int64_t* body_length) {
  const int64_t L = (int64_t)nodes.size();
  const int64_t M = (int64_t)lens.size();
  int64_t body = 0;
  const int64_t fb_size = 88 + 16 * (L + M);
  std::vector<uint8_t> meta(8 + fb_size, 0);
  uint8_t* h = meta.data();
  Put<uint32_t>(h, 0xFFFFFFFFu);
  Put<int32_t>(h + 4, (int32_t)fb_size);
  uint8_t* f = h + 8;
  Put<uint32_t>(f + 0, 20);
  const uint16_t msg_vt[6] = {12, 22, 6, 5, 8, 12};
  memcpy(f + 8, msg_vt, sizeof(msg_vt));
  Put<int32_t>(f + 20, 12);
  f[25] = 3;
  Put<int16_t>(f + 26, 4);
  Put<uint32_t>(f + 28, 24);
  const uint16_t rb_vt[5] = {10, 24, 12, 4, 8};
  memcpy(f + 42, rb_vt, sizeof(rb_vt));
  Put<int32_t>(f + 52, 10);
  Put<uint32_t>(f + 56, (uint32_t)(16 * M + 28));
  Put<uint32_t>(f + 60, 16);
  Put<int64_t>(f + 64, length);
  Put<uint32_t>(f + 76, (uint32_t)M);
  uint8_t* bm = f + 80;
  for (int64_t i = 0; i < M; i++) {
    Put<int64_t>(bm + 16 * i, body);
    Put<int64_t>(bm + 16 * i + 8, lens[i]);
    body += Pad8(lens[i]);
  }
  Put<int64_t>(f + 32, body);
  uint8_t* nm = f + 84 + 16 * M;
  Put<uint32_t>(nm, (uint32_t)L);
  for (int64_t i = 0; i < L; i++) {
    Put<int64_t>(nm + 4 + 16 * i, nodes[i].length);
    Put<int64_t>(nm + 4 + 16 * i + 8, nodes[i].null_count);
  }
  *body_length = body;
  *out = std::move(meta);
}

int64_t WriteRecordBatchMessage(ByteSink* sink, int64_t length,
                                const std::vector<FieldNodeMeta>& nodes,
                                const std::vector<ChunkedBuffer>& buffers, int64_t* body_length) {
  const int64_t M = (int64_t)buffers.size();
  std::vector<int64_t> lens(M, 0);
  for (int64_t i = 0; i < M; i++)
    for (const Chunk& c : buffers[i]) lens[i] += c.len;
  std::vector<uint8_t> meta;
  RecordBatchHeader(length, nodes, lens, &meta, body_length);
  const int64_t body = *body_length;
  if (!sink->Write(meta.data(), (int64_t)meta.size())) return -1;
  for (int64_t i = 0; i < M; i++) {
    for (const Chunk& c : buffers[i]) {
      if (c.len <= 0) continue;
      if (c.data == nullptr) {
        if (!WriteZeros(sink, c.len)) return -1;
      } else if (!sink->Write(c.data, c.len)) {
        return -1;
      }
    }
    if (!WriteZeros(sink, Pad8(lens[i]) - lens[i])) return -1;
  }
  return (int64_t)meta.size() + body;
}

bool WriteEos(ByteSink* sink) {
  const uint32_t eos[2] = {0xFFFFFFFFu, 0u};
  return sink->Write(eos, 8);
}

}  // namespace gz
