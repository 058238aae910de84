// Arrow IPC framing of emitted partition batches, byte-identical to the Arrow C++ writer
// the reference uses (arrow::ipc::GetRecordBatchPayload + WriteIpcPayload, called from
// CacheRecordBatch / PartitionWriter, native-sql-engine/cpp/src/shuffle/splitter.cc:153-172,
// 585-604), with no codec and metadata version V5.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace gz {

// One body buffer as a list of byte chunks that are concatenated (a buffer assembled from
// several flush pieces).  An empty list is an empty (placeholder) buffer.
struct Chunk {
  const uint8_t* data;  // nullptr with len > 0 means `len` zero bytes
  int64_t len;
  bool dev = false;     // `data` is device memory (or pinned host memory the device reads)
};
using ChunkedBuffer = std::vector<Chunk>;

struct FieldNodeMeta {
  int64_t length;
  int64_t null_count;
};

// Sink for the data-file bytes (memory or a buffered file).
class ByteSink {
 public:
  virtual ~ByteSink() = default;
  virtual bool Write(const void* p, int64_t n) = 0;
  virtual int64_t Tell() const = 0;
};

class MemorySink : public ByteSink {
 public:
  bool Write(const void* p, int64_t n) override;
  int64_t Tell() const override { return (int64_t)buf_.size(); }
  std::vector<uint8_t>& buffer() { return buf_; }

 private:
  std::vector<uint8_t> buf_;
};

class FileSink : public ByteSink {
 public:
  explicit FileSink(const std::string& path);
  ~FileSink() override;
  bool ok() const { return f_ != nullptr; }
  bool Write(const void* p, int64_t n) override;
  int64_t Tell() const override { return pos_; }
  bool Close();

 private:
  bool FlushBuf();
  void* f_ = nullptr;
  std::vector<uint8_t> buf_;
  int64_t pos_ = 0;
};

// Writes one encapsulated RecordBatch message (continuation token, metadata length, the
// flatbuffer Message, 8-byte padded body).  Returns the message bytes written; *body_length
// receives the padded body size (IpcPayload::body_length).  Requires length > 0 and at least
// one non-empty body buffer.
int64_t WriteRecordBatchMessage(ByteSink* sink, int64_t length,
                                const std::vector<FieldNodeMeta>& nodes,
                                const std::vector<ChunkedBuffer>& buffers, int64_t* body_length);

// The metadata of that message (continuation token, metadata length, flatbuffer) for body
// buffers of lengths `lens`; the body follows it, each buffer padded to 8 bytes.
void RecordBatchHeader(int64_t length, const std::vector<FieldNodeMeta>& nodes,
                       const std::vector<int64_t>& lens, std::vector<uint8_t>* out,
                       int64_t* body_length);

// The same for a message whose body buffers are compressed (RecordBatch.compression set to
// LZ4_FRAME / BUFFER); `lens` are the compressed buffer lengths (uncompressed-length prefix
// included).
void CompressedRecordBatchHeader(int64_t length, const std::vector<FieldNodeMeta>& nodes,
                                 const std::vector<int64_t>& lens, std::vector<uint8_t>* out,
                                 int64_t* body_length);

// LZ4 frame format: magic, FLG (version 1, independent blocks, no checksums, no content size),
// BD (64 KiB blocks) and the header checksum byte of those two descriptor bytes.
constexpr uint8_t kLz4Flg = 0x60, kLz4Bd = 0x40;
uint8_t Lz4FrameHeaderChecksum(const uint8_t* desc, int n);

// One block of an LZ4 frame: `size` payload bytes at `data`; `stored`: the payload is the data
// itself (no LZ4 sequences).
struct Lz4BlockRef {
  const uint8_t* data;
  uint32_t size;
  bool stored;
};

// Appends the bytes of one compressed IPC body buffer to `pieces`: the int64 uncompressed length,
// then one LZ4 frame (header, the blocks with their size words, end mark).  The small byte
// strings around the payloads are kept in a new element of `temps`.  Returns the bytes appended.
int64_t AppendLz4Buffer(int64_t uncompressed_len, const std::vector<Lz4BlockRef>& blocks,
                        std::vector<Chunk>* pieces, std::vector<std::vector<uint8_t>>* temps);

// Size of that message without writing it.
int64_t RecordBatchMessageSize(int64_t n_nodes, const std::vector<int64_t>& buffer_lengths,
                               int64_t* body_length);

// The end-of-stream marker {0xFFFFFFFF, 0} (splitter.cc:166-172).
bool WriteEos(ByteSink* sink);

}  // namespace gz
