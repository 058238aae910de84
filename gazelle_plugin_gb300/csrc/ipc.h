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

// Size of that message without writing it.
int64_t RecordBatchMessageSize(int64_t n_nodes, const std::vector<int64_t>& buffer_lengths,
                               int64_t* body_length);

// The end-of-stream marker {0xFFFFFFFF, 0} (splitter.cc:166-172).
bool WriteEos(ByteSink* sink);

}  // namespace gz
