// gz::PartitionReader — the reduce side of the shuffle on the GPU: the Arrow IPC streams of one
// partition (one per map output, each the partition's byte range of a data file: optional schema
// message, record batches, end-of-stream) read into one set of Arrow columns in HBM.
//
// The reference's reduce side reads each stream with Arrow Java (ArrowColumnarBatchSerializer,
// native-sql-engine/core/src/main/scala/org/apache/spark/sql/execution/ArrowColumnarBatchSerializer.scala:110-240)
// and decompresses compressed bodies natively (ShuffleDecompressionJniWrapper, jni_wrapper.cc:1236-1322);
// each record batch becomes one ColumnarBatch.  Here the host parses only the metadata; the bodies
// go to HBM in one copy per stream and device kernels concatenate the batches of all streams
// (values and characters copied, offsets rebased, validity bits shifted into place), so the
// consumer gets one batch per partition.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gz_split.h"
#include "gz_engine.cuh"
#include "schema_ipc.h"
#include "splitter.h"  // Status

namespace gz {

class PartitionReader {
 public:
  static Status Make(std::vector<Field> fields, int device, std::unique_ptr<PartitionReader>* out);
  ~PartitionReader();

  // Parses one IPC stream (host bytes, read before the call returns) and copies its bodies to
  // the device.  Streams may carry the schema message first (write_schema) or not.
  Status AddStream(const uint8_t* data, int64_t len);
  // Concatenates every batch added so far into device columns; waits for the device.
  Status Finish(int64_t* rows, int32_t* batches);
  Status Column(int field, GzDeviceColumn* out) const;
  Status ColumnToHost(int field, uint8_t* validity, void* offsets, uint8_t* values);
  Status ElemValidityToHost(int field, uint8_t* out);
  // The nodes of a field in pre-order: 1 for flat fields, 2 for a list of fixed-width or bool
  // elements (the list, its elements), the type tree of a nested field (a map's entries struct
  // between the map and its key / value).
  int NodeCount(int field) const;
  Status Node(int field, int node, GzDeviceColumn* out) const;
  Status NodeToHost(int field, int node, uint8_t* validity, void* offsets, uint8_t* values);

 private:
  struct BufRef {
    int64_t offset = 0;    // inside the stream's device copy, or its decode arena
    int64_t length = 0;
    bool decoded = false;  // a compressed buffer, decoded into the arena
  };
  struct FrameRef {  // one compressed buffer: its LZ4 frame in the stream, its arena range
    int64_t src = 0, src_len = 0, dst = 0, dst_len = 0;
  };
  // one node of a nested field's record batch
  struct NodeRef {
    int64_t length = 0, null_count = 0;
    BufRef validity, offsets, values;
    int64_t o0 = 0, o1 = 0;  // first and last offset (binary: characters; list / map: child entries)
  };
  struct ColRef {
    int64_t null_count = 0;
    BufRef validity, offsets, values;
    int64_t o0 = 0, o1 = 0;  // binary: first and last offset (the batch's characters; list: elements)
    BufRef cvalidity;        // list: element validity
    int64_t child_nulls = 0;
    std::vector<NodeRef> nodes;  // nested field: its nodes in pre-order
  };
  // a nested field's type tree (pre-order)
  struct RNode {
    int type = 0, width = 0, parent = -1;
    std::vector<int> kids;
  };
  struct OutNode {
    int type = 0;
    int64_t length = 0, null_count = 0;
    uint8_t* validity = nullptr;
    uint8_t* offsets = nullptr;
    uint8_t* values = nullptr;
    int64_t values_bytes = 0;
  };
  struct Batch {
    int stream = 0;
    int64_t rows = 0;
    std::vector<ColRef> cols;  // per schema field
  };
  struct OutCol {
    int64_t null_count = 0;
    uint8_t* validity = nullptr;
    uint8_t* offsets = nullptr;  // int32 or int64 (large types) offsets
    uint8_t* values = nullptr;
    int64_t values_bytes = 0;
    uint8_t* child_validity = nullptr;  // list: element validity
    int64_t child_length = 0, child_null_count = 0;
  };

  PartitionReader() = default;
  Status Cuda(cudaError_t e, const char* what);
  Status ParseStream(const uint8_t* data, int64_t len, int stream, std::vector<Batch>* out,
                     std::vector<FrameRef>* frames, int64_t* arena_bytes);
  const uint8_t* Base(const BufRef& r, int stream) const {
    return (r.decoded ? arenas_[stream] : images_[stream]) + r.offset;
  }

  std::vector<Field> fields_;
  std::vector<std::vector<RNode>> tree_;        // per field: its nodes (nested fields only)
  std::vector<std::vector<OutNode>> out_nodes_;  // per field: the concatenated nodes (nested fields)
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  std::vector<uint8_t*> images_;  // device copy of every stream
  std::vector<uint8_t*> arenas_;  // decoded compressed buffers of every stream
  std::vector<uint8_t*> arena_mem_;  // their allocations
  bool direct_ = false;        // the device reads pageable host memory (coherent link)
  HostCopy* jobs_ = nullptr;   // pinned descriptors of the device's reads of a stream
  size_t jobs_bytes_ = 0, jobs_cap_ = 0;
  std::vector<Batch> batches_;
  std::vector<OutCol> out_;
  uint8_t* out_mem_ = nullptr;
  int64_t rows_ = 0;
  bool finished_ = false;
};

}  // namespace gz
