/*
 * Oracle build (test infrastructure only): a C-ABI driver around the reference Splitter,
 * compiled from the reference source tree by oracle/ref/Makefile into oracle/_ref/.
 *
 * It plays the part of the JNI glue (native-sql-engine/cpp/src/jni/jni_wrapper.cc:1031-1227
 * and jni_common.h:308-382): schema from Arrow IPC bytes, key columns as field references,
 * record batches wrapped zero-copy from flat [validity, (offsets), values] buffer lists, a
 * 0-byte validity buffer meaning null_count = 0.  Used by the pinning tests and by the fixture
 * generator; never shipped and never on the product path.
 */
#include <arrow/api.h>
#include <arrow/io/memory.h>
#include <arrow/ipc/api.h>

#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

#include "shuffle/splitter.h"

using sparkcolumnarplugin::shuffle::SplitOptions;
using sparkcolumnarplugin::shuffle::Splitter;

namespace {

struct Handle {
  std::shared_ptr<Splitter> splitter;
  std::shared_ptr<arrow::Schema> schema;
};

void SetErr(const arrow::Status& s, char* err, int errlen) {
  if (err && errlen > 0) {
    std::snprintf(err, errlen, "%s", s.ToString().c_str());
  }
}

// One array of `type` from the flat buffer list at *idx, in the JNI's order (jni_common.h:
// 186-382 MakeArrayData): [validity, (offsets), values] for flat types, [validity, offsets,
// <child buffers>] for list / large_list / map, [validity, <field buffers>] for struct.
// num_rows < 0: taken from the offsets, the first field or the values (a child).
arrow::Status WrapArray(const std::shared_ptr<arrow::DataType>& type, int64_t num_rows,
                        const std::vector<std::shared_ptr<arrow::Buffer>>& bufs, int* idx,
                        std::shared_ptr<arrow::ArrayData>* out) {
  const int n = (int)bufs.size();
  if (type->id() == arrow::Type::NA) {
    if (*idx + 2 > n) return arrow::Status::Invalid("insufficient number of buffers");
    *idx += 2;
    *out = arrow::ArrayData::Make(type, num_rows, {nullptr}, num_rows);
    return arrow::Status::OK();
  }
  std::vector<std::shared_ptr<arrow::Buffer>> ab;
  if (*idx >= n) return arrow::Status::Invalid("insufficient number of buffers");
  int64_t null_count = bufs[*idx]->size() == 0 ? 0 : arrow::kUnknownNullCount;
  ab.push_back(bufs[(*idx)++]);
  if (type->id() == arrow::Type::STRUCT) {  // [validity] then each field's buffers
    std::vector<std::shared_ptr<arrow::ArrayData>> kids;
    for (int k = 0; k < type->num_fields(); k++) {
      std::shared_ptr<arrow::ArrayData> child;
      ARROW_RETURN_NOT_OK(WrapArray(type->field(k)->type(), -1, bufs, idx, &child));
      kids.push_back(std::move(child));
    }
    if (num_rows < 0) num_rows = kids.empty() ? 0 : kids[0]->length;
    *out = arrow::ArrayData::Make(type, num_rows, std::move(ab), std::move(kids), null_count);
    return arrow::Status::OK();
  }
  if (type->id() == arrow::Type::MAP) {  // [validity, offsets] then the entries struct's
    if (*idx >= n) return arrow::Status::Invalid("insufficient number of buffers");
    if (num_rows < 0) num_rows = bufs[*idx]->size() / 4 - 1;
    ab.push_back(bufs[(*idx)++]);
    std::shared_ptr<arrow::ArrayData> child;
    ARROW_RETURN_NOT_OK(WrapArray(type->field(0)->type(), -1, bufs, idx, &child));
    if (child->null_count == arrow::kUnknownNullCount) {  // the entries' validity is dropped
      child->buffers.at(0) = nullptr;
      child->null_count = 0;
    }
    if (child->child_data.size() != 2) return arrow::Status::Invalid("Map array child array should have two fields");
    if (child->child_data[0]->null_count == arrow::kUnknownNullCount &&
        child->child_data[0]->GetNullCount() != 0)
      return arrow::Status::Invalid("Map array keys array should have no nulls");
    *out = arrow::ArrayData::Make(type, num_rows, std::move(ab), {child}, null_count);
    return arrow::Status::OK();
  }
  if (type->id() == arrow::Type::LIST || type->id() == arrow::Type::LARGE_LIST) {
    if (*idx >= n) return arrow::Status::Invalid("insufficient number of buffers");
    const int ow = type->id() == arrow::Type::LIST ? 4 : 8;
    if (num_rows < 0) num_rows = bufs[*idx]->size() / ow - 1;
    ab.push_back(bufs[(*idx)++]);
    std::shared_ptr<arrow::ArrayData> child;
    ARROW_RETURN_NOT_OK(WrapArray(type->field(0)->type(), -1, bufs, idx, &child));
    *out = arrow::ArrayData::Make(type, num_rows, std::move(ab), {child}, null_count);
    return arrow::Status::OK();
  }
  if (arrow::is_binary_like(type->id()) || arrow::is_large_binary_like(type->id())) {
    if (*idx >= n) return arrow::Status::Invalid("insufficient number of buffers");
    const int ow = arrow::is_binary_like(type->id()) ? 4 : 8;
    if (num_rows < 0) num_rows = bufs[*idx]->size() / ow - 1;
    ab.push_back(bufs[(*idx)++]);
  }
  if (*idx >= n) return arrow::Status::Invalid("insufficient number of buffers");
  if (num_rows < 0) {
    const int bw = arrow::bit_width(type->id());
    num_rows = bw > 0 ? bufs[*idx]->size() * 8 / bw : 0;
  }
  ab.push_back(bufs[(*idx)++]);
  *out = arrow::ArrayData::Make(type, num_rows, std::move(ab), null_count);
  return arrow::Status::OK();
}

arrow::Status WrapBatch(const std::shared_ptr<arrow::Schema>& schema, int32_t num_rows,
                        const int64_t* addrs, const int64_t* sizes, int32_t n,
                        std::shared_ptr<arrow::RecordBatch>* out) {
  std::vector<std::shared_ptr<arrow::Buffer>> bufs;
  for (int i = 0; i < n; i++) {
    if (addrs[i] != 0) {
      bufs.push_back(std::make_shared<arrow::Buffer>(
          reinterpret_cast<const uint8_t*>(addrs[i]), sizes[i]));
    } else {
      bufs.push_back(std::make_shared<arrow::Buffer>(nullptr, 0));
    }
  }
  std::vector<std::shared_ptr<arrow::ArrayData>> arrays;
  int idx = 0;
  for (int f = 0; f < schema->num_fields(); f++) {
    std::shared_ptr<arrow::ArrayData> a;
    ARROW_RETURN_NOT_OK(WrapArray(schema->field(f)->type(), num_rows, bufs, &idx, &a));
    arrays.push_back(std::move(a));
  }
  *out = arrow::RecordBatch::Make(schema, num_rows, std::move(arrays));
  return arrow::Status::OK();
}

}  // namespace

extern "C" {

void* gzref_make(const char* short_name, const uint8_t* schema_ipc, int64_t schema_len,
                 int32_t num_partitions,
                 const int32_t* key_cols, int32_t n_keys, int64_t offheap_per_task,
                 int32_t buffer_size, int32_t prefer_spill, int32_t write_schema,
                 const char* data_file, const char* local_dirs, char* err, int errlen) {
  auto buf = std::make_shared<arrow::Buffer>(schema_ipc, schema_len);
  arrow::io::BufferReader reader(buf);
  arrow::ipc::DictionaryMemo memo;
  auto maybe_schema = arrow::ipc::ReadSchema(&reader, &memo);
  if (!maybe_schema.ok()) {
    SetErr(maybe_schema.status(), err, errlen);
    return nullptr;
  }
  auto schema = *maybe_schema;
  if (local_dirs && local_dirs[0]) setenv("NATIVESQL_SPARK_LOCAL_DIRS", local_dirs, 1);

  gandiva::ExpressionVector exprs;
  for (int i = 0; i < n_keys; i++) {
    auto f = schema->field(key_cols[i]);
    exprs.push_back(gandiva::TreeExprBuilder::MakeExpression(
        gandiva::TreeExprBuilder::MakeField(f), f));
  }
  auto opts = SplitOptions::Defaults();
  opts.offheap_per_task = offheap_per_task;
  if (buffer_size > 0) opts.buffer_size = buffer_size;
  opts.prefer_spill = prefer_spill != 0;
  opts.write_schema = write_schema != 0;
  opts.buffered_write = true;
  opts.data_file = data_file ? data_file : "";
  auto maybe = Splitter::Make(short_name ? short_name : "hash", schema, num_partitions, exprs,
                              std::move(opts));
  if (!maybe.ok()) {
    SetErr(maybe.status(), err, errlen);
    return nullptr;
  }
  auto* h = new Handle{*maybe, schema};
  return h;
}

int gzref_split(void* hp, int32_t num_rows, const int64_t* addrs, const int64_t* sizes,
                int32_t n, char* err, int errlen) {
  auto* h = static_cast<Handle*>(hp);
  std::shared_ptr<arrow::RecordBatch> rb;
  auto st = WrapBatch(h->schema, num_rows, addrs, sizes, n, &rb);
  if (st.ok()) st = h->splitter->Split(*rb);
  if (!st.ok()) {
    SetErr(st, err, errlen);
    return 1;
  }
  return 0;
}

int64_t gzref_compressed_size(void* hp, int32_t num_rows, const int64_t* addrs,
                              const int64_t* sizes, int32_t n) {
  auto* h = static_cast<Handle*>(hp);
  std::shared_ptr<arrow::RecordBatch> rb;
  if (!WrapBatch(h->schema, num_rows, addrs, sizes, n, &rb).ok()) return -1;
  return h->splitter->CompressedSize(*rb);
}

/* metrics: [bytes_written, bytes_spilled] */
int gzref_stop(void* hp, int64_t* lengths, int64_t* raw_lengths, int64_t* metrics, char* err,
               int errlen) {
  auto* h = static_cast<Handle*>(hp);
  auto st = h->splitter->Stop();
  if (!st.ok()) {
    SetErr(st, err, errlen);
    return 1;
  }
  const auto& pl = h->splitter->PartitionLengths();
  const auto& rl = h->splitter->RawPartitionLengths();
  for (size_t i = 0; i < pl.size(); i++) {
    lengths[i] = pl[i];
    raw_lengths[i] = rl[i];
  }
  metrics[0] = h->splitter->TotalBytesWritten();
  metrics[1] = h->splitter->TotalBytesSpilled();
  return 0;
}

int gzref_spill(void* hp, int64_t size, int64_t* actual) {
  auto* h = static_cast<Handle*>(hp);
  return h->splitter->SpillFixedSize(size, actual).ok() ? 0 : 1;
}

void gzref_close(void* hp) { delete static_cast<Handle*>(hp); }

}  // extern "C"
