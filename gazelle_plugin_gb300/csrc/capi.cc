// C ABI of the GB300 hash split (include/gz_split.h).
//
// Handles live in a mutex-guarded table with ids starting at 4, like the JNI layer's
// ConcurrentMap (native-sql-engine/cpp/src/jni/concurrent_map.h:35-80).  A call on one handle
// is not synchronised against another call on the same handle: one splitter per task thread,
// as in the reference.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>

#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "../../include/gz_split.h"
#include "hash_static.h"
#include "reader.h"
#include "host_util.h"
#include "schema_ipc.h"
#include "serve.h"
#include "splitter.h"
#include "tune.h"

namespace {

struct Entry {
  std::unique_ptr<gz::Splitter> splitter;
  std::string last_error;
  int64_t server = 0;   // serving loop of a served task (0: called directly)
  int32_t slot = 0;     // its worker
  int64_t reserve = 0;  // HBM budget it holds until it stops
};

// Process-wide tables are never destroyed: handles still open at exit are not torn down by
// static destructors, whose order across files (the pinned pool, the CUDA runtime) is unspecified.
std::mutex& g_mu = *new std::mutex;
std::map<int64_t, std::shared_ptr<Entry>>& g_table = *new std::map<int64_t, std::shared_ptr<Entry>>;
int64_t g_next_id = 4;
thread_local std::string t_make_error;

std::shared_ptr<Entry> Lookup(int64_t id) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(id);
  return it == g_table.end() ? nullptr : it->second;
}

GzStatus Report(Entry* e, const gz::Status& st) {
  if (!st.ok() && e) e->last_error = st.msg;
  return st.code;
}

std::map<int64_t, std::shared_ptr<gz::ServeLoop>>& g_servers = *new std::map<int64_t, std::shared_ptr<gz::ServeLoop>>;

std::shared_ptr<gz::ServeLoop> LookupServer(int64_t id) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_servers.find(id);
  return it == g_servers.end() ? nullptr : it->second;
}

GzStatus MakeCommon(const char* short_name, int32_t num_partitions, std::vector<gz::Field> fields,
                    const int32_t* key_cols, int32_t n_keys, const GzSplitOptions* opts,
                    int64_t* out_handle, std::shared_ptr<Entry>* out_entry = nullptr) {
  if (out_handle == nullptr || short_name == nullptr || (key_cols == nullptr && n_keys > 0)) {
    t_make_error = "null argument";
    return GZ_INVALID;
  }
  GzSplitOptions o;
  if (opts) o = *opts;
  else gz_split_default_options(&o);
  std::vector<int32_t> keys(key_cols, key_cols + (n_keys > 0 ? n_keys : 0));
  std::unique_ptr<gz::Splitter> s;
  gz::Status st = gz::Splitter::Make(short_name, std::move(fields), num_partitions, keys, o, &s);
  if (!st.ok()) {
    t_make_error = "Failed create native shuffle splitter: " + st.msg;
    return st.code;
  }
  auto e = std::make_shared<Entry>();
  e->splitter = std::move(s);
  if (out_entry) *out_entry = e;
  std::lock_guard<std::mutex> lk(g_mu);
  *out_handle = g_next_id++;
  g_table[*out_handle] = e;
  return GZ_OK;
}

struct ReaderEntry {
  std::unique_ptr<gz::PartitionReader> reader;
  std::string last_error;
};
std::map<int64_t, std::shared_ptr<ReaderEntry>>& g_readers = *new std::map<int64_t, std::shared_ptr<ReaderEntry>>;

std::shared_ptr<ReaderEntry> LookupReader(int64_t id) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_readers.find(id);
  if (it == g_readers.end()) {
    t_make_error = "Invalid reader id " + std::to_string(id);
    return nullptr;
  }
  return it->second;
}

GzStatus ReportReader(ReaderEntry* e, const gz::Status& st) {
  if (!st.ok()) {
    e->last_error = st.msg;
    t_make_error = st.msg;
  }
  return st.code;
}

GzStatus MakeReader(std::vector<gz::Field> fields, int32_t device, int64_t* out_handle) {
  std::unique_ptr<gz::PartitionReader> r;
  gz::Status st = gz::PartitionReader::Make(std::move(fields), device, &r);
  if (!st.ok()) {
    t_make_error = "reader: " + st.msg;
    return st.code;
  }
  auto e = std::make_shared<ReaderEntry>();
  e->reader = std::move(r);
  std::lock_guard<std::mutex> lk(g_mu);
  *out_handle = g_next_id++;
  g_readers[*out_handle] = e;
  return GZ_OK;
}

// A GzField tree as the splitter's Field: a map's key and value go under an "entries" struct
// (Arrow's map layout), and a list whose one child is a fixed-width or bool leaf takes the simple
// form (elem) that the schema parser also gives it.
gz::Field FieldFrom(const GzField& g, int depth) {
  gz::Field f;
  f.type = g.type;
  f.nullable = g.nullable != 0;
  f.precision = g.precision;
  f.scale = g.scale;
  f.unit = g.unit;
  f.elem = g.elem_type;
  f.name = g.name ? g.name : "";
  if (g.n_children <= 0 || g.children == nullptr || depth > 16) return f;
  std::vector<gz::Field> kids;
  for (int k = 0; k < g.n_children; k++) kids.push_back(FieldFrom(g.children[k], depth + 1));
  if (f.type == GZ_TYPE_MAP) {
    gz::Field e;
    e.type = GZ_TYPE_STRUCT;
    e.name = "entries";
    e.nullable = false;
    e.children = std::move(kids);
    f.children.push_back(std::move(e));
    return f;
  }
  if (f.type == GZ_TYPE_LIST && kids.size() == 1 && !kids[0].nested() &&
      (kids[0].type == GZ_TYPE_BOOL || (kids[0].type != GZ_TYPE_NULL && kids[0].type < GZ_TYPE_STRING))) {
    const gz::Field& e = kids[0];
    f.elem = e.type;
    f.elem_name = e.name;
    f.elem_nullable = e.nullable;
    f.precision = e.precision;
    f.scale = e.scale;
    f.unit = e.unit;
    return f;
  }
  f.children = std::move(kids);
  return f;
}

std::vector<gz::Field> FieldsFrom(const GzField* fields, int32_t n_fields) {
  std::vector<gz::Field> fs;
  for (int i = 0; i < n_fields; i++) fs.push_back(FieldFrom(fields[i], 0));
  return fs;
}

}  // namespace

extern "C" {

void gz_split_default_options(GzSplitOptions* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->offheap_per_task = 0;
  o->buffer_size = 4096;
  o->num_sub_dirs = 64;
  o->batch_compress_threshold = 256;
  o->compression = 0;
  o->prefer_spill = 1;
  o->write_schema = 1;
  o->buffered_write = 0;
  o->input_kind = GZ_INPUT_HOST;
  o->device = 0;
  o->keep_output_on_device = -1;
  o->flush_bytes = 512ll << 20;
  o->device_budget = 64ll << 30;
  o->data_file = nullptr;
  o->local_dirs = nullptr;
  o->host_budget = 0;
}

GzStatus gz_split_make(const char* short_name, int32_t num_partitions, const uint8_t* schema_ipc,
                       int64_t schema_len, const int32_t* key_cols, int32_t n_keys,
                       const GzSplitOptions* opts, int64_t* out_handle) {
  std::vector<gz::Field> fields;
  std::string err;
  if (!gz::ParseSchemaIpc(schema_ipc, schema_len, &fields, &err)) {
    t_make_error = "Make splitter schema: " + err;
    return err.find("not implemented") != std::string::npos ? GZ_NOT_IMPLEMENTED : GZ_INVALID;
  }
  return MakeCommon(short_name, num_partitions, std::move(fields), key_cols, n_keys, opts, out_handle);
}

GzStatus gz_split_make_fields(const char* short_name, int32_t num_partitions,
                              const GzField* fields, int32_t n_fields, const int32_t* key_cols,
                              int32_t n_keys, const GzSplitOptions* opts, int64_t* out_handle) {
  if (fields == nullptr && n_fields > 0) {
    t_make_error = "Make splitter schema can't be null";
    return GZ_INVALID;
  }
  return MakeCommon(short_name, num_partitions, FieldsFrom(fields, n_fields), key_cols, n_keys, opts, out_handle);
}

GzStatus gz_split_split(int64_t handle, int32_t num_rows, const int64_t* buf_addrs,
                        const int64_t* buf_sizes, int32_t n_bufs, int32_t first_batch,
                        int64_t* out_compressed_size) {
  auto e = Lookup(handle);
  if (!e) {
    t_make_error = "Invalid splitter id " + std::to_string(handle);
    return GZ_INVALID;
  }
  if (buf_addrs == nullptr || buf_sizes == nullptr) {
    e->last_error = "Native split: buf_addrs can't be null";
    return GZ_INVALID;
  }
  if (first_batch) {
    int64_t cs = -1;
    GzStatus s = Report(e.get(), e->splitter->CompressedSize(num_rows, buf_addrs, buf_sizes, n_bufs, &cs));
    if (out_compressed_size) *out_compressed_size = cs;
    return s;
  }
  if (out_compressed_size) *out_compressed_size = -1;
  return Report(e.get(), e->splitter->Split(num_rows, buf_addrs, buf_sizes, n_bufs));
}

GzStatus gz_split_split_batches(int64_t handle, int32_t n_batches, const int32_t* rows,
                                const int64_t* buf_addrs, const int64_t* buf_sizes, int32_t n_bufs) {
  auto e = Lookup(handle);
  if (!e) {
    t_make_error = "Invalid splitter id " + std::to_string(handle);
    return GZ_INVALID;
  }
  if (!rows || !buf_addrs || !buf_sizes) {
    e->last_error = "Native split: null buffer list";
    return GZ_INVALID;
  }
  return Report(e.get(), e->splitter->SplitBatches(n_batches, rows, buf_addrs, buf_sizes, n_bufs));
}

GzStatus gz_split_split_group(int32_t n_tasks, const int64_t* handles, const int32_t* n_batches,
                              const int32_t* rows, const int64_t* buf_addrs, const int64_t* buf_sizes,
                              const int32_t* n_bufs) {
  if (n_tasks < 0 || (n_tasks > 0 && (!handles || !n_batches || !rows || !buf_addrs || !buf_sizes || !n_bufs))) {
    t_make_error = "gz_split_split_group: null argument";
    return GZ_INVALID;
  }
  std::vector<std::shared_ptr<Entry>> es;
  std::vector<gz::Splitter*> ts;
  for (int i = 0; i < n_tasks; i++) {
    auto e = Lookup(handles[i]);
    if (!e) {
      t_make_error = "Invalid splitter id " + std::to_string(handles[i]);
      return GZ_INVALID;
    }
    for (int j = 0; j < i; j++)
      if (handles[j] == handles[i]) {
        t_make_error = "gz_split_split_group: a task appears twice";
        return GZ_INVALID;
      }
    es.push_back(e);
    ts.push_back(e->splitter.get());
  }
  int failed = -1;
  gz::Status st = gz::SplitGroup(ts, n_batches, rows, buf_addrs, buf_sizes, n_bufs, &failed);
  if (!st.ok()) {
    if (failed >= 0) es[failed]->last_error = st.msg;
    t_make_error = "task " + std::to_string(failed) + ": " + st.msg;
  }
  return st.code;
}

GzStatus gz_split_sync_group(int32_t n_tasks, const int64_t* handles) {
  if (n_tasks < 0 || (n_tasks > 0 && !handles)) {
    t_make_error = "gz_split_sync_group: null argument";
    return GZ_INVALID;
  }
  std::vector<std::shared_ptr<Entry>> es;
  std::vector<gz::Splitter*> ts;
  for (int i = 0; i < n_tasks; i++) {
    auto e = Lookup(handles[i]);
    if (!e) {
      t_make_error = "Invalid splitter id " + std::to_string(handles[i]);
      return GZ_INVALID;
    }
    es.push_back(e);
    ts.push_back(e->splitter.get());
  }
  int failed = -1;
  gz::Status st = gz::SyncGroup(ts, &failed);
  if (!st.ok()) {
    if (failed >= 0) es[failed]->last_error = st.msg;
    t_make_error = "task " + std::to_string(failed) + ": " + st.msg;
  }
  return st.code;
}

GzStatus gz_split_sync(int64_t handle) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  return Report(e.get(), e->splitter->Sync());
}

GzStatus gz_split_stop(int64_t handle, GzSplitResult* out) {
  auto e = Lookup(handle);
  if (!e) {
    t_make_error = "Invalid splitter id " + std::to_string(handle);
    return GZ_INVALID;
  }
  // a served task was stopped by its loop; its results are read here
  GzStatus s = (e->server && e->splitter->stopped()) ? GZ_OK : Report(e.get(), e->splitter->Stop());
  if (s != GZ_OK || out == nullptr) return s;
  gz::Splitter& sp = *e->splitter;
  out->total_compute_pid_time = sp.TotalComputePidTime();
  out->total_write_time = sp.TotalWriteTime();
  out->total_spill_time = sp.TotalSpillTime();
  out->total_compress_time = sp.TotalCompressTime();
  out->total_bytes_written = sp.TotalBytesWritten();
  out->total_bytes_spilled = sp.TotalBytesSpilled();
  const auto& pl = sp.PartitionLengths();
  const auto& rl = sp.RawPartitionLengths();
  if (out->partition_lengths) memcpy(out->partition_lengths, pl.data(), pl.size() * sizeof(int64_t));
  if (out->raw_partition_lengths) memcpy(out->raw_partition_lengths, rl.data(), rl.size() * sizeof(int64_t));
  return GZ_OK;
}

GzStatus gz_split_data(int64_t handle, uint8_t* dst, int64_t* out_size) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  const auto& d = e->splitter->DataBytes();
  if (out_size) *out_size = (int64_t)d.size();
  if (dst && !d.empty()) memcpy(dst, d.data(), d.size());
  return GZ_OK;
}

GzStatus gz_split_spill(int64_t handle, int64_t size, int64_t* actual) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  int64_t a = 0;
  GzStatus s = Report(e.get(), e->splitter->SpillFixedSize(size, &a));
  if (actual) *actual = a;
  return s;
}

GzStatus gz_split_set_compress(int64_t handle, int32_t codec) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  return Report(e.get(), e->splitter->SetCompressType(codec));
}

GzStatus gz_split_close(int64_t handle) {
  std::shared_ptr<Entry> e;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find(handle);
    if (it == g_table.end()) return GZ_OK;  // closing twice is harmless, as in the JNI layer
    e = it->second;
    g_table.erase(it);
  }
  if (e->server && e->reserve > 0) {  // a served task closed without stopping
    auto srv = LookupServer(e->server);
    if (srv) srv->Release(e->reserve);
    e->reserve = 0;
  }
  return GZ_OK;
}

GzStatus gz_split_last_pids(int64_t handle, uint16_t* out, int32_t num_rows) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  return Report(e.get(), e->splitter->LastPids(out, num_rows));
}

GzStatus gz_last_error(int64_t handle, char* buf, size_t len) {
  if (!buf || len == 0) return GZ_INVALID;
  std::string msg;
  if (handle == 0) {
    msg = t_make_error;
  } else {
    auto e = Lookup(handle);
    msg = e ? e->last_error : t_make_error;
  }
  snprintf(buf, len, "%s", msg.c_str());
  return GZ_OK;
}

GzStatus gz_split_kernel_times(int64_t handle, double* out4) {
  auto e = Lookup(handle);
  if (!e || !out4) return GZ_INVALID;
  return Report(e.get(), e->splitter->KernelTimes(out4));
}

GzStatus gz_reader_make(const uint8_t* schema_ipc, int64_t schema_len, int32_t device, int64_t* out_handle) {
  std::vector<gz::Field> fields;
  std::string err;
  if (out_handle == nullptr || !gz::ParseSchemaIpc(schema_ipc, schema_len, &fields, &err)) {
    t_make_error = "reader schema: " + (out_handle ? err : std::string("null out_handle"));
    return GZ_INVALID;
  }
  return MakeReader(std::move(fields), device, out_handle);
}

GzStatus gz_reader_make_fields(const GzField* fields, int32_t n_fields, int32_t device, int64_t* out_handle) {
  if (out_handle == nullptr || (fields == nullptr && n_fields > 0)) {
    t_make_error = "reader: null argument";
    return GZ_INVALID;
  }
  return MakeReader(FieldsFrom(fields, n_fields), device, out_handle);
}

GzStatus gz_reader_add_stream(int64_t handle, const uint8_t* stream, int64_t len) {
  auto r = LookupReader(handle);
  if (!r) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->AddStream(stream, len));
}

GzStatus gz_reader_finish(int64_t handle, int64_t* out_rows, int32_t* out_batches) {
  auto r = LookupReader(handle);
  if (!r) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->Finish(out_rows, out_batches));
}

GzStatus gz_reader_column(int64_t handle, int32_t field, GzDeviceColumn* out) {
  auto r = LookupReader(handle);
  if (!r || out == nullptr) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->Column(field, out));
}

GzStatus gz_reader_column_to_host(int64_t handle, int32_t field, uint8_t* validity, void* offsets,
                                  uint8_t* values) {
  auto r = LookupReader(handle);
  if (!r) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->ColumnToHost(field, validity, offsets, values));
}

GzStatus gz_reader_elem_validity_to_host(int64_t handle, int32_t field, uint8_t* out) {
  auto r = LookupReader(handle);
  if (!r) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->ElemValidityToHost(field, out));
}

GzStatus gz_reader_node_count(int64_t handle, int32_t field, int32_t* out_nodes) {
  auto r = LookupReader(handle);
  if (!r || !out_nodes) return GZ_INVALID;
  const int n = r->reader->NodeCount(field);
  if (n <= 0) return ReportReader(r.get(), gz::Status::Error(GZ_INVALID, "field out of range"));
  *out_nodes = n;
  return GZ_OK;
}

GzStatus gz_reader_node(int64_t handle, int32_t field, int32_t node, GzDeviceColumn* out) {
  auto r = LookupReader(handle);
  if (!r || !out) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->Node(field, node, out));
}

GzStatus gz_reader_node_to_host(int64_t handle, int32_t field, int32_t node, uint8_t* validity, void* offsets,
                                uint8_t* values) {
  auto r = LookupReader(handle);
  if (!r) return GZ_INVALID;
  return ReportReader(r.get(), r->reader->NodeToHost(field, node, validity, offsets, values));
}

GzStatus gz_reader_close(int64_t handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_readers.erase(handle);
  return GZ_OK;
}

GzStatus gz_debug_set_spin_limit(int64_t handle, uint32_t polls) {
  auto e = Lookup(handle);
  if (!e) return GZ_INVALID;
  e->splitter->SetSpinLimit(polls);
  return GZ_OK;
}

GzStatus gz_split_stats(int64_t handle, int64_t* out8) {
  auto e = Lookup(handle);
  if (!e || !out8) return GZ_INVALID;
  e->splitter->Stats(out8);
  return GZ_OK;
}

GzStatus gz_split_disk_spill(int64_t handle, int64_t* out3) {
  auto e = Lookup(handle);
  if (!e || !out3) return GZ_INVALID;
  e->splitter->DiskSpillStats(out3);
  return GZ_OK;
}

GzStatus gz_serve_start(int32_t slots, int64_t hbm_budget, int64_t* out_server) {
  if (out_server == nullptr || hbm_budget <= 0) {
    t_make_error = "gz_serve_start: null out_server or non-positive budget";
    return GZ_INVALID;
  }
  auto srv = std::make_shared<gz::ServeLoop>(slots, hbm_budget);
  std::lock_guard<std::mutex> lk(g_mu);
  *out_server = g_next_id++;
  g_servers[*out_server] = srv;
  return GZ_OK;
}

GzStatus gz_serve_open(int64_t server, const char* short_name, int32_t num_partitions, const GzField* fields,
                       int32_t n_fields, const int32_t* key_cols, int32_t n_keys, const GzSplitOptions* opts,
                       int64_t* out_task) {
  auto srv = LookupServer(server);
  if (!srv || out_task == nullptr || (fields == nullptr && n_fields > 0)) {
    t_make_error = "gz_serve_open: invalid server or arguments";
    return GZ_INVALID;
  }
  GzSplitOptions o;
  if (opts) o = *opts;
  else gz_split_default_options(&o);
  // its share of the budget: resident partition data up to the spill threshold, two staging
  // buffers and the pass scratch (a pass size of 0 is the autotuner's choice, else 512 MiB)
  int64_t flush = o.flush_bytes;
  if (flush <= 0) {
    gz::TuneChoice tc;
    const std::vector<int32_t> keys(key_cols, key_cols + (key_cols && n_keys > 0 ? n_keys : 0));
    flush = gz::TuneLookup(gz::SchemaSignature(short_name ? short_name : "", FieldsFrom(fields, n_fields), keys,
                                               num_partitions), &tc)
                ? tc.flush_bytes
                : (512ll << 20);
  }
  flush = std::min<int64_t>(flush, 1ll << 30);
  const int64_t reserve = std::max<int64_t>(o.device_budget, 0) + 3 * flush + (64ll << 20);
  gz::Status st = srv->Admit(reserve);
  if (!st.ok()) {
    t_make_error = "gz_serve_open: " + st.msg;
    return st.code;
  }
  std::shared_ptr<Entry> e;
  GzStatus s = MakeCommon(short_name, num_partitions, FieldsFrom(fields, n_fields), key_cols, n_keys, &o,
                          out_task, &e);
  if (s != GZ_OK) {
    srv->Release(reserve);
    return s;
  }
  e->server = server;
  e->slot = srv->AssignSlot();
  e->reserve = reserve;
  return GZ_OK;
}

GzStatus gz_serve_split(int64_t server, int64_t task, int32_t num_rows, const int64_t* buf_addrs,
                        const int64_t* buf_sizes, int32_t n_bufs, int64_t* out_ticket) {
  auto srv = LookupServer(server);
  auto e = Lookup(task);
  if (!srv || !e || e->server != server || !buf_addrs || !buf_sizes || !out_ticket) {
    t_make_error = "gz_serve_split: invalid server, task or arguments";
    return GZ_INVALID;
  }
  *out_ticket = srv->Submit(e->slot, e->splitter.get(), e, gz::ServeLoop::kSplit, num_rows, buf_addrs, buf_sizes,
                            n_bufs, 0);
  return GZ_OK;
}

GzStatus gz_serve_stop(int64_t server, int64_t task, int64_t* out_ticket) {
  auto srv = LookupServer(server);
  auto e = Lookup(task);
  if (!srv || !e || e->server != server || !out_ticket) {
    t_make_error = "gz_serve_stop: invalid server, task or arguments";
    return GZ_INVALID;
  }
  const int64_t release = e->reserve;
  e->reserve = 0;
  *out_ticket = srv->Submit(e->slot, e->splitter.get(), e, gz::ServeLoop::kStop, 0, nullptr, nullptr, 0, release);
  return GZ_OK;
}

GzStatus gz_serve_sync(int64_t server, int64_t task, int64_t* out_ticket) {
  auto srv = LookupServer(server);
  auto e = Lookup(task);
  if (!srv || !e || e->server != server || !out_ticket) {
    t_make_error = "gz_serve_sync: invalid server, task or arguments";
    return GZ_INVALID;
  }
  *out_ticket = srv->Submit(e->slot, e->splitter.get(), e, gz::ServeLoop::kSync, 0, nullptr, nullptr, 0, 0);
  return GZ_OK;
}

GzStatus gz_serve_wait(int64_t server, int64_t ticket, int64_t* out_latency_ns, int64_t* out_service_ns) {
  auto srv = LookupServer(server);
  if (!srv) {
    t_make_error = "gz_serve_wait: invalid server";
    return GZ_INVALID;
  }
  gz::Status st = srv->Wait(ticket, out_latency_ns, out_service_ns);
  if (!st.ok()) t_make_error = st.msg;
  return st.code;
}

GzStatus gz_autotune(const char* short_name, int32_t num_partitions, const GzField* fields, int32_t n_fields,
                     const int32_t* key_cols, int32_t n_keys, const GzSplitOptions* opts, int32_t n_batches,
                     const int32_t* rows, const int64_t* buf_addrs, const int64_t* buf_sizes, int32_t n_bufs,
                     GzTuneResult* out) {
  if (!short_name || (!fields && n_fields > 0) || n_batches <= 0 || !rows || !buf_addrs || !buf_sizes ||
      n_bufs <= 0 || (!key_cols && n_keys > 0)) {
    t_make_error = "gz_autotune: invalid arguments";
    return GZ_INVALID;
  }
  GzSplitOptions base;
  if (opts) base = *opts;
  else gz_split_default_options(&base);
  base.data_file = nullptr;  // nothing is written: the candidates are never stopped
  const std::vector<gz::Field> fs = FieldsFrom(fields, n_fields);
  const std::vector<int32_t> keys(key_cols, key_cols + (n_keys > 0 ? n_keys : 0));
  int64_t sample = 0;
  for (int64_t i = 0; i < (int64_t)n_batches * n_bufs; i++) sample += std::max<int64_t>(buf_sizes[i], 0);
  int32_t runs = 0;
  // one candidate: made, warmed up once, then timed from the first Split to the end of its device work
  auto measure = [&](int64_t flush, int32_t seg, double* gbs) -> gz::Status {
    GzSplitOptions o = base;
    o.flush_bytes = flush;
    o.seg_tiles = seg;
    for (int rep = 0; rep < 2; rep++) {
      std::unique_ptr<gz::Splitter> sp;
      gz::Status st = gz::Splitter::Make(short_name, fs, num_partitions, keys, o, &sp);
      if (!st.ok()) return st;
      const auto t0 = std::chrono::steady_clock::now();
      st = sp->SplitBatches(n_batches, rows, buf_addrs, buf_sizes, n_bufs);
      if (st.ok()) st = sp->Sync();
      const auto t1 = std::chrono::steady_clock::now();
      if (!st.ok()) return st;
      if (rep == 1) {
        *gbs = (double)sample / std::chrono::duration<double>(t1 - t0).count() / 1e9;
        runs++;
      }
    }
    return gz::Status::OK();
  };
  gz::TuneChoice best;
  double def_gbs = 0;
  gz::Status st;
  // pass sizes 16 MiB .. 1 GiB; once one pass holds the whole sample, larger ones are the same
  double last = 0;
  bool covered = false;
  for (int64_t flush = 16ll << 20; flush <= (1ll << 30) && st.ok(); flush *= 2) {
    double g = last;
    if (!covered) {
      st = measure(flush, 0, &g);
      if (!st.ok()) break;
      if (g > best.gbs) best = gz::TuneChoice{flush, 0, g};
      last = g;
      covered = flush >= sample;
    }
    if (flush == (512ll << 20)) def_gbs = g;
  }
  // segment lengths at the best pass size
  for (int32_t seg : {1, 4, 8, 16, 32}) {
    if (!st.ok()) break;
    double g = 0;
    st = measure(best.flush_bytes, seg, &g);
    if (st.ok() && g > best.gbs) best = gz::TuneChoice{best.flush_bytes, seg, g};
  }
  if (!st.ok()) {
    t_make_error = "gz_autotune: " + st.msg;
    return st.code;
  }
  gz::TuneStore(gz::SchemaSignature(short_name, fs, keys, num_partitions), best);
  if (out) {
    out->flush_bytes = best.flush_bytes;
    out->seg_tiles = best.seg_tiles;
    out->runs = runs;
    out->best_gbs = best.gbs;
    out->default_gbs = def_gbs;
  }
  return GZ_OK;
}

GzStatus gz_tune_save(const char* path) {
  if (!path) return GZ_INVALID;
  gz::Status st = gz::TuneSave(path);
  if (!st.ok()) t_make_error = st.msg;
  return st.code;
}

GzStatus gz_tune_load(const char* path) {
  if (!path) return GZ_INVALID;
  gz::Status st = gz::TuneLoad(path);
  if (!st.ok()) t_make_error = st.msg;
  return st.code;
}

GzStatus gz_pinned_reserve(int64_t bytes, int64_t* out_reserved) {
  const int64_t got = gz::PinnedReserve(bytes, gz::kPinnedSlab);
  if (out_reserved) *out_reserved = got;
  if (got < bytes) {
    t_make_error = "gz_pinned_reserve: pinned host memory ran out after " + std::to_string(got) + " bytes";
    return GZ_OOM;
  }
  return GZ_OK;
}

GzStatus gz_serve_shutdown(int64_t server) {
  std::shared_ptr<gz::ServeLoop> srv;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_servers.find(server);
    if (it == g_servers.end()) return GZ_OK;
    srv = it->second;
    g_servers.erase(it);
  }
  srv.reset();  // finishes queued calls and joins the workers (when no other call holds it)
  return GZ_OK;
}

GzStatus gz_hash_partition_static(int32_t device, int32_t num_partitions, const GzKeyColumn* keys,
                                  int32_t n_keys, int32_t num_rows, uint16_t* d_pids,
                                  int64_t* d_counts, void* stream) {
  std::string msg;
  GzStatus st = gz::HashPartitionStatic(device, num_partitions, keys, n_keys, num_rows, d_pids,
                                        d_counts, static_cast<cudaStream_t>(stream), &msg);
  if (st != GZ_OK) t_make_error = "gz_hash_partition_static: " + msg;
  return st;
}

GzStatus gz_debug_encode_record_batch(int64_t length, const int64_t* nodes, int32_t n_nodes,
                                      const uint8_t* const* bufs, const int64_t* buf_lens,
                                      int32_t n_bufs, uint8_t* out, int64_t out_cap,
                                      int64_t* out_len) {
  std::vector<gz::FieldNodeMeta> nm;
  for (int i = 0; i < n_nodes; i++) nm.push_back(gz::FieldNodeMeta{nodes[2 * i], nodes[2 * i + 1]});
  std::vector<gz::ChunkedBuffer> bb;
  for (int i = 0; i < n_bufs; i++) {
    gz::ChunkedBuffer c;
    if (buf_lens[i] > 0) c.push_back(gz::Chunk{bufs[i], buf_lens[i]});
    bb.push_back(c);
  }
  gz::MemorySink sink;
  int64_t body = 0;
  if (gz::WriteRecordBatchMessage(&sink, length, nm, bb, &body) < 0) return GZ_IO;
  *out_len = (int64_t)sink.buffer().size();
  if (*out_len > out_cap) return GZ_INVALID;
  memcpy(out, sink.buffer().data(), sink.buffer().size());
  return GZ_OK;
}

GzStatus gz_debug_encode_record_batch_lz4_stored(int64_t length, const int64_t* nodes, int32_t n_nodes,
                                                const uint8_t* const* bufs, const int64_t* buf_lens,
                                                int32_t n_bufs, uint8_t* out, int64_t out_cap,
                                                int64_t* out_len) {
  std::vector<gz::FieldNodeMeta> nm;
  for (int i = 0; i < n_nodes; i++) nm.push_back(gz::FieldNodeMeta{nodes[2 * i], nodes[2 * i + 1]});
  std::vector<std::vector<uint8_t>> temps;
  temps.reserve(n_bufs);
  std::vector<std::vector<gz::Chunk>> pieces(n_bufs);
  std::vector<int64_t> lens(n_bufs, 0);
  for (int i = 0; i < n_bufs; i++) {
    if (buf_lens[i] <= 0) continue;  // an empty buffer stays empty
    std::vector<gz::Lz4BlockRef> blocks;
    for (int64_t x = 0; x < buf_lens[i]; x += 65536)
      blocks.push_back(gz::Lz4BlockRef{bufs[i] + x, (uint32_t)std::min<int64_t>(65536, buf_lens[i] - x), true});
    lens[i] = gz::AppendLz4Buffer(buf_lens[i], blocks, &pieces[i], &temps);
  }
  std::vector<uint8_t> meta;
  int64_t body = 0;
  gz::CompressedRecordBatchHeader(length, nm, lens, &meta, &body);
  gz::MemorySink sink;
  sink.Write(meta.data(), (int64_t)meta.size());
  static const uint8_t kZ[8] = {0};
  for (int i = 0; i < n_bufs; i++) {
    for (const gz::Chunk& c : pieces[i]) sink.Write(c.data, c.len);
    sink.Write(kZ, ((lens[i] + 7) & ~int64_t(7)) - lens[i]);
  }
  *out_len = (int64_t)sink.buffer().size();
  if (*out_len > out_cap) return GZ_INVALID;
  memcpy(out, sink.buffer().data(), sink.buffer().size());
  return GZ_OK;
}

GzStatus gz_debug_reencode_schema(const uint8_t* schema_ipc, int64_t len, uint8_t* out, int64_t cap,
                                  int64_t* out_len) {
  std::vector<gz::Field> fields;
  std::string err;
  if (!gz::ParseSchemaIpc(schema_ipc, len, &fields, &err)) {
    t_make_error = err;
    return GZ_INVALID;
  }
  const std::vector<uint8_t> msg = gz::EncodeSchemaMessage(fields);
  *out_len = (int64_t)msg.size();
  if (*out_len > cap) return GZ_INVALID;
  memcpy(out, msg.data(), msg.size());
  return GZ_OK;
}

GzStatus gz_debug_parse_schema(const uint8_t* schema_ipc, int64_t len, int32_t* types,
                               int32_t* nullable, int32_t cap, int32_t* n_fields) {
  std::vector<gz::Field> fields;
  std::string err;
  if (!gz::ParseSchemaIpc(schema_ipc, len, &fields, &err)) {
    t_make_error = err;
    return GZ_INVALID;
  }
  *n_fields = (int32_t)fields.size();
  for (int i = 0; i < (int)fields.size() && i < cap; i++) {
    types[i] = fields[i].type;
    nullable[i] = fields[i].nullable ? 1 : 0;
  }
  return GZ_OK;
}

}  // extern "C"
