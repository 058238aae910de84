// Simulated Spark map tasks over the splitter's C ABI (there is no JVM here).
//
// Each task runs the writer loop of ColumnarShuffleWriter.write
// (native-sql-engine/core/src/main/scala/org/apache/spark/shuffle/ColumnarShuffleWriter.scala:105-188):
// nativeMake, one split call per record batch on host buffers, stop (the data file written),
// close.  Tasks run on their own threads at the same time, as an executor runs its task slots;
// each task takes a contiguous range of the batches.  Only the public entry points of
// include/gz_split.h are called, exactly as the JNI wrapper would call them.
//
// Built into its own library (libgztask.so), apart from the splitter: it is a caller, used by the
// benchmark and the tests.
#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gz_split.h"
#include "../../include/gz_task.h"

namespace {

double Now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// 64-bit checksum of a byte string: four lanes of multiply / xor-shift over 32-byte blocks, the
// tail zero-padded, the lanes and the length folded together.  Not cryptographic; it tells two
// data files apart.
struct Digest {
  uint64_t h[4] = {0x9e3779b97f4a7c15ull, 0xbf58476d1ce4e5b9ull, 0x94d049bb133111ebull, 0x2545f4914f6cdd1dull};
  uint64_t n = 0;
  uint8_t tail[32];
  int nt = 0;
  static inline uint64_t Mix(uint64_t x, uint64_t w) {
    x = (x ^ w) * 0xff51afd7ed558ccdull;
    return x ^ (x >> 29);
  }
  void Block(const uint8_t* p) {
    uint64_t w[4];
    memcpy(w, p, 32);
    for (int j = 0; j < 4; j++) h[j] = Mix(h[j], w[j]);
  }
  void Update(const uint8_t* p, size_t len) {
    n += len;
    if (nt) {
      const size_t k = std::min<size_t>(32 - nt, len);
      memcpy(tail + nt, p, k);
      nt += (int)k;
      p += k;
      len -= k;
      if (nt < 32) return;
      Block(tail);
      nt = 0;
    }
    for (; len >= 32; p += 32, len -= 32) Block(p);
    memcpy(tail, p, len);
    nt = (int)len;
  }
  uint64_t Final() {
    if (nt) {
      memset(tail + nt, 0, 32 - nt);
      Block(tail);
    }
    uint64_t x = n * 0xc4ceb9fe1a85ec53ull;
    for (int j = 0; j < 4; j++) x = Mix(x + j, h[j]);
    return x;
  }
};

}  // namespace

extern "C" {

int gz_task_digest_file(const char* path, uint64_t* out, int64_t* out_bytes) {
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return -1;
  std::vector<uint8_t> buf(8u << 20);
  Digest d;
  int64_t total = 0;
  for (;;) {
    const ssize_t r = read(fd, buf.data(), buf.size());
    if (r < 0) {
      if (errno == EINTR) continue;
      close(fd);
      return -1;
    }
    if (r == 0) break;
    d.Update(buf.data(), (size_t)r);
    total += r;
  }
  close(fd);
  *out = d.Final();
  if (out_bytes) *out_bytes = total;
  return 0;
}

uint64_t gz_task_digest(const uint8_t* data, int64_t len) {
  Digest d;
  if (len > 0) d.Update(data, (size_t)len);
  return d.Final();
}

int gz_task_run(const GzTaskJob* job, GzTaskResult* out) {
  if (!job || !out || job->n_tasks < 1 || job->n_batches < 0 || (job->n_batches > 0 && (!job->rows || !job->addrs || !job->sizes))) {
    if (out) snprintf(out->error, sizeof(out->error), "gz_task_run: bad arguments");
    return GZ_INVALID;
  }
  const int T = job->n_tasks;
  const int P = job->short_name && strcmp(job->short_name, "single") == 0 ? 1 : job->num_partitions;
  std::vector<double> t_split(T, 0), t_stop(T, 0), t_end(T, 0);
  std::vector<int64_t> raw(T, 0), written(T, 0), in_bytes(T, 0);
  std::vector<int> status(T, GZ_OK);
  std::vector<std::string> err(T);
  std::atomic<int> ready{0};
  std::atomic<bool> go{false};
  double t_go = 0;

  auto task = [&](int t) {
    const int64_t b0 = (int64_t)job->n_batches * t / T, b1 = (int64_t)job->n_batches * (t + 1) / T;
    GzSplitOptions o;
    if (job->opts) o = *job->opts;
    else gz_split_default_options(&o);
    char path[1024] = {0};
    if (job->data_dir && job->data_dir[0]) {
      snprintf(path, sizeof(path), "%s/task-%04d.data", job->data_dir, t);
      o.data_file = path;
    } else {
      o.data_file = nullptr;
    }
    std::vector<int64_t> pl(P), rl(P);
    ready.fetch_add(1);
    while (!go.load(std::memory_order_acquire)) std::this_thread::yield();
    int64_t h = 0;
    int s = gz_split_make_fields(job->short_name, job->num_partitions, job->fields, job->n_fields,
                                 job->key_cols, job->n_keys, &o, &h);
    const double ts = Now();
    for (int64_t b = b0; s == GZ_OK && b < b1; b++) {
      const int64_t* a = job->addrs + b * job->n_bufs;
      const int64_t* z = job->sizes + b * job->n_bufs;
      if (job->rows[b] == 0) continue;  // the writer skips empty batches
      for (int j = 0; j < job->n_bufs; j++) in_bytes[t] += z[j];
      s = gz_split_split(h, job->rows[b], a, z, job->n_bufs, 0, nullptr);
    }
    const double tp = Now();
    GzSplitResult r{};
    r.partition_lengths = pl.data();
    r.raw_partition_lengths = rl.data();
    if (s == GZ_OK) s = gz_split_stop(h, &r);
    const double te = Now();
    if (s != GZ_OK) {
      char buf[512];
      gz_last_error(h, buf, sizeof(buf));
      err[t] = buf;
    } else {
      for (int p = 0; p < P; p++) raw[t] += rl[p];
      written[t] = r.total_bytes_written;
      if (out->partition_lengths)
        memcpy(out->partition_lengths + (size_t)t * P, pl.data(), sizeof(int64_t) * P);
    }
    if (h) gz_split_close(h);
    t_split[t] = tp - ts;
    t_stop[t] = te - tp;
    t_end[t] = Now();
    status[t] = s;
  };

  std::vector<std::thread> th;
  for (int t = 0; t < T; t++) th.emplace_back(task, t);
  while (ready.load() < T) std::this_thread::yield();
  t_go = Now();
  go.store(true, std::memory_order_release);
  for (auto& x : th) x.join();

  out->wall_s = 0;
  out->split_s_max = out->stop_s_max = 0;
  out->input_bytes = out->raw_partition_bytes = out->bytes_written = 0;
  int rc = GZ_OK;
  for (int t = 0; t < T; t++) {
    out->wall_s = std::max(out->wall_s, t_end[t] - t_go);
    out->split_s_max = std::max(out->split_s_max, t_split[t]);
    out->stop_s_max = std::max(out->stop_s_max, t_stop[t]);
    out->input_bytes += in_bytes[t];
    out->raw_partition_bytes += raw[t];
    out->bytes_written += written[t];
    if (status[t] != GZ_OK && rc == GZ_OK) {
      rc = status[t];
      snprintf(out->error, sizeof(out->error), "task %d: %s", t, err[t].c_str());
    }
  }
  return rc;
}

}  // extern "C"
