/*
 * gz_task.h — simulated Spark map tasks over the splitter's C ABI (libgztask.so).
 *
 * Not part of the drop-in boundary: this is a caller of it, standing in for the JVM.  Each task
 * runs the loop of ColumnarShuffleWriter.write
 * (native-sql-engine/core/src/main/scala/org/apache/spark/shuffle/ColumnarShuffleWriter.scala:105-188):
 * gz_split_make_fields, one gz_split_split per record batch, gz_split_stop (data file written),
 * gz_split_close.  Tasks run at the same time on their own threads, as an executor's task slots
 * do, each over a contiguous range of the batches.  Used by the benchmark and the tests.
 */
#ifndef GZ_TASK_H
#define GZ_TASK_H

#include <stddef.h>
#include <stdint.h>

#include "gz_split.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GzTaskJob {
  const char* short_name;       /* Splitter::Make short name */
  int32_t num_partitions;
  const GzField* fields;
  int32_t n_fields;
  const int32_t* key_cols;
  int32_t n_keys;
  const GzSplitOptions* opts;   /* NULL: defaults; its data_file is replaced per task */
  const char* data_dir;         /* task t writes <data_dir>/task-<tttt>.data; NULL/"": in memory */
  int32_t n_tasks;
  int32_t n_batches;
  const int32_t* rows;          /* [n_batches] */
  const int64_t* addrs;         /* [n_batches][n_bufs] host buffer addresses */
  const int64_t* sizes;         /* [n_batches][n_bufs] */
  int32_t n_bufs;
  int32_t reserved;
} GzTaskJob;

typedef struct GzTaskResult {
  double wall_s;                /* all tasks released together -> the last task closed */
  double split_s_max;           /* longest split loop of a task */
  double stop_s_max;            /* longest gz_split_stop of a task */
  int64_t input_bytes;          /* sum of the buffer sizes passed to split */
  int64_t raw_partition_bytes;  /* sum of RawPartitionLengths over tasks */
  int64_t bytes_written;        /* sum of TotalBytesWritten over tasks */
  int64_t* partition_lengths;   /* caller array [n_tasks][num_partitions], or NULL */
  char error[512];
} GzTaskResult;

/* Runs the tasks and returns the first failing task's status (GZ_OK when all succeeded). */
int gz_task_run(const GzTaskJob* job, GzTaskResult* out);

/* 64-bit checksum of a file's bytes / of a byte string (tells two data files apart; not
 * cryptographic).  gz_task_digest_file returns 0, or -1 when the file cannot be read. */
int gz_task_digest_file(const char* path, uint64_t* out, int64_t* out_bytes);
uint64_t gz_task_digest(const uint8_t* data, int64_t len);

#ifdef __cplusplus
}
#endif

#endif /* GZ_TASK_H */
