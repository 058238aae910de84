/*
 * gz_split.h — C ABI of the GB300 columnar shuffle hash split.
 *
 * A drop-in for Gazelle's native shuffle splitter boundary: each entry point replaces one
 * JNI method of com.intel.oap.vectorized.ShuffleSplitterJniWrapper, implemented in
 * native-sql-engine/cpp/src/jni/jni_wrapper.cc, over the C++ Splitter of
 * native-sql-engine/cpp/src/shuffle/splitter.h.  Plain pointers and sizes only.
 *
 * Errors: every call returns a GzStatus; gz_last_error() gives the message of the last
 * failing call on a handle (or of the last failing gz_split_make on this thread when
 * handle == 0).  Device-side work is asynchronous: a CUDA failure surfaces on the next
 * call on the same handle, and at the latest from gz_split_stop.
 */
#ifndef GZ_SPLIT_H
#define GZ_SPLIT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum GzStatus {
  GZ_OK = 0,
  GZ_INVALID = 1,          /* bad argument / id: the JNI layer throws (jni_wrapper.cc:1160-1163) */
  GZ_OOM = 2,              /* arrow::Status::OutOfMemory */
  GZ_IO = 3,               /* data / spill file errors */
  GZ_NOT_IMPLEMENTED = 4,  /* arrow::Status::NotImplemented (types, codecs, partitioners) */
  GZ_TIMEOUT = 5,          /* a bounded device-side wait gave up */
  GZ_CUDA = 6              /* a CUDA runtime error */
} GzStatus;

/* Arrow field types accepted by the splitter (utils.h:116-158 ToSplitterTypeId subset). */
typedef enum GzType {
  GZ_TYPE_NULL = 0, GZ_TYPE_BOOL = 1, GZ_TYPE_INT8 = 2, GZ_TYPE_UINT8 = 3,
  GZ_TYPE_INT16 = 4, GZ_TYPE_UINT16 = 5, GZ_TYPE_HALF_FLOAT = 6, GZ_TYPE_INT32 = 7,
  GZ_TYPE_UINT32 = 8, GZ_TYPE_FLOAT32 = 9, GZ_TYPE_DATE32 = 10, GZ_TYPE_TIME32 = 11,
  GZ_TYPE_INT64 = 12, GZ_TYPE_UINT64 = 13, GZ_TYPE_FLOAT64 = 14, GZ_TYPE_DATE64 = 15,
  GZ_TYPE_TIME64 = 16, GZ_TYPE_TIMESTAMP = 17, GZ_TYPE_DECIMAL128 = 18,
  GZ_TYPE_STRING = 19, GZ_TYPE_BINARY = 20,
  /* 64-bit offsets (SplitBinaryType<LargeBinaryType::offset_type>, splitter.cc:1291-1299):
   * payload columns only; one batch's column may hold at most 2^31 - 1 character bytes */
  GZ_TYPE_LARGE_STRING = 21, GZ_TYPE_LARGE_BINARY = 22,
  /* list (SplitListArray / AppendList, splitter.cc:1322-1344; payload columns only): of
   * fixed-width or bool elements given by GzField.elem_type, buffers [validity, int32 offsets,
   * element validity, element values]; or with one child field of any type */
  GZ_TYPE_LIST = 23,
  /* nested payload columns with child fields (jni_common.h:186-300 reads their buffers depth
   * first: [validity, (offsets)] then each child's): large_list (int64 offsets; one child),
   * struct (its fields), map (two children, key and value; the entries struct between them takes
   * one buffer entry, its validity, which is ignored) */
  GZ_TYPE_LARGE_LIST = 24, GZ_TYPE_STRUCT = 25, GZ_TYPE_MAP = 26
} GzType;

/* One schema field.  `unit`: time/timestamp unit (0 s, 1 ms, 2 us, 3 ns); `precision` /
 * `scale`: decimal128.  Only used when writing the schema message (write_schema). */
typedef struct GzField {
  int32_t type;       /* GzType */
  int32_t nullable;
  int32_t precision;
  int32_t scale;
  int32_t unit;
  int32_t elem_type;  /* GZ_TYPE_LIST without children: the element type (fixed width or bool;
                         precision / scale / unit then describe the element, named "item" and
                         nullable) */
  const char* name;
  int32_t n_children;              /* nested types: child fields (a map: key, then value) */
  const struct GzField* children;
} GzField;

/* Codec of the emitted record batches (the JNI's codec strings "uncompressed", "lz4",
 * "fastpfor"; GetCompressionType in jni_wrapper.cc).  Batches of at most
 * batch_compress_threshold rows are written uncompressed (splitter.cc:586-600). */
typedef enum GzCodec {
  GZ_CODEC_UNCOMPRESSED = 0,
  GZ_CODEC_LZ4_FRAME = 1,  /* Arrow IPC body compression: int64 length + one LZ4 frame per buffer */
  GZ_CODEC_FASTPFOR = 2    /* not implemented */
} GzCodec;

/* Where Split reads its buffers from. */
typedef enum GzInputKind {
  GZ_INPUT_HOST = 0,            /* host memory, borrowed for the call (the JNI contract) */
  GZ_INPUT_DEVICE_RETAINED = 1  /* device memory the caller keeps valid and unchanged
                                   until gz_split_stop returns (resident inputs) */
} GzInputKind;

/* How host inputs (GZ_INPUT_HOST) reach the device before gz_split_split returns. */
typedef enum GzHostRead {
  GZ_HOST_READ_AUTO = 0,     /* the GPU reads the caller's buffers itself when it can walk the
                                host page tables (coherent CPU-GPU link), else as CPU_COPY */
  GZ_HOST_READ_CPU_COPY = 1  /* CPU copy into pinned staging, then one copy per device pass */
} GzHostRead;

/* SplitOptions (native-sql-engine/cpp/src/shuffle/type.h:39-59) plus device knobs.
 * Initialise with gz_split_default_options(). */
typedef struct GzSplitOptions {
  int64_t offheap_per_task;          /* 0: partition buffers hold buffer_size rows */
  int32_t buffer_size;               /* rows per partition buffer, <= 32768 (default 4096) */
  int32_t num_sub_dirs;              /* spill sub-directories (default 64) */
  int32_t batch_compress_threshold;  /* default 256; compression itself is off */
  int32_t compression;               /* GzCodec (default GZ_CODEC_UNCOMPRESSED) */
  int32_t prefer_spill;              /* default 1 */
  int32_t write_schema;              /* default 1: schema message before each partition */
  int32_t buffered_write;            /* accepted for compatibility */
  int32_t input_kind;                /* GzInputKind, default GZ_INPUT_HOST */
  int32_t device;                    /* CUDA device ordinal, default 0 */
  int32_t keep_output_on_device;     /* 1: partition data stays in HBM until Stop or until
                                        device_budget is exceeded; 0: every device pass's
                                        partition data is copied to pinned host memory as soon
                                        as the pass is done; -1 (default): 0 for host inputs,
                                        1 for device-retained inputs */
  int64_t flush_bytes;               /* input bytes gathered before one device pass
                                        (default 512 MiB, at most 1 GiB; 0: the choice
                                        gz_autotune cached for this schema, else 512 MiB) */
  int64_t device_budget;             /* HBM bytes for resident partition data before it is
                                        moved to pinned host memory (default 64 GiB) */
  const char* data_file;             /* written at Stop; NULL/"" keeps the bytes in memory */
  const char* local_dirs;            /* comma separated spill dirs (the executor's local dirs):
                                        partition data past host_budget goes to temp_shuffle_*
                                        files in their num_sub_dirs sub-directories */
  int32_t host_read;                 /* GzHostRead, default GZ_HOST_READ_AUTO */
  int32_t seg_tiles;                 /* 1024-row tiles per k_hash_count segment, 1..32;
                                        0 (default): the gz_autotune choice for this schema,
                                        else 4..32 growing with num_partitions */
  int64_t host_budget;               /* pinned host bytes of partition data a splitter keeps
                                        before its oldest passes move to files under local_dirs
                                        (read back through a mapping at Stop, deleted after it);
                                        0 (default): no limit */
} GzSplitOptions;

/* SplitResult (native-sql-engine/core/src/main/java/com/intel/oap/vectorized/SplitResult.java:21-39).
 * partition_lengths / raw_partition_lengths are caller arrays of num_partitions int64. */
typedef struct GzSplitResult {
  int64_t total_compute_pid_time;  /* ns */
  int64_t total_write_time;        /* ns */
  int64_t total_spill_time;        /* ns */
  int64_t total_compress_time;     /* ns */
  int64_t total_bytes_written;
  int64_t total_bytes_spilled;
  int64_t* partition_lengths;
  int64_t* raw_partition_lengths;
} GzSplitResult;

/* Fills `opts` with the reference defaults (SplitOptions::Defaults, type.h:39-59). */
void gz_split_default_options(GzSplitOptions* opts);

/* Replaces ShuffleSplitterJniWrapper.nativeMake (jni_wrapper.cc:1031-1134).
 * `short_name` (Splitter::Make, splitter.cc:190-208): "hash" (by `key_cols`), "rr"
 * (round-robin, the selection carried from batch to batch), "single" (one partition, whatever
 * `num_partitions` says; Stop fills one length), "range" (FallbackRangeSplitter: schema field 0
 * holds int32 partition ids, left out of the output; an id < 0 or >= num_partitions fails the
 * split with GZ_INVALID, reported by the next synchronising call); "rr", "single" and "range"
 * ignore `key_cols`.  Any other name returns GZ_NOT_IMPLEMENTED.
 * `schema_ipc`: Arrow IPC encapsulated Schema message (what MakeSchema reads,
 * jni_common.h:393-406).  `key_cols`: schema indices of the hash keys, in order; they stand
 * for the gandiva field-reference expressions (ColumnarShuffleExchangeExec.scala:307-326). */
GzStatus gz_split_make(const char* short_name, int32_t num_partitions, const uint8_t* schema_ipc,
                       int64_t schema_len, const int32_t* key_cols, int32_t n_keys,
                       const GzSplitOptions* opts, int64_t* out_handle);

/* Same as gz_split_make with the schema given as a field array instead of IPC bytes. */
GzStatus gz_split_make_fields(const char* short_name, int32_t num_partitions,
                              const GzField* fields, int32_t n_fields, const int32_t* key_cols,
                              int32_t n_keys, const GzSplitOptions* opts, int64_t* out_handle);

/* Replaces ShuffleSplitterJniWrapper.split (jni_wrapper.cc:1156-1195).
 * Buffers: flat list in schema order, [validity, (offsets), values] per non-null field; a
 * zero address or size means an empty buffer, an empty validity buffer means no nulls
 * (jni_common.h:308-382).  With first_batch != 0 the batch is not split and
 * *out_compressed_size receives its IPC body length (Splitter::CompressedSize,
 * splitter.cc:358-369); otherwise *out_compressed_size = -1.  Host inputs are fully read
 * before the call returns. */
GzStatus gz_split_split(int64_t handle, int32_t num_rows, const int64_t* buf_addrs,
                        const int64_t* buf_sizes, int32_t n_bufs, int32_t first_batch,
                        int64_t* out_compressed_size);

/* Calls gz_split_split(handle, rows[i], addrs + i * n_bufs, sizes + i * n_bufs, n_bufs, 0,
 * NULL) for i = 0 .. n_batches-1 (the writer's per-batch loop, ColumnarShuffleWriter.scala:131-185,
 * run inside the library); stops at the first error.  No reference counterpart. */
GzStatus gz_split_split_batches(int64_t handle, int32_t n_batches, const int32_t* rows,
                                const int64_t* buf_addrs, const int64_t* buf_sizes, int32_t n_bufs);

/* gz_split_split_batches for several tasks (different splitters, schemas and partition counts)
 * in one call: task i (handles[i]) gets n_batches[i] batches of n_bufs[i] buffers; the rows,
 * addresses and sizes of the tasks follow one another in `rows`, `buf_addrs`, `buf_sizes`.  All
 * tasks' host reads are started before any is waited for, so they are in flight together; host
 * inputs are read when the call returns.  Errors: gz_last_error(0, ...) names the failing task.
 * No reference counterpart (the batched form's window of calls). */
GzStatus gz_split_split_group(int32_t n_tasks, const int64_t* handles, const int32_t* n_batches,
                              const int32_t* rows, const int64_t* buf_addrs, const int64_t* buf_sizes,
                              const int32_t* n_bufs);

/* Runs the device pass over the batches gathered so far and waits for all device work of
 * this handle: afterwards every split batch is in its partition buffers, as after a
 * reference Split call returns.  No reference counterpart (reference Split is synchronous). */
GzStatus gz_split_sync(int64_t handle);
/* gz_split_sync of several tasks: every task's pending device pass is queued before any task is
 * waited for (their last passes and copies back overlap). */
GzStatus gz_split_sync_group(int32_t n_tasks, const int64_t* handles);

/* Replaces ShuffleSplitterJniWrapper.stop (jni_wrapper.cc:1197-1227): emits every pending
 * partition buffer, writes the data file (or keeps it in memory) and fills `out`. */
GzStatus gz_split_stop(int64_t handle, GzSplitResult* out);

/* Size of the data-file bytes produced by Stop; with `dst` non-NULL also copies them
 * (tests and in-memory callers). */
GzStatus gz_split_data(int64_t handle, uint8_t* dst, int64_t* out_size);

/* Replaces ShuffleSplitterJniWrapper.nativeSpill (jni_wrapper.cc:984-999 -> SpillFixedSize,
 * splitter.cc:741-756).  *actual = bytes the reference policy would release. */
GzStatus gz_split_spill(int64_t handle, int64_t size, int64_t* actual);

/* Replaces ShuffleSplitterJniWrapper.setCompressType (jni_wrapper.cc:1136-1154): GzCodec
 * UNCOMPRESSED or LZ4_FRAME (FASTPFOR is GZ_NOT_IMPLEMENTED).  Record batches are encoded at
 * Stop, so the codec set last applies to every batch of the split. */
GzStatus gz_split_set_compress(int64_t handle, int32_t codec);

/* Replaces ShuffleSplitterJniWrapper.close (jni_wrapper.cc:1229-1234). */
GzStatus gz_split_close(int64_t handle);

/* Partition ids of the rows of the most recent gz_split_split call (one uint16 per row,
 * Spark pmod of the Murmur3 chain).  Test hook; forces the pending device work to finish. */
GzStatus gz_split_last_pids(int64_t handle, uint16_t* out, int32_t num_rows);

/* Message of the last error on `handle` (0: the calling thread's last make error). */
GzStatus gz_last_error(int64_t handle, char* buf, size_t len);

/* Device time (ms, CUDA events on the stream each family runs on) spent in each kernel family
 * since make: [hash+count, plan+scan, scatter, total device].  The families of neighbouring
 * passes run at the same time, so an event span can include other families' work.  Test /
 * bench hook. */
GzStatus gz_split_kernel_times(int64_t handle, double* out4);

/* Counters of this handle: [0] device passes, [1] input bytes gathered, [2] bytes copied
 * host-to-device, [3] partition bytes copied device-to-host, [4] partition bytes resident in
 * HBM, [5] batches split, [6] rows split, [7] emitted record batches (after Stop, else -1).
 * No reference counterpart. */
GzStatus gz_split_stats(int64_t handle, int64_t* out8);

/* Local-dir spill files of this handle (host_budget): [0] files written, [1] their bytes,
 * [2] files present now (they are deleted once Stop has read them).  No reference counterpart. */
GzStatus gz_split_disk_spill(int64_t handle, int64_t* out3);

/* ---- Autotuner (no reference counterpart) ---------------------------------------------
 * The device pass has two run-time knobs: flush_bytes (its size) and seg_tiles (the segment
 * length of k_hash_count and the plan).  gz_autotune splits the sample batches with candidate
 * settings (opts otherwise as given; each candidate once to warm up, once timed from the first
 * Split to the end of the device work) and caches the fastest under the schema's signature
 * (field types, key columns, num_partitions).  Splitters made later in the process with
 * flush_bytes 0 / seg_tiles 0 take the cached choice.  gz_tune_save / gz_tune_load write / merge
 * the cache as a text file; $GZ_TUNE_CACHE, when set, is loaded on first use.  Tile size, rows
 * per warp and staging depth of k_scatter are compile-time constants, not tuned. */
typedef struct GzTuneResult {
  int64_t flush_bytes;  /* chosen pass size */
  int32_t seg_tiles;    /* chosen segment length */
  int32_t runs;         /* timed candidate runs */
  double best_gbs;      /* sample input GB/s at the chosen settings */
  double default_gbs;   /* sample input GB/s at 512 MiB passes and automatic segments */
} GzTuneResult;

GzStatus gz_autotune(const char* short_name, int32_t num_partitions, const GzField* fields,
                     int32_t n_fields, const int32_t* key_cols, int32_t n_keys,
                     const GzSplitOptions* opts, int32_t n_batches, const int32_t* rows,
                     const int64_t* buf_addrs, const int64_t* buf_sizes, int32_t n_bufs,
                     GzTuneResult* out);
GzStatus gz_tune_save(const char* path);
GzStatus gz_tune_load(const char* path);

/* ---- served form (no reference counterpart) --------------------------------------------
 * Split / Stop calls of many concurrent tasks, each an ordinary splitter with its own schema,
 * batch sizes and partition count, executed by one serving loop on one GPU.  Each task is
 * pinned to one of `slots` workers: its calls run in order, calls of tasks on other workers run
 * at the same time and their device work overlaps.  A task is admitted when its share of
 * `hbm_budget` is free: its spill threshold (opts.device_budget: partition data kept in HBM
 * before it moves to pinned host memory) + 3 * opts.flush_bytes + 64 MiB; it returns the share
 * when it stops or closes.  Calls are asynchronous: each returns a ticket; gz_serve_wait gives
 * the call's status and its latency from submission to completion (host inputs read, batch
 * queued for the device; for a stop, the data file written).  Buffers passed to gz_serve_split
 * stay valid until its ticket completes.  After the stop ticket completes, gz_split_stop(task)
 * fills the SplitResult and gz_split_data(task) gives the bytes; gz_split_close(task) frees the
 * task.  A served task must not be called directly (gz_split_split) while it is served.  Errors
 * of these calls: gz_last_error(0, ...) on the calling thread. */

/* Starts a serving loop with `slots` workers and an HBM budget in bytes. */
GzStatus gz_serve_start(int32_t slots, int64_t hbm_budget, int64_t* out_server);

/* Opens a task (gz_split_make_fields arguments); blocks until the budget admits it.  The task id
 * is a splitter handle. */
GzStatus gz_serve_open(int64_t server, const char* short_name, int32_t num_partitions,
                       const GzField* fields, int32_t n_fields, const int32_t* key_cols,
                       int32_t n_keys, const GzSplitOptions* opts, int64_t* out_task);

/* Queues one Split call of `task` (gz_split_split arguments, first_batch = 0). */
GzStatus gz_serve_split(int64_t server, int64_t task, int32_t num_rows, const int64_t* buf_addrs,
                        const int64_t* buf_sizes, int32_t n_bufs, int64_t* out_ticket);

/* Queues the Stop of `task`, after its queued splits. */
GzStatus gz_serve_stop(int64_t server, int64_t task, int64_t* out_ticket);

/* Queues a wait for all device work of `task` so far (gz_split_sync), after its queued calls. */
GzStatus gz_serve_sync(int64_t server, int64_t task, int64_t* out_ticket);

/* Waits for a ticket: the call's status; *out_latency_ns = submission to completion,
 * *out_service_ns = the part its worker spent on it (the rest queued).  Either may be NULL. */
GzStatus gz_serve_wait(int64_t server, int64_t ticket, int64_t* out_latency_ns,
                       int64_t* out_service_ns);

/* Adds about `bytes` of pinned host memory to the library's pool up front, in the chunks that
 * partition data moved out of HBM is carved from.  Pinning is slow; a server calls this at
 * start so that spills inside calls do not pay it.  *out_reserved = bytes added. */
GzStatus gz_pinned_reserve(int64_t bytes, int64_t* out_reserved);

/* Finishes the queued calls and stops the workers. */
GzStatus gz_serve_shutdown(int64_t server);

/* ---- partition ids without device allocation (no counterpart in the reference) -------- */

/* One hash-key column of a batch that is already in device memory. */
typedef struct GzKeyColumn {
  int32_t type;             /* GzType: BOOL, INT8, INT16, INT32, FLOAT32, DATE32, INT64, FLOAT64;
                               NULL: a null-type key, which leaves the hash unchanged */
  int32_t reserved;
  const uint8_t* validity;  /* device address of the validity bitmap (LSB first); NULL: no nulls */
  const uint8_t* values;    /* device address of the values (bit-packed for BOOL) */
} GzKeyColumn;

/* Partition id of every row (one uint16 each, into d_pids) and the row count of every
 * partition (num_partitions int64, into d_counts) of one batch whose hash keys are already on
 * device `device`, with the splitter's Spark hash: Murmur3 chained from seed 42 over the keys in
 * order, a null key passing the seed through, pid = pmod(hash, num_partitions).  Has no
 * counterpart in the reference.
 *
 * It allocates no device memory, for callers that cannot call cudaMalloc: processes whose
 * device memory all belongs to another allocator (a pool that reserved the free HBM up front,
 * or an executor that charges every device byte to a task's memory budget, which a hidden
 * cudaMalloc would escape), and code that must not stall the device, as cudaMalloc and
 * cudaFree may synchronise it.  Inputs and outputs are the caller's device memory.
 *
 * Its scratch, the per-tile row counts, is one 16 MiB array in the library's own device
 * memory, held until the process exits on every device where the library has run.  With CUDA's
 * lazy module loading (the default) the array is reserved on a device by the first call there,
 * so make that first call (a zero-row call will do) before a pool reserves the device's free
 * memory; if it cannot be reserved the call returns GZ_OOM.  A call needs
 * ceil(num_rows / 1024) * num_partitions 32-bit counters, at most 4,194,304 (e.g. 65,536 rows
 * at 65,536 partitions, or 21 million rows at 200); a larger call returns GZ_INVALID.  All calls
 * on a device share the array and it keeps the last call's contents (each call clears what it
 * uses), so calls that may overlap on the GPU (other streams, other threads) race and give
 * wrong counts: put them on one stream.  The first call on a device looks up the array's device
 * address with that device current; make that first call before any stream capture.  Only the
 * device's primary context (the CUDA runtime's) is supported.  A CUDA error already pending on
 * the calling thread is reported as GZ_CUDA before anything is launched and is left pending.
 *
 * The work is enqueued on `stream` (a cudaStream_t of that device, NULL: its default stream)
 * and the call returns without waiting; the calling thread's current device is left as it
 * was.  On error, gz_last_error(0, ...) on the same thread gives the message. */
GzStatus gz_hash_partition_static(int32_t device, int32_t num_partitions, const GzKeyColumn* keys,
                                  int32_t n_keys, int32_t num_rows, uint16_t* d_pids,
                                  int64_t* d_counts, void* stream);

/* ---- reduce-side read (replaces the reference's read of a partition's shuffle blocks) ---
 * The reference reads each map output's bytes of a partition with Arrow Java
 * (ArrowColumnarBatchSerializer.scala:110-240: an IPC stream reader, one ColumnarBatch per
 * record batch) and decompresses compressed bodies through ShuffleDecompressionJniWrapper
 * (jni_wrapper.cc:1236-1322).  Here the streams of one partition are read into HBM: the host
 * parses the IPC metadata, the bodies go to the device in one copy per stream, and device
 * kernels concatenate the record batches of all streams into one set of Arrow columns (values
 * and characters copied, offsets rebased, validity bits moved to their rows).  The result stays
 * in device memory owned by the reader until gz_reader_close. */

/* One column of the concatenated partition, in device memory. */
typedef struct GzDeviceColumn {
  int32_t type;            /* GzType */
  int32_t reserved;
  int64_t length;          /* rows */
  int64_t null_count;
  const uint8_t* validity; /* LSB-first bitmap, (length + 7) / 8 bytes; NULL: no nulls */
  const void* offsets;     /* binary / utf8: length + 1 int32 offsets from 0 (int64 for the large
                            * types); NULL otherwise */
  const uint8_t* values;   /* fixed width: length * width bytes; bool: bitmap; binary: characters;
                            * list: the element values */
  int64_t values_bytes;
  const uint8_t* child_validity;  /* list: element validity bitmap; NULL: no null element */
  int64_t child_length;           /* list: elements */
  int64_t child_null_count;
} GzDeviceColumn;

/* A reader for partitions of `schema_ipc` (an encapsulated Arrow IPC Schema message, as
 * ShuffleDecompressionJniWrapper.make receives) on CUDA device `device`. */
GzStatus gz_reader_make(const uint8_t* schema_ipc, int64_t schema_len, int32_t device, int64_t* out_handle);

/* Same with the schema as a field array. */
GzStatus gz_reader_make_fields(const GzField* fields, int32_t n_fields, int32_t device, int64_t* out_handle);

/* Adds one IPC stream of the partition (host bytes: a map output's partition_lengths[p] bytes of
 * its data file, with or without the schema message in front, ending with the end-of-stream
 * marker); the bytes are read before the call returns.  Compressed bodies return
 * GZ_NOT_IMPLEMENTED. */
GzStatus gz_reader_add_stream(int64_t handle, const uint8_t* stream, int64_t len);

/* Concatenates the record batches of every stream added, in order, into device columns and
 * waits for the device; *out_rows = rows, *out_batches = record batches read. */
GzStatus gz_reader_finish(int64_t handle, int64_t* out_rows, int32_t* out_batches);

/* The concatenated column of schema field `field` (after gz_reader_finish). */
GzStatus gz_reader_column(int64_t handle, int32_t field, GzDeviceColumn* out);

/* Copies the concatenated column of `field` to host memory: `validity` ((length + 7) / 8 bytes;
 * skipped when NULL or when the column has no nulls), `offsets` (length + 1 offsets of the
 * column's offset width, binary only), `values` (values_bytes bytes).  Waits for the copies. */
GzStatus gz_reader_column_to_host(int64_t handle, int32_t field, uint8_t* validity, void* offsets,
                                  uint8_t* values);

/* A list column's element validity ((child_length + 7) / 8 bytes) to host memory; nothing when
 * the column has no null element.  Waits for the copy. */
GzStatus gz_reader_elem_validity_to_host(int64_t handle, int32_t field, uint8_t* out);

/* The nodes of field `field` in pre-order (the Arrow children layout the record batches carry):
 * 1 for a flat field, 2 for a list of fixed-width or bool elements (the list; its elements), the
 * type tree of a nested field (a map's entries struct between the map and its key and value).
 * Each node as a column: its entries, validity (nullptr: no nulls), offsets (list / map / binary;
 * 64-bit for large types), values (fixed width, bool bits, characters; nullptr for list, map and
 * struct nodes).  Reduce-side counterpart of Arrow Java's nested vectors
 * (ArrowColumnarBatchSerializer.scala:110-240). */
GzStatus gz_reader_node_count(int64_t handle, int32_t field, int32_t* out_nodes);
GzStatus gz_reader_node(int64_t handle, int32_t field, int32_t node, GzDeviceColumn* out);
GzStatus gz_reader_node_to_host(int64_t handle, int32_t field, int32_t node, uint8_t* validity, void* offsets,
                                uint8_t* values);

/* Frees the reader and its device columns. */
GzStatus gz_reader_close(int64_t handle);

/* ---- test hooks (no reference counterpart; used by the unit tests) ------------------- */

/* Encodes one Arrow IPC RecordBatch message with the splitter's encoder.  nodes: L pairs
 * {length, null_count}; bufs/buf_lens: M body buffers.  Writes into `out` (capacity
 * out_cap) and sets *out_len; GZ_INVALID when it does not fit. */
GzStatus gz_debug_encode_record_batch(int64_t length, const int64_t* nodes, int32_t n_nodes,
                                      const uint8_t* const* bufs, const int64_t* buf_lens,
                                      int32_t n_bufs, uint8_t* out, int64_t out_cap,
                                      int64_t* out_len);

/* The same message with LZ4_FRAME body compression, every non-empty buffer written as an
 * uncompressed length and an LZ4 frame of stored (uncompressed) blocks of at most 64 KiB: checks
 * the compressed message layout and the frame framing without the device compressor. */
GzStatus gz_debug_encode_record_batch_lz4_stored(int64_t length, const int64_t* nodes, int32_t n_nodes,
                                                const uint8_t* const* bufs, const int64_t* buf_lens,
                                                int32_t n_bufs, uint8_t* out, int64_t out_cap,
                                                int64_t* out_len);

/* Parses an Arrow IPC Schema message and encodes it again with the splitter's schema writer (the
 * message written before each partition when write_schema is set). */
GzStatus gz_debug_reencode_schema(const uint8_t* schema_ipc, int64_t len, uint8_t* out, int64_t cap,
                                  int64_t* out_len);

/* Sets how many times k_scatter polls a wait for a staged slice or a free staging slot in the
 * handle's later device passes before it gives up (0: the default, about 2^26).  A block that
 * gives up stops issuing copies, waits (with the default limit) for the copies already in flight,
 * skips its remaining work and sets an error bit: the next synchronising call returns GZ_TIMEOUT
 * and the device stays usable.  Lets a test make the bounded waits run out. */
GzStatus gz_debug_set_spin_limit(int64_t handle, uint32_t polls);

/* Parses an Arrow IPC Schema message; writes up to `cap` GzType codes and nullable flags. */
GzStatus gz_debug_parse_schema(const uint8_t* schema_ipc, int64_t len, int32_t* types,
                               int32_t* nullable, int32_t cap, int32_t* n_fields);

#ifdef __cplusplus
}
#endif

#endif /* GZ_SPLIT_H */
