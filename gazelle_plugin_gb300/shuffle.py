"""Python mirror of the reference's shuffle-splitter boundary, over libgzsplit.so.

``ShuffleSplitterJniWrapper`` keeps the method names, argument meaning and error behaviour of
com.intel.oap.vectorized.ShuffleSplitterJniWrapper
(native-sql-engine/core/src/main/java/com/intel/oap/vectorized/ShuffleSplitterJniWrapper.java:41-135)
and ``SplitResult`` the fields of SplitResult.java:21-39.  Every call goes through the C ABI in
include/gz_split.h; there is no Python or CPU fallback: a missing library raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgzsplit.so")

GZ_OK, GZ_INVALID, GZ_OOM, GZ_IO, GZ_NOT_IMPLEMENTED, GZ_TIMEOUT, GZ_CUDA = range(7)
GZ_INPUT_HOST, GZ_INPUT_DEVICE_RETAINED = 0, 1
GZ_HOST_READ_AUTO, GZ_HOST_READ_CPU_COPY = 0, 1
_STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "OOM", 3: "IO", 4: "NOT_IMPLEMENTED", 5: "TIMEOUT",
                 6: "CUDA"}


class SplitterError(RuntimeError):
    """A non-OK GzStatus (the JNI layer throws a Java exception in the same places)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class GzSplitOptions(ctypes.Structure):
    _fields_ = [
        ("offheap_per_task", ctypes.c_int64),
        ("buffer_size", ctypes.c_int32),
        ("num_sub_dirs", ctypes.c_int32),
        ("batch_compress_threshold", ctypes.c_int32),
        ("compression", ctypes.c_int32),
        ("prefer_spill", ctypes.c_int32),
        ("write_schema", ctypes.c_int32),
        ("buffered_write", ctypes.c_int32),
        ("input_kind", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("keep_output_on_device", ctypes.c_int32),
        ("flush_bytes", ctypes.c_int64),
        ("device_budget", ctypes.c_int64),
        ("data_file", ctypes.c_char_p),
        ("local_dirs", ctypes.c_char_p),
        ("host_read", ctypes.c_int32),
        ("seg_tiles", ctypes.c_int32),
        ("host_budget", ctypes.c_int64),
    ]


class GzField(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("nullable", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("scale", ctypes.c_int32),
        ("unit", ctypes.c_int32),
        ("elem_type", ctypes.c_int32),
        ("name", ctypes.c_char_p),
        ("n_children", ctypes.c_int32),
        ("children", ctypes.c_void_p),
    ]


class GzSplitResult(ctypes.Structure):
    _fields_ = [
        ("total_compute_pid_time", ctypes.c_int64),
        ("total_write_time", ctypes.c_int64),
        ("total_spill_time", ctypes.c_int64),
        ("total_compress_time", ctypes.c_int64),
        ("total_bytes_written", ctypes.c_int64),
        ("total_bytes_spilled", ctypes.c_int64),
        ("partition_lengths", ctypes.POINTER(ctypes.c_int64)),
        ("raw_partition_lengths", ctypes.POINTER(ctypes.c_int64)),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    """The C-ABI library; raises when it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        c_i64p = ctypes.POINTER(ctypes.c_int64)
        L.gz_split_default_options.argtypes = [ctypes.POINTER(GzSplitOptions)]
        L.gz_split_make.restype = ctypes.c_int
        L.gz_split_make.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(GzSplitOptions),
                                    c_i64p]
        L.gz_split_make_fields.restype = ctypes.c_int
        L.gz_split_make_fields.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(GzField),
                                           ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.POINTER(GzSplitOptions), c_i64p]
        L.gz_split_split.restype = ctypes.c_int
        L.gz_split_split.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_int32, ctypes.c_int32, c_i64p]
        L.gz_split_split_batches.restype = ctypes.c_int
        L.gz_split_split_batches.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
        L.gz_split_split_group.restype = ctypes.c_int
        L.gz_split_split_group.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.gz_split_sync.restype = ctypes.c_int
        L.gz_split_sync.argtypes = [ctypes.c_int64]
        L.gz_split_sync_group.restype = ctypes.c_int
        L.gz_split_sync_group.argtypes = [ctypes.c_int32, ctypes.c_void_p]
        L.gz_split_stop.restype = ctypes.c_int
        L.gz_split_stop.argtypes = [ctypes.c_int64, ctypes.POINTER(GzSplitResult)]
        L.gz_split_data.restype = ctypes.c_int
        L.gz_split_data.argtypes = [ctypes.c_int64, ctypes.c_void_p, c_i64p]
        L.gz_split_spill.restype = ctypes.c_int
        L.gz_split_spill.argtypes = [ctypes.c_int64, ctypes.c_int64, c_i64p]
        L.gz_split_set_compress.restype = ctypes.c_int
        L.gz_split_set_compress.argtypes = [ctypes.c_int64, ctypes.c_int32]
        L.gz_split_close.restype = ctypes.c_int
        L.gz_split_close.argtypes = [ctypes.c_int64]
        L.gz_split_last_pids.restype = ctypes.c_int
        L.gz_split_last_pids.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32]
        L.gz_last_error.restype = ctypes.c_int
        L.gz_last_error.argtypes = [ctypes.c_int64, ctypes.c_char_p, ctypes.c_size_t]
        L.gz_debug_set_spin_limit.restype = ctypes.c_int
        L.gz_debug_set_spin_limit.argtypes = [ctypes.c_int64, ctypes.c_uint32]
        L.gz_split_stats.restype = ctypes.c_int
        L.gz_split_stats.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
        L.gz_split_kernel_times.restype = ctypes.c_int
        L.gz_split_kernel_times.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
        L.gz_reader_make.restype = ctypes.c_int
        L.gz_reader_make.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, c_i64p]
        L.gz_reader_make_fields.restype = ctypes.c_int
        L.gz_reader_make_fields.argtypes = [ctypes.POINTER(GzField), ctypes.c_int32, ctypes.c_int32, c_i64p]
        L.gz_reader_add_stream.restype = ctypes.c_int
        L.gz_reader_add_stream.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
        L.gz_reader_finish.restype = ctypes.c_int
        L.gz_reader_finish.argtypes = [ctypes.c_int64, c_i64p, ctypes.POINTER(ctypes.c_int32)]
        L.gz_reader_column.restype = ctypes.c_int
        L.gz_reader_column.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(GzDeviceColumn)]
        L.gz_reader_column_to_host.restype = ctypes.c_int
        L.gz_reader_column_to_host.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]
        L.gz_reader_elem_validity_to_host.restype = ctypes.c_int
        L.gz_reader_elem_validity_to_host.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
        L.gz_reader_node_count.restype = ctypes.c_int
        L.gz_reader_node_count.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        L.gz_reader_node.restype = ctypes.c_int
        L.gz_reader_node.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
        L.gz_reader_node_to_host.restype = ctypes.c_int
        L.gz_reader_node_to_host.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
        L.gz_reader_close.restype = ctypes.c_int
        L.gz_reader_close.argtypes = [ctypes.c_int64]
        L.gz_serve_start.restype = ctypes.c_int
        L.gz_serve_start.argtypes = [ctypes.c_int32, ctypes.c_int64, c_i64p]
        L.gz_serve_open.restype = ctypes.c_int
        L.gz_serve_open.argtypes = [ctypes.c_int64, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(GzField),
                                    ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                    ctypes.POINTER(GzSplitOptions), c_i64p]
        L.gz_serve_split.restype = ctypes.c_int
        L.gz_serve_split.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int32, c_i64p]
        L.gz_serve_stop.restype = ctypes.c_int
        L.gz_serve_stop.argtypes = [ctypes.c_int64, ctypes.c_int64, c_i64p]
        L.gz_serve_sync.restype = ctypes.c_int
        L.gz_serve_sync.argtypes = [ctypes.c_int64, ctypes.c_int64, c_i64p]
        L.gz_serve_wait.restype = ctypes.c_int
        L.gz_serve_wait.argtypes = [ctypes.c_int64, ctypes.c_int64, c_i64p, c_i64p]
        L.gz_pinned_reserve.restype = ctypes.c_int
        L.gz_pinned_reserve.argtypes = [ctypes.c_int64, c_i64p]
        L.gz_serve_shutdown.restype = ctypes.c_int
        L.gz_serve_shutdown.argtypes = [ctypes.c_int64]
        L.gz_autotune.restype = ctypes.c_int
        L.gz_autotune.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(GzField), ctypes.c_int32,
                                  ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(GzSplitOptions),
                                  ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_int32, ctypes.POINTER(GzTuneResult)]
        L.gz_tune_save.restype = ctypes.c_int
        L.gz_tune_save.argtypes = [ctypes.c_char_p]
        L.gz_tune_load.restype = ctypes.c_int
        L.gz_tune_load.argtypes = [ctypes.c_char_p]
        _lib = L
    return _lib


TASK_LIB_PATH = os.path.join(HERE, "libgztask.so")


class GzTaskJob(ctypes.Structure):
    _fields_ = [
        ("short_name", ctypes.c_char_p),
        ("num_partitions", ctypes.c_int32),
        ("fields", ctypes.POINTER(GzField)),
        ("n_fields", ctypes.c_int32),
        ("key_cols", ctypes.c_void_p),
        ("n_keys", ctypes.c_int32),
        ("opts", ctypes.POINTER(GzSplitOptions)),
        ("data_dir", ctypes.c_char_p),
        ("n_tasks", ctypes.c_int32),
        ("n_batches", ctypes.c_int32),
        ("rows", ctypes.c_void_p),
        ("addrs", ctypes.c_void_p),
        ("sizes", ctypes.c_void_p),
        ("n_bufs", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class GzTaskResult(ctypes.Structure):
    _fields_ = [
        ("wall_s", ctypes.c_double),
        ("split_s_max", ctypes.c_double),
        ("stop_s_max", ctypes.c_double),
        ("input_bytes", ctypes.c_int64),
        ("raw_partition_bytes", ctypes.c_int64),
        ("bytes_written", ctypes.c_int64),
        ("partition_lengths", ctypes.POINTER(ctypes.c_int64)),
        ("error", ctypes.c_char * 512),
    ]


_task_lib = None


def task_lib() -> ctypes.CDLL:
    """libgztask.so: simulated map tasks calling the C ABI (include/gz_task.h)."""
    global _task_lib
    if _task_lib is None:
        lib()  # the splitter library first
        if not os.path.exists(TASK_LIB_PATH):
            raise RuntimeError(f"{TASK_LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(TASK_LIB_PATH)
        L.gz_task_run.restype = ctypes.c_int
        L.gz_task_run.argtypes = [ctypes.POINTER(GzTaskJob), ctypes.POINTER(GzTaskResult)]
        L.gz_task_digest_file.restype = ctypes.c_int
        L.gz_task_digest_file.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64),
                                          ctypes.POINTER(ctypes.c_int64)]
        L.gz_task_digest.restype = ctypes.c_uint64
        L.gz_task_digest.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        _task_lib = L
    return _task_lib


def run_map_tasks(part: "NativePartitioning", rows, bufAddrs, bufSizes, nTasks: int,
                  dataDir: str = "", **options) -> dict:
    """Runs `nTasks` simulated map tasks (the writer's make / split per batch / stop / close loop,
    natively, on their own threads) over contiguous ranges of the batches; each writes
    <dataDir>/task-<t>.data.  Returns the timings, byte counts and per-task partition lengths."""
    o, keep = split_options(**options)
    arr, names = _fields(part.fields)
    keys = np.asarray(list(part.keyColumns), np.int32)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    addrs = np.ascontiguousarray(bufAddrs, dtype=np.int64)
    sizes = np.ascontiguousarray(bufSizes, dtype=np.int64)
    P = 1 if part.shortName == "single" else part.numPartitions
    pl = np.zeros((nTasks, P), np.int64)
    job = GzTaskJob(part.shortName.encode(), part.numPartitions, arr, len(part.fields), keys.ctypes.data,
                    len(keys), ctypes.pointer(o), dataDir.encode(), nTasks, len(rows), rows.ctypes.data,
                    addrs.ctypes.data, sizes.ctypes.data, addrs.shape[1], 0)
    res = GzTaskResult()
    res.partition_lengths = pl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    st = task_lib().gz_task_run(ctypes.byref(job), ctypes.byref(res))
    del keep, names
    if st != GZ_OK:
        raise SplitterError(st, res.error.decode(errors="replace"))
    return {"wall_s": res.wall_s, "split_s_max": res.split_s_max, "stop_s_max": res.stop_s_max,
            "input_bytes": res.input_bytes, "raw_partition_bytes": res.raw_partition_bytes,
            "bytes_written": res.bytes_written, "partition_lengths": pl}


def digest_file(path: str):
    """(checksum, size) of a file, as libgztask computes it."""
    d, n = ctypes.c_uint64(0), ctypes.c_int64(0)
    if task_lib().gz_task_digest_file(path.encode(), ctypes.byref(d), ctypes.byref(n)) != 0:
        raise OSError(f"cannot read {path}")
    return d.value, n.value


def digest_bytes(data) -> int:
    b = np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else data
    return int(task_lib().gz_task_digest(b.ctypes.data if b.nbytes else None, b.nbytes))


class GzDeviceColumn(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("length", ctypes.c_int64),
        ("null_count", ctypes.c_int64),
        ("validity", ctypes.c_void_p),
        ("offsets", ctypes.c_void_p),
        ("values", ctypes.c_void_p),
        ("values_bytes", ctypes.c_int64),
        ("child_validity", ctypes.c_void_p),
        ("child_length", ctypes.c_int64),
        ("child_null_count", ctypes.c_int64),
    ]


def _check(status: int, handle: int = 0) -> None:
    if status != GZ_OK:
        buf = ctypes.create_string_buffer(1024)
        lib().gz_last_error(handle, buf, 1024)
        raise SplitterError(status, buf.value.decode(errors="replace"))


def default_options() -> GzSplitOptions:
    o = GzSplitOptions()
    lib().gz_split_default_options(ctypes.byref(o))
    return o


GZ_CODEC_UNCOMPRESSED, GZ_CODEC_LZ4_FRAME, GZ_CODEC_FASTPFOR = 0, 1, 2


def codec_code(codec: Optional[str]) -> int:
    """GzCodec of the JNI's codec string (GetCompressionType): "lz4" is LZ4_FRAME."""
    if codec in (None, "", "uncompressed", "none"):
        return GZ_CODEC_UNCOMPRESSED
    return {"lz4": GZ_CODEC_LZ4_FRAME, "lz4_frame": GZ_CODEC_LZ4_FRAME,
            "fastpfor": GZ_CODEC_FASTPFOR}.get(codec.lower(), 99)


def split_options(offheapPerTask: int = 0, bufferSize: int = 4096, codec: Optional[str] = None,
                  batchCompressThreshold: int = 256, dataFile: str = "", subDirsPerLocalDir: int = 64,
                  localDirs: str = "", preferSpill: bool = True, writeSchema: bool = False,
                  **device_options):
    """GzSplitOptions from nativeMake's arguments plus device knobs; returns (options, the byte
    strings the options point to, which must outlive the call that reads them)."""
    o = default_options()
    o.offheap_per_task = offheapPerTask
    if bufferSize > 0:
        o.buffer_size = bufferSize
    if subDirsPerLocalDir > 0:
        o.num_sub_dirs = subDirsPerLocalDir
    o.batch_compress_threshold = batchCompressThreshold
    o.compression = codec_code(codec)
    o.prefer_spill = int(preferSpill)
    o.write_schema = int(writeSchema)
    o.buffered_write = 1
    keep = [dataFile.encode(), localDirs.encode()]
    o.data_file = keep[0]
    o.local_dirs = keep[1]
    for k, v in device_options.items():
        setattr(o, k, v)
    return o, keep


def _fields(schema):
    """A GzField array of the schema (children of nested fields in arrays of their own) and the
    objects that must stay alive with it."""
    from . import workloads as W
    arr = (GzField * len(schema))()
    keep = [arr]
    for i, f in enumerate(schema):
        arr[i].type = f.code
        arr[i].nullable = int(f.nullable)
        arr[i].precision, arr[i].scale, arr[i].unit = f.params
        if f.is_list:
            arr[i].elem_type = W.TYPE_CODES[f.elem]
            arr[i].precision, arr[i].scale, arr[i].unit = W.Field("item", f.elem).params
        if f.is_nested:
            kids, kkeep = _fields(list(f.kids))
            keep.append(kkeep)
            arr[i].n_children = len(f.kids)
            arr[i].children = ctypes.addressof(kids)
        name = f.name.encode()
        keep.append(name)
        arr[i].name = name
    return arr, keep


@dataclasses.dataclass
class SplitResult:
    """SplitResult.java:21-39."""
    totalComputePidTime: int
    totalWriteTime: int
    totalSpillTime: int
    totalCompressTime: int
    totalBytesWritten: int
    totalBytesSpilled: int
    partitionLengths: np.ndarray
    rawPartitionLengths: np.ndarray


@dataclasses.dataclass
class NativePartitioning:
    """NativePartitioning.java: short name, partition count, Arrow IPC schema bytes and the
    hash keys.  Short names as Splitter::Make takes them (splitter.cc:190-208): "hash" (by the
    key columns), "rr" (round-robin), "single" (one partition, whatever the count) and
    "range" (int32 partition ids in schema field 0, which the output leaves out).  The keys are
    schema column indices (the field-reference expressions Spark sends,
    ColumnarShuffleExchangeExec.scala:307-326); the other partitioners ignore them.  ``fields``
    may stand in for the schema bytes (a list of gazelle_plugin_gb300.workloads.Field)."""
    shortName: str
    numPartitions: int
    schema: Optional[bytes] = None
    keyColumns: Sequence[int] = ()
    fields: Optional[list] = None


class ShuffleSplitterJniWrapper:
    """Method-for-method mirror of ShuffleSplitterJniWrapper.java."""

    def __init__(self):
        self._partitions = {}  # handle -> partition count (the length of its SplitResult arrays)

    def make(self, part: NativePartitioning, offheapPerTask: int = 0, bufferSize: int = 4096,
             codec: Optional[str] = None, batchCompressThreshold: int = 256,
             dataFile: str = "", subDirsPerLocalDir: int = 64, localDirs: str = "",
             preferSpill: bool = True, memoryPoolId: int = 0, writeSchema: bool = False,
             **device_options) -> int:
        o, self._keep = split_options(offheapPerTask, bufferSize, codec, batchCompressThreshold, dataFile,
                                      subDirsPerLocalDir, localDirs, preferSpill, writeSchema, **device_options)
        keys = np.asarray(list(part.keyColumns), np.int32)
        h = ctypes.c_int64(0)
        if part.schema is not None:
            sb = ctypes.create_string_buffer(part.schema, len(part.schema))
            st = lib().gz_split_make(part.shortName.encode(), part.numPartitions, sb,
                                     len(part.schema), keys.ctypes.data, len(keys),
                                     ctypes.byref(o), ctypes.byref(h))
        else:
            arr, self._names = _fields(part.fields)
            st = lib().gz_split_make_fields(part.shortName.encode(), part.numPartitions, arr,
                                            len(part.fields), keys.ctypes.data, len(keys),
                                            ctypes.byref(o), ctypes.byref(h))
        _check(st, 0)
        self._partitions[h.value] = 1 if part.shortName == "single" else part.numPartitions
        return h.value

    def nativeSpill(self, splitterId: int, size: int, callBySelf: bool = False) -> int:
        actual = ctypes.c_int64(0)
        _check(lib().gz_split_spill(splitterId, size, ctypes.byref(actual)), splitterId)
        return actual.value

    def split(self, splitterId: int, numRows: int, bufAddrs, bufSizes,
              firstRecordBatch: bool = False) -> int:
        addrs = np.ascontiguousarray(bufAddrs, dtype=np.int64)
        sizes = np.ascontiguousarray(bufSizes, dtype=np.int64)
        if len(addrs) != len(sizes):
            raise SplitterError(GZ_INVALID, "Native split: length of buf_addrs and buf_sizes mismatch")
        out = ctypes.c_int64(-1)
        _check(lib().gz_split_split(splitterId, numRows, addrs.ctypes.data, sizes.ctypes.data,
                                    len(addrs), int(firstRecordBatch), ctypes.byref(out)),
               splitterId)
        return out.value

    def setCompressType(self, splitterId: int, compressType: str) -> None:
        _check(lib().gz_split_set_compress(splitterId, codec_code(compressType)), splitterId)

    def stop(self, splitterId: int, numPartitions: Optional[int] = None) -> SplitResult:
        P = numPartitions or self._partitions[splitterId]
        pl = np.zeros(P, np.int64)
        rl = np.zeros(P, np.int64)
        r = GzSplitResult()
        r.partition_lengths = pl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        r.raw_partition_lengths = rl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        _check(lib().gz_split_stop(splitterId, ctypes.byref(r)), splitterId)
        return SplitResult(r.total_compute_pid_time, r.total_write_time, r.total_spill_time,
                           r.total_compress_time, r.total_bytes_written, r.total_bytes_spilled,
                           pl, rl)

    def close(self, splitterId: int) -> None:
        _check(lib().gz_split_close(splitterId))

    # helpers beyond the Java surface -----------------------------------------------------
    def data(self, splitterId: int) -> bytes:
        n = ctypes.c_int64(0)
        _check(lib().gz_split_data(splitterId, None, ctypes.byref(n)), splitterId)
        buf = np.zeros(n.value, np.uint8)
        if n.value:
            _check(lib().gz_split_data(splitterId, buf.ctypes.data, ctypes.byref(n)), splitterId)
        return buf.tobytes()

    def lastPids(self, splitterId: int, numRows: int) -> np.ndarray:
        out = np.zeros(numRows, np.uint16)
        _check(lib().gz_split_last_pids(splitterId, out.ctypes.data, numRows), splitterId)
        return out

    def splitBatches(self, splitterId: int, rows, bufAddrs, bufSizes) -> None:
        """Split many batches in one call: rows[i], bufAddrs[i, :], bufSizes[i, :]."""
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        addrs = np.ascontiguousarray(bufAddrs, dtype=np.int64)
        sizes = np.ascontiguousarray(bufSizes, dtype=np.int64)
        assert addrs.shape == sizes.shape and addrs.shape[0] == rows.shape[0]
        _check(lib().gz_split_split_batches(splitterId, len(rows), rows.ctypes.data,
                                            addrs.ctypes.data, sizes.ctypes.data, addrs.shape[1]),
               splitterId)

    def splitGroup(self, splitterIds, rows, bufAddrs, bufSizes) -> None:
        """Split calls of several tasks at once: task i gets rows[i] (array of row counts) with
        bufAddrs[i] / bufSizes[i] (arrays [batches, buffers]); every task's host reads are in
        flight together."""
        h = np.ascontiguousarray(splitterIds, dtype=np.int64)
        nb = np.array([len(r) for r in rows], np.int32)
        nbuf = np.array([np.asarray(a).shape[1] if len(r) else 0 for r, a in zip(rows, bufAddrs)], np.int32)
        r = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int32) for x in rows]) if len(rows) else
                                 np.zeros(0, np.int32))
        a = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int64).reshape(-1) for x in bufAddrs]))
        z = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int64).reshape(-1) for x in bufSizes]))
        _check(lib().gz_split_split_group(len(h), h.ctypes.data, nb.ctypes.data, r.ctypes.data, a.ctypes.data,
                                          z.ctypes.data, nbuf.ctypes.data))

    def sync(self, splitterId: int) -> None:
        _check(lib().gz_split_sync(splitterId), splitterId)

    def syncGroup(self, splitterIds) -> None:
        """sync of several tasks, every task's pending pass queued before any is waited for."""
        h = np.ascontiguousarray(splitterIds, dtype=np.int64)
        _check(lib().gz_split_sync_group(len(h), h.ctypes.data))

    def setSpinLimit(self, splitterId: int, polls: int) -> None:
        """Test hook: polls of k_scatter's bounded waits in later passes (0: the default)."""
        _check(lib().gz_debug_set_spin_limit(splitterId, polls), splitterId)

    def stats(self, splitterId: int) -> List[int]:
        """[passes, input bytes, H2D bytes, D2H bytes, HBM-resident bytes, batches, rows,
        emitted record batches]."""
        out = (ctypes.c_int64 * 8)()
        _check(lib().gz_split_stats(splitterId, out), splitterId)
        return list(out)

    def diskSpill(self, splitterId: int) -> List[int]:
        """Local-dir spill files (host_budget): [files written, their bytes, files present now]."""
        out = (ctypes.c_int64 * 3)()
        _check(lib().gz_split_disk_spill(splitterId, out), splitterId)
        return list(out)

    def kernelTimes(self, splitterId: int) -> List[float]:
        out = (ctypes.c_double * 4)()
        _check(lib().gz_split_kernel_times(splitterId, out), splitterId)
        return list(out)


def split_batches(schema, batches, num_partitions: int, key_cols: Sequence[int],
                  shortName: str = "hash", **make_kwargs):
    """Make -> Split every batch -> Stop through the C ABI; returns (SplitResult, data)."""
    w = ShuffleSplitterJniWrapper()
    h = w.make(NativePartitioning(shortName, num_partitions, None, key_cols, list(schema)),
               **make_kwargs)
    try:
        for b in batches:
            addrs, sizes = b.addrs_sizes()
            w.split(h, b.num_rows, addrs, sizes, False)
        res = w.stop(h)
        data = w.data(h)
    finally:
        w.close(h)
    return res, data


class GzTuneResult(ctypes.Structure):
    _fields_ = [("flush_bytes", ctypes.c_int64), ("seg_tiles", ctypes.c_int32), ("runs", ctypes.c_int32),
                ("best_gbs", ctypes.c_double), ("default_gbs", ctypes.c_double)]


def autotune(schema, num_partitions: int, key_cols: Sequence[int], batches, shortName: str = "hash",
             **make_kwargs) -> dict:
    """gz_autotune over sample batches (workloads.Batch, host memory unless input_kind says
    otherwise): times candidate pass sizes and segment lengths and caches the fastest for this
    schema, key columns and partition count; splitters made afterwards with flush_bytes=0 and
    seg_tiles=0 use it.  Returns the choice and the sample throughputs."""
    o, keep = split_options(**make_kwargs)
    arr, names = _fields(schema)
    keys = np.ascontiguousarray(key_cols, dtype=np.int32)
    rows = np.ascontiguousarray([b.num_rows for b in batches], dtype=np.int32)
    pairs = [b.addrs_sizes() for b in batches]
    addrs = np.ascontiguousarray(np.stack([a for a, _ in pairs]), dtype=np.int64)
    sizes = np.ascontiguousarray(np.stack([z for _, z in pairs]), dtype=np.int64)
    r = GzTuneResult()
    _check(lib().gz_autotune(shortName.encode(), num_partitions, arr, len(schema), keys.ctypes.data, len(keys),
                             ctypes.byref(o), len(batches), rows.ctypes.data, addrs.ctypes.data,
                             sizes.ctypes.data, addrs.shape[1], ctypes.byref(r)), 0)
    return {"flush_bytes": r.flush_bytes, "seg_tiles": r.seg_tiles, "runs": r.runs,
            "best_gbs": r.best_gbs, "default_gbs": r.default_gbs}


def tune_save(path: str) -> None:
    _check(lib().gz_tune_save(path.encode()), 0)


def tune_load(path: str) -> None:
    _check(lib().gz_tune_load(path.encode()), 0)


def pinned_reserve(nbytes: int) -> int:
    """Pins about `nbytes` of host memory into the library's pool up front (gz_pinned_reserve)."""
    got = ctypes.c_int64(0)
    _check(lib().gz_pinned_reserve(nbytes, ctypes.byref(got)), 0)
    return got.value


class ServeLoop:
    """The served form (gz_serve_*): Split / Stop calls of many concurrent tasks on one GPU,
    asynchronous, with per-call latency.  A task is an ordinary splitter handle, so
    ShuffleSplitterJniWrapper.stop / data / close read its results after its stop ticket."""

    def __init__(self, slots: int = 4, hbmBudget: int = 40 << 30):
        h = ctypes.c_int64(0)
        _check(lib().gz_serve_start(slots, hbmBudget, ctypes.byref(h)), 0)
        self.handle = h.value
        self._keep = {}

    def open(self, schema, numPartitions: int, keyColumns: Sequence[int], shortName: str = "hash",
             **make_kwargs) -> int:
        """Blocks until the HBM budget admits the task; returns its splitter handle."""
        o, keep = split_options(**make_kwargs)
        arr, names = _fields(schema)
        keys = np.asarray(list(keyColumns), np.int32)
        t = ctypes.c_int64(0)
        _check(lib().gz_serve_open(self.handle, shortName.encode(), numPartitions, arr, len(schema), keys.ctypes.data,
                                   len(keys), ctypes.byref(o), ctypes.byref(t)), 0)
        self._keep[t.value] = (keep, names)
        return t.value

    def split(self, task: int, numRows: int, bufAddrs, bufSizes) -> int:
        """Queues one Split; the buffers stay valid until wait(ticket) returns."""
        addrs = np.ascontiguousarray(bufAddrs, dtype=np.int64)
        sizes = np.ascontiguousarray(bufSizes, dtype=np.int64)
        t = ctypes.c_int64(0)
        _check(lib().gz_serve_split(self.handle, task, numRows, addrs.ctypes.data, sizes.ctypes.data,
                                    len(addrs), ctypes.byref(t)), 0)
        return t.value

    def stop(self, task: int) -> int:
        t = ctypes.c_int64(0)
        _check(lib().gz_serve_stop(self.handle, task, ctypes.byref(t)), 0)
        return t.value

    def sync(self, task: int) -> int:
        """Queues a wait for the task's device work so far; returns the ticket."""
        t = ctypes.c_int64(0)
        _check(lib().gz_serve_sync(self.handle, task, ctypes.byref(t)), 0)
        return t.value

    def wait(self, ticket: int, service: bool = False):
        """Latency of the call in ns (submission to completion), and with service=True also the
        ns its worker spent on it; raises on its error."""
        lat = ctypes.c_int64(0)
        svc = ctypes.c_int64(0)
        _check(lib().gz_serve_wait(self.handle, ticket, ctypes.byref(lat), ctypes.byref(svc)), 0)
        return (lat.value, svc.value) if service else lat.value

    def shutdown(self) -> None:
        if self.handle:
            lib().gz_serve_shutdown(self.handle)
            self.handle = 0


class PartitionReader:
    """The reduce side: the IPC streams of one partition (a map output's partition_lengths[p]
    bytes of its data file each) read into one set of Arrow columns in device memory.  Stands in
    for the reference's ArrowColumnarBatchSerializer + ShuffleDecompressionJniWrapper read path."""

    def __init__(self, schema, device: int = 0):
        h = ctypes.c_int64(0)
        if isinstance(schema, (bytes, bytearray)):
            sb = ctypes.create_string_buffer(bytes(schema), len(schema))
            _check(lib().gz_reader_make(sb, len(schema), device, ctypes.byref(h)))
        else:
            arr, self._names = _fields(schema)
            _check(lib().gz_reader_make_fields(arr, len(schema), device, ctypes.byref(h)))
        self.h = h.value
        self.schema = schema

    def addStream(self, data) -> None:
        b = np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else data.view(np.uint8)
        _check(lib().gz_reader_add_stream(self.h, b.ctypes.data if b.nbytes else None, b.nbytes))

    def finish(self):
        rows, nb = ctypes.c_int64(0), ctypes.c_int32(0)
        _check(lib().gz_reader_finish(self.h, ctypes.byref(rows), ctypes.byref(nb)))
        return rows.value, nb.value

    def column(self, field: int) -> GzDeviceColumn:
        c = GzDeviceColumn()
        _check(lib().gz_reader_column(self.h, field, ctypes.byref(c)))
        return c

    def column_to_host(self, field: int):
        """(validity bytes or None, offsets or None, values bytes) of a concatenated column."""
        c = self.column(field)
        valid = np.zeros((c.length + 7) // 8, np.uint8) if c.validity else None
        offs = np.zeros(c.length + 1, np.int64 if c.type in (21, 22, 24) else np.int32) if c.offsets else None
        vals = np.zeros(c.values_bytes, np.uint8)
        _check(lib().gz_reader_column_to_host(self.h, field, valid.ctypes.data if valid is not None else None,
                                              offs.ctypes.data if offs is not None else None,
                                              vals.ctypes.data if vals.nbytes else None))
        return valid, offs, vals

    def node_count(self, field: int) -> int:
        """Nodes of a field in pre-order (gz_reader_node_count)."""
        n = ctypes.c_int32(0)
        _check(lib().gz_reader_node_count(self.h, field, ctypes.byref(n)))
        return n.value

    def node_to_host(self, field: int, node: int):
        """(length, null_count, validity bytes or None, offsets or None, values bytes) of one node."""
        c = GzDeviceColumn()
        _check(lib().gz_reader_node(self.h, field, node, ctypes.byref(c)))
        valid = np.zeros((c.length + 7) // 8, np.uint8) if c.validity else None
        offs = np.zeros(c.length + 1, np.int64 if c.type in (21, 22, 24) else np.int32) if c.offsets else None
        vals = np.zeros(c.values_bytes, np.uint8)
        _check(lib().gz_reader_node_to_host(self.h, field, node, valid.ctypes.data if valid is not None else None,
                                            offs.ctypes.data if offs is not None else None,
                                            vals.ctypes.data if vals.nbytes else None))
        return c.length, c.null_count, valid, offs, vals

    def element_validity_to_host(self, field: int):
        """A list column's element validity bytes, or None without a null element."""
        c = self.column(field)
        if not c.child_validity:
            return None
        out = np.zeros((c.child_length + 7) // 8, np.uint8)
        _check(lib().gz_reader_elem_validity_to_host(self.h, field, out.ctypes.data))
        return out

    def close(self) -> None:
        if self.h:
            lib().gz_reader_close(self.h)
            self.h = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
