"""ORACLE - test infrastructure only.

ctypes front-ends for
  * ``libgz_oracle.so``  - the CPU restatement of the reference Splitter (hash, rr, single,
    range partitioning)
    (oracle/split_oracle.cc); travels everywhere, built by ``build()``;
  * ``_ref/libgzref_splitter.so`` - the reference Splitter itself compiled from the
    reference tree (oracle/ref/Makefile); exists only where the reference sources and
    pyarrow are present, and is used to pin the restatement and to make golden fixtures.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libgz_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgzref_splitter.so")
REF_HASH_SO = os.path.join(HERE, "_ref", "libgzref_hash.so")

_I64P = ctypes.POINTER(ctypes.c_int64)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("split_oracle.cc", "lz4_oracle.cc")]
    deps = srcs + [os.path.join(HERE, "spark_hash.h")]
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(map(os.path.getmtime, deps)):
        tmp = ORACLE_SO + f".{os.getpid()}.tmp"
        subprocess.check_call(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", *srcs, "-o", tmp])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_root():
    """The reference source tree to compile and read fixtures from: $GZ_REFERENCE_ROOT, else the
    recipe's default (REF in oracle/ref/Makefile); None when neither names a tree."""
    root = os.environ.get("GZ_REFERENCE_ROOT")
    if not root:
        try:
            out = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "print-ref"],
                                 capture_output=True, text=True, timeout=30)
            root = out.stdout.strip() if out.returncode == 0 else ""
        except (OSError, subprocess.SubprocessError):
            root = ""
    return root if root and os.path.isdir(os.path.join(root, "native-sql-engine")) else None


def build_ref(ref_root: str) -> bool:
    """Compile the reference Splitter (x86_64 + pyarrow + reference tree only)."""
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "native-sql-engine")):
        return False
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}"])
    return os.path.exists(REF_SO)


@dataclass
class SplitOutput:
    partition_lengths: np.ndarray
    raw_partition_lengths: np.ndarray
    bytes_written: int
    bytes_spilled: int
    data: bytes

    def partition_bytes(self, pid: int) -> bytes:
        start = int(self.partition_lengths[:pid].sum())
        return self.data[start:start + int(self.partition_lengths[pid])]


class OracleSplitter:
    """Restated reference Splitter (compression off), partitioned by ``short_name``: "hash"
    (the key columns), "rr", "single" or "range" (int32 partition ids in schema field 0, which
    the output leaves out).  With write_schema the schema message is serialised by Arrow itself
    (pyarrow), as the reference's GetSchemaPayload does."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(build_oracle())
            lib.gzo_make.restype = ctypes.c_void_p
            lib.gzo_make.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                     ctypes.c_int]
            lib.gzo_split.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p,
                                      ctypes.c_int]
            lib.gzo_stop.restype = ctypes.c_int64
            lib.gzo_stop.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                     ctypes.c_int]
            lib.gzo_file_bytes.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            lib.gzo_last_pids.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            lib.gzo_spill.restype = ctypes.c_int64
            lib.gzo_spill.argtypes = [ctypes.c_void_p, ctypes.c_int64]
            lib.gzo_close.argtypes = [ctypes.c_void_p]
            lib.gzo_set_schema_message.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
            lib.gzo_hash_int.restype = ctypes.c_int32
            lib.gzo_hash_int.argtypes = [ctypes.c_int32, ctypes.c_int32]
            lib.gzo_hash_long.restype = ctypes.c_int32
            lib.gzo_hash_long.argtypes = [ctypes.c_int64, ctypes.c_int32]
            lib.gzo_murmur3_bytes.restype = ctypes.c_uint32
            lib.gzo_murmur3_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32]
            lib.gzo_xxh32.restype = ctypes.c_uint32
            lib.gzo_xxh32.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32]
            lib.gzo_lz4f_decompress.restype = ctypes.c_int64
            lib.gzo_lz4f_decompress.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
            lib.gzo_pmod.restype = ctypes.c_int32
            lib.gzo_pmod.argtypes = [ctypes.c_int32, ctypes.c_int32]
            cls._lib = lib
        return cls._lib

    def __init__(self, schema, num_partitions: int, key_cols: Sequence[int],
                 offheap_per_task: int = 0, buffer_size: int = 4096, prefer_spill: bool = True,
                 write_schema: bool = False, short_name: str = "hash"):
        self.P = 1 if short_name == "single" else num_partitions
        # the fields' type trees in pre-order (child counts above the low byte)
        types = np.array([c for f in schema for c in f.type_nodes()], np.int32)
        keys = np.array(key_cols, np.int32)
        err = ctypes.create_string_buffer(512)
        self.h = self.lib().gzo_make(short_name.encode(), types.ctypes.data, len(schema),
                                     num_partitions, keys.ctypes.data, len(keys),
                                     offheap_per_task, buffer_size, int(prefer_spill), err, 512)
        if not self.h:
            raise ValueError(err.value.decode())
        if write_schema:
            out_schema = list(schema)[1:] if short_name == "range" else schema
            msg = to_pyarrow_schema(out_schema).serialize().to_pybytes()
            self.lib().gzo_set_schema_message(self.h, msg, len(msg))

    def split(self, batch) -> None:
        addrs, sizes = batch.addrs_sizes()
        err = ctypes.create_string_buffer(512)
        if self.lib().gzo_split(self.h, batch.num_rows, addrs.ctypes.data, sizes.ctypes.data,
                                len(addrs), err, 512):
            raise ValueError(err.value.decode())

    def last_pids(self, num_rows: int) -> np.ndarray:
        out = np.zeros(num_rows, np.uint16)
        self.lib().gzo_last_pids(self.h, out.ctypes.data)
        return out

    def spill(self, size: int) -> int:
        return self.lib().gzo_spill(self.h, size)

    def stop(self) -> SplitOutput:
        lengths = np.zeros(self.P, np.int64)
        raw = np.zeros(self.P, np.int64)
        metrics = np.zeros(3, np.int64)
        err = ctypes.create_string_buffer(512)
        n = self.lib().gzo_stop(self.h, None, lengths.ctypes.data, raw.ctypes.data,
                                metrics.ctypes.data, err, 512)
        if n < 0:
            raise ValueError(err.value.decode())
        data = np.zeros(n, np.uint8)
        if n:
            self.lib().gzo_file_bytes(self.h, data.ctypes.data)
        return SplitOutput(lengths, raw, int(metrics[0]), int(metrics[1]), data.tobytes())

    def close(self):
        if self.h:
            self.lib().gzo_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_oracle(schema, batches, num_partitions, key_cols, **opts) -> SplitOutput:
    s = OracleSplitter(schema, num_partitions, key_cols, **opts)
    for b in batches:
        s.split(b)
    out = s.stop()
    s.close()
    return out


# ---------------------------------------------------------------------------------------
# the reference itself (this container only)
def to_pyarrow_schema(schema):
    import pyarrow as pa
    m = {"null": pa.null(), "bool": pa.bool_(), "int8": pa.int8(), "uint8": pa.uint8(),
         "int16": pa.int16(), "uint16": pa.uint16(), "float16": pa.float16(),
         "int32": pa.int32(), "uint32": pa.uint32(), "float32": pa.float32(),
         "date32": pa.date32(), "time32": pa.time32("ms"), "int64": pa.int64(),
         "uint64": pa.uint64(), "float64": pa.float64(), "date64": pa.date64(),
         "time64": pa.time64("us"), "timestamp": pa.timestamp("us"),
         "decimal128": pa.decimal128(30, 2), "utf8": pa.string(), "binary": pa.binary(),
         "large_utf8": pa.large_string(), "large_binary": pa.large_binary()}
    units = ["s", "ms", "us", "ns"]

    def fld(k):
        return pa.field(k.name, typ(k), k.nullable)

    def typ(f):
        if f.type == "list":  # a simple list's element field: Arrow's default "item", nullable
            return pa.list_(fld(f.kids[0]))
        if f.type == "large_list":
            return pa.large_list(fld(f.kids[0]))
        if f.type == "struct":
            return pa.struct([fld(k) for k in f.kids])
        if f.type == "map":
            return pa.map_(typ(f.kids[0]), fld(f.kids[1]))
        prec, scale, unit = f.params
        if f.type == "decimal128":
            return pa.decimal128(prec, scale)
        if f.type == "time32":
            return pa.time32(units[unit])
        if f.type == "time64":
            return pa.time64(units[unit])
        if f.type == "timestamp":
            return pa.timestamp(units[unit])
        return m[f.type]
    return pa.schema([pa.field(f.name, typ(f), f.nullable) for f in schema])


class RefSplitter:
    """The reference Splitter compiled from the reference tree (oracle/_ref)."""

    _lib = None

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(REF_SO)

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = ctypes.CDLL(REF_SO)
            lib.gzref_make.restype = ctypes.c_void_p
            lib.gzref_make.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
                                       ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_int]
            lib.gzref_split.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p,
                                        ctypes.c_int]
            lib.gzref_stop.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
            lib.gzref_compressed_size.restype = ctypes.c_int64
            lib.gzref_compressed_size.argtypes = [ctypes.c_void_p, ctypes.c_int32,
                                                  ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_int32]
            lib.gzref_spill.argtypes = [ctypes.c_void_p, ctypes.c_int64, _I64P]
            lib.gzref_close.argtypes = [ctypes.c_void_p]
            cls._lib = lib
        return cls._lib

    def __init__(self, schema, num_partitions: int, key_cols: Sequence[int],
                 offheap_per_task: int = 0, buffer_size: int = 4096, prefer_spill: bool = True,
                 write_schema: bool = False, short_name: str = "hash"):
        self.P = 1 if short_name == "single" else num_partitions
        self.tmp = tempfile.TemporaryDirectory(prefix="gzref-")
        self.data_file = os.path.join(self.tmp.name, "data")
        sbytes = to_pyarrow_schema(schema).serialize().to_pybytes()
        self._sbuf = ctypes.create_string_buffer(sbytes, len(sbytes))
        keys = np.array(key_cols, np.int32)
        err = ctypes.create_string_buffer(512)
        self.h = self.lib().gzref_make(short_name.encode(), self._sbuf, len(sbytes), num_partitions,
                                       keys.ctypes.data, len(keys), offheap_per_task,
                                       buffer_size, int(prefer_spill), int(write_schema),
                                       self.data_file.encode(),
                                       os.path.join(self.tmp.name, "local").encode(), err, 512)
        if not self.h:
            raise ValueError(err.value.decode())

    def split(self, batch) -> None:
        addrs, sizes = batch.addrs_sizes()
        err = ctypes.create_string_buffer(512)
        if self.lib().gzref_split(self.h, batch.num_rows, addrs.ctypes.data, sizes.ctypes.data,
                                  len(addrs), err, 512):
            raise ValueError(err.value.decode())

    def compressed_size(self, batch) -> int:
        addrs, sizes = batch.addrs_sizes()
        return self.lib().gzref_compressed_size(self.h, batch.num_rows, addrs.ctypes.data,
                                                sizes.ctypes.data, len(addrs))

    def spill(self, size: int) -> int:
        actual = ctypes.c_int64(0)
        self.lib().gzref_spill(self.h, size, ctypes.byref(actual))
        return actual.value

    def stop(self) -> SplitOutput:
        lengths = np.zeros(self.P, np.int64)
        raw = np.zeros(self.P, np.int64)
        metrics = np.zeros(2, np.int64)
        err = ctypes.create_string_buffer(512)
        if self.lib().gzref_stop(self.h, lengths.ctypes.data, raw.ctypes.data,
                                 metrics.ctypes.data, err, 512):
            raise ValueError(err.value.decode())
        with open(self.data_file, "rb") as f:
            data = f.read()
        return SplitOutput(lengths, raw, int(metrics[0]), int(metrics[1]), data)

    def close(self):
        if self.h:
            self.lib().gzref_close(self.h)
            self.h = None
        self.tmp.cleanup()


def run_ref(schema, batches, num_partitions, key_cols, **opts) -> SplitOutput:
    s = RefSplitter(schema, num_partitions, key_cols, **opts)
    for b in batches:
        s.split(b)
    out = s.stop()
    s.close()
    return out


# ---------------------------------------------------------------------------------------
# LZ4 frame decoding (oracle/lz4_oracle.cc)
def xxh32(data: bytes, seed: int = 0) -> int:
    b = np.frombuffer(data, np.uint8)
    return OracleSplitter.lib().gzo_xxh32(b.ctypes.data if b.nbytes else None, b.nbytes, seed)


def lz4f_decompress(frame: bytes, size: int) -> bytes:
    """Decodes one LZ4 frame that holds `size` bytes; raises on a malformed frame."""
    src = np.frombuffer(frame, np.uint8)
    dst = np.zeros(max(size, 1), np.uint8)
    n = OracleSplitter.lib().gzo_lz4f_decompress(src.ctypes.data, src.nbytes, dst.ctypes.data, size)
    if n != size:
        raise ValueError(f"bad LZ4 frame (decoded {n} of {size} bytes)")
    return dst[:size].tobytes()
