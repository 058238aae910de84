"""The C-ABI library: it loads without a GPU, exports every declared entry point, and its
host-side encoders (Arrow IPC record-batch framing, schema parsing) match Arrow C++."""
import ctypes
import os
import re

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="gz_split.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(gz_\w+)\(", src, re.M)))


def test_every_header_is_checked():
    assert sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")) == \
        ["gz_split.h", "gz_task.h"]


def test_library_exports_every_declared_symbol():
    lib = S.lib()
    names = declared_symbols()
    assert "gz_split_make" in names and "gz_split_stop" in names
    for n in names:
        assert hasattr(lib, n), n


def test_task_driver_exports_every_declared_symbol():
    """libgztask.so, the simulated map tasks that call the C ABI (include/gz_task.h)."""
    lib = S.task_lib()
    names = declared_symbols("gz_task.h")
    assert "gz_task_run" in names
    for n in names:
        assert hasattr(lib, n), n


def test_default_options_are_the_reference_defaults():
    o = S.default_options()
    assert (o.buffer_size, o.num_sub_dirs, o.batch_compress_threshold, o.prefer_spill,
            o.write_schema, o.compression) == (4096, 64, 256, 1, 1, 0)


def encode(length, nodes, bufs):
    lib = S.lib()
    lib.gz_debug_encode_record_batch.restype = ctypes.c_int
    lib.gz_debug_encode_record_batch.argtypes = [
        ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    n = np.array(nodes, np.int64).reshape(-1)
    ptrs = (ctypes.c_void_p * max(len(bufs), 1))(*[b.ctypes.data if b.nbytes else None for b in bufs])
    lens = np.array([b.nbytes for b in bufs], np.int64)
    out = np.zeros(1 << 20, np.uint8)
    olen = ctypes.c_int64(0)
    st = lib.gz_debug_encode_record_batch(ctypes.c_int64(length), n.ctypes.data, len(nodes), ptrs,
                                          lens.ctypes.data, len(bufs), out.ctypes.data,
                                          ctypes.c_int64(out.nbytes), ctypes.byref(olen))
    assert st == 0
    return out[:olen.value].tobytes()


def test_ipc_encoder_matches_arrow_writer():
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(3)
    for trial in range(40):
        n = int(rng.integers(1, 300))
        cols = []
        for c in range(int(rng.integers(1, 7))):
            kind = rng.integers(0, 5)
            mask = rng.random(n) < rng.choice([0.0, 0.2])
            if kind == 0:
                cols.append(pa.array(rng.integers(-100, 100, n), pa.int32(), mask=mask))
            elif kind == 1:
                cols.append(pa.array(rng.standard_normal(n), pa.float64(), mask=mask))
            elif kind == 2:
                cols.append(pa.array(["x" * int(k) for k in rng.integers(0, 9, n)], pa.string(), mask=mask))
            elif kind == 3:
                cols.append(pa.array(rng.integers(0, 2, n).astype(bool), pa.bool_(), mask=mask))
            elif c > 0:
                cols.append(pa.nulls(n))
            else:  # the splitter always has a data column, so the body is never empty
                cols.append(pa.array(rng.integers(-5, 5, n), pa.int8()))
        rb = pa.record_batch(cols, names=[f"c{i}" for i in range(len(cols))])
        expect = rb.serialize().to_pybytes()
        nodes, bufs = [], []
        for col in rb.columns:
            nodes.append((len(col), col.null_count))
            if col.type == pa.null():
                continue
            bs = col.buffers()
            bufs.append(np.frombuffer(bs[0], np.uint8).copy() if (bs[0] is not None and col.null_count)
                        else np.zeros(0, np.uint8))
            if pa.types.is_string(col.type):
                off = np.frombuffer(bs[1], np.int32)[: n + 1]
                bufs.append(off.view(np.uint8).copy())
                bufs.append(np.frombuffer(bs[2], np.uint8)[: off[-1]].copy() if bs[2] is not None
                            else np.zeros(0, np.uint8))
            elif pa.types.is_boolean(col.type):
                bufs.append(np.frombuffer(bs[1], np.uint8)[: (n + 7) // 8].copy())
            else:
                w = col.type.bit_width // 8
                bufs.append(np.frombuffer(bs[1], np.uint8)[: n * w].copy())
        got = encode(n, nodes, bufs)
        # pyarrow pads the body of its own buffers identically; compare metadata and body
        assert got[:8 + int.from_bytes(expect[4:8], "little")] == \
            expect[:8 + int.from_bytes(expect[4:8], "little")], trial


def parse_schema(sbytes):
    lib = S.lib()
    lib.gz_debug_parse_schema.restype = ctypes.c_int
    lib.gz_debug_parse_schema.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_int32)]
    types = np.zeros(64, np.int32)
    nulls = np.zeros(64, np.int32)
    n = ctypes.c_int32(0)
    st = lib.gz_debug_parse_schema(sbytes, len(sbytes), types.ctypes.data, nulls.ctypes.data, 64,
                                   ctypes.byref(n))
    return st, list(types[:n.value]), list(nulls[:n.value])


def test_schema_ipc_parser():
    pa = pytest.importorskip("pyarrow")
    from oracle.oracle import to_pyarrow_schema
    from gazelle_plugin_gb300 import workloads as W
    schema = [W.Field(f"c{i}", t, i % 2 == 0, "int64" if t == "list" else None)
              for i, t in enumerate(W.TYPE_CODES) if t not in ("large_list", "struct", "map")]
    st, types, nulls = parse_schema(to_pyarrow_schema(schema).serialize().to_pybytes())
    assert st == 0
    expect = [f.code for f in schema]
    # time32/time64/date64/timestamp round-trip through their Arrow units
    assert types == expect
    assert nulls == [int(f.nullable) for f in schema]
    # nested types of any depth parse (their top-level type codes are reported)
    for t, code in ((pa.list_(pa.list_(pa.int32())), 23), (pa.list_(pa.utf8()), 23),
                    (pa.struct([pa.field("a", pa.int32())]), 25), (pa.large_list(pa.int8()), 24),
                    (pa.map_(pa.utf8(), pa.list_(pa.bool_())), 26)):
        st, types, _ = parse_schema(pa.schema([pa.field("l", t)]).serialize().to_pybytes())
        assert st == 0 and types == [code], t
    # null children, empty structs and other nested types are refused
    for t in (pa.list_(pa.null()), pa.struct([]), pa.list_(pa.int32(), 3),
              pa.struct([pa.field("u", pa.dense_union([pa.field("x", pa.int8())]))])):
        st, _, _ = parse_schema(pa.schema([pa.field("l", t)]).serialize().to_pybytes())
        assert st != 0, t


def test_schema_message_matches_arrow_writer():
    """The schema message written before each partition (write_schema) is byte for byte what
    Arrow C++ writes for the same schema (GetSchemaPayload + WriteIpcPayload, which
    pyarrow.Schema.serialize also uses): 300 random schemas over every splittable type."""
    pa = pytest.importorskip("pyarrow")
    import random
    lib = S.lib()
    lib.gz_debug_reencode_schema.restype = ctypes.c_int
    lib.gz_debug_reencode_schema.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    types = [pa.bool_(), pa.int8(), pa.int16(), pa.int32(), pa.int64(), pa.uint8(), pa.uint16(),
             pa.uint32(), pa.uint64(), pa.float16(), pa.float32(), pa.float64(), pa.date32(),
             pa.date64(), pa.time32("s"), pa.time32("ms"), pa.time64("us"), pa.time64("ns"),
             pa.timestamp("s"), pa.timestamp("ms"), pa.timestamp("us"), pa.timestamp("ns"),
             pa.timestamp("us", tz="UTC"), pa.timestamp("ns", tz="America/New_York"),
             pa.decimal128(10, 2), pa.decimal128(38, 0), pa.decimal128(1, 0), pa.utf8(),
             pa.binary(), pa.null(), pa.large_utf8(), pa.large_binary(),
             pa.list_(pa.int32()), pa.list_(pa.float64()), pa.list_(pa.field("element", pa.int64(), False)),
             pa.list_(pa.decimal128(12, 3)), pa.list_(pa.timestamp("us", tz="UTC")), pa.list_(pa.date32()),
             # nested types
             pa.list_(pa.utf8()), pa.list_(pa.list_(pa.int32())), pa.large_list(pa.list_(pa.utf8())),
             pa.list_(pa.struct([pa.field("a", pa.int32()), pa.field("b", pa.utf8(), False)])),
             pa.list_(pa.map_(pa.utf8(), pa.utf8())), pa.map_(pa.int32(), pa.list_(pa.float64())),
             pa.map_(pa.utf8(), pa.utf8(), keys_sorted=True), pa.large_list(pa.bool_()),
             pa.struct([pa.field("a", pa.list_(pa.int32())), pa.field("s", pa.struct([pa.field("t", pa.bool_())]))])]
    rnd = random.Random(7)
    out = np.zeros(1 << 16, np.uint8)
    n = ctypes.c_int64(0)
    for _ in range(300):
        fields = []
        for i in range(rnd.randint(1, 24)):
            t = rnd.choice(types)
            name = "c%d_%s" % (i, "x" * rnd.randint(0, 13))
            fields.append(pa.field(name, t, True if t == pa.null() else rnd.random() < 0.7))
        want = pa.schema(fields).serialize().to_pybytes()
        assert lib.gz_debug_reencode_schema(want, len(want), out.ctypes.data, out.nbytes,
                                            ctypes.byref(n)) == 0
        assert out[: n.value].tobytes() == want, pa.schema(fields)


def test_make_rejects_bad_arguments_before_touching_the_device():
    """Splitter::Make's argument checks (splitter.cc:190-208, 219-221; key types of
    HashSplitter::CreateProjector) answer before any CUDA call, so they run without a GPU."""
    from gazelle_plugin_gb300 import workloads as W
    lib = S.lib()
    o = S.default_options()

    def make(short_name, P, schema, keys, null_keys=False, **opt):
        for k, v in opt.items():
            setattr(o, k, v)
        arr, names = S._fields(schema)
        ks = np.asarray(keys, np.int32)
        h = ctypes.c_int64(0)
        st = lib.gz_split_make_fields(short_name.encode(), P, arr, len(schema),
                                      None if null_keys else ks.ctypes.data, len(ks),
                                      ctypes.byref(o), ctypes.byref(h))
        o.buffer_size = 4096
        return st

    c1 = list(W.C1_SCHEMA)
    assert make("roundrobin", 4, c1, [0]) == S.GZ_NOT_IMPLEMENTED
    assert make("range", 4, [], []) == S.GZ_INVALID
    assert make("hash", 0, c1, [0]) == S.GZ_INVALID
    assert make("hash", 65537, c1, [0]) == S.GZ_INVALID
    assert make("rr", 4, c1, [], buffer_size=40000) == S.GZ_INVALID
    c1b = c1 + [W.Field("b", "binary"), W.Field("d", "decimal128")]
    assert make("hash", 4, c1b, [4]) == S.GZ_NOT_IMPLEMENTED  # binary key: no Spark-compatible hash here
    assert make("hash", 4, c1b, [5]) == S.GZ_NOT_IMPLEMENTED  # decimal key: neither
    assert make("hash", 4, c1, [9]) == S.GZ_INVALID          # key column out of range
    assert make("hash", 4, c1, [0], null_keys=True) == S.GZ_INVALID
