"""Reduce-side read: a partition's IPC streams (its bytes of several map outputs' data files)
concatenated into one set of Arrow columns.

CPU: the oracle's reader (oracle/ipc_read.py) against pyarrow's IPC stream reader and
concat_batches on streams the oracle splitter wrote.  GPU: the CUDA reader (gz_reader_*, through
the C ABI) against the oracle's reader, byte for byte, on streams written by the oracle and by the
CUDA splitter, with and without the schema message, one or several streams per partition, empty
streams, and the error paths."""
import numpy as np
import pytest

from gazelle_plugin_gb300 import workloads as W
from oracle import ipc_read as R
from oracle import oracle as O


def map_outputs(schema, keys, P, seeds, make, write_schema=False, **opts):
    """Oracle splits of several map tasks' batches: [SplitOutput]."""
    return [O.run_oracle(schema, make(s), P, keys, write_schema=write_schema, **opts) for s in seeds]


def c1_make(seed):
    return W.c1_batches(seed, 6, 3000)


def c2_make(seed):
    return W.c2_batches(seed, 5, 4096)


def streams_of(outputs, p):
    return [o.partition_bytes(p) for o in outputs]


# ---------------------------------------------------------------------------------------- CPU
def _pyarrow_concat(schema, streams):
    pa = pytest.importorskip("pyarrow")
    sch = O.to_pyarrow_schema(schema)
    head = sch.serialize().to_pybytes()
    batches = []
    for s in streams:
        if not s:
            continue
        data = s if s[:8] == head[:8] and s.startswith(head) else head + s
        batches += list(pa.ipc.open_stream(data))
    return pa.Table.from_batches(batches, schema=sch).combine_chunks()


@pytest.mark.parametrize("write_schema", [False, True])
@pytest.mark.parametrize("which", ["c1", "c2"])
def test_oracle_reader_matches_pyarrow(which, write_schema):
    pytest.importorskip("pyarrow")
    schema, keys, P, make = ((W.C1_SCHEMA, W.C1_KEYS, 8, c1_make) if which == "c1"
                             else (W.C2_SCHEMA, W.C2_KEYS, 16, c2_make))
    outs = map_outputs(schema, keys, P, [1, 2, 3], make, write_schema=write_schema, buffer_size=1024)
    for p in range(P):
        streams = streams_of(outs, p)
        rows, cols = R.read_partition(schema, streams)
        t = _pyarrow_concat(schema, streams)
        assert t.num_rows == rows
        for fi, f in enumerate(schema):
            col = t.column(fi).chunks[0] if t.num_rows else None
            valid, offs, vals = cols[fi]
            if col is None:
                continue
            assert (valid is None) == (col.null_count == 0)
            if valid is not None:
                assert np.array_equal(valid, col.is_valid().to_numpy(zero_copy_only=False))
            bufs = col.buffers()
            if f.type == "bool":
                assert np.array_equal(vals, np.unpackbits(np.frombuffer(bufs[1], np.uint8), bitorder="little")
                                      [col.offset:col.offset + rows].astype(bool))
            elif f.is_binary:
                o = np.frombuffer(bufs[1], np.int32)[col.offset:col.offset + rows + 1]
                assert np.array_equal(offs, o - o[0])
                assert vals == bufs[2].to_pybytes()[o[0]:o[-1]]
            else:
                w = R.BYTE_WIDTH[f.type]
                assert vals == bufs[1].to_pybytes()[col.offset * w:(col.offset + rows) * w]


# ---------------------------------------------------------------------------------------- GPU
def _gpu_read(schema, streams):
    from gazelle_plugin_gb300 import shuffle as S
    r = S.PartitionReader(list(schema))
    try:
        for s in streams:
            r.addStream(s)
        rows, nb = r.finish()
        return rows, nb, [r.column_to_host(i) for i in range(len(schema))]
    finally:
        r.close()


def _check(schema, streams):
    rows, cols = R.read_partition(schema, streams)
    grows, _, gcols = _gpu_read(schema, streams)
    assert grows == rows
    for fi, f in enumerate(schema):
        valid, offs, vals = cols[fi]
        gv, go, gvals = gcols[fi]
        if f.type == "null":
            continue
        assert (gv is None) == (valid is None), f.name
        if valid is not None:
            assert gv.tobytes() == R.pack_bits(valid), f.name
        if f.type == "bool":
            assert gvals.tobytes() == R.pack_bits(vals), f.name
        elif f.is_binary:
            assert np.array_equal(go, offs), f.name
            assert gvals.tobytes() == vals, f.name
        else:
            assert gvals.tobytes() == vals, f.name


@pytest.mark.gpu
def test_gpu_reader_matches_oracle_on_oracle_streams():
    outs = map_outputs(W.C1_SCHEMA, W.C1_KEYS, 8, [4, 5, 6], c1_make, buffer_size=700)
    for p in range(8):
        _check(W.C1_SCHEMA, streams_of(outs, p))


@pytest.mark.gpu
def test_gpu_reader_streams_with_schema_message():
    """The splitter's streams with write_schema: a schema message before each partition's batches."""
    from gazelle_plugin_gb300 import shuffle as S
    P = 8
    outs = []
    for seed in (11, 12):
        res, data = S.split_batches(W.C1_SCHEMA, c1_make(seed), P, W.C1_KEYS, writeSchema=True, bufferSize=900)
        starts = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
        outs.append([data[starts[p]:starts[p + 1]] for p in range(P)])
    for p in range(P):
        _check(W.C1_SCHEMA, [o[p] for o in outs])


@pytest.mark.gpu
def test_gpu_reader_on_cuda_splitter_streams_of_many_map_outputs():
    from gazelle_plugin_gb300 import shuffle as S
    P = 200
    outs = []
    for seed in (7, 8, 9, 10):
        res, data = S.split_batches(W.C2_SCHEMA, c2_make(seed), P, W.C2_KEYS, writeSchema=False)
        lens = np.asarray(res.partitionLengths)
        starts = np.concatenate([[0], np.cumsum(lens)])
        outs.append([data[starts[p]:starts[p + 1]] for p in range(P)])
    for p in range(0, P, 7):
        _check(W.C2_SCHEMA, [o[p] for o in outs])


@pytest.mark.gpu
def test_gpu_readers_on_concurrent_threads():
    """Eight reduce tasks at once, each on its own thread with its own readers (as the benchmark's
    reduce side runs them): every partition equal to the oracle's reading."""
    from concurrent.futures import ThreadPoolExecutor
    from gazelle_plugin_gb300 import shuffle as S
    P = 64
    outs = []
    for seed in (21, 22, 23):
        res, data = S.split_batches(W.C2_SCHEMA, c2_make(seed), P, W.C2_KEYS, writeSchema=False)
        starts = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
        outs.append([data[starts[p]:starts[p + 1]] for p in range(P)])

    def task(ps):
        for p in ps:
            _check(W.C2_SCHEMA, [o[p] for o in outs])
        return len(ps)

    with ThreadPoolExecutor(max_workers=8) as ex:
        assert sum(ex.map(task, [list(range(P))[i::8] for i in range(8)])) == P


@pytest.mark.gpu
def test_gpu_reader_random_schemas_bool_and_empty_streams():
    rng = np.random.default_rng(12)
    for trial in range(6):
        schema = W.random_schema(rng, int(rng.integers(1, 8)))
        keys = [0]
        if schema[0].type in ("null", "utf8", "binary", "uint8", "uint16", "uint32", "uint64", "float16",
                              "date64", "time32", "time64", "timestamp", "decimal128"):
            schema = [W.Field("k", "int32")] + list(schema)
        batches = [W.random_batch(rng, schema, int(rng.integers(1, 2000)), 0.1) for _ in range(3)]
        out = O.run_oracle(schema, batches, 4, keys, buffer_size=int(rng.integers(64, 1024)))
        for p in range(4):
            streams = [out.partition_bytes(p), b"", out.partition_bytes(p)]
            _check(schema, streams)


@pytest.mark.gpu
def test_gpu_reader_errors():
    from gazelle_plugin_gb300 import shuffle as S
    out = O.run_oracle(W.C1_SCHEMA, c1_make(3), 8, W.C1_KEYS)
    s = out.partition_bytes(0)
    r = S.PartitionReader(list(W.C1_SCHEMA))
    with pytest.raises(S.SplitterError) as e:
        r.addStream(s[:(len(s) // 2) | 3])  # cut inside a message (messages are multiples of 8)
    assert e.value.status == S.GZ_INVALID
    r.addStream(s)
    assert r.finish()[0] > 0
    with pytest.raises(S.SplitterError):
        r.addStream(s)  # finished
    r.close()
