"""Nested columns of any depth: list / large_list / map / struct over fixed-width, bool, binary and
nested children (list_array_idx_ columns split by SplitListArray / AppendList,
splitter.cc:1322-1344, through the Arrow builders' AppendArraySlice; finished by
CacheRecordBatch, :532-545).

CPU: the oracle against fixtures made by the reference Splitter itself (nested_columns.json,
tests/golden/make_golden.py: the unit tests' shapes, shuffle_split_test.cc:509-1060, and more),
and its output read back by pyarrow as the input rows of each partition in input order."""
import hashlib
import json
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O
from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
NESTED = json.load(open(os.path.join(HERE, "golden", "nested_columns.json")))["cases"]


def _schema(case):
    return [G.field_from_json(f) for f in case["schema"]]


@pytest.mark.parametrize("case", NESTED, ids=[c["name"] for c in NESTED])
def test_oracle_matches_reference_nested_columns(case):
    batches = G.regenerate(case)
    assert G.input_digest(batches) == case["input_sha256"], "input generator changed"
    out = O.run_oracle(_schema(case), batches, case["num_partitions"], case["keys"], **case["options"])
    assert list(out.partition_lengths) == case["partition_lengths"]
    assert list(out.raw_partition_lengths) == case["raw_partition_lengths"]
    assert out.bytes_spilled == case["bytes_spilled"]
    assert hashlib.sha256(out.data).hexdigest() == case["data_sha256"]


def _random_case(seed, nb=3, rows=600):
    """An int key and 1-3 random nested fields (random_nested_field), batches of random length."""
    rng = np.random.default_rng(seed)
    schema = [W.Field("k", "int64", False)] + [W.random_nested_field(rng, f"N{i}")
                                                 for i in range(int(rng.integers(1, 4)))]
    spans = bool(rng.random() < 0.5)
    batches = []
    for _ in range(nb):
        n = int(rng.integers(1, rows))
        bufs = W._column(rng, schema[0], n, rng.integers(0, 1 << 40, size=n), 0.0)
        for f in schema[1:]:
            bufs += W.nested_column(rng, f, n, float(rng.choice([0.0, 0.1, 0.5])), int(rng.choice([1, 3, 6])),
                                    True, spans)
        batches.append(W.Batch(n, bufs))
    return schema, batches


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_live_reference_on_random_nested_schemas(seed):
    if not O.RefSplitter.available():
        pytest.skip("reference build not available")
    schema, batches = _random_case(7000 + seed)
    P = [1, 5, 64][seed % 3]
    a = O.run_oracle(schema, batches, P, [0], buffer_size=[16, 100, 4096][seed % 3])
    b = O.run_ref(schema, batches, P, [0], buffer_size=[16, 100, 4096][seed % 3])
    assert a.data == b.data
    assert list(a.raw_partition_lengths) == list(b.raw_partition_lengths)


def _arrow_array(pa, f, t, bufs, at, n):
    """The Arrow array of field f (type t) from the flat buffer list at `at`; returns it and the
    next buffer index."""
    def buf(i, validity=False):
        return pa.py_buffer(bufs[i].tobytes()) if bufs[i].nbytes else (None if validity else pa.py_buffer(b""))

    if f.type in ("list", "large_list", "map"):
        offs = np.frombuffer(bufs[at + 1], np.int64 if f.type == "large_list" else np.int32)
        m = int(offs[n]) if n else 0
        own = [buf(at, True), buf(at + 1)]
        at += 2
        if f.type == "map":
            st = pa.struct([t.key_field, t.item_field])
            at += 1  # the entries struct's validity (dropped)
            key, at = _arrow_array(pa, f.kids[0], t.key_type, bufs, at, m)
            item, at = _arrow_array(pa, f.kids[1], t.item_type, bufs, at, m)
            entries = pa.Array.from_buffers(st, m, [None], children=[key, item])
            return pa.Array.from_buffers(t, n, own, children=[entries]), at
        child, at = _arrow_array(pa, f.kids[0], t.value_type, bufs, at, m)
        return pa.Array.from_buffers(t, n, own, children=[child]), at
    if f.type == "struct":
        own = [buf(at, True)]
        at += 1
        kids = []
        for k, kf in zip(f.kids, t):
            a, at = _arrow_array(pa, k, kf.type, bufs, at, n)
            kids.append(a)
        return pa.Array.from_buffers(t, n, own, children=kids), at
    nb = f.buffer_count
    return pa.Array.from_buffers(t, n, [buf(at + j, j == 0) for j in range(nb)]), at + nb


def test_nested_output_read_by_arrow_as_the_input_rows():
    pa = pytest.importorskip("pyarrow")
    for seed in (6000, 6003, 6007, 6012):
        schema, batches, P, keys, opts = G.nested_case(seed)
        o = O.OracleSplitter(schema, P, keys, **opts)
        pids = []
        for b in batches:
            o.split(b)
            pids.append(o.last_pids(b.num_rows))
        out = o.stop()
        o.close()
        sch = O.to_pyarrow_schema(schema)
        head = sch.serialize().to_pybytes()
        rbs = []
        for b in batches:
            cols, at = [], 0
            for f in schema:
                a, at = _arrow_array(pa, f, sch.field(f.name).type, b.buffers, at, b.num_rows)
                cols.append(a)
            rbs.append(pa.record_batch(cols, schema=sch))
        table = pa.Table.from_batches(rbs)
        all_pids = np.concatenate(pids)
        for p in range(P):
            s = out.partition_bytes(p)
            got = pa.Table.from_batches(list(pa.ipc.open_stream(head + s)), schema=sch) if s else table.slice(0, 0)
            want = table.take(pa.array(np.nonzero(all_pids == p)[0]))
            assert got.equals(want), (seed, p)


def test_oracle_refuses_unsupported_nested_types():
    F = W.Field
    for bad in (F("n", "list", True, None, (F("item", "null"),)),
                F("n", "struct", True, None, ())):
        with pytest.raises(ValueError):
            O.OracleSplitter([F("k", "int32", False), bad], 4, [0])


# ---------------------------------------------------------------------------------------- GPU
def _all_shapes(seed, nb=4, rows=3000, spans=True):
    """An int64 key and one column of every nested shape of the fixtures."""
    rng = np.random.default_rng(seed)
    schema = [W.Field("k", "int64", False)] + [G.NESTED_SHAPES[i](f"N{i}") for i in range(len(G.NESTED_SHAPES))]
    batches = []
    for _ in range(nb):
        n = int(rng.integers(rows // 2, rows + 1))
        bufs = W._column(rng, schema[0], n, rng.integers(0, 1 << 40, size=n), 0.0)
        for f in schema[1:]:
            bufs += W.nested_column(rng, f, n, 0.15, 4, True, spans)
        batches.append(W.Batch(n, bufs))
    return schema, batches


@pytest.mark.gpu
@pytest.mark.parametrize("case", NESTED, ids=[c["name"] for c in NESTED])
def test_gpu_nested_columns_golden(case):
    """The fixture's data file, lengths and spills; and every batch's body length under no codec
    (split with firstRecordBatch: Splitter::CompressedSize, splitter.cc:358-369)."""
    from gazelle_plugin_gb300 import shuffle as S
    o = case["options"]
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", case["num_partitions"], None, case["keys"], _schema(case)),
               bufferSize=o.get("buffer_size", 4096), preferSpill=o.get("prefer_spill", True),
               offheapPerTask=o.get("offheap_per_task", 0), writeSchema=o.get("write_schema", False))
    try:
        bodies = []
        for b in G.regenerate(case):
            a, z = b.addrs_sizes()
            bodies.append(w.split(h, b.num_rows, a, z, True))
            w.split(h, b.num_rows, a, z)
        res = w.stop(h)
        data = w.data(h)
    finally:
        w.close(h)
    assert bodies == case["body_lengths"]
    assert list(res.partitionLengths) == case["partition_lengths"]
    assert list(res.rawPartitionLengths) == case["raw_partition_lengths"]
    assert res.totalBytesSpilled == case["bytes_spilled"]
    assert hashlib.sha256(data).hexdigest() == case["data_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("P", [1, 7, 200, 3000])
def test_gpu_nested_columns_vs_oracle(P):
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _all_shapes(80 + P)
    res, data = S.split_batches(schema, batches, P, [0], writeSchema=False)
    ref = O.run_oracle(schema, batches, P, [0])
    assert data == ref.data
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(12))
def test_gpu_random_nested_schemas_vs_oracle(seed):
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _random_case(7000 + seed)
    P = [1, 5, 64][seed % 3]
    bs = [16, 100, 4096][seed % 3]
    res, data = S.split_batches(schema, batches, P, [0], writeSchema=False, bufferSize=bs)
    ref = O.run_oracle(schema, batches, P, [0], buffer_size=bs)
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
@pytest.mark.parametrize("null_frac,max_len", [(1.0, 3), (0.0, 0), (0.5, 0), (1.0, 0)])
def test_gpu_nested_columns_all_null_and_empty(null_frac, max_len):
    """Columns whose entries are all null, or whose lists / maps / strings are all empty (empty
    child buffers), single-row batches among them."""
    from gazelle_plugin_gb300 import shuffle as S
    rng = np.random.default_rng(int(null_frac * 10) + max_len)
    schema = [W.Field("k", "int64", False)] + [G.NESTED_SHAPES[i](f"N{i}") for i in range(len(G.NESTED_SHAPES))]
    batches = []
    for n in (1, 700, 1, 2500):
        bufs = W._column(rng, schema[0], n, rng.integers(0, 1 << 40, size=n), 0.0)
        for f in schema[1:]:
            bufs += W.nested_column(rng, f, n, null_frac, max_len)
        batches.append(W.Batch(n, bufs))
    res, data = S.split_batches(schema, batches, 13, [0], writeSchema=False)
    ref = O.run_oracle(schema, batches, 13, [0])
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
@pytest.mark.parametrize("short_name", ["rr", "single", "range"])
def test_gpu_nested_columns_other_partitioners(short_name):
    """Round-robin, single and range (int32 partition ids in field 0, not written out) with nested
    columns beside them."""
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _all_shapes(121, nb=3, rows=2000)
    P = 9
    if short_name == "range":
        rng = np.random.default_rng(5)
        schema = [W.Field("pid", "int32", False)] + schema
        batches = [W.Batch(b.num_rows, [np.zeros(0, np.uint8),
                                        rng.integers(0, P, size=b.num_rows).astype(np.int32).view(np.uint8)]
                           + b.buffers) for b in batches]
    keys = [0] if short_name == "range" else []
    res, data = S.split_batches(schema, batches, P, keys, shortName=short_name, writeSchema=False)
    ref = O.run_oracle(schema, batches, P, keys, short_name=short_name)
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_nested_columns_cpu_copy_staging_many_passes():
    """Host inputs copied by the CPU into pinned staging (GZ_HOST_READ_CPU_COPY) instead of read by
    the device, over many passes, through the batched call."""
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _all_shapes(95, nb=6)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 33, None, [0], list(schema)), writeSchema=False,
               host_read=S.GZ_HOST_READ_CPU_COPY, flush_bytes=1 << 18)
    for b in batches:
        a, z = b.addrs_sizes()
        w.splitBatches(h, [b.num_rows], a[None, :], z[None, :])
    assert w.stats(h)[0] >= 3
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(schema, batches, 33, [0])
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_nested_columns_device_resident_many_passes():
    torch = pytest.importorskip("torch")
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _all_shapes(91, nb=10)
    keep = []
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 64, None, [0], list(schema)), writeSchema=False,
               input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=1 << 18)
    for b in batches:
        ts = [torch.from_numpy(x.copy()).cuda() if x.nbytes else torch.zeros(0, dtype=torch.uint8).cuda()
              for x in b.buffers]
        keep += ts
        w.split(h, b.num_rows, [t.data_ptr() if t.numel() else 0 for t in ts], [t.numel() for t in ts])
    assert w.stats(h)[0] >= 3
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(schema, batches, 64, [0])
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_nested_columns_lz4():
    from gazelle_plugin_gb300 import shuffle as S
    from oracle import ipc_read as R
    schema, batches = _all_shapes(93, nb=3)
    P = 12
    res_u, data_u = S.split_batches(schema, batches, P, [0], writeSchema=False)
    res_z, data_z = S.split_batches(schema, batches, P, [0], writeSchema=False, codec="lz4")
    assert np.array_equal(res_u.rawPartitionLengths, res_z.rawPartitionLengths)
    su = np.concatenate([[0], np.cumsum(np.asarray(res_u.partitionLengths))])
    sz = np.concatenate([[0], np.cumsum(np.asarray(res_z.partitionLengths))])
    for p in range(P):
        assert R.parse_stream_raw(data_u[su[p]:su[p + 1]]) == R.parse_stream_raw(data_z[sz[p]:sz[p + 1]])


@pytest.mark.gpu
def test_gpu_nested_rejections():
    """A null entry below a list holding elements (its builder would drop them) and nested keys
    are refused."""
    from gazelle_plugin_gb300 import shuffle as S
    F = W.Field
    lst = F("a", "list", True, None, (F("item", "list", True, "int32"),))
    schema = [F("k", "int32", False), lst]
    w = S.ShuffleSplitterJniWrapper()
    with pytest.raises(S.SplitterError) as e:
        w.make(S.NativePartitioning("hash", 4, None, [1], list(schema)), writeSchema=False)
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    h = w.make(S.NativePartitioning("hash", 4, None, [0], list(schema)), writeSchema=False)
    keys = np.arange(2, dtype=np.int32)
    offs = np.array([0, 1, 2], np.int32)              # each row: one inner list
    inner_valid = np.array([0b01], np.uint8)          # the second inner list is null ...
    inner_offs = np.array([0, 1, 3], np.int32)        # ... and holds two elements
    vals = np.arange(3, dtype=np.int32)
    bufs = [np.zeros(0, np.uint8), keys, np.zeros(0, np.uint8), offs, inner_valid, inner_offs,
            np.zeros(0, np.uint8), vals]
    addrs = [b.ctypes.data if b.nbytes else 0 for b in bufs]
    with pytest.raises(S.SplitterError) as e:
        w.split(h, 2, addrs, [b.nbytes for b in bufs])
        w.stop(h)
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    w.close(h)


# ---------------------------------------------------------------------------------------- reader
def _arrow_nodes(pa, arr):
    """Pre-order nodes of an Arrow array in read_partition_nodes' form."""
    t = arr.type
    n = len(arr)
    nulls = arr.null_count
    valid = arr.is_valid().to_numpy(zero_copy_only=False) if nulls else None
    if pa.types.is_struct(t):
        out = [(n, nulls, valid, None, b"")]
        for i in range(t.num_fields):
            out += _arrow_nodes(pa, arr.field(i))
        return out
    if pa.types.is_list(t) or pa.types.is_large_list(t) or pa.types.is_map(t):
        o = np.asarray(arr.offsets)
        offs = (o - o[0]).astype(np.int64 if pa.types.is_large_list(t) else np.int32)
        child = arr.values.slice(int(o[0]), int(o[-1] - o[0]))
        out = [(n, nulls, valid, offs, b"")]
        if pa.types.is_map(t):  # the entries struct, then key and value
            out.append((len(child), 0, None, None, b""))
            out += _arrow_nodes(pa, child.field(0)) + _arrow_nodes(pa, child.field(1))
        else:
            out += _arrow_nodes(pa, child)
        return out
    if pa.types.is_binary(t) or pa.types.is_string(t) or pa.types.is_large_binary(t) or pa.types.is_large_string(t):
        big = pa.types.is_large_binary(t) or pa.types.is_large_string(t)
        o = np.frombuffer(arr.buffers()[1], np.int64 if big else np.int32)[arr.offset:arr.offset + n + 1]
        data = arr.buffers()[2].to_pybytes() if arr.buffers()[2] is not None else b""
        return [(n, nulls, valid, (o - o[0]).astype(np.int64 if big else np.int32), data[int(o[0]):int(o[-1])])]
    if pa.types.is_boolean(t):
        bits = np.unpackbits(np.frombuffer(arr.buffers()[1], np.uint8), bitorder="little")
        return [(n, nulls, valid, None, bits[arr.offset:arr.offset + n].astype(bool))]
    w = t.bit_width // 8
    return [(n, nulls, valid, None, arr.buffers()[1].to_pybytes()[arr.offset * w:(arr.offset + n) * w])]


def _same_nodes(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x[0] == y[0] and x[1] == y[1]
        assert (x[2] is None) == (y[2] is None) and (x[2] is None or np.array_equal(x[2], y[2]))
        assert (x[3] is None) == (y[3] is None) and (x[3] is None or np.array_equal(x[3], y[3]))
        if isinstance(x[4], np.ndarray) or isinstance(y[4], np.ndarray):
            assert np.array_equal(np.asarray(x[4], bool), np.asarray(y[4], bool))
        else:
            assert x[4] == y[4]


def test_oracle_reader_concatenates_nested_columns_like_arrow():
    pa = pytest.importorskip("pyarrow")
    from oracle import ipc_read as R
    schema, _ = _all_shapes(0, nb=1, rows=10)
    outs = [O.run_oracle(schema, _all_shapes(100 + s, nb=2, rows=400)[1], 5, [0], buffer_size=128)
            for s in range(3)]
    sch = O.to_pyarrow_schema(schema)
    head = sch.serialize().to_pybytes()
    for p in range(5):
        streams = [o.partition_bytes(p) for o in outs]
        got = R.read_partition_nodes(schema, streams)
        bs = [b for s in streams if s for b in pa.ipc.open_stream(head + s)]
        t = pa.Table.from_batches(bs, schema=sch).combine_chunks()
        for fi in range(len(schema)):
            col = t.column(fi).chunks[0] if t.num_rows else pa.array([], sch.field(fi).type)
            _same_nodes(got[fi], _arrow_nodes(pa, col))


@pytest.mark.gpu
@pytest.mark.parametrize("codec", [None, "lz4"])
def test_gpu_reader_nested_columns(codec):
    from gazelle_plugin_gb300 import shuffle as S
    from oracle import ipc_read as R
    P = 9
    outs = []
    for seed in (111, 112, 113):
        schema, batches = _all_shapes(seed, nb=2, rows=1500)
        kw = {"codec": codec} if codec else {}
        res, data = S.split_batches(schema, batches, P, [0], writeSchema=bool(seed % 2), **kw)
        st = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
        outs.append([data[st[p]:st[p + 1]] for p in range(P)])
    for p in range(P):
        streams = [o[p] for o in outs]
        want = R.read_partition_nodes(schema, streams)
        r = S.PartitionReader(list(schema))
        for s in streams:
            r.addStream(s)
        r.finish()
        for fi in range(len(schema)):
            assert r.node_count(fi) == len(want[fi])
            for q, (length, nulls, valid, offs, vals) in enumerate(want[fi]):
                gl, gn, gv, go, gvals = r.node_to_host(fi, q)
                assert (gl, gn) == (length, nulls), (p, fi, q)
                assert (gv is None) == (valid is None)
                if valid is not None:
                    assert gv.tobytes() == R.pack_bits(valid)
                assert (go is None) == (offs is None)
                if offs is not None:
                    assert np.array_equal(go, offs)
                want_vals = R.pack_bits(vals) if isinstance(vals, np.ndarray) else vals
                assert gvals.tobytes() == want_vals, (p, fi, q)
        r.close()
