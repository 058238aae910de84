"""List columns of fixed-width elements (SplitListArray / AppendList, splitter.cc:1322-1344; the
builders' output finished by CacheRecordBatch, :532-545).

CPU: the oracle against fixtures made by the reference Splitter itself (list_columns.json,
tests/golden/make_golden.py), and its output read back by pyarrow as the input rows of each
partition in input order.  GPU: the CUDA splitter, through the C ABI, against those fixtures and
against the oracle with host and device-resident inputs over several passes, LZ4_FRAME output
and the error paths."""
import hashlib
import json
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import workloads as W
from oracle import ipc_read as R
from oracle import oracle as O
from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
LISTS = json.load(open(os.path.join(HERE, "golden", "list_columns.json")))["cases"]


def _schema(case):
    return [W.Field(*f) for f in case["schema"]]


@pytest.mark.parametrize("case", LISTS, ids=[c["name"] for c in LISTS])
def test_oracle_matches_reference_list_columns(case):
    batches = G.regenerate(case)
    assert G.input_digest(batches) == case["input_sha256"], "input generator changed"
    out = O.run_oracle(_schema(case), batches, case["num_partitions"], case["keys"], **case["options"])
    assert list(out.partition_lengths) == case["partition_lengths"]
    assert list(out.raw_partition_lengths) == case["raw_partition_lengths"]
    assert out.bytes_spilled == case["bytes_spilled"]
    assert hashlib.sha256(out.data).hexdigest() == case["data_sha256"]


def _wide(seed, nb=6, rows=4096, elem_nulls=0.05):
    """An int64 key, an int32, list<int32>, list<float64>, list<decimal128>, a utf8, list<bool>."""
    rng = np.random.default_rng(seed)
    schema = [W.Field("k", "int64", False), W.Field("i", "int32"), W.Field("a", "list", True, "int32"),
              W.Field("b", "list", True, "float64"), W.Field("d", "list", True, "decimal128"),
              W.Field("s", "utf8"), W.Field("q", "list", True, "bool")]
    out = []
    for _ in range(nb):
        bufs = W._column(rng, schema[0], rows, rng.integers(0, 1 << 40, size=rows), 0.0)
        bufs += W._column(rng, schema[1], rows, rng.integers(-9, 9, size=rows), 0.1)
        bufs += W.list_column(rng, schema[2], rows, 0.1, elem_nulls, 8)
        bufs += W.list_column(rng, schema[3], rows, 0.0, 0.0, 3)
        bufs += W.list_column(rng, schema[4], rows, 0.3, elem_nulls, 2)
        bufs += W._column(rng, schema[5], rows, None, 0.05, (0, 12, W.AZ))
        bufs += W.list_column(rng, schema[6], rows, 0.1, elem_nulls, 37)
        out.append(W.Batch(rows, bufs))
    return schema, out


def test_list_output_read_by_arrow_as_the_input_rows():
    pa = pytest.importorskip("pyarrow")
    schema, batches = _wide(3, nb=3, rows=1000)
    P = 7
    out = O.run_oracle(schema, batches, P, [0], buffer_size=256)
    o = O.OracleSplitter(schema, P, [0])
    pids = []
    for b in batches:
        o.split(b)
        pids.append(o.last_pids(b.num_rows))
    o.close()
    sch = O.to_pyarrow_schema(schema)
    head = sch.serialize().to_pybytes()
    # the input as Arrow arrays: each list column from its four buffers
    def arrays(b):
        cols, i = [], 0
        for f in schema:
            t = sch.field(f.name).type
            bufs = [pa.py_buffer(x.tobytes()) if x.nbytes else None for x in b.buffers[i:i + f.buffer_count]]
            n = b.num_rows
            if f.is_list:
                m = int(np.frombuffer(b.buffers[i + 1], np.int32)[-1])
                child = pa.Array.from_buffers(t.value_type, m, [bufs[2], bufs[3]])
                cols.append(pa.Array.from_buffers(t, n, [bufs[0], bufs[1]], children=[child]))
            else:
                cols.append(pa.Array.from_buffers(t, n, bufs))
            i += f.buffer_count
        return pa.record_batch(cols, schema=sch)
    table = pa.Table.from_batches([arrays(b) for b in batches])
    all_pids = np.concatenate(pids)
    for p in range(P):
        s = out.partition_bytes(p)
        got = pa.Table.from_batches(list(pa.ipc.open_stream(head + s)), schema=sch) if s else table.slice(0, 0)
        want = table.take(pa.array(np.nonzero(all_pids == p)[0]))
        assert got.equals(want), p


# ---------------------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", LISTS, ids=[c["name"] for c in LISTS])
def test_gpu_list_columns_golden(case):
    from gazelle_plugin_gb300 import shuffle as S
    o = case["options"]
    res, data = S.split_batches(_schema(case), G.regenerate(case), case["num_partitions"], case["keys"],
                                bufferSize=o.get("buffer_size", 4096), preferSpill=o.get("prefer_spill", True),
                                offheapPerTask=o.get("offheap_per_task", 0),
                                writeSchema=o.get("write_schema", False))
    assert list(res.partitionLengths) == case["partition_lengths"]
    assert list(res.rawPartitionLengths) == case["raw_partition_lengths"]
    assert res.totalBytesSpilled == case["bytes_spilled"]
    assert hashlib.sha256(data).hexdigest() == case["data_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("P", [1, 16, 200, 3000])
def test_gpu_list_columns_vs_oracle(P):
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _wide(40 + P)
    res, data = S.split_batches(schema, batches, P, [0], writeSchema=False)
    ref = O.run_oracle(schema, batches, P, [0])
    assert data == ref.data
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_list_columns_device_resident_many_passes():
    torch = pytest.importorskip("torch")
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _wide(51, nb=12)
    keep = []
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 200, None, [0], list(schema)), writeSchema=False,
               input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=1 << 20)
    for b in batches:
        ts = [torch.from_numpy(x.copy()).cuda() if x.nbytes else torch.zeros(0, dtype=torch.uint8).cuda()
              for x in b.buffers]
        keep += ts
        w.split(h, b.num_rows, [t.data_ptr() if t.numel() else 0 for t in ts], [t.numel() for t in ts])
    assert w.stats(h)[0] >= 3
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(schema, batches, 200, [0])
    assert data == ref.data
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_list_columns_lz4():
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _wide(61, nb=4)
    P = 16
    res_u, data_u = S.split_batches(schema, batches, P, [0], writeSchema=False)
    res_z, data_z = S.split_batches(schema, batches, P, [0], writeSchema=False, codec="lz4")
    assert np.array_equal(res_u.rawPartitionLengths, res_z.rawPartitionLengths)
    su = np.concatenate([[0], np.cumsum(np.asarray(res_u.partitionLengths))])
    sz = np.concatenate([[0], np.cumsum(np.asarray(res_z.partitionLengths))])
    for p in range(P):
        bu = R.parse_stream(data_u[su[p]:su[p + 1]], schema)
        bz = R.parse_stream(data_z[sz[p]:sz[p + 1]], schema)
        assert [r for r, _ in bu] == [r for r, _ in bz]
        for (_, cu), (_, cz) in zip(bu, bz):
            assert [(f[0], f[2:], [bytes(x) for x in f[1]]) for f in cu] == \
                   [(f[0], f[2:], [bytes(x) for x in f[1]]) for f in cz]


@pytest.mark.gpu
def test_gpu_list_column_rejections():
    from gazelle_plugin_gb300 import shuffle as S
    w = S.ShuffleSplitterJniWrapper()
    schema = [W.Field("k", "int32", False), W.Field("a", "list", True, "int32")]
    with pytest.raises(S.SplitterError) as e:  # a list key: the fork's generic hash32
        w.make(S.NativePartitioning("hash", 4, None, [1], list(schema)), writeSchema=False)
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    h = w.make(S.NativePartitioning("hash", 4, None, [0], list(schema)), writeSchema=False)
    keys = np.arange(8, dtype=np.int32)
    offs = np.arange(9, dtype=np.int32) * 2
    offs[8] = 100  # beyond the 16 elements given
    vals = np.zeros(16, np.int32)
    with pytest.raises(S.SplitterError) as e:
        w.split(h, 8, [0, keys.ctypes.data, 0, offs.ctypes.data, 0, vals.ctypes.data],
                [0, keys.nbytes, 0, offs.nbytes, 0, vals.nbytes])
    assert e.value.status == S.GZ_INVALID
    w.close(h)


# ---------------------------------------------------------------------------------- reduce side
def _streams(outs, p):
    return [o.partition_bytes(p) for o in outs]


def test_oracle_reader_concatenates_list_columns_like_arrow():
    pa = pytest.importorskip("pyarrow")
    schema, _ = _wide(0, nb=1, rows=10)
    outs = [O.run_oracle(schema, _wide(70 + s, nb=2, rows=700)[1], 5, [0], buffer_size=128) for s in range(3)]
    sch = O.to_pyarrow_schema(schema)
    head = sch.serialize().to_pybytes()
    for p in range(5):
        streams = _streams(outs, p)
        rows, cols = R.read_partition(schema, streams)
        bs = [b for s in streams if s for b in pa.ipc.open_stream(head + s)]
        t = pa.Table.from_batches(bs, schema=sch).combine_chunks()
        assert t.num_rows == rows
        for fi, f in enumerate(schema):
            if not f.is_list:
                continue
            col = t.column(fi).chunks[0]
            valid, offs, (evalid, vals) = cols[fi]
            assert (valid is None) == (col.null_count == 0)
            o = np.asarray(col.offsets)
            assert np.array_equal(offs, o - o[0])
            child = col.values.slice(o[0], o[-1] - o[0])
            assert (evalid is None) == (child.null_count == 0)
            if evalid is not None:
                assert np.array_equal(evalid, child.is_valid().to_numpy(zero_copy_only=False))
            if f.elem == "bool":
                bits = np.unpackbits(np.frombuffer(child.buffers()[1], np.uint8), bitorder="little")
                assert np.array_equal(vals, bits[child.offset:child.offset + len(child)].astype(bool))
                continue
            w = W.BYTE_WIDTH[f.elem]
            assert vals == child.buffers()[1].to_pybytes()[child.offset * w:(child.offset + len(child)) * w]


@pytest.mark.gpu
@pytest.mark.parametrize("codec", [None, "lz4"])
def test_gpu_reader_list_columns(codec):
    from gazelle_plugin_gb300 import shuffle as S
    P = 16
    outs = []
    for seed in (81, 82, 83):
        schema, batches = _wide(seed, nb=3)
        kw = {"codec": codec} if codec else {}
        res, data = S.split_batches(schema, batches, P, [0], writeSchema=bool(seed % 2), **kw)
        st = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
        outs.append([data[st[p]:st[p + 1]] for p in range(P)])
    for p in range(P):
        streams = [o[p] for o in outs]
        rows, cols = R.read_partition(schema, streams)
        r = S.PartitionReader(list(schema))
        for s in streams:
            r.addStream(s)
        assert r.finish()[0] == rows
        for fi, f in enumerate(schema):
            valid, offs, vals = cols[fi]
            gv, go, gvals = r.column_to_host(fi)
            assert (gv is None) == (valid is None)
            if valid is not None:
                assert gv.tobytes() == R.pack_bits(valid)
            if f.is_list:
                evalid, vals = vals
                assert np.array_equal(go, offs)
                ge = r.element_validity_to_host(fi)
                assert (ge is None) == (evalid is None)
                if evalid is not None:
                    assert ge.tobytes() == R.pack_bits(evalid)
            elif f.is_binary:
                assert np.array_equal(go, offs)
            if f.is_list and f.elem == "bool":
                vals = R.pack_bits(vals)
            assert gvals.tobytes() == vals
        r.close()
