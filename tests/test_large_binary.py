"""large_utf8 / large_binary columns (64-bit offsets, the reference's
SplitBinaryType<LargeBinaryType::offset_type>, splitter.cc:1291-1299, and the offset widths of
CacheRecordBatch / AllocatePartitionBuffers, splitter.cc:476-529, 619-660).

CPU: the oracle against fixtures made by the reference Splitter itself (large_binary.json,
tests/golden/make_golden.py), and its output read back by pyarrow's IPC reader.  GPU: the CUDA
splitter, through the C ABI, against those fixtures and against the oracle with host and
device-resident inputs, LZ4_FRAME output, and the reduce-side reader; the error paths."""
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
LARGE = json.load(open(os.path.join(HERE, "golden", "large_binary.json")))["cases"]


def _schema(case):
    return [W.Field(n, t, nl) for n, t, nl in case["schema"]]


def _check_case(case, data, partition_lengths, raw_lengths):
    assert list(partition_lengths) == case["partition_lengths"]
    assert list(raw_lengths) == case["raw_partition_lengths"]
    assert hashlib.sha256(data).hexdigest() == case["data_sha256"]


@pytest.mark.parametrize("case", LARGE, ids=[c["name"] for c in LARGE])
def test_oracle_matches_reference_large_binary(case):
    batches = G.regenerate(case)
    assert G.input_digest(batches) == case["input_sha256"], "input generator changed"
    out = O.run_oracle(_schema(case), batches, case["num_partitions"], case["keys"], **case["options"])
    _check_case(case, out.data, out.partition_lengths, out.raw_partition_lengths)
    assert out.bytes_spilled == case["bytes_spilled"]


def test_large_binary_cases_hold_64_bit_columns():
    assert all(any(f[1].startswith("large_") for f in c["schema"]) for c in LARGE)
    # every 64-bit binary column before every 32-bit one (where the reference is well defined)
    for c in LARGE:
        kinds = [f[1].startswith("large_") for f in c["schema"] if f[1] in
                 ("utf8", "binary", "large_utf8", "large_binary")]
        assert kinds == sorted(kinds, reverse=True)


def test_large_binary_output_read_by_arrow():
    pa = pytest.importorskip("pyarrow")
    schema, batches, P, keys, opts = G.large_case(4003)
    out = O.run_oracle(schema, batches, P, keys, **opts)
    sch = O.to_pyarrow_schema(schema)
    head = sch.serialize().to_pybytes()
    for p in range(P):
        s = out.partition_bytes(p)
        if not s:
            continue
        t = pa.Table.from_batches(list(pa.ipc.open_stream(head + s)), schema=sch).combine_chunks()
        rows, cols = R.read_partition(schema, [s])
        assert t.num_rows == rows
        for fi, f in enumerate(schema):
            if not f.is_binary:
                continue
            col = t.column(fi).chunks[0]
            bufs = col.buffers()
            o = np.frombuffer(bufs[1], f.offset_dtype)[col.offset:col.offset + rows + 1]
            assert np.array_equal(cols[fi][1], o - o[0])
            assert cols[fi][2] == bufs[2].to_pybytes()[o[0]:o[-1]]


# ---------------------------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", LARGE, ids=[c["name"] for c in LARGE])
def test_gpu_large_binary_golden(case):
    from gazelle_plugin_gb300 import shuffle as S
    o = case["options"]
    res, data = S.split_batches(_schema(case), G.regenerate(case), case["num_partitions"], case["keys"],
                                bufferSize=o.get("buffer_size", 4096), preferSpill=o.get("prefer_spill", True),
                                offheapPerTask=o.get("offheap_per_task", 0),
                                writeSchema=o.get("write_schema", False))
    _check_case(case, data, res.partitionLengths, res.rawPartitionLengths)
    assert res.totalBytesSpilled == case["bytes_spilled"]


def _large_wide(seed, nb, rows):
    """An int64 key, an int32, two large_utf8 columns of 0-80 characters and a large_binary
    column of 0-8 bytes (nulls in the payload), plus a utf8 column after them."""
    rng = np.random.default_rng(seed)
    schema = [W.Field("k", "int64", False), W.Field("a", "large_utf8"), W.Field("i", "int32"),
              W.Field("b", "large_utf8"), W.Field("c", "large_binary"), W.Field("s", "utf8")]
    out = []
    for _ in range(nb):
        bufs = W._column(rng, schema[0], rows, rng.integers(0, 1 << 40, size=rows), 0.0)
        bufs += W._column(rng, schema[1], rows, None, 0.05, (0, 80, W.AZ))
        bufs += W._column(rng, schema[2], rows, rng.integers(-1000, 1000, size=rows), 0.05)
        bufs += W._column(rng, schema[3], rows, None, 0.0, (0, 80, W.AZ))
        bufs += W._column(rng, schema[4], rows, None, 0.3, (0, 8, bytes(range(256))))
        bufs += W._column(rng, schema[5], rows, None, 0.05, (0, 12, W.AZ))
        out.append(W.Batch(rows, bufs))
    return schema, out


@pytest.mark.gpu
@pytest.mark.parametrize("P", [1, 16, 200, 3000])
def test_gpu_large_binary_vs_oracle(P):
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _large_wide(50 + P, 12, 4096)
    res, data = S.split_batches(schema, batches, P, [0], writeSchema=False)
    ref = O.run_oracle(schema, batches, P, [0])
    assert data == ref.data
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths)


@pytest.mark.gpu
def test_gpu_large_binary_device_resident_many_passes():
    torch = pytest.importorskip("torch")
    from gazelle_plugin_gb300 import shuffle as S
    schema, batches = _large_wide(61, 20, 4096)
    keep = []
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 200, None, [0], list(schema)), writeSchema=False,
               input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=2 << 20)
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
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)


@pytest.mark.gpu
def test_gpu_large_binary_lz4_and_reader():
    """LZ4_FRAME output decodes to the uncompressed split's buffers, and the reduce-side reader
    concatenates the partitions of several map outputs (compressed or not) like the oracle's."""
    from gazelle_plugin_gb300 import shuffle as S
    P = 16
    outs_u, outs_z = [], []
    for seed in (71, 72, 73):
        schema, batches = _large_wide(seed, 4, 4096)
        for codec, outs in ((None, outs_u), ("lz4", outs_z)):
            kw = {"codec": codec} if codec else {}
            res, data = S.split_batches(schema, batches, P, [0], writeSchema=False, **kw)
            st = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
            outs.append([data[st[p]:st[p + 1]] for p in range(P)])
    for p in range(P):
        bu = [b for o in outs_u for b in R.parse_stream(o[p], schema)]
        bz = [b for o in outs_z for b in R.parse_stream(o[p], schema)]
        assert [r for r, _ in bu] == [r for r, _ in bz]
        for (_, cu), (_, cz) in zip(bu, bz):
            assert [[bytes(x) for x in f[1]] for f in cu] == [[bytes(x) for x in f[1]] for f in cz]
        rows, cols = R.read_partition(schema, [o[p] for o in outs_u])
        for outs in (outs_u, outs_z):
            r = S.PartitionReader(list(schema))
            for o in outs:
                r.addStream(o[p])
            assert r.finish()[0] == rows
            for fi, f in enumerate(schema):
                valid, offs, vals = cols[fi]
                gv, go, gvals = r.column_to_host(fi)
                assert (gv is None) == (valid is None)
                if valid is not None:
                    assert gv.tobytes() == R.pack_bits(valid)
                if f.is_binary:
                    assert go.dtype == f.offset_dtype and np.array_equal(go, offs)
                assert gvals.tobytes() == vals
            r.close()


@pytest.mark.gpu
def test_gpu_large_binary_rejections():
    from gazelle_plugin_gb300 import shuffle as S
    schema = [W.Field("k", "int32", False), W.Field("a", "large_utf8")]
    w = S.ShuffleSplitterJniWrapper()
    # a 64-bit-offset column as a hash key: the fork's generic hash32, no Spark hash
    with pytest.raises(S.SplitterError) as e:
        w.make(S.NativePartitioning("hash", 4, None, [1], list(schema)), writeSchema=False)
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    # a batch whose character buffer is claimed above 2^31 - 1 bytes: rejected before any read
    h = w.make(S.NativePartitioning("hash", 4, None, [0], list(schema)), writeSchema=False)
    keys = np.arange(8, dtype=np.int32)
    offs = np.zeros(9, np.int64)
    chars = np.zeros(16, np.uint8)
    addrs = [0, keys.ctypes.data, 0, offs.ctypes.data, chars.ctypes.data]
    sizes = [0, keys.nbytes, 0, offs.nbytes, 1 << 31]
    with pytest.raises(S.SplitterError) as e:
        w.split(h, 8, addrs, sizes)
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    # 64-bit offsets beyond the characters
    bad = offs.copy()
    bad[8] = 17
    with pytest.raises(S.SplitterError) as e:
        w.split(h, 8, [0, keys.ctypes.data, 0, bad.ctypes.data, chars.ctypes.data],
                [0, keys.nbytes, 0, bad.nbytes, chars.nbytes])
    assert e.value.status == S.GZ_INVALID
    w.close(h)
