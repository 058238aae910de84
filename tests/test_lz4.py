"""LZ4_FRAME shuffle compression: the framing on the host, the oracle decoder, and (GPU) the
CUDA compressor's output.

CPU: the oracle's LZ4 frame decoder (oracle/lz4_oracle.cc) against the LZ4 library pyarrow
ships; xxHash32 against its published empty-input value; the splitter's compressed record-batch
message (BodyCompression metadata, buffers as uncompressed length + LZ4 frame) read back by
pyarrow's IPC reader, with frames of stored blocks.
"""
import ctypes

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from oracle import oracle as O


def test_xxh32_published_value():
    assert O.xxh32(b"") == 0x02CC5D05


@pytest.mark.parametrize("n", [1, 5, 100, 4096, 70000, 300000])
@pytest.mark.parametrize("kind", ["random", "repeat", "text"])
def test_oracle_lz4_decoder_matches_lz4_library(n, kind):
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(n)
    if kind == "random":
        d = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
    elif kind == "repeat":
        d = (b"abcabcabd" * (n // 9 + 1))[:n]
    else:
        d = rng.choice(np.frombuffer(b"abcdefghij  ", np.uint8), n).tobytes()
    frame = pa.compress(d, codec="lz4", asbytes=True)
    assert O.lz4f_decompress(frame, n) == d


def encode_lz4_stored(length, nodes, bufs):
    lib = S.lib()
    f = lib.gz_debug_encode_record_batch_lz4_stored
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    n = np.array(nodes, np.int64).reshape(-1)
    ptrs = (ctypes.c_void_p * max(len(bufs), 1))(*[b.ctypes.data if b.nbytes else None for b in bufs])
    lens = np.array([b.nbytes for b in bufs], np.int64)
    out = np.zeros(4 << 20, np.uint8)
    olen = ctypes.c_int64(0)
    assert f(length, n.ctypes.data, len(nodes), ptrs, lens.ctypes.data, len(bufs), out.ctypes.data,
             out.nbytes, ctypes.byref(olen)) == 0
    return out[:olen.value].tobytes()


def test_compressed_record_batch_message_read_by_arrow():
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(5)
    for trial in range(20):
        n = int(rng.integers(1, 100000 if trial % 5 == 0 else 500))
        mask = rng.random(n) < 0.1
        cols = [pa.array(rng.integers(-100, 100, n), pa.int64(), mask=mask),
                pa.array(["y" * int(k) for k in rng.integers(0, 12, n)], pa.string(),
                         mask=rng.random(n) < 0.05),
                pa.array(rng.integers(0, 2, n).astype(bool), pa.bool_()),
                pa.array(rng.integers(0, 9, n), pa.int32())]
        rb = pa.record_batch(cols, names=["a", "s", "b", "c"])
        nodes, bufs = [], []
        for col in rb.columns:
            nodes.append((len(col), col.null_count))
            bs = col.buffers()
            bufs.append(np.frombuffer(bs[0], np.uint8)[: (n + 7) // 8].copy() if (bs[0] is not None and col.null_count)
                        else np.zeros(0, np.uint8))
            if pa.types.is_string(col.type):
                off = np.frombuffer(bs[1], np.int32)[: n + 1]
                bufs.append(off.view(np.uint8).copy())
                bufs.append(np.frombuffer(bs[2], np.uint8)[: off[-1]].copy())
            elif pa.types.is_boolean(col.type):
                bufs.append(np.frombuffer(bs[1], np.uint8)[: (n + 7) // 8].copy())
            else:
                bufs.append(np.frombuffer(bs[1], np.uint8)[: n * (col.type.bit_width // 8)].copy())
        msg = pa.ipc.read_message(pa.py_buffer(encode_lz4_stored(n, nodes, bufs)))
        got = pa.ipc.read_record_batch(msg, rb.schema)
        assert got.equals(rb), trial


# ---------------------------------------------------------------------------------------- GPU
def _split(schema, batches, P, keys, **kw):
    return S.split_batches(schema, batches, P, keys, writeSchema=False, **kw)


def _partition_streams(res, data):
    starts = np.concatenate([[0], np.cumsum(np.asarray(res.partitionLengths))])
    return [data[starts[p]:starts[p + 1]] for p in range(len(starts) - 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["c1", "c2", "c3"])
def test_gpu_lz4_split_decodes_to_the_uncompressed_batches(which):
    """LZ4_FRAME output of the CUDA splitter: every record batch above batch_compress_threshold
    rows carries body compression, the others do not; decoded by the oracle's LZ4 frame decoder,
    every batch's buffers equal the uncompressed split's, which equal the oracle's."""
    from gazelle_plugin_gb300 import workloads as W
    from oracle import ipc_read as R
    if which == "c1":
        schema, keys, P, batches, kw = W.C1_SCHEMA, W.C1_KEYS, 8, W.c1_batches(21, 6, 4096), dict(bufferSize=1500)
    elif which == "c2":
        schema, keys, P, batches, kw = W.C2_SCHEMA, W.C2_KEYS, 200, W.c2_batches(22, 40, 4096), {}
    else:
        schema, keys, P, batches, kw = W.C3_SCHEMA, W.C3_KEYS, 16, W.c3_batches(23, 2, 32768, 0.2, 0.0), {}
    res_u, data_u = _split(schema, batches, P, keys, **kw)
    ref = O.run_oracle(schema, batches, P, keys, buffer_size=kw.get("bufferSize", 4096))
    assert data_u == ref.data
    res_z, data_z = _split(schema, batches, P, keys, codec="lz4", **kw)
    assert np.array_equal(res_z.rawPartitionLengths, res_u.rawPartitionLengths)
    # (random test data barely compresses: the frames may even add a few bytes)
    assert sum(res_z.partitionLengths) < 1.05 * sum(res_u.partitionLengths) + 4096
    for su, sz in zip(_partition_streams(res_u, data_u), _partition_streams(res_z, data_z)):
        bu, bz = R.parse_stream(su, schema), R.parse_stream(sz, schema)
        assert [r for r, _ in bu] == [r for r, _ in bz]
        assert R.batches_compressed(sz) == [r > 256 for r, _ in bz]
        for (_, cu), (_, cz) in zip(bu, bz):
            for fu, fz in zip(cu, cz):
                assert fu[0] == fz[0]  # null counts
                assert [bytes(b) for b in fu[1]] == [bytes(b) for b in fz[1]]


@pytest.mark.gpu
def test_gpu_reader_reads_lz4_streams():
    from gazelle_plugin_gb300 import workloads as W
    from oracle import ipc_read as R
    P = 200
    outs_u, outs_z = [], []
    for seed in (31, 32, 33):
        batches = W.c2_batches(seed, 6, 4096)
        outs_u.append(_partition_streams(*_split(W.C2_SCHEMA, batches, P, W.C2_KEYS)))
        outs_z.append(_partition_streams(*_split(W.C2_SCHEMA, batches, P, W.C2_KEYS, codec="lz4")))
    for p in range(0, P, 9):
        rows, cols = R.read_partition(W.C2_SCHEMA, [o[p] for o in outs_u])
        r = S.PartitionReader(list(W.C2_SCHEMA))
        for o in outs_z:
            r.addStream(o[p])
        assert r.finish()[0] == rows
        for fi, f in enumerate(W.C2_SCHEMA):
            valid, offs, vals = cols[fi]
            gv, go, gvals = r.column_to_host(fi)
            assert (gv is None) == (valid is None)
            if valid is not None:
                assert gv.tobytes() == R.pack_bits(valid)
            if f.is_binary:
                assert np.array_equal(go, offs)
            assert gvals.tobytes() == vals
        r.close()


@pytest.mark.gpu
def test_gpu_compressed_size_of_first_batch():
    """split(firstRecordBatch=True) with LZ4_FRAME: the batch's compressed IPC body length (the
    writer compares it between codecs, ColumnarShuffleWriter.scala:147-175), close to the body
    of the same batch split into one partition and compressed at Stop."""
    from gazelle_plugin_gb300 import workloads as W
    from oracle import ipc_read as R
    b = W.c2_batches(41, 1, 4096)[0]
    a, z = b.addrs_sizes()
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("single", 1, None, [], list(W.C2_SCHEMA)), codec="lz4", writeSchema=False)
    plain = S.ShuffleSplitterJniWrapper()
    hp = plain.make(S.NativePartitioning("single", 1, None, [], list(W.C2_SCHEMA)), writeSchema=False)
    cs_lz4 = w.split(h, b.num_rows, a, z, True)
    cs_raw = plain.split(hp, b.num_rows, a, z, True)
    w.split(h, b.num_rows, a, z)
    w.stop(h)
    data = w.data(h)
    w.close(h)
    plain.close(hp)
    assert 0 < cs_lz4 < cs_raw
    # the body of the one record batch written: its message minus the metadata
    meta_len = int.from_bytes(data[4:8], "little")
    body = len(data) - 8 - 8 - meta_len  # continuation + length prefix, EOS at the end
    assert R.batches_compressed(data) == [True]
    assert abs(cs_lz4 - body) <= 0.01 * body + 64
