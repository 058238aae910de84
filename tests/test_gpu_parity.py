"""GPU parity: the CUDA split, called through the C ABI, against the oracle and against the
golden fixtures made by the reference Splitter.  Every comparison is byte-for-byte."""
import hashlib
import json
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O
from tests.golden import make_golden as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "splits.json")))["cases"]


def gpu_split(schema, batches, P, keys, buffer_size=4096, prefer_spill=True, offheap_per_task=0,
              write_schema=False, **dev):
    return S.split_batches(schema, batches, P, keys, bufferSize=buffer_size,
                           preferSpill=prefer_spill, offheapPerTask=offheap_per_task,
                           writeSchema=write_schema, **dev)


def assert_same(res, data, ref, tag=""):
    assert np.array_equal(res.partitionLengths, ref.partition_lengths), tag
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths), tag
    for p in range(len(ref.partition_lengths)):
        s0 = int(ref.partition_lengths[:p].sum())
        a = data[s0:s0 + int(ref.partition_lengths[p])]
        b = ref.partition_bytes(p)
        assert a == b, f"{tag} partition {p}"
    assert data == ref.data, tag
    assert res.totalBytesSpilled == ref.bytes_spilled, tag
    assert res.totalBytesWritten == ref.bytes_written, tag


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_golden(case):
    batches = G.regenerate(case)
    schema = [W.Field(n, t, nl) for n, t, nl in case["schema"]]
    res, data = gpu_split(schema, batches, case["num_partitions"], case["keys"], **case["options"])
    assert list(res.partitionLengths) == case["partition_lengths"]
    assert list(res.rawPartitionLengths) == case["raw_partition_lengths"]
    assert res.totalBytesSpilled == case["bytes_spilled"]
    assert hashlib.sha256(data).hexdigest() == case["data_sha256"]


def test_reference_unit_test_batches():
    meta = json.load(open(os.path.join(HERE, "golden", "ref_fixture.json")))
    z = np.load(os.path.join(HERE, "golden", "ref_fixture.npz"))
    schema = [W.Field(n, t, nl) for n, t, nl in meta["schema"]]
    bs = []
    for i in range(2):
        nbuf = len([k for k in z.files if k.startswith(f"b{i}_buf")])
        bs.append(W.Batch(int(z[f"b{i}_rows"][0]), [z[f"b{i}_buf{j}"] for j in range(nbuf)]))
    seq = [bs[i] for i in meta["sequence"]]
    for r in meta["runs"]:
        res, data = gpu_split(schema, seq, r["num_partitions"], r["keys"], buffer_size=r["buffer_size"])
        assert data == z[f"{r['tag']}_data"].tobytes(), r["tag"]
        assert np.array_equal(res.partitionLengths, z[f"{r['tag']}_lengths"])
        assert np.array_equal(res.rawPartitionLengths, z[f"{r['tag']}_raw"])


def test_partition_ids_match_oracle():
    w = S.ShuffleSplitterJniWrapper()
    for schema, keys, P, batches in [
        (W.C1_SCHEMA, W.C1_KEYS, 8, W.c1_batches(0, 2, 4096)),
        (W.C2_SCHEMA, W.C2_KEYS, 200, W.c2_batches(1, 2, 4096)),
        (W.C3_SCHEMA, W.C3_KEYS, 8000, W.c3_batches(2, 1, 20000, 0.2, 0.1)),
    ]:
        h = w.make(S.NativePartitioning("hash", P, None, keys, list(schema)), writeSchema=False)
        o = O.OracleSplitter(schema, P, keys)
        for b in batches:
            addrs, sizes = b.addrs_sizes()
            w.split(h, b.num_rows, addrs, sizes)
            o.split(b)
            assert np.array_equal(w.lastPids(h, b.num_rows), o.last_pids(b.num_rows))
        w.close(h)
        o.close()


@pytest.mark.parametrize("seed", range(40))
def test_random_vs_oracle(seed):
    schema, batches, P, keys, opts = G.random_case(7000 + seed)
    ref = O.run_oracle(schema, batches, P, keys, **opts)
    res, data = gpu_split(schema, batches, P, keys, **opts)
    assert_same(res, data, ref, f"seed {seed}")


@pytest.mark.parametrize("flush_bytes", [1, 5000, 100000])
def test_flush_grouping_does_not_change_bytes(flush_bytes):
    """Batches cut into device passes at arbitrary points (partition batches then span
    several passes) give the same bytes."""
    batches = W.c1_batches(3, 12, 1000)
    ref = O.run_oracle(W.C1_SCHEMA, batches, 8, W.C1_KEYS, buffer_size=700)
    res, data = gpu_split(W.C1_SCHEMA, batches, 8, W.C1_KEYS, buffer_size=700,
                          flush_bytes=flush_bytes)
    assert_same(res, data, ref)


@pytest.mark.parametrize("host_read,flush_mb", [(S.GZ_HOST_READ_AUTO, 4), (S.GZ_HOST_READ_AUTO, 64),
                                               (S.GZ_HOST_READ_CPU_COPY, 4)])
def test_host_read_modes_batched_call(host_read, flush_mb):
    """Both ways host inputs reach the device (the GPU reading host memory itself, or a CPU copy
    into pinned staging), many batches per call, staging buffers reused across passes."""
    batches = W.c2_batches(11, 100, 4096)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS, buffer_size=1024)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 200, None, W.C2_KEYS, list(W.C2_SCHEMA)),
               bufferSize=1024, writeSchema=False, host_read=host_read, flush_bytes=flush_mb << 20,
               keep_output_on_device=0)
    try:
        rows = np.array([b.num_rows for b in batches], np.int32)
        pairs = [b.addrs_sizes() for b in batches]
        w.splitBatches(h, rows, np.stack([a for a, _ in pairs]), np.stack([z for _, z in pairs]))
        res = w.stop(h)
        data = w.data(h)
    finally:
        w.close(h)
    assert_same(res, data, ref)


@pytest.mark.parametrize("shift", [1, 4, 8, 13])
def test_unaligned_host_buffers(shift):
    """Host buffers at every alignment: each buffer of each batch starts `shift` + (its index)
    bytes past a 64-byte boundary, so values, offsets and characters arrive at all phases."""
    batches = W.c2_batches(13, 6, 3000)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS, buffer_size=2048)
    keep = []
    shifted = []
    for b in batches:
        bufs = []
        for i, x in enumerate(b.buffers):
            raw = x.view(np.uint8).ravel()
            off = (shift + i) % 64
            host = np.zeros(raw.nbytes + 128, np.uint8)
            base = (-host.ctypes.data) % 64 + off
            host[base:base + raw.nbytes] = raw
            keep.append(host)
            bufs.append(host[base:base + raw.nbytes])
        shifted.append(W.Batch(b.num_rows, bufs))
    res, data = gpu_split(W.C2_SCHEMA, shifted, 200, W.C2_KEYS, buffer_size=2048)
    assert_same(res, data, ref)


def test_host_buffers_reusable_when_split_returns():
    """The JNI contract: the writer may overwrite or free a batch's buffers as soon as split
    returns, so every host byte must have been read by then."""
    batches = W.c1_batches(12, 20, 4096)
    ref = O.run_oracle(W.C1_SCHEMA, batches, 8, W.C1_KEYS)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 8, None, W.C1_KEYS, list(W.C1_SCHEMA)), writeSchema=False)
    try:
        for b in batches:
            work = W.Batch(b.num_rows, [x.copy() for x in b.buffers])
            addrs, sizes = work.addrs_sizes()
            w.split(h, work.num_rows, addrs, sizes)
            for x in work.buffers:
                x.view(np.uint8)[:] = 0xA5
        res = w.stop(h)
        data = w.data(h)
    finally:
        w.close(h)
    assert_same(res, data, ref)


def test_output_copied_to_host_every_pass():
    batches = W.c2_batches(5, 24, 4096)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS, buffer_size=512)
    res, data = gpu_split(W.C2_SCHEMA, batches, 200, W.C2_KEYS, buffer_size=512,
                          keep_output_on_device=0, flush_bytes=1 << 20)
    assert_same(res, data, ref)


@pytest.mark.parametrize("P,null_frac,key_nulls", [(16, 0.0, 0.0), (200, 0.2, 0.0),
                                                   (2000, 0.2, 0.05), (8000, 0.0, 0.0)])
def test_zipf_fanout(P, null_frac, key_nulls):
    batches = W.c3_batches(2, 3, 32768, null_frac, key_nulls)
    ref = O.run_oracle(W.C3_SCHEMA, batches, P, W.C3_KEYS)
    res, data = gpu_split(W.C3_SCHEMA, batches, P, W.C3_KEYS)
    assert_same(res, data, ref, f"P={P}")


def test_wide_schema_many_batches():
    batches = W.c2_batches(9, 300, 4096)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS)
    res, data = gpu_split(W.C2_SCHEMA, batches, 200, W.C2_KEYS, flush_bytes=64 << 20)
    assert_same(res, data, ref)


def test_prefer_spill_off_and_native_spill():
    batches = W.c1_batches(0, 30, 512)
    o = O.OracleSplitter(W.C1_SCHEMA, 8, W.C1_KEYS, buffer_size=512, prefer_spill=False)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 8, None, W.C1_KEYS, list(W.C1_SCHEMA)),
               bufferSize=512, preferSpill=False, writeSchema=False)
    for i, b in enumerate(batches):
        o.split(b)
        addrs, sizes = b.addrs_sizes()
        w.split(h, b.num_rows, addrs, sizes)
        if i in (12, 25):
            assert w.nativeSpill(h, 20000) == o.spill(20000)
    ref = o.stop()
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    assert_same(res, data, ref)


def test_offheap_split_size():
    schema = [W.Field("k", "int64"), W.Field("s", "utf8"), W.Field("t", "utf8")]
    rng = np.random.default_rng(4)
    batches = [W.random_batch(rng, schema, 300, 0.1) for _ in range(10)]
    # first batch: every string empty, so the empirical sizes are learned later
    b0 = batches[0]
    b0.buffers[3] = np.zeros(301 * 4, np.uint8)
    b0.buffers[4] = np.zeros(0, np.uint8)
    for opts in [dict(offheap_per_task=1 << 16, prefer_spill=False),
                 dict(offheap_per_task=1 << 18, prefer_spill=False)]:
        ref = O.run_oracle(schema, batches, 7, [0], **opts)
        res, data = gpu_split(schema, batches, 7, [0], **opts)
        assert_same(res, data, ref, str(opts))


def test_empty_batches_are_ignored():
    batches = W.c1_batches(1, 4, 900)
    empty = W.Batch(0, [np.zeros(0, np.uint8) for _ in batches[0].buffers])
    seq = [empty, batches[0], empty, batches[1], batches[2], empty, batches[3]]
    ref = O.run_oracle(W.C1_SCHEMA, batches, 8, W.C1_KEYS)
    res, data = gpu_split(W.C1_SCHEMA, seq, 8, W.C1_KEYS)
    assert_same(res, data, ref)


def test_device_resident_inputs():
    torch = pytest.importorskip("torch")
    batches = W.c2_batches(11, 20, 4096)
    keep = []
    dev_batches = []
    for b in batches:
        bufs = []
        for buf in b.buffers:
            t = torch.from_numpy(buf.copy()).cuda() if buf.nbytes else torch.zeros(0, dtype=torch.uint8).cuda()
            keep.append(t)
            bufs.append(t)
        dev_batches.append((b.num_rows, bufs))
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 200, None, W.C2_KEYS, list(W.C2_SCHEMA)),
               writeSchema=False, input_kind=S.GZ_INPUT_DEVICE_RETAINED)
    for n, bufs in dev_batches:
        addrs = [t.data_ptr() if t.numel() else 0 for t in bufs]
        sizes = [t.numel() for t in bufs]
        w.split(h, n, addrs, sizes)
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS)
    assert_same(res, data, ref)


def _device_batches(torch, batches):
    keep, out = [], []
    for b in batches:
        bufs = []
        for buf in b.buffers:
            t = torch.from_numpy(buf.copy()).cuda() if buf.nbytes else torch.zeros(0, dtype=torch.uint8).cuda()
            keep.append(t)
            bufs.append(t)
        out.append((b.num_rows, [t.data_ptr() if t.numel() else 0 for t in bufs], [t.numel() for t in bufs]))
    return keep, out


@pytest.mark.parametrize("flush,keep_dev,budget", [(1 << 20, 1, 64 << 30), (3 << 20, 0, 64 << 30),
                                                   (2 << 20, 1, 4 << 20)])
def test_device_resident_inputs_many_passes(flush, keep_dev, budget):
    # device-resident inputs: each pass's k_scatter is queued when the next pass is flushed;
    # outputs moved to host after every pass, or past a small HBM budget
    torch = pytest.importorskip("torch")
    batches = W.c2_batches(12, 24, 4096) + W.c2_batches(13, 3, 1000)
    keep, dev = _device_batches(torch, batches)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 200, None, W.C2_KEYS, list(W.C2_SCHEMA)),
               writeSchema=False, input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=flush,
               keep_output_on_device=keep_dev, device_budget=budget)
    for i, (n, addrs, sizes) in enumerate(dev):
        w.split(h, n, addrs, sizes)
        if i == 10:
            w.sync(h)  # a sync in the middle queues the pending k_scatter early
    assert w.stats(h)[0] >= 4
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS)
    assert_same(res, data, ref)


@pytest.mark.parametrize("input_kind", ["device", "host"])
def test_passes_of_changing_size_reuse_and_grow_scratch(input_kind):
    """Passes of many small batches, then of single large ones, then small again: the per-pass
    scratch buffers (three, reused in turn while the passes before are still queued) grow in the
    middle of the split; every byte equal to the oracle's."""
    torch = pytest.importorskip("torch")
    batches = (W.c2_batches(21, 30, 200) + W.c2_batches(22, 6, 4096) + W.c2_batches(23, 3, 16384) +
               W.c2_batches(24, 20, 300) + W.c2_batches(25, 2, 16384))
    w = S.ShuffleSplitterJniWrapper()
    part = S.NativePartitioning("hash", 200, None, W.C2_KEYS, list(W.C2_SCHEMA))
    if input_kind == "device":
        keep, dev = _device_batches(torch, batches)
        h = w.make(part, writeSchema=False, input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=1 << 20)
        for n, addrs, sizes in dev:
            w.split(h, n, addrs, sizes)
    else:
        h = w.make(part, writeSchema=False, flush_bytes=1 << 20)
        for b in batches:
            a, z = b.addrs_sizes()
            w.split(h, b.num_rows, a, z)
    assert w.stats(h)[0] >= 8
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    assert_same(res, data, O.run_oracle(W.C2_SCHEMA, batches, 200, W.C2_KEYS))


def test_device_resident_inputs_offheap_split_size():
    # device inputs with offheap_per_task: the batches whose call flag is read back get their own
    # pass while earlier passes' k_scatter are still queued behind them
    torch = pytest.importorskip("torch")
    schema = [W.Field("k", "int64"), W.Field("s", "utf8"), W.Field("t", "utf8")]
    rng = np.random.default_rng(14)
    batches = [W.random_batch(rng, schema, 300, 0.1) for _ in range(12)]
    b0 = batches[0]
    b0.buffers[3] = np.zeros(301 * 4, np.uint8)
    b0.buffers[4] = np.zeros(0, np.uint8)
    keep, dev = _device_batches(torch, batches)
    opts = dict(offheap_per_task=1 << 16, prefer_spill=False)
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 7, None, [0], list(schema)), writeSchema=False,
               input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=1 << 14,
               offheapPerTask=opts["offheap_per_task"], preferSpill=False)
    for n, addrs, sizes in dev:
        w.split(h, n, addrs, sizes)
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(schema, batches, 7, [0], **opts)
    assert_same(res, data, ref)


def test_schema_ipc_make():
    pa = pytest.importorskip("pyarrow")
    batches = W.c1_batches(0, 2, 4096)
    sbytes = O.to_pyarrow_schema(W.C1_SCHEMA).serialize().to_pybytes()
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", 8, sbytes, W.C1_KEYS), writeSchema=False)
    for b in batches:
        addrs, sizes = b.addrs_sizes()
        w.split(h, b.num_rows, addrs, sizes)
    res = w.stop(h, 8)
    data = w.data(h)
    w.close(h)
    assert data == O.run_oracle(W.C1_SCHEMA, batches, 8, W.C1_KEYS).data


def test_errors_are_reported_not_crashed():
    w = S.ShuffleSplitterJniWrapper()
    with pytest.raises(S.SplitterError) as e:
        w.make(S.NativePartitioning("roundrobin", 4, None, [0], list(W.C1_SCHEMA)))
    assert e.value.status == S.GZ_NOT_IMPLEMENTED
    with pytest.raises(S.SplitterError):
        w.make(S.NativePartitioning("hash", 0, None, [0], list(W.C1_SCHEMA)))
    with pytest.raises(S.SplitterError):  # binary key: no Spark-compatible hash
        w.make(S.NativePartitioning("hash", 4, None, [4], list(W.C1_SCHEMA) + [W.Field("b", "binary")]))
    h = w.make(S.NativePartitioning("hash", 4, None, [0], list(W.C1_SCHEMA)), writeSchema=False)
    b = W.c1_batches(0, 1, 100)[0]
    addrs, sizes = b.addrs_sizes()
    with pytest.raises(S.SplitterError):
        w.split(h, b.num_rows, addrs[:3], sizes[:3])
    sizes2 = sizes.copy()
    sizes2[3] = 8  # int64 values buffer too small
    with pytest.raises(S.SplitterError):
        w.split(h, b.num_rows, addrs, sizes2)
    with pytest.raises(S.SplitterError):
        w.split(12345, 1, addrs, sizes)
    w.split(h, b.num_rows, addrs, sizes)
    w.stop(h)
    w.close(h)


@pytest.mark.gpu
def test_large_data_file_written_through_mapping(tmp_path):
    """A data file of 256 MiB or more is written through a memory mapping (partitions copied in
    in parallel); its bytes equal the in-memory data of the same split."""
    batches = W.c2_batches(77, 400, 4096)  # ~290 MB of partition data
    path = str(tmp_path / "data")
    res_f, _ = S.split_batches(W.C2_SCHEMA, batches, W.C2_PARTITIONS, W.C2_KEYS, dataFile=path)
    res_m, data = S.split_batches(W.C2_SCHEMA, batches, W.C2_PARTITIONS, W.C2_KEYS)
    assert len(data) >= 256 << 20
    with open(path, "rb") as f:
        assert f.read() == data
    assert np.array_equal(res_f.partitionLengths, res_m.partitionLengths)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(4))
def test_utf8_hash_keys_vs_oracle(seed):
    """utf8 key columns (the reference's hashbuf_spark, restated as Spark's hashUnsafeBytes),
    alone and chained with an int key, with null keys and empty strings, over strings of every
    length mod 4 and alignment phase."""
    rng = np.random.default_rng(900 + seed)
    schema = [W.Field("s", "utf8"), W.Field("k", "int32"), W.Field("v", "int64"), W.Field("t", "utf8")]
    keys = [[0], [0, 1], [3, 1, 0], [1, 3]][seed]
    batches = [W.random_batch(rng, schema, int(rng.integers(500, 5000)), 0.15) for _ in range(4)]
    # bytes >= 0x80 too: the tail bytes of a string are hashed sign-extended
    hi = bytes(range(1, 256))
    for b in batches[::2]:
        b.buffers[0:3] = W._column(rng, schema[0], b.num_rows, None, 0.1, (0, 23, hi))
    P = [7, 64, 200, 1000][seed]
    want = O.run_oracle(schema, batches, P, keys)
    res, data = S.split_batches(schema, batches, P, keys, writeSchema=False)
    assert data == want.data
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", P, None, keys, schema), writeSchema=False)
    o = O.OracleSplitter(schema, P, keys)
    for b in batches:
        a, z = b.addrs_sizes()
        w.split(h, b.num_rows, a, z)
        o.split(b)
        assert np.array_equal(w.lastPids(h, b.num_rows), o.last_pids(b.num_rows))
    w.close(h)
    o.close()


@pytest.mark.gpu
def test_split_group_of_tasks_equals_per_task_calls():
    """gz_split_split_group: batches of three tasks (three schemas, three partition counts) in one
    call per window, then one gz_split_sync_group, give each task the bytes of splitting its own
    batches one by one (oracle)."""
    rng = np.random.default_rng(5)
    specs = [(W.C1_SCHEMA, W.C1_KEYS, 8), (W.C2_SCHEMA, W.C2_KEYS, 200), (W.C4_SCHEMA_3, W.C4_KEYS_3, 64)]
    batches = [[W.c4_batch(rng, si, int(rng.integers(500, 9000))) for _ in range(7)] for si in range(3)]
    w = S.ShuffleSplitterJniWrapper()
    hs = [w.make(S.NativePartitioning("hash", P, None, keys, list(sch)), writeSchema=False, flush_bytes=1 << 20)
          for sch, keys, P in specs]
    for lo in range(0, 7, 3):
        win = [b[lo:lo + 3] for b in batches]
        w.splitGroup(hs, [[b.num_rows for b in x] for x in win],
                     [np.stack([b.addrs_sizes()[0] for b in x]) for x in win],
                     [np.stack([b.addrs_sizes()[1] for b in x]) for x in win])
    w.syncGroup(hs)  # every task's last pass queued, then waited for
    for (sch, keys, P), h, bs in zip(specs, hs, batches):
        assert w.stats(h)[0] >= 1
        w.stop(h, P)
        assert w.data(h) == O.run_oracle(sch, bs, P, keys).data
        w.close(h)
