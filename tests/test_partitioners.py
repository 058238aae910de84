"""The round-robin, single and range partitioners (Splitter::Make "rr", "single", "range",
native-sql-engine/cpp/src/shuffle/splitter.cc:190-208, 1369-1387, 1475-1521).  They share the
hash split's pipeline; only the partition id of a row differs: the running round-robin
selection (carried from batch to batch and pass to pass), or the int32 id in schema field 0,
which the output leaves out.

CPU: the oracle against the fixtures the reference Splitter made (partitioners.json) and
against the reference unit tests' own expectations.  GPU: the CUDA split, through the C ABI,
against the same fixtures and the oracle, over many device passes, host and device inputs."""
import hashlib
import json
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O
from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "partitioners.json")))["cases"]


def case_inputs(case):
    return G.partitioner_inputs(case["short_name"], case["gen"], case["num_partitions"])


def check_case(case, lengths, raw, spilled, data):
    assert list(lengths) == case["partition_lengths"], case["name"]
    assert list(raw) == case["raw_partition_lengths"], case["name"]
    assert spilled == case["bytes_spilled"], case["name"]
    assert hashlib.sha256(data).hexdigest() == case["data_sha256"], case["name"]


def assert_same(res, data, ref, tag=""):
    assert np.array_equal(res.partitionLengths, ref.partition_lengths), tag
    assert np.array_equal(res.rawPartitionLengths, ref.raw_partition_lengths), tag
    assert data == ref.data, tag
    assert res.totalBytesSpilled == ref.bytes_spilled, tag


# ---------------------------------------------------------------------------------------
# CPU: the oracle is pinned
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_fixtures(case):
    schema, batches = case_inputs(case)
    out = O.run_oracle(schema, batches, case["num_partitions"], [], short_name=case["short_name"],
                       **case["options"])
    check_case(case, out.partition_lengths, out.raw_partition_lengths, out.bytes_spilled, out.data)


def _read_partition(out, p):
    pa = pytest.importorskip("pyarrow")
    return list(pa.ipc.open_stream(out.partition_bytes(p)))


@pytest.mark.parametrize("short_name,P", [("single", 1), ("rr", 2), ("range", 2)])
def test_oracle_meets_reference_unit_test_expectations(short_name, P):
    """TestSingleSplitter / TestRoundRobinSplitter / TestFallbackRangeSplitter
    (shuffle_split_test.cc:210-253, 255-319, 390-472): splits [b1, b2, b1]; partition 0 of the
    two-partition splits holds rows [0, 2, 4, 6, 8] of b1, row 0 of b2, then b1's rows again,
    partition 1 the odd rows; the single split holds the three batches whole."""
    pytest.importorskip("pyarrow")
    b1, b2 = G.ref_fixture_batches()
    seq = [G.to_batch(b) for b in (b1, b2, b1)]
    schema = list(G.REF_FIXTURE_SCHEMA)
    if short_name == "range":
        schema, seq = W.with_partition_ids(schema, seq, [np.arange(b.num_rows) % 2 for b in seq])
    out = O.run_oracle(schema, seq, P, [], short_name=short_name,
                       buffer_size=10 if short_name == "single" else 4, write_schema=True)
    assert len(out.partition_lengths) == P
    assert int(out.partition_lengths.sum()) == len(out.data)
    if short_name == "single":
        expected = [[b1, b2, b1]]
    else:
        expected = [[b1.take([0, 2, 4, 6, 8]), b2.take([0]), b1.take([0, 2, 4, 6, 8])],
                    [b1.take([1, 3, 5, 7, 9]), b2.take([1]), b1.take([1, 3, 5, 7, 9])]]
    for p in range(P):
        got = _read_partition(out, p)
        assert [g.schema.names for g in got] == [[f.name for f in G.REF_FIXTURE_SCHEMA]] * 3
        assert [g.to_pylist() for g in got] == [e.to_pylist() for e in expected[p]], p


def test_oracle_range_rejects_bad_ids():
    schema, batches = W.with_partition_ids(W.C1_SCHEMA, W.c1_batches(0, 1, 100),
                                           [np.r_[np.zeros(99, np.int32), 8]])
    with pytest.raises(ValueError, match="equal or greater"):
        O.run_oracle(schema, batches, 8, [], short_name="range")
    schema, batches = W.with_partition_ids(W.C1_SCHEMA, W.c1_batches(0, 1, 100),
                                           [np.r_[np.zeros(99, np.int32), -1]])
    with pytest.raises(ValueError, match="negative"):
        O.run_oracle(schema, batches, 8, [], short_name="range")


@pytest.mark.skipif(not O.RefSplitter.available(), reason="reference build absent here")
@pytest.mark.parametrize("short_name", ["rr", "single", "range"])
def test_oracle_matches_live_reference(short_name):
    for seed in range(6000, 6030):
        schema, batches, P, _, opts = G.random_case(seed)
        if short_name == "range":
            rng = np.random.default_rng(seed)
            schema, batches = W.with_partition_ids(
                schema, batches, [rng.integers(0, P, size=b.num_rows) for b in batches])
        r = O.run_ref(schema, batches, P, [], short_name=short_name, **opts)
        o = O.run_oracle(schema, batches, P, [], short_name=short_name, **opts)
        assert r.data == o.data, seed
        assert (r.partition_lengths == o.partition_lengths).all(), seed
        assert (r.raw_partition_lengths == o.raw_partition_lengths).all(), seed


# ---------------------------------------------------------------------------------------
# GPU: the CUDA split through the C ABI
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_matches_reference_fixtures(case):
    schema, batches = case_inputs(case)
    o = case["options"]
    res, data = S.split_batches(schema, batches, case["num_partitions"], [], shortName=case["short_name"],
                                bufferSize=o.get("buffer_size", 4096),
                                preferSpill=o.get("prefer_spill", True),
                                offheapPerTask=o.get("offheap_per_task", 0),
                                writeSchema=o.get("write_schema", False))
    check_case(case, res.partitionLengths, res.rawPartitionLengths, res.totalBytesSpilled, data)


def _inputs(short_name, P, seed):
    batches = W.c2_batches(seed, 20, 4096) + W.c2_batches(seed + 1, 3, 1000)
    schema = list(W.C2_SCHEMA)
    if short_name == "range":
        rng = np.random.default_rng(seed)
        schema, batches = W.with_partition_ids(
            schema, batches, [rng.integers(0, P, size=b.num_rows) for b in batches])
    return schema, batches


@pytest.mark.gpu
@pytest.mark.parametrize("short_name,P", [("rr", 200), ("rr", 7), ("single", 1), ("range", 200),
                                          ("range", 3000)])
@pytest.mark.parametrize("flush", [1 << 20, 5 << 20])
def test_gpu_many_passes_host_inputs(short_name, P, flush):
    # several device passes: the round-robin selection continues across them
    schema, batches = _inputs(short_name, P, 21)
    res, data = S.split_batches(schema, batches, P, [], shortName=short_name, writeSchema=False,
                                flush_bytes=flush)
    ref = O.run_oracle(schema, batches, P, [], short_name=short_name)
    assert_same(res, data, ref, (short_name, P, flush))


@pytest.mark.gpu
@pytest.mark.parametrize("short_name,P", [("rr", 200), ("range", 200)])
def test_gpu_many_passes_device_inputs(short_name, P):
    torch = pytest.importorskip("torch")
    schema, batches = _inputs(short_name, P, 31)
    keep, dev = [], []
    for b in batches:
        # byte views: a buffer's size is its byte count (the id column is int32)
        bufs = [torch.from_numpy(np.ascontiguousarray(x).view(np.uint8).copy()).cuda() if x.nbytes
                else torch.zeros(0, dtype=torch.uint8).cuda() for x in b.buffers]
        keep += bufs
        dev.append((b.num_rows, [t.data_ptr() if t.numel() else 0 for t in bufs], [t.numel() for t in bufs]))
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning(short_name, P, None, [], schema), writeSchema=False,
               input_kind=S.GZ_INPUT_DEVICE_RETAINED, flush_bytes=2 << 20)
    for n, addrs, sizes in dev:
        w.split(h, n, addrs, sizes)
    assert w.stats(h)[0] >= 4
    res = w.stop(h)
    data = w.data(h)
    w.close(h)
    ref = O.run_oracle(schema, batches, P, [], short_name=short_name)
    assert_same(res, data, ref, short_name)


@pytest.mark.gpu
def test_gpu_round_robin_ids_continue_from_batch_to_batch():
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("rr", 7, None, [], list(W.C1_SCHEMA)), writeSchema=False)
    o = O.OracleSplitter(W.C1_SCHEMA, 7, [], short_name="rr")
    for b in W.c1_batches(3, 5, 1001):
        addrs, sizes = b.addrs_sizes()
        w.split(h, b.num_rows, addrs, sizes)
        o.split(b)
        assert np.array_equal(w.lastPids(h, b.num_rows), o.last_pids(b.num_rows))
    w.stop(h)
    w.close(h)


@pytest.mark.gpu
def test_gpu_single_has_one_partition():
    batches = W.c1_batches(4, 3, 4096)
    res, data = S.split_batches(W.C1_SCHEMA, batches, 16, [], shortName="single", writeSchema=False)
    ref = O.run_oracle(W.C1_SCHEMA, batches, 16, [], short_name="single")
    assert len(res.partitionLengths) == 1
    assert_same(res, data, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [8, 1 << 20, -1])
def test_gpu_range_bad_partition_id_is_invalid(bad):
    # FallbackRangeSplitter rejects an id >= P (splitter.cc:1510-1514); a negative id too.  The
    # kernel counts such a row in partition 0, copies nothing of the pass and sets an error
    # bit that the next synchronising call reports
    ids = np.zeros(100, np.int32)
    ids[57] = bad
    schema, batches = W.with_partition_ids(W.C1_SCHEMA, W.c1_batches(0, 1, 100), [ids])
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("range", 8, None, [], schema), writeSchema=False)
    addrs, sizes = batches[0].addrs_sizes()
    w.split(h, batches[0].num_rows, addrs, sizes)
    with pytest.raises(S.SplitterError) as e:
        w.stop(h)
    assert e.value.status == S.GZ_INVALID
    w.close(h)


@pytest.mark.gpu
def test_gpu_range_id_field_must_be_int32():
    schema = [W.Field("pid", "int64", False)] + list(W.C1_SCHEMA)
    b = W.c1_batches(0, 1, 64)[0]
    batch = W.Batch(64, [np.zeros(0, np.uint8), np.zeros(64, np.int64)] + list(b.buffers))
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("range", 4, None, [], schema), writeSchema=False)
    addrs, sizes = batch.addrs_sizes()
    with pytest.raises(S.SplitterError) as e:
        w.split(h, batch.num_rows, addrs, sizes)
    assert e.value.status == S.GZ_INVALID
    w.close(h)
