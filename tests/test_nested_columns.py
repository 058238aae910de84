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
