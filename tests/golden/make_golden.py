"""Generate the golden fixtures in this directory from the reference Splitter itself.

Run in a checkout where the reference sources and pyarrow are present:

    python tests/golden/make_golden.py [/path/to/gazelle_plugin] [--only=large|list|nested]

(--only=large / list / nested rewrite large_binary.json / list_columns.json /
nested_columns.json alone.)

It compiles the reference Splitter (oracle/ref/Makefile -> oracle/_ref/) and runs it on
seeded inputs from gazelle_plugin_gb300.workloads, recording for every case the SHA-256 of
the input buffers, of the whole shuffle data file and of every partition's bytes, plus
partition_lengths, raw_partition_lengths and bytes spilled.  The reference's own unit-test
batches (native-sql-engine/cpp/src/tests/shuffle_split_test.cc:186-208) are materialised
into ref_fixture.npz together with the expected data-file bytes.  partitioners.json records
the same digests for the round-robin, single and range partitioners (Splitter::Make "rr",
"single", "range"), on those unit-test batches and on seeded workloads.

The reference hashes through gandiva, which is absent; oracle/ref/stub supplies the same
Spark Murmur3 chain (oracle/spark_hash.h), so what these fixtures pin is everything after
the hash: pmod, histogram, stable scatter, buffer/emit policy, validity, IPC and file bytes.
Configurations on which the reference has undefined behaviour are excluded: with
prefer_spill, a reallocation (new size > capacity) reads partition_buffers_ after
CacheRecordBatch cleared it (splitter.cc:907-909, 766-773), which happens whenever a
partition receives more rows in one batch than its buffer holds or offheap_per_task > 0.

large_binary.json holds schemas with large_utf8 / large_binary columns (64-bit offsets).  The
reference sizes their offset buffers through one `sizeof_binary_offset` variable per call that
a 32-bit binary column sets and a later 64-bit one does not reset (splitter.cc:476-485,
619-632): a 64-bit column after a 32-bit one gets a half-size offsets buffer and is cut with
32-bit reads.  These cases put every 64-bit column before every 32-bit one, where the
reference is well defined.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gazelle_plugin_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(b) -> str:
    return hashlib.sha256(b).hexdigest()


def input_digest(batches) -> str:
    h = hashlib.sha256()
    for b in batches:
        h.update(np.int64(b.num_rows).tobytes())
        for buf in b.buffers:
            h.update(np.int64(buf.nbytes).tobytes())
            h.update(buf.tobytes())
    return h.hexdigest()


def field_json(f):
    """[name, type, nullable] (+ [elem] for a simple list, + [None, [children]] when nested)."""
    if f.is_nested:
        return [f.name, f.type, f.nullable, None, [field_json(k) for k in f.children]]
    return [f.name, f.type, f.nullable] + ([f.elem] if f.is_list else [])


def field_from_json(x):
    if len(x) > 4:
        return W.Field(x[0], x[1], x[2], None, tuple(field_from_json(k) for k in x[4]))
    return W.Field(*x)


def record(name, schema, batches, P, keys, opts, gen, short_name="hash"):
    out = O.run_ref(schema, batches, P, keys, short_name=short_name, **opts)
    P = len(out.partition_lengths)
    rec = {"short_name": short_name} if short_name != "hash" else {}
    if gen.get("workload") == "nested":  # Splitter::CompressedSize of each input batch (uncompressed)
        r = O.RefSplitter(schema, P, keys, short_name=short_name, **opts)
        rec["body_lengths"] = [int(r.compressed_size(b)) for b in batches]
        r.close()
    return {
        **rec,
        "name": name,
        "gen": gen,
        "schema": [field_json(f) for f in schema],
        "num_partitions": P,
        "keys": [int(k) for k in keys],
        "options": opts,
        "input_sha256": input_digest(batches),
        "data_sha256": sha(out.data),
        "partition_sha256": ([sha(out.partition_bytes(p)) for p in range(P)] if P <= 256
                             else None),
        "partition_lengths": out.partition_lengths.tolist(),
        "raw_partition_lengths": out.raw_partition_lengths.tolist(),
        "bytes_spilled": out.bytes_spilled,
        "bytes_written": out.bytes_written,
    }


def cases():
    """(name, schema, batches, P, keys, options, generator description)"""
    yield ("c1", W.C1_SCHEMA, W.c1_batches(0, 10, 4096), 8, W.C1_KEYS, {},
           {"workload": "c1", "seed": 0, "num_batches": 10, "rows": 4096})
    yield ("c1_buf512_nospill", W.C1_SCHEMA, W.c1_batches(0, 10, 512), 8, W.C1_KEYS,
           {"buffer_size": 512, "prefer_spill": False},
           {"workload": "c1", "seed": 0, "num_batches": 10, "rows": 512})
    yield ("c2_16x4096", W.C2_SCHEMA, W.c2_batches(1, 16, 4096), 200, W.C2_KEYS, {},
           {"workload": "c2", "seed": 1, "num_batches": 16, "rows": 4096})
    yield ("c3_p16_nulls", W.C3_SCHEMA, W.c3_batches(2, 6, 4096, 0.2, 0.05), 16, W.C3_KEYS, {},
           {"workload": "c3", "seed": 2, "num_batches": 6, "rows": 4096, "null_frac": 0.2,
            "key_nulls": 0.05})
    yield ("c3_p2000", W.C3_SCHEMA, W.c3_batches(2, 3, 4096, 0.0, 0.0), 2000, W.C3_KEYS,
           {"buffer_size": 8},
           {"workload": "c3", "seed": 2, "num_batches": 3, "rows": 4096, "null_frac": 0.0,
            "key_nulls": 0.0})
    for seed in range(24):
        rng = np.random.default_rng(1000 + seed)
        schema = W.random_schema(rng, int(rng.integers(1, 9)))
        keys = [i for i, f in enumerate(schema) if f.type in W.KEY_TYPES]
        keys = [int(k) for k in rng.choice(keys, size=int(rng.integers(1, len(keys) + 1)),
                                           replace=False)]
        P = int(rng.choice([1, 2, 3, 7, 16, 64, 200]))
        bsz = int(rng.choice([16, 64, 100, 4096]))
        nb = int(rng.integers(1, 10))
        ps = bool(rng.random() < 0.6)
        opts = {"buffer_size": bsz, "prefer_spill": ps,
                "offheap_per_task": 0 if ps else int(rng.choice([0, 1 << 16, 1 << 20]))}
        nullf = float(rng.choice([0.0, 0.01, 0.3, 0.9]))
        batches = [W.random_batch(rng, schema, int(rng.integers(1, bsz + 1)), nullf)
                   for _ in range(nb)]
        yield (f"random_{seed}", schema, batches, P, keys, opts,
               {"workload": "random", "seed": 1000 + seed})
    # with the schema message before every partition (write_schema)
    yield ("c1_write_schema", W.C1_SCHEMA, W.c1_batches(0, 4, 4096), 8, W.C1_KEYS,
           {"write_schema": True}, {"workload": "c1", "seed": 0, "num_batches": 4, "rows": 4096})
    yield ("c2_write_schema", W.C2_SCHEMA, W.c2_batches(1, 3, 4096), 200, W.C2_KEYS,
           {"write_schema": True}, {"workload": "c2", "seed": 1, "num_batches": 3, "rows": 4096})
    for seed in range(8):
        schema, batches, P, keys, opts = random_case(1000 + seed)
        yield (f"random_{seed}_write_schema", schema, batches, P, keys, dict(opts, write_schema=True),
               {"workload": "random", "seed": 1000 + seed})


def random_case(seed):
    """Re-create the inputs of a `random_<n>` case (same draw order as cases())."""
    rng = np.random.default_rng(seed)
    schema = W.random_schema(rng, int(rng.integers(1, 9)))
    keys = [i for i, f in enumerate(schema) if f.type in W.KEY_TYPES]
    keys = [int(k) for k in rng.choice(keys, size=int(rng.integers(1, len(keys) + 1)),
                                       replace=False)]
    P = int(rng.choice([1, 2, 3, 7, 16, 64, 200]))
    bsz = int(rng.choice([16, 64, 100, 4096]))
    nb = int(rng.integers(1, 10))
    ps = bool(rng.random() < 0.6)
    opts = {"buffer_size": bsz, "prefer_spill": ps,
            "offheap_per_task": 0 if ps else int(rng.choice([0, 1 << 16, 1 << 20]))}
    nullf = float(rng.choice([0.0, 0.01, 0.3, 0.9]))
    batches = [W.random_batch(rng, schema, int(rng.integers(1, bsz + 1)), nullf)
               for _ in range(nb)]
    return schema, batches, P, keys, opts


def large_case(seed):
    """Schema, batches, P, keys and options of a `large_<n>` case: an int key, 0-3 fixed-width
    columns, 1-3 large_utf8 / large_binary columns and 0-2 utf8 / binary columns, the binary
    ones in schema order large first, interleaved at random with the others."""
    rng = np.random.default_rng(seed)
    others = [W.Field("k", str(rng.choice(["int32", "int64"])), bool(rng.random() < 0.5))]
    others += [W.Field(f"f{i}", str(rng.choice(["int16", "int32", "int64", "float64", "bool"])))
               for i in range(int(rng.integers(0, 4)))]
    binary = [W.Field(f"L{i}", str(rng.choice(["large_utf8", "large_binary"])))
              for i in range(int(rng.integers(1, 4)))]
    binary += [W.Field(f"s{i}", str(rng.choice(["utf8", "binary"]))) for i in range(int(rng.integers(0, 3)))]
    pick = rng.permutation(len(others) + len(binary)) < len(others)  # True: an `others` slot
    oi, bi, schema = iter(others), iter(binary), []
    for is_other in pick:
        schema.append(next(oi) if is_other else next(bi))
    keys = [i for i, f in enumerate(schema) if f.name == "k"]
    P = int(rng.choice([1, 3, 16, 200]))
    bsz = int(rng.choice([16, 100, 4096]))
    ps = bool(rng.random() < 0.6)
    opts = {"buffer_size": bsz, "prefer_spill": ps,
            "offheap_per_task": 0 if ps else int(rng.choice([0, 1 << 16]))}
    nullf = float(rng.choice([0.0, 0.05, 0.5]))
    batches = [W.random_batch(rng, schema, int(rng.integers(1, bsz + 1)), nullf)
               for _ in range(int(rng.integers(1, 8)))]
    return schema, batches, P, keys, opts


LIST_ELEMS = ["int8", "int16", "int32", "int64", "float32", "float64", "date32", "decimal128", "timestamp",
              "bool"]


def list_case(seed, force_elem=None):
    """Schema, batches, P, keys and options of a `list_<n>` case: an int key, 0-2 fixed-width
    columns, 1-3 list columns of fixed-width elements (list and element nulls, or none, or no
    validity buffers) and 0-1 utf8 column, in random order."""
    rng = np.random.default_rng(seed)
    fields = [W.Field("k", str(rng.choice(["int32", "int64"])), False)]
    fields += [W.Field(f"f{i}", str(rng.choice(["int32", "float64", "bool"]))) for i in range(int(rng.integers(0, 3)))]
    fields += [W.Field(f"L{i}", "list", True, str(rng.choice(LIST_ELEMS))) for i in range(int(rng.integers(1, 4)))]
    if force_elem:  # the first list column's elements
        fields = [W.Field(f.name, f.type, f.nullable, force_elem) if f.name == "L0" else f for f in fields]
    fields += [W.Field("s", "utf8")] * int(rng.integers(0, 2))
    schema = [fields[i] for i in rng.permutation(len(fields))]
    keys = [i for i, f in enumerate(schema) if f.name == "k"]
    P = int(rng.choice([1, 3, 16, 200]))
    bsz = int(rng.choice([8, 100, 4096]))
    ps = bool(rng.random() < 0.6)
    opts = {"buffer_size": bsz, "prefer_spill": ps,
            "offheap_per_task": 0 if ps else int(rng.choice([0, 1 << 16]))}
    batches = []
    for _ in range(int(rng.integers(1, 6))):
        n = int(rng.integers(1, bsz + 1))
        bufs = []
        for f in schema:
            if f.is_list:
                bufs += W.list_column(rng, f, n, float(rng.choice([0.0, 0.1, 0.4])),
                                      float(rng.choice([0.0, 0.05, 0.5])), int(rng.choice([0, 3, 12])))
            else:
                bufs += W.random_batch(rng, [f], n, 0.1).buffers
        batches.append(W.Batch(n, bufs))
    return schema, batches, P, keys, opts


def list_cases():
    for seed in range(16):
        schema, batches, P, keys, opts = list_case(5000 + seed)
        yield (f"list_{seed}", schema, batches, P, keys, opts, {"workload": "list", "seed": 5000 + seed})
    schema, batches, P, keys, opts = list_case(5100)
    yield ("list_write_schema", schema, batches, P, keys, dict(opts, write_schema=True),
           {"workload": "list", "seed": 5100})
    for seed in range(4):
        schema, batches, P, keys, opts = list_case(5200 + seed, "bool")
        yield (f"list_bool_{seed}", schema, batches, P, keys, opts,
               {"workload": "list", "seed": 5200 + seed, "force_elem": "bool"})


def _F(name, t, nullable=True, elem=None, *kids):
    return W.Field(name, t, nullable, elem, tuple(kids))


# nested column shapes: the reference unit tests' (shuffle_split_test.cc:509-1060) and more
NESTED_SHAPES = [
    lambda n: _F(n, "list", True, None, _F("item", "utf8")),
    lambda n: _F(n, "list", True, None, _F("item", "list", True, "int32")),
    lambda n: _F(n, "large_list", True, None, _F("item", "list", True, None, _F("item", "utf8"))),
    lambda n: _F(n, "large_list", True, None, _F("item", "list", True, "int32")),
    lambda n: _F(n, "list", True, None, _F("item", "struct", True, None, _F("a", "int32"), _F("b", "utf8"))),
    lambda n: _F(n, "list", True, None, _F("item", "map", True, None, _F("key", "utf8", False), _F("value", "utf8"))),
    lambda n: _F(n, "struct", True, None, _F("a", "list", True, "int32"), _F("b", "utf8")),
    lambda n: _F(n, "map", True, None, _F("key", "utf8", False), _F("value", "utf8")),
    lambda n: _F(n, "struct", True, None, _F("a", "int32"), _F("b", "bool"), _F("c", "decimal128"),
                 _F("d", "large_utf8")),
    lambda n: _F(n, "list", True, None, _F("item", "large_binary")),
    lambda n: _F(n, "map", True, None, _F("key", "int32", False), _F("value", "list", True, "float64")),
    lambda n: _F(n, "struct", True, None, _F("s", "struct", True, None, _F("a", "int16"), _F("b", "utf8")),
                 _F("t", "bool")),
    lambda n: _F(n, "list", True, None, _F("item", "list", True, None, _F("item", "list", True, "bool"))),
]


def nested_case(seed):
    """Schema, batches, P, keys and options of a `nested_<n>` case: an int key, 0-1 fixed-width
    and 0-1 simple list columns and 1-3 nested columns (list / large_list / map / struct of any
    depth) in random order; entries null at 0-40% at every level, with null top-level entries
    keeping non-empty ranges in half the cases."""
    rng = np.random.default_rng(seed)
    fields = [W.Field("k", str(rng.choice(["int32", "int64"])), False)]
    fields += [W.Field("f", str(rng.choice(["int32", "float64", "bool"])))] * int(rng.integers(0, 2))
    fields += [W.Field("L", "list", True, "int64")] * int(rng.integers(0, 2))
    fields += [NESTED_SHAPES[int(rng.integers(0, len(NESTED_SHAPES)))](f"N{i}")
               for i in range(int(rng.integers(1, 4)))]
    schema = [fields[i] for i in rng.permutation(len(fields))]
    keys = [i for i, f in enumerate(schema) if f.name == "k"]
    P = int(rng.choice([1, 3, 16, 200]))
    bsz = int(rng.choice([8, 100, 4096]))
    ps = bool(rng.random() < 0.6)
    opts = {"buffer_size": bsz, "prefer_spill": ps,
            "offheap_per_task": 0 if ps else int(rng.choice([0, 1 << 16]))}
    spans = bool(rng.random() < 0.5)
    batches = []
    for _ in range(int(rng.integers(1, 6))):
        n = int(rng.integers(1, bsz + 1))
        bufs = []
        for f in schema:
            if f.is_nested:
                bufs += W.nested_column(rng, f, n, float(rng.choice([0.0, 0.1, 0.4])),
                                        int(rng.choice([0, 2, 5])), True, spans)
            elif f.is_list:
                bufs += W.list_column(rng, f, n, 0.1, 0.1, 4)
            else:
                bufs += W.random_batch(rng, [f], n, 0.1).buffers
        batches.append(W.Batch(n, bufs))
    return schema, batches, P, keys, opts


def nested_cases():
    for seed in range(24):
        schema, batches, P, keys, opts = nested_case(6000 + seed)
        yield (f"nested_{seed}", schema, batches, P, keys, opts, {"workload": "nested", "seed": 6000 + seed})
    for seed in range(2):
        schema, batches, P, keys, opts = nested_case(6100 + seed)
        yield (f"nested_write_schema_{seed}", schema, batches, P, keys, dict(opts, write_schema=True),
               {"workload": "nested", "seed": 6100 + seed})


def large_cases():
    for seed in range(16):
        schema, batches, P, keys, opts = large_case(4000 + seed)
        yield (f"large_{seed}", schema, batches, P, keys, opts, {"workload": "large", "seed": 4000 + seed})
    schema, batches, P, keys, opts = large_case(4100)
    yield ("large_write_schema", schema, batches, P, keys, dict(opts, write_schema=True),
           {"workload": "large", "seed": 4100})


def regenerate(case):
    """Inputs of a recorded case, rebuilt from its generator description."""
    g = case["gen"]
    if g["workload"] == "large":
        return large_case(g["seed"])[1]
    if g["workload"] == "list":
        return list_case(g["seed"], g.get("force_elem"))[1]
    if g["workload"] == "nested":
        return nested_case(g["seed"])[1]
    if g["workload"] == "c1":
        return W.c1_batches(g["seed"], g["num_batches"], g["rows"])
    if g["workload"] == "c2":
        return W.c2_batches(g["seed"], g["num_batches"], g["rows"])
    if g["workload"] == "c3":
        return W.c3_batches(g["seed"], g["num_batches"], g["rows"], g["null_frac"],
                            g["key_nulls"])
    if g["workload"] == "random":
        return random_case(g["seed"])[1]
    raise KeyError(g["workload"])


# ---------------------------------------------------------------------------------------
# the reference unit-test batches (shuffle_split_test.cc:99-127, 186-208)
REF_FIXTURE_SCHEMA = [
    W.Field("f_na", "null"), W.Field("f_int8_a", "int8"), W.Field("f_int8_b", "int8"),
    W.Field("f_int32", "int32"), W.Field("f_uint64", "uint64"), W.Field("f_double", "float64"),
    W.Field("f_bool", "bool"), W.Field("f_string", "utf8"),
    W.Field("f_nullable_string", "utf8"), W.Field("f_decimal128", "decimal128"),
]


def ref_fixture_batches():
    import pyarrow as pa
    from decimal import Decimal
    d1 = [
        [None] * 10,
        [1, 2, 3, None, 4, None, 5, 6, None, 7],
        [1, -1, None, None, -2, 2, None, None, 3, -3],
        [1, 2, 3, 4, None, 5, 6, 7, 8, None],
        [None] * 10,
        [-0.1234567, None, 0.1234567, None, -0.142857, None, 0.142857, 0.285714, 0.428617,
         None],
        [None, True, False, None, True, True, False, True, None, None],
        ["alice0", "bob1", "alice2", "bob3", "Alice4", "Bob5", "AlicE6", "boB7", "ALICE8",
         "BOB9"],
        ["alice", "bob", None, None, "Alice", "Bob", None, "alicE", None, "boB"],
        ["-1.01", "2.01", "-3.01", None, "0.11", "3.14", "2.27", None, "-3.14", None],
    ]
    d2 = [
        [None, None], [None, None], [1, -1], [100, None], [1, 1], [0.142857, -0.142857],
        [True, False], ["bob", "alice" * 40], [None, None], [None, None],
    ]
    pschema = O.to_pyarrow_schema(REF_FIXTURE_SCHEMA)
    pschema = pa.schema([f.with_type(pa.decimal128(10, 2)) if f.name == "f_decimal128" else f
                         for f in pschema])
    out = []
    for data in (d1, d2):
        cols = []
        for f, vals in zip(pschema, data):
            if f.name == "f_decimal128":
                vals = [None if v is None else Decimal(v) for v in vals]
            cols.append(pa.array(vals, f.type))
        out.append(pa.record_batch(cols, schema=pschema))
    return out


def to_batch(rb) -> W.Batch:
    bufs = []
    for col in rb.columns:
        if str(col.type) == "null":
            bufs += [np.zeros(0, np.uint8), np.zeros(0, np.uint8)]
            continue
        arr_bufs = col.buffers()
        v = arr_bufs[0]
        bufs.append(np.frombuffer(v, np.uint8).copy() if (v is not None and col.null_count)
                    else np.zeros(0, np.uint8))
        for b in arr_bufs[1:]:
            bufs.append(np.frombuffer(b, np.uint8).copy() if b is not None
                        else np.zeros(0, np.uint8))
    return W.Batch(rb.num_rows, bufs)


# ---------------------------------------------------------------------------------------
# round-robin / single / range partitioners
def ref_unit_sequence():
    """The reference unit-test batches in the order its tests split them ([b1, b2, b1]), read
    back from ref_fixture.npz (no pyarrow needed)."""
    z = np.load(os.path.join(HERE, "ref_fixture.npz"))
    bs = []
    for i in range(2):
        nbuf = len([k for k in z.files if k.startswith(f"b{i}_buf")])
        bs.append(W.Batch(int(z[f"b{i}_rows"][0]), [z[f"b{i}_buf{j}"] for j in range(nbuf)]))
    return [bs[0], bs[1], bs[0]]


def _pids(gen, batches, P):
    """Partition ids of a range case: 0, 1, 0, 1, ... per batch ("alternate", the reference's
    TestFallbackRangeSplitter) or seeded uniform draws in [0, P)."""
    if gen["pids"] == "alternate":
        return [np.arange(b.num_rows, dtype=np.int32) % 2 for b in batches]
    rng = np.random.default_rng(gen["pid_seed"])
    return [rng.integers(0, P, size=b.num_rows).astype(np.int32) for b in batches]


def _base_batches(gen):
    if gen["workload"] == "ref_unit":
        return REF_FIXTURE_SCHEMA, ref_unit_sequence()
    if gen["workload"] == "random":
        schema, batches, _, _, _ = random_case(gen["seed"])
        return schema, batches
    schema = {"c1": W.C1_SCHEMA, "c2": W.C2_SCHEMA, "c3": W.C3_SCHEMA}[gen["workload"]]
    return schema, regenerate({"gen": gen})


def partitioner_inputs(short_name, gen, P):
    """(schema, batches) of a partitioner case; range cases get the id column in front."""
    schema, batches = _base_batches(gen)
    if short_name == "range":
        return W.with_partition_ids(schema, batches, _pids(gen, batches, P))
    return list(schema), batches


def partitioner_cases():
    """(name, short_name, P, options, generator description)"""
    # TestSingleSplitter, TestRoundRobinSplitter, TestFallbackRangeSplitter
    # (shuffle_split_test.cc:210-253, 255-319, 390-472)
    unit = {"workload": "ref_unit"}
    yield ("ref_single_b10", "single", 1, {"buffer_size": 10}, unit)
    yield ("ref_rr_p2_b4", "rr", 2, {"buffer_size": 4}, unit)
    yield ("ref_range_p2_b4", "range", 2, {"buffer_size": 4}, dict(unit, pids="alternate"))
    yield ("ref_rr_p3_write_schema", "rr", 3, {"write_schema": True}, unit)
    yield ("ref_range_p2_write_schema", "range", 2, {"write_schema": True}, dict(unit, pids="alternate"))
    c1 = {"workload": "c1", "seed": 0, "num_batches": 10, "rows": 4096}
    c2 = {"workload": "c2", "seed": 1, "num_batches": 6, "rows": 4096}
    c3 = {"workload": "c3", "seed": 2, "num_batches": 3, "rows": 4096, "null_frac": 0.2,
          "key_nulls": 0.0}
    yield ("c1_rr_p8", "rr", 8, {}, c1)
    yield ("c1_single", "single", 1, {}, c1)
    yield ("c2_rr_p200", "rr", 200, {}, c2)
    yield ("c2_range_p200", "range", 200, {}, dict(c2, pids="uniform", pid_seed=11))
    yield ("c3_range_p2000_buf8", "range", 2000, {"buffer_size": 8}, dict(c3, pids="uniform", pid_seed=12))
    yield ("c3_rr_p7", "rr", 7, {}, c3)
    for seed in range(12):
        _, batches, P, _, opts = random_case(2000 + seed)
        g = {"workload": "random", "seed": 2000 + seed}
        if seed % 2:
            yield (f"random_{seed}_range", "range", P, opts, dict(g, pids="uniform", pid_seed=3000 + seed))
        else:
            yield (f"random_{seed}_rr", "rr", P, opts, g)


def write_cases(cases, file_name):
    recs = []
    for name, schema, batches, P, keys, opts, gen in cases:
        recs.append(record(name, schema, batches, P, keys, opts, gen))
        print(name, recs[-1]["data_sha256"][:16])
    with open(os.path.join(HERE, file_name), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": recs}, f, indent=1)


def write_large():
    write_cases(large_cases(), "large_binary.json")


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref_root = args[0] if args else O.reference_root()
    if not O.build_ref(ref_root):
        raise SystemExit("reference tree not found")
    if "--only=large" in sys.argv:
        write_large()
        return
    if "--only=list" in sys.argv:
        write_cases(list_cases(), "list_columns.json")
        return
    if "--only=nested" in sys.argv:
        write_cases(nested_cases(), "nested_columns.json")
        return
    write_large()
    write_cases(list_cases(), "list_columns.json")
    write_cases(nested_cases(), "nested_columns.json")
    recs = []
    for name, schema, batches, P, keys, opts, gen in cases():
        recs.append(record(name, schema, batches, P, keys, opts, gen))
        print(name, recs[-1]["data_sha256"][:16])
    with open(os.path.join(HERE, "splits.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": recs}, f, indent=1)

    # the reference's own unit-test batches, sequence [b1, b2, b1] as in TestHashSplitter
    b1, b2 = [to_batch(rb) for rb in ref_fixture_batches()]
    seq = [b1, b2, b1]
    arrays = {}
    for i, b in enumerate((b1, b2)):
        arrays[f"b{i}_rows"] = np.array([b.num_rows])
        for j, buf in enumerate(b.buffers):
            arrays[f"b{i}_buf{j}"] = buf
    meta = []
    for P, bsz, keys in [(2, 4, [1, 2, 3]), (3, 4096, [3, 5]), (5, 2, [6, 1])]:
        out = O.run_ref(REF_FIXTURE_SCHEMA, seq, P, keys, buffer_size=bsz)
        tag = f"p{P}_b{bsz}"
        arrays[f"{tag}_data"] = np.frombuffer(out.data, np.uint8)
        arrays[f"{tag}_lengths"] = out.partition_lengths
        arrays[f"{tag}_raw"] = out.raw_partition_lengths
        meta.append({"tag": tag, "num_partitions": P, "buffer_size": bsz, "keys": keys})
    np.savez_compressed(os.path.join(HERE, "ref_fixture.npz"), **arrays)
    with open(os.path.join(HERE, "ref_fixture.json"), "w") as f:
        json.dump({"schema": [[x.name, x.type, x.nullable] for x in REF_FIXTURE_SCHEMA],
                   "sequence": [0, 1, 0], "runs": meta}, f, indent=1)
    print("ref fixture", [m["tag"] for m in meta])

    precs = []
    for name, short_name, P, opts, gen in partitioner_cases():
        schema, batches = partitioner_inputs(short_name, gen, P)
        precs.append(record(name, schema, batches, P, [], opts, gen, short_name))
        print(name, precs[-1]["data_sha256"][:16])
    with open(os.path.join(HERE, "partitioners.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": precs}, f, indent=1)


if __name__ == "__main__":
    main()
