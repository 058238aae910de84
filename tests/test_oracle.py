"""The oracle itself: pinned against published hash check values, against the reference's
own hash code and against golden fixtures made by running the reference Splitter."""
import hashlib
import json
import os

import numpy as np
import pytest

from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O
from tests.golden import make_golden as G

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "splits.json")))["cases"]


def lib():
    return O.OracleSplitter.lib()


def test_murmur3_smhasher_verification():
    """SMHasher's verification procedure for MurmurHash3_x86_32: hash keys {0}, {0,1}, ...
    with seed 256-i, then hash the concatenated hashes with seed 0 -> 0xB0F57EE3."""
    key = np.arange(256, dtype=np.uint8)
    hashes = np.zeros(256, np.uint32)
    for i in range(256):
        hashes[i] = lib().gzo_murmur3_bytes(key.ctypes.data, i, 256 - i)
    final = lib().gzo_murmur3_bytes(hashes.ctypes.data, 1024, 0)
    assert final == 0xB0F57EE3


def test_spark_hash_equals_generic_murmur3():
    rng = np.random.default_rng(7)
    for v, seed in zip(rng.integers(-2**31, 2**31, 2000), rng.integers(-2**31, 2**31, 2000)):
        b = np.array([v], np.int32)
        g = lib().gzo_murmur3_bytes(b.ctypes.data, 4, int(seed) & 0xFFFFFFFF)
        assert lib().gzo_hash_int(int(v), int(seed)) & 0xFFFFFFFF == g
    for v, seed in zip(rng.integers(-2**63, 2**63, 2000, dtype=np.int64),
                       rng.integers(-2**31, 2**31, 2000)):
        b = np.array([v], np.int64)
        g = lib().gzo_murmur3_bytes(b.ctypes.data, 8, int(seed) & 0xFFFFFFFF)
        assert lib().gzo_hash_long(int(v), int(seed)) & 0xFFFFFFFF == g


def test_spark_hash_long_matches_reference_murmurhash32():
    if not os.path.exists(O.REF_HASH_SO):
        pytest.skip("reference hash helper not built here (needs the reference tree)")
    import ctypes
    ref = ctypes.CDLL(O.REF_HASH_SO)
    ref.gzref_hash_long.restype = ctypes.c_int32
    ref.gzref_hash_long.argtypes = [ctypes.c_int64, ctypes.c_int32]
    rng = np.random.default_rng(11)
    for v, seed in zip(rng.integers(-2**63, 2**63, 5000, dtype=np.int64),
                       rng.integers(-2**31, 2**31, 5000)):
        assert lib().gzo_hash_long(int(v), int(seed)) == ref.gzref_hash_long(int(v), int(seed))


def test_pmod():
    for h in [-2**31, -7, -1, 0, 1, 7, 2**31 - 1]:
        for p in [1, 2, 7, 200, 65536]:
            assert lib().gzo_pmod(h, p) == h % p  # python % is the positive modulus


def check_against(case, out):
    assert list(out.partition_lengths) == case["partition_lengths"]
    assert list(out.raw_partition_lengths) == case["raw_partition_lengths"]
    assert out.bytes_spilled == case["bytes_spilled"]
    assert out.bytes_written == case["bytes_written"]
    if case["partition_sha256"] is not None:
        for p, h in enumerate(case["partition_sha256"]):
            assert hashlib.sha256(out.partition_bytes(p)).hexdigest() == h, f"partition {p}"
    assert hashlib.sha256(out.data).hexdigest() == case["data_sha256"]


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_oracle_matches_reference_golden(case):
    batches = G.regenerate(case)
    assert G.input_digest(batches) == case["input_sha256"], \
        "input generator differs from the one the fixture was made with"
    schema = [W.Field(n, t, nl) for n, t, nl in case["schema"]]
    out = O.run_oracle(schema, batches, case["num_partitions"], case["keys"], **case["options"])
    check_against(case, out)


def ref_fixture():
    meta = json.load(open(os.path.join(HERE, "golden", "ref_fixture.json")))
    z = np.load(os.path.join(HERE, "golden", "ref_fixture.npz"))
    schema = [W.Field(n, t, nl) for n, t, nl in meta["schema"]]
    batches = []
    for i in range(2):
        nbuf = len([k for k in z.files if k.startswith(f"b{i}_buf")])
        batches.append(W.Batch(int(z[f"b{i}_rows"][0]), [z[f"b{i}_buf{j}"] for j in range(nbuf)]))
    return schema, [batches[i] for i in meta["sequence"]], meta["runs"], z


def test_oracle_matches_reference_unit_test_batches():
    schema, seq, runs, z = ref_fixture()
    for r in runs:
        out = O.run_oracle(schema, seq, r["num_partitions"], r["keys"], buffer_size=r["buffer_size"])
        assert out.data == z[f"{r['tag']}_data"].tobytes(), r["tag"]
        assert (out.partition_lengths == z[f"{r['tag']}_lengths"]).all()
        assert (out.raw_partition_lengths == z[f"{r['tag']}_raw"]).all()


@pytest.mark.skipif(not O.RefSplitter.available(), reason="reference build absent here")
def test_oracle_matches_live_reference_random():
    for seed in range(5000, 5060):
        schema, batches, P, keys, opts = G.random_case(seed)
        r = O.run_ref(schema, batches, P, keys, **opts)
        o = O.run_oracle(schema, batches, P, keys, **opts)
        assert r.data == o.data, seed
        assert (r.raw_partition_lengths == o.raw_partition_lengths).all(), seed
        assert r.bytes_spilled == o.bytes_spilled, seed


def test_oracle_spill_fixed_size_matches_reference_policy():
    """SpillFixedSize only finds cached (unspilled) batches when prefer_spill is off."""
    batches = W.c1_batches(0, 24, 512)
    s = O.OracleSplitter(W.C1_SCHEMA, 8, [0], buffer_size=512, prefer_spill=True)
    for b in batches:
        s.split(b)
    assert s.spill(1 << 30) == 0
    s2 = O.OracleSplitter(W.C1_SCHEMA, 8, [0], buffer_size=512, prefer_spill=False)
    for b in batches:
        s2.split(b)
    assert s2.spill(1 << 30) > 0
    if O.RefSplitter.available():
        r = O.RefSplitter(W.C1_SCHEMA, 8, [0], buffer_size=512, prefer_spill=False)
        for b in batches:
            r.split(b)
        s3 = O.OracleSplitter(W.C1_SCHEMA, 8, [0], buffer_size=512, prefer_spill=False)
        for b in batches:
            s3.split(b)
        assert r.spill(100000) == s3.spill(100000)
        ro, so = r.stop(), s3.stop()
        assert ro.data == so.data and ro.bytes_spilled == so.bytes_spilled
        r.close()


def _null_key_case():
    """The c1 workload with a null-type field in front of it, listed first among the keys."""
    schema = [W.Field("n", "null")] + list(W.C1_SCHEMA)
    empty = np.zeros(0, np.uint8)
    batches = [W.Batch(b.num_rows, [empty, empty] + list(b.buffers)) for b in W.c1_batches(3, 4, 2000)]
    return schema, batches, [0] + [k + 1 for k in W.C1_KEYS]


def test_oracle_null_type_key_leaves_hash_unchanged():
    """CreateProjector adds nothing to the chain for a NullType key (splitter.cc:1407-1408)."""
    schema, batches, keys = _null_key_case()
    with_null = O.run_oracle(schema, batches, 8, keys)
    without = O.run_oracle(schema, batches, 8, keys[1:])
    assert with_null.data == without.data
    assert (with_null.partition_lengths == without.partition_lengths).all()


@pytest.mark.skipif(not O.RefSplitter.available(), reason="reference build absent here")
def test_oracle_null_type_key_matches_live_reference():
    schema, batches, keys = _null_key_case()
    r = O.run_ref(schema, batches, 8, keys)
    o = O.run_oracle(schema, batches, 8, keys)
    assert r.data == o.data
    assert (r.raw_partition_lengths == o.raw_partition_lengths).all()


@pytest.mark.skipif(not O.RefSplitter.available(), reason="reference build absent here")
def test_oracle_utf8_keys_match_live_reference():
    """utf8 hash keys: the reference's hashbuf_spark has no body in the reference tree; both the
    oracle and the reference build's gandiva stand-in restate Spark's hashUnsafeBytes, so this
    checks the chain, nulls and tail-byte handling end to end, not the fork's body."""
    rng = np.random.default_rng(77)
    schema = [W.Field("s", "utf8"), W.Field("k", "int32"), W.Field("v", "int64")]
    hi = bytes(range(1, 256))
    for trial in range(6):
        batches = [W.random_batch(rng, schema, int(rng.integers(100, 2000)), 0.2) for _ in range(3)]
        for b in batches[::2]:
            b.buffers[0:3] = W._column(rng, schema[0], b.num_rows, None, 0.1, (0, 23, hi))
        keys = [[0], [0, 1], [1, 0]][trial % 3]
        r = O.run_ref(schema, batches, 16, keys)
        o = O.run_oracle(schema, batches, 16, keys)
        assert r.data == o.data, trial
