"""gz_hash_partition_static, the entry point that allocates no device memory.

Some callers cannot call cudaMalloc: their device memory all belongs to another allocator (a
pool that reserved the free HBM up front, or an executor that charges every device byte to a
task's budget), or they must not let cudaMalloc / cudaFree stall the device.  For them the
library computes a batch's partition ids and per-partition row counts with its scratch in a
fixed 16 MiB device array of its own.

Checked through the C ABI, exactly, against the oracle's partition ids and against the
splitter's own (gz_split_last_pids) for the same batch, on calls in a row that share and reuse
that array (shared-memory and global-memory count paths, then the first case again, and a key
list with a null-type key, which leaves the hash unchanged).  Around every call after the first,
the device's free memory must not change: the call allocates nothing.  Collected last so that a
run stopping at the first failure has run every other test first; it also passes alone in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MAX_COUNTERS = 4 * 1024 * 1024  # per-tile counters the static array holds
TILE_ROWS = 1024


class GzKeyColumn(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("validity", ctypes.c_void_p), ("values", ctypes.c_void_p)]


def _entry():
    f = S.lib().gz_hash_partition_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(GzKeyColumn), ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    S.lib().gz_last_error(0, buf, len(buf))
    return buf.value.decode()


def _splitter_pids(schema, keys, P, batch):
    """Partition ids from the existing entry points: make, split (host buffers), last_pids."""
    w = S.ShuffleSplitterJniWrapper()
    h = w.make(S.NativePartitioning("hash", P, None, keys, list(schema)), writeSchema=False)
    try:
        addrs, sizes = batch.addrs_sizes()
        w.split(h, batch.num_rows, addrs, sizes)
        return w.lastPids(h, batch.num_rows)
    finally:
        w.close(h)


def _oracle_pids(schema, keys, P, batch):
    o = O.OracleSplitter(schema, P, keys)
    try:
        o.split(batch)
        return o.last_pids(batch.num_rows)
    finally:
        o.close()


def _device_keys(schema, keys, batch):
    """Key columns copied to the device; returns the ctypes array and the tensors that own it."""
    first = []
    b = 0
    for f in schema:
        first.append(b)
        b += 3 if f.is_binary else 2
    hold, cols = [], (GzKeyColumn * len(keys))()
    for j, k in enumerate(keys):
        cols[j].type = schema[k].code
        if schema[k].type == "null":  # no buffers are read
            cols[j].values = None
            cols[j].validity = None
            continue
        valid = batch.buffers[first[k]].view(np.uint8)
        vals = batch.buffers[first[k] + 1].view(np.uint8)
        dv = torch.from_numpy(vals.copy()).cuda()
        hold.append(dv)
        cols[j].values = dv.data_ptr()
        if valid.nbytes:
            dm = torch.from_numpy(valid.copy()).cuda()
            hold.append(dm)
            cols[j].validity = dm.data_ptr()
        else:
            cols[j].validity = None
    return cols, hold


def _static_call(schema, keys, P, batch):
    cols, hold = _device_keys(schema, keys, batch)
    n = batch.num_rows
    pids16 = torch.full((max(n, 1),), -1, dtype=torch.int16, device="cuda")  # 0xFFFF: unwritten
    counts = torch.full((P,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    st = _entry()(0, P, cols, len(keys), n, pids16.data_ptr(), counts.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
    assert st == 0, _last_error()
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    del hold
    got = pids16[:n].cpu().numpy().view(np.uint16)
    return got, counts.cpu().numpy(), free_before - free_after


def _with_null_key():
    """The c1 schema with a null-type field in front, listed first among the keys."""
    schema = [W.Field("n", "null")] + list(W.C1_SCHEMA)
    b = W.c1_batches(44, 1, 3000)[0]
    empty = np.zeros(0, np.uint8)
    batch = W.Batch(b.num_rows, [empty, empty] + list(b.buffers))
    return schema, [0] + [k + 1 for k in W.C1_KEYS], batch


CASES = [
    # P <= 12288: the tile histogram is counted in shared memory
    ("c2", W.C2_SCHEMA, W.C2_KEYS, 200, lambda: W.c2_batches(41, 1, 20000)[0]),
    # P > 12288: counted in the static array itself (cleared per tile), null keys
    ("c3", W.C3_SCHEMA, W.C3_KEYS, 20000, lambda: W.c3_batches(42, 1, 32768, 0.2, 0.05)[0]),
    # the first case again, after the second left its counts in the array
    ("c2-again", W.C2_SCHEMA, W.C2_KEYS, 200, lambda: W.c2_batches(41, 1, 20000)[0]),
    ("c1", W.C1_SCHEMA, W.C1_KEYS, 8, lambda: W.c1_batches(43, 1, 5000)[0]),
]


def test_static_scratch_matches_oracle_and_splitter_on_consecutive_calls():
    cases = [(tag, schema, keys, P, make()) for tag, schema, keys, P, make in CASES]
    nschema, nkeys, nbatch = _with_null_key()
    cases.append(("null-type key", nschema, nkeys, 8, nbatch))
    for i, (tag, schema, keys, P, batch) in enumerate(cases):
        want = _oracle_pids(schema, keys, P, batch)
        assert np.array_equal(_splitter_pids(schema, keys, P, batch), want), tag
        got, counts, grown = _static_call(schema, keys, P, batch)
        assert np.array_equal(got, want), tag
        assert np.array_equal(counts, np.bincount(want, minlength=P).astype(np.int64)), tag
        if i > 0:  # the first call on the device may load the module that holds the array
            assert grown == 0, f"{tag}: free device memory fell by {grown} bytes during the call"


def test_static_scratch_rejects_oversized_call():
    cols = (GzKeyColumn * 1)()
    dummy = torch.zeros(8, dtype=torch.int64, device="cuda")
    cols[0].type = W.TYPE_CODES["int64"]
    cols[0].values = dummy.data_ptr()
    P = 65536
    rows = (MAX_COUNTERS // P) * TILE_ROWS + 1  # one tile more than the array holds
    st = _entry()(0, P, cols, 1, rows, dummy.data_ptr(), dummy.data_ptr(), None)
    assert st == S.GZ_INVALID
    assert "static scratch" in _last_error()
