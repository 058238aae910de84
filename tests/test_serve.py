"""The served form: Split / Stop calls of many concurrent tasks through the serving loop.

Each task's output must be byte-identical to the same task split alone through the plain
per-call API (itself checked against the oracle elsewhere), whatever the interleaving, the
worker count or the spills forced by a small spill threshold; admission must hold a task back
until the HBM budget has room for it.
"""
import threading
import time

import numpy as np
import pytest

from gazelle_plugin_gb300 import shuffle as S
from gazelle_plugin_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tasks(seed, n_tasks, batches_per_task, max_rows=20000):
    rng = np.random.Generator(np.random.PCG64(seed))
    tasks = []
    for t in range(n_tasks):
        si = t % 3
        schema, keys = W.C4_SCHEMAS[si]
        P = W.C4_PARTITIONS[(t // 3) % 3]
        rows = np.minimum(W.c4_rows(rng, batches_per_task), max_rows)
        batches = [W.c4_batch(rng, si, int(r)) for r in rows]
        tasks.append((schema, keys, P, batches))
    return tasks


OPTS = dict(bufferSize=4096, writeSchema=False, flush_bytes=2 << 20, device_budget=4 << 20)


def _alone(schema, keys, P, batches):
    return S.split_batches(schema, batches, P, keys, **OPTS)


def _served(tasks, slots, budget=8 << 30, in_flight=8, seed=0):
    srv = S.ServeLoop(slots=slots, hbmBudget=budget)
    w = S.ShuffleSplitterJniWrapper()
    try:
        handles = [srv.open(schema, P, keys, **OPTS) for schema, keys, P, _ in tasks]
        # interleave the tasks' calls in a random order, keeping up to `in_flight` outstanding
        order = [t for t, (_, _, _, b) in enumerate(tasks) for _ in b]
        np.random.Generator(np.random.PCG64(seed)).shuffle(order)
        nxt = [0] * len(tasks)
        pending, lat = [], []
        for t in order:
            b = tasks[t][3][nxt[t]]
            nxt[t] += 1
            a, z = b.addrs_sizes()
            pending.append((srv.split(handles[t], b.num_rows, a, z), b))
            if len(pending) >= in_flight:
                lat.append(srv.wait(pending.pop(0)[0]))
        for tk, _ in pending:
            lat.append(srv.wait(tk))
        for h in handles:
            srv.wait(srv.stop(h))
        out = []
        for h, (_, _, P, _) in zip(handles, tasks):
            out.append((w.stop(h, P), w.data(h)))
            w.close(h)
        return out, lat
    finally:
        srv.shutdown()


@pytest.mark.parametrize("slots", [1, 4])
def test_served_mix_equals_alone(slots):
    tasks = _tasks(31, 9, 6)
    served, lat = _served(tasks, slots)
    assert len(lat) == sum(len(b) for *_, b in tasks) and min(lat) > 0
    for i, (schema, keys, P, batches) in enumerate(tasks):
        res, data = _alone(schema, keys, P, batches)
        sres, sdata = served[i]
        assert sdata == data, f"task {i}"
        assert np.array_equal(sres.partitionLengths, res.partitionLengths), f"task {i}"
        assert np.array_equal(sres.rawPartitionLengths, res.rawPartitionLengths), f"task {i}"


def test_served_task_matches_oracle():
    schema, keys, P, batches = _tasks(32, 3, 5)[2]
    served, _ = _served([(schema, keys, P, batches)], 2)
    ref = O.run_oracle(schema, batches, P, keys, buffer_size=4096)
    res, data = served[0]
    assert data == ref.data
    assert np.array_equal(res.partitionLengths, ref.partition_lengths)


def test_admission_waits_for_budget():
    # each task needs device_budget + 3 * flush_bytes + 64 MiB = 80 MiB: two do not fit in 120 MiB
    opts = dict(bufferSize=1024, writeSchema=False, flush_bytes=1 << 20, device_budget=13 << 20)
    srv = S.ServeLoop(slots=2, hbmBudget=120 << 20)
    w = S.ShuffleSplitterJniWrapper()
    try:
        first = srv.open(W.C1_SCHEMA, 8, W.C1_KEYS, **opts)
        got = {}

        def second():
            got["task"] = srv.open(W.C1_SCHEMA, 8, W.C1_KEYS, **opts)

        th = threading.Thread(target=second)
        th.start()
        time.sleep(0.5)
        assert "task" not in got  # held back: the budget is taken
        b = W.c1_batches(5, 1, 1000)[0]
        a, z = b.addrs_sizes()
        srv.wait(srv.split(first, b.num_rows, a, z))
        srv.wait(srv.stop(first))
        th.join(timeout=30)
        assert "task" in got  # admitted once the first task stopped
        srv.wait(srv.stop(got["task"]))
        w.close(first)
        w.close(got["task"])
    finally:
        srv.shutdown()


def test_task_larger_than_budget_is_rejected():
    srv = S.ServeLoop(slots=1, hbmBudget=32 << 20)
    try:
        with pytest.raises(S.SplitterError) as e:
            srv.open(W.C1_SCHEMA, 8, W.C1_KEYS, writeSchema=False, device_budget=1 << 30)
        assert e.value.status == S.GZ_INVALID
    finally:
        srv.shutdown()


def test_served_nested_tasks_equal_alone():
    """Tasks with nested columns (list / map / struct) beside flat ones through the serving loop."""
    from tests.golden import make_golden as G
    rng = np.random.default_rng(17)
    tasks = []
    for t in range(4):
        schema = [W.Field("k", "int64", False), G.NESTED_SHAPES[(3 * t) % len(G.NESTED_SHAPES)]("a"),
                  G.NESTED_SHAPES[(3 * t + 1) % len(G.NESTED_SHAPES)]("b")]
        batches = []
        for _ in range(5):
            n = int(rng.integers(500, 4000))
            bufs = W._column(rng, schema[0], n, rng.integers(0, 1 << 40, size=n), 0.0)
            for f in schema[1:]:
                bufs += W.nested_column(rng, f, n, 0.2, 4)
            batches.append(W.Batch(n, bufs))
        tasks.append((schema, [0], [16, 200][t % 2], batches))
    served, _ = _served(tasks, slots=2)
    for (schema, keys, P, batches), (res, data) in zip(tasks, served):
        _, want = _alone(schema, keys, P, batches)
        assert data == want
        assert data == O.run_oracle(schema, batches, P, keys, buffer_size=4096).data
