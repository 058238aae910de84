#!/usr/bin/env python
"""Hash-split throughput of the GB300 shuffle splitter on the wide fact-table workload.

Workload (one step): 200M rows in 4096-row record batches, 16 columns = 4 int64 keys
U[0,6e8), 4 float64 U[0,1e5) at 0.01 granularity, 2 int32 U[8000,10600), 3 single-char utf8
flags over 3-symbol alphabets, 3 utf8 comments of U{10..44} chars over [a-z ]; 2% nulls in the
12 non-key columns; hash keys = columns 0 and 1; 200 partitions; compression off.  The rows
are generated on the device with a seeded torch RNG (36 GB of inputs, far above the 126 MB
L2, so every step reads HBM).

Lines:
  value : the split with the inputs resident in HBM (GZ_INPUT_DEVICE_RETAINED), the batches
          handed over by gz_split_split_batches (the writer's per-batch loop run inside the
          library), until the device work is complete.  Explains the kernels; not the drop-in.
  e2e   : the drop-in as a Spark executor calls it: T map tasks at once (one per host core, as
          the CPU arm), each a native loop of make / one gz_split_split per 4096-row batch on
          pageable host buffers / gz_split_stop writing its data file to tmpfs / close
          (libgztask.so, ColumnarShuffleWriter.write's loop); plus the same with one task.
  metric: (input buffer bytes + raw partition bytes) / time, in GB/s.
  output check: the e2e data files are digested and compared with the oracle's data files for
          the same task shards (the CPU baseline leg, which splits the whole workload on all
          host cores with Stop writing its files too).
  forms : batched (512 uneven batches of 3 schemas, autotuned passes), served (32 tasks through
          the serving loop, per-Split latency) and fanout (Zipf keys, 16..8000 partitions), each
          beside its plain per-batch counterpart where it has one; --no-forms skips them.

--partitioner rr | range times the same table split by the round-robin selection or by an
int32 partition id column U[0, 200) put in front of it (Splitter::Make "rr" / "range"); the
headline is hash.

--impl reference times the CPU splitter (the oracle's restatement of the reference Splitter;
the reference itself needs the Arrow fork and x86) as map tasks on all host cores, split and
Stop with data files, over a bounded sample of the same batches.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "hash-split GB/s ((input + partition bytes) / split time)"
WORKLOAD = ("wide fact-table split: 200M rows, 4096-row batches, 16 columns "
            "(4 int64 keys, 4 float64, 2 int32, 3 utf8 flags, 3 utf8 comments), "
            "2% nulls, hash on keys 0-1, 200 partitions")
BATCH_ROWS = 4096
PARTITIONS = 200
# ncu DRAM traffic of one k_scatter launch of this workload (dram__bytes_read.sum +
# dram__bytes_write.sum) against its algorithmic bytes, written with the command that made it
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "k_scatter_traffic.json")
# The restatement runs slower than the reference Splitter itself: measured on one x86 core on
# 256 batches of this workload, split + Stop with a data file: 0.910 GB/s restated vs 1.120 GB/s
# for the reference compiled from its sources (split alone 1.103 vs 1.456).  The reference
# cannot be built on the Arm host (its x86 intrinsics and the Arrow library it links).
REFERENCE_OVER_PORT = 1.120 / 0.910
KEYS = [0, 1]


def schema():
    from gazelle_plugin_gb300 import workloads as W
    return W.C2_SCHEMA


def metric_and_workload(partitioner: str):
    """The headline is the hash split; --partitioner rr / range time the same table split by
    the round-robin selection or by a uniform int32 partition id column in front of it."""
    if partitioner == "hash":
        return METRIC, WORKLOAD
    what = {"rr": "round-robin", "range": "int32 partition ids U[0, 200) as field 0"}[partitioner]
    return (METRIC.replace("hash-split", f"{partitioner}-split"),
            WORKLOAD.replace("hash on keys 0-1", what))


def workload_inputs(total_rows: int, seed: int, partitioner: str):
    """(schema, keys, rows, addrs, sizes, tensors) of the workload on cuda:0; the range split
    gets its partition id column as field 0."""
    import torch
    from gazelle_plugin_gb300 import workloads as W
    rows, addrs, sizes, keep = generate_on_device(total_rows, seed=seed)
    sch, keys = list(schema()), list(KEYS)
    if partitioner != "hash":
        keys = []
    if partitioner == "range":
        g = torch.Generator(device="cuda")
        g.manual_seed(1000 + seed)
        nb = len(rows)
        pid = torch.randint(0, PARTITIONS, (nb * BATCH_ROWS,), generator=g, device="cuda",
                            dtype=torch.int32)
        r64 = rows.astype(np.int64)
        pa = pid.data_ptr() + np.arange(nb, dtype=np.int64) * BATCH_ROWS * 4
        addrs = np.concatenate([np.zeros((nb, 1), np.int64), pa[:, None], addrs], axis=1)
        sizes = np.concatenate([np.zeros((nb, 1), np.int64), (r64 * 4)[:, None], sizes], axis=1)
        keep = [None, pid] + list(keep)
        sch = [W.Field("pid", "int32", False)] + sch
        torch.cuda.synchronize()
    return sch, keys, rows, addrs, sizes, keep


# ---------------------------------------------------------------------------------------
def generate_on_device(total_rows: int, seed: int = 1):
    """Seeded workload batches on cuda:0.  Returns (rows[int32], addrs[nb, nbufs],
    sizes[nb, nbufs], tensors) where column j of addrs points into tensors[j] (None for the
    empty validity buffers of the key columns)."""
    import torch
    dev = "cuda"
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    br = BATCH_ROWS
    nb = (total_rows + br - 1) // br
    npad = nb * br
    rows = np.full(nb, br, np.int32)
    rows[-1] = total_rows - (nb - 1) * br
    r64 = rows.astype(np.int64)
    b_idx = np.arange(nb, dtype=np.int64)
    weights = (2 ** torch.arange(8, device=dev, dtype=torch.int32)).to(torch.int32)
    bufcols = []  # (tensor or None, addr[nb], size[nb])

    def add(t, addr, size):
        bufcols.append((t, np.asarray(addr, np.int64), np.asarray(size, np.int64)))

    def validity():
        v = torch.rand(npad, generator=g, device=dev) >= 0.02
        bits = (v.view(-1, 8).to(torch.int32) * weights).sum(1).to(torch.uint8)
        add(bits, bits.data_ptr() + b_idx * (br // 8), (r64 + 7) // 8)
        return v

    for _ in range(4):
        t = torch.randint(0, 600_000_000, (npad,), generator=g, device=dev, dtype=torch.int64)
        add(None, np.zeros(nb), np.zeros(nb))
        add(t, t.data_ptr() + b_idx * br * 8, r64 * 8)
    for _ in range(4):
        validity()
        t = torch.floor(torch.rand(npad, generator=g, device=dev, dtype=torch.float64) * 1e7) / 100.0
        add(t, t.data_ptr() + b_idx * br * 8, r64 * 8)
    for _ in range(2):
        validity()
        t = torch.randint(8000, 10600, (npad,), generator=g, device=dev, dtype=torch.int32)
        add(t, t.data_ptr() + b_idx * br * 4, r64 * 4)
    for alphabet, lo, hi in [(b"AFN", 1, 1), (b"OFP", 1, 1), (b"RAN", 1, 1),
                             (b"abcdefghijklmnopqrstuvwxyz ", 10, 44),
                             (b"abcdefghijklmnopqrstuvwxyz ", 10, 44),
                             (b"abcdefghijklmnopqrstuvwxyz ", 10, 44)]:
        v = validity()
        lens = torch.randint(lo, hi + 1, (npad,), generator=g, device=dev, dtype=torch.int32)
        lens = lens * v.to(torch.int32)  # a null slot has no characters
        off = torch.zeros((nb, br + 1), dtype=torch.int32, device=dev)
        off[:, 1:] = torch.cumsum(lens.view(nb, br), dim=1, dtype=torch.int32)
        last = torch.from_numpy(rows.astype(np.int64)).to(dev)
        totals = off.gather(1, last.view(-1, 1)).view(-1).to(torch.int64)
        starts = torch.cumsum(totals, 0) - totals
        alpha = torch.tensor(list(alphabet), dtype=torch.uint8, device=dev)
        chars = alpha[torch.randint(0, len(alphabet), (int(totals.sum().item()) + 16,),
                                    generator=g, device=dev)]
        add(off, off.data_ptr() + b_idx * (br + 1) * 4, (r64 + 1) * 4)
        add(chars, chars.data_ptr() + starts.cpu().numpy(), totals.cpu().numpy())
    addrs = np.stack([c[1] for c in bufcols], axis=1)
    sizes = np.stack([c[2] for c in bufcols], axis=1)
    addrs[sizes == 0] = 0
    torch.cuda.synchronize()
    return rows, addrs, sizes, [c[0] for c in bufcols]


def reduce_over_ranks(x: float, op: str = "max") -> float:
    """Max or sum of a per-rank figure over the process group (identity without one): replicas
    split disjoint inputs with no data-path collective, only their times and bytes are combined."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def link_bandwidth(nbytes: int = 1 << 30) -> dict:
    """Host link of this box: one pinned 1 GiB buffer copied host->device and device->host (best
    of 3, CUDA events).  The end-to-end figure moves the input and the partition bytes over it."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = 0.0
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            best = max(best, nbytes / (a.elapsed_time(b) * 1e-3) / 1e9)
        out[name] = best
    del h, d
    return out


def pageable_copy(addrs, sizes, tensors):
    """Ordinary (pageable) host copies of the generated buffers, laid out like the device ones:
    the kind of memory Arrow Java's off-heap buffers live in.  Returns (host addrs, arrays)."""
    import torch
    haddrs = np.zeros_like(addrs)
    keep = []
    for j, t in enumerate(tensors):
        if t is None:
            continue
        h = t.view(-1).view(torch.uint8).cpu().numpy()  # torch's CPU allocator: not pinned
        keep.append(h)
        haddrs[:, j] = addrs[:, j] - t.data_ptr() + h.ctypes.data
    haddrs[sizes == 0] = 0
    return haddrs, keep


def scratch_dir() -> str:
    """A fresh directory for data files, on tmpfs when the box has one."""
    import tempfile
    base = "/dev/shm" if os.path.isdir("/dev/shm") and os.access("/dev/shm", os.W_OK) else None
    return tempfile.mkdtemp(prefix="gz-bench-", dir=base)


def remove_dir(d: str) -> None:
    import shutil
    shutil.rmtree(d, ignore_errors=True)


def task_files(ddir: str, n: int):
    return [os.path.join(ddir, f"task-{t:04d}.data") for t in range(n)]


def digests(paths):
    """(checksum, bytes) of every file, computed on all host cores."""
    from concurrent.futures import ThreadPoolExecutor
    from gazelle_plugin_gb300 import shuffle as S
    with ThreadPoolExecutor(max_workers=min(len(paths), os.cpu_count() or 1)) as ex:
        return list(ex.map(S.digest_file, paths))


def read_back(sch, paths, lengths, partitions=None, tasks: int = 1):
    """The reduce side: every partition's streams of all map outputs (the task files, memory
    mapped: page-cache bytes, as a shuffle fetch leaves them) read into device columns by the
    CUDA reader, one reader per partition, `tasks` reduce tasks at once (each on its own thread,
    as an executor's task slots run them, taking the partitions in turn).
    GB/s = (stream bytes + column bytes) / time."""
    from concurrent.futures import ThreadPoolExecutor
    from gazelle_plugin_gb300 import shuffle as S
    maps = [np.memmap(p, dtype=np.uint8, mode="r") for p in paths]
    starts = [np.concatenate([[0], np.cumsum(l)]) for l in lengths]
    P = lengths[0].shape[0]
    parts = list(range(P) if partitions is None else partitions)

    def task(ps):
        ib = ob = 0
        for p in ps:
            r = S.PartitionReader(list(sch))
            for m, st in zip(maps, starts):
                if st[p + 1] > st[p]:
                    r.addStream(m[st[p]:st[p + 1]])
                    ib += int(st[p + 1] - st[p])
            r.finish()
            for f in range(len(sch)):
                c = r.column(f)
                ob += c.values_bytes + (c.length + 1) * 4 * (c.offsets is not None) + \
                    ((c.length + 7) // 8 if c.validity else 0)
            r.close()
        return ib, ob

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=tasks) as ex:
        done = list(ex.map(task, [parts[i::tasks] for i in range(tasks)]))
    dt = time.perf_counter() - t0
    in_bytes = sum(d[0] for d in done)
    out_bytes = sum(d[1] for d in done)
    del maps
    return {"value": (in_bytes + out_bytes) / dt / 1e9, "unit": "GB/s", "seconds": dt,
            "stream_bytes": in_bytes, "column_bytes": out_bytes, "partitions": len(parts),
            "reduce_tasks": tasks,
            "what": ("each partition's streams of all map outputs (memory-mapped data files) into one "
                     "set of device columns (host parse, one copy per stream, device concatenation), "
                     f"{tasks} reduce tasks at once")}


def oracle_tasks(sch, keys, partitioner, rows, haddrs, sizes, n_tasks: int, ddir: str, digest: bool = False):
    """The CPU splitter as map tasks: `n_tasks` oracle splitters on their own threads, each over a
    contiguous range of the batches (the same ranges the GPU tasks take), split then Stop writing
    <ddir>/task-<t>.data.  Returns (wall seconds, input bytes, raw partition bytes, [per-task
    partition lengths], [per-task (checksum, size)] or None).  With `digest`, each task checksums
    and deletes its file after its clock has stopped (keeps host memory low)."""
    import ctypes
    from oracle import oracle as O
    L = O.OracleSplitter.lib()
    nb = len(rows)
    rows = np.ascontiguousarray(rows, np.int32)
    haddrs = np.ascontiguousarray(haddrs, np.int64)
    sizes = np.ascontiguousarray(sizes, np.int64)
    nbufs = haddrs.shape[1]
    paths = task_files(ddir, n_tasks)
    res = [None] * n_tasks
    errs = [None] * n_tasks
    sps = [O.OracleSplitter(sch, PARTITIONS, keys, short_name=partitioner) for _ in range(n_tasks)]
    barrier = threading.Barrier(n_tasks + 1)
    a0, z0, row_bytes = haddrs.ctypes.data, sizes.ctypes.data, nbufs * 8

    def work(t):
        b0, b1 = nb * t // n_tasks, nb * (t + 1) // n_tasks
        sp = sps[t]
        P = sp.P
        err = ctypes.create_string_buffer(512)
        lengths, raw, m = np.zeros(P, np.int64), np.zeros(P, np.int64), np.zeros(3, np.int64)
        barrier.wait()
        for b in range(b0, b1):
            if rows[b] == 0:
                continue
            if L.gzo_split(sp.h, int(rows[b]), a0 + b * row_bytes, z0 + b * row_bytes, nbufs, err, 512):
                errs[t] = err.value.decode()
                return
        if L.gzo_stop(sp.h, paths[t].encode(), lengths.ctypes.data, raw.ctypes.data, m.ctypes.data,
                      err, 512) < 0:
            errs[t] = err.value.decode()
            return
        sp.close()
        t_end = time.perf_counter()
        dig = None
        if digest:
            from gazelle_plugin_gb300 import shuffle as S
            dig = S.digest_file(paths[t])
            os.remove(paths[t])
        res[t] = (t_end, int(raw.sum()), lengths, dig)

    ths = [threading.Thread(target=work, args=(t,)) for t in range(n_tasks)]
    for t in ths:
        t.start()
    barrier.wait()
    t0 = time.perf_counter()
    for t in ths:
        t.join()
    if any(r is None for r in res):
        raise RuntimeError(f"an oracle task failed: {[e for e in errs if e]}")
    wall = max(r[0] for r in res) - t0
    return (wall, int(sizes[:nb].sum()), sum(r[1] for r in res), [r[2] for r in res],
            [r[3] for r in res] if digest else None)


# ---------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sms) if sms else None,
                "sm_max_mhz": max(maxs) if maxs else None,
                "reasons": sorted(reasons), "samples": len(sms)}


def traffic_per_launch(alg_per_launch: float, given=None):
    """DRAM bytes of one k_scatter launch: given, else the algorithmic bytes of this run's average
    launch times the DRAM / algorithmic ratio of the committed ncu capture (None without one)."""
    if given:
        return given
    try:
        with open(TRAFFIC_FILE) as f:
            t = json.load(f)
        return alg_per_launch * t["dram_bytes"] / t["algorithmic_bytes"]
    except (OSError, KeyError, ValueError, ZeroDivisionError):
        return None


def measured_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------------------
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch
    threads = args.tasks or min(os.cpu_count() or 1, 16)
    n_rows = min(args.ref_rows, args.rows)
    sch, keys, rows, addrs, sizes, keep = workload_inputs(n_rows, 1, args.partitioner)
    haddrs, host = pageable_copy(addrs, sizes, keep)
    del keep
    torch.cuda.empty_cache()
    ddir = scratch_dir()
    try:
        for _ in range(args.warmup):
            oracle_tasks(sch, keys, args.partitioner, rows, haddrs, sizes, threads, ddir)
        times, nbytes = [], 0
        for _ in range(args.steps):
            dt, nin, nraw, _, _ = oracle_tasks(sch, keys, args.partitioner, rows, haddrs, sizes, threads, ddir)
            times.append(dt)
            nbytes = nin + nraw
    finally:
        remove_dir(ddir)
    total = sum(times)
    value = nbytes * args.steps / total / 1e9
    sample = (f"the first {n_rows} rows ({len(rows)} batches) of the workload per step, as {threads} map "
              f"tasks over contiguous ranges, each split then Stop writing its data file to tmpfs")
    metric, workload = metric_and_workload(args.partitioner)
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded torch RNG, same distributions)",
        "config": {"workload": workload, "sample": sample},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": sample,
                         "reference_over_port": REFERENCE_OVER_PORT,
                         "reference_estimate": value * REFERENCE_OVER_PORT},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
# Mixed-task forms.  Batches of three schemas (workload c1's, the wide fact table's, and
# 6 int32 + 2 utf8 hashed on the first int32), rows log-uniform 1k-64k, partitions 64 / 200 / 1024.
# A batch of r rows is the first r rows of one 65536-row batch per schema (slices of its
# buffers), so no time goes into generating gigabytes of input.
def _mixed_pool(seed: int):
    from gazelle_plugin_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    return [W.c4_batch(rng, s, 65536) for s in range(3)]


def _prefix_batch(batch, schema, r: int):
    from gazelle_plugin_gb300 import workloads as W
    bufs, i = [], 0
    for f in schema:
        if f.type == "null":
            bufs += [batch.buffers[i], batch.buffers[i + 1]]
            i += 2
            continue
        v = batch.buffers[i]
        bufs.append(v[: (r + 7) // 8] if v.nbytes else v)
        i += 1
        if f.is_binary:
            off = batch.buffers[i].view(np.int32)
            bufs.append(off[: r + 1].view(np.uint8))
            bufs.append(batch.buffers[i + 1][: int(off[r])])
            i += 2
        else:
            nb = (r + 7) // 8 if f.type == "bool" else r * W.BYTE_WIDTH[f.type]
            bufs.append(batch.buffers[i][:nb])
            i += 1
    return W.Batch(r, bufs)


def run_batched(seed: int = 3, n_batches: int = 512, window: int = 128, tune_batches: int = 64):
    """Config 4: 512 uneven batches, each task = (schema, partitions).  plain = the drop-in as it
    ships: one split call per batch with the default options (deferred passes, no wait per
    call); batched = the stream cut into windows of `window` batches, all tasks' batches of a
    window handed over in one splitGroup call (every task's host reads in flight together),
    each task's batches fused into device passes
    whose size (and segment length) the autotuner chose for the task's schema from its first
    `tune_batches` batches (outside the timed region), and one syncGroup at the end (every
    task's last pass queued before any task is waited for; plain: one sync per task).  Both run
    until every task's device work is done; the tasks' passes overlap on the GPU in both."""
    from gazelle_plugin_gb300 import shuffle as S
    from gazelle_plugin_gb300 import workloads as W
    pool = _mixed_pool(seed)
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    calls = []
    for _ in range(n_batches):
        si = int(rng.integers(0, 3))
        P = int(rng.choice(W.C4_PARTITIONS))
        r = int(W.c4_rows(rng))
        calls.append((si, P, _prefix_batch(pool[si], W.C4_SCHEMAS[si][0], r)))
    in_bytes = sum(b.nbytes for _, _, b in calls)
    bufs = [b.addrs_sizes() for _, _, b in calls]
    tuned = {}
    for key in sorted({c[:2] for c in calls}):
        si, P = key
        schema, keys = W.C4_SCHEMAS[si]
        sample = [b for c_si, c_P, b in calls if (c_si, c_P) == key][:tune_batches]
        t = S.autotune(schema, P, keys, sample, writeSchema=False)
        tuned[f"schema{si}_P{P}"] = {"flush_bytes": t["flush_bytes"], "seg_tiles": t["seg_tiles"],
                                     "sample_gbs": round(t["best_gbs"], 2),
                                     "sample_gbs_default": round(t["default_gbs"], 2)}

    # each window's arguments, per task: (task, row counts, buffer addresses, buffer sizes), built
    # before the timed region as the plain arm's per-batch arguments are
    windows = []
    for w0 in range(0, len(calls), window):
        groups = {}
        for i in range(w0, min(w0 + window, len(calls))):
            groups.setdefault(calls[i][:2], []).append(i)
        windows.append([(k, [calls[i][2].num_rows for i in g], np.stack([bufs[i][0] for i in g]),
                         np.stack([bufs[i][1] for i in g])) for k, g in groups.items()])

    def one(plain: bool):
        w = S.ShuffleSplitterJniWrapper()
        hs = {}
        for si, P, _ in calls:
            if (si, P) not in hs:
                schema, keys = W.C4_SCHEMAS[si]
                hs[(si, P)] = w.make(S.NativePartitioning("hash", P, None, keys, list(schema)),
                                     writeSchema=False, dataFile="/dev/null",
                                     **({} if plain else dict(flush_bytes=0, seg_tiles=0)))
        t0 = time.perf_counter()
        if plain:
            for (si, P, b), (a, z) in zip(calls, bufs):
                w.split(hs[(si, P)], b.num_rows, a, z)
        else:
            for win in windows:
                w.splitGroup([hs[k] for k, _, _, _ in win], [r for _, r, _, _ in win],
                             [a for _, _, a, _ in win], [z for _, _, _, z in win])
        if plain:
            for h in hs.values():
                w.sync(h)
        else:  # every task's last pass queued before any is waited for
            w.syncGroup(list(hs.values()))
        dt = time.perf_counter() - t0
        out = 0
        for (si, P), h in hs.items():
            out += int(w.stop(h, P).rawPartitionLengths.sum())
            w.close(h)
        return dt, out

    one(False)  # warm-up (allocations, pinned pools)
    # each arm 3 times, alternating; the median of each (a timed region is ~10-25 ms)
    runs_p, runs_b = [], []
    for _ in range(3):
        dt_p, out = one(True)
        runs_p.append(dt_p)
        runs_b.append(one(False)[0])
    dt_p, dt_b = float(np.median(runs_p)), float(np.median(runs_b))
    alg = in_bytes + out
    return {"workload": f"{n_batches} batches, rows log-uniform 1k-64k, 3 schemas x P in {{64,200,1024}}",
            "window_batches": window, "autotuned": tuned, "input_bytes": in_bytes, "partition_bytes": out,
            "plain_gbs": alg / dt_p / 1e9, "batched_gbs": alg / dt_b / 1e9, "speedup": dt_p / dt_b,
            "runs": "median of 3 alternating runs per arm",
            "plain_gbs_runs": [round(alg / t / 1e9, 1) for t in runs_p],
            "batched_gbs_runs": [round(alg / t / 1e9, 1) for t in runs_b]}


def run_fanout(distinct: int = 256, reps: int = 12, rows: int = 32768):
    """Config 3 (skew and fan-out): Zipf(1.1) int64 key over 1e7 values, 2x int64 + float64 +
    utf8 0-64 payload, 0% and 20% nulls, P in {16, 200, 2000, 8000}; ~100M rows = `distinct`
    seeded 32768-row batches resident in HBM, split `reps` times over.  Per (nulls, P): one
    warm-up split (stopped, for the partition bytes), then one timed split through
    gz_split_split_batches until its device work is done."""
    import torch
    from gazelle_plugin_gb300 import shuffle as S
    from gazelle_plugin_gb300 import workloads as W
    out = []
    w = S.ShuffleSplitterJniWrapper()
    for nullf in (0.0, 0.2):
        batches = W.c3_batches(2, distinct, rows, nullf, 0.0)
        dev = [[torch.from_numpy(x.view(np.uint8).copy()).cuda() if x.nbytes else None for x in b.buffers]
               for b in batches]
        a1 = np.array([[t.data_ptr() if t is not None else 0 for t in ts] for ts in dev], np.int64)
        z1 = np.array([[x.nbytes for x in b.buffers] for b in batches], np.int64)
        addrs, sizes = np.tile(a1, (reps, 1)), np.tile(z1, (reps, 1))
        nrows = np.full(distinct * reps, rows, np.int32)
        in_bytes = int(sizes.sum())
        for P in (16, 200, 2000, 8000):
            part = S.NativePartitioning("hash", P, None, W.C3_KEYS, list(W.C3_SCHEMA))
            opts = dict(writeSchema=False, dataFile="/dev/null", input_kind=S.GZ_INPUT_DEVICE_RETAINED,
                        flush_bytes=1 << 30)
            h = w.make(part, **opts)
            w.splitBatches(h, nrows, addrs, sizes)
            part_bytes = int(w.stop(h, P).rawPartitionLengths.sum())
            w.close(h)
            h = w.make(part, **opts)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w.splitBatches(h, nrows, addrs, sizes)
            w.sync(h)
            dt = time.perf_counter() - t0
            w.close(h)
            out.append({"nulls": nullf, "P": P, "gbs": round((in_bytes + part_bytes) / dt / 1e9, 1),
                        "ms": round(dt * 1e3, 2)})
        del dev
    return {"workload": (f"Zipf(1.1) int64 key over 1e7 values + 2x int64 + float64 + utf8 0-64, "
                         f"{distinct * reps * rows} rows ({distinct} distinct 32768-row batches x {reps}), "
                         f"resident in HBM"), "splits": out}


def _served_stream(seed: int, n_tasks: int, rate: float, gb_per_task: float):
    """Config 5 call stream: Poisson arrivals (`rate` Split calls/s in total), each to a random
    task still below its input quota; returns (task specs, [(t, task, si, rows)])."""
    from gazelle_plugin_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = [(int(rng.integers(0, 3)), int(rng.choice(W.C4_PARTITIONS))) for _ in range(n_tasks)]
    pool = _mixed_pool(seed)
    # bytes of an r-row prefix, by schema, from the pool's cumulative sizes
    per_row = [b.nbytes / b.num_rows for b in pool]
    quota = gb_per_task * 1e9
    got = [0.0] * n_tasks
    live = list(range(n_tasks))
    t, calls = 0.0, []
    while live:
        t += rng.exponential(1.0 / rate)
        k = live[int(rng.integers(0, len(live)))]
        r = int(W.c4_rows(rng))
        calls.append((t, k, specs[k][0], r))
        got[k] += r * per_row[specs[k][0]]
        if got[k] >= quota:
            live.remove(k)
    return specs, calls, pool


def run_served(seed: int = 4, n_tasks: int = 32, rate: float = 4000.0, gb_per_task: float = 2.0,
               slots: int = 8, budget: int = 40 << 30, threshold: int = 256 << 20):
    """Config 5: the call stream through the serving loop, and the same calls made one at a time
    by the plain path (each Split its own device pass, waited for, in arrival order).  Each is run
    paced at the arrival times (latency at the offered load) and unpaced (capacity)."""
    import queue
    from gazelle_plugin_gb300 import shuffle as S
    from gazelle_plugin_gb300 import workloads as W
    specs, calls, pool = _served_stream(seed, n_tasks, rate, gb_per_task)
    batches = {}

    def batch(si, r):
        key = (si, r)
        if key not in batches:
            batches[key] = _prefix_batch(pool[si], W.C4_SCHEMAS[si][0], r)
        return batches[key]

    in_bytes = sum(batch(si, r).nbytes for _, _, si, r in calls)
    last = {}
    for i, (_, k, _, _) in enumerate(calls):
        last[k] = i
    opts = dict(writeSchema=False, dataFile="/dev/null", device_budget=threshold, flush_bytes=64 << 20)
    # pinned host memory for the partition data spilled past the thresholds, taken up front as a
    # server would at start (not timed)
    S.pinned_reserve(max(0, int(1.1 * in_bytes) - n_tasks * threshold))
    w = S.ShuffleSplitterJniWrapper()

    def served(paced: bool):
        """Submitter at the arrival times (or as fast as possible), a waiter collecting latencies."""
        srv = S.ServeLoop(slots=slots, hbmBudget=budget)
        tasks = [srv.open(W.C4_SCHEMAS[si][0], P, W.C4_SCHEMAS[si][1], **opts) for si, P in specs]
        tickets = queue.Queue()
        lat = []

        def waiter():
            while True:
                tk = tickets.get()
                if tk is None:
                    return
                lat.append(srv.wait(tk))

        th = threading.Thread(target=waiter)
        th.start()
        syncs = []
        t0 = time.perf_counter()
        for i, (t, k, si, r) in enumerate(calls):
            if paced:
                d = t0 + t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            b = batch(si, r)
            a, z = b.addrs_sizes()
            tickets.put(srv.split(tasks[k], r, a, z))
            if last[k] == i:
                syncs.append(srv.sync(tasks[k]))  # the task's device work, after its last call
        tickets.put(None)
        th.join()
        for tk in syncs:
            srv.wait(tk)
        dt = time.perf_counter() - t0
        out = 0
        for k, h in enumerate(tasks):
            srv.wait(srv.stop(h))
            out += int(w.stop(h, specs[k][1]).rawPartitionLengths.sum())
            w.close(h)
        srv.shutdown()
        return lat, dt, out

    def plain(paced: bool):
        """The drop-in as an executor calls it: each task on its own thread (a task slot) makes
        its split calls itself, at their arrival times; a call's latency ends when split returns
        (its inputs read, its rows queued for the device), the same point as a served call's.
        Each thread then waits for its task's device work, as the served form's syncs do."""
        hs = [w.make(S.NativePartitioning("hash", P, None, W.C4_SCHEMAS[si][1], list(W.C4_SCHEMAS[si][0])),
                     **opts) for si, P in specs]
        per_task = [[] for _ in specs]
        for c in calls:
            per_task[c[1]].append(c)
        lats = [[] for _ in specs]
        start = threading.Barrier(len(specs) + 1)
        t0 = [0.0]

        def task(k):
            start.wait()
            for t, _, si, r in per_task[k]:
                if paced:
                    d = t0[0] + t - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                arrive = t0[0] + t if paced else time.perf_counter()
                b = batch(si, r)
                a, z = b.addrs_sizes()
                w.split(hs[k], r, a, z)
                lats[k].append((time.perf_counter() - arrive) * 1e9)
            w.sync(hs[k])

        ths = [threading.Thread(target=task, args=(k,)) for k in range(len(specs))]
        for th in ths:
            th.start()
        t0[0] = time.perf_counter()
        start.wait()
        for th in ths:
            th.join()
        dt = time.perf_counter() - t0[0]
        out = 0
        for k, h in enumerate(hs):
            out += int(w.stop(h, specs[k][1]).rawPartitionLengths.sum())
            w.close(h)
        return [x for l in lats for x in l], dt, out

    def pct(v, q):
        return float(np.percentile(np.asarray(v, np.float64), q)) / 1e6

    res = {}
    for name, fn in (("served", served), ("plain", plain)):
        lat, dt, out = fn(True)
        _, dt_cap, _ = fn(False)
        alg = in_bytes + out
        res[name] = {"p50_ms": pct(lat, 50), "p90_ms": pct(lat, 90), "p99_ms": pct(lat, 99),
                     "max_ms": max(lat) / 1e6, "gbs_at_offered_load": alg / dt / 1e9,
                     "capacity_gbs": alg / dt_cap / 1e9, "capacity_splits_per_s": len(calls) / dt_cap}
        res["partition_bytes"] = out
    return {"workload": (f"{n_tasks} tasks, Poisson {rate:.0f} Split/s, rows log-uniform 1k-64k, "
                         f"3 schemas x P in {{64,200,1024}}, stop after {gb_per_task:g} GB input per task, "
                         f"spill threshold {threshold >> 20} MiB, HBM budget {budget >> 30} GiB, "
                         f"{slots} serving workers"),
            "latency": ("per Split call, its arrival time to the point where its inputs are read and its "
                        "rows queued for the device (served: the ticket completes; plain: split returns)"),
            "plain_path": "each task on its own thread calling split itself (the drop-in as an executor calls it)",
            "capacity": "the same calls submitted without pacing",
            "calls": len(calls), "input_bytes": in_bytes, "partition_bytes": res.pop("partition_bytes"),
            "served": res["served"], "plain": res["plain"],
            "capacity_ratio": res["served"]["capacity_gbs"] / res["plain"]["capacity_gbs"]}


# ---------------------------------------------------------------------------------------
def run_gpu(args):
    import torch
    from gazelle_plugin_gb300 import shuffle as S
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w = S.ShuffleSplitterJniWrapper()
    sch, keys, rows, addrs, sizes, keep = workload_inputs(args.rows, 1 + rank, args.partitioner)
    part = S.NativePartitioning(args.partitioner, PARTITIONS, None, keys, sch)
    in_bytes = int(sizes.sum())

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # -- value: inputs resident in HBM ---------------------------------------------------
    dev_opts = dict(writeSchema=False, input_kind=S.GZ_INPUT_DEVICE_RETAINED,
                    flush_bytes=args.flush_mb << 20, device_budget=200 << 30)

    def one_step(opts, a, s, stats=None):
        h = w.make(part, **opts)
        w.splitBatches(h, rows, a, s)
        w.sync(h)
        if stats is not None:
            stats.append(w.kernelTimes(h) + w.stats(h))
        w.close(h)

    # one full run with Stop for the partition bytes (raw lengths) and the Stop cost
    h = w.make(part, dataFile="/dev/null", **dev_opts)
    w.splitBatches(h, rows, addrs, sizes)
    t0 = time.perf_counter()
    res = w.stop(h, PARTITIONS)
    stop_s = time.perf_counter() - t0
    w.close(h)
    out_bytes = int(res.rawPartitionLengths.sum())
    alg_bytes = in_bytes + out_bytes
    # Stop again with the pinned pool warm, writing a real data file to tmpfs
    sdir = scratch_dir()
    try:
        h = w.make(part, dataFile=os.path.join(sdir, "stop.data"), **dev_opts)
        w.splitBatches(h, rows, addrs, sizes)
        w.sync(h)
        t0 = time.perf_counter()
        w.stop(h, PARTITIONS)
        stop_warm_s = time.perf_counter() - t0
        w.close(h)
    finally:
        remove_dir(sdir)

    for _ in range(args.warmup):
        one_step(dev_opts, addrs, sizes)
    barrier()
    clocks = ClockSampler()
    clocks.start()
    stats = []
    times = []
    for _ in range(args.steps):
        barrier()
        t0 = time.perf_counter()
        one_step(dev_opts, addrs, sizes, stats)
        barrier()
        times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    t_local = sum(times)
    t_max = reduce_over_ranks(t_local, "max")
    alg_all = reduce_over_ranks(float(alg_bytes), "sum")  # every rank's own partition bytes
    in_all = reduce_over_ranks(float(in_bytes), "sum")
    value = alg_all * args.steps / t_max / 1e9
    ms_per_step = t_max / args.steps * 1e3
    # kernel timings (CUDA events on the splitter's stream), per step
    k_hash = statistics.mean(s[0] for s in stats)
    k_plan = statistics.mean(s[1] for s in stats)
    k_scat = statistics.mean(s[2] for s in stats)
    flushes = statistics.mean(s[4] for s in stats)
    peak, peak_kind = measured_peak_gbs()
    scat_gbs = alg_bytes / (k_scat / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_scatter", "achieved": scat_gbs, "peak": peak,
                "unit": "GB/s", "frac": scat_gbs / peak, "peak_source": peak_kind,
                "traffic": traffic_per_launch(alg_bytes / max(flushes, 1), args.traffic_per_launch),
                "traffic_source": ("--traffic-per-launch" if args.traffic_per_launch else
                                   "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_scatter "
                                   "launch of this workload (its ratio to that launch's algorithmic "
                                   "bytes, from the committed capture summary), scaled to this run's "
                                   "average launch"),
                "overlap": ("k_scatter of pass i runs beside k_hash_count and the plan kernels of "
                            "pass i + 1 (their own streams; k_hash_count at the lowest priority); "
                            "its duration is the live one"),
                "launches_per_step": flushes,
                "algorithmic_bytes_per_launch": alg_bytes / max(flushes, 1),
                "avg_launch_ms": k_scat / max(flushes, 1)}

    # -- e2e: the drop-in as an executor's map tasks call it --------------------------------
    e2e = None
    cpu = None
    out_check = None
    tasks = args.tasks or min(os.cpu_count() or 1, 16)
    if not args.no_e2e:
        link = link_bandwidth()
        haddrs, host = pageable_copy(addrs, sizes, keep)
        ddir = scratch_dir()
        e2e_opts = dict(writeSchema=False, input_kind=S.GZ_INPUT_HOST,
                        flush_bytes=args.e2e_flush_mb << 20, host_read=args.host_read)
        try:
            for _ in range(max(1, args.warmup - 1)):
                S.run_map_tasks(part, rows, haddrs, sizes, tasks, ddir, **e2e_opts)
            runs = []
            for _ in range(args.steps):
                barrier()
                runs.append(S.run_map_tasks(part, rows, haddrs, sizes, tasks, ddir, **e2e_opts))
                barrier()
            gpu_files = digests(task_files(ddir, tasks))
            gpu_lengths = runs[-1]["partition_lengths"]
            read = None if args.no_read else read_back(sch, task_files(ddir, tasks), gpu_lengths, tasks=tasks)
            remove_dir(ddir)
            ddir = scratch_dir()
            one = S.run_map_tasks(part, rows, haddrs, sizes, 1, ddir, **e2e_opts)
            remove_dir(ddir)
            ddir = scratch_dir()
            lz4 = None
            if not args.no_lz4:
                z_opts = dict(e2e_opts, codec="lz4")
                S.run_map_tasks(part, rows, haddrs, sizes, tasks, ddir, **z_opts)  # warm-up
                zr = S.run_map_tasks(part, rows, haddrs, sizes, tasks, ddir, **z_opts)
                z_alg = zr["input_bytes"] + zr["raw_partition_bytes"]
                lz4 = {"value": z_alg / zr["wall_s"] / 1e9, "unit": "GB/s", "tasks": tasks,
                       "wall_s": zr["wall_s"], "split_s_max": zr["split_s_max"], "stop_s_max": zr["stop_s_max"],
                       "bytes_written": zr["bytes_written"],
                       "compression_ratio": zr["raw_partition_bytes"] / max(zr["bytes_written"], 1),
                       "what": ("the e2e run with LZ4_FRAME: record batches above 256 rows compressed by the "
                                "device at Stop; metric bytes as for e2e (uncompressed sizes)")}
                remove_dir(ddir)
                ddir = scratch_dir()
            e_t = reduce_over_ranks(sum(r["wall_s"] for r in runs), "max")
            e_alg = runs[-1]["input_bytes"] + runs[-1]["raw_partition_bytes"]
            e2e = {"value": reduce_over_ranks(float(e_alg), "sum") * args.steps / e_t / 1e9, "unit": "GB/s",
                   "h2d_bytes_per_step": int(reduce_over_ranks(float(runs[-1]["input_bytes"]), "sum")),
                   "d2h_bytes_per_step": int(reduce_over_ranks(float(runs[-1]["raw_partition_bytes"]), "sum")),
                   "ms_per_step": e_t / args.steps * 1e3,
                   "path": (f"{tasks} map tasks at once, each make / gz_split_split per 4096-row batch on "
                            f"pageable host buffers / gz_split_stop writing its data file to "
                            f"{os.path.dirname(ddir)} / close (native loop, libgztask.so)"),
                   "tasks": tasks, "host_read": args.host_read, "flush_mb": args.e2e_flush_mb,
                   "split_s_max": statistics.mean(r["split_s_max"] for r in runs),
                   "stop_s_max": statistics.mean(r["stop_s_max"] for r in runs),
                   "bytes_written_per_step": runs[-1]["bytes_written"],
                   "lz4": lz4,
                   "read": read,
                   "one_task": {"value": (one["input_bytes"] + one["raw_partition_bytes"]) / one["wall_s"] / 1e9,
                                "unit": "GB/s", "wall_s": one["wall_s"], "split_s": one["split_s_max"],
                                "stop_s": one["stop_s_max"]},
                   "link": link}
            # -- CPU baseline on the whole workload, and the output check ------------------------
            if rank == 0 and world == 1 and not args.no_cpu:
                dt, nin, nraw, cpu_lengths, cpu_files = oracle_tasks(sch, keys, args.partitioner, rows, haddrs,
                                                                     sizes, tasks, ddir, digest=True)
                cpu = {"value": (nin + nraw) / dt / 1e9, "unit": "GB/s", "cores": tasks, "kind": "port",
                       "sample": (f"the whole workload ({args.rows} rows) as {tasks} map tasks over the same "
                                  f"batch ranges, split then Stop writing each task's data file"),
                       "seconds": dt, "reference_over_port": REFERENCE_OVER_PORT,
                       "reference_estimate": (nin + nraw) / dt / 1e9 * REFERENCE_OVER_PORT}
                same_files = [g == c for g, c in zip(gpu_files, cpu_files)]
                same_lengths = all(np.array_equal(g, c) for g, c in zip(gpu_lengths, cpu_lengths))
                out_check = {"tasks": tasks, "data_files_identical": all(same_files),
                             "partition_lengths_identical": bool(same_lengths),
                             "files_differing": [t for t, ok in enumerate(same_files) if not ok],
                             "bytes_compared": int(sum(n for _, n in gpu_files)),
                             "how": "64-bit checksum + size of every task's data file, GPU e2e run vs oracle"}
        finally:
            remove_dir(ddir)
        del host

    if rank == 0:
        metric, workload = metric_and_workload(args.partitioner)
        line = {
            "metric": metric, "value": value, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded torch RNG on the device, workload distributions)",
            "config": {"workload": workload, "rows": int(args.rows), "batch_rows": BATCH_ROWS,
                       "num_partitions": PARTITIONS, "input_bytes": in_bytes,
                       "partition_bytes": out_bytes,
                       "l2": "inputs (36 GB) larger than L2; no flush needed",
                       "flush_mb": args.flush_mb},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "output_check": out_check,
            "clocks": clk,
            # per device pass: k_hash_count, k_plan_prep, k_plan_rows, k_plan_bytes (utf8
            # columns present), k_plan_scan, k_scatter
            "gpu_launches": int(round(6 * flushes * args.steps)),
            "kernels_ms_per_step": {"k_hash_count": k_hash, "k_plan": k_plan, "k_scatter": k_scat},
            "rows_per_s": args.rows * args.steps * world / t_max,
            "input_gbs": in_all * args.steps / t_max / 1e9,
            "stop_s": stop_s,
            "stop_warm_s": stop_warm_s,
        }
        if not args.no_forms:
            line["batched"] = run_batched()
            line["served"] = run_served(gb_per_task=args.served_gb_per_task)
            line["fanout"] = run_fanout()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--rows", type=int, default=200_000_000)
    ap.add_argument("--flush-mb", type=int, default=1024)
    ap.add_argument("--ref-rows", type=int, default=25_000_000,
                    help="rows of the workload the reference arm splits per step")
    ap.add_argument("--tasks", type=int, default=0, help="map tasks of the e2e run (0: host cores, at most 16)")
    ap.add_argument("--e2e-flush-mb", type=int, default=256)
    ap.add_argument("--host-read", type=int, default=0, help="GzHostRead of the e2e run (0 auto, 1 CPU copy)")
    ap.add_argument("--traffic-per-launch", type=float, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-read", action="store_true", help="skip the reduce-side read line")
    ap.add_argument("--no-lz4", action="store_true", help="skip the LZ4_FRAME e2e line")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and served forms")
    ap.add_argument("--served-gb-per-task", type=float, default=2.0)
    ap.add_argument("--partitioner", default="hash", choices=["hash", "rr", "range"],
                    help="Splitter::Make short name; the headline is hash")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
