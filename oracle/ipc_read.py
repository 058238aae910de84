"""ORACLE - test infrastructure only.

A plain-Python restatement of the reduce-side read of the shuffle: Arrow IPC streams (the
encapsulated message format the reference's partition writers produce, splitter.cc:84-172, and
Arrow Java reads back on the reduce side, ArrowColumnarBatchSerializer.scala:110-240) parsed
message by message, and the record batches of all streams of a partition concatenated into one
set of columns, as numpy arrays.  Pinned against pyarrow's IPC reader and concat in the CPU
tests; the GPU tests check the CUDA reader (gz_reader_*) against it.

Only tests/ use this file.
"""
from __future__ import annotations

import struct
from typing import List, Optional, Sequence, Tuple

import numpy as np

# Arrow Message.fbs: MessageHeader union values
HEADER_SCHEMA, HEADER_RECORD_BATCH = 1, 3
BYTE_WIDTH = {"int8": 1, "uint8": 1, "int16": 2, "uint16": 2, "float16": 2, "int32": 4, "uint32": 4,
              "float32": 4, "date32": 4, "time32": 4, "int64": 8, "uint64": 8, "float64": 8,
              "date64": 8, "time64": 8, "timestamp": 8, "decimal128": 16}


class _Flat:
    """Flatbuffer tables: field `i` of the table at `t` through its vtable."""

    def __init__(self, b: bytes):
        self.b = b

    def u32(self, p):
        return struct.unpack_from("<I", self.b, p)[0]

    def field(self, t, i):
        vt = t - struct.unpack_from("<i", self.b, t)[0]
        vsize = struct.unpack_from("<H", self.b, vt)[0]
        if 4 + 2 * i >= vsize:
            return None
        off = struct.unpack_from("<H", self.b, vt + 4 + 2 * i)[0]
        return t + off if off else None

    def scalar(self, t, i, fmt, default=0):
        f = self.field(t, i)
        return struct.unpack_from("<" + fmt, self.b, f)[0] if f is not None else default

    def table(self, t, i):
        f = self.field(t, i)
        return None if f is None else f + self.u32(f)


def parse_stream(data: bytes, schema) -> List[Tuple[int, list]]:
    """Record batches of one stream: [(rows, [per field (null_count, [buffer bytes...])])]."""
    out = []
    pos = 0
    n = len(data)
    while pos < n:
        first = struct.unpack_from("<I", data, pos)[0]
        if first == 0xFFFFFFFF:
            meta_len = struct.unpack_from("<i", data, pos + 4)[0]
            meta_pos = pos + 8
        else:
            meta_len, meta_pos = first, pos + 4
        if meta_len == 0:
            break
        fb = _Flat(data[meta_pos:meta_pos + meta_len])
        msg = fb.u32(0)
        htype = fb.scalar(msg, 1, "B")
        body_len = fb.scalar(msg, 3, "q")
        body = meta_pos + meta_len
        if htype == HEADER_RECORD_BATCH:
            rb = fb.table(msg, 2)
            compressed = fb.table(rb, 3) is not None  # BodyCompression {LZ4_FRAME, BUFFER}
            rows = fb.scalar(rb, 0, "q")
            nodes, bufs = fb.table(rb, 1), fb.table(rb, 2)
            nn, nb = fb.u32(nodes), fb.u32(bufs)
            node_list = [struct.unpack_from("<qq", fb.b, nodes + 4 + 16 * i) for i in range(nn)]
            buf_list = [struct.unpack_from("<qq", fb.b, bufs + 4 + 16 * i) for i in range(nb)]
            cols, bi, ni = [], 0, 0
            for f in schema:
                length, nulls = node_list[ni]
                ni += 1
                assert length == rows
                child_nulls = None
                if f.is_list:  # the element node follows the list's
                    child_nulls = node_list[ni][1]
                    ni += 1
                k = 0 if f.type == "null" else f.buffer_count
                bufs = [data[body + o: body + o + l] for o, l in buf_list[bi:bi + k]]
                if compressed:
                    bufs = [_decompress(b) for b in bufs]
                cols.append((nulls, bufs) if child_nulls is None else (nulls, bufs, child_nulls))
                bi += k
            out.append((rows, cols))
        elif htype != HEADER_SCHEMA:
            raise ValueError(f"message type {htype}")
        pos = body + ((body_len + 7) & ~7)
    return out


def parse_stream_raw(data: bytes) -> List[Tuple[int, list, list]]:
    """Record batches of one stream without a schema: [(rows, [(length, null_count) per node],
    [buffer bytes, decompressed])]."""
    out = []
    pos, n = 0, len(data)
    while pos < n:
        first = struct.unpack_from("<I", data, pos)[0]
        if first == 0xFFFFFFFF:
            meta_len, meta_pos = struct.unpack_from("<i", data, pos + 4)[0], pos + 8
        else:
            meta_len, meta_pos = first, pos + 4
        if meta_len == 0:
            break
        fb = _Flat(data[meta_pos:meta_pos + meta_len])
        msg = fb.u32(0)
        body_len = fb.scalar(msg, 3, "q")
        body = meta_pos + meta_len
        if fb.scalar(msg, 1, "B") == HEADER_RECORD_BATCH:
            rb = fb.table(msg, 2)
            compressed = fb.table(rb, 3) is not None
            nodes, bufs = fb.table(rb, 1), fb.table(rb, 2)
            node_list = [struct.unpack_from("<qq", fb.b, nodes + 4 + 16 * i) for i in range(fb.u32(nodes))]
            raw = [data[body + o: body + o + l]
                   for o, l in (struct.unpack_from("<qq", fb.b, bufs + 4 + 16 * i) for i in range(fb.u32(bufs)))]
            out.append((fb.scalar(rb, 0, "q"), node_list, [_decompress(b) for b in raw] if compressed else raw))
        pos = body + ((body_len + 7) & ~7)
    return out


def _decompress(b: bytes) -> bytes:
    """A compressed body buffer: int64 uncompressed length, then one LZ4 frame (-1: raw bytes)."""
    if not b:
        return b
    n = struct.unpack_from("<q", b, 0)[0]
    if n == -1:
        return b[8:]
    from oracle import oracle as O
    return O.lz4f_decompress(b[8:], n)


def batches_compressed(data: bytes) -> List[bool]:
    """Whether each record batch of a stream carries body compression."""
    out, pos = [], 0
    while pos < len(data):
        first = struct.unpack_from("<I", data, pos)[0]
        meta_len, meta_pos = (struct.unpack_from("<i", data, pos + 4)[0], pos + 8) if first == 0xFFFFFFFF \
            else (first, pos + 4)
        if meta_len == 0:
            break
        fb = _Flat(data[meta_pos:meta_pos + meta_len])
        msg = fb.u32(0)
        if fb.scalar(msg, 1, "B") == HEADER_RECORD_BATCH:
            out.append(fb.table(fb.table(msg, 2), 3) is not None)
        pos = meta_pos + meta_len + ((fb.scalar(msg, 3, "q") + 7) & ~7)
    return out


def _bits(buf: bytes, n: int) -> np.ndarray:
    return np.unpackbits(np.frombuffer(buf, np.uint8), bitorder="little")[:n].astype(bool)


def read_partition(schema, streams: Sequence[bytes]):
    """Concatenation of the record batches of `streams`, in order: (rows, per field (validity
    bits as a bool array or None when the column has no nulls, offsets (int32, int64 for the
    large types) or None, values as bytes; bool values as a bool array))."""
    batches = [b for s in streams for b in parse_stream(s, schema)]
    rows = sum(r for r, _ in batches)
    cols = []
    for fi, f in enumerate(schema):
        if f.type == "null":
            cols.append((None, None, b""))
            continue
        nulls = sum(c[fi][0] for _, c in batches)
        valid = None
        if nulls:
            valid = np.concatenate([_bits(c[fi][1][0], r) if c[fi][0] else np.ones(r, bool)
                                    for r, c in batches]) if batches else np.zeros(0, bool)
        if f.type == "bool":
            vals = np.concatenate([_bits(c[fi][1][1], r) for r, c in batches]) if batches else np.zeros(0, bool)
            cols.append((valid, None, vals))
        elif f.is_list:  # (validity, offsets, (element validity or None, element values))
            if f.elem == "bool":  # element values as a bool array
                offs, vals, evalid, base = [np.zeros(1, np.int32)], [], [], 0
                any_null = any(c[fi][2] for _, c in batches)
                for r, c in batches:
                    o = np.frombuffer(c[fi][1][1], np.int32)[:r + 1]
                    m = int(o[r] - o[0])
                    vals.append(_bits(c[fi][1][3], int(o[r]))[o[0]:])
                    offs.append((o[1:] - o[0] + base).astype(np.int32))
                    if any_null:
                        evalid.append(_bits(c[fi][1][2], int(o[r]))[o[0]:] if c[fi][2] else np.ones(m, bool))
                    base += m
                ev = (np.concatenate(evalid) if evalid else np.zeros(0, bool)) if any_null else None
                cols.append((valid, np.concatenate(offs), (ev, np.concatenate(vals) if vals else np.zeros(0, bool))))
                continue
            w = BYTE_WIDTH[f.elem]
            offs, vals, evalid, base = [np.zeros(1, np.int32)], [], [], 0
            any_null = any(c[fi][2] for _, c in batches)
            for r, c in batches:
                o = np.frombuffer(c[fi][1][1], np.int32)[:r + 1]
                m = int(o[r] - o[0])
                vals.append(c[fi][1][3][o[0] * w:o[r] * w])
                offs.append((o[1:] - o[0] + base).astype(np.int32))
                if any_null:
                    evalid.append(_bits(c[fi][1][2], int(o[r]))[o[0]:] if c[fi][2] else np.ones(m, bool))
                base += m
            ev = (np.concatenate(evalid) if evalid else np.zeros(0, bool)) if any_null else None
            cols.append((valid, np.concatenate(offs), (ev, b"".join(vals))))
        elif f.is_binary:
            odt = f.offset_dtype  # int32, int64 for the large types
            offs, chars, base = [np.zeros(1, odt)], [], 0
            for r, c in batches:
                o = np.frombuffer(c[fi][1][1], odt)[:r + 1]
                chars.append(c[fi][1][2][o[0]:o[r]])
                offs.append((o[1:] - o[0] + base).astype(odt))
                base += int(o[r] - o[0])
            cols.append((valid, np.concatenate(offs), b"".join(chars)))
        else:
            w = BYTE_WIDTH[f.type]
            cols.append((valid, None, b"".join(c[fi][1][1][:r * w] for r, c in batches)))
    return rows, cols


def read_partition_nodes(schema, streams: Sequence[bytes]):
    """Every field of a partition as its nodes in pre-order (a map's entries struct included),
    each concatenated over all record batches of all streams: (length, null_count, validity as a
    bool array or None when no entry is null, offsets (int32 / int64, from 0) or None, values:
    bytes, or a bool array for bool nodes).  Offsets of a list / map start at 0 in every batch
    (the writers' layout); binary characters are taken from the first to the last offset."""
    from gazelle_plugin_gb300.workloads import BYTE_WIDTH as BW, TYPE_CODES
    names = {v: k for k, v in TYPE_CODES.items()}
    trees = [[names[c & 0xff] for c in f.type_nodes()] for f in schema]

    def nbuf(t):
        return 0 if t == "null" else 1 if t == "struct" else 2 if t in ("list", "large_list", "map") else \
            3 if t in ("utf8", "binary", "large_utf8", "large_binary") else 2

    acc = [[{"len": 0, "nulls": 0, "valid": [], "offs": [], "vals": [], "base": 0} for _ in tree] for tree in trees]
    for s in streams:
        for _, nodes, bufs in parse_stream_raw(s):
            ni = bi = 0
            for fi, tree in enumerate(trees):
                for q, t in enumerate(tree):
                    length, nulls = nodes[ni]
                    ni += 1
                    own = bufs[bi:bi + nbuf(t)]
                    bi += nbuf(t)
                    a = acc[fi][q]
                    a["len"] += length
                    a["nulls"] += nulls
                    a["valid"].append(_bits(own[0], length) if nulls else np.ones(length, bool))
                    if t in ("list", "large_list", "map", "utf8", "binary", "large_utf8", "large_binary"):
                        o = np.frombuffer(own[1], np.int64 if t.startswith("large") else np.int32)[:length + 1]
                        if not len(o):
                            o = np.zeros(1, np.int32)
                        a["offs"].append(o[:-1] - o[0] + a["base"])
                        a["base"] += int(o[-1] - o[0])
                        a["last"] = a["base"]
                        if t not in ("list", "large_list", "map"):
                            a["vals"].append(own[2][int(o[0]):int(o[-1])])
                    elif t == "bool":
                        a["vals"].append(_bits(own[1], length))
                    elif t not in ("struct", "null"):
                        a["vals"].append(own[1][:length * BW[t]])
    out = []
    for fi, tree in enumerate(trees):
        nodes = []
        for q, t in enumerate(tree):
            a = acc[fi][q]
            valid = np.concatenate(a["valid"]) if a["nulls"] else None
            offs = None
            if t in ("list", "large_list", "map", "utf8", "binary", "large_utf8", "large_binary"):
                dt = np.int64 if t.startswith("large") else np.int32
                offs = np.concatenate(a["offs"] + [np.array([a["base"]])]).astype(dt)
            if t == "bool":
                vals = np.concatenate(a["vals"]) if a["vals"] else np.zeros(0, bool)
            else:
                vals = b"".join(a["vals"])
            nodes.append((a["len"], a["nulls"], valid, offs, vals))
        out.append(nodes)
    return out


def pack_bits(v: Optional[np.ndarray]) -> Optional[bytes]:
    """An LSB-first bitmap of a bool array, zero padded (None stays None)."""
    if v is None:
        return None
    return np.packbits(v.astype(np.uint8), bitorder="little").tobytes()
