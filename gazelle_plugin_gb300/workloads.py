"""Seeded synthetic record batches for the shuffle hash-split workloads.

A batch is held the way the reference's JNI boundary receives it
(native-sql-engine/cpp/src/jni/jni_common.h:308-382): one flat list of Arrow buffers in
schema order, ``[validity, (offsets), values]`` per field (a null-type field takes two
empty buffers, as the JNI's generic branch consumes them), where an empty validity buffer
means the column has no nulls.  Nothing here needs pyarrow.

Workloads (seeded numpy PCG64; nulls i.i.d. per cell; a null utf8 cell is a zero-length
slot; a null fixed-width cell keeps its generated value):

* ``c1``  - 10 x 4096 rows: k:int32 U[0,2^31) non-null (key), v1:int64 full range,
  v2:float64 N(0,1), s:utf8 len U{0..16} over [a-z]; 5% nulls in v1/v2/s; P = 8.
* ``c2``  - wide fact table, 4096-row batches: 4 int64 keys U[0,6e8), 4 float64 U[0,1e5)
  at 0.01 granularity, 2 int32 U[8000,10600), 3 utf8 single-char flags over 3-symbol
  alphabets, 3 utf8 comments len U{10..44} over [a-z ]; 2% nulls in the 12 non-key
  columns; hash keys = columns 0 and 1; P = 200.
* ``c3``  - Zipf(s=1.1) int64 key over 1e7 ranks mapped through a seeded permutation,
  payload 2 x int64 + float64 + utf8 len U{0..64}; 0% or 20% nulls in non-key columns.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence, Tuple

import numpy as np

# Type codes of the C ABI (include/gz_split.h GZ_TYPE_*).
TYPE_CODES = {
    "null": 0, "bool": 1, "int8": 2, "uint8": 3, "int16": 4, "uint16": 5,
    "float16": 6, "int32": 7, "uint32": 8, "float32": 9, "date32": 10, "time32": 11,
    "int64": 12, "uint64": 13, "float64": 14, "date64": 15, "time64": 16,
    "timestamp": 17, "decimal128": 18, "utf8": 19, "binary": 20,
    "large_utf8": 21, "large_binary": 22, "list": 23, "large_list": 24, "struct": 25,
    "map": 26,
}
BYTE_WIDTH = {
    "int8": 1, "uint8": 1, "int16": 2, "uint16": 2, "float16": 2, "int32": 4,
    "uint32": 4, "float32": 4, "date32": 4, "time32": 4, "int64": 8, "uint64": 8,
    "float64": 8, "date64": 8, "time64": 8, "timestamp": 8, "decimal128": 16,
}
NUMPY_DTYPE = {
    "int8": np.int8, "uint8": np.uint8, "int16": np.int16, "uint16": np.uint16,
    "float16": np.float16, "int32": np.int32, "uint32": np.uint32, "float32": np.float32,
    "date32": np.int32, "time32": np.int32, "int64": np.int64, "uint64": np.uint64,
    "float64": np.float64, "date64": np.int64, "time64": np.int64, "timestamp": np.int64,
}


@dataclasses.dataclass(frozen=True)
class Field:
    name: str
    type: str
    nullable: bool = True
    elem: Optional[str] = None  # list: the element type (fixed width or bool; elements nullable)
    # nested types: a list / large_list's element field, a map's key and value fields (the
    # entries struct between them is implicit), a struct's fields
    children: Tuple["Field", ...] = ()

    @property
    def code(self) -> int:
        return TYPE_CODES[self.type]

    @property
    def is_list(self) -> bool:
        """A list of fixed-width or bool elements given by `elem`."""
        return self.type == "list" and not self.children

    @property
    def is_nested(self) -> bool:
        """Any other list, large_list, struct or map (children given by `children`)."""
        return self.type in ("large_list", "struct", "map") or (self.type == "list" and bool(self.children))

    @property
    def kids(self) -> Tuple["Field", ...]:
        if self.is_list:
            return (Field("item", self.elem, True),)
        return self.children

    def type_nodes(self) -> List[int]:
        """The field's type tree in pre-order, each node's code with its child count above the
        low byte (a map's entries struct included)."""
        kids = self.kids
        if self.type == "map":
            kids = (Field("entries", "struct", False, children=self.children),)
        out = [self.code | (len(kids) << 8)]
        for k in kids:
            out += k.type_nodes()
        return out

    @property
    def buffer_count(self) -> int:
        """Entries of the field in a batch's flat buffer list: [validity, (offsets), values];
        a list: [validity, offsets, element validity, element values]; nested types depth
        first as the JNI's MakeArrayData reads them: [validity, (offsets)] then the children's
        (a map's entries struct adds its validity entry)."""
        if self.is_nested:
            own = 1 if self.type == "struct" else 2
            return own + (self.type == "map") + sum(k.buffer_count for k in self.kids)
        return 4 if self.is_list else 3 if self.is_binary else 2

    @property
    def is_binary(self) -> bool:
        return self.type in ("utf8", "binary", "large_utf8", "large_binary")

    @property
    def offset_dtype(self):
        """Offsets of a binary field: int32, int64 for the large types."""
        return np.int64 if self.type.startswith("large_") else np.int32

    @property
    def params(self):
        """(precision, scale, time unit 0 s / 1 ms / 2 us / 3 ns) of the Arrow type the field
        stands for: time32[ms], time64[us], timestamp[us], decimal128(30, 2)."""
        return {"decimal128": (30, 2, 0), "time32": (0, 0, 1), "time64": (0, 0, 2),
                "timestamp": (0, 0, 2)}.get(self.type, (0, 0, 0))


@dataclasses.dataclass
class Batch:
    num_rows: int
    buffers: List[np.ndarray]  # uint8-viewable, flat [validity, (offsets), values] list

    def addrs_sizes(self):
        addrs = np.array([b.ctypes.data if b.nbytes else 0 for b in self.buffers], np.int64)
        sizes = np.array([b.nbytes for b in self.buffers], np.int64)
        return addrs, sizes

    @property
    def nbytes(self) -> int:
        return int(sum(b.nbytes for b in self.buffers))


def pack_validity(valid: np.ndarray) -> np.ndarray:
    """Arrow LSB-first validity bitmap; an all-valid column gets an empty buffer."""
    if valid.all():
        return np.zeros(0, np.uint8)
    return np.packbits(valid.astype(np.uint8), bitorder="little")


def _strings(rng, n, lo, hi, alphabet: bytes, valid, offset_dtype=np.int32):
    lens = rng.integers(lo, hi + 1, size=n).astype(np.int32)
    if valid is not None:
        lens = np.where(valid, lens, 0).astype(np.int32)
    offsets = np.zeros(n + 1, offset_dtype)
    np.cumsum(lens, out=offsets[1:])
    alpha = np.frombuffer(alphabet, np.uint8)
    chars = alpha[rng.integers(0, len(alpha), size=int(offsets[-1]))]
    return offsets, chars.astype(np.uint8)


def _column(rng, field: Field, n: int, values: np.ndarray | None, null_frac: float,
            str_spec=None) -> List[np.ndarray]:
    valid = rng.random(n) >= null_frac if null_frac > 0 else np.ones(n, bool)
    vbuf = pack_validity(valid)
    if field.is_binary:
        lo, hi, alphabet = str_spec
        offsets, chars = _strings(rng, n, lo, hi, alphabet, valid, field.offset_dtype)
        return [vbuf, offsets.view(np.uint8), chars]
    if field.type == "bool":
        bits = values.astype(bool)
        return [vbuf, np.packbits(bits.astype(np.uint8), bitorder="little")]
    return [vbuf, np.ascontiguousarray(values.astype(NUMPY_DTYPE[field.type])).view(np.uint8)]


# --------------------------------------------------------------------------------------
# workload c1
C1_SCHEMA = [Field("k", "int32", False), Field("v1", "int64"), Field("v2", "float64"),
             Field("s", "utf8")]
C1_KEYS = [0]
C1_PARTITIONS = 8
AZ = b"abcdefghijklmnopqrstuvwxyz"
AZ_BYTES = np.frombuffer(AZ, np.uint8)


def c1_batch(rng, n: int = 4096) -> Batch:
    bufs = []
    bufs += _column(rng, C1_SCHEMA[0], n, rng.integers(0, 2**31, size=n), 0.0)
    bufs += _column(rng, C1_SCHEMA[1], n,
                    rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, size=n,
                                 dtype=np.int64, endpoint=True), 0.05)
    bufs += _column(rng, C1_SCHEMA[2], n, rng.standard_normal(n), 0.05)
    bufs += _column(rng, C1_SCHEMA[3], n, None, 0.05, (0, 16, AZ))
    return Batch(n, bufs)


def c1_batches(seed: int = 0, num_batches: int = 10, rows: int = 4096) -> List[Batch]:
    rng = np.random.Generator(np.random.PCG64(seed))
    return [c1_batch(rng, rows) for _ in range(num_batches)]


# --------------------------------------------------------------------------------------
# workload c2
C2_SCHEMA = (
    [Field(f"key{i}", "int64", False) for i in range(4)]
    + [Field(f"amt{i}", "float64") for i in range(4)]
    + [Field(f"day{i}", "int32") for i in range(2)]
    + [Field(f"flag{i}", "utf8") for i in range(3)]
    + [Field(f"comment{i}", "utf8") for i in range(3)]
)
C2_KEYS = [0, 1]
C2_PARTITIONS = 200
C2_FLAG_ALPHABETS = [b"AFN", b"OFP", b"RAN"]
AZ_SPACE = b"abcdefghijklmnopqrstuvwxyz "


def c2_batch(rng, n: int = 4096) -> Batch:
    bufs = []
    for i in range(4):
        bufs += _column(rng, C2_SCHEMA[i], n, rng.integers(0, 600_000_000, size=n), 0.0)
    for i in range(4):
        v = np.floor(rng.random(n) * 1e7) / 100.0
        bufs += _column(rng, C2_SCHEMA[4 + i], n, v, 0.02)
    for i in range(2):
        bufs += _column(rng, C2_SCHEMA[8 + i], n, rng.integers(8000, 10600, size=n), 0.02)
    for i in range(3):
        bufs += _column(rng, C2_SCHEMA[10 + i], n, None, 0.02, (1, 1, C2_FLAG_ALPHABETS[i]))
    for i in range(3):
        bufs += _column(rng, C2_SCHEMA[13 + i], n, None, 0.02, (10, 44, AZ_SPACE))
    return Batch(n, bufs)


def c2_batches(seed: int = 1, num_batches: int = 16, rows: int = 4096) -> List[Batch]:
    rng = np.random.Generator(np.random.PCG64(seed))
    return [c2_batch(rng, rows) for _ in range(num_batches)]


# --------------------------------------------------------------------------------------
# workload c3
C3_SCHEMA = [Field("key", "int64"), Field("p0", "int64"), Field("p1", "int64"),
             Field("p2", "float64"), Field("s", "utf8")]
C3_KEYS = [0]


def zipf_keys(rng, n: int, s: float = 1.1, ranks: int = 10_000_000,
              perm_seed: int = 2) -> np.ndarray:
    """Zipf(s) over `ranks` ranks, inverse-CDF sampled; rank r maps to a seeded
    pseudo-random int64 (a fixed odd multiplier permutation of the rank)."""
    # inverse CDF of the continuous approximation, clamped to [1, ranks]
    u = rng.random(n)
    hs = (ranks ** (1 - s) - 1) / (1 - s)
    r = np.floor(((u * hs) * (1 - s) + 1) ** (1 / (1 - s))).astype(np.int64)
    r = np.clip(r, 1, ranks)
    mult = np.int64(0x9E3779B97F4A7C15 & 0x7FFFFFFFFFFFFFFF) | 1
    with np.errstate(over="ignore"):
        return (r * mult + np.int64(perm_seed)).astype(np.int64)


def c3_batch(rng, n: int = 32768, null_frac: float = 0.0, key_nulls: float = 0.0) -> Batch:
    bufs = []
    bufs += _column(rng, C3_SCHEMA[0], n, zipf_keys(rng, n), key_nulls)
    bufs += _column(rng, C3_SCHEMA[1], n, rng.integers(-2**62, 2**62, size=n), null_frac)
    bufs += _column(rng, C3_SCHEMA[2], n, rng.integers(-2**62, 2**62, size=n), null_frac)
    bufs += _column(rng, C3_SCHEMA[3], n, rng.standard_normal(n), null_frac)
    bufs += _column(rng, C3_SCHEMA[4], n, None, null_frac, (0, 64, AZ))
    return Batch(n, bufs)


def c3_batches(seed: int = 2, num_batches: int = 4, rows: int = 32768, null_frac=0.0,
               key_nulls=0.0) -> List[Batch]:
    rng = np.random.Generator(np.random.PCG64(seed))
    return [c3_batch(rng, rows, null_frac, key_nulls) for _ in range(num_batches)]


# --------------------------------------------------------------------------------------
# mixed-task workloads (batched and served forms): uneven batches from three schemas
C4_SCHEMA_3 = [Field(f"i{k}", "int32") for k in range(6)] + [Field("u0", "utf8"), Field("u1", "utf8")]
C4_KEYS_3 = [0]
C4_SCHEMAS = [(C1_SCHEMA, C1_KEYS), (C2_SCHEMA, C2_KEYS), (C4_SCHEMA_3, C4_KEYS_3)]
C4_PARTITIONS = [64, 200, 1024]


def c4_schema3_batch(rng, n: int) -> Batch:
    bufs = []
    for k in range(6):
        bufs += _column(rng, C4_SCHEMA_3[k], n, rng.integers(-2**31, 2**31, size=n), 0.0 if k == 0 else 0.02)
    for k in range(2):
        bufs += _column(rng, C4_SCHEMA_3[6 + k], n, None, 0.02, (0, 32, AZ))
    return Batch(n, bufs)


def c4_batch(rng, schema_index: int, n: int) -> Batch:
    """A batch of `n` rows of mixed-task schema 0 (workload c1), 1 (c2) or 2 (6 int32 + 2 utf8)."""
    if schema_index == 0:
        return c1_batch(rng, n)
    if schema_index == 1:
        return c2_batch(rng, n)
    return c4_schema3_batch(rng, n)


def list_column(rng, field: Field, n: int, null_frac: float, elem_null_frac: float, max_len: int,
                values=None) -> List[np.ndarray]:
    """Buffers of a list column of `n` rows: lengths U{0..max_len} (0 for a null row), elements
    of field.elem drawn like a flat column's (or taken from `values`; bool elements bit-packed),
    element nulls i.i.d."""
    valid = rng.random(n) >= null_frac if null_frac > 0 else np.ones(n, bool)
    lens = np.where(valid, rng.integers(0, max_len + 1, size=n), 0).astype(np.int32)
    offsets = np.zeros(n + 1, np.int32)
    np.cumsum(lens, out=offsets[1:])
    m = int(offsets[-1])
    ef = Field("item", field.elem)
    if values is None:
        if field.elem == "decimal128":
            values = rng.integers(0, 2**63, size=2 * m, dtype=np.uint64)
        elif field.elem in ("float16", "float32", "float64"):
            values = rng.standard_normal(m) * 1e3
        elif field.elem == "bool":
            values = rng.integers(0, 2, size=m)
        else:
            w = BYTE_WIDTH[field.elem]
            hi = 2 ** (8 * w - 1) if w < 8 else 2**62
            values = rng.integers(-hi if field.elem[0] != "u" else 0, hi, size=m)
    evalid = rng.random(m) >= elem_null_frac if elem_null_frac > 0 else np.ones(m, bool)
    if field.elem == "bool":
        vals = np.packbits((np.asarray(values) % 2).astype(np.uint8), bitorder="little")
    elif field.elem == "decimal128":
        vals = np.ascontiguousarray(np.asarray(values, np.uint64)).view(np.uint8)
    else:
        vals = np.ascontiguousarray(np.asarray(values).astype(NUMPY_DTYPE[ef.type])).view(np.uint8)
    return [pack_validity(valid), offsets.view(np.uint8), pack_validity(evalid), vals]


def nested_column(rng, field: Field, n: int, null_frac: float = 0.1, max_len: int = 4,
                  top: bool = True, spans: bool = False) -> List[np.ndarray]:
    """Buffers of `n` entries of a field of any nesting, depth first (MakeArrayData order).
    Entries are null with probability null_frac (never a map key); list / map lengths
    U{0..max_len}, strings 0-7 letters.  A null list / map / string entry holds no elements,
    except with `spans` at the top level (or under top-level structs), where it keeps a
    non-empty range that the split must drop."""
    valid = rng.random(n) >= null_frac if (null_frac > 0 and field.nullable) else np.ones(n, bool)
    vbuf = pack_validity(valid)
    t = field.type

    def lengths(hi):
        lens = rng.integers(0, hi + 1, size=n)
        return lens if (spans and top) else np.where(valid, lens, 0)

    if t in ("list", "large_list", "map"):
        offs = np.zeros(n + 1, np.int64 if t == "large_list" else np.int32)
        np.cumsum(lengths(max_len), out=offs[1:])
        m = int(offs[-1])
        out = [vbuf, offs.view(np.uint8)]
        if t == "map":
            key, val = field.kids
            out.append(np.zeros(0, np.uint8))  # the entries struct: no validity
            out += nested_column(rng, key, m, 0.0, max_len, False)
            out += nested_column(rng, val, m, null_frac, max_len, False)
        else:
            out += nested_column(rng, field.kids[0], m, null_frac, max_len, False)
        return out
    if t == "struct":
        out = [vbuf]
        for k in field.kids:
            out += nested_column(rng, k, n, null_frac, max_len, top, spans)
        return out
    if field.is_binary:
        offs = np.zeros(n + 1, field.offset_dtype)
        np.cumsum(lengths(7), out=offs[1:])
        chars = AZ_BYTES[rng.integers(0, 26, size=int(offs[-1]))]
        return [vbuf, offs.view(np.uint8), chars.astype(np.uint8)]
    if t == "bool":
        return [vbuf, np.packbits(rng.integers(0, 2, size=n).astype(np.uint8), bitorder="little")]
    if t == "decimal128":
        return [vbuf, rng.integers(0, 2**63, size=2 * n, dtype=np.uint64).view(np.uint8)]
    w = BYTE_WIDTH[t]
    hi = 2 ** (8 * w - 1) if w < 8 else 2**62
    v = rng.integers(-hi if t[0] != "u" else 0, hi, size=n).astype(NUMPY_DTYPE[t])
    return [vbuf, v.view(np.uint8)]


NESTED_LEAVES = ["int8", "int16", "int32", "int64", "float32", "float64", "date32", "decimal128",
                 "timestamp", "bool", "utf8", "binary", "large_utf8"]


def random_nested_field(rng, name: str, depth: int = 0) -> Field:
    """A random nested field: list / large_list / map / struct down to depth 3 over NESTED_LEAVES
    (map keys: int32 or utf8, not nullable)."""
    kind = str(rng.choice(["list", "large_list", "map", "struct"]))

    def child(nm):
        if depth >= 2 or rng.random() < 0.45:
            return Field(nm, str(rng.choice(NESTED_LEAVES)), bool(rng.random() < 0.8))
        return random_nested_field(rng, nm, depth + 1)

    if kind == "struct":
        kids = tuple(child(f"s{i}") for i in range(int(rng.integers(1, 4))))
    elif kind == "map":
        kids = (Field("key", str(rng.choice(["int32", "utf8"])), False), child("value"))
    else:
        kids = (child("item"),)
    return Field(name, kind, bool(rng.random() < 0.8), None, kids)


def c4_rows(rng, size=None):
    """Batch rows log-uniform over [1000, 65536]."""
    return np.exp(rng.uniform(np.log(1000), np.log(65536), size=size)).astype(np.int64)


# --------------------------------------------------------------------------------------
# random schemas for property tests
RANDOM_TYPES = ["bool", "int8", "int16", "int32", "int64", "float32", "float64", "date32",
                "uint64", "decimal128", "utf8", "binary", "null", "timestamp", "float16"]
KEY_TYPES = ["bool", "int8", "int16", "int32", "int64", "float32", "float64", "date32"]


def random_schema(rng, n_fields: int) -> List[Field]:
    fields = [Field(f"c{i}", str(rng.choice(RANDOM_TYPES))) for i in range(n_fields)]
    if not any(f.type in KEY_TYPES for f in fields):
        fields[0] = Field("c0", str(rng.choice(KEY_TYPES)))
    return fields


def random_batch(rng, schema: Sequence[Field], n: int, null_frac: float) -> Batch:
    bufs = []
    for f in schema:
        if f.type == "null":
            bufs += [np.zeros(0, np.uint8), np.zeros(0, np.uint8)]
            continue
        nf = null_frac if rng.random() < 0.7 else 0.0
        if f.is_binary:
            bufs += _column(rng, f, n, None, nf, (0, int(rng.integers(0, 40)), AZ))
        elif f.type == "bool":
            bufs += _column(rng, f, n, rng.integers(0, 2, size=n), nf)
        elif f.type == "decimal128":
            v = rng.integers(0, 2**63, size=2 * n, dtype=np.uint64).view(np.uint8)
            valid = rng.random(n) >= nf if nf > 0 else np.ones(n, bool)
            bufs += [pack_validity(valid), v.copy()]
        elif f.type in ("float32", "float64", "float16"):
            bufs += _column(rng, f, n, rng.standard_normal(n) * 1e3, nf)
        else:
            w = BYTE_WIDTH[f.type]
            hi = 2 ** (8 * w - 1) if w < 8 else 2**62
            bufs += _column(rng, f, n, rng.integers(-hi if f.type[0] != "u" else 0, hi, size=n), nf)
    return Batch(n, bufs)


def with_partition_ids(schema: Sequence[Field], batches: Sequence[Batch], pids) -> tuple:
    """The range partitioner's input (FallbackRangeSplitter, splitter.cc:1486-1519): int32
    partition ids as schema field 0, in front of ``schema`` and of every batch's buffers.
    ``pids[i]`` holds batch i's ids; an id's validity is never read, so the column has none."""
    s = [Field("pid", "int32", False)] + list(schema)
    out = []
    for b, p in zip(batches, pids):
        p = np.ascontiguousarray(p, dtype=np.int32)
        assert p.shape == (b.num_rows,)
        out.append(Batch(b.num_rows, [np.zeros(0, np.uint8), p] + list(b.buffers)))
    return s, out
