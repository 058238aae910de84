// Reads the Arrow IPC Schema message the JNI layer receives (MakeSchema,
// native-sql-engine/cpp/src/jni/jni_common.h:393-406) into the splitter's field list.
// A small flatbuffer reader over the Arrow format's Message / Schema / Field tables.
#include "schema_ipc.h"

#include <string.h>

#include <algorithm>

#include "../../include/gz_split.h"
#include "flatbuf.h"

namespace gz {
namespace {

// One Field table (and its children, for nested types).  A list whose element is a fixed-width
// or bool leaf keeps the simple form (elem, no children).
bool DecodeField(FlatReader& r, int64_t ft, int depth, Field* out, std::string* err) {
  if (depth > 16) {
    *err = "nesting too deep";
    return false;
  }
  Field f;
  if (!r.String(ft, 0, &f.name)) {
    *err = "bad field name";
    return false;
  }
  f.nullable = r.Scalar<uint8_t>(ft, 1, 0) != 0;
  uint8_t tt = r.Scalar<uint8_t>(ft, 2, 0);
  int64_t tp = r.Table(ft, 3);
  if (tt == 12 || tt == 13 || tt == 17 || tt == 21) {  // List, Struct_, Map, LargeList
    int64_t ch = r.Table(ft, 5);
    uint32_t nch = 0;
    if (ch >= 0 && !r.Get(ch, &nch)) {
      *err = "bad children vector";
      return false;
    }
    for (uint32_t k = 0; k < nch; k++) {
      const int64_t ct = r.Deref(ch + 4 + 4 * (int64_t)k);
      Field c;
      if (ct < 0 || !DecodeField(r, ct, depth + 1, &c, err)) {
        if (err->empty()) *err = "bad child field";
        return false;
      }
      f.children.push_back(std::move(c));
    }
    if ((tt == 12 || tt == 21) && nch != 1) {
      *err = "list field without one element field";
      return false;
    }
    if (tt == 13 && nch == 0) {
      *err = "struct field without fields";
      return false;
    }
    if (tt == 17) {
      if (nch != 1 || f.children[0].type != GZ_TYPE_STRUCT || f.children[0].children.size() != 2) {
        *err = "map field without an entries struct of key and value";
        return false;
      }
      f.keys_sorted = tp >= 0 && r.Scalar<uint8_t>(tp, 0, 0) != 0;
    }
    for (const Field& c : f.children)
      if (c.type == GZ_TYPE_NULL) {
        *err = "null-type fields inside nested types are not implemented by the GPU splitter";
        return false;
      }
    f.type = tt == 12 ? GZ_TYPE_LIST : tt == 13 ? GZ_TYPE_STRUCT : tt == 17 ? GZ_TYPE_MAP : GZ_TYPE_LARGE_LIST;
    if (tt == 12) {
      const Field& e = f.children[0];
      if (!e.nested() && (e.type == GZ_TYPE_BOOL || (e.type != GZ_TYPE_NULL && e.type < GZ_TYPE_STRING))) {
        // the simple form
        f.elem = e.type;
        f.elem_name = e.name;
        f.elem_nullable = e.nullable;
        f.precision = e.precision;
        f.scale = e.scale;
        f.unit = e.unit;
        f.timezone = e.timezone;
        f.children.clear();
      }
    }
    *out = std::move(f);
    return true;
  }
  switch (tt) {
    case 1: f.type = GZ_TYPE_NULL; break;
    case 2: {
      int32_t bw = tp >= 0 ? r.Scalar<int32_t>(tp, 0, 0) : 0;
      bool sg = tp >= 0 && r.Scalar<uint8_t>(tp, 1, 0) != 0;
      switch (bw) {
        case 8: f.type = sg ? GZ_TYPE_INT8 : GZ_TYPE_UINT8; break;
        case 16: f.type = sg ? GZ_TYPE_INT16 : GZ_TYPE_UINT16; break;
        case 32: f.type = sg ? GZ_TYPE_INT32 : GZ_TYPE_UINT32; break;
        case 64: f.type = sg ? GZ_TYPE_INT64 : GZ_TYPE_UINT64; break;
        default: *err = "bad integer width"; return false;
      }
      break;
    }
    case 3: {
      int16_t prec = tp >= 0 ? r.Scalar<int16_t>(tp, 0, 0) : 0;
      f.type = prec == 0 ? GZ_TYPE_HALF_FLOAT : prec == 1 ? GZ_TYPE_FLOAT32 : GZ_TYPE_FLOAT64;
      break;
    }
    case 4: f.type = GZ_TYPE_BINARY; break;
    case 5: f.type = GZ_TYPE_STRING; break;
    case 19: f.type = GZ_TYPE_LARGE_BINARY; break;
    case 20: f.type = GZ_TYPE_LARGE_STRING; break;
    case 6: f.type = GZ_TYPE_BOOL; break;
    case 7: {
      int32_t bw = tp >= 0 ? r.Scalar<int32_t>(tp, 2, 128) : 128;
      if (bw != 128) {
        *err = "only decimal128 is supported";
        return false;
      }
      f.type = GZ_TYPE_DECIMAL128;
      f.precision = tp >= 0 ? r.Scalar<int32_t>(tp, 0, 0) : 0;
      f.scale = tp >= 0 ? r.Scalar<int32_t>(tp, 1, 0) : 0;
      break;
    }
    case 8: {
      int16_t unit = tp >= 0 ? r.Scalar<int16_t>(tp, 0, 1) : 1;
      f.type = unit == 0 ? GZ_TYPE_DATE32 : GZ_TYPE_DATE64;
      break;
    }
    case 9: {
      f.unit = tp >= 0 ? r.Scalar<int16_t>(tp, 0, 1) : 1;
      int32_t bw = tp >= 0 ? r.Scalar<int32_t>(tp, 1, 32) : 32;
      f.type = bw == 64 ? GZ_TYPE_TIME64 : GZ_TYPE_TIME32;
      break;
    }
    case 10:
      f.type = GZ_TYPE_TIMESTAMP;
      f.unit = tp >= 0 ? r.Scalar<int16_t>(tp, 0, 0) : 0;
      if (tp >= 0) r.String(tp, 1, &f.timezone);
      break;
    default:
      *err = "field type " + std::to_string(tt) + " is not implemented by the GPU splitter";
      return false;
  }
  *out = std::move(f);
  return true;
}

}  // namespace

bool ParseSchemaIpc(const uint8_t* data, int64_t len, std::vector<Field>* out, std::string* err) {
  if (data == nullptr || len < 8) {
    *err = "schema message too short";
    return false;
  }
  int64_t start = 4;
  uint32_t first;
  memcpy(&first, data, 4);
  if (first == 0xFFFFFFFFu) start = 8;  // continuation token, then the metadata length
  FlatReader r(data + start, len - start);
  uint32_t root_rel;
  if (!r.Get(0, &root_rel)) {
    *err = "bad schema flatbuffer";
    return false;
  }
  int64_t msg = root_rel;
  uint8_t header_type = r.Scalar<uint8_t>(msg, 1, 0);
  if (header_type != 1) {
    *err = "IPC message is not a Schema";
    return false;
  }
  int64_t schema = r.Table(msg, 2);
  if (schema < 0) {
    *err = "Schema header missing";
    return false;
  }
  int64_t fields = r.Table(schema, 1);
  uint32_t nf = 0;
  if (fields >= 0 && !r.Get(fields, &nf)) {
    *err = "bad field vector";
    return false;
  }
  out->clear();
  for (uint32_t i = 0; i < nf; i++) {
    int64_t fpos = fields + 4 + 4 * (int64_t)i;
    int64_t ft = r.Deref(fpos);
    if (ft < 0) {
      *err = "bad field table";
      return false;
    }
    Field f;
    if (!DecodeField(r, ft, 0, &f, err)) return false;
    out->push_back(f);
  }
  return true;
}

// ---------------------------------------------------------------------------------------
// Writing: a flatbuffers builder following the published flatbuffers algorithm (the buffer
// grows toward the front, offsets are distances from its end, each table ends with a vtable that
// is shared with an identical earlier one) and Arrow's schema tables built in the order, and
// with the field order inside each table, that Arrow C++ uses, so the bytes match.
namespace {

class Builder {
 public:
  uint32_t Size() const { return (uint32_t)buf_.size(); }
  void Pad(size_t n) { buf_.insert(buf_.begin(), n, 0); }
  void Align(size_t a) {
    minalign_ = std::max(minalign_, a);
    Pad((~buf_.size() + 1) & (a - 1));
  }
  void PreAlign(size_t len, size_t a) {
    if (len == 0) return;
    minalign_ = std::max(minalign_, a);
    Pad((~(buf_.size() + len) + 1) & (a - 1));
  }
  template <typename T>
  uint32_t Push(T v) {
    Align(sizeof(T));
    uint8_t tmp[sizeof(T)];
    memcpy(tmp, &v, sizeof(T));
    buf_.insert(buf_.begin(), tmp, tmp + sizeof(T));
    return Size();
  }
  uint32_t ReferTo(uint32_t off) {
    Align(4);
    return Size() - off + 4;
  }
  uint32_t String(const std::string& s) {
    PreAlign(s.size() + 1, 4);
    buf_.insert(buf_.begin(), 1, 0);
    buf_.insert(buf_.begin(), s.begin(), s.end());
    return Push<uint32_t>((uint32_t)s.size());
  }
  uint32_t OffsetVector(const std::vector<uint32_t>& offs) {
    PreAlign(offs.size() * 4, 4);
    for (size_t i = offs.size(); i-- > 0;) Push<uint32_t>(ReferTo(offs[i]));
    return Push<uint32_t>((uint32_t)offs.size());
  }
  void StartTable() {
    fields_.clear();
    table_start_ = Size();
  }
  template <typename T>
  void AddScalar(uint16_t voff, T v, T def) {
    if (v == def) return;  // defaults are not stored
    fields_.push_back({voff, Push<T>(v)});
  }
  void AddOffset(uint16_t voff, uint32_t off) {
    if (off == 0) return;
    fields_.push_back({voff, Push<uint32_t>(ReferTo(off))});
  }
  uint32_t EndTable() {
    const uint32_t loc = Push<int32_t>(0);
    uint16_t vsize = 4;
    for (auto& f : fields_) vsize = std::max<uint16_t>(vsize, (uint16_t)(f.first + 2));
    std::vector<uint16_t> vt(vsize / 2, 0);
    vt[0] = vsize;
    vt[1] = (uint16_t)(loc - table_start_);
    for (auto& f : fields_) vt[f.first / 2] = (uint16_t)(loc - f.second);
    std::vector<uint8_t> bytes(vsize);
    memcpy(bytes.data(), vt.data(), vsize);
    uint32_t use = 0;
    for (uint32_t prev : vtables_) {  // the first identical vtable written
      if (memcmp(&buf_[buf_.size() - prev], bytes.data(), vsize) == 0) {
        uint16_t psize;
        memcpy(&psize, &buf_[buf_.size() - prev], 2);
        if (psize == vsize) {
          use = prev;
          break;
        }
      }
    }
    if (use == 0) {
      buf_.insert(buf_.begin(), bytes.begin(), bytes.end());
      use = Size();
      vtables_.push_back(use);
    }
    const int32_t soff = (int32_t)use - (int32_t)loc;
    memcpy(&buf_[buf_.size() - loc], &soff, 4);
    return loc;
  }
  std::vector<uint8_t> Finish(uint32_t root) {
    PreAlign(4, minalign_);
    Push<uint32_t>(ReferTo(root));
    return buf_;
  }

 private:
  std::vector<uint8_t> buf_;
  size_t minalign_ = 1;
  uint32_t table_start_ = 0;
  std::vector<std::pair<uint16_t, uint32_t>> fields_;
  std::vector<uint32_t> vtables_;
};

// Arrow Schema.fbs: the Type union tag and table of a field.  Inside a table the fields are
// added largest first and, among equal sizes, last declared first (the generated Create*).
uint8_t TypeTable(Builder& b, const Field& f, uint32_t* table) {
  auto empty = [&]() {
    b.StartTable();
    return b.EndTable();
  };
  auto integer = [&](int32_t bits, bool sign) {
    b.StartTable();
    b.AddScalar<int32_t>(4, bits, 0);
    b.AddScalar<uint8_t>(6, sign ? 1 : 0, 0);
    return b.EndTable();
  };
  auto floating = [&](int16_t prec) {
    b.StartTable();
    b.AddScalar<int16_t>(4, prec, 0);
    return b.EndTable();
  };
  switch (f.type) {
    case GZ_TYPE_NULL: *table = empty(); return 1;
    case GZ_TYPE_BOOL: *table = empty(); return 6;
    case GZ_TYPE_INT8: *table = integer(8, true); return 2;
    case GZ_TYPE_UINT8: *table = integer(8, false); return 2;
    case GZ_TYPE_INT16: *table = integer(16, true); return 2;
    case GZ_TYPE_UINT16: *table = integer(16, false); return 2;
    case GZ_TYPE_INT32: *table = integer(32, true); return 2;
    case GZ_TYPE_UINT32: *table = integer(32, false); return 2;
    case GZ_TYPE_INT64: *table = integer(64, true); return 2;
    case GZ_TYPE_UINT64: *table = integer(64, false); return 2;
    case GZ_TYPE_HALF_FLOAT: *table = floating(0); return 3;
    case GZ_TYPE_FLOAT32: *table = floating(1); return 3;
    case GZ_TYPE_FLOAT64: *table = floating(2); return 3;
    case GZ_TYPE_BINARY: *table = empty(); return 4;
    case GZ_TYPE_STRING: *table = empty(); return 5;
    case GZ_TYPE_LARGE_BINARY: *table = empty(); return 19;  // Schema.fbs Type.LargeBinary
    case GZ_TYPE_LARGE_STRING: *table = empty(); return 20;  // Type.LargeUtf8
    case GZ_TYPE_LIST: *table = empty(); return 12;           // Type.List (its element: a child field)
    case GZ_TYPE_LARGE_LIST: *table = empty(); return 21;     // Type.LargeList
    case GZ_TYPE_STRUCT: *table = empty(); return 13;         // Type.Struct_ (its fields: children)
    case GZ_TYPE_MAP:                                         // Type.Map { keysSorted }
      b.StartTable();
      b.AddScalar<uint8_t>(4, f.keys_sorted ? 1 : 0, 0);
      *table = b.EndTable();
      return 17;
    case GZ_TYPE_DECIMAL128:  // Decimal { precision, scale, bitWidth = 128 }
      b.StartTable();
      b.AddScalar<int32_t>(8, 128, 128);
      b.AddScalar<int32_t>(6, f.scale, 0);
      b.AddScalar<int32_t>(4, f.precision, 0);
      *table = b.EndTable();
      return 7;
    case GZ_TYPE_DATE32:
    case GZ_TYPE_DATE64:  // Date { unit = MILLISECOND }
      b.StartTable();
      b.AddScalar<int16_t>(4, f.type == GZ_TYPE_DATE32 ? 0 : 1, 1);
      *table = b.EndTable();
      return 8;
    case GZ_TYPE_TIME32:
    case GZ_TYPE_TIME64:  // Time { unit = MILLISECOND, bitWidth = 32 }
      b.StartTable();
      b.AddScalar<int32_t>(6, f.type == GZ_TYPE_TIME32 ? 32 : 64, 32);
      b.AddScalar<int16_t>(4, (int16_t)f.unit, 1);
      *table = b.EndTable();
      return 9;
    case GZ_TYPE_TIMESTAMP: {  // Timestamp { unit, timezone }
      const uint32_t tz = f.timezone.empty() ? 0 : b.String(f.timezone);
      b.StartTable();
      b.AddOffset(6, tz);
      b.AddScalar<int16_t>(4, (int16_t)f.unit, 0);
      *table = b.EndTable();
      return 10;
    }
    default: *table = empty(); return 0;
  }
}

}  // namespace

namespace {

// One Field table: the children first (a list's element field, a map's entries, a struct's
// fields: each its own Field table), then the type, the name, the children vector and the Field
// table itself.
uint32_t FieldTable(Builder& b, const Field& f) {
  std::vector<uint32_t> kids;
  for (const Field& c : f.children) kids.push_back(FieldTable(b, c));
  if (f.type == GZ_TYPE_LIST && !f.nested()) {
    Field e;
    e.type = f.elem;
    e.nullable = f.elem_nullable;
    e.precision = f.precision;
    e.scale = f.scale;
    e.unit = f.unit;
    e.timezone = f.timezone;
    e.name = f.elem_name;
    kids.push_back(FieldTable(b, e));
  }
  uint32_t type_table = 0;
  const uint8_t tag = TypeTable(b, f, &type_table);  // type first, then name, then children
  const uint32_t name = b.String(f.name);
  const uint32_t children = b.OffsetVector(kids);
  b.StartTable();  // Field { name, nullable, type_type, type, dictionary, children, custom_metadata }
  b.AddOffset(14, children);
  b.AddOffset(10, type_table);
  b.AddOffset(4, name);
  b.AddScalar<uint8_t>(8, tag, 0);
  b.AddScalar<uint8_t>(6, f.nullable ? 1 : 0, 0);
  return b.EndTable();
}

}  // namespace

std::vector<uint8_t> EncodeSchemaMessage(const std::vector<Field>& fields) {
  Builder b;
  std::vector<uint32_t> offs;
  for (const Field& f : fields) offs.push_back(FieldTable(b, f));
  const uint32_t vec = b.OffsetVector(offs);
  b.StartTable();  // Schema { endianness = Little, fields, custom_metadata, features }
  b.AddOffset(6, vec);
  b.AddScalar<int16_t>(4, 0, 0);
  const uint32_t schema = b.EndTable();
  b.StartTable();  // Message { version, header_type, header, bodyLength, custom_metadata }
  b.AddScalar<int64_t>(10, 0, 0);
  b.AddOffset(8, schema);
  b.AddScalar<int16_t>(4, 4 /* V5 */, 0);
  b.AddScalar<uint8_t>(6, 1 /* Schema */, 0);
  const uint32_t msg = b.EndTable();
  const std::vector<uint8_t> meta = b.Finish(msg);
  // encapsulation: continuation marker, metadata length (padded to 8), metadata, padding
  const size_t padded = (meta.size() + 8 + 7) & ~size_t(7);
  std::vector<uint8_t> out(padded, 0);
  const uint32_t cont = 0xFFFFFFFFu;
  const int32_t mlen = (int32_t)(padded - 8);
  memcpy(out.data(), &cont, 4);
  memcpy(out.data() + 4, &mlen, 4);
  memcpy(out.data() + 8, meta.data(), meta.size());
  return out;
}

}  // namespace gz
