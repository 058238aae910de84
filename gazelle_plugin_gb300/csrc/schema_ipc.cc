// Reads the Arrow IPC Schema message the JNI layer receives (MakeSchema,
// native-sql-engine/cpp/src/jni/jni_common.h:393-406) into the splitter's field list.
// A small flatbuffer reader over the Arrow format's Message / Schema / Field tables.
#include "schema_ipc.h"

#include <string.h>

#include "../../include/gz_split.h"

namespace gz {

namespace {

class Reader {
 public:
  Reader(const uint8_t* p, int64_t n) : p_(p), n_(n) {}
  bool ok(int64_t pos, int64_t len) const { return pos >= 0 && len >= 0 && pos + len <= n_; }
  template <typename T>
  bool Get(int64_t pos, T* out) const {
    if (!ok(pos, sizeof(T))) return false;
    memcpy(out, p_ + pos, sizeof(T));
    return true;
  }
  // absolute position of field `idx` of the table at `t`, or 0 when absent / invalid
  int64_t Field(int64_t t, int idx) const {
    int32_t vt_rel;
    if (!Get(t, &vt_rel)) return 0;
    int64_t vt = t - vt_rel;
    uint16_t vt_size;
    if (!Get(vt, &vt_size)) return 0;
    if (4 + 2 * idx >= vt_size) return 0;
    uint16_t off;
    if (!Get(vt + 4 + 2 * idx, &off) || off == 0) return 0;
    return t + off;
  }
  int64_t Deref(int64_t pos) const {
    uint32_t rel;
    if (!Get(pos, &rel)) return -1;
    return pos + rel;
  }
  template <typename T>
  T Scalar(int64_t t, int idx, T def) const {
    int64_t f = Field(t, idx);
    T v = def;
    if (f) Get(f, &v);
    return v;
  }
  int64_t Table(int64_t t, int idx) const {
    int64_t f = Field(t, idx);
    return f ? Deref(f) : -1;
  }
  bool String(int64_t t, int idx, std::string* s) const {
    int64_t pos = Table(t, idx);
    if (pos < 0) {
      s->clear();
      return true;
    }
    uint32_t len;
    if (!Get(pos, &len) || !ok(pos + 4, len)) return false;
    s->assign(reinterpret_cast<const char*>(p_ + pos + 4), len);
    return true;
  }

 private:
  const uint8_t* p_;
  int64_t n_;
};

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
  Reader r(data + start, len - start);
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
    if (!r.String(ft, 0, &f.name)) {
      *err = "bad field name";
      return false;
    }
    f.nullable = r.Scalar<uint8_t>(ft, 1, 0) != 0;
    uint8_t tt = r.Scalar<uint8_t>(ft, 2, 0);
    int64_t tp = r.Table(ft, 3);
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
        break;
      default:
        *err = "field type " + std::to_string(tt) + " is not implemented by the GPU splitter";
        return false;
    }
    out->push_back(f);
  }
  return true;
}

}  // namespace gz
