// A small bounds-checked reader of flatbuffers (the Arrow IPC metadata encoding): table fields
// through their vtables, offsets, scalars, strings.  Every access is checked against the buffer.
#pragma once
#include <stdint.h>
#include <string.h>

#include <string>

namespace gz {

class FlatReader {
 public:
  FlatReader(const uint8_t* p, int64_t n) : p_(p), n_(n) {}
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


}  // namespace gz
