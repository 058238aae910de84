// gz::tune (tune.h).
#include "tune.h"

#include <stdio.h>
#include <stdlib.h>

#include <map>
#include <mutex>

namespace gz {

namespace {

struct Cache {
  std::mutex mu;
  std::map<std::string, TuneChoice> entries;
  bool env_loaded = false;
};

// Immortal: splitters made from static destructors of other libraries may still look it up.
Cache& cache() {
  static Cache* c = new Cache();
  return *c;
}

Status LoadLocked(Cache& c, const std::string& path) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return Status::Error(GZ_IO, "cannot open tuning cache " + path);
  char line[4096];
  while (fgets(line, sizeof(line), f)) {
    // <signature> <flush_bytes> <seg_tiles> <gbs>; the signature holds no blanks
    char sig[4000];
    long long flush = 0;
    int seg = 0;
    double gbs = 0;
    if (sscanf(line, "%3999s %lld %d %lf", sig, &flush, &seg, &gbs) == 4 && flush > 0 && seg >= 0)
      c.entries[sig] = TuneChoice{(int64_t)flush, (int32_t)seg, gbs};
  }
  fclose(f);
  return Status::OK();
}

void LoadEnvOnce(Cache& c) {
  if (c.env_loaded) return;
  c.env_loaded = true;
  const char* p = getenv("GZ_TUNE_CACHE");
  if (p && *p) (void)LoadLocked(c, p);  // a missing file is an empty cache
}

}  // namespace

// A field's type: its code, then a list's element type or a nested field's children in brackets.
static std::string TypeTag(const Field& f) {
  std::string s = std::to_string(f.type);
  if (f.type == GZ_TYPE_LIST && !f.nested()) return s + "[" + std::to_string(f.elem) + "]";
  if (!f.nested()) return s;
  s += "[";
  for (size_t i = 0; i < f.children.size(); i++) s += (i ? "," : "") + TypeTag(f.children[i]);
  return s + "]";
}

std::string SchemaSignature(const std::string& short_name, const std::vector<Field>& fields,
                            const std::vector<int32_t>& keys, int32_t P) {
  const bool hash = short_name == "hash";
  if (short_name == "single") P = 1;  // whatever count was asked for
  std::string s = hash ? "t=" : "m=" + short_name + ";t=";
  for (size_t i = 0; i < fields.size(); i++) s += (i ? "," : "") + TypeTag(fields[i]);
  s += ";k=";
  for (size_t i = 0; hash && i < keys.size(); i++) s += (i ? "," : "") + std::to_string(keys[i]);
  s += ";P=" + std::to_string(P);
  return s;
}

bool TuneLookup(const std::string& signature, TuneChoice* out) {
  Cache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  LoadEnvOnce(c);
  auto it = c.entries.find(signature);
  if (it == c.entries.end()) return false;
  *out = it->second;
  return true;
}

void TuneStore(const std::string& signature, const TuneChoice& choice) {
  Cache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  LoadEnvOnce(c);
  c.entries[signature] = choice;
}

Status TuneSave(const std::string& path) {
  Cache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return Status::Error(GZ_IO, "cannot write tuning cache " + path);
  for (const auto& e : c.entries)
    fprintf(f, "%s %lld %d %.3f\n", e.first.c_str(), (long long)e.second.flush_bytes, e.second.seg_tiles,
            e.second.gbs);
  const bool ok = fclose(f) == 0;
  return ok ? Status::OK() : Status::Error(GZ_IO, "cannot write tuning cache " + path);
}

Status TuneLoad(const std::string& path) {
  Cache& c = cache();
  std::lock_guard<std::mutex> lk(c.mu);
  LoadEnvOnce(c);
  return LoadLocked(c, path);
}

}  // namespace gz
