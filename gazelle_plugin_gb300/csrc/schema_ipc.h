#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace gz {

struct Field {
  int type = 0;  // GzType
  bool nullable = true;
  int precision = 0;
  int scale = 0;
  int unit = 0;
  std::string name;
  std::string timezone;  // timestamp only; empty: none
  // a list of fixed-width or bool elements ("simple list", no children): the element field
  // (its precision / scale / unit are the ones above)
  int elem = 0;
  std::string elem_name = "item";
  bool elem_nullable = true;
  // nested types (list / large_list / map / struct with `children`): a list's element field,
  // a map's entries struct (whose children are the key and the value), a struct's fields
  std::vector<Field> children;
  bool keys_sorted = false;  // map
  bool nested() const { return !children.empty(); }
};

// Parses an Arrow IPC Schema message (encapsulated or legacy framing).
bool ParseSchemaIpc(const uint8_t* data, int64_t len, std::vector<Field>* out, std::string* err);

// The encapsulated Arrow IPC Schema message of `fields` (MetadataVersion V5, little endian, no
// metadata), byte for byte what Arrow C++'s GetSchemaPayload + WriteIpcPayload write for the same
// schema (the reference's schema message, splitter.cc:145-151, 1355-1364).
std::vector<uint8_t> EncodeSchemaMessage(const std::vector<Field>& fields);

}  // namespace gz
