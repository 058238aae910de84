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
  // list: the element field (a fixed-width type; its precision / scale / unit are the ones above)
  int elem = 0;
  std::string elem_name = "item";
  bool elem_nullable = true;
};

// Parses an Arrow IPC Schema message (encapsulated or legacy framing).
bool ParseSchemaIpc(const uint8_t* data, int64_t len, std::vector<Field>* out, std::string* err);

// The encapsulated Arrow IPC Schema message of `fields` (MetadataVersion V5, little endian, no
// metadata), byte for byte what Arrow C++'s GetSchemaPayload + WriteIpcPayload write for the same
// schema (the reference's schema message, splitter.cc:145-151, 1355-1364).
std::vector<uint8_t> EncodeSchemaMessage(const std::vector<Field>& fields);

}  // namespace gz
