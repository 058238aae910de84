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
};

// Parses an Arrow IPC Schema message (encapsulated or legacy framing).
bool ParseSchemaIpc(const uint8_t* data, int64_t len, std::vector<Field>* out, std::string* err);

}  // namespace gz
