/* Oracle build shim (test infrastructure only): see uuid_generators.hpp. */
#pragma once
#include <cstdio>
#include <string>
#include "uuid_generators.hpp"
namespace boost {
namespace uuids {
inline std::string to_string(const uuid& u) {
  char buf[40];
  std::snprintf(buf, sizeof(buf), "%016llx%016llx", u.hi, u.lo);
  return std::string(buf);
}
}  // namespace uuids
}  // namespace boost
