/*
 * Oracle build (test infrastructure only): exposes the reference's own Spark-form 64-bit
 * Murmur3 (native-sql-engine/cpp/src/third_party/murmurhash/murmurhash32.h:74-108,
 * compiled from the reference tree) so the tests can pin the restated hashLong against it.
 */
#include <cstdint>

#include "third_party/murmurhash/murmurhash32.h"

extern "C" int32_t gzref_hash_long(int64_t v, int32_t seed) {
  return sparkcolumnarplugin::thirdparty::murmurhash32::hash32<int64_t>(v, seed);
}
