/* Oracle build shim (test infrastructure only): the reference names its temp files with a
 * boost uuid (native-sql-engine/cpp/src/shuffle/utils.h:50-53); boost is not installed, so a
 * random 128-bit hex string stands in.  File names never reach the shuffle output bytes. */
#pragma once
#include <random>
#include <string>
namespace boost {
namespace uuids {
struct uuid {
  unsigned long long hi, lo;
};
class random_generator {
 public:
  uuid operator()() {
    static thread_local std::mt19937_64 rng{std::random_device{}()};
    return uuid{rng(), rng()};
  }
};
}  // namespace uuids
}  // namespace boost
