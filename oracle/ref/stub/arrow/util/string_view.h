/* Oracle build shim (test infrastructure only): Arrow 25 dropped arrow/util/string_view.h,
 * which the reference's murmurhash32.h still includes. */
#pragma once
#include <string_view>
namespace arrow {
namespace util {
using std::string_view;
}
}  // namespace arrow
