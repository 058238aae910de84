/* Oracle build shim (test infrastructure only), force-included before the reference's
 * splitter.cc when it is compiled against the libarrow 25 that ships with pyarrow:
 *  - arrow::BitUtil was renamed arrow::bit_util;
 *  - splitter.cc relies on arrow/builder.h and arrow/array.h arriving transitively;
 *  - the fork's io::UnlockedBufferedOutputStream is upstream's io::BufferedOutputStream
 *    (same Create signature; buffering never changes the bytes written).
 * The FASTPFOR codec and Codec::CreateInt32 exist only in the Arrow fork; the build maps
 * them with -D flags (see Makefile) and only the uncompressed branch is ever taken. */
#pragma once
#include <arrow/api.h>
#include <arrow/array.h>
#include <arrow/builder.h>
#include <arrow/io/buffered.h>
#include <arrow/ipc/api.h>
#include <arrow/util/bit_util.h>
namespace arrow {
namespace BitUtil = ::arrow::bit_util;
namespace io {
using UnlockedBufferedOutputStream = BufferedOutputStream;
}
}
