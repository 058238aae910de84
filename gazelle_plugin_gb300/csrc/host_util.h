// Host-side helpers of the splitter: a process-wide pool of pinned host blocks (flush outputs
// copied out of HBM) and a small thread pool that spreads large memcpys over several cores
// (staging a caller's host batch before Split returns).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <functional>
#include <vector>

namespace gz {

struct PinnedBlock {
  uint8_t* ptr = nullptr;
  size_t cap = 0;
};

// Pinned (page-locked) host blocks, reused across splitters.  Acquire returns a block of at
// least `bytes` (cap = its size); ptr == nullptr when cudaHostAlloc failed.  Release takes back
// exactly a block Acquire returned.
PinnedBlock PinnedAcquire(size_t bytes);
void PinnedRelease(PinnedBlock b);
// Adds about `bytes` of pinned slabs of `block` bytes to the pool up front (cudaHostAlloc is
// slow, so a server takes that cost at start instead of inside calls); returns the bytes added.
int64_t PinnedReserve(int64_t bytes, size_t block);
constexpr size_t kPinnedSlab = size_t(1) << 30;

struct CopyJob {
  uint8_t* dst;
  const uint8_t* src;
  size_t n;
};

// Copies every job; large totals are split over worker threads and the caller.  Returns when
// all bytes are copied.
void ParallelCopy(const std::vector<CopyJob>& jobs, size_t total_bytes);

// Runs fn(i) for every i in [0, n) on the calling thread and up to `max_helpers` threads of a
// process-wide pool (shared by all splitters: concurrent calls share its workers); returns when
// every fn(i) has returned.  Items are claimed one at a time, so long and short items balance.
void ParallelFor(size_t n, const std::function<void(size_t)>& fn, int max_helpers = 15);

}  // namespace gz
