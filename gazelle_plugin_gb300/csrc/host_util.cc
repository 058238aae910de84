#include "host_util.h"

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

namespace gz {

// ---------------------------------------------------------------------------------------
// Pinned pool: slabs of page-locked memory (cudaHostAlloc is slow and never undone here),
// carved best-fit into blocks in 64 KiB units; a freed block merges with free neighbours of the
// same slab.  Blocks never span two slabs, so each is inside one cudaHostAlloc allocation.
namespace {
constexpr size_t kPinUnit = size_t(64) << 10;
constexpr size_t kSlab = size_t(1) << 30;

struct PinPool {
  std::mutex mu;
  std::map<uint8_t*, std::pair<size_t, int>> free_by_addr;  // start -> (bytes, slab)
  std::multimap<size_t, uint8_t*> free_by_size;              // bytes -> start
  std::vector<std::pair<uint8_t*, size_t>> slabs;

  void insert(uint8_t* p, size_t n, int slab) {
    free_by_addr[p] = {n, slab};
    free_by_size.emplace(n, p);
  }
  void erase_size(uint8_t* p, size_t n) {
    auto r = free_by_size.equal_range(n);
    for (auto it = r.first; it != r.second; ++it)
      if (it->second == p) {
        free_by_size.erase(it);
        return;
      }
  }
  int slab_of(uint8_t* p) const {
    for (size_t i = 0; i < slabs.size(); i++)
      if (p >= slabs[i].first && p < slabs[i].first + slabs[i].second) return (int)i;
    return -1;
  }
  bool add_slab(size_t n) {  // mu held
    void* p = nullptr;
    if (cudaHostAlloc(&p, n, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    slabs.push_back({static_cast<uint8_t*>(p), n});
    insert(static_cast<uint8_t*>(p), n, (int)slabs.size() - 1);
    return true;
  }
};
// never destroyed: splitters may give blocks back during exit
PinPool& g_pin = *new PinPool;
}  // namespace

PinnedBlock PinnedAcquire(size_t bytes) {
  const size_t n = (std::max<size_t>(bytes, 1) + kPinUnit - 1) / kPinUnit * kPinUnit;
  std::lock_guard<std::mutex> lk(g_pin.mu);
  auto it = g_pin.free_by_size.lower_bound(n);
  if (it == g_pin.free_by_size.end()) {
    if (!g_pin.add_slab(std::max(n, kSlab))) return PinnedBlock{};
    it = g_pin.free_by_size.lower_bound(n);
  }
  uint8_t* p = it->second;
  const size_t have = it->first;
  g_pin.free_by_size.erase(it);
  const int slab = g_pin.free_by_addr[p].second;
  g_pin.free_by_addr.erase(p);
  if (have > n) g_pin.insert(p + n, have - n, slab);
  return PinnedBlock{p, n};
}

void PinnedRelease(PinnedBlock b) {
  if (!b.ptr) return;
  std::lock_guard<std::mutex> lk(g_pin.mu);
  uint8_t* p = b.ptr;
  size_t n = b.cap;
  const int slab = g_pin.slab_of(p);
  auto next = g_pin.free_by_addr.find(p + n);
  if (next != g_pin.free_by_addr.end() && next->second.second == slab) {
    n += next->second.first;
    g_pin.erase_size(next->first, next->second.first);
    g_pin.free_by_addr.erase(next);
  }
  auto prev = g_pin.free_by_addr.lower_bound(p);
  if (prev != g_pin.free_by_addr.begin()) {
    --prev;
    if (prev->first + prev->second.first == p && prev->second.second == slab) {
      p = prev->first;
      n += prev->second.first;
      g_pin.erase_size(prev->first, prev->second.first);
      g_pin.free_by_addr.erase(prev);
    }
  }
  g_pin.insert(p, n, slab);
}

int64_t PinnedReserve(int64_t bytes, size_t block) {
  int64_t got = 0;
  std::lock_guard<std::mutex> lk(g_pin.mu);
  while (got < bytes) {
    if (!g_pin.add_slab(block)) break;
    got += (int64_t)block;
  }
  return got;
}

// ---------------------------------------------------------------------------------------
namespace {

constexpr size_t kChunk = 256u << 10;

// One parallel copy: chunks of the concatenated job space are claimed with an atomic
// counter.  Each worker holds its own reference to the task it woke up for, so a worker that
// arrives after the task finished only sees an exhausted counter.
struct CopyTask {
  const std::vector<CopyJob>* jobs;
  std::vector<size_t> prefix;
  size_t total, nchunks;
  std::atomic<size_t> next{0}, done{0};

  void Work() {
    for (;;) {
      const size_t c = next.fetch_add(1);
      if (c >= nchunks) return;
      const size_t lo = c * kChunk, hi = std::min(total, lo + kChunk);
      const std::vector<CopyJob>& js = *jobs;
      size_t j = std::upper_bound(prefix.begin(), prefix.end(), lo) - prefix.begin() - 1;
      size_t pos = lo;
      while (pos < hi && j < js.size()) {
        const size_t jlo = prefix[j], jhi = prefix[j + 1];
        const size_t a = std::max(pos, jlo), b = std::min(hi, jhi);
        if (b > a) memcpy(js[j].dst + (a - jlo), js[j].src + (a - jlo), b - a);
        pos = std::max(pos, b);
        j++;
      }
      done.fetch_add(1, std::memory_order_release);
    }
  }
};

class CopyPool {
 public:
  static CopyPool& Get() {
    static CopyPool* pool = new CopyPool();  // workers live until process exit
    return *pool;
  }

  void Run(const std::vector<CopyJob>& jobs, size_t total) {
    auto task = std::make_shared<CopyTask>();
    task->jobs = &jobs;
    task->prefix.resize(jobs.size() + 1);
    task->prefix[0] = 0;
    for (size_t i = 0; i < jobs.size(); i++) task->prefix[i + 1] = task->prefix[i] + jobs[i].n;
    task->total = total;
    task->nchunks = (total + kChunk - 1) / kChunk;
    {
      std::lock_guard<std::mutex> lk(mu_);
      current_ = task;
      gen_++;
    }
    cv_.notify_all();
    task->Work();
    while (task->done.load(std::memory_order_acquire) < task->nchunks) std::this_thread::yield();
  }

 private:
  CopyPool() {
    unsigned hc = std::thread::hardware_concurrency();
    int n = (int)std::min<unsigned>(7, hc > 2 ? hc / 2 : 1);
    for (int i = 0; i < n; i++) std::thread([this] { Loop(); }).detach();
  }

  void Loop() {
    uint64_t seen = 0;
    for (;;) {
      std::shared_ptr<CopyTask> task;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        task = current_;
      }
      if (task) task->Work();
    }
  }

  std::mutex mu_;
  std::condition_variable cv_;
  uint64_t gen_ = 0;
  std::shared_ptr<CopyTask> current_;
};

}  // namespace

// ---------------------------------------------------------------------------------------
namespace {

struct ForJob {
  const std::function<void(size_t)>* fn;
  size_t n;
  std::atomic<size_t> next{0};
  std::atomic<size_t> done{0};
  std::mutex mu;
  std::condition_variable cv;

  void Work() {
    for (;;) {
      const size_t i = next.fetch_add(1);
      if (i >= n) return;
      (*fn)(i);
      if (done.fetch_add(1) + 1 == n) {
        std::lock_guard<std::mutex> lk(mu);
        cv.notify_all();
      }
    }
  }
};

class ForPool {
 public:
  static ForPool& Get() {
    static ForPool* pool = new ForPool();  // workers live until process exit
    return *pool;
  }
  int workers() const { return n_; }
  void Post(const std::shared_ptr<ForJob>& job, int tickets) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (int i = 0; i < tickets; i++) q_.push_back(job);
    }
    if (tickets == 1) cv_.notify_one();
    else cv_.notify_all();
  }

 private:
  ForPool() {
    const unsigned hc = std::thread::hardware_concurrency();
    n_ = (int)std::max<unsigned>(1, std::min<unsigned>(31, hc > 1 ? hc - 1 : 1));
    for (int i = 0; i < n_; i++) std::thread([this] { Loop(); }).detach();
  }
  void Loop() {
    for (;;) {
      std::shared_ptr<ForJob> job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !q_.empty(); });
        job = q_.front();
        q_.pop_front();
      }
      job->Work();
    }
  }
  int n_ = 1;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<ForJob>> q_;
};

}  // namespace

void ParallelFor(size_t n, const std::function<void(size_t)>& fn, int max_helpers) {
  if (n == 0) return;
  if (n == 1 || max_helpers <= 0) {
    for (size_t i = 0; i < n; i++) fn(i);
    return;
  }
  auto job = std::make_shared<ForJob>();
  job->fn = &fn;
  job->n = n;
  ForPool& pool = ForPool::Get();
  const int helpers = (int)std::min<size_t>({(size_t)max_helpers, (size_t)pool.workers(), n - 1});
  pool.Post(job, helpers);
  job->Work();
  std::unique_lock<std::mutex> lk(job->mu);
  job->cv.wait(lk, [&] { return job->done.load() == n; });
}

void ParallelCopy(const std::vector<CopyJob>& jobs, size_t total_bytes) {
  if (total_bytes < (1u << 20)) {
    for (const CopyJob& j : jobs)
      if (j.n) memcpy(j.dst, j.src, j.n);
    return;
  }
  CopyPool::Get().Run(jobs, total_bytes);
}

}  // namespace gz
