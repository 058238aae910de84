#include "host_util.h"

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

namespace gz {

// ---------------------------------------------------------------------------------------
namespace {
std::mutex g_pin_mu;
std::multimap<size_t, uint8_t*> g_pin_free;  // cap -> block
}  // namespace

PinnedBlock PinnedAcquire(size_t bytes) {
  const size_t gran = 2u << 20;
  const size_t cap = (bytes + gran - 1) / gran * gran;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin_free.lower_bound(cap);
    if (it != g_pin_free.end() && it->first <= 2 * cap + gran) {
      PinnedBlock b{it->second, it->first};
      g_pin_free.erase(it);
      return b;
    }
  }
  void* p = nullptr;
  if (cudaHostAlloc(&p, cap, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return PinnedBlock{};
  }
  return PinnedBlock{static_cast<uint8_t*>(p), cap};
}

void PinnedRelease(PinnedBlock b) {
  if (!b.ptr) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.emplace(b.cap, b.ptr);
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

void ParallelCopy(const std::vector<CopyJob>& jobs, size_t total_bytes) {
  if (total_bytes < (1u << 20)) {
    for (const CopyJob& j : jobs)
      if (j.n) memcpy(j.dst, j.src, j.n);
    return;
  }
  CopyPool::Get().Run(jobs, total_bytes);
}

}  // namespace gz
