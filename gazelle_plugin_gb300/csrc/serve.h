// gz::ServeLoop — the served form: Split / Stop calls of many concurrent tasks, each with its own
// schema, batch sizes and partition count, on one GPU.
//
// A task is an ordinary splitter whose calls go through the loop instead of being made by the
// task's own thread.  Each task is pinned to one of `slots` workers, so its calls run in order,
// while the calls of tasks on other workers run at the same time: their host reads, device
// passes and copies back overlap on the GPU (every splitter has its own streams).  A task is
// admitted only when its share of the HBM budget is free — its spill threshold (partition data
// kept resident before it moves to pinned host memory) plus its staging — and gives the share
// back when it stops.  Every call is timed from submission to completion (its host buffers read
// and its batch queued for the device), which is the per-Split latency reported by the benchmark.
#pragma once

#include <stdint.h>

#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "splitter.h"

namespace gz {

class ServeLoop {
 public:
  ServeLoop(int32_t slots, int64_t hbm_budget);
  ~ServeLoop();  // finishes the queued calls, then joins the workers

  // Blocks until `bytes` of the HBM budget are free and takes them; INVALID when `bytes` exceeds
  // the whole budget.
  Status Admit(int64_t bytes);
  void Release(int64_t bytes);
  // Worker of a new task (round robin).
  int32_t AssignSlot();

  enum Kind { kSplit = 0, kStop = 1, kSync = 2 };
  // Queues a call on `slot`; `keep` holds the splitter alive.  For kSplit the caller keeps the
  // buffers valid until Wait(ticket) returns.  Returns the ticket.
  int64_t Submit(int32_t slot, Splitter* s, std::shared_ptr<void> keep, Kind kind, int32_t rows,
                 const int64_t* addrs, const int64_t* sizes, int32_t n, int64_t release_bytes);
  // Waits for a ticket; its status, message, latency (ns, submission to completion) and service
  // time (ns the worker spent on it; the rest of the latency was queueing).
  Status Wait(int64_t ticket, int64_t* latency_ns, int64_t* service_ns = nullptr);

  int64_t reserved() const;

 private:
  struct Request {
    int64_t ticket;
    Splitter* s;
    std::shared_ptr<void> keep;
    Kind kind;
    int32_t rows;
    std::vector<int64_t> addrs, sizes;
    int64_t t_submit;
    int64_t release_bytes;  // budget returned once a kStop completes
  };
  struct Done {
    bool done = false;
    Status status;
    int64_t latency_ns = 0;
    int64_t service_ns = 0;
  };
  struct Worker {
    std::thread thread;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request> queue;
    bool stop = false;
  };
  void Run(Worker* w);

  int64_t budget_;
  mutable std::mutex mu_;              // budget, tickets
  std::condition_variable budget_cv_;
  std::condition_variable done_cv_;
  int64_t reserved_ = 0;
  int64_t next_ticket_ = 1;
  int32_t next_slot_ = 0;
  std::unordered_map<int64_t, Done> done_;
  std::vector<std::unique_ptr<Worker>> workers_;
};

}  // namespace gz
