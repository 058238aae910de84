// gz::ServeLoop (serve.h).
#include "serve.h"

#include <chrono>

namespace gz {

namespace {
int64_t NowNs() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
}  // namespace

ServeLoop::ServeLoop(int32_t slots, int64_t hbm_budget) : budget_(hbm_budget) {
  if (slots < 1) slots = 1;
  for (int32_t i = 0; i < slots; i++) {
    workers_.push_back(std::make_unique<Worker>());
    Worker* w = workers_.back().get();
    w->thread = std::thread([this, w] { Run(w); });
  }
}

ServeLoop::~ServeLoop() {
  for (auto& w : workers_) {
    {
      std::lock_guard<std::mutex> lk(w->mu);
      w->stop = true;
    }
    w->cv.notify_all();
  }
  for (auto& w : workers_) w->thread.join();
}

Status ServeLoop::Admit(int64_t bytes) {
  std::unique_lock<std::mutex> lk(mu_);
  if (bytes > budget_)
    return Status::Error(GZ_INVALID, "task needs " + std::to_string(bytes) + " bytes of an HBM budget of " +
                                         std::to_string(budget_));
  budget_cv_.wait(lk, [&] { return reserved_ + bytes <= budget_; });
  reserved_ += bytes;
  return Status::OK();
}

void ServeLoop::Release(int64_t bytes) {
  {
    std::lock_guard<std::mutex> lk(mu_);
    reserved_ -= bytes;
  }
  budget_cv_.notify_all();
}

int64_t ServeLoop::reserved() const {
  std::lock_guard<std::mutex> lk(mu_);
  return reserved_;
}

int32_t ServeLoop::AssignSlot() {
  std::lock_guard<std::mutex> lk(mu_);
  const int32_t s = next_slot_;
  next_slot_ = (next_slot_ + 1) % (int32_t)workers_.size();
  return s;
}

int64_t ServeLoop::Submit(int32_t slot, Splitter* s, std::shared_ptr<void> keep, Kind kind, int32_t rows,
                          const int64_t* addrs, const int64_t* sizes, int32_t n, int64_t release_bytes) {
  Request r;
  r.s = s;
  r.keep = std::move(keep);
  r.kind = kind;
  r.rows = rows;
  if (kind == kSplit && n > 0) {
    r.addrs.assign(addrs, addrs + n);
    r.sizes.assign(sizes, sizes + n);
  }
  r.release_bytes = release_bytes;
  {
    std::lock_guard<std::mutex> lk(mu_);
    r.ticket = next_ticket_++;
    done_[r.ticket] = Done();
  }
  r.t_submit = NowNs();
  const int64_t t = r.ticket;
  Worker* w = workers_[(size_t)slot % workers_.size()].get();
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->queue.push_back(std::move(r));
  }
  w->cv.notify_one();
  return t;
}

Status ServeLoop::Wait(int64_t ticket, int64_t* latency_ns, int64_t* service_ns) {
  std::unique_lock<std::mutex> lk(mu_);
  auto it = done_.find(ticket);
  if (it == done_.end()) return Status::Error(GZ_INVALID, "unknown ticket " + std::to_string(ticket));
  done_cv_.wait(lk, [&] { return done_[ticket].done; });
  Done d = done_[ticket];
  done_.erase(ticket);
  if (latency_ns) *latency_ns = d.latency_ns;
  if (service_ns) *service_ns = d.service_ns;
  return d.status;
}

void ServeLoop::Run(Worker* w) {
  for (;;) {
    Request r;
    {
      std::unique_lock<std::mutex> lk(w->mu);
      w->cv.wait(lk, [&] { return w->stop || !w->queue.empty(); });
      if (w->queue.empty()) return;  // stop requested and nothing left
      r = std::move(w->queue.front());
      w->queue.pop_front();
    }
    Status st;
    const int64_t t_start = NowNs();
    if (r.kind == kSplit) {
      st = r.s->Split(r.rows, r.addrs.data(), r.sizes.data(), (int32_t)r.addrs.size());
    } else if (r.kind == kSync) {
      st = r.s->Sync();
    } else {
      st = r.s->Stop();
      if (r.release_bytes > 0) Release(r.release_bytes);
    }
    const int64_t lat = NowNs() - r.t_submit;
    r.keep.reset();
    {
      std::lock_guard<std::mutex> lk(mu_);
      Done& d = done_[r.ticket];
      d.done = true;
      d.status = st;
      d.latency_ns = lat;
      d.service_ns = NowNs() - t_start;
    }
    done_cv_.notify_all();
  }
}

}  // namespace gz
