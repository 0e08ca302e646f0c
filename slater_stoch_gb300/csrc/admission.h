// admission.h -- admission of asynchronous jobs by device-memory footprint and concurrency.
//
// Host-only C++ (no CUDA), shared by the job API and its host test.  Jobs are admitted strictly
// in submission order: a job starts when it is at the head of the queue, fewer than max_running
// jobs run, and its footprint fits in what the running jobs leave of the budget.  A job always
// starts when nothing else runs, so lowering the limits can never strand a queued job, and a job
// whose footprint alone exceeds the budget is refused when it is enqueued.
#pragma once
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <set>

namespace ss {

class JobAdmission {
 public:
  struct Stats {
    int running = 0, queued = 0, peak_running = 0;
    size_t used = 0, peak_used = 0;
  };

  // budget_bytes == 0: no memory limit; max_running == 0: no concurrency limit
  void set_limits(size_t budget_bytes, int max_running) {
    std::lock_guard<std::mutex> lk(mu_);
    budget_ = budget_bytes;
    max_running_ = max_running;
    cv_.notify_all();
  }

  // a ticket in submission order, or -1 when the job alone exceeds the budget
  int64_t enqueue(size_t bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    if (budget_ && bytes > budget_) return -1;
    return next_++;
  }

  // a ticket whose job will never call admit (its thread did not start)
  void abandon(int64_t ticket) {
    std::lock_guard<std::mutex> lk(mu_);
    skipped_.insert(ticket);
    advance_head();
    cv_.notify_all();
  }

  // blocks until the job may start; the caller must release(bytes) when it ends.  Returns the
  // job's rank among the admitted jobs (0, 1, ...), taken under the admission's lock.
  int64_t admit(int64_t ticket, size_t bytes) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] {
      if (head_ != ticket) return false;
      if (running_ == 0) return true;
      if (max_running_ && running_ >= max_running_) return false;
      return !budget_ || used_ + bytes <= budget_;
    });
    running_++;
    used_ += bytes;
    if (running_ > peak_running_) peak_running_ = running_;
    if (used_ > peak_used_) peak_used_ = used_;
    head_++;
    advance_head();
    cv_.notify_all();
    return admitted_++;
  }

  void release(size_t bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    running_--;
    used_ -= bytes;
    cv_.notify_all();
  }

  Stats stats() {
    std::lock_guard<std::mutex> lk(mu_);
    Stats s;
    s.running = running_;
    s.queued = (int)(next_ - head_ - (int64_t)skipped_.size());
    s.peak_running = peak_running_;
    s.used = used_;
    s.peak_used = peak_used_;
    return s;
  }

 private:
  void advance_head() {  // skip abandoned tickets at the head (mu_ held)
    while (!skipped_.empty() && *skipped_.begin() == head_) {
      skipped_.erase(skipped_.begin());
      head_++;
    }
  }

  std::mutex mu_;
  std::condition_variable cv_;
  size_t budget_ = 0, used_ = 0, peak_used_ = 0;
  int max_running_ = 0, running_ = 0, peak_running_ = 0;
  int64_t next_ = 0, head_ = 0, admitted_ = 0;
  std::set<int64_t> skipped_;
};

// Device bytes per quartet that a two-electron job keeps while it runs: quartet indices (16),
// work list and slot codes (16), partial sums of the bra slices (>= 8), Gaussian-fit ERIs (8), MC
// mean and error (16), MC accumulators (16), merged ERIs (8), rounded up.  The job's ERI-buffer
// footprint, by which it is admitted, is this times its number of quartets.
constexpr size_t JOB_BYTES_PER_QUARTET = 96;

}  // namespace ss
