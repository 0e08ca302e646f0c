// Host build of the job admission (slater_stoch_gb300/csrc/admission.h) driven by fake jobs:
// threads that enqueue, wait for admission, record what ran concurrently, sleep and release.
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "admission.h"

extern "C" {

// njobs jobs of bytes[j]; limits (budget, max_running); job j abandons its ticket if abandon[j].
// Outputs: start_order[j] = rank of job j's start (-1: refused or abandoned), refused[j],
// peak_running (observed by the jobs themselves), peak_bytes (observed), and the admission's own
// stats (stat_peak_running, stat_peak_bytes).
int ss_host_admission_run(int njobs, const long long* bytes, const int* abandon, long long budget,
                          int max_running, int sleep_ms, int* start_order, int* refused,
                          int* peak_running, long long* peak_bytes, int* stat_peak_running,
                          long long* stat_peak_bytes) {
  ss::JobAdmission adm;
  adm.set_limits((size_t)budget, max_running);
  std::mutex mu;
  int running = 0;
  long long used = 0;
  *peak_running = 0;
  *peak_bytes = 0;
  std::vector<std::thread> th;
  for (int j = 0; j < njobs; j++) {
    start_order[j] = -1;
    const int64_t ticket = adm.enqueue((size_t)bytes[j]);
    refused[j] = ticket < 0;
    if (ticket < 0) continue;
    if (abandon[j]) {
      adm.abandon(ticket);
      continue;
    }
    th.emplace_back([&, j, ticket]() {
      // the rank is taken inside the admission's critical section: two jobs admitted back to
      // back may reach the lock below in either order
      const int64_t rank = adm.admit(ticket, (size_t)bytes[j]);
      {
        std::lock_guard<std::mutex> lk(mu);
        start_order[j] = (int)rank;
        running++;
        used += bytes[j];
        if (running > *peak_running) *peak_running = running;
        if (used > *peak_bytes) *peak_bytes = used;
      }
      std::this_thread::sleep_for(std::chrono::milliseconds(sleep_ms));
      {
        std::lock_guard<std::mutex> lk(mu);
        running--;
        used -= bytes[j];
      }
      adm.release((size_t)bytes[j]);
    });
  }
  for (auto& t : th) t.join();
  const ss::JobAdmission::Stats s = adm.stats();
  *stat_peak_running = s.peak_running;
  *stat_peak_bytes = (long long)s.peak_used;
  return s.running == 0 && s.queued == 0 ? 0 : 1;
}

}  // extern "C"

#ifdef SS_ADMISSION_MAIN
// standalone run of the scenarios for the thread-sanitizer build: exit status 0 when every
// scenario drained its queue
int main() {
  const long long b6[6] = {100, 100, 100, 100, 100, 100};
  const int none[6] = {0, 0, 0, 0, 0, 0}, ab[6] = {0, 1, 0, 0, 0, 0};
  int order[6], refused[6], pr, spr;
  long long pb, spb;
  int rc = 0;
  rc |= ss_host_admission_run(6, b6, none, 0, 2, 5, order, refused, &pr, &pb, &spr, &spb);
  rc |= ss_host_admission_run(6, b6, none, 250, 0, 5, order, refused, &pr, &pb, &spr, &spb);
  rc |= ss_host_admission_run(6, b6, ab, 0, 1, 5, order, refused, &pr, &pb, &spr, &spb);
  rc |= ss_host_admission_run(6, b6, none, 0, 0, 5, order, refused, &pr, &pb, &spr, &spb);
  return rc;
}
#endif
