// jobs.cu -- asynchronous two-electron jobs (ss_job_submit / ss_job_poll / ss_job_result).
//
// The reference runs one job per process (src/two_e_slater.F90:219-564) and has no job API; a
// serving caller wants to hand several jobs to one GPU and collect them later.  A submitted job
// copies the context's basis and quartet list at submit time, then runs on a worker thread with
// a private context (its own stream and device buffers) on the same device, so jobs of one
// context overlap each other and later changes to the submitting context do not affect them.
// Results are kept in host memory until ss_job_result collects them.  Jobs are admitted in
// submission order by their ERI-buffer footprint and a concurrency limit (ss_job_limits,
// admission.h): a worker thread waits for its turn before it creates its context.
#include <string.h>

#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

struct JobState {
  std::thread th;
  std::atomic<int> done{0};
  int rc = SS_OK;
  std::string err;
  std::vector<double> eri, sigma;
};

// wait for every job of a context that is being destroyed (results are dropped)
void jobs_shutdown(ss_ctx* c) {
  for (auto& kv : c->jobs)
    if (kv.second->th.joinable()) kv.second->th.join();
  c->jobs.clear();
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_job_submit(ss_ctx* c, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks, int estimator,
                  int precision, double sigma_target, int64_t* job_id) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  if (!job_id) {
    ss_set_error_msg("ss_job_submit: job_id is NULL");
    return SS_ERR_ARG;
  }
  if (!c->n || !c->nint) {
    ss_set_error_msg("ss_job_submit needs ss_basis_set and ss_quartets_set first");
    return SS_ERR_STATE;
  }
  if (!c->admission) c->admission = std::make_shared<JobAdmission>();
  const size_t foot = JOB_BYTES_PER_QUARTET * (size_t)c->nint;
  const int64_t ticket = c->admission->enqueue(foot);
  if (ticket < 0) {
    ss_set_error_msg("ss_job_submit: the job's ERI buffers (%zu bytes) exceed the job budget", foot);
    return SS_ERR_NOMEM;
  }
  std::shared_ptr<JobAdmission> adm = c->admission;
  auto js = std::make_shared<JobState>();
  js->eri.assign(c->nint, 0.0);
  js->sigma.assign(c->nint, 0.0);
  // inputs copied now (the caller may change or free its arrays and the context afterwards)
  const int device = c->device, n = c->n, ld = c->ld;
  const size_t budget = c->budget;
  std::vector<double> center = c->h_center, cg = c->h_cg, gg = c->h_gg, gs = c->h_gs;
  std::vector<int> npower = c->h_npower, nsto = c->h_nsto, itype = c->h_itype, ng = c->h_ng;
  std::vector<int32_t> is = c->h_is, jsv = c->h_js, ks = c->h_ks, ls = c->h_ls;
  const int64_t nint = c->nint;
  const bool exact_mono = c->exact_monocenter;
  const double eps_screen = c->eri_eps_screen, eps32 = c->eri_eps32;
  JobState* st = js.get();
  try {
    js->th = std::thread([=]() {
      adm->admit(ticket, foot);
      ss_ctx* w = ss_create(device, budget);
      int rc = w ? SS_OK : SS_ERR_CUDA;
      if (!rc)
        rc = ss_basis_set(w, n, center.data(), npower.data(), nsto.data(), itype.data(), ng.data(), cg.data(), ld,
                          gg.data(), gs.data());
      if (!rc) rc = ss_quartets_set(w, nint, is.data(), jsv.data(), ks.data(), ls.data());
      if (!rc) rc = ss_set_exact_monocenter(w, exact_mono ? 1 : 0);
      if (!rc) rc = ss_set_eri_tiers(w, eps_screen, eps32);
      if (!rc)
        rc = ss_two_e_job(w, a_zv, seed, samples_per_block, nblocks, estimator, precision, sigma_target,
                          st->eri.data(), st->sigma.data());
      if (rc) {
        const char* m = ss_last_error();
        st->err = m ? m : "";
      }
      st->rc = rc;
      if (w) ss_destroy(w);
      adm->release(foot);
      st->done.store(1);
    });
  } catch (const std::exception& ex) {
    adm->abandon(ticket);
    ss_set_error_msg("ss_job_submit: cannot start a worker thread (%s)", ex.what());
    return SS_ERR_STATE;
  }
  const int64_t id = c->next_job++;
  c->jobs[id] = js;
  *job_id = id;
  return SS_OK;
}

int ss_job_poll(ss_ctx* c, int64_t job_id, int* done) {
  if (!c || !done) {
    ss_set_error_msg("ss_job_poll: null argument");
    return SS_ERR_ARG;
  }
  auto it = c->jobs.find(job_id);
  if (it == c->jobs.end()) {
    ss_set_error_msg("ss_job_poll: unknown job %lld", (long long)job_id);
    return SS_ERR_ARG;
  }
  *done = it->second->done.load();
  return SS_OK;
}

int ss_job_result(ss_ctx* c, int64_t job_id, double* eri, double* sigma) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  auto it = c->jobs.find(job_id);
  if (it == c->jobs.end()) {
    ss_set_error_msg("ss_job_result: unknown job %lld", (long long)job_id);
    return SS_ERR_ARG;
  }
  std::shared_ptr<JobState> js = it->second;
  if (js->th.joinable()) js->th.join();
  c->jobs.erase(it);
  if (js->rc) {
    ss_set_error_msg("job %lld: %s", (long long)job_id, js->err.c_str());
    return js->rc;
  }
  const size_t bytes = sizeof(double) * js->eri.size();
  if (eri) memcpy(eri, js->eri.data(), bytes);
  if (sigma) memcpy(sigma, js->sigma.data(), bytes);
  return SS_OK;
}

int ss_job_limits(ss_ctx* c, size_t eri_budget_bytes, int max_running) {
  if (!c || max_running < 0) {
    ss_set_error_msg("ss_job_limits: bad arguments");
    return SS_ERR_ARG;
  }
  if (!c->admission) c->admission = std::make_shared<JobAdmission>();
  c->admission->set_limits(eri_budget_bytes, max_running);
  return SS_OK;
}

int ss_job_stats(ss_ctx* c, int* running, int* queued, int* peak_running, size_t* peak_bytes) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  JobAdmission::Stats s;
  if (c->admission) s = c->admission->stats();
  if (running) *running = s.running;
  if (queued) *queued = s.queued;
  if (peak_running) *peak_running = s.peak_running;
  if (peak_bytes) *peak_bytes = s.peak_used;
  return SS_OK;
}

size_t ss_job_footprint(int64_t nint) { return nint > 0 ? JOB_BYTES_PER_QUARTET * (size_t)nint : 0; }

}  // extern "C"
