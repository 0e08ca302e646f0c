// jobs.cu -- asynchronous two-electron jobs (ss_job_submit / ss_job_poll / ss_job_result).
//
// The reference runs one job per process (src/two_e_slater.F90:219-564) and has no job API; a
// serving caller hands many jobs of uneven size to one GPU and collects them as they finish.
// A submitted job copies its inputs (the context's basis and quartets, or the arrays passed to
// ss_job_submit_inputs) at submit time and runs on its own host thread.  Jobs are admitted in
// submission order by their ERI-buffer footprint and a concurrency limit (ss_job_limits,
// admission.h); an admitted job takes an idle worker context (its own stream and device
// buffers) from the submitting context's pool, or creates one, and returns it when it ends.
// Worker contexts are kept for the next jobs: their buffers only grow, so a steady stream of
// jobs reuses device memory instead of allocating and freeing it (cudaFree waits for the whole
// device, which would serialise the jobs that run beside it).  Jobs on different workers
// overlap on the GPU; each stops at its block boundary once its largest error bar reaches its
// sigma target.  Results stay in host memory until ss_job_result collects them.
#include <string.h>

#include <atomic>
#include <chrono>
#include <memory>
#include <mutex>
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
  double wait_s = 0.0, run_s = 0.0, max_sigma = 0.0;  // admission wait, run time, achieved error
  int blocks = 0;                                     // MC blocks the job used
};

// Idle worker contexts of one submitting context (one device, one HBM budget).
struct WorkerPool {
  std::mutex mu;
  std::vector<ss_ctx*> idle;
  int device = 0;
  size_t budget = 0;

  ss_ctx* take() {
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!idle.empty()) {
        ss_ctx* w = idle.back();
        idle.pop_back();
        return w;
      }
    }
    return ss_create(device, budget);
  }
  void give(ss_ctx* w) {
    std::lock_guard<std::mutex> lk(mu);
    idle.push_back(w);
  }
  ~WorkerPool() {
    for (ss_ctx* w : idle) ss_destroy(w);
  }
};

// Everything a job needs, copied at submission.
struct JobInputs {
  int n = 0, ld = 0;
  std::vector<double> center, cg, gg, gs;
  std::vector<int> npower, nsto, itype, ng;
  std::vector<int32_t> is, js, ks, ls;
  int64_t nint = 0;
  bool exact_mono = false;
  double eps_screen = PRIM_SCREEN_EPS, eps32 = PRIM_FP32_EPS;
};

// wait for every job of a context that is being destroyed (results are dropped), then release
// the idle worker contexts
void jobs_shutdown(ss_ctx* c) {
  for (auto& kv : c->jobs)
    if (kv.second->th.joinable()) kv.second->th.join();
  c->jobs.clear();
  c->job_pool.reset();
}

static int submit(ss_ctx* c, std::shared_ptr<JobInputs> in, double a_zv, uint64_t seed, int64_t samples_per_block,
                  int nblocks, int estimator, int precision, double sigma_target, int64_t* job_id) {
  if (!c->admission) c->admission = std::make_shared<JobAdmission>();
  if (!c->job_pool) {
    c->job_pool = std::make_shared<WorkerPool>();
    c->job_pool->device = c->device;
    c->job_pool->budget = c->budget;
  }
  const size_t foot = JOB_BYTES_PER_QUARTET * (size_t)in->nint;
  const int64_t ticket = c->admission->enqueue(foot);
  if (ticket < 0) {
    ss_set_error_msg("ss_job_submit: the job's ERI buffers (%zu bytes) exceed the job budget", foot);
    return SS_ERR_NOMEM;
  }
  std::shared_ptr<JobAdmission> adm = c->admission;
  std::shared_ptr<WorkerPool> pool = c->job_pool;
  auto js = std::make_shared<JobState>();
  js->eri.assign(in->nint, 0.0);
  js->sigma.assign(in->nint, 0.0);
  JobState* st = js.get();
  const auto t_submit = std::chrono::steady_clock::now();
  try {
    js->th = std::thread([=]() {
      adm->admit(ticket, foot);
      const auto t_admit = std::chrono::steady_clock::now();
      ss_ctx* w = pool->take();
      int rc = w ? SS_OK : SS_ERR_CUDA;
      if (!rc)
        rc = ss_basis_set(w, in->n, in->center.data(), in->npower.data(), in->nsto.data(), in->itype.data(),
                          in->ng.data(), in->cg.data(), in->ld, in->gg.data(), in->gs.data());
      if (!rc) rc = ss_quartets_set(w, in->nint, in->is.data(), in->js.data(), in->ks.data(), in->ls.data());
      if (!rc) rc = ss_set_exact_monocenter(w, in->exact_mono ? 1 : 0);
      if (!rc) rc = ss_set_eri_tiers(w, in->eps_screen, in->eps32);
      if (!rc && (estimator & SS_JOB_MC_ONLY))  // the MC correction and its error bar only
        rc = ss_zvmc(w, a_zv, seed, samples_per_block, nblocks, estimator & ~SS_JOB_MC_ONLY, precision,
                     sigma_target, st->eri.data(), st->sigma.data());
      else if (!rc)
        rc = ss_two_e_job(w, a_zv, seed, samples_per_block, nblocks, estimator, precision, sigma_target,
                          st->eri.data(), st->sigma.data());
      if (rc) {
        const char* m = ss_last_error();
        st->err = m ? m : "";
      }
      if (w) {
        st->blocks = ss_mc_blocks_done(w);
        st->max_sigma = ss_mc_max_sigma(w);
      }
      st->rc = rc;
      const auto t_end = std::chrono::steady_clock::now();
      st->wait_s = std::chrono::duration<double>(t_admit - t_submit).count();
      st->run_s = std::chrono::duration<double>(t_end - t_admit).count();
      if (w) {
        if (rc == SS_OK || rc == SS_ERR_ARG || rc == SS_ERR_STATE || rc == SS_ERR_UNSUPPORTED)
          pool->give(w);  // reusable: its stream and buffers are intact
        else
          ss_destroy(w);  // a CUDA, memory or numeric failure: do not hand this context on
      }
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
  if (!c->h_sys.empty() && c->h_sys.back() > 0) {
    ss_set_error_msg("ss_job_submit: the basis holds several systems; submit each with ss_job_submit_inputs");
    return SS_ERR_STATE;
  }
  auto in = std::make_shared<JobInputs>();
  in->n = c->n;
  in->ld = c->ld;
  in->center = c->h_center;
  in->cg = c->h_cg;
  in->gg = c->h_gg;
  in->gs = c->h_gs;
  in->npower = c->h_npower;
  in->nsto = c->h_nsto;
  in->itype = c->h_itype;
  in->ng = c->h_ng;
  in->is = c->h_is;
  in->js = c->h_js;
  in->ks = c->h_ks;
  in->ls = c->h_ls;
  in->nint = c->nint;
  in->exact_mono = c->exact_monocenter;
  in->eps_screen = c->eri_eps_screen;
  in->eps32 = c->eri_eps32;
  return submit(c, in, a_zv, seed, samples_per_block, nblocks, estimator, precision, sigma_target, job_id);
}

int ss_job_submit_inputs(ss_ctx* c, int nbasis, const double* center, const int* npower, const int* n_sto,
                         const int* i_type, const int* n_gauss, const double* c_gauss, int ld, const double* g_gauss,
                         const double* g_slater, int64_t nint, const int32_t* is, const int32_t* js,
                         const int32_t* ks, const int32_t* ls, double a_zv, uint64_t seed, int64_t samples_per_block,
                         int nblocks, int estimator, int precision, double sigma_target, int64_t* job_id) {
  if (!c || !job_id) {
    ss_set_error_msg("ss_job_submit_inputs: null context or job_id");
    return SS_ERR_ARG;
  }
  if (nbasis < 1 || ld < 1 || nint < 1 || !center || !npower || !n_sto || !i_type || !n_gauss || !c_gauss ||
      !g_gauss || !g_slater || !is || !js || !ks || !ls) {
    ss_set_error_msg("ss_job_submit_inputs: empty basis or quartet list, or a null array");
    return SS_ERR_ARG;
  }
  auto in = std::make_shared<JobInputs>();
  const size_t n = (size_t)nbasis, L = (size_t)ld;
  in->n = nbasis;
  in->ld = ld;
  in->center.assign(center, center + 3 * n);
  in->npower.assign(npower, npower + 3 * n);
  in->nsto.assign(n_sto, n_sto + n);
  in->itype.assign(i_type, i_type + n);
  in->ng.assign(n_gauss, n_gauss + n);
  in->cg.assign(c_gauss, c_gauss + L * n * 2);
  in->gg.assign(g_gauss, g_gauss + L * n);
  in->gs.assign(g_slater, g_slater + n);
  in->is.assign(is, is + nint);
  in->js.assign(js, js + nint);
  in->ks.assign(ks, ks + nint);
  in->ls.assign(ls, ls + nint);
  in->nint = nint;
  in->exact_mono = c->exact_monocenter;
  in->eps_screen = c->eri_eps_screen;
  in->eps32 = c->eri_eps32;
  return submit(c, in, a_zv, seed, samples_per_block, nblocks, estimator, precision, sigma_target, job_id);
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

int ss_job_info(ss_ctx* c, int64_t job_id, double* wait_s, double* run_s, int* blocks, double* max_sigma) {
  if (!c) {
    ss_set_error_msg("null context");
    return SS_ERR_ARG;
  }
  auto it = c->jobs.find(job_id);
  if (it == c->jobs.end()) {
    ss_set_error_msg("ss_job_info: unknown job %lld", (long long)job_id);
    return SS_ERR_ARG;
  }
  JobState* js = it->second.get();
  if (!js->done.load()) {
    ss_set_error_msg("ss_job_info: job %lld has not finished", (long long)job_id);
    return SS_ERR_STATE;
  }
  if (wait_s) *wait_s = js->wait_s;
  if (run_s) *run_s = js->run_s;
  if (blocks) *blocks = js->blocks;
  if (max_sigma) *max_sigma = js->max_sigma;
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
