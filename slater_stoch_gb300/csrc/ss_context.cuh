// ss_context.cuh -- the ss_ctx object behind the C ABI (device-resident job state).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "admission.h"
#include "ss_common.cuh"

namespace ss {

// A device allocation tracked against the context's HBM budget.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct EriPlan {
  // one entry per (class L) bucket; work lists hold quartet indices
  std::vector<int> L;
  std::vector<int64_t> begin, count;  // into work[]
  std::vector<int> split;
  std::vector<int64_t> partial_begin;  // into partial[]
  std::vector<int> max_ket;            // largest ket primitive-pair count in the bucket
  int64_t total_partial = 0;
};

// Parameters of the shared-walker proposal: a mixture of ZV-map densities
// p_c(u) = exp(-|u-G_c|/(2 c_c)) / ((2 pi)^{3/2} 2 c_c^{3/2} |u-G_c|^{3/2}).
struct Mixture {
  int m = 0;
  std::vector<double> G;       // 3*m
  std::vector<double> c;       // m
  std::vector<double> weight;  // m, sums to 1
  std::vector<double> cdf;     // m
};

}  // namespace ss

namespace ss {
struct JobState;    // jobs.cu
struct WorkerPool;  // jobs.cu: idle worker contexts reused by the jobs
}

struct ss_ctx {
  int device = 0;
  size_t budget = 0, used = 0;
  cudaStream_t stream = nullptr;
  // side streams of the analytic stage: the ERI classes are launched across them so that one
  // class's CTAs fill the tail of another's launch (created on first use)
  static constexpr int ERI_STREAMS = 4;
  cudaStream_t eri_stream[ERI_STREAMS] = {};
  cudaEvent_t eri_fork = nullptr, eri_join[ERI_STREAMS] = {};
  // ss_two_e_job queues the analytic stage on ana_stream (ana_fork orders it after the context
  // stream's earlier work, ana_done marks its end) while the MC runs on the context stream
  cudaStream_t ana_stream = nullptr;
  cudaEvent_t ana_fork = nullptr, ana_done = nullptr;
  // pinned staging buffer of h2d_async (pin_evt: the last copy out of it)
  void* pin = nullptr;
  size_t pin_cap = 0;
  cudaEvent_t pin_evt = nullptr;
  int64_t launches = 0;
  int num_sms = 0;

  // basis (device copies)
  int n = 0, ld = 0;
  std::vector<double> h_center, h_gg, h_cg, h_gs;
  std::vector<int> h_npower, h_nsto, h_itype, h_ng;
  ss::DevBuf d_center, d_npower, d_nsto, d_itype, d_ng, d_cg, d_gg, d_gs;
  std::vector<int> h_sys;  // system of each function (ss_basis_systems), empty for one system
  ss::DevBuf d_sys;
  ss::BasisDev basis{};

  // nuclei for the one-electron nuclear attraction (ss_nuclei_set)
  std::vector<double> h_nuc_xyz, h_nuc_charge;

  // primitive pairs
  ss::DevBuf d_pp, d_pp_off, d_pp_cnt;
  ss::DevBuf d_ppf;  // FP32 copies of the sorted primitive pairs (mixed-precision tier)
  std::vector<int> h_pp_cnt;
  std::vector<int64_t> h_pp_off;

  // quartets
  int64_t nint = 0;
  std::vector<int32_t> h_is, h_js, h_ks, h_ls;
  ss::DevBuf d_is, d_js, d_ks, d_ls;

  // analytic results
  bool have_precond = false, have_gauss = false;
  // primitive screening and FP32-tier thresholds of the analytic stage (ss_set_eri_tiers)
  double eri_eps_screen = ss::PRIM_SCREEN_EPS, eri_eps32 = ss::PRIM_FP32_EPS;
  std::vector<double> h_precond;
  ss::DevBuf d_precond, d_gauss;
  int64_t n_removed = 0;

  // exact one-centre Slater ERIs (monocenter.cu)
  bool exact_monocenter = false;  // ss_set_exact_monocenter: used by ss_combine and the jobs
  bool have_mono = false;
  int64_t n_mono = 0;
  ss::DevBuf d_mono_val, d_mono_mask, d_mono_status;

  // MC results
  bool have_mc = false;
  bool have_resid = false;  // shared-walker residual tables of the current basis (pool "rs_*")

  // asynchronous jobs (jobs.cu) and their admission (admission.h)
  std::map<int64_t, std::shared_ptr<ss::JobState>> jobs;
  std::shared_ptr<ss::JobAdmission> admission;
  std::shared_ptr<ss::WorkerPool> job_pool;
  int64_t next_job = 1;
  ss::DevBuf d_mean, d_sigma;

  // scratch reused across calls
  ss::DevBuf d_scratch_a, d_scratch_b, d_scratch_c, d_scratch_d;
  // named device buffers of the MC and cleanup stages
  std::map<std::string, ss::DevBuf> pool;
  int mc_blocks_done = 0;
  double mc_max_sigma = 0.0;
};

namespace ss {
int dev_alloc(ss_ctx* c, DevBuf& b, size_t bytes);   // (re)allocates only when growing
void dev_free(ss_ctx* c, DevBuf& b);
int h2d(ss_ctx* c, DevBuf& b, const void* src, size_t bytes);
// as h2d, through the context's pinned staging buffer, so that the call returns without waiting
// for the stream (a pageable copy waits for the stream's earlier work)
int h2d_async(ss_ctx* c, DevBuf& b, const void* src, size_t bytes);
int ensure_precond(ss_ctx* c);
// named pool buffer of at least `bytes`; *out receives the device pointer
int pool_get(ss_ctx* c, const char* name, size_t bytes, void** out);
int ensure_gauss(ss_ctx* c);
}  // namespace ss
