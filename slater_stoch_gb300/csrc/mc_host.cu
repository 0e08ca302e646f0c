// mc_host.cu -- host orchestration of the ZV-MC entry points (faithful estimator).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "mc.cuh"
#include "shared.cuh"
#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

int ensure_mono(ss_ctx* c);
int launch_combine_mono(ss_ctx* c, double* out);

__global__ void combine_kernel(int64_t nint, const double* __restrict__ g, const double* __restrict__ m,
                               double* __restrict__ out) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < nint) out[q] = m[q] + g[q];  // src/two_e_slater.F90:564
}

// used pairs and the quartet CSR grouped by bra pair
struct PairPlan {
  int npairs = 0, nbra = 0;
  std::vector<int> pidx;  // n*n -> compact pair or -1
  std::vector<int> pi, pk;
  std::vector<int> bra;
  std::vector<int64_t> off, q;
  std::vector<int> ket;
};

static void build_pair_plan(const ss_ctx* c, PairPlan& P) {
  const int n = c->n;
  P.pidx.assign((size_t)n * n, -1);
  P.pi.clear();
  P.pk.clear();
  auto use = [&](int i, int k) {
    int& v = P.pidx[i + (size_t)n * k];
    if (v < 0) {
      v = P.npairs++;
      P.pi.push_back(i);
      P.pk.push_back(k);
    }
    return v;
  };
  std::vector<int> p1(c->nint), p2(c->nint);
  for (int64_t t = 0; t < c->nint; t++) {
    p1[t] = use(c->h_is[t] - 1, c->h_ks[t] - 1);
    p2[t] = use(c->h_js[t] - 1, c->h_ls[t] - 1);
  }
  std::vector<int64_t> cnt(P.npairs + 1, 0);
  for (int64_t t = 0; t < c->nint; t++) cnt[p1[t]]++;
  P.bra.clear();
  P.off.assign(1, 0);
  std::vector<int64_t> start(P.npairs, -1);
  for (int p = 0; p < P.npairs; p++)
    if (cnt[p]) {
      start[p] = P.off.back();
      P.bra.push_back(p);
      P.off.push_back(P.off.back() + cnt[p]);
    }
  P.nbra = (int)P.bra.size();
  P.q.assign(c->nint, 0);
  P.ket.assign(c->nint, 0);
  std::vector<int64_t> fill(start);
  for (int64_t t = 0; t < c->nint; t++) {
    int64_t e = fill[p1[t]]++;
    P.q[e] = t;
    P.ket[e] = p2[t];
  }
}

#define TRY(x)                 \
  do {                         \
    int _rc = (x);             \
    if (_rc) return _rc;       \
  } while (0)
#define CUTRY(x) SS_CUDA_TRY(x)

template <class T>
static int upload(ss_ctx* c, const char* name, const std::vector<T>& v, T** out) {
  void* p;
  TRY(pool_get(c, name, sizeof(T) * std::max<size_t>(v.size(), 1), &p));
  if (!v.empty()) CUTRY(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream));
  *out = (T*)p;
  return SS_OK;
}

// Faithful estimator over blocks; walkers from Philox(seed) or from host arrays hr1/hr2.
static int run_faithful(ss_ctx* c, double a_zv, uint64_t seed, const double* hr1, const double* hr2,
                        int64_t npts, int nblocks, int prec, double sigma_target) {
  if (prec != SS_PREC_FP64 && prec != SS_PREC_REF32) {
    ss_set_error_msg("faithful estimator: precision must be FP64 or REF32");
    return SS_ERR_ARG;
  }
  PairPlan P;
  build_pair_plan(c, P);
  const int np = P.npairs;
  std::vector<double> G(3 * (size_t)np), fzv(np), fjac(np);
  for (int p = 0; p < np; p++) {
    int i = P.pi[p], k = P.pk[p];
    double gi = c->h_gs[i], gk = c->h_gs[k];
    for (int l = 0; l < 3; l++)  // src/two_e_slater.F90:344
      G[3 * p + l] = (gi * c->h_center[l + 3 * i] + gk * c->h_center[l + 3 * k]) / (gi + gk);
    fzv[p] = 0.5 * a_zv / (gi + gk);  // :406
    fjac[p] = a_zv / (gi + gk);       // src/compute_jacobian_and_pi0.F90:22
  }
  ZvPairs dP;
  ZvCsr dQ;
  {
    int *pi, *pk, *bra, *ket;
    double *dG, *dfzv, *dfjac;
    int64_t *off, *q;
    TRY(upload(c, "zv_pi", P.pi, &pi));
    TRY(upload(c, "zv_pk", P.pk, &pk));
    TRY(upload(c, "zv_G", G, &dG));
    TRY(upload(c, "zv_fzv", fzv, &dfzv));
    TRY(upload(c, "zv_fjac", fjac, &dfjac));
    TRY(upload(c, "zv_bra", P.bra, &bra));
    TRY(upload(c, "zv_off", P.off, &off));
    TRY(upload(c, "zv_q", P.q, &q));
    TRY(upload(c, "zv_ket", P.ket, &ket));
    dP = ZvPairs{pi, pk, dG, dfzv, dfjac};
    dQ = ZvCsr{bra, off, q, ket};
  }
  // chunk size: ~1 GiB of pair columns
  const int ncols = (prec == SS_PREC_FP64) ? 10 : 12;
  int64_t Sc = (int64_t)(1.0e9 / (8.0 * ncols * std::max(np, 1)));
  Sc = std::max<int64_t>(1024, std::min<int64_t>(Sc, 1 << 18));
  Sc = std::min<int64_t>(Sc, npts);
  void* buf;
  TRY(pool_get(c, "zv_cols", sizeof(double) * (size_t)ncols * np * Sc, &buf));
  double* cols = (double*)buf;
  ZvChunk Z{};
  Z.ld = Sc;
  double** fields[12] = {&Z.u1x, &Z.u1y, &Z.u1z, &Z.u2x, &Z.u2y, &Z.u2z, &Z.a_s, &Z.a_g, &Z.b_s, &Z.b_g, &Z.j1, &Z.j2};
  for (int f = 0; f < ncols; f++) *fields[f] = cols + (size_t)f * np * Sc;
  double *r1, *r2, *r1m, *r2m, *pi0;
  TRY(pool_get(c, "zv_r1", sizeof(double) * 3 * Sc, &buf)); r1 = (double*)buf;
  TRY(pool_get(c, "zv_r2", sizeof(double) * 3 * Sc, &buf)); r2 = (double*)buf;
  TRY(pool_get(c, "zv_r1m", sizeof(double) * Sc, &buf)); r1m = (double*)buf;
  TRY(pool_get(c, "zv_r2m", sizeof(double) * Sc, &buf)); r2m = (double*)buf;
  TRY(pool_get(c, "zv_pi0", sizeof(double) * Sc, &buf)); pi0 = (double*)buf;
  const int64_t nint = c->nint;
  int nsplit = (int)std::max<int64_t>(1, std::min<int64_t>((4 * c->num_sms + P.nbra - 1) / std::max(P.nbra, 1),
                                                          std::max<int64_t>(1, Sc / 256)));
  double *partS, *partG, *eS, *eG, *acc, *acc2;
  TRY(pool_get(c, "zv_partS", sizeof(double) * nint * nsplit, &buf)); partS = (double*)buf;
  TRY(pool_get(c, "zv_partG", sizeof(double) * nint * nsplit, &buf)); partG = (double*)buf;
  TRY(pool_get(c, "zv_eS", sizeof(double) * nint, &buf)); eS = (double*)buf;
  TRY(pool_get(c, "zv_eG", sizeof(double) * nint, &buf)); eG = (double*)buf;
  TRY(pool_get(c, "zv_acc", sizeof(double) * nint, &buf)); acc = (double*)buf;
  TRY(pool_get(c, "zv_acc2", sizeof(double) * nint, &buf)); acc2 = (double*)buf;
  unsigned long long* maxbits;
  TRY(pool_get(c, "zv_maxbits", sizeof(unsigned long long), &buf)); maxbits = (unsigned long long*)buf;
  CUTRY(cudaMemsetAsync(eS, 0, sizeof(double) * nint, c->stream));
  CUTRY(cudaMemsetAsync(eG, 0, sizeof(double) * nint, c->stream));
  CUTRY(cudaMemsetAsync(acc, 0, sizeof(double) * nint, c->stream));
  CUTRY(cudaMemsetAsync(acc2, 0, sizeof(double) * nint, c->stream));
  TRY(dev_alloc(c, c->d_mean, sizeof(double) * nint));
  TRY(dev_alloc(c, c->d_sigma, sizeof(double) * nint));

  int done = 0;
  for (int b = 0; b < nblocks; b++) {
    for (int64_t c0 = 0; c0 < npts; c0 += Sc) {
      const int64_t ns = std::min(Sc, npts - c0);
      const int64_t first = (int64_t)b * npts + c0;
      if (hr1) {
        CUTRY(cudaMemcpyAsync(r1, hr1 + 3 * first, sizeof(double) * 3 * ns, cudaMemcpyHostToDevice, c->stream));
        CUTRY(cudaMemcpyAsync(r2, hr2 + 3 * first, sizeof(double) * 3 * ns, cudaMemcpyHostToDevice, c->stream));
      } else {
        CUTRY(launch_draw_walkers(c->stream, seed, first, ns, r1, r2));
        c->launches++;
      }
      CUTRY(launch_walker_aux(c->stream, ns, r1, r2, r1m, r2m, pi0));
      CUTRY(launch_zv_pairs(c->stream, prec, c->basis, dP, np, ns, r1, r2, r1m, r2m, pi0, Z));
      CUTRY(launch_zv_accum(c->stream, prec, P.nbra, nsplit, ns, dQ, Z, pi0, partS, partG));
      CUTRY(launch_zv_reduce(c->stream, nint, nsplit, partS, partG, eS, eG));
      c->launches += 4;
    }
    CUTRY(launch_zv_block_stats(c->stream, nint, npts, eS, eG, acc, acc2));
    c->launches++;
    done = b + 1;
    if (sigma_target > 0.0 && done >= 2 && done < nblocks) {
      CUTRY(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), c->stream));
      CUTRY(launch_zv_final(c->stream, nint, done, 0, acc, acc2, (double*)c->d_mean.ptr,
                            (double*)c->d_sigma.ptr, maxbits));
      c->launches++;
      unsigned long long h = 0;
      CUTRY(cudaMemcpyAsync(&h, maxbits, sizeof h, cudaMemcpyDeviceToHost, c->stream));
      CUTRY(cudaStreamSynchronize(c->stream));
      double ms;
      memcpy(&ms, &h, sizeof ms);
      if (ms <= sigma_target) break;
    }
  }
  CUTRY(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), c->stream));
  CUTRY(launch_zv_final(c->stream, nint, done, 0, acc, acc2, (double*)c->d_mean.ptr, (double*)c->d_sigma.ptr,
                        maxbits));
  c->launches++;
  unsigned long long h = 0;
  CUTRY(cudaMemcpyAsync(&h, maxbits, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CUTRY(cudaStreamSynchronize(c->stream));
  memcpy(&c->mc_max_sigma, &h, sizeof(double));
  c->mc_blocks_done = done;
  c->have_mc = true;
  return SS_OK;
}

static int cuda_rc(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SS_OK;
  ss_set_cuda_error(e, what, __FILE__, __LINE__);
  return SS_ERR_CUDA;
}

static int copy_out(ss_ctx* c, double* mean, double* sigma) {
  if (mean)
    CUTRY(cudaMemcpyAsync(mean, c->d_mean.ptr, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, c->stream));
  if (sigma)
    CUTRY(cudaMemcpyAsync(sigma, c->d_sigma.ptr, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, c->stream));
  CUTRY(cudaStreamSynchronize(c->stream));
  return SS_OK;
}

}  // namespace ss

using namespace ss;

#define SS_CTX(c)                                      \
  do {                                                 \
    if (!(c)) {                                        \
      ss_set_error_msg("null ss_ctx");                 \
      return SS_ERR_ARG;                               \
    }                                                  \
    SS_CUDA_TRY(cudaSetDevice((c)->device));           \
    if (!(c)->n || !(c)->nint) {                       \
      ss_set_error_msg("basis and quartets must be set first"); \
      return SS_ERR_STATE;                             \
    }                                                  \
  } while (0)

extern "C" {

int ss_zvmc(ss_ctx* c, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks, int estimator,
            int precision, double sigma_target, double* mean, double* sigma) {
  SS_CTX(c);
  if (samples_per_block <= 0 || nblocks <= 0 || !(a_zv > 0.0)) {
    ss_set_error_msg("ss_zvmc: need samples_per_block > 0, nblocks > 0, a_zv > 0");
    return SS_ERR_ARG;
  }
  if (!c->h_sys.empty() && c->h_sys.back() > 0) {
    ss_set_error_msg("ss_zvmc: the basis holds several systems (ss_basis_systems); run each system's MC as its own job");
    return SS_ERR_STATE;
  }
  int rc;
  if (estimator == SS_EST_FAITHFUL) {
    if (samples_per_block % 40 != 0) {  // src/two_e_slater.F90:148
      ss_set_error_msg("npts_two_elec must be a multiple of nw (40)");
      return SS_ERR_ARG;
    }
    rc = run_faithful(c, a_zv, seed, nullptr, nullptr, samples_per_block, nblocks, precision, sigma_target);
  } else if (estimator == SS_EST_SHARED) {
    rc = run_shared(c, a_zv, seed, samples_per_block, nblocks, precision, sigma_target);
  } else {
    ss_set_error_msg("unknown estimator %d", estimator);
    return SS_ERR_ARG;
  }
  if (rc) return rc;
  return copy_out(c, mean, sigma);
}

int ss_zvmc_walkers(ss_ctx* c, double a_zv, const double* r1, const double* r2, int64_t npts, int nblocks,
                    int precision, double* mean, double* sigma) {
  SS_CTX(c);
  if (!r1 || !r2 || npts <= 0 || nblocks <= 0 || npts % 40 != 0 || !(a_zv > 0.0)) {
    ss_set_error_msg("ss_zvmc_walkers: bad arguments (npts must be a positive multiple of 40)");
    return SS_ERR_ARG;
  }
  int rc = run_faithful(c, a_zv, 0, r1, r2, npts, nblocks, precision, 0.0);
  if (rc) return rc;
  return copy_out(c, mean, sigma);
}

int ss_draw_walkers(ss_ctx* c, uint64_t seed, int64_t first, int64_t S, double* r1, double* r2) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (S <= 0 || first < 0 || !r1 || !r2) {
    ss_set_error_msg("ss_draw_walkers: bad arguments");
    return SS_ERR_ARG;
  }
  void *a, *b;
  TRY(pool_get(c, "draw_r1", sizeof(double) * 3 * S, &a));
  TRY(pool_get(c, "draw_r2", sizeof(double) * 3 * S, &b));
  SS_CUDA_TRY(launch_draw_walkers(c->stream, seed, first, S, (double*)a, (double*)b));
  c->launches++;
  SS_CUDA_TRY(cudaMemcpyAsync(r1, a, sizeof(double) * 3 * S, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(r2, b, sizeof(double) * 3 * S, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SS_OK;
}

int ss_invalidate(ss_ctx* c) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  c->have_precond = c->have_gauss = c->have_mc = c->have_mono = false;
  return SS_OK;
}

double ss_mc_max_sigma(const ss_ctx* c) { return c ? c->mc_max_sigma : -1.0; }
int ss_mc_blocks_done(const ss_ctx* c) { return c ? c->mc_blocks_done : -1; }
void* ss_stream(ss_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ss_two_e_job(ss_ctx* c, double a_zv, uint64_t seed, int64_t samples_per_block, int nblocks, int estimator,
                 int precision, double sigma_target, double* eri, double* sigma) {
  SS_CTX(c);
  c->have_precond = c->have_gauss = c->have_mc = false;
  // The analytic stage and the MC meet only in ss_combine.  The analytic stage is queued on its
  // own lowest-priority stream (ensure_gauss returns once its launches are queued) and the MC
  // runs on the context stream (greatest priority) meanwhile: the MC kernels take SM slots as
  // ERI CTAs retire instead of waiting for the whole stage (measured on the 26-function H2O job:
  // 1.771 s -> 1.740 s; without the priorities the two streams gave no gain).  Results are
  // bitwise the same.  The context stream waits for the analytic stage before the combine.
  if (!c->ana_stream) {
    int lo = 0, hi = 0;
    SS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    SS_CUDA_TRY(cudaStreamCreateWithPriority(&c->ana_stream, cudaStreamNonBlocking, lo));
    SS_CUDA_TRY(cudaEventCreateWithFlags(&c->ana_fork, cudaEventDisableTiming));
    SS_CUDA_TRY(cudaEventCreateWithFlags(&c->ana_done, cudaEventDisableTiming));
  }
  SS_CUDA_TRY(cudaEventRecord(c->ana_fork, c->stream));  // after the basis and quartet uploads
  SS_CUDA_TRY(cudaStreamWaitEvent(c->ana_stream, c->ana_fork, 0));
  cudaStream_t ctx_stream = c->stream;
  c->stream = c->ana_stream;
  int rc = ensure_gauss(c);
  if (!rc) rc = cuda_rc(cudaEventRecord(c->ana_done, c->ana_stream), "cudaEventRecord");
  c->stream = ctx_stream;
  if (rc) {
    cudaStreamSynchronize(c->ana_stream);
    return rc;
  }
  rc = ss_zvmc(c, a_zv, seed, samples_per_block, nblocks, estimator, precision, sigma_target, nullptr, nullptr);
  // the join is queued on every path, so no analytic work outlives the call unobserved
  const int jrc = cuda_rc(cudaStreamWaitEvent(c->stream, c->ana_done, 0), "cudaStreamWaitEvent");
  if (rc || jrc) {
    cudaStreamSynchronize(c->ana_stream);
    return rc ? rc : jrc;
  }
  TRY(ss_combine(c, eri));
  if (sigma) TRY(copy_out(c, nullptr, sigma));
  return SS_OK;
}

int ss_combine(ss_ctx* c, double* out) {
  SS_CTX(c);
  if (!c->have_mc) {
    ss_set_error_msg("ss_combine needs ss_zvmc first");
    return SS_ERR_STATE;
  }
  TRY(ensure_gauss(c));
  void* o;
  TRY(pool_get(c, "combined", sizeof(double) * c->nint, &o));
  if (c->exact_monocenter) {  // src/two_e_slater.F90:558-564 with do_exact_monocenter
    TRY(ensure_mono(c));
    TRY(launch_combine_mono(c, (double*)o));
  } else {
    combine_kernel<<<(unsigned)((c->nint + 255) / 256), 256, 0, c->stream>>>(
        c->nint, (const double*)c->d_gauss.ptr, (const double*)c->d_mean.ptr, (double*)o);
    SS_CUDA_TRY(cudaGetLastError());
    c->launches++;
  }
  if (out) SS_CUDA_TRY(cudaMemcpyAsync(out, o, sizeof(double) * c->nint, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SS_OK;
}

}  // extern "C"
