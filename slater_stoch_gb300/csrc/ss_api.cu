// ss_api.cu -- context, basis/quartet setup and the analytic-ERI entry points of the C ABI.
#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {
cudaError_t eri_init_constants();
void eri_tile(int LK, bool t2, int max_cnt, int* ktile, size_t* smem);
cudaError_t launch_eri_class(int L, int LK, int tc, dim3 grid, int ktile, size_t smem, cudaStream_t st,
                             const BasisDev& B, const PrimPair* pp, const int64_t* off, const int* cnt,
                             const int64_t* work, int split, const int32_t* is, const int32_t* js,
                             const int32_t* ks, const int32_t* ls, const double* pre, double eps,
                             double eps32, double* partial, double* self_out, const PrimPairF* ppf);
__global__ void prim_pair_to_f32(int64_t npp, const PrimPair* in, PrimPairF* out);
__global__ void prim_pair_sort(const PrimPair* in, const int64_t* off, const int* cnt, PrimPair* out);
__global__ void prim_pair_count(BasisDev B, int npairs, int* cnt);
void jobs_shutdown(ss_ctx* c);
__global__ void prim_pair_fill(BasisDev B, int npairs, const int64_t* off, PrimPair* out);
__global__ void eri_finalize(int64_t nint, const int32_t* is, const int32_t* js, const int32_t* ks,
                             const int32_t* ls, const int64_t* slot, const double* partial,
                             const double* pre, int n, double* out);
}  // namespace ss

static thread_local std::string g_err;

void ss_set_error_msg(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
}

void ss_set_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  ss_set_error_msg("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e),
                   what, file, line);
}

#define SS_CHECK_CTX(c)                                \
  do {                                                 \
    if (!(c)) {                                        \
      ss_set_error_msg("null ss_ctx");                 \
      return SS_ERR_ARG;                               \
    }                                                  \
    cudaError_t _se = cudaSetDevice((c)->device);      \
    if (_se != cudaSuccess) {                          \
      ss_set_cuda_error(_se, "cudaSetDevice", __FILE__, __LINE__); \
      return SS_ERR_CUDA;                              \
    }                                                  \
  } while (0)

namespace ss {

int dev_alloc(ss_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.ptr && b.bytes >= bytes) return SS_OK;
  size_t old = b.bytes;
  if (c->budget && c->used - old + bytes > c->budget) {
    ss_set_error_msg("device allocation of %zu bytes exceeds the context HBM budget (%zu of %zu used)",
                     bytes, c->used, c->budget);
    return SS_ERR_NOMEM;
  }
  if (b.ptr) {
    cudaFree(b.ptr);
    c->used -= old;
    b.ptr = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    ss_set_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
    return SS_ERR_NOMEM;
  }
  b.bytes = bytes;
  c->used += bytes;
  return SS_OK;
}

void dev_free(ss_ctx* c, DevBuf& b) {
  if (b.ptr) {
    cudaFree(b.ptr);
    c->used -= b.bytes;
  }
  b.ptr = nullptr;
  b.bytes = 0;
}

int h2d(ss_ctx* c, DevBuf& b, const void* src, size_t bytes) {
  int rc = dev_alloc(c, b, bytes);
  if (rc) return rc;
  SS_CUDA_TRY(cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, c->stream));
  return SS_OK;
}

int h2d_async(ss_ctx* c, DevBuf& b, const void* src, size_t bytes) {
  int rc = dev_alloc(c, b, bytes);
  if (rc) return rc;
  if (!c->pin_evt) SS_CUDA_TRY(cudaEventCreateWithFlags(&c->pin_evt, cudaEventDisableTiming));
  SS_CUDA_TRY(cudaEventSynchronize(c->pin_evt));  // the previous copy has left the buffer
  if (c->pin_cap < bytes) {
    if (c->pin) SS_CUDA_TRY(cudaFreeHost(c->pin));
    c->pin = nullptr;
    c->pin_cap = 0;
    SS_CUDA_TRY(cudaHostAlloc(&c->pin, bytes, cudaHostAllocDefault));
    c->pin_cap = bytes;
  }
  memcpy(c->pin, src, bytes);
  SS_CUDA_TRY(cudaMemcpyAsync(b.ptr, c->pin, bytes, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaEventRecord(c->pin_evt, c->stream));
  return SS_OK;
}

// per-axis maximum of (power of f1 + power of f2) over the cartesian components of the fits
static int pair_L(const ss_ctx* c, int f1, int f2) {
  int L = 0;
  for (int ax = 0; ax < 3; ax++) {
    int a = c->h_npower[3 * f1 + ax] + (c->h_itype[f1] == 2 ? 2 : 0);
    int b = c->h_npower[3 * f2 + ax] + (c->h_itype[f2] == 2 ? 2 : 0);
    L = std::max(L, a + b);
  }
  return L;
}

// Run the ERI kernels for the quartets listed in (qis..qls) restricted to `sel` (indices into
// them); partial sums are written to d_scratch_b and slot[q] gives the partial row of q.
static int run_eri(ss_ctx* c, const int32_t* d_qis, const int32_t* d_qjs, const int32_t* d_qks,
                   const int32_t* d_qls, const std::vector<int32_t>& qis, const std::vector<int32_t>& qjs,
                   const std::vector<int32_t>& qks, const std::vector<int32_t>& qls,
                   const std::vector<int64_t>& sel, std::vector<int64_t>& slot_of_sel, int64_t& npartial,
                   const double* d_pre, double eps, double eps32, double* self_out = nullptr) {
  // bucket by class (L = max(bra L, ket L), tc = number of r^2-type fits among the four
  // functions) and the ket bound of the light-ket rule (ss_light_ket): v = LK + 1, or 0 for the
  // full-L instance.  A light-ket quartet is evaluated as (jl|ik) when (j,l) is the lighter pair
  // (bit 62 of its work entry).  Bucket index 4 (5 L + tc) + v.
  const int NB = 4 * 5 * (SS_MAX_POW + 1);
  const int64_t SWAP = int64_t(1) << 62;
  std::vector<std::vector<int64_t>> bucket(NB);
  for (int64_t t : sel) {
    int i = qis[t] - 1, k = qks[t] - 1, j = qjs[t] - 1, l = qls[t] - 1;
    const int Lb = pair_L(c, i, k), Lk = pair_L(c, j, l);
    int L = std::max(Lb, Lk);
    int nt = (c->h_itype[i] == 2) + (c->h_itype[k] == 2) + (c->h_itype[j] == 2) + (c->h_itype[l] == 2);
    const int v = self_out ? 0 : ss_light_ket(L, std::min(Lb, Lk)) + 1;
    bucket[4 * (5 * L + nt) + v].push_back(v && Lk > Lb ? (t | SWAP) : t);
  }
  // Each class is split into enough bra slices that its launch has ~8 CTAs per SM (classes
  // with few quartets, such as the Schwarz diagonal's or the four-r^2-fit class, up to 127 ways,
  // the largest split a slot code holds).
  const int64_t target = (int64_t)c->num_sms * 8;
  std::vector<int64_t> work;
  work.reserve(sel.size());
  std::vector<int64_t> begin(NB), count(NB), pbase(NB + 1, 0);
  std::vector<int> maxk(NB, 0), bsplit(NB, 1);
  slot_of_sel.assign(qis.size(), -1);
  for (int bk = 0; bk < NB; bk++) {
    begin[bk] = (int64_t)work.size();
    const int64_t cnt = (int64_t)bucket[bk].size();
    bsplit[bk] = cnt ? (int)std::min<int64_t>((1 << SLOT_SPLIT_BITS) - 1,
                                              std::max<int64_t>(1, (target + cnt - 1) / cnt))
                     : 1;
    int64_t local = 0;
    for (int64_t te : bucket[bk]) {
      const int64_t t = te & (SWAP - 1);
      slot_of_sel[t] = ((pbase[bk] + local * bsplit[bk]) << SLOT_SPLIT_BITS) | bsplit[bk];
      local++;
      work.push_back(te);
      const bool swp = (te & SWAP) != 0;
      const int j = (swp ? qis[t] : qjs[t]) - 1, l = (swp ? qks[t] : qls[t]) - 1;  // the ket pair
      maxk[bk] = std::max(maxk[bk], c->h_pp_cnt[ss_pair_index(j, l)]);
    }
    count[bk] = cnt;
    pbase[bk + 1] = pbase[bk] + cnt * bsplit[bk];
  }
  npartial = pbase[NB];
  int rc = dev_alloc(c, c->d_scratch_b, sizeof(double) * std::max<int64_t>(npartial, 1));
  if (rc) return rc;
  if (work.empty()) return SS_OK;  // e.g. a one-function basis: its only quartet is diagonal
  rc = h2d(c, c->d_scratch_a, work.data(), sizeof(int64_t) * work.size());
  if (rc) return rc;
  const int64_t* d_work = (const int64_t*)c->d_scratch_a.ptr;
  double* d_partial = (double*)c->d_scratch_b.ptr;
  // classes launched round-robin over the side streams, largest launch first; the side streams
  // start after everything queued on the context stream and the context stream waits for all
  if (!c->eri_fork) {
    int lo = 0, hi = 0;  // lowest priority: the MC of a job runs beside the analytic stage
    SS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int s = 0; s < ss_ctx::ERI_STREAMS; s++) {
      SS_CUDA_TRY(cudaStreamCreateWithPriority(&c->eri_stream[s], cudaStreamNonBlocking, lo));
      SS_CUDA_TRY(cudaEventCreateWithFlags(&c->eri_join[s], cudaEventDisableTiming));
    }
    SS_CUDA_TRY(cudaEventCreateWithFlags(&c->eri_fork, cudaEventDisableTiming));
  }
  std::vector<int> order;
  for (int bk = 0; bk < NB; bk++)
    if (count[bk]) order.push_back(bk);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return count[a] * bsplit[a] > count[b] * bsplit[b]; });
  SS_CUDA_TRY(cudaEventRecord(c->eri_fork, c->stream));
  for (int s = 0; s < ss_ctx::ERI_STREAMS; s++) SS_CUDA_TRY(cudaStreamWaitEvent(c->eri_stream[s], c->eri_fork, 0));
  int launch_rc = SS_OK;
  for (size_t oi = 0; oi < order.size() && !launch_rc; oi++) {
    const int bk = order[oi];
    cudaStream_t st = c->eri_stream[oi % ss_ctx::ERI_STREAMS];
    const int L = (bk / 4) / 5;
    const int tc = (bk / 4) % 5;
    const int LK = (bk % 4) ? bk % 4 - 1 : L;
    const bool t2 = tc > 0;
    int ktile;
    size_t smem;
    eri_tile(LK, t2, std::max(maxk[bk], 1), &ktile, &smem);
    // grid.x is limited to 2^31-1: launch in chunks of quartets
    const int split = bsplit[bk];
    const int64_t chunk = (int64_t)(2147483647 / split);
    for (int64_t s0 = 0; s0 < count[bk]; s0 += chunk) {
      int64_t nq = std::min(chunk, count[bk] - s0);
      dim3 grid((unsigned)(nq * split));
      cudaError_t e = launch_eri_class(L, LK, tc, grid, ktile, smem, st, c->basis,
                                       (const PrimPair*)c->d_pp.ptr, (const int64_t*)c->d_pp_off.ptr,
                                       (const int*)c->d_pp_cnt.ptr, d_work + begin[bk] + s0, split, d_qis,
                                       d_qjs, d_qks, d_qls, d_pre, eps, eps32, d_partial + pbase[bk] + s0 * split,
                                       self_out, (const PrimPairF*)c->d_ppf.ptr);
      if (e != cudaSuccess) {
        ss_set_cuda_error(e, "eri_kernel launch", __FILE__, __LINE__);
        launch_rc = SS_ERR_CUDA;
        break;
      }
      c->launches++;
    }
  }
  for (int s = 0; s < ss_ctx::ERI_STREAMS; s++) {
    SS_CUDA_TRY(cudaEventRecord(c->eri_join[s], c->eri_stream[s]));
    SS_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->eri_join[s], 0));
  }
  return launch_rc;
}

int build_pair_tables(ss_ctx* c);

int pool_get(ss_ctx* c, const char* name, size_t bytes, void** out) {
  DevBuf& b = c->pool[name];
  int rc = dev_alloc(c, b, bytes);
  if (rc) return rc;
  *out = b.ptr;
  return SS_OK;
}

#define TRY(x)           \
  do {                   \
    int rc_ = (x);       \
    if (rc_) return rc_; \
  } while (0)

// Sort the primitive pairs of every function pair by decreasing Schwarz factor (the order the
// primitive screening of the ERI kernel relies on).
static int sort_prim_pairs(ss_ctx* c) {
  const int npairs = c->n * (c->n + 1) / 2;
  const size_t bytes = sizeof(PrimPair) * std::max<int64_t>(c->h_pp_off[npairs], 1);
  void* p;
  TRY(pool_get(c, "pp_sorted", bytes, &p));
  prim_pair_sort<<<npairs, 512, 0, c->stream>>>((const PrimPair*)c->d_pp.ptr, (const int64_t*)c->d_pp_off.ptr,
                                                 (const int*)c->d_pp_cnt.ptr, (PrimPair*)p);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  SS_CUDA_TRY(cudaMemcpyAsync(c->d_pp.ptr, p, bytes, cudaMemcpyDeviceToDevice, c->stream));
  // FP32 copies in the same order
  const int64_t npp = std::max<int64_t>(c->h_pp_off[npairs], 1);
  TRY(dev_alloc(c, c->d_ppf, sizeof(PrimPairF) * npp));
  prim_pair_to_f32<<<(unsigned)((npp + 255) / 256), 256, 0, c->stream>>>(npp, (const PrimPair*)c->d_pp.ptr,
                                                                          (PrimPairF*)c->d_ppf.ptr);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  return SS_OK;
}

int ensure_precond(ss_ctx* c) {
  if (c->have_precond) return SS_OK;
  if (!c->n) {
    ss_set_error_msg("no basis set");
    return SS_ERR_STATE;
  }
  // diagonal quartets (ik|ik), i >= k, in pair-index order (src/two_e_slater.F90:230-236)
  int n = c->n;
  int64_t np = (int64_t)n * (n + 1) / 2;
  std::vector<int32_t> qi(np), qk(np);
  for (int i = 0; i < n; i++)
    for (int k = 0; k <= i; k++) {
      int64_t p = ss_pair_index(i, k);
      qi[p] = i + 1;
      qk[p] = k + 1;
    }
  DevBuf di, dk;
  int rc = h2d(c, di, qi.data(), sizeof(int32_t) * np);
  if (!rc) rc = h2d(c, dk, qk.data(), sizeof(int32_t) * np);
  // a pair without primitive pairs (all screened, or functions of two systems) has (ik|ik) = 0
  std::vector<int64_t> sel, slot;
  sel.reserve(np);
  for (int64_t p = 0; p < np; p++)
    if (c->h_pp_cnt[p] > 0) sel.push_back(p);
  int64_t npartial = 0;
  // 1. primitive-pair Schwarz factors (items (P,P) of the diagonal quartets) into pad[0],
  // 2. per-pair sort by decreasing factor, 3. the diagonal quartets themselves
  if (!rc)
    rc = run_eri(c, (const int32_t*)di.ptr, (const int32_t*)di.ptr, (const int32_t*)dk.ptr,
                 (const int32_t*)dk.ptr, qi, qi, qk, qk, sel, slot, npartial, nullptr, 0.0, 0.0,
                 (double*)((char*)c->d_pp.ptr + offsetof(PrimPair, pad)));
  if (!rc) rc = sort_prim_pairs(c);
  if (!rc)
    rc = run_eri(c, (const int32_t*)di.ptr, (const int32_t*)di.ptr, (const int32_t*)dk.ptr,
                 (const int32_t*)dk.ptr, qi, qi, qk, qk, sel, slot, npartial, nullptr, 0.0, 0.0);
  if (rc) {
    dev_free(c, di);
    dev_free(c, dk);
    return rc;
  }
  // slots are a permutation of pair indices: gather partials back into pair order on the host side
  // by re-sorting (cheap: np entries)
  std::vector<double> part((size_t)std::max<int64_t>(npartial, 1));
  rc = dev_alloc(c, c->d_precond, sizeof(double) * n * n);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(part.data(), c->d_scratch_b.ptr, sizeof(double) * part.size(),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  dev_free(c, di);
  dev_free(c, dk);
  if (e != cudaSuccess) {
    ss_set_cuda_error(e, "precond copy", __FILE__, __LINE__);
    return SS_ERR_CUDA;
  }
  c->h_precond.assign((size_t)n * n, 0.0);
  for (int64_t p = 0; p < np; p++) {
    double v = 0.0;
    if (slot[p] >= 0)
      for (int t = 0; t < slot_split(slot[p]); t++) v = v + part[slot_offset(slot[p]) + t];
    int i = qi[p] - 1, k = qk[p] - 1;
    c->h_precond[i + (size_t)n * k] = v;
    c->h_precond[k + (size_t)n * i] = v;
  }
  SS_CUDA_TRY(cudaMemcpyAsync(c->d_precond.ptr, c->h_precond.data(), sizeof(double) * n * n,
                              cudaMemcpyHostToDevice, c->stream));
  c->have_precond = true;
  return SS_OK;
}

int ensure_gauss(ss_ctx* c) {
  if (c->have_gauss) return SS_OK;
  if (!c->nint) {
    ss_set_error_msg("no quartets set");
    return SS_ERR_STATE;
  }
  int rc = ensure_precond(c);
  if (rc) return rc;
  const int n = c->n;
  const double seuil = 1.e-15;  // src/two_e_slater.F90:13
  std::vector<int64_t> sel;
  sel.reserve(c->nint);
  int64_t nzero = 0;
  for (int64_t q = 0; q < c->nint; q++) {
    int i = c->h_is[q] - 1, k = c->h_ks[q] - 1, j = c->h_js[q] - 1, l = c->h_ls[q] - 1;
    double pik = c->h_precond[i + (size_t)n * k], pjl = c->h_precond[j + (size_t)n * l];
    bool small = fabs(pik * pjl) < seuil * seuil;
    if (small) nzero++;
    if (i == j && k == l) continue;
    if (!small) sel.push_back(q);
  }
  c->n_removed = nzero;
  std::vector<int64_t> slot;
  int64_t npartial = 0;
  rc = run_eri(c, (const int32_t*)c->d_is.ptr, (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
               (const int32_t*)c->d_ls.ptr, c->h_is, c->h_js, c->h_ks, c->h_ls, sel, slot, npartial,
               (const double*)c->d_precond.ptr, c->eri_eps_screen, c->eri_eps32);
  if (rc) return rc;
  rc = h2d_async(c, c->d_scratch_c, slot.data(), sizeof(int64_t) * c->nint);
  if (rc) return rc;
  rc = dev_alloc(c, c->d_gauss, sizeof(double) * c->nint);
  if (rc) return rc;
  int64_t nb = (c->nint + 255) / 256;
  eri_finalize<<<(unsigned)nb, 256, 0, c->stream>>>(
      c->nint, (const int32_t*)c->d_is.ptr, (const int32_t*)c->d_js.ptr, (const int32_t*)c->d_ks.ptr,
      (const int32_t*)c->d_ls.ptr, (const int64_t*)c->d_scratch_c.ptr,
      (const double*)c->d_scratch_b.ptr, (const double*)c->d_precond.ptr, n, (double*)c->d_gauss.ptr);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  c->have_gauss = true;
  return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

const char* ss_strerror(int code) {
  switch (code) {
    case SS_OK: return "ok";
    case SS_ERR_ARG: return "invalid argument";
    case SS_ERR_STATE: return "call out of order";
    case SS_ERR_CUDA: return "CUDA runtime error";
    case SS_ERR_NOMEM: return "out of device memory or over the HBM budget";
    case SS_ERR_UNSUPPORTED: return "input outside the kernels' limits";
    case SS_ERR_TIMEOUT: return "bounded device wait timed out";
    case SS_ERR_NUMERIC: return "non-finite result";
    default: return "unknown error";
  }
}

const char* ss_last_error(void) { return g_err.c_str(); }

int ss_set_eri_tiers(ss_ctx* c, double screen_eps, double fp32_eps) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  // the screen's skipped part of an ERI is below 900^2 * screen_eps of its Schwarz bound, so
  // 1e-18 keeps it under 1e-12; the FP32 tier's error grows ~linearly with fp32_eps (measured
  // sums of |FP32 - FP64| over a quartet's tier: 1.6e-17 at 1e-13, 1.8e-15 at 1e-11, 1.8e-14
  // at 1e-10 of the Schwarz bound at 20-Gaussian fits)
  if (!(screen_eps >= 0.0 && screen_eps <= 1e-18) || !(fp32_eps >= 0.0 && fp32_eps <= 1e-10)) {
    ss_set_error_msg("ss_set_eri_tiers: need 0 <= screen_eps <= 1e-18 and 0 <= fp32_eps <= 1e-10 (got %g, %g)",
                     screen_eps, fp32_eps);
    return SS_ERR_ARG;
  }
  if (c->eri_eps_screen != screen_eps || c->eri_eps32 != fp32_eps) c->have_gauss = false;
  c->eri_eps_screen = screen_eps;
  c->eri_eps32 = fp32_eps;
  return SS_OK;
}

ss_ctx* ss_create(int device, size_t hbm_budget) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) {
    ss_set_cuda_error(e, "cudaGetDeviceCount", __FILE__, __LINE__);
    return nullptr;
  }
  if (device < 0 || device >= ndev) {
    ss_set_error_msg("device %d out of range (%d devices)", device, ndev);
    return nullptr;
  }
  e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    ss_set_cuda_error(e, "cudaSetDevice", __FILE__, __LINE__);
    return nullptr;
  }
  ss_ctx* c = new ss_ctx();
  c->device = device;
  c->budget = hbm_budget;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (c->num_sms <= 0) c->num_sms = 152;
  {  // the context stream has the greatest priority: in ss_two_e_job the MC kernels queued on it
     // take SM slots as the analytic stage's (lowest-priority) CTAs retire
    int lo = 0, hi = 0;
    e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, hi);
  }
  if (e != cudaSuccess) {
    ss_set_cuda_error(e, "cudaStreamCreate", __FILE__, __LINE__);
    delete c;
    return nullptr;
  }
  return c;
}

void ss_destroy(ss_ctx* c) {
  if (!c) return;
  jobs_shutdown(c);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->ana_stream) cudaStreamSynchronize(c->ana_stream);
  DevBuf* bufs[] = {&c->d_center, &c->d_npower, &c->d_nsto, &c->d_itype, &c->d_ng, &c->d_cg, &c->d_gg,
                    &c->d_gs, &c->d_pp, &c->d_ppf, &c->d_pp_off, &c->d_pp_cnt, &c->d_is, &c->d_js, &c->d_ks,
                    &c->d_ls, &c->d_precond, &c->d_gauss, &c->d_mean, &c->d_sigma, &c->d_scratch_a,
                    &c->d_scratch_b, &c->d_scratch_c, &c->d_scratch_d, &c->d_mono_val, &c->d_mono_mask,
                    &c->d_mono_status, &c->d_sys};
  for (DevBuf* b : bufs) dev_free(c, *b);
  for (auto& kv : c->pool) dev_free(c, kv.second);
  for (int s = 0; s < ss_ctx::ERI_STREAMS; s++) {
    if (c->eri_stream[s]) cudaStreamDestroy(c->eri_stream[s]);
    if (c->eri_join[s]) cudaEventDestroy(c->eri_join[s]);
  }
  if (c->eri_fork) cudaEventDestroy(c->eri_fork);
  if (c->ana_stream) cudaStreamDestroy(c->ana_stream);
  if (c->ana_fork) cudaEventDestroy(c->ana_fork);
  if (c->ana_done) cudaEventDestroy(c->ana_done);
  if (c->pin_evt) {
    cudaEventSynchronize(c->pin_evt);
    cudaEventDestroy(c->pin_evt);
  }
  if (c->pin) cudaFreeHost(c->pin);
  cudaStreamDestroy(c->stream);
  delete c;
}

int64_t ss_launch_count(const ss_ctx* c) { return c ? c->launches : -1; }

int ss_basis_set(ss_ctx* c, int nbasis, const double* center, const int* npower, const int* n_sto,
                 const int* i_type, const int* n_gauss, const double* c_gauss, int ld,
                 const double* g_gauss, const double* g_slater) {
  SS_CHECK_CTX(c);
  if (nbasis <= 0 || ld <= 0 || !center || !npower || !n_sto || !i_type || !n_gauss || !c_gauss ||
      !g_gauss || !g_slater) {
    ss_set_error_msg("ss_basis_set: bad arguments (nbasis=%d ld=%d)", nbasis, ld);
    return SS_ERR_ARG;
  }
  for (int i = 0; i < nbasis; i++) {
    if (n_gauss[i] < 1 || n_gauss[i] > ld || n_gauss[i] > SS_MAX_NG) {
      ss_set_error_msg("function %d: n_gauss=%d outside 1..min(ld=%d,%d)", i + 1, n_gauss[i], ld, SS_MAX_NG);
      return SS_ERR_ARG;
    }
    if (i_type[i] == 3) {  // the reference stops here too (src/build_c_g_gauss_STO.F90:27)
      ss_set_error_msg("function %d: i_type=3 is not supported", i + 1);
      return SS_ERR_UNSUPPORTED;
    }
    if (i_type[i] != 1 && i_type[i] != 2) {
      ss_set_error_msg("function %d: invalid i_type=%d", i + 1, i_type[i]);
      return SS_ERR_ARG;
    }
    for (int ax = 0; ax < 3; ax++)
      if (npower[3 * i + ax] < 0) {
        ss_set_error_msg("function %d: negative power", i + 1);
        return SS_ERR_ARG;
      }
    if (!(g_slater[i] > 0.0)) {
      ss_set_error_msg("function %d: zeta must be > 0", i + 1);
      return SS_ERR_ARG;
    }
  }
  c->n = nbasis;
  c->ld = ld;
  c->h_center.assign(center, center + 3 * nbasis);
  c->h_npower.assign(npower, npower + 3 * nbasis);
  c->h_nsto.assign(n_sto, n_sto + nbasis);
  c->h_itype.assign(i_type, i_type + nbasis);
  c->h_ng.assign(n_gauss, n_gauss + nbasis);
  c->h_cg.assign(c_gauss, c_gauss + (size_t)ld * nbasis * 2);
  c->h_gg.assign(g_gauss, g_gauss + (size_t)ld * nbasis);
  c->h_gs.assign(g_slater, g_slater + nbasis);
  for (int i = 0; i < nbasis; i++)
    for (int k = 0; k <= i; k++)
      if (pair_L(c, i, k) > SS_MAX_POW) {
        ss_set_error_msg("functions %d,%d: per-axis angular power %d exceeds the kernel limit %d "
                         "(s, p, d and r^2-type s fits are supported)", i + 1, k + 1, pair_L(c, i, k), SS_MAX_POW);
        c->n = 0;
        return SS_ERR_UNSUPPORTED;
      }
  int rc = 0;
  rc |= h2d(c, c->d_center, center, sizeof(double) * 3 * nbasis);
  rc |= h2d(c, c->d_npower, npower, sizeof(int) * 3 * nbasis);
  rc |= h2d(c, c->d_nsto, n_sto, sizeof(int) * nbasis);
  rc |= h2d(c, c->d_itype, i_type, sizeof(int) * nbasis);
  rc |= h2d(c, c->d_ng, n_gauss, sizeof(int) * nbasis);
  rc |= h2d(c, c->d_cg, c_gauss, sizeof(double) * ld * nbasis * 2);
  rc |= h2d(c, c->d_gg, g_gauss, sizeof(double) * ld * nbasis);
  rc |= h2d(c, c->d_gs, g_slater, sizeof(double) * nbasis);
  if (rc) return SS_ERR_NOMEM;
  c->basis = BasisDev{nbasis, ld, (const double*)c->d_center.ptr, (const int*)c->d_npower.ptr,
                      (const int*)c->d_nsto.ptr, (const int*)c->d_itype.ptr, (const int*)c->d_ng.ptr,
                      (const double*)c->d_cg.ptr, (const double*)c->d_gg.ptr, (const double*)c->d_gs.ptr,
                      nullptr};
  c->h_sys.clear();
  return build_pair_tables(c);
}

int ss_basis_systems(ss_ctx* c, int nsys, const int* first) {
  SS_CHECK_CTX(c);
  if (!c->n) {
    ss_set_error_msg("ss_basis_systems needs ss_basis_set first");
    return SS_ERR_STATE;
  }
  if (nsys < 1 || !first || first[0] != 1 || first[nsys] != c->n + 1) {
    ss_set_error_msg("ss_basis_systems: need nsys >= 1 and first[0] = 1, first[nsys] = nbasis + 1");
    return SS_ERR_ARG;
  }
  std::vector<int> sys(c->n);
  for (int s = 0; s < nsys; s++) {
    if (first[s + 1] <= first[s]) {
      ss_set_error_msg("ss_basis_systems: system %d is empty or out of order", s + 1);
      return SS_ERR_ARG;
    }
    for (int f = first[s] - 1; f < first[s + 1] - 1; f++) sys[f] = s;
  }
  int rc = h2d(c, c->d_sys, sys.data(), sizeof(int) * c->n);
  if (rc) return rc;
  c->h_sys = sys;
  c->basis.sys = (const int*)c->d_sys.ptr;
  return build_pair_tables(c);
}

}  // extern "C"

namespace ss {
// Primitive-pair tables of every function pair i >= k (pairs across systems have none)
int build_pair_tables(ss_ctx* c) {
  const int nbasis = c->n;
  int npairs = nbasis * (nbasis + 1) / 2;
  int rc;
  rc = dev_alloc(c, c->d_pp_cnt, sizeof(int) * npairs);
  if (rc) return rc;
  SS_CUDA_TRY(eri_init_constants());
  prim_pair_count<<<npairs, 128, 0, c->stream>>>(c->basis, npairs, (int*)c->d_pp_cnt.ptr);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  c->h_pp_cnt.assign(npairs, 0);
  SS_CUDA_TRY(cudaMemcpyAsync(c->h_pp_cnt.data(), c->d_pp_cnt.ptr, sizeof(int) * npairs,
                              cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->h_pp_off.assign(npairs + 1, 0);
  for (int p = 0; p < npairs; p++) c->h_pp_off[p + 1] = c->h_pp_off[p] + c->h_pp_cnt[p];
  rc = h2d(c, c->d_pp_off, c->h_pp_off.data(), sizeof(int64_t) * (npairs + 1));
  if (rc) return rc;
  rc = dev_alloc(c, c->d_pp, sizeof(PrimPair) * std::max<int64_t>(c->h_pp_off[npairs], 1));
  if (rc) return rc;
  prim_pair_fill<<<npairs, 32, 0, c->stream>>>(c->basis, npairs, (const int64_t*)c->d_pp_off.ptr,
                                               (PrimPair*)c->d_pp.ptr);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  c->have_precond = c->have_gauss = c->have_mc = false;
  c->have_resid = c->have_mono = false;
  return SS_OK;
}
}  // namespace ss

extern "C" {

int ss_quartets_set(ss_ctx* c, int64_t nint, const int32_t* is, const int32_t* js, const int32_t* ks,
                    const int32_t* ls) {
  SS_CHECK_CTX(c);
  if (!c->n) {
    ss_set_error_msg("ss_quartets_set before ss_basis_set");
    return SS_ERR_STATE;
  }
  if (nint < 0 || (nint > 0 && (!is || !js || !ks || !ls))) {
    ss_set_error_msg("ss_quartets_set: bad arguments");
    return SS_ERR_ARG;
  }
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q], j = js[q], k = ks[q], l = ls[q];
    if (i < 1 || j < 1 || k < 1 || l < 1 || i > c->n || j > c->n || k > c->n || l > c->n || i < k || j < l) {
      ss_set_error_msg("quartet %lld: (%d,%d,%d,%d) needs 1 <= k <= i <= n and 1 <= l <= j <= n",
                       (long long)q + 1, i, j, k, l);
      return SS_ERR_ARG;
    }
  }
  c->nint = nint;
  c->h_is.assign(is, is + nint);
  c->h_js.assign(js, js + nint);
  c->h_ks.assign(ks, ks + nint);
  c->h_ls.assign(ls, ls + nint);
  int rc = 0;
  size_t b = sizeof(int32_t) * std::max<int64_t>(nint, 1);
  rc |= h2d(c, c->d_is, is, sizeof(int32_t) * nint);
  rc |= h2d(c, c->d_js, js, sizeof(int32_t) * nint);
  rc |= h2d(c, c->d_ks, ks, sizeof(int32_t) * nint);
  rc |= h2d(c, c->d_ls, ls, sizeof(int32_t) * nint);
  (void)b;
  if (rc) return SS_ERR_NOMEM;
  c->have_gauss = c->have_mc = c->have_mono = false;
  return SS_OK;
}

int ss_precond(ss_ctx* c, double* precond) {
  SS_CHECK_CTX(c);
  int rc = ensure_precond(c);
  if (rc) return rc;
  if (precond) memcpy(precond, c->h_precond.data(), sizeof(double) * c->n * c->n);
  return SS_OK;
}

int ss_gauss_eri(ss_ctx* c, double* out, int64_t* n_removed) {
  SS_CHECK_CTX(c);
  int rc = ensure_gauss(c);
  if (rc) return rc;
  if (out) {
    SS_CUDA_TRY(cudaMemcpyAsync(out, c->d_gauss.ptr, sizeof(double) * c->nint, cudaMemcpyDeviceToHost,
                                c->stream));
  }
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (n_removed) *n_removed = c->n_removed;
  return SS_OK;
}

}  // extern "C"
