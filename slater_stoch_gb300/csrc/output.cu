// output.cu -- the reference's bielec_ao text output written by the library
// (src/two_e_slater.F90:603-613: write(104,'(4(I5,X),2D22.15)') i,j,k,l, ijkl(kcp), ijkl2(kcp)).
//
// ss_write_bielec_ao streams the context's merged ERIs and MC errors from the device in chunks
// (one chunk copied while the previous one is formatted); ss_write_bielec_ao_arrays formats
// caller arrays.  Dw.d as gfortran writes it: "0." followed by d significant digits, "D",
// the sign and two exponent digits (three-digit exponents drop the "D"), right-justified in w.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

int pool_get(ss_ctx* c, const char* name, size_t bytes, void** out);

// Fortran D22.15 of x into out (22 characters, no terminator)
static void fortran_d22_15(double x, char* out) {
  char body[40];
  if (x == 0.0) {
    snprintf(body, sizeof body, "0.000000000000000D+00");
  } else if (!std::isfinite(x)) {
    snprintf(body, sizeof body, "%s", std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
  } else {
    char e[40];
    snprintf(e, sizeof e, "%.14E", fabs(x));  // d.dddddddddddddde+XX, 15 significant digits
    char digits[16];
    digits[0] = e[0];
    memcpy(digits + 1, e + 2, 14);
    digits[15] = 0;
    const int e10 = atoi(strchr(e, 'E') + 1) + 1;
    const char sg = e10 >= 0 ? '+' : '-';
    const int ae = e10 >= 0 ? e10 : -e10;
    if (ae > 99)
      snprintf(body, sizeof body, "%s0.%s%c%03d", x < 0 ? "-" : "", digits, sg, ae);
    else
      snprintf(body, sizeof body, "%s0.%sD%c%02d", x < 0 ? "-" : "", digits, sg, ae);
  }
  const int len = (int)strlen(body);
  const int pad = 22 - len;
  for (int t = 0; t < pad; t++) out[t] = ' ';
  memcpy(out + (pad > 0 ? pad : 0), body + (pad < 0 ? -pad : 0), (size_t)(pad < 0 ? 22 : len));
}

// one record: 4(I5,X) then 2D22.15, newline (78 + 1 characters)
static size_t format_record(char* out, int i, int j, int k, int l, double v, double s) {
  int nc = snprintf(out, 32, "%5d %5d %5d %5d ", i, j, k, l);
  fortran_d22_15(v, out + nc);
  fortran_d22_15(s, out + nc + 22);
  out[nc + 44] = '\n';
  return (size_t)nc + 45;
}

static int write_records(FILE* f, int64_t q0, int64_t n, const int32_t* is, const int32_t* js, const int32_t* ks,
                         const int32_t* ls, const double* v, const double* s, std::vector<char>& buf) {
  buf.resize((size_t)n * 96);
  size_t pos = 0;
  for (int64_t t = 0; t < n; t++) {
    const int64_t q = q0 + t;
    pos += format_record(buf.data() + pos, is[q], js[q], ks[q], ls[q], v[t], s ? s[t] : 0.0);
  }
  if (fwrite(buf.data(), 1, pos, f) != pos) {
    ss_set_error_msg("bielec_ao: write failed");
    return SS_ERR_STATE;
  }
  return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_write_bielec_ao_arrays(const char* path, int64_t nint, const int32_t* is, const int32_t* js,
                              const int32_t* ks, const int32_t* ls, const double* eri, const double* sigma) {
  if (!path || nint < 0 || (nint > 0 && (!is || !js || !ks || !ls || !eri))) {
    ss_set_error_msg("ss_write_bielec_ao_arrays: bad arguments");
    return SS_ERR_ARG;
  }
  FILE* f = fopen(path, "w");
  if (!f) {
    ss_set_error_msg("bielec_ao: cannot open %s", path);
    return SS_ERR_ARG;
  }
  std::vector<char> buf;
  int rc = SS_OK;
  const int64_t chunk = 1 << 16;
  for (int64_t q0 = 0; q0 < nint && !rc; q0 += chunk) {
    const int64_t n = std::min(chunk, nint - q0);
    rc = write_records(f, q0, n, is, js, ks, ls, eri + q0, sigma ? sigma + q0 : nullptr, buf);
  }
  if (fclose(f) != 0 && !rc) {
    ss_set_error_msg("bielec_ao: close failed");
    rc = SS_ERR_STATE;
  }
  return rc;
}

// one-electron matrix file of one_e_slater (src/one_e_slater.F90:125-135):
// write(u,'(2(I5,X),D22.15)') i,k,M(i,k) for i = 1..n (outer), k = 1..n
int ss_write_one_e_matrix(const char* path, int n, const double* m) {
  if (!path || n < 0 || (n > 0 && !m)) {
    ss_set_error_msg("ss_write_one_e_matrix: bad arguments");
    return SS_ERR_ARG;
  }
  FILE* f = fopen(path, "w");
  if (!f) {
    ss_set_error_msg("one-electron output: cannot open %s", path);
    return SS_ERR_ARG;
  }
  std::vector<char> buf((size_t)std::max(n, 1) * 64);
  int rc = SS_OK;
  for (int i = 0; i < n && !rc; i++) {
    size_t pos = 0;
    for (int k = 0; k < n; k++) {
      int nc = snprintf(buf.data() + pos, 32, "%5d %5d ", i + 1, k + 1);
      fortran_d22_15(m[i + (size_t)n * k], buf.data() + pos + nc);
      buf[pos + nc + 22] = '\n';
      pos += (size_t)nc + 23;
    }
    if (fwrite(buf.data(), 1, pos, f) != pos) {
      ss_set_error_msg("one-electron output: write failed");
      rc = SS_ERR_STATE;
    }
  }
  if (fclose(f) != 0 && !rc) {
    ss_set_error_msg("one-electron output: close failed");
    rc = SS_ERR_STATE;
  }
  return rc;
}

int ss_write_bielec_ao(ss_ctx* c, const char* path) {
  if (!c || !path) {
    ss_set_error_msg("ss_write_bielec_ao: null argument");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->have_mc) {
    ss_set_error_msg("ss_write_bielec_ao needs a finished job (ss_two_e_job or ss_zvmc + ss_combine)");
    return SS_ERR_STATE;
  }
  int rc = ss_combine(c, nullptr);  // merged ERIs into the "combined" device buffer
  if (rc) return rc;
  void* p;
  rc = pool_get(c, "combined", sizeof(double) * c->nint, &p);
  if (rc) return rc;
  const double* d_eri = (const double*)p;
  const double* d_sig = (const double*)c->d_sigma.ptr;
  FILE* f = fopen(path, "w");
  if (!f) {
    ss_set_error_msg("bielec_ao: cannot open %s", path);
    return SS_ERR_ARG;
  }
  // two pinned staging chunks: chunk t+1 is copied while chunk t is formatted and written
  const int64_t chunk = 1 << 18;
  double* h = nullptr;
  cudaError_t e = cudaMallocHost(&h, sizeof(double) * 4 * chunk);
  if (e != cudaSuccess) {
    fclose(f);
    ss_set_cuda_error(e, "cudaMallocHost", __FILE__, __LINE__);
    return SS_ERR_NOMEM;
  }
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (ev[0]) cudaEventDestroy(ev[0]);
    cudaFreeHost(h);
    fclose(f);
    ss_set_cuda_error(e, "cudaEventCreate", __FILE__, __LINE__);
    return SS_ERR_CUDA;
  }
  auto issue = [&](int64_t q0, int slot) {
    const int64_t n = std::min(chunk, c->nint - q0);
    double* hv = h + (size_t)slot * 2 * chunk;
    cudaMemcpyAsync(hv, d_eri + q0, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(hv + chunk, d_sig + q0, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaEventRecord(ev[slot], c->stream);
  };
  std::vector<char> buf;
  if (c->nint > 0) issue(0, 0);
  int slot = 0;
  for (int64_t q0 = 0; q0 < c->nint && !rc; q0 += chunk, slot ^= 1) {
    if (q0 + chunk < c->nint) issue(q0 + chunk, slot ^ 1);
    e = cudaEventSynchronize(ev[slot]);
    if (e != cudaSuccess) {
      ss_set_cuda_error(e, "bielec_ao copy", __FILE__, __LINE__);
      rc = SS_ERR_CUDA;
      break;
    }
    const int64_t n = std::min(chunk, c->nint - q0);
    const double* hv = h + (size_t)slot * 2 * chunk;
    rc = write_records(f, q0, n, c->h_is.data(), c->h_js.data(), c->h_ks.data(), c->h_ls.data(), hv, hv + chunk,
                       buf);
  }
  cudaStreamSynchronize(c->stream);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  cudaFreeHost(h);
  if (fclose(f) != 0 && !rc) {
    ss_set_error_msg("bielec_ao: close failed");
    rc = SS_ERR_STATE;
  }
  return rc;
}

}  // extern "C"
