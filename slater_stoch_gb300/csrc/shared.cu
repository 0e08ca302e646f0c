// shared.cu -- shared-walker estimator: mixture sampler, FP32 orbital densities, split-BF16
// operand producer, block statistics, and the host loop around the tcgen05 GEMM.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mc.cuh"
#include "philox.cuh"
#include "shared.cuh"
#include "ss_common.cuh"
#include "ss_context.cuh"

namespace ss {

struct MixDev {
  int m;
  const double* G;      // [3m] component centres
  const float* Gf;      // [3m] centres rounded to float (hi part)
  const float* Glo;     // [3m] G - Gf (lo part)
  const float* cf;      // [m] ZV-map scale c of each component
  const float* inv2c;   // 1/(2c)
  const float* norm;    // w_c / ((2 pi)^{3/2} 2 c^{3/2})
};

// standard normal from one 32-bit word: bit 0 the sign, bits 1..31 the tail probability
// p in (0, 1/2) (|x| up to 6.2)
__device__ __forceinline__ float normal_from_word(uint32_t w) {
  const float p = ((float)(w >> 1) + 0.5f) * 2.3283064365386963e-10f;  // 2^-32
  const float x = normcdfinvf(p);                                      // <= 0
  return (w & 1u) ? x : -x;
}

// mixture density pi(u) = sum_c norm_c exp(-|u-G_c|/(2c)) |u-G_c|^{-3/2} at u = G_d + off, in
// FP32: u - G_c = (Gf_d - Gf_c) + ((Glo_d - Glo_c) + off), exact where G_c == G_d and within
// ~1e-7 bohr elsewhere
__device__ __forceinline__ float mixture_density(const MixDev& M, int d, const float (&off)[3]) {
  const float h0 = M.Gf[3 * d], h1 = M.Gf[3 * d + 1], h2 = M.Gf[3 * d + 2];
  const float l0 = M.Glo[3 * d], l1 = M.Glo[3 * d + 1], l2 = M.Glo[3 * d + 2];
  float tot = 0.f;
  for (int c = 0; c < M.m; c++) {
    const float dx = (h0 - M.Gf[3 * c]) + ((l0 - M.Glo[3 * c]) + off[0]);
    const float dy = (h1 - M.Gf[3 * c + 1]) + ((l1 - M.Glo[3 * c + 1]) + off[1]);
    const float dz = (h2 - M.Gf[3 * c + 2]) + ((l2 - M.Glo[3 * c + 2]) + off[2]);
    const float rho = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    const float ir = rsqrtf(rho);
    tot += M.norm[c] * __expf(-rho * M.inv2c[c]) * (ir * ir * ir);
  }
  return tot;
}

// Samples of one block.  Per sample one Philox4x32-10 call for each electron: word 0 picks the
// mixture component (equal weights: floor(word * m / 2^32)), words 1..3 give r ~ N(0, I3); the ZV
// map u = G_c + c |r| r (offset in FP32).  Output: SampleF64 (u1, u2 [3S] double, w [S] double;
// ss_shared_samples) or SampleF32 (u as two-float hi + lo [3S] each, w [S] float; the estimator's
// own kernels, which then run without FP64 instructions).
struct SampleF64 {
  static constexpr bool f64 = true;
  double *u1, *u2, *w;
};
struct SampleF32 {
  static constexpr bool f64 = false;
  float *u1h, *u1l, *u2h, *u2l, *w;
};

// hi + lo = a + b (Knuth's two-sum, exact in round-to-nearest)
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
  hi = a + b;
  const float bb = hi - a;
  lo = (a - (hi - bb)) + (b - bb);
}

template <class Out>
__global__ void shared_sample_kernel(uint64_t seed, int64_t first, int64_t S, MixDev M, Out out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= S) return;
  const int64_t g = first + s;
  int d[2];
  float off[2][3];
#pragma unroll
  for (int e = 0; e < 2; e++) {
    uint32_t cnt[4] = {(uint32_t)g, (uint32_t)((uint64_t)g >> 32), (uint32_t)e, STREAM_SHARED};
    philox4x32_10(cnt, (uint32_t)seed, (uint32_t)(seed >> 32));
    d[e] = (int)(((uint64_t)cnt[0] * (uint32_t)M.m) >> 32);
    const float n0 = normal_from_word(cnt[1]), n1 = normal_from_word(cnt[2]), n2 = normal_from_word(cnt[3]);
    const float sc = M.cf[d[e]] * sqrtf(fmaf(n0, n0, fmaf(n1, n1, n2 * n2)));
    off[e][0] = sc * n0;
    off[e][1] = sc * n1;
    off[e][2] = sc * n2;
  }
  const float p1 = mixture_density(M, d[0], off[0]), p2 = mixture_density(M, d[1], off[1]);
  float r2 = 0.f;
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float dl = (M.Gf[3 * d[0] + l] - M.Gf[3 * d[1] + l]) +
                     ((M.Glo[3 * d[0] + l] - M.Glo[3 * d[1] + l]) + (off[0][l] - off[1][l]));
    r2 = fmaf(dl, dl, r2);
    if constexpr (Out::f64) {
      out.u1[3 * s + l] = M.G[3 * d[0] + l] + (double)off[0][l];
      out.u2[3 * s + l] = M.G[3 * d[1] + l] + (double)off[1][l];
    } else {  // u = Gf + Glo + off to ~2^-48 relative
      float h, lo;
      two_sum(M.Gf[3 * d[0] + l], off[0][l], h, lo);
      out.u1h[3 * s + l] = h;
      out.u1l[3 * s + l] = lo + M.Glo[3 * d[0] + l];
      two_sum(M.Gf[3 * d[1] + l], off[1][l], h, lo);
      out.u2h[3 * s + l] = h;
      out.u2l[3 * s + l] = lo + M.Glo[3 * d[1] + l];
    }
  }
  const float ww = 1.0f / (sqrtf(r2) * p1 * p2);
  if constexpr (Out::f64) out.w[s] = isfinite(ww) ? (double)ww : 0.0;
  else out.w[s] = isfinite(ww) ? ww : 0.f;
}

// Fit residual of one shell as a function of t = sqrt(r): cubic Hermite table on a uniform grid
// t_j = j h, j = 0..N, nodes (delta(t_j), h d(delta)/dt(t_j)), delta = u_orb - u_gauss.  Built in
// FP64 on the host from the fit (build_resid_tables); beyond t_max both radial parts are below
// e^-60 of their scale and the residual is u_orb.
struct ResidDev {
  const float2* node;   // all shells, concatenated
  const int* off;       // first node of each shell (nshell + 1 entries)
  const float* inv_h;   // 1/h per shell
  const float* tmax;    // t_max per shell
};

// Orbital values at the samples (the factors of src/compute_densities.F90:51-53):
// phiS_i = poly_i u_orb_i, phiG_i = poly_i u_gauss_i and the fit residual
// delta_i = poly_i (u_orb_i - u_gauss_i).  With 20-Gaussian fits delta/phi is 1e-5..1e-8; the
// residual comes from its FP64-built table (interpolation error below 1e-6 of the shell's largest
// residual), so the whole evaluation runs in FP32: u_orb = r^n_sto e^(-zeta r), u_gauss = u_orb -
// delta.  One block row per shell (consecutive functions sharing centre, STO exponent and fit,
// which differ only by their cartesian monomial).  out[plane][i][s], planes {S1,G1,D1,S2,G2,D2}.
// Coordinates relative to the shell centre from two-float samples and centres:
// (uh - Ah) + (ul - Al), exact in its first difference wherever u is near A.
__global__ void shared_fn_density_kernel(BasisDev B, int64_t S, int64_t ld, const int* __restrict__ shell_start,
                                         ResidDev R, const float* __restrict__ Ahl, SampleF32 U,
                                         float* __restrict__ out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int sh = blockIdx.y;
  if (s >= S) return;
  const int i = shell_start[sh], i_end = shell_start[sh + 1];
  const float* Ah = Ahl + 8 * sh;  // centre hi[3], lo[3], STO exponent, pad
  const int nsto = B.n_sto[i];
  const float zeta = Ah[6];
  const float2* tab = R.node + R.off[sh];
  const int nint = R.off[sh + 1] - R.off[sh] - 1;
  const float inv_h = R.inv_h[sh], tmax = R.tmax[sh];
  const int64_t plane = (int64_t)B.n * ld;
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const float* uh = e == 0 ? U.u1h : U.u2h;
    const float* ul = e == 0 ? U.u1l : U.u2l;
    const float dx = (uh[3 * s] - Ah[0]) + (ul[3 * s] - Ah[3]);
    const float dy = (uh[3 * s + 1] - Ah[1]) + (ul[3 * s + 1] - Ah[4]);
    const float dz = (uh[3 * s + 2] - Ah[2]) + (ul[3 * s + 2] - Ah[5]);
    const float r = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    float uo = expf(-zeta * r);
    for (int t = 0; t < nsto; t++) uo *= r;
    const float t = sqrtf(r);
    float res = uo;
    if (t < tmax) {
      const float x = t * inv_h;
      const int j = min((int)x, nint - 1);
      const float v = x - (float)j;
      const float2 a = tab[j], b = tab[j + 1];
      const float v2 = v * v, v3 = v2 * v;
      res = fmaf(2.f * v3 - 3.f * v2 + 1.f, a.x,
                 fmaf(v3 - 2.f * v2 + v, a.y, fmaf(3.f * v2 - 2.f * v3, b.x, (v3 - v2) * b.y)));
    }
    const float ug = uo - res;
    for (int f = i; f < i_end; f++) {
      float poly = 1.f;
      for (int t2 = 0; t2 < B.npower[3 * f]; t2++) poly *= dx;
      for (int t2 = 0; t2 < B.npower[3 * f + 1]; t2++) poly *= dy;
      for (int t2 = 0; t2 < B.npower[3 * f + 2]; t2++) poly *= dz;
      const int64_t o = (int64_t)f * ld + s;
      out[(3 * e) * plane + o] = poly * uo;
      out[(3 * e + 1) * plane + o] = poly * ug;
      out[(3 * e + 2) * plane + o] = poly * res;
    }
  }
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// operands of one sub-chunk: A = [Delta1 | rhoG1], B = [rhoS2 w | Delta2 w], rows = pairs,
// K = 2*Kh (Kh >= S, padded samples are zero); hi/lo BF16 split.  Each thread forms V consecutive
// samples of one pair (vector loads of the orbital values, V*2-byte stores of each operand
// plane); ld (the orbital-value row stride) and Kh are multiples of V.
template <int V>
struct VecF;
template <>
struct VecF<1> {
  static __device__ __forceinline__ void load(const float* p, float (&x)[1]) { x[0] = *p; }
};
template <>
struct VecF<2> {
  static __device__ __forceinline__ void load(const float* p, float (&x)[2]) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    x[0] = v.x; x[1] = v.y;
  }
};
template <>
struct VecF<4> {
  static __device__ __forceinline__ void load(const float* p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
  }
};
template <>
struct VecF<8> {
  static __device__ __forceinline__ void load(const float* p, float (&x)[8]) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
  }
};

// V bf16 values as one V*2-byte store
template <int V>
__device__ __forceinline__ void store_bf16(__nv_bfloat16* dst, const __nv_bfloat16 (&v)[V]) {
  if constexpr (V == 1) {
    dst[0] = v[0];
  } else {
    uint32_t w32[V / 2];
#pragma unroll
    for (int t = 0; t < V / 2; t++)
      w32[t] = (uint32_t)__bfloat16_as_ushort(v[2 * t]) | ((uint32_t)__bfloat16_as_ushort(v[2 * t + 1]) << 16);
    if constexpr (V == 2) *reinterpret_cast<uint32_t*>(dst) = w32[0];
    else if constexpr (V == 4) *reinterpret_cast<uint2*>(dst) = make_uint2(w32[0], w32[1]);
    else *reinterpret_cast<uint4*>(dst) = make_uint4(w32[0], w32[1], w32[2], w32[3]);
  }
}

template <int V>
__global__ void shared_operand_kernel(int64_t S, int64_t Kh, int64_t ld, int n, const int* __restrict__ pi,
                                      const int* __restrict__ pk, const float* __restrict__ F,
                                      const float* __restrict__ w, __nv_bfloat16* __restrict__ Ahi,
                                      __nv_bfloat16* __restrict__ Alo, __nv_bfloat16* __restrict__ Bhi,
                                      __nv_bfloat16* __restrict__ Blo) {
  // pairs along x: consecutive CTAs read the orbital values of the same samples, which stay in
  // L2 while all pairs use them (with samples along x the whole sub-chunk's values, 24 n bytes
  // per sample, streamed through L2 once per pair)
  const int64_t s0 = (blockIdx.y * (int64_t)blockDim.x + threadIdx.x) * V;
  const int p = blockIdx.x;
  if (s0 >= Kh) return;
  float d1[V], g1[V], s2w[V], d2w[V];
#pragma unroll
  for (int e = 0; e < V; e++) d1[e] = g1[e] = s2w[e] = d2w[e] = 0.f;
  if (s0 < S) {
    const int i = pi[p], k = pk[p];
    const int64_t plane = (int64_t)n * ld;
    const int64_t oi = (int64_t)i * ld + s0, ok = (int64_t)k * ld + s0;
    float a1S[V], a1G[V], a1D[V], b1G[V], b1D[V], a2S[V], a2D[V], b2S[V], b2G[V], b2D[V], ww[V];
    VecF<V>::load(F + oi, a1S);
    VecF<V>::load(F + plane + oi, a1G);
    VecF<V>::load(F + 2 * plane + oi, a1D);
    VecF<V>::load(F + plane + ok, b1G);
    VecF<V>::load(F + 2 * plane + ok, b1D);
    VecF<V>::load(F + 3 * plane + oi, a2S);
    VecF<V>::load(F + 5 * plane + oi, a2D);
    VecF<V>::load(F + 3 * plane + ok, b2S);
    VecF<V>::load(F + 4 * plane + ok, b2G);
    VecF<V>::load(F + 5 * plane + ok, b2D);
    VecF<V>::load(w + s0, ww);
#pragma unroll
    for (int e = 0; e < V; e++) {
      if (s0 + e >= S) break;  // samples past the sub-chunk's end stay zero
      // rhoS - rhoG = phiS_i delta_k + delta_i phiG_k (exact identity, no cancellation)
      d1[e] = fmaf(a1S[e], b1D[e], a1D[e] * b1G[e]);
      g1[e] = a1G[e] * b1G[e];
      s2w[e] = (a2S[e] * b2S[e]) * ww[e];
      d2w[e] = fmaf(a2S[e], b2D[e], a2D[e] * b2G[e]) * ww[e];
    }
  }
  const int64_t K = 2 * Kh;
  const int64_t r = (int64_t)p * K + s0;
  __nv_bfloat16 h[V], l[V];
#pragma unroll
  for (int e = 0; e < V; e++) split_bf16(d1[e], h[e], l[e]);
  store_bf16<V>(Ahi + r, h); store_bf16<V>(Alo + r, l);
#pragma unroll
  for (int e = 0; e < V; e++) split_bf16(g1[e], h[e], l[e]);
  store_bf16<V>(Ahi + r + Kh, h); store_bf16<V>(Alo + r + Kh, l);
#pragma unroll
  for (int e = 0; e < V; e++) split_bf16(s2w[e], h[e], l[e]);
  store_bf16<V>(Bhi + r, h); store_bf16<V>(Blo + r, l);
#pragma unroll
  for (int e = 0; e < V; e++) split_bf16(d2w[e], h[e], l[e]);
  store_bf16<V>(Bhi + r + Kh, h); store_bf16<V>(Blo + r + Kh, l);
}

// Cblk[P][P] (double) += sum over K slices of the fp32 partial products.  The slices are summed
// as an unevaluated FP32 pair hi + lo (two-sum: hi exact-rounded, lo collecting the rounding
// errors; error ~2^-48 of the sum of magnitudes, as a double sum of the FP32 partials) so that
// the FP64 pipe sees two conversions and two adds per element instead of 2 per slice.
__global__ void shared_accumulate_block(int P, int ksplit, const float* __restrict__ Cp, double* __restrict__ Cblk) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t PP = (int64_t)P * P;
  if (e >= PP) return;
  float hi = 0.f, lo = 0.f;
#pragma unroll 4
  for (int t = 0; t < ksplit; t++) {
    float h, l;
    two_sum(hi, Cp[t * PP + e], h, l);
    hi = h;
    lo += l;
  }
  Cblk[e] += (double)hi + (double)lo;
}

// per-quartet block value x = (C[ik][jl] + C[jl][ik]) / (2 npts)  (electron-swap symmetrised)
__global__ void shared_block_stats(int64_t nint, int P, int64_t npts, const int* __restrict__ p1,
                                   const int* __restrict__ p2, double* __restrict__ Cblk,
                                   double* __restrict__ acc, double* __restrict__ acc2) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nint) return;
  const int64_t a = (int64_t)p1[q] * P + p2[q], b = (int64_t)p2[q] * P + p1[q];
  const double x = 0.5 * (Cblk[a] + Cblk[b]) / (double)npts;
  acc[q] += x;
  acc2[q] += x * x;
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
#define TRY(x)           \
  do {                   \
    int _rc = (x);       \
    if (_rc) return _rc; \
  } while (0)

template <class T>
static int upload_v(ss_ctx* c, const char* name, const std::vector<T>& v, T** out) {
  void* p;
  TRY(pool_get(c, name, sizeof(T) * std::max<size_t>(v.size(), 1), &p));
  if (!v.empty()) SS_CUDA_TRY(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c->stream));
  *out = (T*)p;
  return SS_OK;
}

struct SharedPlan {
  int npairs = 0;
  std::vector<int> pi, pk, p1, p2;  // used pairs; per-quartet pair indices
  int* d_pi = nullptr; int* d_pk = nullptr; int* d_p1 = nullptr; int* d_p2 = nullptr;
  std::vector<int> shell_start;     // consecutive functions with identical radial part
  int* d_shell = nullptr;
  float* d_Ahl = nullptr;           // per shell: centre as float hi[3], lo[3], STO exponent, pad
  MixDev mix{};
  ResidDev resid{};
};

static bool same_radial(const ss_ctx* c, int a, int b) {
  if (c->h_nsto[a] != c->h_nsto[b] || c->h_itype[a] != c->h_itype[b] || c->h_ng[a] != c->h_ng[b] ||
      c->h_gs[a] != c->h_gs[b])
    return false;
  for (int l = 0; l < 3; l++)
    if (c->h_center[3 * a + l] != c->h_center[3 * b + l]) return false;
  const size_t ld = c->ld, n = c->n;
  for (int m = 0; m < c->h_ng[a]; m++) {
    if (c->h_gg[m + ld * a] != c->h_gg[m + ld * b]) return false;
    for (int t = 0; t < 2; t++)
      if (c->h_cg[m + ld * (a + n * t)] != c->h_cg[m + ld * (b + n * t)]) return false;
  }
  return true;
}

// Residual tables of the shells (cached per basis): for each shell a cubic Hermite table of
// delta(t) = u_orb - u_gauss on t = sqrt(r) in [0, t_max], r_max = max(60/zeta, sqrt(60/g_min)),
// built in FP64.  N starts at 4096 intervals and doubles until the error at every interval
// midpoint (with the FP32-rounded nodes) is below 1e-6 of the shell's largest |delta|.
static int build_resid_tables(ss_ctx* c, const std::vector<int>& shell_start, ResidDev* out) {
  const int n = c->n, ld = c->ld;
  const int nsh = (int)shell_start.size() - 1;
  if (!c->have_resid) {
    std::vector<float2> node;
    std::vector<int> off(nsh + 1, 0);
    std::vector<float> invh(nsh), tmax(nsh);
    for (int sh = 0; sh < nsh; sh++) {
      const int f = shell_start[sh];
      const double zeta = c->h_gs[f];
      const int k = c->h_nsto[f], ng = c->h_ng[f];
      const double* c1 = &c->h_cg[(size_t)ld * f];
      const double* c2 = &c->h_cg[(size_t)ld * (f + n)];
      const double* g = &c->h_gg[(size_t)ld * f];
      double gmin = 1e300;
      for (int m = 0; m < ng; m++) gmin = std::min(gmin, g[m]);
      const double rmax = std::max(60.0 / zeta, ng > 0 ? sqrt(60.0 / gmin) : 0.0);
      const double tm = sqrt(rmax);
      auto eval = [&](double r, double* d, double* dd) {  // delta and d(delta)/dr
        const double ez = exp(-zeta * r);
        double rk = 1.0, rk1 = 0.0;  // r^k, k r^(k-1)
        for (int t = 0; t < k; t++) {
          rk1 = rk1 * r + rk;
          rk *= r;
        }
        double ug = 0.0, dug = 0.0;
        for (int m = 0; m < ng; m++) {
          const double eg = exp(-g[m] * r * r);
          const double poly = c1[m] + c2[m] * r * r;
          ug += poly * eg;
          dug += (2.0 * c2[m] * r - 2.0 * g[m] * r * poly) * eg;
        }
        *d = rk * ez - ug;
        *dd = (rk1 - zeta * rk) * ez - dug;
      };
      std::vector<float2> tab;
      double h = 0.0;
      for (int N = 4096;; N *= 2) {
        h = tm / N;
        tab.resize(N + 1);
        double dmax = 0.0;
        for (int j = 0; j <= N; j++) {
          const double t = j * h;
          double d, dd;
          eval(t * t, &d, &dd);
          tab[j] = make_float2((float)d, (float)(h * 2.0 * t * dd));
          dmax = std::max(dmax, fabs(d));
        }
        double emax = 0.0;
        for (int j = 0; j < N; j++) {
          const double t = (j + 0.5) * h;
          double d, dd;
          eval(t * t, &d, &dd);
          const double interp = 0.5 * ((double)tab[j].x + (double)tab[j + 1].x) +
                                0.125 * ((double)tab[j].y - (double)tab[j + 1].y);
          emax = std::max(emax, fabs(interp - d));
        }
        if (emax <= 1e-6 * dmax || dmax == 0.0) break;
        if (N >= 65536) {
          ss_set_error_msg("shared estimator: the fit residual of function %d is not resolved by a "
                           "65536-interval table (error %.3g of its maximum)", f + 1, emax / dmax);
          return SS_ERR_UNSUPPORTED;
        }
      }
      off[sh] = (int)node.size();
      node.insert(node.end(), tab.begin(), tab.end());
      invh[sh] = (float)(1.0 / h);
      tmax[sh] = (float)tm;
    }
    off[nsh] = (int)node.size();
    float2* dn;
    int* doff;
    float *dih, *dtm;
    TRY(upload_v(c, "rs_node", node, &dn));
    TRY(upload_v(c, "rs_off", off, &doff));
    TRY(upload_v(c, "rs_invh", invh, &dih));
    TRY(upload_v(c, "rs_tmax", tmax, &dtm));
    c->have_resid = true;
  }
  void* p;
  ResidDev R;
  TRY(pool_get(c, "rs_node", 0, &p)); R.node = (const float2*)p;
  TRY(pool_get(c, "rs_off", 0, &p)); R.off = (const int*)p;
  TRY(pool_get(c, "rs_invh", 0, &p)); R.inv_h = (const float*)p;
  TRY(pool_get(c, "rs_tmax", 0, &p)); R.tmax = (const float*)p;
  *out = R;
  return SS_OK;
}

static int build_shared_plan(ss_ctx* c, double a_zv, SharedPlan& S) {
  const int n = c->n;
  std::vector<int> pidx((size_t)n * n, -1);
  auto use = [&](int i, int k) {
    int& v = pidx[i + (size_t)n * k];
    if (v < 0) {
      v = S.npairs++;
      S.pi.push_back(i);
      S.pk.push_back(k);
    }
    return v;
  };
  S.p1.resize(c->nint);
  S.p2.resize(c->nint);
  for (int64_t q = 0; q < c->nint; q++) {
    S.p1[q] = use(c->h_is[q] - 1, c->h_ks[q] - 1);
    S.p2[q] = use(c->h_js[q] - 1, c->h_ls[q] - 1);
  }
  // mixture: the distinct ZV-map densities (G_ik, c_ik) of the used pairs, equal weights
  std::vector<double> G, cc;
  for (int p = 0; p < S.npairs; p++) {
    int i = S.pi[p], k = S.pk[p];
    double gi = c->h_gs[i], gk = c->h_gs[k];
    double g[3], cv = 0.5 * a_zv / (gi + gk);
    for (int l = 0; l < 3; l++) g[l] = (gi * c->h_center[l + 3 * i] + gk * c->h_center[l + 3 * k]) / (gi + gk);
    bool dup = false;
    for (size_t t = 0; t < cc.size() && !dup; t++)
      dup = fabs(cc[t] - cv) <= 1e-12 * cv && fabs(G[3 * t] - g[0]) <= 1e-12 && fabs(G[3 * t + 1] - g[1]) <= 1e-12 &&
            fabs(G[3 * t + 2] - g[2]) <= 1e-12;
    if (!dup) {
      G.insert(G.end(), g, g + 3);
      cc.push_back(cv);
    }
  }
  const int m = (int)cc.size();
  std::vector<float> Gf(3 * m), Glo(3 * m), cf(m), inv2c(m), norm(m);
  const double wgt = 1.0 / m;
  const double k0 = pow(2.0 * M_PI, 1.5) * 2.0;
  for (int t = 0; t < m; t++) {
    for (int l = 0; l < 3; l++) {
      Gf[3 * t + l] = (float)G[3 * t + l];
      Glo[3 * t + l] = (float)(G[3 * t + l] - (double)Gf[3 * t + l]);
    }
    cf[t] = (float)cc[t];
    inv2c[t] = (float)(1.0 / (2.0 * cc[t]));
    norm[t] = (float)(wgt / (k0 * pow(cc[t], 1.5)));
  }
  double* dG;
  float *dGf, *dGlo, *dcf, *di2c, *dn;
  TRY(upload_v(c, "sh_G", G, &dG));
  TRY(upload_v(c, "sh_Gf", Gf, &dGf));
  TRY(upload_v(c, "sh_Glo", Glo, &dGlo));
  TRY(upload_v(c, "sh_cf", cf, &dcf));
  TRY(upload_v(c, "sh_i2c", inv2c, &di2c));
  TRY(upload_v(c, "sh_norm", norm, &dn));
  S.mix = MixDev{m, dG, dGf, dGlo, dcf, di2c, dn};
  TRY(upload_v(c, "sh_pi", S.pi, &S.d_pi));
  TRY(upload_v(c, "sh_pk", S.pk, &S.d_pk));
  TRY(upload_v(c, "sh_p1", S.p1, &S.d_p1));
  TRY(upload_v(c, "sh_p2", S.p2, &S.d_p2));
  S.shell_start.assign(1, 0);
  for (int f = 1; f < c->n; f++)
    if (!same_radial(c, f, S.shell_start.back())) S.shell_start.push_back(f);
  S.shell_start.push_back(c->n);
  TRY(upload_v(c, "sh_shell", S.shell_start, &S.d_shell));
  std::vector<float> Ahl(8 * (S.shell_start.size() - 1), 0.f);
  for (size_t sh = 0; sh + 1 < S.shell_start.size(); sh++) {
    for (int l = 0; l < 3; l++) {
      const double A = c->h_center[3 * (size_t)S.shell_start[sh] + l];
      const float hi = (float)A;
      Ahl[8 * sh + l] = hi;
      Ahl[8 * sh + 3 + l] = (float)(A - (double)hi);
    }
    Ahl[8 * sh + 6] = (float)c->h_gs[S.shell_start[sh]];
  }
  TRY(upload_v(c, "sh_Ahl", Ahl, &S.d_Ahl));
  TRY(build_resid_tables(c, S.shell_start, &S.resid));
  return SS_OK;
}

int run_shared(ss_ctx* c, double a_zv, uint64_t seed, int64_t npts, int nblocks, int prec, double sigma_target) {
  if (prec != SS_PREC_SPLIT_BF16) {
    ss_set_error_msg("shared estimator: only the SPLIT_BF16 precision runs on the device");
    return SS_ERR_UNSUPPORTED;
  }
  SharedPlan SP;
  TRY(build_shared_plan(c, a_zv, SP));
  const int P = SP.npairs, n = c->n;
  const int64_t nint = c->nint;
  // sub-chunk of samples whose GEMM accumulates in one FP32 TMEM accumulator: up to 262,144
  // samples while its BF16 operands (16 P bytes per sample) stay within 1.5 GB, at least 65,536.
  // Fewer, longer sub-chunks amortise the per-sub-chunk launches, K-slice epilogues and partial
  // sums (26-function H2O job, 2^26 pairs: 65,536 -> 262,144 samples took the job from 1.695
  // to 1.654 s; smaller sub-chunks whose operands would stay in L2 were slower: 16,384 -> 1.96 s).
  int64_t sc_max = 262144;
  while (sc_max > 65536 && 16.0 * P * (double)sc_max > 1.5e9) sc_max /= 2;
  const int64_t Sc = std::min<int64_t>(npts, sc_max);
  const int64_t Kh = (Sc + 31) / 32 * 32;  // K = 2 Kh is a multiple of 64
  const int64_t K = 2 * Kh;
  const int T = (P + 127) / 128;
  const int64_t ktiles = K / 64;
  // K slices so that the T x T x ksplit CTAs (one per SM) fill at most two whole waves: a third,
  // nearly empty wave costs as much as a full one (GEMM 113.5 -> 103.1 ms per job)
  int ksplit = (int)std::max<int64_t>(1, std::min<int64_t>(ktiles, (2 * c->num_sms) / (T * T)));
  void* p;
  double *Cblk, *acc, *acc2;
  float *F, *Cp, *w;
  SampleF32 smp;
  __nv_bfloat16 *Ahi, *Alo, *Bhi, *Blo;
  int* err;
  TRY(pool_get(c, "sh_u1h", sizeof(float) * 3 * Sc, &p)); smp.u1h = (float*)p;
  TRY(pool_get(c, "sh_u1l", sizeof(float) * 3 * Sc, &p)); smp.u1l = (float*)p;
  TRY(pool_get(c, "sh_u2h", sizeof(float) * 3 * Sc, &p)); smp.u2h = (float*)p;
  TRY(pool_get(c, "sh_u2l", sizeof(float) * 3 * Sc, &p)); smp.u2l = (float*)p;
  // orbital-value rows and weights padded to a multiple of 8 samples (the operand kernel's vector
  // loads); entries past a sub-chunk's last sample are never used
  const int64_t ldF = (Sc + 7) / 8 * 8;
  TRY(pool_get(c, "sh_w", sizeof(float) * ldF, &p)); w = (float*)p;
  smp.w = w;
  TRY(pool_get(c, "sh_F", sizeof(float) * 6 * (size_t)n * ldF, &p)); F = (float*)p;
  const size_t opb = sizeof(__nv_bfloat16) * (size_t)P * K;
  TRY(pool_get(c, "sh_Ahi", opb, &p)); Ahi = (__nv_bfloat16*)p;
  TRY(pool_get(c, "sh_Alo", opb, &p)); Alo = (__nv_bfloat16*)p;
  TRY(pool_get(c, "sh_Bhi", opb, &p)); Bhi = (__nv_bfloat16*)p;
  TRY(pool_get(c, "sh_Blo", opb, &p)); Blo = (__nv_bfloat16*)p;
  TRY(pool_get(c, "sh_Cp", sizeof(float) * (size_t)ksplit * P * P, &p)); Cp = (float*)p;
  TRY(pool_get(c, "sh_Cblk", sizeof(double) * (size_t)P * P, &p)); Cblk = (double*)p;
  TRY(pool_get(c, "sh_acc", sizeof(double) * nint, &p)); acc = (double*)p;
  TRY(pool_get(c, "sh_acc2", sizeof(double) * nint, &p)); acc2 = (double*)p;
  TRY(pool_get(c, "sh_err", sizeof(int), &p)); err = (int*)p;
  unsigned long long* maxbits;
  TRY(pool_get(c, "sh_maxbits", sizeof(unsigned long long), &p)); maxbits = (unsigned long long*)p;
  SS_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(double) * nint, c->stream));
  SS_CUDA_TRY(cudaMemsetAsync(acc2, 0, sizeof(double) * nint, c->stream));
  SS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  TRY(dev_alloc(c, c->d_mean, sizeof(double) * nint));
  TRY(dev_alloc(c, c->d_sigma, sizeof(double) * nint));
  const int64_t PP = (int64_t)P * P;
  int done = 0;
  for (int b = 0; b < nblocks; b++) {
    SS_CUDA_TRY(cudaMemsetAsync(Cblk, 0, sizeof(double) * PP, c->stream));
    for (int64_t c0 = 0; c0 < npts; c0 += Sc) {
      const int64_t ns = std::min(Sc, npts - c0);
      const int64_t first = (int64_t)b * npts + c0;
      shared_sample_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, c->stream>>>(seed, first, ns, SP.mix, smp);
      SS_CUDA_TRY(cudaGetLastError());
      shared_fn_density_kernel<<<dim3((unsigned)((ns + 127) / 128), (unsigned)(SP.shell_start.size() - 1)), 128, 0,
                                 c->stream>>>(c->basis, ns, ldF, SP.d_shell, SP.resid, SP.d_Ahl, smp, F);
      SS_CUDA_TRY(cudaGetLastError());
      // four samples per thread (8-byte stores): per job 0.263 s of MC with one, 0.245 s with
      // two, 0.226 s with four, 0.262 s with eight
      shared_operand_kernel<4><<<dim3((unsigned)P, (unsigned)((Kh / 4 + 255) / 256)), 256, 0, c->stream>>>(
          ns, Kh, ldF, n, SP.d_pi, SP.d_pk, F, w, Ahi, Alo, Bhi, Blo);
      SS_CUDA_TRY(cudaGetLastError());
      TRY(launch_split_bf16_gemm(c->stream, Ahi, Alo, Bhi, Blo, P, K, ksplit, Cp, err));
      shared_accumulate_block<<<(unsigned)((PP + 255) / 256), 256, 0, c->stream>>>(P, ksplit, Cp, Cblk);
      SS_CUDA_TRY(cudaGetLastError());
      c->launches += 5;
    }
    shared_block_stats<<<(unsigned)((nint + 255) / 256), 256, 0, c->stream>>>(nint, P, npts, SP.d_p1, SP.d_p2, Cblk,
                                                                               acc, acc2);
    SS_CUDA_TRY(cudaGetLastError());
    c->launches++;
    done = b + 1;
    if (sigma_target > 0.0 && done >= 2 && done < nblocks) {
      SS_CUDA_TRY(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), c->stream));
      SS_CUDA_TRY(launch_zv_final(c->stream, nint, done, 1, acc, acc2, (double*)c->d_mean.ptr,
                                  (double*)c->d_sigma.ptr, maxbits));
      c->launches++;
      unsigned long long h = 0;
      SS_CUDA_TRY(cudaMemcpyAsync(&h, maxbits, sizeof h, cudaMemcpyDeviceToHost, c->stream));
      SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
      double ms;
      memcpy(&ms, &h, sizeof ms);
      if (ms <= sigma_target) break;
    }
  }
  SS_CUDA_TRY(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), c->stream));
  SS_CUDA_TRY(launch_zv_final(c->stream, nint, done, 1, acc, acc2, (double*)c->d_mean.ptr, (double*)c->d_sigma.ptr,
                              maxbits));
  c->launches++;
  unsigned long long h = 0;
  int herr = 0;
  SS_CUDA_TRY(cudaMemcpyAsync(&h, maxbits, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (herr) {
    ss_set_error_msg("tcgen05 GEMM: a bounded wait gave up (code %d)", herr);
    return SS_ERR_TIMEOUT;
  }
  memcpy(&c->mc_max_sigma, &h, sizeof(double));
  c->mc_blocks_done = done;
  c->have_mc = true;
  return SS_OK;
}

}  // namespace ss

using namespace ss;

__global__ void sum_slices_kernel(int64_t PP, int ksplit, const float* __restrict__ Cp, float* __restrict__ C) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= PP) return;
  double v = 0.0;
  for (int t = 0; t < ksplit; t++) v += (double)Cp[t * PP + e];
  C[e] = (float)v;
}

extern "C" int ss_split_bf16_gemm(ss_ctx* c, int P, int64_t K, const uint16_t* a_hi, const uint16_t* a_lo,
                                  const uint16_t* b_hi, const uint16_t* b_lo, int ksplit, float* out) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (P <= 0 || K <= 0 || K % 64 != 0 || !a_hi || !a_lo || !b_hi || !b_lo || !out || ksplit < 0) {
    ss_set_error_msg("ss_split_bf16_gemm: need P > 0, K a positive multiple of 64, non-null buffers");
    return SS_ERR_ARG;
  }
  const int T = (P + 127) / 128;
  if (ksplit == 0) ksplit = (int)std::max<int64_t>(1, std::min<int64_t>(K / 64, (2 * c->num_sms) / (T * T)));
  const size_t ob = sizeof(uint16_t) * (size_t)P * K;
  const int64_t PP = (int64_t)P * P;
  void *ah, *al, *bh, *bl, *cp, *cc, *err;
  TRY(pool_get(c, "gm_ah", ob, &ah));
  TRY(pool_get(c, "gm_al", ob, &al));
  TRY(pool_get(c, "gm_bh", ob, &bh));
  TRY(pool_get(c, "gm_bl", ob, &bl));
  TRY(pool_get(c, "gm_cp", sizeof(float) * PP * ksplit, &cp));
  TRY(pool_get(c, "gm_c", sizeof(float) * PP, &cc));
  TRY(pool_get(c, "gm_err", sizeof(int), &err));
  SS_CUDA_TRY(cudaMemcpyAsync(ah, a_hi, ob, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(al, a_lo, ob, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(bh, b_hi, ob, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(bl, b_lo, ob, cudaMemcpyHostToDevice, c->stream));
  SS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
  TRY(launch_split_bf16_gemm(c->stream, ah, al, bh, bl, P, K, ksplit, (float*)cp, (int*)err));
  sum_slices_kernel<<<(unsigned)((PP + 255) / 256), 256, 0, c->stream>>>(PP, ksplit, (const float*)cp, (float*)cc);
  SS_CUDA_TRY(cudaGetLastError());
  c->launches += 2;
  int herr = 0;
  SS_CUDA_TRY(cudaMemcpyAsync(out, cc, sizeof(float) * PP, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (herr) {
    ss_set_error_msg("tcgen05 GEMM: a bounded wait gave up (code %d)", herr);
    return SS_ERR_TIMEOUT;
  }
  return SS_OK;
}

extern "C" int ss_shared_samples(ss_ctx* c, double a_zv, uint64_t seed, int64_t first, int64_t S, double* u1,
                                 double* u2, double* w) {
  if (!c) {
    ss_set_error_msg("null ss_ctx");
    return SS_ERR_ARG;
  }
  SS_CUDA_TRY(cudaSetDevice(c->device));
  if (!c->n || !c->nint) {
    ss_set_error_msg("basis and quartets must be set first");
    return SS_ERR_STATE;
  }
  if (S <= 0 || first < 0 || !u1 || !u2 || !w || !(a_zv > 0.0)) {
    ss_set_error_msg("ss_shared_samples: bad arguments");
    return SS_ERR_ARG;
  }
  SharedPlan SP;
  TRY(build_shared_plan(c, a_zv, SP));
  void *a, *b, *ww;
  TRY(pool_get(c, "smp_u1", sizeof(double) * 3 * S, &a));
  TRY(pool_get(c, "smp_u2", sizeof(double) * 3 * S, &b));
  TRY(pool_get(c, "smp_w", sizeof(double) * S, &ww));
  shared_sample_kernel<<<(unsigned)((S + 127) / 128), 128, 0, c->stream>>>(
      seed, first, S, SP.mix, SampleF64{(double*)a, (double*)b, (double*)ww});
  SS_CUDA_TRY(cudaGetLastError());
  c->launches++;
  SS_CUDA_TRY(cudaMemcpyAsync(u1, a, sizeof(double) * 3 * S, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(u2, b, sizeof(double) * 3 * S, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaMemcpyAsync(w, ww, sizeof(double) * S, cudaMemcpyDeviceToHost, c->stream));
  SS_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return SS_OK;
}
