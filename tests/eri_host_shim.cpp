// Host build of the analytic ERI kernel's arithmetic (slater_stoch_gb300/csrc/eri_kernel.cuh):
// the contracted ERI of each quartet from the kernel's own templates (pair_polys, prim_quartet,
// the Boys tables), with the device's choice of template instance and light-ket orientation,
// over all primitive pairs (no screening, FP64 only).  The primitive pairs are built as
// prim_pair_fill builds them (csrc/eri.cu), including the folding of same-fit pairs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../slater_stoch_gb300/csrc/eri_kernel.cuh"

using namespace ss;

namespace {

const double* boys_tables() {
  static std::vector<double> t;
  if (t.empty()) {
    t.insert(t.end(), boys_hi_tab, boys_hi_tab + BOYS_HI_K * BOYS_HI_J);
    t.insert(t.end(), boys_lo_tab, boys_lo_tab + BOYS_LO_K * BOYS_LO_N);
    t.insert(t.end(), exp2_32_tab, exp2_32_tab + 32);
  }
  return t.data();
}

bool fold_pair_h(const BasisDev& B, int i, int k) {
  if (i == k) return true;
  const int ng = B.n_gauss[i];
  if (ng != B.n_gauss[k] || B.i_type[i] != B.i_type[k]) return false;
  for (int ax = 0; ax < 3; ax++)
    if (B.center[3 * i + ax] != B.center[3 * k + ax]) return false;
  const int64_t t = B.i_type[i] == 2 ? 1 : 0;
  for (int m = 0; m < ng; m++) {
    if (B.g_gauss[m + (int64_t)B.ld * i] != B.g_gauss[m + (int64_t)B.ld * k]) return false;
    if (B.c_gauss[m + (int64_t)B.ld * (i + B.n * t)] != B.c_gauss[m + (int64_t)B.ld * (k + B.n * t)]) return false;
  }
  return true;
}

std::vector<PrimPair> build_pairs(const BasisDev& B, int i, int k, bool fold_enabled) {
  std::vector<PrimPair> out;
  const int ngi = B.n_gauss[i], ngk = B.n_gauss[k];
  const double* A = B.center + 3 * i;
  const double* Bc = B.center + 3 * k;
  const int ti = B.i_type[i] == 2 ? 1 : 0, tk = B.i_type[k] == 2 ? 1 : 0;
  const bool fold = fold_enabled && fold_pair_h(B, i, k);
  for (int m1 = 0; m1 < ngi; m1++)
    for (int m2 = (fold ? m1 : 0); m2 < ngk; m2++) {
      const double a = B.g_gauss[m1 + (int64_t)B.ld * i], b = B.g_gauss[m2 + (int64_t)B.ld * k];
      const double p = a + b;
      const double p_inv = 1.0 / (a + b);
      double ab = a * b;
      const double x0 = A[0] - Bc[0], x1 = A[1] - Bc[1], x2 = A[2] - Bc[2];
      ab = ab * p_inv;
      const double kk = ab * (x0 * x0 + x1 * x1 + x2 * x2);
      if (kk > 40.0) continue;
      const double K = std::exp(-kk);
      if (K < 1.e-15) continue;
      PrimPair r{};
      r.p = p;
      r.p_inv = 1.0 / p;
      r.fact = K;
      for (int ax = 0; ax < 3; ax++) {
        r.P[ax] = (a * A[ax] + b * Bc[ax]) * p_inv;
        r.PA[ax] = r.P[ax] - A[ax];
        r.PB[ax] = r.P[ax] - Bc[ax];
      }
      r.coef = B.c_gauss[m1 + (int64_t)B.ld * (i + (int64_t)B.n * ti)] *
               B.c_gauss[m2 + (int64_t)B.ld * (k + (int64_t)B.n * tk)];
      if (fold && m1 != m2) r.coef = 2.0 * r.coef;
      r.pad[2] = (r.fact * r.coef) * r.p_inv;
      out.push_back(r);
    }
  return out;
}

int pair_L(const BasisDev& B, int f1, int f2) {
  int L = 0;
  for (int ax = 0; ax < 3; ax++) {
    const int a = B.npower[3 * f1 + ax] + (B.i_type[f1] == 2 ? 2 : 0);
    const int b = B.npower[3 * f2 + ax] + (B.i_type[f2] == 2 ? 2 : 0);
    L = std::max(L, a + b);
  }
  return L;
}

template <int L, int TC, int LK>
double quartet_value(const BasisDev& B, int fi, int fk, int fj, int fl, bool fold) {
  constexpr bool T2 = TC > 0;
  constexpr int NO = T2 ? 4 : 1;
  constexpr int QW = 3 * NO * (LK + 1);
  const std::vector<PrimPair> bra = build_pairs(B, fi, fk, fold), ket = build_pairs(B, fj, fl, fold);
  const QuartetShape S = quartet_shape<T2>(B, fi, fk, fj, fl);
  std::vector<double> q(ket.size() * QW, 0.0);
  for (size_t t = 0; t < ket.size(); t++) pair_polys<LK, T2, double>(S, 1, ket[t], &q[t * QW]);
  const double* tab = boys_tables();
  double acc = 0.0;
  double Pn[3 * NO * (L + 1)] = {};
  for (const PrimPair& P : bra) {
    pair_polys<L, T2, double>(S, 0, P, Pn);
    for (size_t t = 0; t < ket.size(); t++) {
      acc += prim_quartet<L, TC, double, LK>(S, view64(P), Pn, view64(ket[t]), &q[t * QW], tab);
    }
  }
  return PI_5_2 * acc;
}

// the instance launch_eri_class (csrc/eri.cu) runs for (L, LK, tc): SS_HOST_DISPATCH(F, args)
// returns F<L, TC, LK>(args) for it (bad = 1 when there is none)
#define SS_HOST_DISPATCH(F, ...)                                   \
  do {                                                             \
    if (LK < L) {                                                  \
      if (LK == 0) {                                               \
        if (L == 1 && tc == 0) return F<1, 0, 0>(__VA_ARGS__);     \
        if (L == 2 && tc == 0) return F<2, 0, 0>(__VA_ARGS__);     \
        if (L == 2 && tc == 1) return F<2, 1, 0>(__VA_ARGS__);     \
        if (L == 3 && tc == 0) return F<3, 0, 0>(__VA_ARGS__);     \
        if (L == 3 && tc == 1) return F<3, 1, 0>(__VA_ARGS__);     \
      } else if (LK == 1) {                                        \
        if (L == 2 && tc == 0) return F<2, 0, 1>(__VA_ARGS__);     \
        if (L == 2 && tc == 1) return F<2, 1, 1>(__VA_ARGS__);     \
        if (L == 3 && tc == 0) return F<3, 0, 1>(__VA_ARGS__);     \
        if (L == 3 && tc == 1) return F<3, 1, 1>(__VA_ARGS__);     \
        if (L == 3 && tc == 2) return F<3, 2, 1>(__VA_ARGS__);     \
        if (L == 4 && tc == 0) return F<4, 0, 1>(__VA_ARGS__);     \
        if (L == 4 && tc == 1) return F<4, 1, 1>(__VA_ARGS__);     \
        if (L == 4 && tc == 2) return F<4, 2, 1>(__VA_ARGS__);     \
      } else if (LK == 2) {                                        \
        if (L == 3 && tc == 0) return F<3, 0, 2>(__VA_ARGS__);     \
        if (L == 3 && tc == 1) return F<3, 1, 2>(__VA_ARGS__);     \
        if (L == 3 && tc == 2) return F<3, 2, 2>(__VA_ARGS__);     \
        if (L == 4 && tc == 0) return F<4, 0, 2>(__VA_ARGS__);     \
        if (L == 4 && tc == 1) return F<4, 1, 2>(__VA_ARGS__);     \
        if (L == 4 && tc == 2) return F<4, 2, 2>(__VA_ARGS__);     \
        if (L == 4 && tc == 3) return F<4, 3, 2>(__VA_ARGS__);     \
      }                                                            \
    } else if (tc == 0) {                                          \
      if (L == 0) return F<0, 0, 0>(__VA_ARGS__);                  \
      if (L == 1) return F<1, 0, 1>(__VA_ARGS__);                  \
      if (L == 2) return F<2, 0, 2>(__VA_ARGS__);                  \
      if (L == 3) return F<3, 0, 3>(__VA_ARGS__);                  \
      if (L == 4) return F<4, 0, 4>(__VA_ARGS__);                  \
    } else if (tc == 1) {                                          \
      if (L <= 2) return F<2, 1, 2>(__VA_ARGS__);                  \
      if (L == 3) return F<3, 1, 3>(__VA_ARGS__);                  \
      if (L == 4) return F<4, 1, 4>(__VA_ARGS__);                  \
    } else if (tc == 2) {                                          \
      if (L <= 2) return F<2, 2, 2>(__VA_ARGS__);                  \
      if (L == 3) return F<3, 2, 3>(__VA_ARGS__);                  \
      if (L == 4) return F<4, 2, 4>(__VA_ARGS__);                  \
    } else if (tc == 3) {                                          \
      if (L <= 4) return F<4, 3, 4>(__VA_ARGS__);                  \
    } else if (tc == 4) {                                          \
      if (L <= 4) return F<4, 4, 4>(__VA_ARGS__);                  \
    }                                                              \
  } while (0)

double dispatch(int L, int LK, int tc, const BasisDev& B, int fi, int fk, int fj, int fl, bool fold, int* bad) {
  SS_HOST_DISPATCH(quartet_value, B, fi, fk, fj, fl, fold);
  *bad = 1;
  return 0.0;
}

// Schwarz factors S_P = sqrt(c_P^2 (PP|PP)) of a pair list, as the kernel's self mode computes
// them (the instance of the quartet (ik|ik))
template <int L, int TC, int LK>
std::vector<double> self_factors(const BasisDev& B, int i, int k, const std::vector<PrimPair>& pairs) {
  constexpr bool T2 = TC > 0;
  constexpr int NO = T2 ? 4 : 1;
  const QuartetShape S = quartet_shape<T2>(B, i, k, i, k);
  const double* tab = boys_tables();
  std::vector<double> out(pairs.size());
  double Pn[3 * NO * (L + 1)] = {}, Qn[3 * NO * (LK + 1)] = {};
  for (size_t t = 0; t < pairs.size(); t++) {
    pair_polys<L, T2, double>(S, 0, pairs[t], Pn);
    pair_polys<LK, T2, double>(S, 1, pairs[t], Qn);
    const double v = prim_quartet<L, TC, double, LK>(S, view64(pairs[t]), Pn, view64(pairs[t]), Qn, tab);
    out[t] = std::sqrt(std::fmax(PI_5_2 * v, 0.0));
  }
  return out;
}

std::vector<double> schwarz(const BasisDev& B, int i, int k, const std::vector<PrimPair>& pairs, int* bad) {
  const int L = pair_L(B, i, k), LK = L;
  const int tc = 2 * ((B.i_type[i] == 2) + (B.i_type[k] == 2));
  SS_HOST_DISPATCH(self_factors, B, i, k, pairs);
  *bad = 1;
  return {};
}

PrimPairF to_f32(const PrimPair& a) {  // prim_pair_to_f32 (csrc/eri.cu)
  PrimPairF f{};
  f.p = (float)a.p;
  f.p_inv = (float)a.p_inv;
  f.fc = (float)a.pad[2];
  for (int ax = 0; ax < 3; ax++) {
    f.P[ax] = (float)a.P[ax];
    f.PA[ax] = (float)a.PA[ax];
    f.PB[ax] = (float)a.PB[ax];
  }
  return f;
}

struct Fp32Err {
  double all = 0.0, tier = 0.0;  // max |v32 - v64| / (S_P S_Q) over primitive quartets
  int64_t n_all = 0, n_tier = 0;
  // over quartets: max |sum_tier (v32 - v64)| / sqrt((ik|ik)(jl|jl)) (what the tier changes in
  // the ERI) and max sum_tier |v32 - v64| / sqrt((ik|ik)(jl|jl)) (no cancellation between terms)
  double q_signed = 0.0, q_abs = 0.0;
  // max over quartets of |FP32 running sums - exact sum of the FP32 terms| / Schwarz bound, the
  // tier's items dealt to 128 threads in contiguous runs (bra-major), each summed in float
  double q_acc = 0.0;
};

// the FP32 evaluation of every primitive quartet of one quartet against the FP64 one, as the
// kernel's tiers form them (bra polynomials in FP32 from the FP32 pair copy, ket polynomials
// rounded from FP64, K_AB c folded into the FP32 factor)
template <int L, int TC, int LK>
int fp32_errors(const BasisDev& B, int fi, int fk, int fj, int fl, double sch, double eps32, Fp32Err* e) {
  constexpr bool T2 = TC > 0;
  constexpr int NO = T2 ? 4 : 1;
  constexpr int QW = 3 * NO * (LK + 1);
  const std::vector<PrimPair> bra = build_pairs(B, fi, fk, true), ket = build_pairs(B, fj, fl, true);
  int bad = 0;
  const std::vector<double> Sb = schwarz(B, fi, fk, bra, &bad), Sk = schwarz(B, fj, fl, ket, &bad);
  if (bad) return 1;
  const QuartetShape S = quartet_shape<T2>(B, fi, fk, fj, fl);
  std::vector<double> q(ket.size() * QW, 0.0);
  std::vector<float> qf(ket.size() * QW, 0.f);
  for (size_t t = 0; t < ket.size(); t++) {
    pair_polys<LK, T2, double>(S, 1, ket[t], &q[t * QW]);
    for (int w = 0; w < QW; w++) qf[t * QW + w] = (float)q[t * QW + w];
  }
  const double* tab = boys_tables();
  double Pn[3 * NO * (L + 1)] = {};
  float Pf[3 * NO * (L + 1)] = {};
  double s_signed = 0.0, s_abs = 0.0;
  std::vector<float> tier_terms;
  for (size_t b = 0; b < bra.size(); b++) {
    const PrimPair& P = bra[b];
    const PrimPairF P32 = to_f32(P);
    pair_polys<L, T2, double>(S, 0, P, Pn);
    pair_polys<L, T2, float>(S, 0, P32, Pf);
    for (size_t t = 0; t < ket.size(); t++) {
      // both tiers return the term divided by 2 pi^{5/2} (the kernel applies it to the sum)
      const double v64 = PI_5_2 * prim_quartet<L, TC, double, LK>(S, view64(P), Pn, view64(ket[t]), &q[t * QW], tab);
      const float t32 =
          prim_quartet<L, TC, float, LK>(S, view32(P32), Pf, view32(to_f32(ket[t])), &qf[t * QW], boys32_tab);
      const double v32 = PI_5_2 * (double)t32;
      const double bound = Sb[b] * Sk[t];
      if (!(bound > 0.0)) continue;
      const double r = std::fabs(v32 - v64) / bound;
      e->all = std::max(e->all, r);
      e->n_all++;
      if (bound < eps32 * sch) {
        e->tier = std::max(e->tier, r);
        e->n_tier++;
        s_signed += v32 - v64;
        s_abs += std::fabs(v32 - v64);
        tier_terms.push_back(t32);
      }
    }
  }
  if (sch > 0.0) {
    e->q_signed = std::max(e->q_signed, std::fabs(s_signed) / sch);
    e->q_abs = std::max(e->q_abs, s_abs / sch);
    const size_t nt = tier_terms.size(), per = (nt + 127) / 128;
    double dev = 0.0, exact = 0.0;
    for (size_t t0 = 0; t0 < nt; t0 += per) {
      float acc32 = 0.f;
      for (size_t t = t0; t < std::min(nt, t0 + per); t++) {
        acc32 += tier_terms[t];
        exact += (double)tier_terms[t];
      }
      dev += (double)acc32;
    }
    e->q_acc = std::max(e->q_acc, PI_5_2 * std::fabs(dev - exact) / sch);
  }
  return 0;
}

int dispatch_fp32(int L, int LK, int tc, const BasisDev& B, int fi, int fk, int fj, int fl, double sch,
                  double eps32, Fp32Err* e) {
  SS_HOST_DISPATCH(fp32_errors, B, fi, fk, fj, fl, sch, eps32, e);
  return 1;
}

}  // namespace

extern "C" {

// mode 0: the device's instance choice (light-ket instances, lighter pair as the ket);
// mode 1: full instances only (LK = L), no swap; mode 2: full instances, every quartet as (jl|ik).
// fold: fold the same-fit pairs as the device does.  lk_out[q] = the ket bound used.
int ss_host_eri(int n, int ld, const double* center, const int* npower, const int* nsto, const int* itype,
                const int* ng, const double* cg, const double* gg, const double* gs, int64_t nint,
                const int32_t* is, const int32_t* js, const int32_t* ks, const int32_t* ls, int mode, int fold,
                double* out, int* lk_out) {
  BasisDev B{n, ld, center, npower, nsto, itype, ng, cg, gg, gs};
  int bad = 0;
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    const int Lb = pair_L(B, i, k), Lk = pair_L(B, j, l);
    const int L = std::max(Lb, Lk);
    const int tc = (itype[i] == 2) + (itype[k] == 2) + (itype[j] == 2) + (itype[l] == 2);
    const int lmin = std::min(Lb, Lk);
    const int v = mode == 0 ? ss_light_ket(L, lmin) + 1 : 0;
    const bool swp = (v && Lk > Lb) || mode == 2;
    if (swp) {
      std::swap(i, j);
      std::swap(k, l);
    }
    const int LK = v ? v - 1 : L;
    lk_out[q] = LK;
    out[q] = dispatch(L, LK, tc, B, i, k, j, l, fold != 0, &bad);
  }
  return bad;
}

// Largest |FP32 - FP64| of a primitive quartet relative to its Schwarz bound S_P S_Q, over all
// primitive quartets of the listed quartets and over those below the FP32-tier threshold
// (S_P S_Q < eps32 sqrt((ik|ik)(jl|jl)); the kernel's eps32 is PRIM_FP32_EPS; pre = the Schwarz
// diagonal, n x n column-major).
int ss_host_fp32_error(int n, int ld, const double* center, const int* npower, const int* nsto, const int* itype,
                       const int* ng, const double* cg, const double* gg, const double* gs, int64_t nint,
                       const int32_t* is, const int32_t* js, const int32_t* ks, const int32_t* ls,
                       const double* pre, double eps32,
                       double* out /* max_all, max_tier, n_all, n_tier, q_signed, q_abs, q_acc */) {
  BasisDev B{n, ld, center, npower, nsto, itype, ng, cg, gg, gs};
  Fp32Err e;
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    const int Lb = pair_L(B, i, k), Lk = pair_L(B, j, l);
    const int L = std::max(Lb, Lk);
    const int tc = (itype[i] == 2) + (itype[k] == 2) + (itype[j] == 2) + (itype[l] == 2);
    const int lmin = std::min(Lb, Lk);
    const int v = ss_light_ket(L, lmin) + 1;
    const double sch = std::sqrt(pre[i + (int64_t)n * k] * pre[j + (int64_t)n * l]);
    if (v && Lk > Lb) {
      std::swap(i, j);
      std::swap(k, l);
    }
    if (dispatch_fp32(L, v ? v - 1 : L, tc, B, i, k, j, l, sch, eps32, &e)) return 1;
  }
  out[0] = e.all;
  out[1] = e.tier;
  out[2] = (double)e.n_all;
  out[3] = (double)e.n_tier;
  out[4] = e.q_signed;
  out[5] = e.q_abs;
  out[6] = e.q_acc;
  return 0;
}

// Per quartet: the template instance the device runs (L, LK, tc) and how its primitive quartets
// split into the kernel's three tiers, from the same pair records and Schwarz factors S_P as the
// device (no integral is evaluated): counts[4q + 0] screened (S_P S_Q < eps_screen * sch),
// [4q + 1] FP32 tier (eps_screen * sch <= S_P S_Q < eps32 * sch), [4q + 2] FP64, [4q + 3] all,
// with sch = sqrt((ik|ik)(jl|jl)) from pre (n x n column-major).  cls[3q..3q+2] = L, LK, tc.
int ss_host_tier_counts(int n, int ld, const double* center, const int* npower, const int* nsto, const int* itype,
                        const int* ng, const double* cg, const double* gg, const double* gs, int64_t nint,
                        const int32_t* is, const int32_t* js, const int32_t* ks, const int32_t* ls,
                        const double* pre, double eps_screen, double eps32, double* counts, int* cls) {
  BasisDev B{n, ld, center, npower, nsto, itype, ng, cg, gg, gs};
  std::vector<std::vector<double>> fac((size_t)n * (n + 1) / 2);
  std::vector<char> have(fac.size(), 0);
  int bad = 0;
  auto factors = [&](int i, int k) -> const std::vector<double>& {
    if (i < k) std::swap(i, k);
    const size_t p = (size_t)ss_pair_index(i, k);
    if (!have[p]) {
      std::vector<double> f = schwarz(B, i, k, build_pairs(B, i, k, true), &bad);
      std::sort(f.begin(), f.end(), [](double a, double b) { return a > b; });
      fac[p] = std::move(f);
      have[p] = 1;
    }
    return fac[p];
  };
  // number of (b, t) with Sb[b] * Sk[t] >= thr, both lists in decreasing order (two pointers)
  auto count_ge = [](const std::vector<double>& Sb, const std::vector<double>& Sk, double thr) {
    double c = 0.0;
    size_t hi = Sk.size();  // kets [0, hi) pass for the current bra; hi shrinks as Sb decreases
    for (size_t b = 0; b < Sb.size(); b++) {
      while (hi > 0 && !(Sb[b] * Sk[hi - 1] >= thr)) hi--;
      c += (double)hi;
    }
    return c;
  };
  for (int64_t q = 0; q < nint; q++) {
    int i = is[q] - 1, k = ks[q] - 1, j = js[q] - 1, l = ls[q] - 1;
    const int Lb = pair_L(B, i, k), Lk = pair_L(B, j, l);
    const int L = std::max(Lb, Lk);
    const int tc = (itype[i] == 2) + (itype[k] == 2) + (itype[j] == 2) + (itype[l] == 2);
    const int lmin = std::min(Lb, Lk);
    const int v = ss_light_ket(L, lmin) + 1;
    cls[3 * q] = L;
    cls[3 * q + 1] = v ? v - 1 : L;
    cls[3 * q + 2] = tc;
    const double sch = std::sqrt(pre[i + (int64_t)n * k] * pre[j + (int64_t)n * l]);
    const std::vector<double>& Sb = factors(i, k);
    const std::vector<double>& Sk = factors(j, l);
    const double all = (double)Sb.size() * (double)Sk.size();
    const double kept = count_ge(Sb, Sk, eps_screen * sch);
    const double f64 = count_ge(Sb, Sk, eps32 * sch);
    counts[4 * q] = all - kept;
    counts[4 * q + 1] = kept - f64;
    counts[4 * q + 2] = f64;
    counts[4 * q + 3] = all;
  }
  return bad;
}

}  // extern "C"
