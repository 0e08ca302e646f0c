// Host build of the ERI kernel's Boys function and exponential (slater_stoch_gb300/csrc/boys.cuh),
// for the accuracy test in test_boys_tables.py.  The arithmetic is the device code's: IEEE
// double with explicit fma, so host and device give the same results (up to the 1-ulp rsqrt
// that only enters F_n, n >= 1, for T >= 1).
#include <vector>

#include "../slater_stoch_gb300/csrc/boys.cuh"

static const double* tables() {
  static std::vector<double> t;
  if (t.empty()) {
    t.insert(t.end(), ss::boys_hi_tab, ss::boys_hi_tab + ss::BOYS_HI_K * ss::BOYS_HI_J);
    t.insert(t.end(), ss::boys_lo_tab, ss::boys_lo_tab + ss::BOYS_LO_K * ss::BOYS_LO_N);
    t.insert(t.end(), ss::exp2_32_tab, ss::exp2_32_tab + 32);
  }
  return t.data();
}

extern "C" int ss_host_boys_smem_doubles() { return ss::BOYS_SMEM_DOUBLES; }

// out[i * 17 + n] = F_n(T[i]), n = 0..nf (nf <= 16)
extern "C" void ss_host_boys(const double* T, int count, int nf, double* out) {
  const double* tab = tables();
  for (int i = 0; i < count; i++) {
    double F[17];
    ss::boys_tab<16>(T[i], nf, F, tab);
    for (int n = 0; n <= 16; n++) out[i * 17 + n] = n <= nf ? F[n] : 0.0;
  }
}

extern "C" void ss_host_exp_neg(const double* x, int count, double* out) {
  const double* e2 = tables() + ss::BOYS_HI_K * ss::BOYS_HI_J + ss::BOYS_LO_K * ss::BOYS_LO_N;
  for (int i = 0; i < count; i++) out[i] = ss::exp_neg(x[i], e2);
}

// out[i * 17 + n] = FP32 F_n(T[i]), n = 0..nf (nf <= 16)
extern "C" void ss_host_boys32(const float* T, int count, int nf, float* out) {
  for (int i = 0; i < count; i++) {
    float F[17];
    ss::boys32<16>(T[i], nf, F, ss::boys32_tab);
    for (int n = 0; n <= 16; n++) out[i * 17 + n] = n <= nf ? F[n] : 0.f;
  }
}
