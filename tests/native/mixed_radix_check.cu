// Host check of the mixed-radix register FFT (msf_mixed.cuh): every register
// radix and the two-pass split of every supported length against a direct
// FP64 DFT.  Prints one line per case and "max_rel_err <e>" at the end.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "msf_mixed.cuh"

using namespace msf;

static std::mt19937_64 rng(7);

static void dft64(const std::vector<float2>& x, std::vector<double>& re, std::vector<double>& im) {
  const int n = (int)x.size();
  re.assign(n, 0.0);
  im.assign(n, 0.0);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      const double a = -2.0 * M_PI * (double)((long long)j * k % n) / n;
      re[k] += x[j].x * std::cos(a) - x[j].y * std::sin(a);
      im[k] += x[j].x * std::sin(a) + x[j].y * std::cos(a);
    }
}

static double rel_err(const std::vector<float2>& got, const std::vector<float2>& x) {
  std::vector<double> re, im;
  dft64(x, re, im);
  double e = 0.0, m = 0.0;
  for (size_t k = 0; k < got.size(); ++k) {
    e = std::fmax(e, std::hypot(got[k].x - re[k], got[k].y - im[k]));
    m = std::fmax(m, std::hypot(re[k], im[k]));
  }
  return e / m;
}

static std::vector<float2> random_line(int n) {
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  std::vector<float2> x(n);
  for (auto& v : x) v = make_float2(u(rng), u(rng));
  return x;
}

template <int R>
static double check_radix() {
  auto x = random_line(R);
  float2 a[R];
  for (int i = 0; i < R; ++i) a[i] = x[i];
  mixed::reg_dftm<R>(a);
  std::vector<float2> got(a, a + R);
  const double e = rel_err(got, x);
  std::printf("radix %d rel_err %.3g\n", R, e);
  return e;
}

template <int N>
static double check_two_pass() {
  constexpr int A = mixed::Split2m<N>::A, B = mixed::Split2m<N>::B;
  static_assert(A * B == N, "split");
  auto x = random_line(N);
  std::vector<float2> y(x);
  for (int n1 = 0; n1 < A; ++n1) {
    float2 v[B];
    for (int n2 = 0; n2 < B; ++n2) v[n2] = y[n1 + A * n2];
    mixed::reg_dftm<B>(v);
    for (int k1 = 1; k1 < B; ++k1) {
      const double a = -2.0 * M_PI * (double)(n1 * k1) / N;
      v[k1] = cmul(v[k1], make_float2((float)std::cos(a), (float)std::sin(a)));
    }
    for (int k1 = 0; k1 < B; ++k1) y[n1 + A * k1] = v[k1];
  }
  std::vector<float2> X(N);
  for (int k1 = 0; k1 < B; ++k1) {
    float2 r[A];
    for (int n1 = 0; n1 < A; ++n1) r[n1] = y[A * k1 + n1];
    mixed::reg_dftm<A>(r);
    for (int k2 = 0; k2 < A; ++k2) X[k1 + B * k2] = r[k2];
  }
  const double e = rel_err(X, x);
  std::printf("length %d (%d x %d) rel_err %.3g\n", N, B, A, e);
  return e;
}

int main() {
  double m = 0.0;
#define R_(R) m = std::fmax(m, check_radix<R>());
  R_(2) R_(3) R_(4) R_(5) R_(6) R_(8) R_(9) R_(10) R_(12) R_(15) R_(16) R_(18) R_(20) R_(25) R_(27) R_(32)
#undef R_
#define N_(N) m = std::fmax(m, check_two_pass<N>());
  MSF_SMOOTH_SIZES(N_)
#undef N_
  std::printf("max_rel_err %.3g\n", m);
  return m < 1e-5 ? 0 : 1;
}
