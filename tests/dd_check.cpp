// Host check of the double-float routines in pcaone_gb300/csrc/dd.cuh (the
// arithmetic of the (k+p)^2 Cholesky and triangular inverse): single operations
// against long double, then the right-looking Cholesky and inverse of Gram
// matrices with graded columns.  Prints one line per check: name, value.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#define __host__
#define __device__
#include "../pcaone_gb300/csrc/dd.cuh"

using namespace pcaone;

static long double ld(dd a) { return (long double)a.hi + (long double)a.lo; }

int main() {
  std::mt19937_64 g(1);
  std::normal_distribution<double> nd;
  double e_mul = 0, e_div = 0, e_sqrt = 0, e_add = 0;
  for (int t = 0; t < 200000; ++t) {
    const double x = nd(g) * std::pow(10.0, (int)(g() % 20) - 10);
    const double y = nd(g) * std::pow(10.0, (int)(g() % 20) - 10);
    const dd a = dd_from_double(x), b = dd_from_double(y);
    const long double X = ld(a), Y = ld(b);
    e_mul = std::fmax(e_mul, (double)fabsl((ld(dd_mul(a, b)) - X * Y) / (X * Y)));
    e_div = std::fmax(e_div, (double)fabsl((ld(dd_div(a, b)) - X / Y) / (X / Y)));
    const dd aa = dd{std::fabs(a.hi), a.hi < 0 ? -a.lo : a.lo};
    e_sqrt = std::fmax(e_sqrt, (double)fabsl((ld(dd_sqrt(aa)) - sqrtl(fabsl(X))) / sqrtl(fabsl(X))));
    e_add = std::fmax(e_add, (double)(fabsl(ld(dd_add(a, b)) - (X + Y)) / (fabsl(X) + fabsl(Y))));
  }
  std::printf("op_mul %.3e\nop_div %.3e\nop_sqrt %.3e\nop_add %.3e\n", e_mul, e_div, e_sqrt, e_add);
  // the integer split and merge of the tall products: values over 2^-70 .. 2^100
  double e_split = 0, e_merge = 0, e_zero = 0;
  for (int t = 0; t < 400000; ++t) {
    const double x = nd(g) * std::ldexp(1.0, (int)(g() % 170) - 70);
    float h, l;
    dd_split_bits(x, h, l);
    e_split = std::fmax(e_split, (double)(fabsl((long double)h + (long double)l - (long double)x) / fabsl(x)));
    if (std::fabs(l) > std::ldexp(std::fabs((double)h), -22)) e_split = 1.0;  // lo below ulp(hi)
    // merge: exactly (double)h + (double)l
    e_merge = std::fmax(e_merge, std::fabs(dd_merge_bits(h, l) - ((double)h + (double)l)));
  }
  float h0, l0;
  dd_split_bits(0.0, h0, l0);
  e_zero = std::fabs(h0) + std::fabs(l0) + std::fabs(dd_merge_bits(0.f, 0.f));
  dd_split_bits(-1.0, h0, l0);
  e_zero += std::fabs(h0 + 1.0f) + std::fabs(l0);
  std::printf("split %.3e\nmerge %.3e\nsplit_exact %.3e\n", e_split, e_merge, e_zero);
  for (int L : {1, 2, 5, 40, 48, 64, 112}) {
    const int rows = 3 * L + 7;
    std::vector<double> A((size_t)rows * L), W((size_t)L * L);
    for (auto& v : A) v = nd(g);
    for (int c = 0; c < L; ++c)
      for (int r = 0; r < rows; ++r) A[(size_t)r * L + c] *= std::pow(10.0, -3.0 * c / L);
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) {
        long double s = 0;
        for (int r = 0; r < rows; ++r) s += (long double)A[(size_t)r * L + i] * A[(size_t)r * L + j];
        W[(size_t)i * L + j] = (double)s;
      }
    std::vector<dd> a((size_t)L * L), x((size_t)L * L), dg(L), rdg(L);
    for (int e = 0; e < L * L; ++e) {
      a[e] = dd_from_double(W[e]);
      x[e] = dd{e / L == e % L ? 1.f : 0.f, 0.f};
    }
    for (int k = 0; k < L; ++k) {
      dg[k] = dd_sqrt(a[k * L + k]);
      rdg[k] = dd_div(dd{1.f, 0.f}, dg[k]);
      for (int j = k + 1; j < L; ++j) a[k * L + j] = dd_mul(a[k * L + j], rdg[k]);
      for (int i = k + 1; i < L; ++i)
        for (int j = i; j < L; ++j) a[i * L + j] = dd_fms(a[i * L + j], a[k * L + i], a[k * L + j]);
    }
    for (int k = L - 1; k >= 0; --k) {
      for (int c = k; c < L; ++c) x[k * L + c] = dd_mul(x[k * L + c], rdg[k]);
      for (int i = 0; i < k; ++i)
        for (int c = k; c < L; ++c) x[i * L + c] = dd_fms(x[i * L + c], a[i * L + k], x[k * L + c]);
    }
    auto R = [&](int i, int j) -> long double { return j > i ? ld(a[i * L + j]) : (j == i ? ld(dg[i]) : 0.0L); };
    auto X = [&](int i, int j) -> long double { return j >= i ? ld(x[i * L + j]) : 0.0L; };
    double e_rr = 0, e_xr = 0, wmax = 0;
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) {
        long double s = 0, t = 0;
        for (int q = 0; q < L; ++q) {
          s += R(q, i) * R(q, j);
          t += X(i, q) * R(q, j);
        }
        e_rr = std::fmax(e_rr, (double)fabsl(s - W[(size_t)i * L + j]));
        e_xr = std::fmax(e_xr, (double)fabsl(t - (i == j ? 1.0L : 0.0L)));
        wmax = std::fmax(wmax, std::fabs(W[(size_t)i * L + j]));
      }
    std::printf("chol_L%d %.3e\ninv_L%d %.3e\n", L, e_rr / wmax, L, e_xr);
  }
  return 0;
}
