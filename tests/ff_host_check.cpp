// Host check of the double-float arithmetic of the mixed form: gpb_ff.cuh and
// the 6×6 factor and solve of gpb_aba.cuh (chol6_ff, solve6_ff), compiled as
// plain C++ against host versions of the round-to-nearest intrinsics (the
// harness header that tests/test_ff_host.py assembles from the kernel
// sources).  References are in long double.  Prints one line per check,
// "name value", and exits non-zero on a failed bound.
#include <cmath>
#include <cstdio>
#include <random>

#include "ff_harness.h"

static int rsqrt_ulps = 0;  // the device rsqrtf is approximate: perturb the host one
float rsqrtf_host(float x) {
  float r = 1.0f / std::sqrt(x);
  for (int k = 0; k < rsqrt_ulps; ++k) r = std::nextafter(r, 1e30f);
  for (int k = 0; k < -rsqrt_ulps; ++k) r = std::nextafter(r, 0.0f);
  return r;
}

static long double val(FF a) { return (long double)a.hi + (long double)a.lo; }
static FF split(double x) {
  FF f;
  f.hi = (float)x;
  f.lo = (float)(x - (double)f.hi);
  return f;
}

int main() {
  std::mt19937_64 g(11);
  std::normal_distribution<double> N(0, 1);
  std::uniform_real_distribution<double> U(-20, 20);
  int fail = 0;
  auto check = [&](const char* name, double v, double bound) {
    std::printf("%s %.3g\n", name, v);
    if (!(v <= bound)) {
      std::printf("FAIL %s %.3g > %.3g\n", name, v, bound);
      fail = 1;
    }
  };

  // error-free transformations and the basic operations
  double e_sum = 0, e_add = 0, e_mul = 0, e_fma = 0, e_rcp = 0;
  long add_order_differs = 0;
  for (int t = 0; t < 200000; ++t) {
    const double x = N(g) * std::exp(U(g)), y = N(g) * std::exp(U(g) * 0.2);
    const float a = (float)x, b = (float)y;
    const FF s = two_sum(a, b);
    e_sum = std::fmax(e_sum, (double)std::fabs(val(s) - ((long double)a + (long double)b)));
    const FF X = split(x), Y = split(y), Z = split(N(g));
    const long double xa = val(X), ya = val(Y), za = val(Z);
    const auto rel = [](long double got, long double ref, long double scale) {
      return (double)(std::fabs(got - ref) / (scale > 0 ? scale : 1));
    };
    e_add = std::fmax(e_add, rel(val(ff_add(X, Y)), xa + ya, std::fabs(xa) + std::fabs(ya)));
    {  // commutative bit for bit (a reduction over lanes gives every lane the same sum)
      const FF s1 = ff_add(X, Y), s2 = ff_add(Y, X);
      add_order_differs += s1.hi != s2.hi || s1.lo != s2.lo;
    }
    e_mul = std::fmax(e_mul, rel(val(ff_mul(X, Y)), xa * ya, std::fabs(xa * ya)));
    e_fma = std::fmax(e_fma, rel(val(ff_fma(X, Y, Z)), za + xa * ya, std::fabs(za) + std::fabs(xa * ya)));
    e_rcp = std::fmax(e_rcp, rel(val(ff_rcp(X)) * xa, 1.0L, 1.0L));
  }
  check("two_sum_abs_err", e_sum, 0.0);
  check("ff_add_order_differs", (double)add_order_differs, 0.0);
  check("ff_add_rel_err", e_add, 3e-14);
  check("ff_mul_rel_err", e_mul, 3e-14);
  check("ff_fma_rel_err", e_fma, 3e-14);
  check("ff_rcp_rel_err", e_rcp, 3e-14);

  // 1/sqrt(x) with the FP32 start off by up to 2 ulp either way
  double e_rs = 0;
  for (rsqrt_ulps = -2; rsqrt_ulps <= 2; ++rsqrt_ulps)
    for (int t = 0; t < 40000; ++t) {
      const FF x = split(std::exp(U(g) * 1.5));
      const FF r = ff_rsqrt(two_sum(x.hi, x.lo));
      e_rs = std::fmax(e_rs, (double)std::fabs(val(r) * std::sqrt(val(x)) - 1));
    }
  rsqrt_ulps = 0;
  // one Newton step leaves 1.5·δ² of a start off by δ (2 ulp and the
  // rounding: δ ≈ 3.4e-7 at the bottom of a binade) plus rounding
  check("ff_rsqrt_rel_err", e_rs, 3e-13);

  // the floating joint's factor and solve on spatial inertias (rigid body
  // plus random positive semidefinite articulated parts)
  double e_solve = 0, e_dinv = 0;
  int flagged = 0;
  for (int t = 0; t < 20000; ++t) {
    double M[6][6];
    const double m = std::exp(N(g)), com[3] = {0.3 * N(g), 0.3 * N(g), 0.3 * N(g)};
    double A[3][3], Jc[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) A[i][j] = N(g);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Jc[i][j] = (i == j) * 0.01 * m;
        for (int k = 0; k < 3; ++k) Jc[i][j] += 0.05 * m * A[i][k] * A[j][k];
      }
    const double c[3] = {m * com[0], m * com[1], m * com[2]};
    const double cx[3][3] = {{0, -c[2], c[1]}, {c[2], 0, -c[0]}, {-c[1], c[0], 0}};
    const double r2 = com[0] * com[0] + com[1] * com[1] + com[2] * com[2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        M[i][j] = Jc[i][j] + m * ((i == j) * r2 - com[i] * com[j]);
        M[i][3 + j] = M[3 + j][i] = cx[i][j];
        M[3 + i][3 + j] = (i == j) * m;
      }
    for (int q = 0; q < t % 4; ++q) {
      double u[6];
      for (int i = 0; i < 6; ++i) u[i] = N(g);
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) M[i][j] += 0.3 * m * u[i] * u[j];
    }
    ABIF I;
    const int sA[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    for (int k = 0; k < 6; ++k) {
      I.A[k] = split(M[sA[k][0]][sA[k][1]]);
      I.C[k] = split(M[3 + sA[k][0]][3 + sA[k][1]]);
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) I.B[3 * i + j] = split(M[i][3 + j]);
    long double H[6][6];  // the matrix the FF words hold exactly
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        FF f;
        if (i < 3 && j < 3) f = symget(I.A, i, j);
        else if (i < 3) f = I.B[3 * i + (j - 3)];
        else if (j < 3) f = I.B[3 * j + (i - 3)];
        else f = symget(I.C, i - 3, j - 3);
        H[i][j] = val(f);
      }
    FF L[21], dinv[6], x[6];
    if (!chol6_ff(I, L, dinv)) {
      ++flagged;
      continue;
    }
    long double b[6];
    for (int i = 0; i < 6; ++i) {
      x[i] = split(10 * N(g));
      b[i] = val(x[i]);
    }
    solve6_ff(L, dinv, x);
    long double Lr[6][6] = {}, y[6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j <= i; ++j) {
        long double s = H[i][j];
        for (int k = 0; k < j; ++k) s -= Lr[i][k] * Lr[j][k];
        Lr[i][j] = i == j ? std::sqrt(s) : s / Lr[j][j];
      }
    for (int i = 0; i < 6; ++i) {
      long double s = b[i];
      for (int k = 0; k < i; ++k) s -= Lr[i][k] * y[k];
      y[i] = s / Lr[i][i];
    }
    for (int i = 5; i >= 0; --i) {
      long double s = y[i];
      for (int k = i + 1; k < 6; ++k) s -= Lr[k][i] * y[k];
      y[i] = s / Lr[i][i];
    }
    long double mx = 0, err = 0;
    for (int i = 0; i < 6; ++i) {
      mx = std::fmax(mx, std::fabs(y[i]));
      err = std::fmax(err, std::fabs(val(x[i]) - y[i]));
      e_dinv = std::fmax(e_dinv, (double)std::fabs(val(dinv[i]) * Lr[i][i] - 1));
    }
    e_solve = std::fmax(e_solve, (double)(err / mx));
  }
  check("chol6_ff_spd_flagged", flagged, 0);
  check("chol6_ff_dinv_rel_err", e_dinv, 1e-12);
  check("solve6_ff_rel_err", e_solve, 1e-10);

  // an indefinite matrix is reported, as chol6 reports it in FP64
  ABIF Z;
  for (int k = 0; k < 6; ++k) Z.A[k] = Z.C[k] = ff(0.0f);
  for (int k = 0; k < 9; ++k) Z.B[k] = ff(0.0f);
  Z.A[0] = Z.A[1] = ff(1.0f);
  Z.A[2] = ff(-1.0f);
  Z.C[0] = Z.C[1] = Z.C[2] = ff(1.0f);
  FF L[21], dinv[6];
  check("chol6_ff_indefinite_missed", chol6_ff(Z, L, dinv) ? 1 : 0, 0);
  return fail;
}
