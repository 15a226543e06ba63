// Host check of the mixed form's contact law (gpb_kernels.cu, compiled as plain
// C++ by tests/test_ff_host.py): the approach speed ż = −v·n and the
// tangential velocity v_t = v + n ż formed in FP64 from the contact point's
// FP64 velocity, rounded to FP32 with the penetration, and the law
// (contact_force_parts<float>) run in FP32, against the FP64 form's
// contact_force<double>.  The error of each force is taken relative to the
// size of the terms the law adds, |k z| + |c ż| (Hunt–Crossley: k z^1.5 +
// |λ z^1.5 ż|) times (1 + μ): what the q̈ of a body carrying the point can
// see.  Prints "name value" lines; exits non-zero on a failed bound.
#include <cmath>
#include <cstdio>
#include <random>

#include "law_harness.h"

using gpb::V3;

int main() {
  std::mt19937_64 g(5);
  std::normal_distribution<double> N(0, 1);
  std::uniform_real_distribution<double> U(0, 1);
  int fail = 0;
  auto check = [&](const char* name, double v, double bound) {
    std::printf("%s %.3g\n", name, v);
    if (!(v <= bound)) {
      std::printf("FAIL %s %.3g > %.3g\n", name, v, bound);
      fail = 1;
    }
  };
  double worst[2] = {0, 0};
  long same = 0, total = 0;
  for (int model = 0; model < 2; ++model)
    for (int t = 0; t < 400000; ++t) {
      // stiffnesses and damping of the configurations (cube 1e5 / 1e3,
      // quadruped foot 2e4 / 5e2), half-space α, μ
      const bool cube = t & 1;
      const double k = cube ? 1e5 : 2e4, c = model == 1 ? (cube ? 1e3 : 5e2) : 0.0;
      const double alpha = 0.9, mu = 0.3 + 0.7 * U(g);
      // penetration: inside the 1e-8 margin, shallow, or deep
      const int zk = t % 5;
      const double z = zk == 0 ? -1e-8 * U(g) : (zk < 3 ? 1e-4 * U(g) : 0.05 * U(g));
      V3<double> n{N(g), N(g), N(g)};
      const double nn = std::sqrt(gpb::dot(n, n));
      n = n * (1.0 / nn);
      // contact-point velocity: O(1), with a tangential part from O(1) down to
      // 1e-9 (sticking, rolling) and through the 1e-3 regularisation scale
      const double vn = N(g), vts = std::pow(10.0, -9.0 + 9.0 * U(g));
      V3<double> tng{N(g), N(g), N(g)};
      tng = tng - n * gpb::dot(tng, n);
      const double tn = std::sqrt(gpb::dot(tng, tng));
      const V3<double> vel = n * vn + tng * (vts / tn) + n * (1e-3 * N(g));
      const V3<double> f64 = gpb::contact_force<double>(model, z, n, vel, k, c, alpha, mu);
      const double zd = -gpb::dot(vel, n);
      const V3<double> vtd = vel + n * zd;
      const V3<float> nf{(float)n.x, (float)n.y, (float)n.z};
      const V3<float> f32 = gpb::contact_force_parts<float>(model, (float)z, (float)zd, nf,
                                                            V3<float>{(float)vtd.x, (float)vtd.y, (float)vtd.z},
                                                            (float)k, (float)c, (float)alpha, (float)mu);
      // the FP64 form's law is the parts form with the same arithmetic
      const V3<double> p64 = gpb::contact_force_parts<double>(model, z, zd, n, vtd, k, c, alpha, mu);
      same += p64.x == f64.x && p64.y == f64.y && p64.z == f64.z;
      ++total;
      double scale;
      if (model == 1) {
        scale = std::fabs(k * z) + std::fabs(c * zd);
      } else {
        const double kk = k * 50e3 / (k + 50e3), zn = z > 0 ? z * std::sqrt(z) : 0.0;
        scale = kk * zn + std::fabs(1.5 * alpha * kk * zn * zd);
      }
      scale *= 1 + mu;
      const V3<double> d{f32.x - f64.x, f32.y - f64.y, f32.z - f64.z};
      const double e = std::sqrt(gpb::dot(d, d)) / (scale > 0 ? scale : 1.0);
      if (e > worst[model]) worst[model] = e;
    }
  check("hunt_crossley_rel_err", worst[0], 1e-6);
  check("spring_damper_rel_err", worst[1], 1e-6);
  check("fp64_parts_differ", (double)(total - same), 0.0);
  return fail;
}
