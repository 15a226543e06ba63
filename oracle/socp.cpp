// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// Primal-dual interior-point solver of the velocity-stepping friction-cone
// program (see socp.h).  With y = D λ, D = diag(1/μ, 1, 1) per contact, the
// cones become standard Lorentz cones Q = {y0 ≥ ‖(y1, y2)‖} and the problem is
//
//     minimise ½ yᵀ P y + qᵀ y  s.t.  y ∈ Q,   P = D G D,  q = D g,
//
// whose optimality conditions are u = P y + q ∈ Q, y ∈ Q, y ∘ u = 0.  Each
// iteration scales y and u by the Nesterov–Todd point of every cone (W u = W⁻¹ y
// = λ), factors P + W⁻² by Cholesky and takes Mehrotra's predictor and
// corrector steps, keeping both iterates strictly inside the cones.
// Dense linear algebra: the programs have at most a few dozen variables.

#include "socp.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace orc_socp {
namespace {

constexpr double INF = 1e300;

double jdot(const double* u, const double* v) { return u[0] * v[0] - u[1] * v[1] - u[2] * v[2]; }

// sup{α ≥ 0 : u + α d ∈ Q} for u inside Q.
double max_step(const double* u, const double* d) {
  if (d[0] >= std::sqrt(d[1] * d[1] + d[2] * d[2])) return INF;  // d ∈ Q: never leaves
  const double a = jdot(d, d), b = jdot(u, d), c = jdot(u, u);  // f(α) = a α² + 2 b α + c
  if (a == 0.0) return b < 0.0 ? -c / (2.0 * b) : INF;
  const double disc = b * b - a * c;
  if (disc < 0.0) return INF;
  const double sq = std::sqrt(disc);
  const double qq = -(b + std::copysign(sq, b));
  double best = INF;
  for (double r : {qq / a, qq != 0.0 ? c / qq : INF})
    if (r > 0.0 && r < best) best = r;
  return best;
}

// Jordan product u ∘ v and the solution x of λ ∘ x = d, per 3-cone.
void jprod(const double* u, const double* v, double* out) {
  out[0] = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
  out[1] = u[0] * v[1] + v[0] * u[1];
  out[2] = u[0] * v[2] + v[0] * u[2];
}
void jsolve(const double* l, const double* d, double* x) {
  const double det = jdot(l, l);
  x[0] = (l[0] * d[0] - l[1] * d[1] - l[2] * d[2]) / det;
  x[1] = (d[1] - x[0] * l[1]) / l[0];
  x[2] = (d[2] - x[0] * l[2]) / l[0];
}

struct Scaling {  // NT scaling of one cone: W, W⁻¹ (3×3 row-major), η
  double W[9], Wi[9], eta;
};
void nt_scaling(const double* s, const double* z, Scaling* S) {
  const double sn = std::sqrt(jdot(s, s)), zn = std::sqrt(jdot(z, z));
  double sb[3], zb[3];
  for (int k = 0; k < 3; ++k) {
    sb[k] = s[k] / sn;
    zb[k] = z[k] / zn;
  }
  const double gamma = std::sqrt((1.0 + sb[0] * zb[0] + sb[1] * zb[1] + sb[2] * zb[2]) / 2.0);
  // normalised scaling point w̄ = (s̄ + J z̄) / 2γ, then v = (w̄ + e) / √(2 (w̄₀ + 1)):
  // W = η (2 v vᵀ − J), W⁻¹ = (2 J v vᵀ J − J) / η, η = (sᵀJs / zᵀJz)^¼
  const double wb[3] = {(sb[0] + zb[0]) / (2.0 * gamma), (sb[1] - zb[1]) / (2.0 * gamma),
                        (sb[2] - zb[2]) / (2.0 * gamma)};
  const double nv = std::sqrt(2.0 * (wb[0] + 1.0));
  const double w[3] = {(wb[0] + 1.0) / nv, wb[1] / nv, wb[2] / nv};
  const double eta = std::sqrt(sn / zn);
  S->eta = eta;
  const double J[3] = {1.0, -1.0, -1.0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const double jij = i == j ? J[i] : 0.0;
      S->W[3 * i + j] = eta * (2.0 * w[i] * w[j] - jij);
      S->Wi[3 * i + j] = (2.0 * J[i] * w[i] * w[j] * J[j] - jij) / eta;
    }
}
void mul3(const double* A, const double* x, double* y) {
  for (int i = 0; i < 3; ++i) y[i] = A[3 * i] * x[0] + A[3 * i + 1] * x[1] + A[3 * i + 2] * x[2];
}

bool cholesky(std::vector<double>& A, int n) {  // in place, lower triangle
  for (int j = 0; j < n; ++j) {
    double d = A[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    A[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = A[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      A[(size_t)i * n + j] = s / d;
    }
  }
  return true;
}
void chol_solve(const std::vector<double>& L, int n, double* b) {
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[(size_t)i * n + k] * b[k];
    b[i] = s / L[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * b[k];
    b[i] = s / L[(size_t)i * n + i];
  }
}

}  // namespace

int solve(int nc, const double* G, const double* g, double mu, double* lambda, Info* info) {
  const int m = 3 * nc;
  if (nc == 0) return 0;
  std::vector<double> D(m), P((size_t)m * m), q(m);
  for (int i = 0; i < m; ++i) D[i] = (i % 3 == 0) ? 1.0 / mu : 1.0;
  for (int i = 0; i < m; ++i) {
    q[i] = D[i] * g[i];
    for (int j = 0; j < m; ++j) P[(size_t)i * m + j] = D[i] * G[(size_t)i * m + j] * D[j];
  }
  double qn = 0.0;
  for (double x : q) qn = std::max(qn, std::fabs(x));
  std::vector<double> y(m, 0.0), z(m, 0.0), r(m), H((size_t)m * m), lam(m), dya(m), dza(m), dy(m), dz(m),
      rs(m), rhs(m), ds(m);
  for (int c = 0; c < nc; ++c) y[3 * c] = z[3 * c] = 1.0;
  std::vector<Scaling> S(nc);
  int it = 0, status = -1;
  bool last_ok = false;
  double rn = 0.0, gap = 0.0;
  auto newton = [&](std::vector<double>& dyo, std::vector<double>& dzo) {
    for (int c = 0; c < nc; ++c) jsolve(&lam[3 * c], &ds[3 * c], &rs[3 * c]);
    for (int c = 0; c < nc; ++c) {
      double t[3];
      mul3(S[c].Wi, &rs[3 * c], t);
      for (int k = 0; k < 3; ++k) rhs[3 * c + k] = -r[3 * c + k] + t[k];
    }
    dyo = rhs;
    chol_solve(H, m, dyo.data());
    // Δz from the complementarity row, W⁻¹(r_s − W⁻¹Δy), where W⁻¹ is small
    // (η ≥ 1: the cone's y is the larger side); from the dual-residual row,
    // P Δy + r, where W⁻¹ is large and the first form cancels.  Equal in exact
    // arithmetic.
    for (int c = 0; c < nc; ++c) {
      if (S[c].eta >= 1.0) {
        double t[3], u[3];
        mul3(S[c].Wi, &dyo[3 * c], t);
        for (int k = 0; k < 3; ++k) u[k] = rs[3 * c + k] - t[k];
        mul3(S[c].Wi, u, &dzo[3 * c]);
      } else {
        for (int k = 0; k < 3; ++k) {
          const int i = 3 * c + k;
          double s2 = r[i];
          for (int j = 0; j < m; ++j) s2 += P[(size_t)i * m + j] * dyo[j];
          dzo[i] = s2;
        }
      }
    }
  };
  for (it = 0; it < 60; ++it) {
    for (int i = 0; i < m; ++i) {
      double s = q[i] - z[i];
      for (int j = 0; j < m; ++j) s += P[(size_t)i * m + j] * y[j];
      r[i] = s;
    }
    rn = 0.0;
    gap = 0.0;
    double obj = 0.0;
    for (int i = 0; i < m; ++i) {
      rn = std::max(rn, std::fabs(r[i]));
      gap += y[i] * z[i];
      obj += y[i] * (q[i] + 0.5 * (r[i] + z[i] - q[i]));
    }
    // stop at a dual residual of 1e-9 and a gap of 1e-10 (relative); when the
    // Newton matrix loses definiteness at the end of the path, or the
    // iterations run out, accept 1e-7 / 1e-8 (Clarabel's defaults are 1e-8)
    const double scale = 1.0 + std::max(qn, std::fabs(obj));
    if (rn <= 1e-9 * (1.0 + qn) && gap <= 1e-10 * scale) {
      status = 0;
      break;
    }
    last_ok = rn <= 1e-7 * (1.0 + qn) && gap <= 1e-8 * scale;
    for (int c = 0; c < nc; ++c) {
      nt_scaling(&y[3 * c], &z[3 * c], &S[c]);
      mul3(S[c].W, &z[3 * c], &lam[3 * c]);
    }
    H = P;
    for (int c = 0; c < nc; ++c)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
          for (int k = 0; k < 3; ++k) s += S[c].Wi[3 * i + k] * S[c].Wi[3 * k + j];
          H[(size_t)(3 * c + i) * m + 3 * c + j] += s;
        }
    if (!cholesky(H, m)) {
      if (last_ok) status = 0;
      break;
    }
    // predictor (affine scaling)
    for (int c = 0; c < nc; ++c) {
      double ll[3];
      jprod(&lam[3 * c], &lam[3 * c], ll);
      for (int k = 0; k < 3; ++k) ds[3 * c + k] = -ll[k];
    }
    newton(dya, dza);
    double aa = 1.0;
    for (int c = 0; c < nc; ++c)
      aa = std::min({aa, max_step(&y[3 * c], &dya[3 * c]), max_step(&z[3 * c], &dza[3 * c])});
    double gap_a = 0.0;
    for (int i = 0; i < m; ++i) gap_a += (y[i] + aa * dya[i]) * (z[i] + aa * dza[i]);
    const double sigma = std::pow(std::max(gap_a, 0.0) / gap, 3.0);
    const double mu_c = gap / nc;
    // corrector
    for (int c = 0; c < nc; ++c) {
      double ll[3], a[3], b[3], ab[3];
      jprod(&lam[3 * c], &lam[3 * c], ll);
      mul3(S[c].Wi, &dya[3 * c], a);
      mul3(S[c].W, &dza[3 * c], b);
      jprod(a, b, ab);
      for (int k = 0; k < 3; ++k) ds[3 * c + k] = -ll[k] - ab[k] + (k == 0 ? sigma * mu_c : 0.0);
    }
    newton(dy, dz);
    double amax = INF;
    for (int c = 0; c < nc; ++c)
      amax = std::min({amax, max_step(&y[3 * c], &dy[3 * c]), max_step(&z[3 * c], &dz[3 * c])});
    const double alpha = std::min(1.0, 0.99 * amax);
    for (int i = 0; i < m; ++i) {
      y[i] += alpha * dy[i];
      z[i] += alpha * dz[i];
    }
  }
  if (status != 0 && last_ok) status = 0;  // out of iterations at reduced accuracy
  for (int i = 0; i < m; ++i) lambda[i] = D[i] * y[i];
  if (info) {
    info->iterations = it;
    info->residual = rn;
    info->gap = gap;
  }
  return status;
}

}  // namespace orc_socp
