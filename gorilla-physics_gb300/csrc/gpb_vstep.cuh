// Velocity stepping for one lane (included by gpb_kernels.cu after the CRBA
// sweeps, the Cholesky factorisation and the collision routine).
//
// gorilla-physics' velocity_stepping (src/integrators.rs:42-51) with
// dynamics_discrete (src/dynamics.rs:367-430):
//   1. v_free = v + dt M⁻¹(τ + τ_spring − c): the CRBA sweeps without contact
//      wrenches, the mass matrix and its Cholesky factor (kept for 4 and 6);
//   2. contacts (collision_detection, src/dynamics.rs:520-650): points inside a
//      half-space (margin 1e-8), spheres within their radius (the centre's
//      projection on the plane), cuboid pairs (GJK/EPA: normal cp_b − cp_a at
//      cp_a); each gives three Jacobian rows C X H (compose_contact_jacobian,
//      src/dynamics.rs:744-820): C = (n, t, b), t = n × x̂ (or n × ŷ), b = n × t,
//      X the point velocity v + ω × p of the world motion-subspace columns, +
//      for the joints supporting body a, − for those supporting body b only;
//   3. the friction-cone program min ½λᵀGλ + gᵀλ, ‖(λ_t, λ_b)‖ ≤ μ λ_n, μ = 0.95,
//      G = J M⁻¹ Jᵀ, g = J v_free (solve_constraint_and_contact,
//      src/dynamics.rs:652-742, which calls Clarabel): a primal-dual
//      interior-point method with Nesterov–Todd scaling and Mehrotra's
//      predictor-corrector on y = (μλ_n, λ_t, λ_b) in standard Lorentz cones;
//   4. v' = v_free + M⁻¹ Jᵀ λ;  q' = q + dt v' (compute_new_q).
// All in FP64.  Working arrays live in the batch's velocity-stepping scratch
// (VSLayout, lane-interleaved).
#pragma once

namespace vstep {

struct View {
  double* p;  // this lane's element 0 of the pack's velocity-stepping scratch
  __device__ __forceinline__ double& operator()(int e) const { return p[(size_t)e * LANES]; }
};

__device__ __forceinline__ double jdot(const double* u, const double* v) {
  return u[0] * v[0] - u[1] * v[1] - u[2] * v[2];
}

// sup{α ≥ 0 : u + α d ∈ Q} for u strictly inside the Lorentz cone Q.
__device__ __forceinline__ double max_step(const double* u, const double* d) {
  const double a = jdot(d, d), b = jdot(u, d), c = jdot(u, u);
  if (d[0] >= 0.0 && a >= 0.0) return 1e300;  // d ∈ Q: the ray never leaves
  if (a == 0.0) return b < 0.0 ? -c / (2.0 * b) : 1e300;
  const double disc = b * b - a * c;
  if (disc < 0.0) return 1e300;
  const double qq = -(b + copysign(sqrt(disc), b));
  double best = 1e300;
  const double r1 = qq / a, r2 = qq != 0.0 ? c / qq : 1e300;
  if (r1 > 0.0 && r1 < best) best = r1;
  if (r2 > 0.0 && r2 < best) best = r2;
  return best;
}

// Nesterov–Todd scaling of one cone pair (s, z): W = η(2vvᵀ − J),
// W⁻¹ = (2JvvᵀJ − J)/η with v built from the normalised scaling point.
__device__ __forceinline__ void nt_scaling(const double* s, const double* z, double* W, double* Wi, double* eta) {
  // reciprocal square roots and one division per reciprocal, multiplications
  // elsewhere (FP64 division and square root are multi-instruction sequences
  // on the FP64 unit; the solver needs no correctly rounded results)
  const double rsn = rsqrt(jdot(s, s)), rzn = rsqrt(jdot(z, z));
  const double sn = jdot(s, s) * rsn;
  double sb[3], zb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    sb[k] = s[k] * rsn;
    zb[k] = z[k] * rzn;
  }
  const double rg2 = 0.5 * rsqrt((1.0 + sb[0] * zb[0] + sb[1] * zb[1] + sb[2] * zb[2]) * 0.5);
  const double w0 = (sb[0] + zb[0]) * rg2, w1 = (sb[1] - zb[1]) * rg2, w2 = (sb[2] - zb[2]) * rg2;
  const double rnv = rsqrt(2.0 * (w0 + 1.0));
  const double v[3] = {(w0 + 1.0) * rnv, w1 * rnv, w2 * rnv};
  const double e = sqrt(sn * rzn), re = 1.0 / e;
  const double J[3] = {1.0, -1.0, -1.0};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double jij = i == j ? J[i] : 0.0;
      W[3 * i + j] = e * (2.0 * v[i] * v[j] - jij);
      Wi[3 * i + j] = (2.0 * J[i] * v[i] * v[j] * J[j] - jij) * re;
    }
  *eta = e;
}

__device__ __forceinline__ void jprod(const double* u, const double* v, double* o) {
  o[0] = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
  o[1] = u[0] * v[1] + v[0] * u[1];
  o[2] = u[0] * v[2] + v[0] * u[2];
}

// In-place Cholesky of the m × m matrix at H (lower triangle, the diagonal
// stored as 1 / L_ii); false if not SPD.
__device__ __forceinline__ bool chol(const View& V, int H, int m) {
  for (int j = 0; j < m; ++j) {
    double d = V(H + j * m + j);
    for (int k = 0; k < j; ++k) d -= V(H + j * m + k) * V(H + j * m + k);
    if (!(d > 0.0)) return false;
    const double di = rsqrt(d);
    V(H + j * m + j) = di;  // the reciprocal: solves multiply
    for (int i = j + 1; i < m; ++i) {
      double s = V(H + i * m + j);
      for (int k = 0; k < j; ++k) s -= V(H + i * m + k) * V(H + j * m + k);
      V(H + i * m + j) = s * di;
    }
  }
  return true;
}
// Solve with the factor of chol(), whose diagonal holds 1 / L_ii.
__device__ __forceinline__ void chol_solve(const View& V, int H, int m, int x) {
  for (int i = 0; i < m; ++i) {
    double s = V(x + i);
    for (int k = 0; k < i; ++k) s -= V(H + i * m + k) * V(x + k);
    V(x + i) = s * V(H + i * m + i);
  }
  for (int i = m - 1; i >= 0; --i) {
    double s = V(x + i);
    for (int k = i + 1; k < m; ++k) s -= V(H + k * m + i) * V(x + k);
    V(x + i) = s * V(H + i * m + i);
  }
}

// Newton direction of the scaled system for the complementarity target ds:
// (P + W⁻²) Δy = −r + W⁻¹(λ⁻¹ ∘ ds);  Δz from the complementarity row where
// η ≥ 1, from the dual-residual row P Δy + r elsewhere (equal in exact
// arithmetic; each form is the accurate one on its side).
__device__ __forceinline__ void newton(const View& V, const VSLayout& L, int nc, int dyo, int dzo) {
  const int m = 3 * nc;
  for (int c = 0; c < nc; ++c) {
    double l[3], d[3], x[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      l[k] = V(L.lam + 3 * c + k);
      d[k] = V(L.ds + 3 * c + k);
    }
    const double rdet = 1.0 / jdot(l, l), rl0 = 1.0 / l[0];
    x[0] = (l[0] * d[0] - l[1] * d[1] - l[2] * d[2]) * rdet;
    x[1] = (d[1] - x[0] * l[1]) * rl0;
    x[2] = (d[2] - x[0] * l[2]) * rl0;
#pragma unroll
    for (int k = 0; k < 3; ++k) V(L.rs + 3 * c + k) = x[k];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double t = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) t += V(L.Wi + 9 * c + 3 * i + k) * x[k];
      V(dyo + 3 * c + i) = -V(L.r + 3 * c + i) + t;
    }
  }
  chol_solve(V, L.H, m, dyo);
  for (int c = 0; c < nc; ++c) {
    if (V(L.eta + c) >= 1.0) {
      double t[3], u[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double a = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) a += V(L.Wi + 9 * c + 3 * i + k) * V(dyo + 3 * c + k);
        t[i] = a;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) u[k] = V(L.rs + 3 * c + k) - t[k];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double a = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) a += V(L.Wi + 9 * c + 3 * i + k) * u[k];
        V(dzo + 3 * c + i) = a;
      }
    } else {
      for (int i = 3 * c; i < 3 * c + 3; ++i) {
        double a = V(L.r + i);
        for (int j = 0; j < m; ++j) a += V(L.P + i * m + j) * V(dyo + j);
        V(dzo + i) = a;
      }
    }
  }
}

// The friction-cone program for nc contacts, G in L.P and g in L.qv on entry:
// λ into L.lam.  Returns 0 on convergence: a dual residual of 1e-9 and a gap
// of 1e-10 (relative), or 1e-7 / 1e-8 when the Newton matrix stops being
// positive definite at the end of the path or the 60 iterations run out
// (Clarabel's defaults are 1e-8).
__device__ __noinline__ int solve_cones(const View V, const VSLayout L, int nc, double mu) {
  const int m = 3 * nc;
  const double imu = 1.0 / mu;
  double qn = 0.0;
  for (int i = 0; i < m; ++i) {  // P = D G D, q = D g, D = diag(1/μ, 1, 1)
    const double di = (i % 3 == 0) ? imu : 1.0;
    for (int j = 0; j < m; ++j) V(L.P + i * m + j) = V(L.P + i * m + j) * (di * ((j % 3 == 0) ? imu : 1.0));
    V(L.qv + i) = di * V(L.qv + i);
    qn = fmax(qn, fabs(V(L.qv + i)));
    V(L.y + i) = (i % 3 == 0) ? 1.0 : 0.0;
    V(L.z + i) = V(L.y + i);
  }
  int status = -1;
  bool last_ok = false;
  for (int it = 0; it < 60; ++it) {
    double rn = 0.0, gap = 0.0, obj = 0.0;
    for (int i = 0; i < m; ++i) {
      double s = V(L.qv + i) - V(L.z + i);
      for (int j = 0; j < m; ++j) s += V(L.P + i * m + j) * V(L.y + j);
      V(L.r + i) = s;
      rn = fmax(rn, fabs(s));
      gap += V(L.y + i) * V(L.z + i);
      obj += V(L.y + i) * (V(L.qv + i) + 0.5 * (s + V(L.z + i) - V(L.qv + i)));
    }
    const double scale = 1.0 + fmax(qn, fabs(obj));
    if (rn <= 1e-9 * (1.0 + qn) && gap <= 1e-10 * scale) {
      status = 0;
      break;
    }
    last_ok = rn <= 1e-7 * (1.0 + qn) && gap <= 1e-8 * scale;
    // scalings, λ = W z, H = P + W⁻²
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) V(L.H + i * m + j) = V(L.P + i * m + j);
    for (int c = 0; c < nc; ++c) {
      double s[3], z[3], W[9], Wi[9], e;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        s[k] = V(L.y + 3 * c + k);
        z[k] = V(L.z + 3 * c + k);
      }
      nt_scaling(s, z, W, Wi, &e);
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        V(L.W + 9 * c + k) = W[k];
        V(L.Wi + 9 * c + k) = Wi[k];
      }
      V(L.eta + c) = e;
#pragma unroll
      for (int i = 0; i < 3; ++i) V(L.lam + 3 * c + i) = W[3 * i] * z[0] + W[3 * i + 1] * z[1] + W[3 * i + 2] * z[2];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          V(L.H + (3 * c + i) * m + 3 * c + j) +=
              Wi[3 * i] * Wi[j] + Wi[3 * i + 1] * Wi[3 + j] + Wi[3 * i + 2] * Wi[6 + j];
    }
    if (!chol(V, L.H, m)) {
      if (last_ok) status = 0;
      break;
    }
    // predictor: ds = −λ ∘ λ
    for (int c = 0; c < nc; ++c) {
      double l[3], ll[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) l[k] = V(L.lam + 3 * c + k);
      jprod(l, l, ll);
#pragma unroll
      for (int k = 0; k < 3; ++k) V(L.ds + 3 * c + k) = -ll[k];
    }
    newton(V, L, nc, L.dya, L.dza);
    double aa = 1.0;
    for (int c = 0; c < nc; ++c) {
      double u[3], d[3], w[3], e[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        u[k] = V(L.y + 3 * c + k);
        d[k] = V(L.dya + 3 * c + k);
        w[k] = V(L.z + 3 * c + k);
        e[k] = V(L.dza + 3 * c + k);
      }
      aa = fmin(aa, fmin(max_step(u, d), max_step(w, e)));
    }
    double gap_a = 0.0;
    for (int i = 0; i < m; ++i) gap_a += (V(L.y + i) + aa * V(L.dya + i)) * (V(L.z + i) + aa * V(L.dza + i));
    const double sr = fmax(gap_a, 0.0) / gap;
    const double sigma = sr * sr * sr, mu_c = gap / nc;
    // corrector: ds = −λ∘λ − (W⁻¹Δy_a) ∘ (W Δz_a) + σ μ e
    for (int c = 0; c < nc; ++c) {
      double l[3], ll[3], a[3], b[3], ab[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) l[k] = V(L.lam + 3 * c + k);
      jprod(l, l, ll);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        double x = 0.0, y = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          x += V(L.Wi + 9 * c + 3 * i + k) * V(L.dya + 3 * c + k);
          y += V(L.W + 9 * c + 3 * i + k) * V(L.dza + 3 * c + k);
        }
        a[i] = x;
        b[i] = y;
      }
      jprod(a, b, ab);
#pragma unroll
      for (int k = 0; k < 3; ++k) V(L.ds + 3 * c + k) = -ll[k] - ab[k] + (k == 0 ? sigma * mu_c : 0.0);
    }
    newton(V, L, nc, L.dy, L.dz);
    double amax = 1e300;
    for (int c = 0; c < nc; ++c) {
      double u[3], d[3], w[3], e[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        u[k] = V(L.y + 3 * c + k);
        d[k] = V(L.dy + 3 * c + k);
        w[k] = V(L.z + 3 * c + k);
        e[k] = V(L.dz + 3 * c + k);
      }
      amax = fmin(amax, fmin(max_step(u, d), max_step(w, e)));
    }
    const double alpha = fmin(1.0, 0.99 * amax);
    for (int i = 0; i < m; ++i) {
      V(L.y + i) = V(L.y + i) + alpha * V(L.dy + i);
      V(L.z + i) = V(L.z + i) + alpha * V(L.dz + i);
    }
  }
  if (status != 0 && last_ok) status = 0;  // out of iterations at reduced accuracy
  for (int i = 0; i < m; ++i) V(L.lam + i) = ((i % 3 == 0) ? imu : 1.0) * V(L.y + i);
  return status;
}

__device__ __forceinline__ V3<double> unit3(V3<double> a) {
  const double n = sqrt(dot(a, a));
  return {a.x / n, a.y / n, a.z / n};
}

// One velocity-stepping step of the lane, in place.  Returns status bits.
__device__ __noinline__ int lane_velocity_step(const LaneCtx<double>& cin, const View V, const VSLayout L,
                                               Col<double> q, Col<double> v, Col<double> tau, bool have_tau,
                                               double dt) {
  LaneCtx<double> c = cin;
  const int nv = c.nv, nh = c.nh;
  // 1. free velocity: sweeps without contact wrenches, keeping every world pose
  LaneCtx<double> cf = c;
  cf.nh = 0;
  cf.nu = 0;
  cf.allx = 1;
  Col<double> none{nullptr};
  Col<double> qdd{&V(L.qdd)};
  int st = lane_sweeps<double, double>(cf, q, v, tau, have_tau, none, false);
  lane_fill<double, double>(cf, 0, 1);
  st |= lane_cholesky_solve<double, double>(cf, qdd);
  if (st) return st;
  for (int i = 0; i < nv; ++i) V(L.vf + i) = v[i] + qdd[i] * dt;
  // 2. contacts: points, then spheres (against every half-space), then cuboid pairs
  int nc = 0;
  for (int pass = 0; pass < 2; ++pass)
    for (int b = 0; b < c.nb; ++b) {
      const uint32_t w1 = c.w(2 * b + 1);
      const int cb0 = (w1 >> 8) & 255, cn = (w1 >> 16) & 255;
      if (!cn) continue;
      M3<double> R;
#pragma unroll
      for (int k = 0; k < 9; ++k) R.a[k] = c.d(c.L.X + 12 * b + k);
      const V3<double> pb{c.d(c.L.X + 12 * b + 9), c.d(c.L.X + 12 * b + 10), c.d(c.L.X + 12 * b + 11)};
      for (int k = cb0; k < cb0 + cn; ++k) {
        const int cd = CTC_D * k;
        const double rad = c.cdd(cd + 4);
        if ((rad > 0.0) != (pass == 1)) continue;
        const V3<double> pw = mul(R, V3<double>{c.cdd(cd), c.cdd(cd + 1), c.cdd(cd + 2)}) + pb;
        for (int h = 0; h < nh; ++h) {
          const int hd = HS_D * h;
          const V3<double> hp{c.hdd(hd), c.hdd(hd + 1), c.hdd(hd + 2)};
          const V3<double> hn{c.hdd(hd + 3), c.hdd(hd + 4), c.hdd(hd + 5)};
          const double d = dot(pw - hp, hn);
          V3<double> at = pw;
          if (pass == 0) {
            if (!(d <= 1e-8)) continue;  // HalfSpace::has_inside
          } else {
            if (!(d <= rad)) continue;   // Sphere::contact_halfspace
            at = pw - hn * d;
          }
          if (nc >= L.mc) return GPB_ST_SOLVER;
          const int e = L.ct + 8 * nc++;
          V(e) = hn.x;
          V(e + 1) = hn.y;
          V(e + 2) = hn.z;
          V(e + 3) = at.x;
          V(e + 4) = at.y;
          V(e + 5) = at.z;
          V(e + 6) = b + 1;
          V(e + 7) = 0;
        }
      }
    }
  if (c.nu > 1) {
    for (int a = 0; a < c.nb; ++a) {
      if (!((c.w(2 * a + 1) >> W1_CUBOID_SHIFT) & 15u)) continue;
      gcol::BoxPose A;
#pragma unroll
      for (int k = 0; k < 9; ++k) A.R[k] = c.d(c.L.X + 12 * a + k);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        A.t[k] = c.d(c.L.X + 12 * a + 9 + k);
        A.dims[k] = c.td(TOPO_D * a + TD_CUBOID + k);
      }
      for (int b = a + 1; b < c.nb; ++b) {
        if (!((c.w(2 * b + 1) >> W1_CUBOID_SHIFT) & 15u)) continue;
        gcol::BoxPose B;
#pragma unroll
        for (int k = 0; k < 9; ++k) B.R[k] = c.d(c.L.X + 12 * b + k);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          B.t[k] = c.d(c.L.X + 12 * b + 9 + k);
          B.dims[k] = c.td(TOPO_D * b + TD_CUBOID + k);
        }
        gcol::D3 ca, cbp;
        const int r = gcol::collide(A, B, true, &ca, &cbp);
        if (r < 0) return GPB_ST_COLLISION;
        if (r != gcol::CG_HIT) continue;
        if (nc >= L.mc) return GPB_ST_SOLVER;
        const V3<double> n = unit3(V3<double>{cbp.x - ca.x, cbp.y - ca.y, cbp.z - ca.z});
        const int e = L.ct + 8 * nc++;
        V(e) = n.x;
        V(e + 1) = n.y;
        V(e + 2) = n.z;
        V(e + 3) = ca.x;
        V(e + 4) = ca.y;
        V(e + 5) = ca.z;
        V(e + 6) = a + 1;
        V(e + 7) = b + 1;
      }
    }
  }
  if (nc > 0) {
    const int m = 3 * nc;
    // 3. Jacobian rows (n, t, b) · (v + ω × p) of the supporting joints' columns
    for (int k = 0; k < nc; ++k) {
      const int e = L.ct + 8 * k;
      const V3<double> n{V(e), V(e + 1), V(e + 2)}, p{V(e + 3), V(e + 4), V(e + 5)};
      const V3<double> cand = cross(n, V3<double>{1.0, 0.0, 0.0});
      const V3<double> t = dot(cand, cand) != 0.0 ? unit3(cand) : unit3(cross(n, V3<double>{0.0, 1.0, 0.0}));
      const V3<double> bb = unit3(cross(n, t));
      uint64_t ma = 0, mb = 0;  // bodies supporting a / b (bit j-1 for body j)
      for (int x = (int)V(e + 6); x != 0; x = (c.w(2 * (x - 1)) >> 4) & 255) ma |= 1ull << (x - 1);
      for (int x = (int)V(e + 7); x != 0; x = (c.w(2 * (x - 1)) >> 4) & 255) mb |= 1ull << (x - 1);
      for (int i = 0; i < 3 * nv; ++i) V(L.J + 3 * k * nv + i) = 0.0;
      for (int j = 0; j < c.nb; ++j) {
        const double sg = ((ma >> j) & 1) ? 1.0 : (((mb >> j) & 1) ? -1.0 : 0.0);
        if (sg == 0.0) continue;
        const uint32_t w0 = c.w(2 * j);
        const int type = w0 & 15, vo = (w0 >> 22) & 1023;
        const int nvj = type == 3 ? 6 : (type == 0 ? 0 : 1);
        for (int col = 0; col < nvj; ++col) {
          const SV<double> s = load_sv(c, c.L.S + 6 * (vo + col));
          const V3<double> pv = s.v + cross(s.w, p);
          V(L.J + (3 * k) * nv + vo + col) = sg * dot(n, pv);
          V(L.J + (3 * k + 1) * nv + vo + col) = sg * dot(t, pv);
          V(L.J + (3 * k + 2) * nv + vo + col) = sg * dot(bb, pv);
        }
      }
    }
    // G = J M⁻¹ Jᵀ (M⁻¹ Jᵀ by the kept Cholesky factor), g = J v_free
    for (int i = 0; i < m; ++i) {
      for (int k = 0; k < nv; ++k) c.x<double>(c.L.rhs + k) = V(L.J + i * nv + k);
      lane_solve<double, double>(c);
      for (int k = 0; k < nv; ++k) V(L.Y + i * nv + k) = c.x<double>(c.L.rhs + k);
    }
    for (int i = 0; i < m; ++i) {
      double gi = 0.0;
      for (int k = 0; k < nv; ++k) gi += V(L.J + i * nv + k) * V(L.vf + k);
      V(L.qv + i) = gi;
      for (int j = 0; j <= i; ++j) {
        double s = 0.0;
        for (int k = 0; k < nv; ++k) s += V(L.J + i * nv + k) * V(L.Y + j * nv + k);
        V(L.P + i * m + j) = s;
        V(L.P + j * m + i) = s;
      }
    }
    // 4. the cone program; v' = v_free + M⁻¹ Jᵀ λ
    if (solve_cones(V, L, nc, 0.95) != 0) return GPB_ST_SOLVER;
    for (int k = 0; k < nv; ++k) {
      double s = 0.0;
      for (int i = 0; i < m; ++i) s += V(L.Y + i * nv + k) * V(L.lam + i);
      V(L.vf + k) = V(L.vf + k) + s;  // M⁻¹Jᵀλ = Σ λ_i (M⁻¹ J_iᵀ)
    }
  }
  for (int i = 0; i < nv; ++i) {
    const double x = V(L.vf + i);
    if (!isfinite(x)) return GPB_ST_NONFINITE;
    v[i] = x;
  }
  advance_q(c, q, v, dt, q);  // compute_new_q with the new velocity
  return 0;
}

}  // namespace vstep
