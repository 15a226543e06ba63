// CUDA kernels (sm_103a) of the batched rigid-body step.
//
// Mapping "lane per instance": one warp owns a pack of 32 instances, one lane
// per instance, and runs the whole step (forward kinematics, twists, bias
// accelerations, contact, Newton–Euler, inward sweep, CRBA fill, Cholesky,
// solve, integrator) serially for its instance.  Every FP64 instruction is
// therefore issued with 32 useful lanes and no redundant work — on GB300 the
// FP64 pipe is the bound of the plain-FP64 form, so work efficiency is what
// counts.  Packs are filled with instances of the same topology class (sorted
// on the host) so lanes stay converged.  A persistent grid pulls packs from a
// device work counter and runs all K steps of a pack before taking the next.
//
// Reference algorithm: gorilla-physics src/dynamics.rs:322-364 (one dynamics
// evaluation), src/integrators.rs:25-39,177-319 (integrators),
// src/simulate.rs:87-112 (the K-step loop).

#include <math.h>
#include <string.h>

#include <mutex>
#include <type_traits>

#include "gpb.h"

#include "gpb_device.cuh"
#include "gpb_ff.cuh"
#include "gpb_internal.h"
#include "gpb_rng.h"
#include "gpb_collide.cuh"

namespace gpb {


__host__ __device__ double open_loop_tau(uint32_t seed, int64_t inst, int64_t block, int32_t dof,
                                         double sigma) {
  return sigma * polar_normal((uint32_t)inst, seed, (uint32_t)block, (uint32_t)dof, RNG_TAG_TAU);
}

// ---------------------------------------------------------------------------
// Lane-strided column accessor: element e of this lane's instance.

template <typename T>
struct Col {
  T* p;
  __device__ __forceinline__ T& operator[](int e) const { return p[(size_t)e * LANES]; }
};
template <typename T>
__device__ __forceinline__ Col<T> col_at(T* base, int64_t row, int lane) {
  return Col<T>{base + row * LANES + lane};
}

template <typename R>
struct RealTopo;
template <>
struct RealTopo<double> {
  __device__ static const double* topo(const DeviceBatch& b) { return b.topoD; }
  __device__ static const double* ctc(const DeviceBatch& b) { return b.ctcD; }
  __device__ static const double* hs(const DeviceBatch& b) { return b.hsD; }
};
template <>
struct RealTopo<float> {
  __device__ static const float* topo(const DeviceBatch& b) { return b.topoF; }
  __device__ static const float* ctc(const DeviceBatch& b) { return b.ctcF; }
  __device__ static const float* hs(const DeviceBatch& b) { return b.hsF; }
};

// Per-lane context for one dynamics evaluation.
template <typename R>
struct LaneCtx {
  int lane, nb, nq, nv, nc, nh, model, chain;
  int kind;     // mechanism kind shared by every lane of the pack (PackDesc::kind)
  int nu;       // cuboid colliders (slots 1..nu in body order)
  int springs;  // prismatic springs act (off for Articulated::free_velocity)
  int armature; // revolute armature adds to M's diagonal: Articulated::free_velocity only
                // (src/hybrid/articulated/mod.rs:244-247; dynamics.rs's mass matrix has none)
  int allx;     // keep every body's world pose in X (velocity stepping)
  double grav;  // gravitational acceleration along −z
  const uint32_t* W;  // topology words (row base applied, lane applied)
  const R* T;         // topology reals
  const int32_t* CI;  // contact ints
  const R* CD;        // contact reals
  const R* HD;        // half-space reals
  const double* TDD;  // the same tables in FP64 (for the FP64 parts of mixed forms)
  const double* CDD;
  const double* HDD;
  ScratchLayout L;
  R* sR;              // scratch viewed as R (row pitch = LANES * 8 bytes)
  double* sD;         // scratch viewed as double
  char* s0;           // scratch row 0, lane 0
  // the mechanism tables are read-only for the whole launch: read them through
  // the non-coherent path, so the loads may be issued early and need no
  // ordering against the scratch stores
  __device__ __forceinline__ uint32_t w(int e) const { return __ldg(W + (size_t)e * LANES); }
  __device__ __forceinline__ R t(int e) const { return __ldg(T + (size_t)e * LANES); }
  __device__ __forceinline__ double td(int e) const { return __ldg(TDD + (size_t)e * LANES); }
  __device__ __forceinline__ double cdd(int e) const { return __ldg(CDD + (size_t)e * LANES); }
  __device__ __forceinline__ double hdd(int e) const { return __ldg(HDD + (size_t)e * LANES); }
  // R-typed scratch element (e in rows of 8-byte words)
  __device__ __forceinline__ R& r(int e) const {
    return *reinterpret_cast<R*>(reinterpret_cast<char*>(sR) + (size_t)e * LANES * 8);
  }
  __device__ __forceinline__ double& d(int e) const { return sD[(size_t)e * LANES]; }
  // T-typed scratch element: the factor and right-hand side are kept in the
  // factorisation's own precision (no conversions on the FP64 pipe)
  template <typename T>
  __device__ __forceinline__ T& x(int e) const {
    return *reinterpret_cast<T*>(s0 + (size_t)e * LANES * 8 + (size_t)lane * sizeof(T));
  }
};

template <typename R>
__device__ __forceinline__ void store_sv(const LaneCtx<R>& c, int base, const SV<R>& s) {
  c.r(base) = s.w.x;
  c.r(base + 1) = s.w.y;
  c.r(base + 2) = s.w.z;
  c.r(base + 3) = s.v.x;
  c.r(base + 4) = s.v.y;
  c.r(base + 5) = s.v.z;
}
template <typename R>
__device__ __forceinline__ SV<R> load_sv(const LaneCtx<R>& c, int base) {
  return {{c.r(base), c.r(base + 1), c.r(base + 2)}, {c.r(base + 3), c.r(base + 4), c.r(base + 5)}};
}
template <typename R>
__device__ __forceinline__ void store_si(const LaneCtx<R>& c, int base, const SI<R>& I) {
#pragma unroll
  for (int k = 0; k < 6; ++k) c.r(base + k) = I.j[k];
  c.r(base + 6) = I.c.x;
  c.r(base + 7) = I.c.y;
  c.r(base + 8) = I.c.z;
  c.r(base + 9) = I.m;
}
template <typename R>
__device__ __forceinline__ SI<R> load_si(const LaneCtx<R>& c, int base) {
  SI<R> I;
#pragma unroll
  for (int k = 0; k < 6; ++k) I.j[k] = c.r(base + k);
  I.c = {c.r(base + 6), c.r(base + 7), c.r(base + 8)};
  I.m = c.r(base + 9);
  return I;
}

// Rotation matrix of a unit quaternion (x, y, z, w).
template <typename R>
__device__ __forceinline__ M3<R> quat_to_mat(R x, R y, R z, R w) {
  R xx = x * x, yy = y * y, zz = z * z, ww = w * w;
  R xy = x * y * R(2), xz = x * z * R(2), yz = y * z * R(2);
  R wx = w * x * R(2), wy = w * y * R(2), wz = w * z * R(2);
  M3<R> m;
  m.a[0] = ww + xx - yy - zz;
  m.a[1] = xy - wz;
  m.a[2] = xz + wy;
  m.a[3] = xy + wz;
  m.a[4] = ww - xx + yy - zz;
  m.a[5] = yz - wx;
  m.a[6] = xz - wy;
  m.a[7] = yz + wx;
  m.a[8] = ww - xx - yy + zz;
  return m;
}

// sin / cos of a joint angle held in double, returned in the sweep precision.
template <typename R>
__device__ __forceinline__ void sincos_q(double q, R* s, R* c);
template <>
__device__ __forceinline__ void sincos_q<double>(double q, double* s, double* c) {
  sincos(q, s, c);
}
template <>
__device__ __forceinline__ void sincos_q<float>(double q, float* s, float* c) {
  // reduce by 2π in double first: float(q) alone loses ~q·6e-8 rad
  const double r = fma(-6.283185307179586477, rint(q * 0.15915494309189533577), q);
  sincosf((float)r, s, c);
}

// Contact force of one point against one half-space (src/contact.rs:260-338),
// or the linear spring–damper law, from the penetration z, the approach speed
// ż = −v·n and the tangential velocity v_t = v + n ż of the contact point.
template <typename R>
__device__ __forceinline__ V3<R> contact_force_parts(int model, R z, R zdot, V3<R> n, V3<R> vt, R k_point,
                                                     R damping, R alpha, R mu) {
  R pi;
  if (model == 1) {
    pi = fmax(k_point * z + damping * zdot, R(0));
  } else {
    // z^1.5 (NaN for z < 0 inside the margin → max(NaN, 0) = 0, like Rust)
    R zn = z * sqrt(z);
    R k = k_point * R(50e3) / (k_point + R(50e3));
    R lam = R(1.5) * alpha * k;
    pi = fmax(lam * zn * zdot + k * zn, R(0));
  }
  V3<R> f = n * pi;
  R vtn = sqrt(dot(vt, vt));
  if (vtn != R(0)) {
    R s = vtn / R(1e-3);
    R mue = s > R(1) ? mu : mu * s;
    R g = -mue * pi / vtn;
    f = f + vt * g;
  }
  return f;
}
// The same law from the contact point's velocity v.
template <typename R>
__device__ __forceinline__ V3<R> contact_force(int model, R z, V3<R> n, V3<R> vel, R k_point,
                                               R damping, R alpha, R mu) {
  const R zdot = -dot(vel, n);
  return contact_force_parts<R>(model, z, zdot, n, vel + n * zdot, k_point, damping, alpha, mu);
}

// ---------------------------------------------------------------------------
// Cuboid colliders (src/contact.rs:191-242).  The outward sweep of each
// dynamics form writes a record per cuboid body (store_cuboid); after it,
// lane_cuboid_pairs runs GJK/EPA on every pair and leaves each body's world
// contact wrench in its record; the form then subtracts that wrench from the
// body's force before its inward sweep.

// World pose, world twist about the world origin (the reference's `twists`)
// and sizes of the cuboid of body b, into slot `slot`.
template <typename R>
__device__ __forceinline__ void store_cuboid(const LaneCtx<R>& c, int slot, int b, const M3<double>& Rw,
                                             V3<double> p, V3<double> om, V3<double> v0) {
  const int u = c.L.U + UREC_D * slot;
#pragma unroll
  for (int k = 0; k < 9; ++k) c.d(u + UR_R + k) = Rw.a[k];
  c.d(u + UR_T) = p.x;
  c.d(u + UR_T + 1) = p.y;
  c.d(u + UR_T + 2) = p.z;
  c.d(u + UR_W) = om.x;
  c.d(u + UR_W + 1) = om.y;
  c.d(u + UR_W + 2) = om.z;
  c.d(u + UR_V) = v0.x;
  c.d(u + UR_V + 1) = v0.y;
  c.d(u + UR_V + 2) = v0.z;
#pragma unroll
  for (int k = 0; k < 3; ++k) c.d(u + UR_DIM + k) = c.td(TOPO_D * b + TD_CUBOID + k);
}
template <typename R>
__device__ __forceinline__ V3<double> rec3(const LaneCtx<R>& c, int e) {
  return {c.d(e), c.d(e + 1), c.d(e + 2)};
}

// calculate_contact_force_collider (src/contact.rs:306-317): Hunt–Crossley
// with k = 5e3 on both shapes, α = 1, μ = 1 (src/contact.rs:260-302); the force
// from B on A.  A zero-depth contact gives a NaN normal, as
// UnitVector3::new_normalize of a zero vector does (the instance then stops as
// non-finite).
__device__ __forceinline__ V3<double> collider_force(V3<double> pa, V3<double> pb, V3<double> vel) {
  const V3<double> pen = pb - pa;
  const double z = sqrt(dot(pen, pen));
  const V3<double> n{pen.x / z, pen.y / z, pen.z / z};
  const double zdot = -dot(vel, n);
  const double k = 5e3 * 5e3 / (5e3 + 5e3);
  const double zn = z * sqrt(z);
  const double pi = fmax(1.5 * 1.0 * k * zn * zdot + k * zn, 0.0);
  V3<double> f = n * pi;
  const V3<double> vt = vel + n * zdot;
  const double vtn = sqrt(dot(vt, vt));
  if (vtn != 0.0) {
    const double sl = vtn / 1e-3;
    const double mue = sl > 1.0 ? 1.0 : sl;
    f = f + vt * (-mue * pi / vtn);
  }
  return f;
}

// Every pair (i < j in body order) of this lane's cuboids through GJK/EPA
// (CollisionDetector, src/collision/mod.rs:48-87); a hit pushes f on the first
// body at its contact point and −f on the second at its own.  Returns
// GPB_ST_COLLISION if a query met a case the reference panics on or ran past
// its storage bounds.
template <typename R>
__device__ __noinline__ int lane_cuboid_pairs(const LaneCtx<R>& cin) {
  const LaneCtx<R> c = cin;
  const int U = c.L.U;
  for (int s = 0; s < c.nu; ++s)
#pragma unroll
    for (int k = 0; k < 6; ++k) c.d(U + UREC_D * s + UR_MOM + k) = 0.0;
  int st = 0;
  for (int a = 0; a + 1 < c.nu; ++a) {
    const int ua = U + UREC_D * a;
    gcol::BoxPose A;
#pragma unroll
    for (int k = 0; k < 9; ++k) A.R[k] = c.d(ua + UR_R + k);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      A.t[k] = c.d(ua + UR_T + k);
      A.dims[k] = c.d(ua + UR_DIM + k);
    }
    for (int b = a + 1; b < c.nu; ++b) {
      const int ub = U + UREC_D * b;
      gcol::BoxPose B;
#pragma unroll
      for (int k = 0; k < 9; ++k) B.R[k] = c.d(ub + UR_R + k);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        B.t[k] = c.d(ub + UR_T + k);
        B.dims[k] = c.d(ub + UR_DIM + k);
      }
      gcol::D3 ca, cb;
      const int r = gcol::collide(A, B, true, &ca, &cb);
      if (r < 0) {
        st |= GPB_ST_COLLISION;
        continue;
      }
      if (r != gcol::CG_HIT) continue;
      const V3<double> pa{ca.x, ca.y, ca.z}, pb{cb.x, cb.y, cb.z};
      const V3<double> va = rec3(c, ua + UR_V) + cross(rec3(c, ua + UR_W), pa);  // Twist::point_velocity
      const V3<double> vb = rec3(c, ub + UR_V) + cross(rec3(c, ub + UR_W), pb);
      const V3<double> f = collider_force(pa, pb, va - vb);
      const V3<double> fm = f * -1.0;
      const V3<double> ma = rec3(c, ua + UR_MOM) + cross(pa, f), fa = rec3(c, ua + UR_FRC) + f;
      const V3<double> mb = rec3(c, ub + UR_MOM) + cross(pb, fm), fb = rec3(c, ub + UR_FRC) + fm;
      c.d(ua + UR_MOM) = ma.x;
      c.d(ua + UR_MOM + 1) = ma.y;
      c.d(ua + UR_MOM + 2) = ma.z;
      c.d(ua + UR_FRC) = fa.x;
      c.d(ua + UR_FRC + 1) = fa.y;
      c.d(ua + UR_FRC + 2) = fa.z;
      c.d(ub + UR_MOM) = mb.x;
      c.d(ub + UR_MOM + 1) = mb.y;
      c.d(ub + UR_MOM + 2) = mb.z;
      c.d(ub + UR_FRC) = fb.x;
      c.d(ub + UR_FRC + 1) = fb.y;
      c.d(ub + UR_FRC + 2) = fb.z;
    }
  }
  return st;
}

// The world wrench (moment about the world origin, force) that the cuboid
// pairs exert on the body of slot `slot`, in the body frame with the moment
// about the body origin: (Rᵀ(m − p × f), Rᵀ f).
template <typename R>
__device__ __forceinline__ SV<double> cuboid_wrench_body(const LaneCtx<R>& c, int slot) {
  const int u = c.L.U + UREC_D * slot;
  M3<double> Rw;
#pragma unroll
  for (int k = 0; k < 9; ++k) Rw.a[k] = c.d(u + UR_R + k);
  const V3<double> p = rec3(c, u + UR_T), m = rec3(c, u + UR_MOM), f = rec3(c, u + UR_FRC);
  const V3<double> mo = m - cross(p, f);
  return {{Rw.a[0] * mo.x + Rw.a[3] * mo.y + Rw.a[6] * mo.z, Rw.a[1] * mo.x + Rw.a[4] * mo.y + Rw.a[7] * mo.z,
           Rw.a[2] * mo.x + Rw.a[5] * mo.y + Rw.a[8] * mo.z},
          {Rw.a[0] * f.x + Rw.a[3] * f.y + Rw.a[6] * f.z, Rw.a[1] * f.x + Rw.a[4] * f.y + Rw.a[7] * f.z,
           Rw.a[2] * f.x + Rw.a[5] * f.y + Rw.a[8] * f.z}};
}

// Offset of H(i, j), i ≥ j, in the tile-major packed lower triangle: 4×4 tiles
// (I, J), I ≥ J, stored one after another (16 words each, row-major inside).
__device__ __forceinline__ int tix(int i, int j) {
  const int I = i >> 2, J = j >> 2;
  return (((I * (I + 1)) >> 1) + J) * 16 + ((i & 3) << 2) + (j & 3);
}
__device__ __forceinline__ int tile(int I, int J) { return (((I * (I + 1)) >> 1) + J) * 16; }

// a·b of two spatial vectors with two independent partial sums.
template <typename R>
__device__ __forceinline__ R sdot2(const SV<R>& a, const SV<R>& b) {
  return (a.w.x * b.w.x + a.w.y * b.w.y + a.w.z * b.w.z) + (a.v.x * b.v.x + a.v.y * b.v.y + a.v.z * b.v.z);
}

template <typename R, typename RC>
__device__ __noinline__ void lane_solve(const LaneCtx<R>& c);

// Diagonal tile J of the left-looking Cholesky H = L Lᵀ: a = A_JJ − Σ_K L_JK
// L_JKᵀ (4×4 register tiles: 16 independent multiply-add chains over 16 loaded
// words), then its own 4×4 factor into tile (J, J) and the reciprocal
// diagonal into D.  Returns GPB_ST_CHOL_FAIL for a non-positive pivot.  Not
// inlined: the one-warp and block-cooperative factorisations call this one
// compiled function, so both round identically.
template <typename R, typename RC>
__device__ __noinline__ int chol_diag(const LaneCtx<R>& cin, int J) {
  const LaneCtx<R> c = cin;
  const int M = c.L.M;
  const int tJJ = M + tile(J, J);
  RC a[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s <= r; ++s) a[r][s] = (c.template x<RC>(tJJ + 4 * r + s));
  for (int K = 0; K < J; ++K) {
    const int tJK = M + tile(J, K);
    RC l[4][4];
#pragma unroll
    for (int e = 0; e < 16; ++e) l[e >> 2][e & 3] = (c.template x<RC>(tJK + e));
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s <= r; ++s)
        a[r][s] -= (l[r][0] * l[s][0] + l[r][1] * l[s][1]) + (l[r][2] * l[s][2] + l[r][3] * l[s][3]);
  }
  int st = 0;
  RC inv[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int s = 0; s <= r; ++s) {
      RC x = a[r][s];
#pragma unroll
      for (int m = 0; m < s; ++m) x -= a[r][m] * a[s][m];
      if (r == s) {
        if (!(x > RC(0))) {
          st |= 2;  // GPB_ST_CHOL_FAIL
          x = RC(1);
        }
        a[r][r] = sqrt(x);
        inv[r] = RC(1) / a[r][r];
      } else {
        a[r][s] = x * inv[s];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int s = 0; s <= r; ++s) c.template x<RC>(tJJ + 4 * r + s) = a[r][s];
    c.template x<RC>(c.L.D + 4 * J + r) = inv[r];
  }
  return st;
}

// Off-diagonal tile (I, J), I > J: b = (A_IJ − Σ_K L_IK L_JKᵀ) L_JJ⁻ᵀ (2 FMAs
// per loaded word).
template <typename R, typename RC>
__device__ __noinline__ void chol_offdiag(const LaneCtx<R>& cin, int I, int J) {
  const LaneCtx<R> c = cin;
  const int M = c.L.M;
  const int tIJ = M + tile(I, J), tJJ = M + tile(J, J);
  RC b[4][4];
#pragma unroll
  for (int e = 0; e < 16; ++e) b[e >> 2][e & 3] = (c.template x<RC>(tIJ + e));
  for (int K = 0; K < J; ++K) {
    const int tIK = M + tile(I, K), tJK = M + tile(J, K);
    RC x[4][4], y[4][4];
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      x[e >> 2][e & 3] = (c.template x<RC>(tIK + e));
      y[e >> 2][e & 3] = (c.template x<RC>(tJK + e));
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int s = 0; s < 4; ++s)
        b[r][s] -= (x[r][0] * y[s][0] + x[r][1] * y[s][1]) + (x[r][2] * y[s][2] + x[r][3] * y[s][3]);
  }
  RC a[4][4], inv[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int s = 0; s <= r; ++s) a[r][s] = c.template x<RC>(tJJ + 4 * r + s);
    inv[r] = c.template x<RC>(c.L.D + 4 * J + r);
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      RC x = b[r][s];
#pragma unroll
      for (int m = 0; m < s; ++m) x -= b[r][m] * a[s][m];
      b[r][s] = x * inv[s];
    }
#pragma unroll
  for (int e = 0; e < 16; ++e) c.template x<RC>(tIJ + e) = b[e >> 2][e & 3];
}

// Identity padding of rows nv..4 nT−1 with I mod nw == w (n padded to a
// multiple of 4).
template <typename R, typename RC>
__device__ __forceinline__ void chol_pad(const LaneCtx<R>& c, int w, int nw) {
  const int nv = c.nv, np = ((nv + 3) >> 2) << 2;
  for (int i = nv; i < np; ++i) {
    if ((i >> 2) % nw != w) continue;
    for (int j = 0; j < i; ++j) c.template x<RC>(c.L.M + tix(i, j)) = RC(0);
    c.template x<RC>(c.L.M + tix(i, i)) = RC(1);
    c.template x<RC>(c.L.rhs + i) = RC(0);
  }
}

// Cholesky H = L Lᵀ (left-looking over 4×4 tiles) and the solves L y = rhs,
// Lᵀ x = y.  Writes q̈ into `qdd`; returns GPB status bits.
template <typename R, typename RC>
__device__ __noinline__ int lane_cholesky_solve(const LaneCtx<R>& cin, Col<double> qdd) {
  const LaneCtx<R> c = cin;  // private copy: stores through scratch pointers cannot alias it
  const int nv = c.nv, nT = (nv + 3) >> 2;
  chol_pad<R, RC>(c, 0, 1);
  int st = 0;
  for (int J = 0; J < nT; ++J) {
    st |= chol_diag<R, RC>(cin, J);
    for (int I = J + 1; I < nT; ++I) chol_offdiag<R, RC>(cin, I, J);
  }
  lane_solve<R, RC>(cin);
  for (int i = 0; i < nv; ++i) {
    const double x = double(c.template x<RC>(c.L.rhs + i));
    qdd[i] = x;
    if (!isfinite(x)) st |= 1;  // GPB_ST_NONFINITE
  }
  return st;
}

// The two triangular solves with the factor left in M / D by
// lane_cholesky_solve, in place on the (padded) rhs vector.
template <typename R, typename RC>
__device__ __noinline__ void lane_solve(const LaneCtx<R>& cin) {
  const LaneCtx<R> c = cin;  // private copy: stores through scratch pointers cannot alias it
  const int nT = (c.nv + 3) >> 2;
  const int M = c.L.M;
  // forward substitution L y = rhs
  for (int I = 0; I < nT; ++I) {
    RC y[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) y[r] = (c.template x<RC>(c.L.rhs + 4 * I + r));
    for (int K = 0; K < I; ++K) {
      const int tIK = M + tile(I, K);
      RC z[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) z[m] = (c.template x<RC>(c.L.rhs + 4 * K + m));
#pragma unroll
      for (int r = 0; r < 4; ++r)
        y[r] -= ((c.template x<RC>(tIK + 4 * r)) * z[0] + (c.template x<RC>(tIK + 4 * r + 1)) * z[1]) +
                ((c.template x<RC>(tIK + 4 * r + 2)) * z[2] + (c.template x<RC>(tIK + 4 * r + 3)) * z[3]);
    }
    const int tII = M + tile(I, I);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      RC x = y[r];
#pragma unroll
      for (int m = 0; m < r; ++m) x -= (c.template x<RC>(tII + 4 * r + m)) * y[m];
      y[r] = x * (c.template x<RC>(c.L.D + 4 * I + r));
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) c.template x<RC>(c.L.rhs + 4 * I + r) = y[r];
  }
  // back substitution Lᵀ x = y
  for (int I = nT - 1; I >= 0; --I) {
    RC x[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) x[r] = (c.template x<RC>(c.L.rhs + 4 * I + r));
    for (int K = I + 1; K < nT; ++K) {
      const int tKI = M + tile(K, I);
      RC z[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) z[m] = (c.template x<RC>(c.L.rhs + 4 * K + m));
#pragma unroll
      for (int r = 0; r < 4; ++r)
        x[r] -= ((c.template x<RC>(tKI + r)) * z[0] + (c.template x<RC>(tKI + 4 + r)) * z[1]) +
                ((c.template x<RC>(tKI + 8 + r)) * z[2] + (c.template x<RC>(tKI + 12 + r)) * z[3]);
    }
    const int tII = M + tile(I, I);
#pragma unroll
    for (int r = 3; r >= 0; --r) {
      RC v = x[r];
#pragma unroll
      for (int m = r + 1; m < 4; ++m) v -= (c.template x<RC>(tII + 4 * m + r)) * x[m];
      x[r] = v * (c.template x<RC>(c.L.D + 4 * I + r));
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) c.template x<RC>(c.L.rhs + 4 * I + r) = x[r];
  }
}

// The sweeps of one dynamics evaluation (src/dynamics.rs:322-364): forward
// kinematics, twists, bias accelerations, contacts and Newton–Euler outward;
// composite inertias and joint forces inward.  Leaves each body's composite
// inertia in the I region, the motion subspaces in S and τ + τ_spring − c in
// rhs (in the factor's precision RC).  Returns GPB_ST_COLLISION if a cuboid
// pair query failed, else 0.
template <typename R, typename RC>
__device__ __noinline__ int lane_sweeps(const LaneCtx<R>& cin, Col<double> q, Col<double> v, Col<double> tau,
                                        bool have_tau, Col<double> cforce, bool want_cf) {
  const LaneCtx<R> c = cin;  // private copy: stores through scratch pointers cannot alias it
  const R g = R(c.grav);
  // ---- outward sweep --------------------------------------------------
  M3<R> Rp;
  V3<R> pp;
  SV<R> Vp, Ap;
  for (int b = 0; b < c.nb; ++b) {
    uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    int type = w0 & 15, parent = (w0 >> 4) & 255, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    uint32_t fl = w1 & 255;
    // parent frame
    M3<R> Rpar;
    V3<R> ppar;
    SV<R> Vpar, Apar;
    if (parent == 0) {
#pragma unroll
      for (int k = 0; k < 9; ++k) Rpar.a[k] = R(0);
      Rpar.a[0] = Rpar.a[4] = Rpar.a[8] = R(1);
      ppar = {R(0), R(0), R(0)};
      Vpar = {{R(0), R(0), R(0)}, {R(0), R(0), R(0)}};
      Apar = {{R(0), R(0), R(0)}, {R(0), R(0), g}};  // inverse gravity (src/dynamics.rs:211-218)
    } else if (parent == b) {
      Rpar = Rp;
      ppar = pp;
      Vpar = Vp;
      Apar = Ap;
    } else {
      int pb = parent - 1;
#pragma unroll
      for (int k = 0; k < 9; ++k) Rpar.a[k] = c.r(c.L.X + 12 * pb + k);
      ppar = {c.r(c.L.X + 12 * pb + 9), c.r(c.L.X + 12 * pb + 10), c.r(c.L.X + 12 * pb + 11)};
      Vpar = load_sv(c, c.L.V + 6 * pb);
      Apar = load_sv(c, c.L.A + 6 * pb);
    }
    const int tb = TOPO_D * b;
    // A = Rpar · Rinit ;  p = ppar + Rpar · tinit
    M3<R> Am;
    if (fl & BF_INIT_ROT_IDENTITY) {
      Am = Rpar;
    } else {
      M3<R> Ri;
#pragma unroll
      for (int k = 0; k < 9; ++k) Ri.a[k] = c.t(tb + TD_RINIT + k);
      Am = mul(Rpar, Ri);
    }
    V3<R> ti{c.t(tb + TD_TINIT), c.t(tb + TD_TINIT + 1), c.t(tb + TD_TINIT + 2)};
    V3<R> pb = ppar + mul(Rpar, ti);
    M3<R> Rb;
    SV<R> vj{{R(0), R(0), R(0)}, {R(0), R(0), R(0)}};  // S q̇ of this joint (world)
    int nvb = 0;
    SV<R> S[6];
    if (type == 1 || type == 2) {  // revolute / prismatic
      V3<R> ax{c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
      V3<R> aw = mul(Am, ax);  // world axis (R_b a = A a)
      if (type == 1) {
        R s, co;
        sincos_q<R>(q[qo], &s, &co);
        if (fl & BF_AXIS_PRINCIPAL) {
          int ai = bf_axis_index(fl);
          R sg = (fl & BF_AXIS_NEG) ? -s : s;
          int i1 = (ai + 1) % 3, i2 = (ai + 2) % 3;
          Rb = Am;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            R a1 = Am.a[3 * r + i1], a2 = Am.a[3 * r + i2];
            Rb.a[3 * r + i1] = a1 * co + a2 * sg;
            Rb.a[3 * r + i2] = a2 * co - a1 * sg;
          }
        } else {
          // Rodrigues: Rot = c 1 + s [a]× + (1−c) a aᵀ ; Rb = A Rot
          R omc = R(1) - co;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            V3<R> ar{Am.a[3 * r], Am.a[3 * r + 1], Am.a[3 * r + 2]};
            V3<R> x = cross(ar, ax);  // row · [a]× = (row × a)ᵀ... row_r [a]× = ar × a
            R d = dot(ar, ax) * omc;
            Rb.a[3 * r] = ar.x * co + x.x * s + ax.x * d;
            Rb.a[3 * r + 1] = ar.y * co + x.y * s + ax.y * d;
            Rb.a[3 * r + 2] = ar.z * co + x.z * s + ax.z * d;
          }
        }
        S[0] = {aw, cross(pb, aw)};
      } else {
        Rb = Am;
        pb = pb + aw * R(q[qo]);
        S[0] = {{R(0), R(0), R(0)}, aw};
      }
      nvb = 1;
      vj = scale(S[0], R(v[vo]));
    } else if (type == 3) {  // floating: pose (x,y,z,w,tx,ty,tz)
      M3<R> Rq = quat_to_mat<R>(R(q[qo]), R(q[qo + 1]), R(q[qo + 2]), R(q[qo + 3]));
      V3<R> tq{R(q[qo + 4]), R(q[qo + 5]), R(q[qo + 6])};
      Rb = mul(Am, Rq);
      pb = pb + mul(Am, tq);
      nvb = 6;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        V3<R> ck = col(Rb, k);
        S[k] = {ck, cross(pb, ck)};
        S[3 + k] = {{R(0), R(0), R(0)}, ck};
      }
      V3<R> om{R(v[vo]), R(v[vo + 1]), R(v[vo + 2])};
      V3<R> lv{R(v[vo + 3]), R(v[vo + 4]), R(v[vo + 5])};
      V3<R> ow = mul(Rb, om);
      vj = {ow, mul(Rb, lv) + cross(pb, ow)};
    } else {  // fixed
      Rb = Am;
    }
    SV<R> Vb = Vpar + vj;
    SV<R> Ab = Apar + crm(Vb, vj);
    for (int k = 0; k < nvb; ++k) store_sv(c, c.L.S + 6 * (vo + k), S[k]);
    // world inertia and Newton–Euler (src/dynamics.rs:41-100)
    SI<R> Ib;
#pragma unroll
    for (int k = 0; k < 6; ++k) Ib.j[k] = c.t(tb + TD_INERTIA + 4 + k);
    Ib.c = {c.t(tb + TD_INERTIA + 1), c.t(tb + TD_INERTIA + 2), c.t(tb + TD_INERTIA + 3)};
    Ib.m = c.t(tb + TD_INERTIA);
    // j order in the table: xx, yy, zz, xy, xz, yz
    SI<R> Iw = to_world(Ib, Rb, pb, (fl & BF_DIAG_INERTIA) != 0);
    SV<R> f = imul(Iw, Ab) + crf(Vb, imul(Iw, Vb));
    // contacts of this body (src/contact.rs:97-128) → f −= W_contact
    int cb = (w1 >> 8) & 255, cn = (w1 >> 16) & 255;
    for (int k = cb; k < cb + cn; ++k) {
      const int cd = CTC_D * k;
      V3<R> loc{c.CD[(size_t)cd * LANES], c.CD[(size_t)(cd + 1) * LANES],
                c.CD[(size_t)(cd + 2) * LANES]};
      R kp = c.CD[(size_t)(cd + 3) * LANES], rad = c.CD[(size_t)(cd + 4) * LANES],
        damp = c.CD[(size_t)(cd + 5) * LANES];
      V3<R> pw = mul(Rb, loc) + pb;
      V3<R> fsum{R(0), R(0), R(0)};
      for (int h = 0; h < c.nh; ++h) {
        const int hd = HS_D * h;
        V3<R> hp{c.HD[(size_t)hd * LANES], c.HD[(size_t)(hd + 1) * LANES], c.HD[(size_t)(hd + 2) * LANES]};
        V3<R> hn{c.HD[(size_t)(hd + 3) * LANES], c.HD[(size_t)(hd + 4) * LANES],
                 c.HD[(size_t)(hd + 5) * LANES]};
        R al = c.HD[(size_t)(hd + 6) * LANES], mu = c.HD[(size_t)(hd + 7) * LANES];
        R dist = dot(pw - hp, hn);
        V3<R> app = pw;
        R pen;
        if (rad > R(0)) {
          if (!(dist - rad <= R(1e-8))) continue;
          pen = rad - dist;
          app = pw - hn * rad;
        } else {
          if (!(dist <= R(1e-8))) continue;  // HalfSpace::has_inside (margin 1e-8)
          pen = -dist;
        }
        V3<R> vel = Vb.v + cross(Vb.w, app);
        V3<R> fc = contact_force<R>(c.model, pen, hn, vel, kp, damp, al, mu);
        f.w = f.w - cross(app, fc);
        f.v = f.v - fc;
        fsum = fsum + fc;
      }
      if (want_cf) {
        int orig = (c.CI[(size_t)k * LANES] >> 8) & 255;
        cforce[3 * orig] = double(fsum.x);
        cforce[3 * orig + 1] = double(fsum.y);
        cforce[3 * orig + 2] = double(fsum.z);
      }
    }
    store_si(c, c.L.I + 10 * b, Iw);
    store_sv(c, c.L.F + 6 * b, f);
    const int uslot = (int)((w1 >> W1_CUBOID_SHIFT) & 15u);
    if (uslot && c.nu > 1) {
      M3<double> Rd;
#pragma unroll
      for (int k = 0; k < 9; ++k) Rd.a[k] = double(Rb.a[k]);
      store_cuboid(c, uslot - 1, b, Rd, V3<double>{double(pb.x), double(pb.y), double(pb.z)},
                   V3<double>{double(Vb.w.x), double(Vb.w.y), double(Vb.w.z)},
                   V3<double>{double(Vb.v.x), double(Vb.v.y), double(Vb.v.z)});
    }
    if (fl & BF_BRANCH || c.allx) {
#pragma unroll
      for (int k = 0; k < 9; ++k) c.r(c.L.X + 12 * b + k) = Rb.a[k];
      c.r(c.L.X + 12 * b + 9) = pb.x;
      c.r(c.L.X + 12 * b + 10) = pb.y;
      c.r(c.L.X + 12 * b + 11) = pb.z;
      store_sv(c, c.L.V + 6 * b, Vb);
      store_sv(c, c.L.A + 6 * b, Ab);
    }
    Rp = Rb;
    pp = pb;
    Vp = Vb;
    Ap = Ab;
  }
  // ---- cuboid pairs: f −= W (world frame, about the world origin) ------
  int st = 0;
  if (c.nu > 1) {
    st = lane_cuboid_pairs(c);
    for (int b = 0; b < c.nb; ++b) {
      const int uslot = (int)((c.w(2 * b + 1) >> W1_CUBOID_SHIFT) & 15u);
      if (!uslot) continue;
      const int u = c.L.U + UREC_D * (uslot - 1);
      const SV<R> f = load_sv(c, c.L.F + 6 * b);
      const SV<R> W{{R(c.d(u + UR_MOM)), R(c.d(u + UR_MOM + 1)), R(c.d(u + UR_MOM + 2))},
                    {R(c.d(u + UR_FRC)), R(c.d(u + UR_FRC + 1)), R(c.d(u + UR_FRC + 2))}};
      store_sv(c, c.L.F + 6 * b, f - W);
    }
  }

  // ---- inward sweep: composite inertia, joint forces ------------------
  SI<R> cI;
  SV<R> cF;
  int ctarget = -1;
  for (int b = c.nb - 1; b >= 0; --b) {
    uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    int type = w0 & 15, parent = (w0 >> 4) & 255, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    SI<R> Ic = load_si(c, c.L.I + 10 * b);
    SV<R> f = load_sv(c, c.L.F + 6 * b);
    if (ctarget == b) {
      iadd(Ic, cI);
      f = f + cF;
    }
    store_si(c, c.L.I + 10 * b, Ic);
    int nvb = type == 3 ? 6 : (type == 0 ? 0 : 1);
    for (int k = 0; k < nvb; ++k) {
      SV<R> Sk = load_sv(c, c.L.S + 6 * (vo + k));
      double rhs = have_tau ? tau[vo + k] : 0.0;
      if (type == 2 && (w1 & BF_SPRING) && c.springs) {  // src/dynamics.rs:298-315
        const int tb = TOPO_D * b;
        double ks = double(c.t(tb + TD_SPRING)), ls = double(c.t(tb + TD_SPRING + 1));
        rhs += -ks * (q[qo] - ls);
      }
      // right-hand side kept in the factorisation's precision
      c.template x<RC>(c.L.rhs + vo + k) = RC(RC(rhs) - RC(sdot(Sk, f)));
    }
    if (parent != 0) {
      int pb = parent - 1;
      if (pb == b - 1) {
        cI = Ic;
        cF = f;
        ctarget = pb;
      } else {
        SI<R> Ip = load_si(c, c.L.I + 10 * pb);
        iadd(Ip, Ic);
        store_si(c, c.L.I + 10 * pb, Ip);
        SV<R> fp = load_sv(c, c.L.F + 6 * pb) + f;
        store_sv(c, c.L.F + 6 * pb, fp);
        ctarget = -1;
      }
    } else {
      ctarget = -1;
    }
  }
  return st;
}

// CRBA fill of the rows of H in the tile rows I with I mod nw == w (all rows
// for nw = 1): row vo+k of body b is F_kᵀ S_l, F_k = Ic_b S_k, for every
// column l of the joint and its ancestors (src/mechanism.rs:592-696).  For a
// tree that is not a chain the owned tile rows are cleared first (non-ancestor
// pairs hold fill-in of the previous factor).  One compiled function serves
// the one-warp and the block-cooperative paths, so both round identically.
template <typename R, typename RC>
__device__ __noinline__ void lane_fill(const LaneCtx<R>& cin, int w, int nw) {
  const LaneCtx<R> c = cin;
  const int nT = (c.nv + 3) >> 2;
  if (!c.chain) {
    for (int I = w; I < nT; I += nw)
      for (int e = tile(I, 0); e < tile(I, I) + 16; ++e) c.template x<RC>(c.L.M + e) = RC(0);
  }
  for (int b = 0; b < c.nb; ++b) {
    const uint32_t w0 = c.w(2 * b);
    const int type = w0 & 15, parent = (w0 >> 4) & 255, vo = (w0 >> 22) & 1023;
    const int nvb = type == 3 ? 6 : (type == 0 ? 0 : 1);
    if (nvb == 0) continue;
    const SI<R> Ic = load_si(c, c.L.I + 10 * b);
    // a revolute joint's armature adds to its diagonal in free_velocity
    // (src/hybrid/articulated/mod.rs:244-247)
    const R arm = type == 1 && c.armature ? c.t(TOPO_D * b + TD_ARMATURE) : R(0);
    for (int k = 0; k < nvb; ++k) {
      const int row = vo + k;
      if ((row >> 2) % nw != w) continue;
      const SV<R> Sk = load_sv(c, c.L.S + 6 * row);
      const SV<R> Fk = imul(Ic, Sk);
      for (int l = 0; l <= k; ++l) {
        const SV<R> Sl = l == k ? Sk : load_sv(c, c.L.S + 6 * (vo + l));
        const R h = sdot2(Fk, Sl);
        c.template x<RC>(c.L.M + tix(row, vo + l)) = RC(l == k ? h + arm : h);
      }
      int a = parent;
      while (a != 0) {
        const uint32_t wa = c.w(2 * (a - 1));
        const int ta = wa & 15, voa = (wa >> 22) & 1023;
        const int nva = ta == 3 ? 6 : (ta == 0 ? 0 : 1);
        for (int l = 0; l < nva; ++l) {
          const SV<R> Sl = load_sv(c, c.L.S + 6 * (voa + l));
          c.template x<RC>(c.L.M + tix(row, voa + l)) = RC(sdot2(Fk, Sl));
        }
        a = (wa >> 4) & 255;
      }
    }
  }
}

// One dynamics evaluation (src/dynamics.rs:322-364): reads q, v, tau (double
// columns), writes q̈ into `qdd`.  Returns GPB status bits.
template <typename R, typename RC>
__device__ __noinline__ int lane_dynamics(const LaneCtx<R>& c, Col<double> q, Col<double> v, Col<double> tau,
                                          bool have_tau, Col<double> qdd, Col<double> cforce, bool want_cf) {
  const int st = lane_sweeps<R, RC>(c, q, v, tau, have_tau, cforce, want_cf);
  lane_fill<R, RC>(c, 0, 1);
  return st | lane_cholesky_solve<R, RC>(c, qdd);
}

#include "gpb_link.cuh"
#include "gpb_aba.cuh"

// MIXED_REFINED: the link-coordinate sweep in FP32 (bias forces, mass matrix,
// Cholesky) gives x0; iterative refinement then solves H δ = τ − ID(q, q̇, x0)
// with the FP32 factor, the residual coming from the same sweep in FP64 without
// the mass matrix, and returns x0 + δ.  The error contracts from e0 ≈ cond·ε32
// by a factor κ ≈ cond·ε32 per step (κ reaches 1e-2 on 48-body chains); a
// second step runs only where the first correction exceeded 1e-4 of max(|q̈|, 1).
// The O(n²)/O(n³) work (fill, factor, solves) stays on the FP32 pipe; the FP64
// pipe does the O(n) residual.
template <typename RC>
__device__ __forceinline__ int refine(const LaneCtx<float>& c, const LaneCtx<double>& c2, Col<double> q,
                                      Col<double> v, Col<double> tau, bool have_tau, Col<double> qdd,
                                      Col<double> cf, bool want_cf) {
  int st = 0;
  for (int it = 0; it < 2; ++it) {
    st |= lane_link<double, RC, true>(c2, q, v, tau, have_tau, qdd, qdd, cf, want_cf && it == 0);
    lane_solve<float, RC>(c);
    double dmax = 0.0, xmax = 1.0;
    for (int i = 0; i < c.nv; ++i) {
      const double d = double(c.template x<RC>(c.L.rhs + i));
      const double x = qdd[i] + d;
      qdd[i] = x;
      dmax = fmax(dmax, fabs(d));
      xmax = fmax(xmax, fabs(x));
      if (!isfinite(x)) st |= 1;  // GPB_ST_NONFINITE
    }
    if (st || !(dmax > 1e-4 * xmax)) break;
  }
  return st;
}
__device__ __noinline__ int lane_dynamics_refined(const LaneCtx<float>& c, const LaneCtx<double>& c2,
                                                  Col<double> q, Col<double> v, Col<double> tau,
                                                  bool have_tau, Col<double> qdd, Col<double> cf,
                                                  bool want_cf) {
  Col<double> none{nullptr};
  int st = lane_link<float, float, false>(c, q, v, tau, have_tau, none, qdd, none, false);
  if (st & 2) {  // FP32 factorisation broke down: factor the same matrix in FP64
    st = lane_link<float, double, false>(c, q, v, tau, have_tau, none, qdd, none, false);
    if (st) return st;
    return refine<double>(c, c2, q, v, tau, have_tau, qdd, cf, want_cf);
  }
  if (st) return st;
  return refine<float>(c, c2, q, v, tau, have_tau, qdd, cf, want_cf);
}

// quaternion_derivative (src/util.rs:83-102) and the pose update of
// euler_step / compute_new_q (src/integrators.rs:247-258,303-313).
__device__ __forceinline__ void pose_advance(Col<double> q, int qo, const double* vel, double dt,
                                             Col<double> qn) {
  double x = q[qo], y = q[qo + 1], z = q[qo + 2], w = q[qo + 3];
  double ox = vel[0], oy = vel[1], oz = vel[2];
  double dw = 0.5 * (-x * ox - y * oy - z * oz);
  double dx = 0.5 * (w * ox - z * oy + y * oz);
  double dy = 0.5 * (z * ox + w * oy - x * oz);
  double dz = 0.5 * (-y * ox + x * oy + w * oz);
  // translation: t += dt · R(q_old) v_lin
  M3<double> Rq = quat_to_mat<double>(x, y, z, w);
  V3<double> td = mul(Rq, V3<double>{vel[3], vel[4], vel[5]});
  double tx = q[qo + 4] + td.x * dt, ty = q[qo + 5] + td.y * dt, tz = q[qo + 6] + td.z * dt;
  double nx = x + dx * dt, ny = y + dy * dt, nz = z + dz * dt, nw = w + dw * dt;
  double inv = 1.0 / ::sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
  qn[qo] = nx * inv;
  qn[qo + 1] = ny * inv;
  qn[qo + 2] = nz * inv;
  qn[qo + 3] = nw * inv;
  qn[qo + 4] = tx;
  qn[qo + 5] = ty;
  qn[qo + 6] = tz;
}

// Advance positions: qn = q + dt·vel (per joint type), vel given as a column.
template <typename R>
__device__ __forceinline__ void advance_q(const LaneCtx<R>& c, Col<double> q, Col<double> vel,
                                          double dt, Col<double> qn) {
  for (int b = 0; b < c.nb; ++b) {
    uint32_t w0 = c.w(2 * b);
    int type = w0 & 15, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    if (type == 1 || type == 2) {
      qn[qo] = q[qo] + vel[vo] * dt;
    } else if (type == 3) {
      double vv[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) vv[k] = vel[vo + k];
      pose_advance(q, qo, vv, dt, qn);
    }
  }
}

#include "gpb_vstep.cuh"

// Dynamics evaluators of the three precision modes (q, v, τ → q̈).
struct EvalFP64 {
  LaneCtx<double> c;
  int algo;  // GPB_ALGO_CRBA / GPB_ALGO_ABA
  __device__ int operator()(Col<double> q, Col<double> v, Col<double> t, bool ht, Col<double> x,
                            Col<double> cf = Col<double>{nullptr}, bool want_cf = false) const {
    if (algo == 1) {
      if (c.kind == KIND_PLANAR_CHAIN) return lane_aba<double, KIND_PLANAR_CHAIN>(c, q, v, t, ht, x, cf, want_cf);
      if (c.kind == KIND_FLOATING_TREE) return lane_aba<double, KIND_FLOATING_TREE>(c, q, v, t, ht, x, cf, want_cf);
      return lane_aba<double, KIND_GENERAL>(c, q, v, t, ht, x, cf, want_cf);
    }
    return lane_dynamics<double, double>(c, q, v, t, ht, x, cf, want_cf);
  }
};
struct EvalMixed {  // CRBA: FP32 sweeps and fill, FP64 Cholesky when n > 12; ABA: double-float articulated inertias
  LaneCtx<float> c;
  int algo;
  __device__ int operator()(Col<double> q, Col<double> v, Col<double> t, bool ht, Col<double> x,
                            Col<double> cf = Col<double>{nullptr}, bool want_cf = false) const {
    if (algo == 1) {
      if (c.kind == KIND_PLANAR_CHAIN) return lane_aba<float, KIND_PLANAR_CHAIN>(c, q, v, t, ht, x, cf, want_cf);
      if (c.kind == KIND_FLOATING_TREE) return lane_aba<float, KIND_FLOATING_TREE>(c, q, v, t, ht, x, cf, want_cf);
      return lane_aba<float, KIND_GENERAL>(c, q, v, t, ht, x, cf, want_cf);
    }
    if (c.nv <= 12) return lane_dynamics<float, float>(c, q, v, t, ht, x, cf, want_cf);
    return lane_dynamics<float, double>(c, q, v, t, ht, x, cf, want_cf);
  }
};
struct EvalRefined {  // FP32 solve + FP64 residual refinement
  LaneCtx<float> c;
  LaneCtx<double> cd;
  __device__ int operator()(Col<double> q, Col<double> v, Col<double> t, bool ht, Col<double> x,
                            Col<double> cf = Col<double>{nullptr}, bool want_cf = false) const {
    return lane_dynamics_refined(c, cd, q, v, t, ht, x, cf, want_cf);
  }
};

template <typename E>
__device__ int lane_step(const E& ev, Col<double> q, Col<double> v, Col<double> tau,
                         bool have_tau, double dt, int integrator) {
  const auto& c = ev.c;
  const int nv = c.nv;
  Col<double> f{&c.d(c.L.facc)};
  Col<double> qs{&c.d(c.L.qs)}, vs{&c.d(c.L.vs)};
  Col<double> tmp{&c.d(c.L.v0)};
  int st = 0;
  if (integrator == 0) {  // semi-implicit Euler (src/integrators.rs:25-39,276-319)
    st |= ev(q, v, tau, have_tau, tmp);
    if (st) return st;
    for (int i = 0; i < nv; ++i) v[i] = v[i] + tmp[i] * dt;
    advance_q(c, q, v, dt, q);
    return st;
  }
  // Runge–Kutta: every stage starts from (q0, v0); positions use v0
  // (src/integrators.rs:177-271).
  // q is not written before the last stage, so it serves as q0.
  Col<double> q0 = q;
  Col<double> k1{&c.d(c.L.v0)};
  st |= ev(q, v, tau, have_tau, k1);
  if (st) return st;
  if (integrator == 1) {  // RK2
    for (int i = 0; i < nv; ++i) vs[i] = v[i] + k1[i] * (dt / 2.0);
    advance_q(c, q0, v, dt / 2.0, qs);
    st |= ev(qs, vs, tau, have_tau, k1);
    if (st) return st;
    advance_q(c, q0, v, dt, q);
    for (int i = 0; i < nv; ++i) v[i] = v[i] + k1[i] * dt;
    return st;
  }
  // RK4
  for (int i = 0; i < nv; ++i) {
    f[i] = k1[i];
    vs[i] = v[i] + k1[i] * (dt / 2.0);
  }
  advance_q(c, q0, v, dt / 2.0, qs);
  st |= ev(qs, vs, tau, have_tau, k1);
  if (st) return st;
  for (int i = 0; i < nv; ++i) {
    f[i] = f[i] + k1[i] * 2.0;
    vs[i] = v[i] + k1[i] * (dt / 2.0);
  }
  // qs already equals q0 + dt/2 · v0
  st |= ev(qs, vs, tau, have_tau, k1);
  if (st) return st;
  for (int i = 0; i < nv; ++i) {
    f[i] = f[i] + k1[i] * 2.0;
    vs[i] = v[i] + k1[i] * dt;
  }
  advance_q(c, q0, v, dt, qs);
  st |= ev(qs, vs, tau, have_tau, k1);
  if (st) return st;
  for (int i = 0; i < nv; ++i) f[i] = (f[i] + k1[i]) / 6.0;
  advance_q(c, q0, v, dt, q);
  for (int i = 0; i < nv; ++i) v[i] = v[i] + f[i] * dt;
  return st;
}

template <typename R>
__device__ __forceinline__ LaneCtx<R> make_ctx(const DeviceBatch& b, const PackDesc& pd, int lane) {
  LaneCtx<R> c;
  c.lane = lane;
  const int32_t* li = b.laneI + pd.lane * LANES + lane;
  c.nb = li[1 * LANES];
  c.nq = li[2 * LANES];
  c.nv = li[3 * LANES];
  c.nc = b.plain ? 0 : li[4 * LANES];  // free_velocity: no contact points
  c.nh = b.plain ? 0 : li[5 * LANES];
  c.model = li[6 * LANES];
  c.nu = b.plain ? 0 : li[7 * LANES];  // free_velocity: no colliders
  c.chain = pd.chain;
  c.kind = pd.kind;
  c.springs = b.plain ? 0 : 1;
  c.armature = b.plain ? 1 : 0;
  c.allx = 0;
  c.grav = b.gravity;
  c.W = b.topoW + pd.topo * 2 * LANES + lane;
  c.T = RealTopo<R>::topo(b) + pd.topo * TOPO_D * LANES + lane;
  c.CI = b.ctcI + pd.ctc * LANES + lane;
  c.CD = RealTopo<R>::ctc(b) + pd.ctc * CTC_D * LANES + lane;
  c.HD = RealTopo<R>::hs(b) + pd.hs * HS_D * LANES + lane;
  c.TDD = b.topoD + pd.topo * TOPO_D * LANES + lane;
  c.CDD = b.ctcD + pd.ctc * CTC_D * LANES + lane;
  c.HDD = b.hsD + pd.hs * HS_D * LANES + lane;
  c.L = scratch_layout(pd.nb, pd.nq, pd.nv, pd.nc, pd.nu);
  c.sD = b.scratch + pd.scr * LANES + lane;
  c.sR = reinterpret_cast<R*>(b.scratch + pd.scr * LANES) + lane;
  c.s0 = reinterpret_cast<char*>(b.scratch + pd.scr * LANES);
  return c;
}

// Step settings and control law of one slot: the launch's, or the request's
// own when the slot holds a serving job.  Built field by field: a modified
// copy of the whole StepParams (136 bytes) was seen to read the launch's dt
// instead of the assigned one in the step kernel (nvcc 13.0, sm_103a), and
// plain per-field values do not depend on how such a copy is lowered.
struct SlotParams {
  int64_t K, step0;
  double dt, sigma, kp, kd;
  uint32_t seed;
  int32_t integrator, control, resample, tau_mode;
};
__device__ __forceinline__ SlotParams slot_params(const DeviceBatch& b, const StepParams& p, int64_t slot) {
  SlotParams s;
  if (b.jobs) {
    const LaneJob& j = b.jobs[slot];
    const int64_t kc = j.chunk > 0 ? j.chunk : p.K;
    s.K = j.steps_left < kc ? j.steps_left : kc;
    s.step0 = j.step_index;
    s.dt = j.dt;
    s.sigma = j.sigma;
    s.kp = j.kp;
    s.kd = j.kd;
    s.seed = j.seed;
    s.integrator = j.integrator;
    s.control = j.control;
    s.resample = j.resample;
    s.tau_mode = j.tau_mode;
  } else {
    s.K = p.K;
    s.step0 = p.step0;
    s.dt = p.dt;
    s.sigma = p.sigma;
    s.kp = p.kp;
    s.kd = p.kd;
    s.seed = p.seed;
    s.integrator = p.integrator;
    s.control = p.control;
    s.resample = p.resample;
    s.tau_mode = p.tau_mode;
  }
  return s;
}

// Control law before a step.
template <typename R>
__device__ __forceinline__ bool control(const LaneCtx<R>& c, const DeviceBatch& b,
                                        const SlotParams& p, int64_t inst, int64_t sidx, bool first,
                                        Col<double> q, Col<double> v, Col<double> tin,
                                        Col<double> tau) {
  if (p.control == 1) {  // open loop
    int rs = p.resample > 0 ? p.resample : 1;
    if (first || sidx % rs == 0) {
      int64_t block = sidx / rs;
      for (int i = 0; i < c.nv; ++i) tau[i] = open_loop_tau(p.seed, inst, block, i, p.sigma);
    }
    return true;
  }
  if (p.control == 2) {  // PD on 1-DOF joints, zero elsewhere
    for (int i = 0; i < c.nv; ++i) tau[i] = 0.0;
    for (int bb = 0; bb < c.nb; ++bb) {
      uint32_t w0 = c.w(2 * bb);
      int type = w0 & 15, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
      if (type == 1 || type == 2) tau[vo] = p.kp * (tin[vo] - q[qo]) + p.kd * -v[vo];
    }
    return true;
  }
  return p.tau_mode != 0;  // host torques live in tin
}

template <int PREC>
struct EvalOf;
template <>
struct EvalOf<0> {
  __device__ static EvalFP64 make(const DeviceBatch& b, const PackDesc& pd, int lane) {
    return EvalFP64{make_ctx<double>(b, pd, lane), b.algorithm};
  }
};
template <>
struct EvalOf<1> {
  __device__ static EvalMixed make(const DeviceBatch& b, const PackDesc& pd, int lane) {
    return EvalMixed{make_ctx<float>(b, pd, lane), b.algorithm};
  }
};
template <>
struct EvalOf<2> {
  __device__ static EvalRefined make(const DeviceBatch& b, const PackDesc& pd, int lane) {
    return EvalRefined{make_ctx<float>(b, pd, lane), make_ctx<double>(b, pd, lane)};
  }
};

#include "gpb_coop.cuh"
#include "gpb_group.cuh"

// The mixed form at three blocks per SM (168 registers per thread): the
// compiler's own allocation for it otherwise grows to 255 with the FP64
// velocity recursion of contact mechanisms, which costs the chains
// (lane-per-instance code without contacts) their spare occupancy.
template <int PREC>
// Resident 4-warp blocks per SM the mixed form's step kernel is compiled for
// (its register budget: 3 blocks = 168 registers a thread, 2 blocks = 255).
#ifndef GPB_MIXED_MIN_BLOCKS
#define GPB_MIXED_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(128, PREC == 1 ? GPB_MIXED_MIN_BLOCKS : 1) simulate_kernel(DeviceBatch b, StepParams p) {
  const int lane = threadIdx.x & 31;
  // packs [0, ncoop): one whole block per pack (large mechanisms, largest first)
  if (PREC != 2 && p.ncoop > 0) {
    __shared__ CoopShared sh;
    __shared__ int s_pk;
    while (true) {
      if (threadIdx.x == 0) s_pk = atomicAdd(b.queue + 1, 1);
      __syncthreads();
      const int pk = s_pk;
      __syncthreads();
      if (pk >= p.ncoop) break;
      coop_pack<PREC == 2 ? 0 : PREC>(b, p, pk, &sh);
    }
  }
  // the rest: one warp per pack
  const int32_t nwork = b.active ? b.nactive : b.npacks;
  while (true) {
    int pk = 0;
    if (lane == 0) {
      const int w = atomicAdd(b.queue, 1) + (b.active ? 0 : p.ncoop);
      pk = w >= nwork ? -1 : (b.active ? b.active[w] : w);
    }
    pk = __shfl_sync(0xffffffffu, pk, 0);
    if (pk < 0) break;
    const PackDesc pd = b.packs[pk];
    if (lane >= pd.count) continue;
    const int64_t slot = (int64_t)pk * LANES + lane;
    // per-slot job of a serving pool: the request's own K, step counter, step
    // size, integrator and control law
    const SlotParams lp = slot_params(b, p, slot);
    const int64_t K = lp.K;
    if (K <= 0) continue;
    const auto ev = EvalOf<PREC>::make(b, pd, lane);
    const auto& c = ev.c;
    int32_t* status = b.status + slot;
    const int64_t inst = b.laneI[pd.lane * LANES + lane];
    Col<double> q = col_at(b.q, pd.q, lane), v = col_at(b.v, pd.v, lane);
    Col<double> tin = col_at(b.tau_in, pd.v, lane);
    Col<double> tau{&c.d(c.L.tau)};
    int64_t done = 0;  // steps this instance completed in this launch
    for (int64_t s = 0; s < K; ++s) {
      if (*status) break;
      const int64_t sidx = lp.step0 + s;
      bool ht = control(c, b, lp, inst, sidx, s == 0, q, v, tin, tau);
      Col<double> tsrc = lp.control == 0 ? tin : tau;
      int st;
      if constexpr (PREC == 0) {  // velocity stepping runs in FP64 only (checked on the host)
        st = lp.integrator == 3 ? vstep::lane_velocity_step(c, vstep::View{b.vscratch + pd.vs * LANES + lane},
                                                             vs_layout(pd.nv, pd.mvs), q, v, tsrc, ht, lp.dt)
                                : lane_step(ev, q, v, tsrc, ht, lp.dt, lp.integrator);
      } else {
        st = lane_step(ev, q, v, tsrc, ht, lp.dt, lp.integrator);
      }
      if (st) {
        *status = st;
        break;
      }
      for (int i = 0; i < c.nq; ++i)
        if (!isfinite(q[i])) *status |= 1;
      done = s + 1;
      if (p.history && p.record_every > 0 && (s + 1) % p.record_every == 0) {
        double* row = p.history + ((s + 1) / p.record_every - 1) * (b.nq_total + b.nv_total);
        const int64_t* qm = b.qmap + pd.q * LANES + lane;
        const int64_t* vm = b.vmap + pd.v * LANES + lane;
        for (int i = 0; i < c.nq; ++i) row[qm[(size_t)i * LANES]] = q[i];
        for (int i = 0; i < c.nv; ++i) row[b.nq_total + vm[(size_t)i * LANES]] = v[i];
      }
    }
    b.done[slot] = done;
    if (b.jobs) {
      LaneJob& j = b.jobs[slot];
      j.steps_left -= done;
      j.step_index += done;
      if (*status) j.steps_left = 0;  // a failed job ends here (step_index = steps run)
      if (j.steps_left == 0) b.finished[atomicAdd(b.nfinished, 1)] = (int32_t)slot;
    }
  }
}

template <int PREC>
__global__ void __launch_bounds__(128) dynamics_kernel(DeviceBatch b, StepParams p) {
  const int lane = threadIdx.x & 31;
  const int pk = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (pk >= b.npacks) return;
  const PackDesc pd = b.packs[pk];
  if (lane >= pd.count) return;
  const auto ev = EvalOf<PREC>::make(b, pd, lane);
  const auto& c = ev.c;
  Col<double> q = col_at(b.q, pd.q, lane), v = col_at(b.v, pd.v, lane);
  Col<double> tin = col_at(b.tau_in, pd.v, lane);
  Col<double> qdd{&c.d(c.L.facc)};
  Col<double> cf{&c.d(c.L.cf)};
  for (int k = 0; k < 3 * c.nc; ++k) cf[k] = 0.0;
  const int st = ev(q, v, tin, p.tau_mode != 0, qdd, cf, true);
  b.status[(int64_t)pk * LANES + lane] |= st;
  const int64_t* vm = b.vmap + pd.v * LANES + lane;
  if (p.free_velocity) {  // Articulated::free_velocity: v + dt·q̈
    for (int i = 0; i < c.nv; ++i) p.qdd_out[vm[(size_t)i * LANES]] = v[i] + qdd[i] * p.vfree_dt;
  } else {
    for (int i = 0; i < c.nv; ++i) p.qdd_out[vm[(size_t)i * LANES]] = qdd[i];
  }
  if (p.cforce_out) {
    const int64_t* cm = b.cmap + pd.ctc * 3 * LANES + lane;
    for (int k = 0; k < 3 * c.nc; ++k) p.cforce_out[cm[(size_t)k * LANES]] = cf[k];
  }
}

__global__ void scatter_kernel(const int64_t* map, int64_t slots, const double* src, double* dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < slots;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = map[i];
    if (u >= 0) dst[i] = src[u];
  }
}
__global__ void gather_kernel(const int64_t* map, int64_t slots, const double* src, double* dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < slots;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t u = map[i];
    if (u >= 0) dst[u] = src[i];
  }
}

__global__ void scatter_words_kernel(ScatterTable table, const uint64_t* key, const uint64_t* bits,
                                     int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint64_t kk = key[k];
  const int t = (int)(kk >> 56);
  const int64_t e = (int64_t)(kk & 0xffffffffffffull);
  if (t >= table.n || e >= table.t[t].count) return;  // the host validates; never write out of bounds
  if (table.t[t].bytes == 8)
    reinterpret_cast<uint64_t*>(table.t[t].base)[e] = bits[k];
  else
    reinterpret_cast<uint32_t*>(table.t[t].base)[e] = (uint32_t)bits[k];
}
cudaError_t launch_scatter_words(const ScatterTable& table, const uint64_t* key, const uint64_t* bits,
                                 int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  scatter_words_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(table, key, bits, n);
  return cudaGetLastError();
}
template <typename T>
__global__ void gather_words_kernel(const T* src, const int64_t* idx, int64_t n, T* dst) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[idx[k]];
}
cudaError_t launch_gather_words(const void* src, int bytes, const int64_t* idx, int64_t n, void* dst,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((n + 255) / 256);
  if (bytes == 8)
    gather_words_kernel<uint64_t><<<g, 256, 0, s>>>((const uint64_t*)src, idx, n, (uint64_t*)dst);
  else
    gather_words_kernel<uint32_t><<<g, 256, 0, s>>>((const uint32_t*)src, idx, n, (uint32_t*)dst);
  return cudaGetLastError();
}

// CollisionDetector queries of independent cuboid pairs, one thread per pair.
__global__ void __launch_bounds__(128) collide_kernel(int64_t n, const double* __restrict__ pa,
                                                      const double* __restrict__ sa, const double* __restrict__ pb,
                                                      const double* __restrict__ sb, int32_t* __restrict__ result,
                                                      double* __restrict__ ca, double* __restrict__ cb) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    gcol::BoxPose A, B;
    gcol::quat_to_matrix(pa[7 * i], pa[7 * i + 1], pa[7 * i + 2], pa[7 * i + 3], A.R);
    gcol::quat_to_matrix(pb[7 * i], pb[7 * i + 1], pb[7 * i + 2], pb[7 * i + 3], B.R);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      A.t[k] = pa[7 * i + 4 + k];
      B.t[k] = pb[7 * i + 4 + k];
      A.dims[k] = sa[3 * i + k];
      B.dims[k] = sb[3 * i + k];
    }
    gcol::D3 x{0.0, 0.0, 0.0}, y{0.0, 0.0, 0.0};
    const int r = gcol::collide(A, B, true, &x, &y);
    result[i] = r;
    if (r != gcol::CG_HIT) x = y = gcol::D3{0.0, 0.0, 0.0};
    ca[3 * i] = x.x;
    ca[3 * i + 1] = x.y;
    ca[3 * i + 2] = x.z;
    cb[3 * i] = y.x;
    cb[3 * i + 1] = y.y;
    cb[3 * i + 2] = y.z;
  }
}

cudaError_t launch_collide(int64_t n, const double* pose_a, const double* size_a, const double* pose_b,
                           const double* size_b, int32_t* result, double* cp_a, double* cp_b, int num_sms,
                           cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((n + 127) / 128, (int64_t)std::max(num_sms, 1) * 16);
  collide_kernel<<<(unsigned)blocks, 128, 0, s>>>(n, pose_a, size_a, pose_b, size_b, result, cp_a, cp_b);
  return cudaGetLastError();
}

cudaError_t launch_simulate(const DeviceBatch& b, const StepParams& p, int num_sms, int warps_per_sm,
                            cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b.queue, 0, 2 * sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  const int threads = 128;
  int per_sm = 0;
  auto kern = p.precision == 2 ? simulate_kernel<2>
                               : (p.precision == 1 ? simulate_kernel<1> : simulate_kernel<0>);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0);
  if (e != cudaSuccess) return e;
  if (warps_per_sm > 0 && warps_per_sm / (threads / 32) < per_sm) per_sm = warps_per_sm / (threads / 32);
  if (per_sm < 1) per_sm = 1;
  const int64_t work = b.active ? b.nactive : b.npacks;
  int64_t want = (work + (threads / 32) - 1) / (threads / 32);
  int64_t grid = (int64_t)num_sms * per_sm;
  if (grid > want) grid = want;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, threads, 0, s>>>(b, p);
  return cudaGetLastError();
}

cudaError_t launch_simulate_group(const DeviceBatch& b, const StepParams& p, int bodies_per_lane, int num_sms,
                                  cudaStream_t s) {
  const bool blk = p.group == 32 * grp::BLK_WARPS;  // a 4-warp block per instance
  if (!(blk || (p.group >= 2 && p.group <= LANES && !(p.group & (p.group - 1)))) || bodies_per_lane < 1 ||
      bodies_per_lane > (blk ? 1 : 2) || p.group_nvp < 0 || p.group_nvp > 2 * LANES)
    return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(b.queue, 0, 2 * sizeof(int32_t), s);
  if (e != cudaSuccess) return e;
  const int threads = 128;
  const size_t smem = blk ? (size_t)(grp::smem_words(p.group_nvp) + grp::BLK_SCAN_WORDS) * sizeof(double)
                          : (size_t)(threads / 32) * (LANES / p.group) * grp::smem_words(p.group_nvp) * sizeof(double);
  auto kern = blk ? group_block_kernel : (bodies_per_lane == 1 ? group_kernel<1> : group_kernel<2>);
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // work items: a pack's 32 / group instances per warp, or one instance per block
  const int64_t items = (int64_t)(b.active ? b.nactive : b.npacks) * (blk ? LANES : p.group);
  int64_t grid = (int64_t)num_sms * per_sm;
  const int64_t want = blk ? items : (items + (threads / 32) - 1) / (threads / 32);
  if (grid > want) grid = want;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, threads, smem, s>>>(b, p);
  return cudaGetLastError();
}

cudaError_t simulate_max_warps_per_sm(int precision, int* warps) {
  auto kern = precision == 2 ? simulate_kernel<2> : (precision == 1 ? simulate_kernel<1> : simulate_kernel<0>);
  int per_sm = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
  *warps = 4 * per_sm;
  return e;
}

cudaError_t launch_dynamics(const DeviceBatch& b, const StepParams& p, cudaStream_t s) {
  const int threads = 128;
  unsigned grid = (unsigned)((b.npacks + 3) / 4);
  if (grid == 0) return cudaSuccess;
  auto kern = p.precision == 2 ? dynamics_kernel<2>
                               : (p.precision == 1 ? dynamics_kernel<1> : dynamics_kernel<0>);
  kern<<<grid, threads, 0, s>>>(b, p);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const int64_t* map, int64_t slots, const double* src, double* dst,
                           cudaStream_t s) {
  if (slots <= 0) return cudaSuccess;
  int64_t blocks = (slots + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  scatter_kernel<<<(unsigned)blocks, 256, 0, s>>>(map, slots, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_gather(const int64_t* map, int64_t slots, const double* src, double* dst,
                          cudaStream_t s) {
  if (slots <= 0) return cudaSuccess;
  int64_t blocks = (slots + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  gather_kernel<<<(unsigned)blocks, 256, 0, s>>>(map, slots, src, dst);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Dynamics without any device allocation.
//
// Some callers cannot allocate device memory when they evaluate the dynamics:
// a control loop with a hard real-time budget, or a host application that hands
// the GPU out through its own memory pool and forbids cudaMalloc after start-up.
// For them the per-instance working memory of one dynamics evaluation (spatial
// quantities, the mass matrix and its factor) lives in the fixed array below
// instead of the batch's scratch buffer.  The array is part of the library
// image: every GPU that loads the library holds GPB_STATIC_SCRATCH_BYTES until
// the process exits.  All calls share it, so calls whose kernels overlap on the
// GPU (on different streams, or from different host threads) race and must be
// ordered by the caller.  The kernel writes every scratch word before it reads
// it (tree-shaped mechanisms clear their mass-matrix triangle in the kernel), so
// nothing is left over from the previous call's contents.

static __device__ __align__(256) double gpb_static_scratch[GPB_STATIC_SCRATCH_BYTES / sizeof(double)];

// Host-side stand-in of the array above is not a device address: the address a
// kernel may use is looked up once per device, with that device current, and
// kept for the life of the process (it does not survive a cudaDeviceReset).
constexpr int kMaxDevices = 64;
static std::mutex g_static_mu;
static double* g_static_ptr[kMaxDevices] = {};

static cudaError_t static_scratch_address(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[device]) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, gpb_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_ptr[device] = p;
  }
  *out = g_static_ptr[device];
  return cudaSuccess;
}

// The dynamics kernel with user-order state read from caller buffers into the
// static scratch (the q / v / τ slots of each instance's scratch layout).
template <typename R>
__global__ void __launch_bounds__(128)
    dynamics_static_kernel(DeviceBatch b, const double* qu, const double* vu,
                           const double* tu, double* qddu) {
  const int lane = threadIdx.x & 31;
  const int pk = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (pk >= b.npacks) return;
  const PackDesc pd = b.packs[pk];
  if (lane >= pd.count) return;
  const auto ev = EvalOf<R::value>::make(b, pd, lane);
  const auto& c = ev.c;
  Col<double> q{&c.d(c.L.qs)}, v{&c.d(c.L.vs)}, tau{&c.d(c.L.tau)}, qdd{&c.d(c.L.facc)};
  const int64_t* qm = b.qmap + pd.q * LANES + lane;
  const int64_t* vm = b.vmap + pd.v * LANES + lane;
  for (int i = 0; i < c.nq; ++i) q[i] = qu[qm[(size_t)i * LANES]];
  for (int i = 0; i < c.nv; ++i) {
    v[i] = vu[vm[(size_t)i * LANES]];
    tau[i] = tu ? tu[vm[(size_t)i * LANES]] : 0.0;
  }
  const int st = ev(q, v, tau, true, qdd);
  b.status[(int64_t)pk * LANES + lane] |= st;
  for (int i = 0; i < c.nv; ++i) qddu[vm[(size_t)i * LANES]] = qdd[i];
}

cudaError_t launch_dynamics_static(const DeviceBatch& batch, int device, int64_t scratch_words,
                                   int precision, const double* q, const double* v,
                                   const double* tau, double* qdd, cudaStream_t s) {
  if (scratch_words > (int64_t)(GPB_STATIC_SCRATCH_BYTES / sizeof(double))) return cudaErrorInvalidValue;
  double* base = nullptr;
  cudaError_t e = static_scratch_address(device, &base);
  if (e != cudaSuccess) return e;
  DeviceBatch b = batch;
  b.scratch = base;
  const int threads = 128;
  unsigned grid = (unsigned)((b.npacks + 3) / 4);
  if (grid == 0) return cudaSuccess;
  if (precision == 1)
    dynamics_static_kernel<std::integral_constant<int, 1>><<<grid, threads, 0, s>>>(b, q, v, tau, qdd);
  else if (precision == 2)
    dynamics_static_kernel<std::integral_constant<int, 2>><<<grid, threads, 0, s>>>(b, q, v, tau, qdd);
  else
    dynamics_static_kernel<std::integral_constant<int, 0>><<<grid, threads, 0, s>>>(b, q, v, tau, qdd);
  return cudaGetLastError();
}

}  // namespace gpb
