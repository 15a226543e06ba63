// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// CPU FP64 restatement of gorilla-physics' continuous step (the Rust crate at
// one-for-all/gorilla-physics, version 0.1.0).  It is the checker for the GPU
// library: only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may
// load it.  It follows the reference's own order of operations (world-frame
// Featherstone RNEA, CRBA with the support-set fill, partial-pivot LU) rather
// than the GPU kernels' restructured form, so that agreement between the two is
// evidence and not a tautology.
//
// Third-party arithmetic: the reference gets its linear algebra from nalgebra
// 0.33.2 (Cargo.lock), which is not vendored.  The restated call sites are
//   UnitQuaternion::from_axis_angle     (src/joint/revolute.rs:99)
//   Isometry3 * Isometry3                (src/spatial/transform.rs:211-222)
//   UnitQuaternion * Vector3             (src/spatial/twist.rs:82-84)
//   UnitQuaternion::to_rotation_matrix   (src/spatial/transform.rs:133-135)
//   UnitQuaternion::from_quaternion      (src/integrators.rs:255,310)
//   DMatrix::lu().solve                  (src/dynamics.rs:267)
// with their textbook formulas (half-angle quaternion, Hamilton product,
// v + w·t + u×t with t = 2u×v, Doolittle LU with partial row pivoting).
// Bit equality with nalgebra is not claimed; the analytic / closed-form /
// RigidBodyDynamics.jl values of the reference's tests pin the results.
//
// Built with -ffp-contract=off so that x86 and Arm hosts agree bit for bit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "collision.h"
#include "gpb.h"
#include "socp.h"

namespace orc {

constexpr double GRAVITY = 9.81;  // src/lib.rs:39

struct V3 {
  double x, y, z;
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

struct M3 {
  double m[3][3];
};
static inline M3 mzero() {
  M3 r;
  std::memset(&r, 0, sizeof(r));
  return r;
}
static inline V3 mul(const M3& a, V3 v) {
  return {a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z,
          a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
          a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}
static inline M3 mul(const M3& a, const M3& b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
  return r;
}
static inline M3 transpose(const M3& a) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
  return r;
}
static inline M3 add(const M3& a, const M3& b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
  return r;
}
static inline M3 sub(const M3& a, const M3& b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
  return r;
}
static inline M3 outer(V3 a, V3 b) {
  M3 r;
  double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[i][j] = av[i] * bv[j];
  return r;
}

// Quaternion with nalgebra's coordinate order in mind: (x, y, z) vector, w scalar.
struct Quat {
  double x, y, z, w;
};
static inline Quat qmul(Quat a, Quat b) {  // Hamilton product
  return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
          a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
          a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w,
          a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
static inline Quat qconj(Quat q) { return {-q.x, -q.y, -q.z, q.w}; }
// UnitQuaternion * Vector3: t = 2 u×v; v' = t w + u×t + v.
static inline V3 qrot(Quat q, V3 v) {
  V3 u{q.x, q.y, q.z};
  V3 t = cross(u, v) * 2.0;
  V3 c = cross(u, t);
  return (t * q.w + c) + v;
}
static inline Quat from_axis_angle(V3 axis, double angle) {
  double half = angle / 2.0;
  double s = std::sin(half), c = std::cos(half);
  return {axis.x * s, axis.y * s, axis.z * s, c};
}
static inline M3 to_rotation_matrix(Quat q) {
  double i = q.x, j = q.y, k = q.z, w = q.w;
  double ww = w * w, ii = i * i, jj = j * j, kk = k * k;
  double ij = i * j * 2.0, wk = w * k * 2.0, wj = w * j * 2.0, ik = i * k * 2.0,
         jk = j * k * 2.0, wi = w * i * 2.0;
  M3 r;
  r.m[0][0] = ww + ii - jj - kk;
  r.m[0][1] = ij - wk;
  r.m[0][2] = wj + ik;
  r.m[1][0] = wk + ij;
  r.m[1][1] = ww - ii + jj - kk;
  r.m[1][2] = jk - wi;
  r.m[2][0] = ik - wj;
  r.m[2][1] = wi + jk;
  r.m[2][2] = ww - ii - jj + kk;
  return r;
}
static inline Quat qnormalize(Quat q) {
  double n = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return {q.x / n, q.y / n, q.z / n, q.w / n};
}

// Isometry3: rotation then translation (maps child-frame points to parent frame).
struct Iso {
  Quat r;
  V3 t;
};
static inline Iso iso_identity() { return {{0, 0, 0, 1}, {0, 0, 0}}; }
static inline Iso iso_mul(const Iso& a, const Iso& b) {  // src/spatial/transform.rs:211-222
  return {qmul(a.r, b.r), a.t + qrot(a.r, b.t)};
}
static inline Iso iso_inv(const Iso& a) {  // src/spatial/transform.rs:125-131
  Quat ri = qconj(a.r);
  return {ri, qrot(ri, -a.t)};
}

// ---------------------------------------------------------------------------
// Spatial quantities (src/spatial/*.rs, src/inertia.rs)

struct SV {  // angular, linear
  V3 ang, lin;
};
static inline SV sv_add(SV a, SV b) { return {a.ang + b.ang, a.lin + b.lin}; }

struct Inertia {  // src/inertia.rs:31-37
  M3 moment;
  V3 cross;
  double mass;
};

// Twist::transform (src/spatial/twist.rs:74-93): quaternion rotate + translation cross.
static inline SV twist_transform(SV tw, const Iso& x) {
  V3 ang = qrot(x.r, tw.ang);
  V3 lin = qrot(x.r, tw.lin) + cross(x.t, ang);
  return {ang, lin};
}
// SpatialAcceleration::transform (src/spatial/spatial_acceleration.rs:33-53): uses rot().
static inline SV accel_transform(SV a, const Iso& x) {
  M3 R = to_rotation_matrix(x.r);
  V3 ang = mul(R, a.ang);
  V3 lin = mul(R, a.lin) + cross(x.t, ang);
  return {ang, lin};
}
// SpatialInertia::transform (src/inertia.rs:106-134).
static Inertia inertia_transform(const Inertia& I, const Iso& x) {
  M3 R = to_rotation_matrix(x.r);
  V3 p = x.t;
  V3 Rmc = mul(R, I.cross);
  V3 mp = p * I.mass;
  V3 mcnew = Rmc + mp;
  M3 X = outer(Rmc, p);
  M3 Y = add(add(X, transpose(X)), outer(mp, p));
  M3 J = sub(mul(mul(R, I.moment), transpose(R)), Y);
  double tr = Y.m[0][0] + Y.m[1][1] + Y.m[2][2];
  M3 trI = mzero();
  trI.m[0][0] = trI.m[1][1] = trI.m[2][2] = tr;
  J = add(J, trI);
  return {J, mcnew, I.mass};
}
static inline void inertia_add(Inertia& a, const Inertia& b) {  // src/inertia.rs:152-162
  a.moment = add(a.moment, b.moment);
  a.cross = a.cross + b.cross;
  a.mass = a.mass + b.mass;
}
// mul_inertia (src/util.rs:18-28)
static inline SV mul_inertia(const Inertia& I, V3 w, V3 v) {
  return {mul(I.moment, w) + cross(I.cross, v), v * I.mass - cross(I.cross, w)};
}

// ---------------------------------------------------------------------------
// Mechanism (src/mechanism.rs:41-58) restated from the flattened tables.

struct Contact {
  V3 loc;
  double k, radius, damping;
};
struct HalfSpace {
  V3 point, normal;
  double alpha, mu;
};
struct Joint {
  int type;
  int parent;  // body number, 0 = world
  Iso init_iso;
  V3 axis;
  double spring_k, spring_l;
  double armature;  // reflected rotor inertia (revolute), src/joint/revolute.rs:29
  int nq, nv, qo, vo;
};
struct Mechanism {
  std::vector<Joint> joints;
  std::vector<Inertia> bodies;
  std::vector<std::vector<Contact>> contacts;  // per body, insertion order
  std::vector<int> contact_index;              // flat contact index per (body, k)
  std::vector<std::vector<int>> contact_ids;
  std::vector<HalfSpace> halfspaces;
  int contact_model;
  std::vector<int> cuboid;          // per body: 1 = cuboid collider
  std::vector<double> cuboid_dims;  // per body: w, d, h
  int nq, nv, ncontacts;
  std::vector<std::vector<int>> supports;  // supports[j] = bodies joint j+1 supports
};

static bool load_mechanism(const gpb_model* m, int64_t inst, Mechanism& out) {
  int32_t j0 = m->joint_offset[inst], j1 = m->joint_offset[inst + 1];
  int nj = j1 - j0;
  out.joints.resize(nj);
  out.bodies.resize(nj);
  out.contacts.assign(nj, {});
  out.contact_ids.assign(nj, {});
  int qo = 0, vo = 0;
  for (int a = 0; a < nj; ++a) {
    int j = j0 + a;
    Joint& J = out.joints[a];
    J.type = m->joint_type[j];
    J.parent = m->joint_parent[j];
    if (J.parent < 0 || J.parent > a) return false;
    const double* iso = m->joint_iso + 7 * (size_t)j;
    J.init_iso = {{iso[0], iso[1], iso[2], iso[3]}, {iso[4], iso[5], iso[6]}};
    const double* ax = m->joint_axis + 3 * (size_t)j;
    J.axis = {ax[0], ax[1], ax[2]};
    J.spring_k = m->joint_spring ? m->joint_spring[2 * (size_t)j] : 0.0;
    J.spring_l = m->joint_spring ? m->joint_spring[2 * (size_t)j + 1] : 0.0;
    J.armature = m->joint_armature ? m->joint_armature[j] : 0.0;
    switch (J.type) {
      case GPB_JOINT_FIXED: J.nq = 0; J.nv = 0; break;
      case GPB_JOINT_REVOLUTE:
      case GPB_JOINT_PRISMATIC: J.nq = 1; J.nv = 1; break;
      case GPB_JOINT_FLOATING: J.nq = 7; J.nv = 6; break;
      default: return false;
    }
    J.qo = qo;
    J.vo = vo;
    qo += J.nq;
    vo += J.nv;
    const double* in = m->body_inertia + 10 * (size_t)j;
    Inertia& I = out.bodies[a];
    I.mass = in[0];
    I.cross = {in[1], in[2], in[3]};
    I.moment = mzero();
    I.moment.m[0][0] = in[4];
    I.moment.m[1][1] = in[5];
    I.moment.m[2][2] = in[6];
    I.moment.m[0][1] = I.moment.m[1][0] = in[7];
    I.moment.m[0][2] = I.moment.m[2][0] = in[8];
    I.moment.m[1][2] = I.moment.m[2][1] = in[9];
  }
  out.nq = qo;
  out.nv = vo;
  int32_t c0 = m->contact_offset ? m->contact_offset[inst] : 0;
  int32_t c1 = m->contact_offset ? m->contact_offset[inst + 1] : 0;
  out.ncontacts = c1 - c0;
  for (int c = c0; c < c1; ++c) {
    int b = m->contact_body[c];
    if (b < 1 || b > nj) return false;
    const double* p = m->contact_params + 6 * (size_t)c;
    out.contacts[b - 1].push_back({{p[0], p[1], p[2]}, p[3], p[4], p[5]});
    out.contact_ids[b - 1].push_back(c - c0);
  }
  int32_t h0 = m->halfspace_offset ? m->halfspace_offset[inst] : 0;
  int32_t h1 = m->halfspace_offset ? m->halfspace_offset[inst + 1] : 0;
  for (int h = h0; h < h1; ++h) {
    const double* p = m->halfspace_params + 8 * (size_t)h;
    out.halfspaces.push_back({{p[0], p[1], p[2]}, {p[3], p[4], p[5]}, p[6], p[7]});
  }
  out.contact_model = m->contact_model ? m->contact_model[inst] : GPB_HUNT_CROSSLEY;
  // cuboid colliders (src/rigid_body.rs:197-199); all-zero sizes = none
  out.cuboid.assign(nj, 0);
  out.cuboid_dims.assign(3 * (size_t)nj, 0.0);
  for (int a = 0; a < nj && m->body_cuboid; ++a) {
    const double* d = m->body_cuboid + 3 * (size_t)(j0 + a);
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) continue;
    if (!(d[0] > 0.0 && d[1] > 0.0 && d[2] > 0.0)) return false;
    out.cuboid[a] = 1;
    for (int e = 0; e < 3; ++e) out.cuboid_dims[3 * (size_t)a + e] = d[e];
  }
  // supports (src/mechanism.rs:118-125)
  out.supports.assign(nj, {});
  for (int a = 0; a < nj; ++a) {
    int body = a + 1;
    out.supports[a].push_back(body);
    int cur = body;
    while (out.joints[cur - 1].parent != 0) {
      int p = out.joints[cur - 1].parent;
      out.supports[p - 1].push_back(body);
      cur = p;
    }
  }
  return true;
}

static bool supports(const Mechanism& M, int joint, int body) {
  for (int b : M.supports[joint - 1])
    if (b == body) return true;
  return false;
}

// Joint transform for the current q (src/joint/revolute.rs:97-102,
// prismatic.rs:82-87, floating.rs:26-31, fixed.rs:6-8).
static Iso joint_transform(const Joint& J, const double* q) {
  switch (J.type) {
    case GPB_JOINT_REVOLUTE: {
      Iso r{from_axis_angle(J.axis, q[J.qo]), {0, 0, 0}};
      return {qmul(J.init_iso.r, r.r), J.init_iso.t};  // Isometry * UnitQuaternion
    }
    case GPB_JOINT_PRISMATIC: {
      V3 tr = J.axis * q[J.qo];
      return {J.init_iso.r, J.init_iso.t + qrot(J.init_iso.r, tr)};  // Isometry * Translation
    }
    case GPB_JOINT_FLOATING: {
      const double* p = q + J.qo;
      Iso pose{{p[0], p[1], p[2], p[3]}, {p[4], p[5], p[6]}};
      return iso_mul(J.init_iso, pose);
    }
    default:
      return J.init_iso;
  }
}

// Joint twist in the child frame (src/spatial/twist.rs:36-61).
static SV joint_twist(const Joint& J, const double* v) {
  switch (J.type) {
    case GPB_JOINT_REVOLUTE: return {J.axis * v[J.vo], {0, 0, 0}};
    case GPB_JOINT_PRISMATIC: return {{0, 0, 0}, J.axis * v[J.vo]};
    case GPB_JOINT_FLOATING: {
      const double* p = v + J.vo;
      return {{p[0], p[1], p[2]}, {p[3], p[4], p[5]}};
    }
    default: return {{0, 0, 0}, {0, 0, 0}};
  }
}

// Motion subspace columns in the child frame (src/joint/*.rs motion_subspace).
static int motion_subspace(const Joint& J, SV* cols) {
  switch (J.type) {
    case GPB_JOINT_REVOLUTE: cols[0] = {J.axis, {0, 0, 0}}; return 1;
    case GPB_JOINT_PRISMATIC: cols[0] = {{0, 0, 0}, J.axis}; return 1;
    case GPB_JOINT_FLOATING: {
      V3 e[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int c = 0; c < 3; ++c) cols[c] = {e[c], {0, 0, 0}};
      for (int c = 0; c < 3; ++c) cols[3 + c] = {{0, 0, 0}, e[c]};
      return 6;
    }
    default: return 0;
  }
}
// GeometricJacobian::transform (src/spatial/geometric_jacobian.rs:87-107): uses rot().
static void jacobian_transform(SV* cols, int n, const Iso& x) {
  M3 R = to_rotation_matrix(x.r);
  for (int c = 0; c < n; ++c) {
    V3 a = mul(R, cols[c].ang);
    V3 l = mul(R, cols[c].lin) + cross(x.t, a);
    cols[c] = {a, l};
  }
}

// The normal force π n plus the regularised Coulomb friction of
// calculate_contact_force (src/contact.rs:260-302).
static V3 friction_force(double pi, V3 normal, V3 velocity, double z_dot, double mu) {
  V3 f_normal = normal * pi;
  V3 v_t = velocity + normal * z_dot;
  double v_t_norm = norm(v_t);
  V3 f_fric{0, 0, 0};
  if (v_t_norm != 0.0) {
    double v_s = 1e-3;
    double s = v_t_norm / v_s;
    double mu_e = s > 1.0 ? mu : mu * s;
    // -μ π (v_t / |v_t|): componentwise division, then the scalar (-μ)·π
    V3 dir{v_t.x / v_t_norm, v_t.y / v_t_norm, v_t.z / v_t_norm};
    f_fric = dir * (-mu_e * pi);
  }
  return f_normal + f_fric;
}

// calculate_contact_force (src/contact.rs:260-302): Hunt–Crossley normal force
// with k = k_a k_b / (k_a + k_b), λ = 1.5 α k.
static V3 hunt_crossley(double z, V3 normal, V3 velocity, double k_a, double k_b, double alpha,
                        double mu) {
  double z_dot = -dot(velocity, normal);
  double zn = std::pow(z, 1.5);
  double k = k_a * k_b / (k_a + k_b);
  double lambda = 3.0 / 2.0 * alpha * k;
  // Rust f64::max returns the non-NaN operand: a NaN z^1.5 (z < 0 within
  // the margin) gives 0, which std::fmax also does.
  double pi = std::fmax(lambda * zn * z_dot + k * zn, 0.0);
  return friction_force(pi, normal, velocity, z_dot, mu);
}

// Point / sphere against a half-space (src/contact.rs:321-338: k_h = 50e3).
// The LINEAR_SPRING_DAMPER law replaces only the normal-force line.
static V3 contact_force(int model, double penetration, V3 normal, V3 velocity, double k_point,
                        double damping, double alpha, double mu) {
  if (model != GPB_LINEAR_SPRING_DAMPER)
    return hunt_crossley(penetration, normal, velocity, k_point, 50e3, alpha, mu);
  double z_dot = -dot(velocity, normal);
  double pi = std::fmax(k_point * penetration + damping * z_dot, 0.0);
  return friction_force(pi, normal, velocity, z_dot, mu);
}

// calculate_contact_force_collider (src/contact.rs:306-317): the force from B
// on A, k = 5e3 for both shapes, α = 1, μ = 1.  A zero-depth contact gives a
// NaN normal, as UnitVector3::new_normalize of a zero vector does.
static V3 collider_force(V3 cp_a, V3 cp_b, V3 velocity) {
  V3 pen = cp_b - cp_a;
  double n = norm(pen);
  V3 normal{pen.x / n, pen.y / n, pen.z / n};
  return hunt_crossley(n, normal, velocity, 5e3, 5e3, 1.0, 1.0);
}

struct Work {
  std::vector<Iso> X;        // bodies_to_root, [0] = world
  std::vector<SV> jt;        // joint twists (child frame)
  std::vector<SV> T;         // world twists, [0] = world
  std::vector<double> M;     // nv x nv
  std::vector<double> c;     // dynamics bias
  std::vector<SV> Wc;        // contact wrench per body, [0] unused
};

static void bodies_to_root(const Mechanism& M, const double* q, std::vector<Iso>& X) {
  int n = (int)M.joints.size();
  X.assign(n + 1, iso_identity());
  for (int a = 0; a < n; ++a) X[a + 1] = iso_mul(X[M.joints[a].parent], joint_transform(M.joints[a], q));
}

static void mass_matrix(const Mechanism& M, const std::vector<Iso>& X, std::vector<double>& H) {
  int n = (int)M.joints.size();
  int nv = M.nv;
  std::vector<double> lower((size_t)nv * nv, 0.0);
  std::vector<std::vector<SV>> S(n, std::vector<SV>(6));
  std::vector<int> dim(n);
  std::vector<Inertia> Iw(n);
  for (int a = 0; a < n; ++a) {
    dim[a] = motion_subspace(M.joints[a], S[a].data());
    jacobian_transform(S[a].data(), dim[a], X[a + 1]);
    Iw[a] = inertia_transform(M.bodies[a], X[a + 1]);
  }
  // compute_crb_inertias (src/mechanism.rs:606-625)
  std::vector<Inertia> Ic(n);
  for (int a = n - 1; a >= 0; --a) {
    Inertia crb = Iw[a];
    for (int ch = 0; ch < n; ++ch)
      if (M.joints[ch].parent == a + 1) inertia_add(crb, Ic[ch]);
    Ic[a] = crb;
  }
  // fill (src/mechanism.rs:652-685)
  int i_index = 0, j_index = 0;
  for (int i = 1; i <= n; ++i) {
    if (M.joints[i - 1].type == GPB_JOINT_FIXED) continue;
    const Inertia& I = Ic[i - 1];
    int nrows = dim[i - 1];
    SV F[6];
    for (int c = 0; c < nrows; ++c) {  // MomentumMatrix::mul (src/momentum.rs:17-32)
      V3 Jw = S[i - 1][c].ang, Jv = S[i - 1][c].lin;
      F[c].ang = mul(I.moment, Jw) + cross(I.cross, Jv);
      F[c].lin = Jv * I.mass - cross(I.cross, Jw);
    }
    for (int j = 1; j <= i; ++j) {
      if (M.joints[j - 1].type == GPB_JOINT_FIXED) continue;
      int ncols = dim[j - 1];
      if (supports(M, j, i)) {
        for (int r = 0; r < nrows; ++r)
          for (int cc = 0; cc < ncols; ++cc) {
            // transpose_mul: angᵀ·ang + linᵀ·lin
            double v = dot(F[r].ang, S[j - 1][cc].ang) + dot(F[r].lin, S[j - 1][cc].lin);
            lower[(size_t)(i_index + r) * nv + (j_index + cc)] = v;
          }
      }
      if (i_index == j_index) {
        i_index += nrows;
        j_index = 0;
      } else {
        j_index += ncols;
      }
    }
  }
  H = lower;
  for (int i = 0; i < nv; ++i)
    for (int j = i + 1; j < nv; ++j) H[(size_t)i * nv + j] = lower[(size_t)j * nv + i];
}

// contact_dynamics (src/contact.rs:97-245): point / sphere contacts against the
// half-spaces, then every pair of cuboid colliders (GJK + EPA in the frame
// translated to the first cuboid, as CollisionDetector does).  Returns 0, or
// GPB_ST_COLLISION where the reference would panic.
static int contact_dynamics(const Mechanism& M, const std::vector<Iso>& X,
                             const std::vector<SV>& T, std::vector<SV>& W, double* force_out) {
  int n = (int)M.joints.size();
  W.assign(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  if (force_out)
    for (int c = 0; c < 3 * M.ncontacts; ++c) force_out[c] = 0.0;
  for (int a = 0; a < n; ++a) {
    const Iso& x = X[a + 1];
    M3 R = to_rotation_matrix(x.r);
    const SV& tw = T[a + 1];
    SV wr{{0, 0, 0}, {0, 0, 0}};
    for (size_t k = 0; k < M.contacts[a].size(); ++k) {
      const Contact& cp = M.contacts[a][k];
      V3 loc = mul(R, cp.loc) + x.t;  // ContactPoint::transform (src/contact.rs:41-58)
      for (const HalfSpace& h : M.halfspaces) {
        V3 app = loc;
        double pen;
        if (cp.radius > 0.0) {
          // sphere vs half-space: center distance d, penetration r - d,
          // force at the sphere point nearest the plane.
          double d = dot(loc - h.point, h.normal);
          if (!(d - cp.radius <= 1e-8)) continue;
          pen = cp.radius - d;
          app = loc - h.normal * cp.radius;
        } else {
          if (!(dot(loc - h.point, h.normal) <= 1e-8)) continue;  // HalfSpace::has_inside
          pen = -dot(loc - h.point, h.normal);                   // compute_contact
        }
        V3 vel = tw.lin + cross(tw.ang, app);  // Twist::point_velocity
        V3 f = contact_force(M.contact_model, pen, h.normal, vel, cp.k, cp.damping, h.alpha, h.mu);
        wr.ang = wr.ang + cross(app, f);  // Wrench::from_force
        wr.lin = wr.lin + f;
        if (force_out) {
          int id = M.contact_ids[a][k];
          force_out[3 * id] += f.x;
          force_out[3 * id + 1] += f.y;
          force_out[3 * id + 2] += f.z;
        }
      }
    }
    W[a + 1] = wr;
  }
  // cuboid pairs (src/contact.rs:191-242); collider poses are the bodies'
  // poses (MechanismState::update_collider_poses, src/mechanism.rs:257-275)
  for (int a = 0; a < n; ++a) {
    if (!M.cuboid[a]) continue;
    for (int b = a + 1; b < n; ++b) {
      if (!M.cuboid[b]) continue;
      const M3 Ra = to_rotation_matrix(X[a + 1].r), Rb = to_rotation_matrix(X[b + 1].r);
      double ra[9], rb[9];
      for (int e = 0; e < 9; ++e) {
        ra[e] = Ra.m[e / 3][e % 3];
        rb[e] = Rb.m[e / 3][e % 3];
      }
      const double ta[3] = {X[a + 1].t.x, X[a + 1].t.y, X[a + 1].t.z};
      const double tb[3] = {X[b + 1].t.x, X[b + 1].t.y, X[b + 1].t.z};
      double ca[3], cb[3];
      const int r = orc_col::collide(ra, ta, &M.cuboid_dims[3 * (size_t)a], rb, tb, &M.cuboid_dims[3 * (size_t)b],
                                     true, ca, cb, nullptr);
      if (r < 0) return GPB_ST_COLLISION;
      if (r != orc_col::COL_HIT) continue;
      const V3 cpa{ca[0], ca[1], ca[2]}, cpb{cb[0], cb[1], cb[2]};
      const V3 va = T[a + 1].lin + cross(T[a + 1].ang, cpa);  // Twist::point_velocity
      const V3 vb = T[b + 1].lin + cross(T[b + 1].ang, cpb);
      const V3 f = collider_force(cpa, cpb, va - vb);
      W[a + 1].ang = W[a + 1].ang + cross(cpa, f);  // Wrench::from_force
      W[a + 1].lin = W[a + 1].lin + f;
      const V3 fn = -f;
      W[b + 1].ang = W[b + 1].ang + cross(cpb, fn);
      W[b + 1].lin = W[b + 1].lin + fn;
    }
  }
  return 0;
}

// dynamics_bias (src/dynamics.rs:233-251) with bias_accelerations (200-224),
// compute_coriolis_bias_accelerations (143-192), newton_euler (41-100) and
// compute_torques (src/spatial/wrench.rs:96-126).
static void dynamics_bias(const Mechanism& M, const std::vector<Iso>& X, const std::vector<SV>& jt,
                          const std::vector<SV>& T, const std::vector<SV>& Wc,
                          std::vector<double>& c, double gravity = GRAVITY) {
  int n = (int)M.joints.size();
  std::vector<SV> cor(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a) {
    Iso root_to_body = iso_inv(X[a + 1]);
    SV bt = twist_transform(T[a + 1], root_to_body);
    const SV& j = jt[a];
    SV ca{cross(bt.ang, j.ang), cross(bt.ang, j.lin) + cross(bt.lin, j.ang)};  // se3_commutator
    ca = accel_transform(ca, X[a + 1]);
    cor[a + 1] = sv_add(cor[M.joints[a].parent], ca);
  }
  std::vector<SV> wr(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a) {
    SV acc{V3{0, 0, 0} + cor[a + 1].ang, V3{0, 0, gravity} + cor[a + 1].lin};
    Inertia I = inertia_transform(M.bodies[a], X[a + 1]);
    const SV& tw = T[a + 1];
    SV f = mul_inertia(I, acc.ang, acc.lin);
    SV h = mul_inertia(I, tw.ang, tw.lin);
    f.ang = f.ang + (cross(tw.ang, h.ang) + cross(tw.lin, h.lin));
    f.lin = f.lin + cross(tw.ang, h.lin);
    wr[a + 1] = f;
  }
  for (int a = 0; a < n; ++a) {
    wr[a + 1].ang = wr[a + 1].ang - Wc[a + 1].ang;
    wr[a + 1].lin = wr[a + 1].lin - Wc[a + 1].lin;
  }
  c.assign(M.nv, 0.0);
  for (int a = n - 1; a >= 0; --a) {
    SV jw = wr[a + 1];
    int p = M.joints[a].parent;
    wr[p].ang = wr[p].ang + jw.ang;
    wr[p].lin = wr[p].lin + jw.lin;
    SV S[6];
    int d = motion_subspace(M.joints[a], S);
    jacobian_transform(S, d, X[a + 1]);
    for (int k = 0; k < d; ++k) c[M.joints[a].vo + k] = dot(S[k].ang, jw.ang) + dot(S[k].lin, jw.lin);
  }
}

// Partial-pivot LU solve in nalgebra's order (Gaussian elimination choosing the
// largest |pivot| in the column, unit-lower forward then upper back substitution).
static bool lu_solve(std::vector<double> A, int n, std::vector<double>& b) {
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  bool ok = true;
  for (int i = 0; i < n; ++i) {
    int piv = i;
    double best = std::fabs(A[(size_t)i * n + i]);
    for (int r = i + 1; r < n; ++r) {
      double v = std::fabs(A[(size_t)r * n + i]);
      if (v > best) {
        best = v;
        piv = r;
      }
    }
    double diag = A[(size_t)piv * n + i];
    if (diag == 0.0) {
      ok = false;
      continue;
    }
    if (piv != i) {
      for (int c = 0; c < n; ++c) std::swap(A[(size_t)i * n + c], A[(size_t)piv * n + c]);
      std::swap(perm[i], perm[piv]);
    }
    double inv = 1.0 / diag;
    for (int r = i + 1; r < n; ++r) {
      A[(size_t)r * n + i] *= inv;
      double l = A[(size_t)r * n + i];
      for (int c = i + 1; c < n; ++c) A[(size_t)r * n + c] -= l * A[(size_t)i * n + c];
    }
  }
  if (!ok) return false;
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[i] = b[perm[i]];
  for (int i = 0; i < n; ++i)
    for (int r = i + 1; r < n; ++r) x[r] -= A[(size_t)r * n + i] * x[i];
  for (int i = n - 1; i >= 0; --i) {
    x[i] /= A[(size_t)i * n + i];
    for (int r = 0; r < i; ++r) x[r] -= A[(size_t)r * n + i] * x[i];
  }
  b = x;
  return true;
}

// Cholesky (row by row) solve, the algorithm the GPU kernels use.
static bool chol_solve(std::vector<double> A, int n, std::vector<double>& b) {
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = A[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        A[(size_t)i * n + i] = std::sqrt(s);
      } else {
        A[(size_t)i * n + j] = s / A[(size_t)j * n + j];
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= A[(size_t)i * n + k] * b[k];
    b[i] = s / A[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int k = i + 1; k < n; ++k) s -= A[(size_t)k * n + i] * b[k];
    b[i] = s / A[(size_t)i * n + i];
  }
  return true;
}

// dynamics_continuous (src/dynamics.rs:322-364).  solver 0 = LU (reference),
// 1 = Cholesky.  Returns 0, GPB_ST_CHOL_FAIL if the solve failed, or
// GPB_ST_COLLISION if the cuboid collision met a case the reference panics on.
static int dynamics(const Mechanism& M, const double* q, const double* v, const double* tau,
                    int solver, double* qdd, double* cforce, Work& w) {
  int n = (int)M.joints.size();
  bodies_to_root(M, q, w.X);
  w.jt.resize(n);
  for (int a = 0; a < n; ++a) w.jt[a] = joint_twist(M.joints[a], v);
  w.T.assign(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a) w.T[a + 1] = sv_add(w.T[M.joints[a].parent], twist_transform(w.jt[a], w.X[a + 1]));
  mass_matrix(M, w.X, w.M);
  const int cst = contact_dynamics(M, w.X, w.T, w.Wc, cforce);
  if (cst) return cst;
  dynamics_bias(M, w.X, w.jt, w.T, w.Wc, w.c);
  std::vector<double> rhs(M.nv);
  for (int i = 0; i < M.nv; ++i) rhs[i] = tau ? tau[i] : 0.0;
  for (int a = 0; a < n; ++a) {  // add_prismatic_joint_spring_force (src/dynamics.rs:298-315)
    const Joint& J = M.joints[a];
    if (J.type == GPB_JOINT_PRISMATIC && J.spring_k != 0.0)
      rhs[J.vo] = rhs[J.vo] + (-J.spring_k * (q[J.qo] - J.spring_l));
  }
  for (int i = 0; i < M.nv; ++i) rhs[i] = rhs[i] - w.c[i];
  if (M.nv == 0) return 0;
  bool ok = solver == 1 ? chol_solve(w.M, M.nv, rhs) : lu_solve(w.M, M.nv, rhs);
  for (int i = 0; i < M.nv; ++i) qdd[i] = rhs[i];
  return ok ? 0 : GPB_ST_CHOL_FAIL;
}

// quaternion_derivative (src/util.rs:83-102): [ẇ, ẋ, ẏ, ż] = ½ mat · ω.
static Quat quat_derivative(Quat q, V3 om) {
  double w = q.w, x = q.x, y = q.y, z = q.z;
  double m[4][3] = {{-x, -y, -z}, {w, -z, y}, {z, w, -x}, {-y, x, w}};
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 3; ++c) m[r][c] = m[r][c] / 2.0;
  double d[4];
  for (int r = 0; r < 4; ++r) d[r] = m[r][0] * om.x + m[r][1] * om.y + m[r][2] * om.z;
  return {d[1], d[2], d[3], d[0]};
}

// Pose update shared by euler_step (src/integrators.rs:247-258) and
// compute_new_q (303-313): the rotation uses the OLD quaternion.
static void pose_advance(const double* q, const double* vel, double dt, double* qn) {
  Quat r{q[0], q[1], q[2], q[3]};
  V3 t{q[4], q[5], q[6]};
  V3 om{vel[0], vel[1], vel[2]}, lin{vel[3], vel[4], vel[5]};
  Quat qd = quat_derivative(r, om);
  V3 td = qrot(r, lin);
  V3 tn = t + td * dt;
  Quat rn = qnormalize({r.x + qd.x * dt, r.y + qd.y * dt, r.z + qd.z * dt, r.w + qd.w * dt});
  qn[0] = rn.x;
  qn[1] = rn.y;
  qn[2] = rn.z;
  qn[3] = rn.w;
  qn[4] = tn.x;
  qn[5] = tn.y;
  qn[6] = tn.z;
}

// euler_step (src/integrators.rs:230-271): v' = v + dt q̈, q' = q + dt v (old v).
static void euler_step(const Mechanism& M, const double* q, const double* v, const double* qdd,
                       double dt, double* qn, double* vn) {
  for (const Joint& J : M.joints) {
    if (J.type == GPB_JOINT_REVOLUTE || J.type == GPB_JOINT_PRISMATIC) {
      vn[J.vo] = v[J.vo] + qdd[J.vo] * dt;
      qn[J.qo] = q[J.qo] + v[J.vo] * dt;
    } else if (J.type == GPB_JOINT_FLOATING) {
      for (int k = 0; k < 6; ++k) vn[J.vo + k] = v[J.vo + k] + qdd[J.vo + k] * dt;
      pose_advance(q + J.qo, v + J.vo, dt, qn + J.qo);
    }
  }
}

// semi_implicit_euler_step + compute_new_q (src/integrators.rs:276-319).
static void sie_step(const Mechanism& M, const double* q, const double* v, const double* qdd,
                     double dt, double* qn, double* vn) {
  for (const Joint& J : M.joints) {
    if (J.type == GPB_JOINT_REVOLUTE || J.type == GPB_JOINT_PRISMATIC) {
      vn[J.vo] = v[J.vo] + qdd[J.vo] * dt;
      qn[J.qo] = q[J.qo] + vn[J.vo] * dt;
    } else if (J.type == GPB_JOINT_FLOATING) {
      for (int k = 0; k < 6; ++k) vn[J.vo + k] = v[J.vo + k] + qdd[J.vo + k] * dt;
      pose_advance(q + J.qo, vn + J.vo, dt, qn + J.qo);
    }
  }
}

// ---------------------------------------------------------------------------
// Velocity stepping (src/integrators.rs:42-51; dynamics_discrete,
// src/dynamics.rs:367-430; collision_detection 520-650;
// solve_constraint_and_contact 652-742; compose_contact_jacobian 744-820).

struct VSContact {
  V3 n, p;   // contact normal (towards body a), contact point (world)
  int a, b;  // body numbers (1-based); b = 0: a static half-space
};

// collision_detection: points inside a half-space (margin 1e-8), spheres
// within their radius (contact at the centre's projection, Sphere::contact_halfspace,
// src/collision/sphere.rs:27-34), then cuboid pairs (normal cp_b − cp_a, point cp_a).
static int vs_contacts(const Mechanism& M, const std::vector<Iso>& X, std::vector<VSContact>& out) {
  const int n = (int)M.joints.size();
  out.clear();
  for (int pass = 0; pass < 2; ++pass)  // ContactPoints, then sphere colliders
    for (int a = 0; a < n; ++a) {
      const M3 R = to_rotation_matrix(X[a + 1].r);
      for (const Contact& cp : M.contacts[a]) {
        if ((cp.radius > 0.0) != (pass == 1)) continue;
        const V3 loc = mul(R, cp.loc) + X[a + 1].t;
        for (const HalfSpace& h : M.halfspaces) {
          const double d = dot(loc - h.point, h.normal);
          if (pass == 0) {
            if (d <= 1e-8) out.push_back({h.normal, loc, a + 1, 0});
          } else if (d <= cp.radius) {
            out.push_back({h.normal, loc - h.normal * d, a + 1, 0});
          }
        }
      }
    }
  for (int a = 0; a < n; ++a) {
    if (!M.cuboid[a]) continue;
    for (int b = a + 1; b < n; ++b) {
      if (!M.cuboid[b]) continue;
      const M3 Ra = to_rotation_matrix(X[a + 1].r), Rb = to_rotation_matrix(X[b + 1].r);
      double ra[9], rb[9];
      for (int e = 0; e < 9; ++e) {
        ra[e] = Ra.m[e / 3][e % 3];
        rb[e] = Rb.m[e / 3][e % 3];
      }
      const double ta[3] = {X[a + 1].t.x, X[a + 1].t.y, X[a + 1].t.z};
      const double tb[3] = {X[b + 1].t.x, X[b + 1].t.y, X[b + 1].t.z};
      double ca[3], cb[3];
      const int r = orc_col::collide(ra, ta, &M.cuboid_dims[3 * (size_t)a], rb, tb, &M.cuboid_dims[3 * (size_t)b],
                                     true, ca, cb, nullptr);
      if (r < 0) return GPB_ST_COLLISION;
      if (r != orc_col::COL_HIT) continue;
      const V3 pa{ca[0], ca[1], ca[2]}, pb{cb[0], cb[1], cb[2]};
      const V3 d = pb - pa;
      const double nd = norm(d);
      out.push_back({{d.x / nd, d.y / nd, d.z / nd}, pa, a + 1, b + 1});
    }
  }
  return 0;
}

static V3 unit(V3 a) {
  const double n = norm(a);
  return {a.x / n, a.y / n, a.z / n};
}

// One velocity-stepping step in place.  Returns status bits; *ncontacts and
// the program's iteration count go to info (may be NULL).
struct VSDetails {  // the program of one step (for tests)
  int nc = 0, iterations = 0;
  std::vector<double> J, Mm, vfree, lambda, vnext;
};

static int velocity_step(const Mechanism& M, double* q, double* v, const double* tau, double dt, Work& w,
                         int* info, VSDetails* det = nullptr) {
  const int n = (int)M.joints.size(), nv = M.nv;
  bodies_to_root(M, q, w.X);
  w.jt.resize(n);
  for (int a = 0; a < n; ++a) w.jt[a] = joint_twist(M.joints[a], v);
  w.T.assign(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a) w.T[a + 1] = sv_add(w.T[M.joints[a].parent], twist_transform(w.jt[a], w.X[a + 1]));
  mass_matrix(M, w.X, w.M);
  w.Wc.assign(n + 1, SV{{0, 0, 0}, {0, 0, 0}});  // no explicit contact wrenches
  dynamics_bias(M, w.X, w.jt, w.T, w.Wc, w.c);
  std::vector<double> t(nv);
  for (int i = 0; i < nv; ++i) t[i] = tau ? tau[i] : 0.0;
  for (int a = 0; a < n; ++a) {  // add_prismatic_joint_spring_force
    const Joint& J = M.joints[a];
    if (J.type == GPB_JOINT_PRISMATIC && J.spring_k != 0.0) t[J.vo] = t[J.vo] + (-J.spring_k * (q[J.qo] - J.spring_l));
  }
  if (nv == 0) return 0;
  // v_free = v + M⁻¹ (τ dt − c dt)   (dynamics_solve(M, c·dt, τ·dt))
  std::vector<double> vf(nv);
  for (int i = 0; i < nv; ++i) vf[i] = t[i] * dt - w.c[i] * dt;
  if (!lu_solve(w.M, nv, vf)) return GPB_ST_CHOL_FAIL;
  for (int i = 0; i < nv; ++i) vf[i] = v[i] + vf[i];
  // contacts and their 3-row Jacobians C X H
  std::vector<VSContact> cts;
  if (int st = vs_contacts(M, w.X, cts)) return st;
  const int nc = (int)cts.size(), m = 3 * nc;
  if (info) info[0] = nc;
  std::vector<double> vn(vf);
  if (nc > 0) {
    std::vector<std::vector<SV>> S(n, std::vector<SV>(6));
    std::vector<int> dim(n);
    for (int a = 0; a < n; ++a) {  // build_jacobian_blocks: world motion-subspace columns
      dim[a] = motion_subspace(M.joints[a], S[a].data());
      jacobian_transform(S[a].data(), dim[a], w.X[a + 1]);
    }
    std::vector<double> Jm((size_t)m * nv, 0.0);
    for (int k = 0; k < nc; ++k) {
      const VSContact& c = cts[k];
      V3 cand = cross(c.n, V3{1, 0, 0});
      const V3 tt = norm(cand) != 0.0 ? unit(cand) : unit(cross(c.n, V3{0, 1, 0}));
      const V3 bb = unit(cross(c.n, tt));
      std::vector<int> ca(n + 1, 0), cb(n + 1, 0);
      for (int x = c.a; x != 0; x = M.joints[x - 1].parent) ca[x] = 1;
      for (int x = c.b; x != 0; x = M.joints[x - 1].parent) cb[x] = 1;
      for (int a = 0; a < n; ++a) {
        const double sg = ca[a + 1] ? 1.0 : (cb[a + 1] ? -1.0 : 0.0);
        if (sg == 0.0) continue;
        const int vo = M.joints[a].vo;
        for (int col = 0; col < dim[a]; ++col) {
          const SV& s = S[a][col];
          const V3 pv = s.lin + cross(s.ang, c.p);  // [−[r]×, I] (ω; v)
          Jm[(size_t)(3 * k) * nv + vo + col] = sg * dot(c.n, pv);
          Jm[(size_t)(3 * k + 1) * nv + vo + col] = sg * dot(tt, pv);
          Jm[(size_t)(3 * k + 2) * nv + vo + col] = sg * dot(bb, pv);
        }
      }
    }
    // G = J M⁻¹ Jᵀ (M⁻¹ by LU, column by column), g = J v_free
    std::vector<double> Minv((size_t)nv * nv);
    for (int j = 0; j < nv; ++j) {
      std::vector<double> e(nv, 0.0);
      e[j] = 1.0;
      if (!lu_solve(w.M, nv, e)) return GPB_ST_CHOL_FAIL;
      for (int i = 0; i < nv; ++i) Minv[(size_t)i * nv + j] = e[i];
    }
    std::vector<double> JMi((size_t)m * nv, 0.0), G((size_t)m * m, 0.0), g(m, 0.0), lam(m, 0.0);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < nv; ++j) {
        double s2 = 0.0;
        for (int k = 0; k < nv; ++k) s2 += Jm[(size_t)i * nv + k] * Minv[(size_t)k * nv + j];
        JMi[(size_t)i * nv + j] = s2;
      }
    for (int i = 0; i < m; ++i) {
      for (int j = 0; j < m; ++j) {
        double s2 = 0.0;
        for (int k = 0; k < nv; ++k) s2 += JMi[(size_t)i * nv + k] * Jm[(size_t)j * nv + k];
        G[(size_t)i * m + j] = s2;
      }
      double s3 = 0.0;
      for (int k = 0; k < nv; ++k) s3 += Jm[(size_t)i * nv + k] * vf[k];
      g[i] = s3;
    }
    if (det) {  // the program, also when it fails
      det->nc = nc;
      det->J = Jm;
      det->Mm = w.M;
      det->vfree = vf;
    }
    orc_socp::Info si;
    const int r = orc_socp::solve(nc, G.data(), g.data(), 0.95, lam.data(), &si);
    if (info) info[1] = si.iterations;
    for (double x : lam)
      if (std::isnan(x) || r != 0) return GPB_ST_SOLVER;
    std::vector<double> imp(nv, 0.0);  // Jᵀ λ
    for (int i = 0; i < m; ++i)
      for (int k = 0; k < nv; ++k) imp[k] += Jm[(size_t)i * nv + k] * lam[i];
    if (!lu_solve(w.M, nv, imp)) return GPB_ST_CHOL_FAIL;
    for (int i = 0; i < nv; ++i) vn[i] = vf[i] + imp[i];
    if (det) {
      det->J = Jm;
      det->lambda = lam;
      det->iterations = si.iterations;
    }
  }
  if (det) {
    det->nc = nc;
    det->Mm = w.M;
    det->vfree = vf;
    det->vnext = vn;
  }
  // compute_new_q with the new velocity (src/integrators.rs:296-319)
  for (const Joint& J : M.joints) {
    if (J.type == GPB_JOINT_REVOLUTE || J.type == GPB_JOINT_PRISMATIC) {
      q[J.qo] = q[J.qo] + vn[J.vo] * dt;
    } else if (J.type == GPB_JOINT_FLOATING) {
      double qn[7];
      pose_advance(q + J.qo, vn.data() + J.vo, dt, qn);
      for (int k = 0; k < 7; ++k) q[J.qo + k] = qn[k];
    }
  }
  for (int i = 0; i < nv; ++i) v[i] = vn[i];
  for (int i = 0; i < M.nq; ++i)
    if (!std::isfinite(q[i])) return GPB_ST_NONFINITE;
  return 0;
}

// One step (src/simulate.rs:20-83) in place.
static int step(const Mechanism& M, double* q, double* v, const double* tau, double dt,
                int integrator, int solver, Work& w) {
  int nq = M.nq, nv = M.nv;
  if (integrator == GPB_VELOCITY_STEPPING) return velocity_step(M, q, v, tau, dt, w, nullptr);
  std::vector<double> qn(q, q + nq), vn(v, v + nv), f1(nv), f2(nv), f3(nv), f4(nv);
  int st = 0;
  if (integrator == GPB_SEMI_IMPLICIT_EULER) {
    st |= dynamics(M, q, v, tau, solver, f1.data(), nullptr, w);
    sie_step(M, q, v, f1.data(), dt, qn.data(), vn.data());
  } else if (integrator == GPB_RUNGE_KUTTA_2) {  // src/integrators.rs:177-193
    std::vector<double> q1(q, q + nq), v1(v, v + nv);
    st |= dynamics(M, q, v, tau, solver, f1.data(), nullptr, w);
    euler_step(M, q, v, f1.data(), dt / 2.0, q1.data(), v1.data());
    st |= dynamics(M, q1.data(), v1.data(), tau, solver, f2.data(), nullptr, w);
    euler_step(M, q, v, f2.data(), dt, qn.data(), vn.data());
  } else {  // RK4, src/integrators.rs:195-225
    std::vector<double> qs(q, q + nq), vs(v, v + nv), ff(nv);
    st |= dynamics(M, q, v, tau, solver, f1.data(), nullptr, w);
    euler_step(M, q, v, f1.data(), dt / 2.0, qs.data(), vs.data());
    st |= dynamics(M, qs.data(), vs.data(), tau, solver, f2.data(), nullptr, w);
    euler_step(M, q, v, f2.data(), dt / 2.0, qs.data(), vs.data());
    st |= dynamics(M, qs.data(), vs.data(), tau, solver, f3.data(), nullptr, w);
    euler_step(M, q, v, f3.data(), dt, qs.data(), vs.data());
    st |= dynamics(M, qs.data(), vs.data(), tau, solver, f4.data(), nullptr, w);
    for (int i = 0; i < nv; ++i) ff[i] = (f1[i] + f2[i] * 2.0 + f3[i] * 2.0 + f4[i]) / 6.0;
    euler_step(M, q, v, ff.data(), dt, qn.data(), vn.data());
  }
  std::memcpy(q, qn.data(), sizeof(double) * nq);
  std::memcpy(v, vn.data(), sizeof(double) * nv);
  return st;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3",
// SC'11) and the Marsaglia polar normal draw used for open-loop torques.

static void philox(uint32_t key0, uint32_t key1, uint32_t ctr[4], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key0, k1 = key1;
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Natural log by range reduction to m ∈ [√½, √2) and the atanh series
// log m = 2 Σ f^(2k+1)/(2k+1), f = (m−1)/(m+1); multiply-adds are explicit
// fma() so that the torque stream is reproducible bit for bit.
static double det_log(double x) {
  int e;
  double m = std::frexp(x, &e);  // x = m 2^e, m ∈ [0.5, 1)
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    e -= 1;
  }
  double f = (m - 1.0) / (m + 1.0);
  double f2 = f * f;
  double s = 0.0;
  for (int k = 12; k >= 0; --k) s = std::fma(s, f2, 1.0 / (2.0 * k + 1.0));
  return std::fma((double)e, 0.69314718055994530942, (2.0 * f) * s);
}

// τ ~ σ N(0,1): Philox key (instance, seed), counter (block, dof, attempt,
// 0x7A17); Marsaglia polar method on two 53-bit uniforms in (−1, 1).
static double open_loop_tau(uint32_t seed, int64_t inst, int64_t block, int32_t dof, double sigma) {
  const double scale = 2.0 / 9007199254740992.0;
  for (uint32_t attempt = 0; attempt < 64; ++attempt) {
    uint32_t ctr[4] = {(uint32_t)block, (uint32_t)dof, attempt, 0x7A17u};
    uint32_t o[4];
    philox((uint32_t)inst, seed, ctr, o);
    double a = (double)((((uint64_t)o[0]) << 21) ^ (o[1] >> 11)) + 0.5;
    double b = (double)((((uint64_t)o[2]) << 21) ^ (o[3] >> 11)) + 0.5;
    double u1 = std::fma(a, scale, -1.0);
    double u2 = std::fma(b, scale, -1.0);
    double s = std::fma(u1, u1, u2 * u2);
    if (s >= 1.0 || s == 0.0) continue;
    return sigma * (u1 * std::sqrt((-2.0 * det_log(s)) / s));
  }
  return 0.0;
}

struct Control {
  int mode;
  uint32_t seed;
  int resample;
  double sigma, kp, kd;
  const double* tau;  // HOST: tau; PD: targets
};

static void control_tau(const Mechanism& M, int64_t inst, int64_t step_index, const Control& c,
                        const double* q, const double* v, double* tau) {
  for (int i = 0; i < M.nv; ++i) tau[i] = 0.0;
  if (c.mode == GPB_CONTROL_HOST_TAU) {
    if (c.tau)
      for (int i = 0; i < M.nv; ++i) tau[i] = c.tau[i];
  } else if (c.mode == GPB_CONTROL_OPEN_LOOP) {
    int64_t block = step_index / (c.resample > 0 ? c.resample : 1);
    for (int i = 0; i < M.nv; ++i) tau[i] = open_loop_tau(c.seed, inst, block, i, c.sigma);
  } else if (c.mode == GPB_CONTROL_PD) {  // form of src/control/quadruped_control.rs:63-66
    for (const Joint& J : M.joints) {
      if (J.nv != 1) continue;
      double target = c.tau ? c.tau[J.vo] : 0.0;
      tau[J.vo] = c.kp * (target - q[J.qo]) + c.kd * -v[J.vo];
    }
  }
}

static void energies(const Mechanism& M, const double* q, const double* v, double* ke, double* pe) {
  Work w;
  int n = (int)M.joints.size();
  bodies_to_root(M, q, w.X);
  std::vector<SV> jt(n);
  for (int a = 0; a < n; ++a) jt[a] = joint_twist(M.joints[a], v);
  std::vector<SV> T(n + 1, SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a) T[a + 1] = sv_add(T[M.joints[a].parent], twist_transform(jt[a], w.X[a + 1]));
  double K = 0.0, P = 0.0;
  for (int a = 0; a < n; ++a) {  // src/mechanism.rs:334-362, src/inertia.rs:180-202
    Inertia I = inertia_transform(M.bodies[a], w.X[a + 1]);
    V3 om = T[a + 1].ang, vl = T[a + 1].lin;
    K += (dot(om, mul(I.moment, om)) + dot(vl, vl * I.mass + cross(om, I.cross) * 2.0)) / 2.0;
    P += M.bodies[a].mass * GRAVITY * w.X[a + 1].t.z;
  }
  *ke = K;
  *pe = P;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C entry points (ctypes).  q / v / tau / outputs are the slices of ONE instance.

extern "C" {

int oracle_dims(const gpb_model* m, int64_t inst, int32_t* nq, int32_t* nv, int32_t* ncontacts) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  *nq = M.nq;
  *nv = M.nv;
  *ncontacts = M.ncontacts;
  return 0;
}

int oracle_dynamics(const gpb_model* m, int64_t inst, const double* q, const double* v,
                    const double* tau, int solver, double* qdd, double* contact_force) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::Work w;
  return orc::dynamics(M, q, v, tau, solver, qdd, contact_force, w);
}

// CollisionDetector::new(A, B) then gjk() and epa() (src/collision/mod.rs:48-87)
// for n pairs of cuboids: pose = (qx, qy, qz, qw, tx, ty, tz), dims = (w, d, h).
// translate = 0 runs gjk / epa on the shapes where they are (the reference's
// gjk / epa unit tests).  result[i] = orc_col outcome code; cp_a / cp_b are
// written for hits; stats (7 ints per pair: GJK iterations, EPA expansions,
// vertices, triangles, edges, heap size, FP64 operations) may be NULL.
int oracle_collide_cuboids(int64_t n, const double* pose_a, const double* dims_a, const double* pose_b,
                           const double* dims_b, int translate, int32_t* result, double* cp_a, double* cp_b,
                           int32_t* stats) {
  for (int64_t i = 0; i < n; ++i) {
    double ra[9], rb[9];
    orc_col::quat_to_matrix(pose_a + 7 * i, ra);
    orc_col::quat_to_matrix(pose_b + 7 * i, rb);
    orc_col::Stats st;
    for (int e = 0; e < 3; ++e) cp_a[3 * i + e] = cp_b[3 * i + e] = 0.0;
    result[i] = orc_col::collide(ra, pose_a + 7 * i + 4, dims_a + 3 * i, rb, pose_b + 7 * i + 4, dims_b + 3 * i,
                                 translate != 0, cp_a + 3 * i, cp_b + 3 * i, &st);
    if (stats) {
      const int32_t v[7] = {st.gjk_iters, st.epa_iters, st.verts, st.tris, st.edges, st.heap, (int32_t)st.flops};
      for (int e = 0; e < 7; ++e) stats[7 * i + e] = v[e];
    }
  }
  return 0;
}

// One velocity-stepping step of instance `inst` with its program: returns the
// status; *nc, and (each sized for max_contacts contacts) J (3nc × nv,
// row-major), M (nv × nv), v_free, λ (3nc), v_next; q, v advanced in place.
int oracle_vs_step(const gpb_model* m, int64_t inst, double* q, double* v, const double* tau, double dt,
                   int max_contacts, int32_t* nc, double* J, double* Mm, double* vfree, double* lambda,
                   double* vnext) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::Work w;
  orc::VSDetails d;
  const int st = orc::velocity_step(M, q, v, tau, dt, w, nullptr, &d);
  *nc = d.nc;
  if (d.nc > max_contacts) return GPB_E_RANGE;
  d.lambda.resize(3 * (size_t)d.nc);
  d.vnext.resize(d.vfree.size());
  std::copy(d.J.begin(), d.J.end(), J);
  std::copy(d.Mm.begin(), d.Mm.end(), Mm);
  std::copy(d.vfree.begin(), d.vfree.end(), vfree);
  std::copy(d.lambda.begin(), d.lambda.end(), lambda);
  std::copy(d.vnext.begin(), d.vnext.end(), vnext);
  return st;
}

// The velocity-stepping friction-cone program on its own (socp.h): nc contacts,
// G row-major (3nc)², g (3nc); info = iterations, residual, gap.
int oracle_socp_solve(int nc, const double* G, const double* g, double mu, double* lambda, double* info) {
  orc_socp::Info in;
  const int r = orc_socp::solve(nc, G, g, mu, lambda, &in);
  if (info) {
    info[0] = in.iterations;
    info[1] = in.residual;
    info[2] = in.gap;
  }
  return r;
}

// Articulated::free_velocity (src/hybrid/articulated/mod.rs:124-199,
// update_mass_matrix 201-262): v + dt · M⁻¹ (τ − c) with the revolute
// armature on M's diagonal (244-247), gravity switchable, no contacts and no
// springs, solved by Cholesky as the reference does (mass_matrix.cholesky()).
int oracle_free_velocity(const gpb_model* m, int64_t inst, const double* q, const double* v,
                         const double* tau, double dt, int gravity_enabled, double* v_free) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::Work w;
  const int n = (int)M.joints.size();
  orc::bodies_to_root(M, q, w.X);
  w.jt.resize(n);
  for (int a = 0; a < n; ++a) w.jt[a] = orc::joint_twist(M.joints[a], v);
  w.T.assign(n + 1, orc::SV{{0, 0, 0}, {0, 0, 0}});
  for (int a = 0; a < n; ++a)
    w.T[a + 1] = orc::sv_add(w.T[M.joints[a].parent], orc::twist_transform(w.jt[a], w.X[a + 1]));
  orc::mass_matrix(M, w.X, w.M);
  for (int a = 0; a < n; ++a) {
    const orc::Joint& J = M.joints[a];
    if (J.nv > 0) w.M[(size_t)J.vo * M.nv + J.vo] += J.armature;
  }
  w.Wc.assign(n + 1, orc::SV{{0, 0, 0}, {0, 0, 0}});
  orc::dynamics_bias(M, w.X, w.jt, w.T, w.Wc, w.c, gravity_enabled ? orc::GRAVITY : 0.0);
  std::vector<double> rhs(M.nv);
  for (int i = 0; i < M.nv; ++i) rhs[i] = (tau ? tau[i] : 0.0) - w.c[i];
  bool ok = M.nv == 0 || orc::chol_solve(w.M, M.nv, rhs);
  for (int i = 0; i < M.nv; ++i) v_free[i] = v[i] + rhs[i] * dt;
  return ok ? 0 : GPB_ST_CHOL_FAIL;
}

int oracle_mass_matrix(const gpb_model* m, int64_t inst, const double* q, double* H) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  std::vector<orc::Iso> X;
  orc::bodies_to_root(M, q, X);
  std::vector<double> h;
  orc::mass_matrix(M, X, h);
  std::memcpy(H, h.data(), sizeof(double) * h.size());
  return 0;
}

int oracle_energy(const gpb_model* m, int64_t inst, const double* q, const double* v, double* ke,
                  double* pe) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::energies(M, q, v, ke, pe);
  return 0;
}

int oracle_step(const gpb_model* m, int64_t inst, double* q, double* v, const double* tau,
                double dt, int integrator, int solver) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::Work w;
  return orc::step(M, q, v, tau, dt, integrator, solver, w);
}

double oracle_open_loop_tau(uint32_t seed, int64_t inst, int64_t block, int32_t dof, double sigma) {
  return orc::open_loop_tau(seed, inst, block, dof, sigma);
}

// simulate (src/simulate.rs:87-112) for K steps with the device-side control
// laws restated; history rows of nq + nv after every record_every-th step.
int oracle_simulate(const gpb_model* m, int64_t inst, double* q, double* v, double dt, int64_t K,
                    int64_t step0, int integrator, int solver, int control_mode, uint32_t seed,
                    int resample, double sigma, double kp, double kd, const double* ctl,
                    int64_t record_every, double* history) {
  orc::Mechanism M;
  if (!orc::load_mechanism(m, inst, M)) return GPB_E_INVAL;
  orc::Work w;
  orc::Control c{control_mode, seed, resample, sigma, kp, kd, ctl};
  std::vector<double> tau(M.nv);
  int st = 0;
  for (int64_t s = 0; s < K; ++s) {
    orc::control_tau(M, inst, step0 + s, c, q, v, tau.data());
    st |= orc::step(M, q, v, tau.data(), dt, integrator, solver, w);
    if (history && record_every > 0 && (s + 1) % record_every == 0) {
      double* row = history + (size_t)((s + 1) / record_every - 1) * (M.nq + M.nv);
      std::memcpy(row, q, sizeof(double) * M.nq);
      std::memcpy(row + M.nq, v, sizeof(double) * M.nv);
    }
  }
  return st;
}

// Many instances on `threads` host threads (the CPU baseline).  q_all / v_all
// are the batch's flattened state with offsets q_off / v_off ([n+1]).
int oracle_simulate_batch(const gpb_model* m, int64_t inst_begin, int64_t inst_end,
                          const int64_t* q_off, const int64_t* v_off, double* q_all,
                          double* v_all, double dt, int64_t K, int64_t step0, int integrator,
                          int solver, int control_mode, uint32_t seed, int resample, double sigma,
                          double kp, double kd, const double* ctl_all, int threads) {
  if (threads < 1) threads = 1;
  std::vector<std::thread> pool;
  std::vector<int> rc(threads, 0);
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t]() {
      for (int64_t i = inst_begin + t; i < inst_end; i += threads) {
        const double* ctl = ctl_all ? ctl_all + v_off[i] : nullptr;
        int r = oracle_simulate(m, i, q_all + q_off[i], v_all + v_off[i], dt, K, step0, integrator,
                                solver, control_mode, seed, resample, sigma, kp, kd, ctl, 0, nullptr);
        if (r < 0) rc[t] = r;
      }
    });
  }
  for (auto& th : pool) th.join();
  for (int r : rc)
    if (r < 0) return r;
  return 0;
}

}  // extern "C"
