// Seeded builders of the benchmark mechanisms (gpb_config_sizes /
// gpb_config_build).  Every draw comes from Philox4x32-10 keyed by
// (instance, seed) with a per-quantity counter, so any subset of a batch can be
// rebuilt alone and host / device agree.
//
// Geometry follows the reference's builders:
//  - links: joint frame at the proximal end, next joint at (0, 0, −l) like
//    build_double_pendulum (src/helpers.rs:49-83) and the rod inertia of
//    src/control/mod.rs:152-156 (moment about the joint, cross part (0,0,−ml/2));
//  - cube: RigidBody::new_cube (src/rigid_body.rs:147-158) with the 8 corner
//    points of add_cube_contacts (src/helpers.rs:388-421);
//  - torso: RigidBody::new_cuboid (src/rigid_body.rs:160-173).

#include <cmath>
#include <cstring>
#include <vector>

#include "gpb.h"
#include "gpb_rng.h"

namespace {

constexpr double PI = 3.14159265358979323846;

struct Draw {
  uint32_t inst, seed, tag;
  uint32_t idx = 0;
  double uniform(double a, double b) {
    double u = gpb::philox_uniform(inst, seed, idx++, 0, tag);
    return a + (b - a) * u;
  }
  double normal(double sd) { return sd * gpb::polar_normal(inst, seed, idx++, 1, tag); }
  int integer(int lo, int hi) {  // uniform on {lo..hi}
    double u = gpb::philox_uniform(inst, seed, idx++, 2, tag);
    int k = lo + (int)std::floor(u * (hi - lo + 1));
    return k > hi ? hi : k;
  }
};

struct Builder {
  // outputs (NULL while only counting)
  int32_t *jo, *jt, *jp;
  double *iso, *axis, *spring, *inertia;
  int32_t *co, *cb;
  double* cp;
  int32_t *ho;
  double* hp;
  int32_t* cm;
  double *q0, *v0, *aux;
  int64_t nj = 0, nc = 0, nh = 0, nq = 0, nv = 0;

  void joint(int type, int parent, const double q[4], const double t[3], const double ax[3],
             double mass, const double cross[3], const double moment[6]) {
    if (jt) {
      jt[nj] = type;
      jp[nj] = parent;
      for (int e = 0; e < 4; ++e) iso[7 * nj + e] = q[e];
      for (int e = 0; e < 3; ++e) iso[7 * nj + 4 + e] = t[e];
      for (int e = 0; e < 3; ++e) axis[3 * nj + e] = ax[e];
      spring[2 * nj] = 0.0;
      spring[2 * nj + 1] = 0.0;
      inertia[10 * nj] = mass;
      for (int e = 0; e < 3; ++e) inertia[10 * nj + 1 + e] = cross[e];
      for (int e = 0; e < 6; ++e) inertia[10 * nj + 4 + e] = moment[e];
    }
    nj++;
  }
  void contact(int body, double x, double y, double z, double k, double r, double c) {
    if (cb) {
      cb[nc] = body;
      double* p = cp + 6 * nc;
      p[0] = x;
      p[1] = y;
      p[2] = z;
      p[3] = k;
      p[4] = r;
      p[5] = c;
    }
    nc++;
  }
  void ground(double alpha, double mu) {
    if (hp) {
      double* p = hp + 8 * nh;
      p[0] = p[1] = p[2] = 0.0;
      p[3] = 0.0;
      p[4] = 0.0;
      p[5] = 1.0;
      p[6] = alpha;
      p[7] = mu;
    }
    nh++;
  }
  void qv(double q, double v) {
    if (q0) {
      q0[nq] = q;
      v0[nv] = v;
      if (aux) aux[nv] = 0.0;
    }
    nq++;
    nv++;
  }
};

const double IDQ[4] = {0, 0, 0, 1};
const double ZERO3[3] = {0, 0, 0};

// Uniform rod of length l and mass m about its proximal end, along −z, with
// radius r (r = 0: the thin rod of src/control/mod.rs:152-156).
void rod(double m, double l, double r, double* cross, double* moment) {
  cross[0] = 0.0;
  cross[1] = 0.0;
  cross[2] = -m * l / 2.0;
  double perp = m * l * l / 3.0 + m * r * r / 4.0;
  moment[0] = perp;
  moment[1] = perp;
  moment[2] = m * r * r / 2.0;
  moment[3] = moment[4] = moment[5] = 0.0;
}

void build_one(int config, int64_t inst, uint32_t seed, int contact_model, Builder& B) {
  Draw d{(uint32_t)inst, seed, (uint32_t)(0xC0F0 + config)};
  if (config == 0) {  // acrobot
    double ax[3] = {0, 1, 0};
    double ls[2] = {1.0, 2.0};
    double c[3], mo[6];
    for (int k = 0; k < 2; ++k) {
      rod(1.0, ls[k], 0.0, c, mo);
      double t[3] = {0, 0, k == 0 ? 0.0 : -ls[0]};
      B.joint(GPB_JOINT_REVOLUTE, k, IDQ, t, ax, 1.0, c, mo);
    }
    for (int k = 0; k < 2; ++k) {
      double q = d.uniform(-PI, PI);
      double v = d.normal(0.5);
      B.qv(q, v);
    }
  } else if (config == 1) {  // serial chain
    // Each rod points away from its joint perpendicular to the joint's own axis
    // (axis x or y: rod along −z; axis z: rod along −x), so that no joint spins
    // its own link about the link's long axis (a near-zero inertia that makes
    // the chain ill-posed).  Rod radius 0.05·l.
    int n = d.integer(2, 48);
    double prev[3] = {0, 0, 0};
    for (int k = 0; k < n; ++k) {
      int a = d.integer(0, 2);
      double ax[3] = {0, 0, 0};
      ax[a] = 1.0;
      double l = d.uniform(0.2, 1.0);
      double m = d.uniform(0.5, 2.0);
      double c[3], mo[6];
      rod(m, l, 0.05 * l, c, mo);  // along −z
      if (a == 2) {                // rotate the rod to −x: swap the x and z roles
        c[0] = c[2];
        c[2] = 0.0;
        double jx = mo[0];
        mo[0] = mo[2];
        mo[2] = jx;
      }
      B.joint(GPB_JOINT_REVOLUTE, k, IDQ, prev, ax, m, c, mo);
      prev[0] = a == 2 ? -l : 0.0;
      prev[1] = 0.0;
      prev[2] = a == 2 ? 0.0 : -l;
    }
    for (int k = 0; k < n; ++k) {
      double q = d.uniform(-PI, PI);
      double v = d.normal(1.0);
      B.qv(q, v);
    }
  } else if (config == 2) {  // free-floating cube
    double s = d.uniform(0.2, 1.0);
    double m = 1000.0 * s * s * s;
    double mom = m * s * s / 6.0;
    double mo[6] = {mom, mom, mom, 0, 0, 0};
    B.joint(GPB_JOINT_FLOATING, 0, IDQ, ZERO3, ZERO3, m, ZERO3, mo);
    double h = s / 2.0;
    const double k = 1e5, c = contact_model == GPB_LINEAR_SPRING_DAMPER ? 1e3 : 0.0;
    const double corners[8][3] = {{h, h, -h}, {h, -h, -h}, {-h, h, -h}, {-h, -h, -h},
                                  {h, h, h},  {h, -h, h},  {-h, h, h},  {-h, -h, h}};
    for (auto& cc : corners) B.contact(1, cc[0], cc[1], cc[2], k, 0.0, c);
    double mu = d.uniform(0.3, 1.0);
    B.ground(0.9, mu);
    double z0 = d.uniform(0.5, 2.0);
    double qq[4];
    double nn = 0.0;
    for (int e = 0; e < 4; ++e) {
      qq[e] = d.normal(1.0);
      nn += qq[e] * qq[e];
    }
    nn = std::sqrt(nn);
    double vel[6];
    for (int e = 0; e < 3; ++e) vel[e] = d.normal(2.0);      // ω, body frame
    for (int e = 0; e < 3; ++e) vel[3 + e] = d.normal(1.0);  // v, body frame
    if (B.q0) {
      for (int e = 0; e < 4; ++e) B.q0[B.nq + e] = qq[e] / nn;
      B.q0[B.nq + 4] = 0.0;
      B.q0[B.nq + 5] = 0.0;
      B.q0[B.nq + 6] = z0;
      for (int e = 0; e < 6; ++e) {
        B.v0[B.nv + e] = vel[e];
        if (B.aux) B.aux[B.nv + e] = 0.0;
      }
    }
    B.nq += 7;
    B.nv += 6;
  } else {  // quadruped
    const double W = 0.6, D = 0.3, H = 0.15, MT = 10.0;
    double mt[6] = {MT * (D * D + H * H) / 12.0, MT * (W * W + H * H) / 12.0,
                    MT * (W * W + D * D) / 12.0, 0, 0, 0};
    B.joint(GPB_JOINT_FLOATING, 0, IDQ, ZERO3, ZERO3, MT, ZERO3, mt);
    const double L = 0.25, ML = 1.0, RF = 0.02;
    const double hips[4][2] = {{W / 2, D / 2}, {W / 2, -D / 2}, {-W / 2, D / 2}, {-W / 2, -D / 2}};
    const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0};
    const double kf = 2e4, cf = contact_model == GPB_LINEAR_SPRING_DAMPER ? 5e2 : 0.0;
    for (int g = 0; g < 4; ++g) {
      int base = 1 + 3 * g;
      double t0[3] = {hips[g][0], hips[g][1], 0.0};
      // hip-abduction body: 1 kg motor housing, sphere of radius 0.05 m
      double ms = 2.0 / 5.0 * ML * 0.05 * 0.05;
      double mh[6] = {ms, ms, ms, 0, 0, 0};
      B.joint(GPB_JOINT_REVOLUTE, 1, IDQ, t0, ex, ML, ZERO3, mh);
      double c[3], mo[6];
      rod(ML, L, 0.02, c, mo);
      B.joint(GPB_JOINT_REVOLUTE, base + 1, IDQ, ZERO3, ey, ML, c, mo);  // thigh (flexion)
      double tk[3] = {0, 0, -L};
      B.joint(GPB_JOINT_REVOLUTE, base + 2, IDQ, tk, ey, ML, c, mo);  // shank (knee)
      B.contact(base + 3, 0.0, 0.0, -L, kf, RF, cf);
    }
    B.ground(0.9, 0.8);
    // state: torso pose at z0 = 0.45 m, legs bent (flex 0.6, knee −1.2) so the feet
    // start just above the ground; PD targets U(−0.5, 0.5) rad on the 12 joints.
    if (B.q0) {
      double* q = B.q0 + B.nq;
      double* v = B.v0 + B.nv;
      for (int e = 0; e < 7; ++e) q[e] = 0.0;
      q[3] = 1.0;
      q[6] = 0.45;
      for (int e = 0; e < 6; ++e) v[e] = 0.0;
      for (int g = 0; g < 4; ++g) {
        q[7 + 3 * g] = 0.0;
        q[8 + 3 * g] = 0.6;
        q[9 + 3 * g] = -1.2;
        for (int e = 0; e < 3; ++e) v[6 + 3 * g + e] = 0.0;
      }
    }
    for (int e = 0; e < 18; ++e) {
      double target = e < 6 ? 0.0 : d.uniform(-0.5, 0.5);
      if (B.aux) B.aux[B.nv + e] = target;
    }
    B.nq += 19;
    B.nv += 18;
  }
}

}  // namespace

extern "C" int gpb_config_sizes(int config, int64_t n, uint32_t seed, int64_t* nj, int64_t* nc,
                                int64_t* nh, int64_t* nq, int64_t* nv) {
  if (config < 0 || config > 3 || n < 0) return GPB_E_INVAL;
  Builder B;
  std::memset(&B, 0, sizeof(B));
  for (int64_t i = 0; i < n; ++i) build_one(config, i, seed, GPB_LINEAR_SPRING_DAMPER, B);
  if (nj) *nj = B.nj;
  if (nc) *nc = B.nc;
  if (nh) *nh = B.nh;
  if (nq) *nq = B.nq;
  if (nv) *nv = B.nv;
  return GPB_OK;
}

extern "C" int gpb_config_build(int config, int64_t n, uint32_t seed, int contact_model,
                                int32_t* joint_offset, int32_t* joint_type, int32_t* joint_parent,
                                double* joint_iso, double* joint_axis, double* joint_spring,
                                double* body_inertia, int32_t* contact_offset, int32_t* contact_body,
                                double* contact_params, int32_t* halfspace_offset,
                                double* halfspace_params, int32_t* contact_model_out, double* q0,
                                double* v0, double* aux) {
  if (config < 0 || config > 3 || n < 0) return GPB_E_INVAL;
  if (!joint_offset || !joint_type || !joint_parent || !joint_iso || !joint_axis || !joint_spring ||
      !body_inertia || !contact_offset || !halfspace_offset || !contact_model_out || !q0 || !v0)
    return GPB_E_INVAL;
  Builder B;
  std::memset(&B, 0, sizeof(B));
  B.jt = joint_type;
  B.jp = joint_parent;
  B.iso = joint_iso;
  B.axis = joint_axis;
  B.spring = joint_spring;
  B.inertia = body_inertia;
  B.cb = contact_body;
  B.cp = contact_params;
  B.hp = halfspace_params;
  B.q0 = q0;
  B.v0 = v0;
  B.aux = aux;
  for (int64_t i = 0; i < n; ++i) {
    joint_offset[i] = (int32_t)B.nj;
    contact_offset[i] = (int32_t)B.nc;
    halfspace_offset[i] = (int32_t)B.nh;
    contact_model_out[i] = contact_model;
    build_one(config, i, seed, contact_model, B);
  }
  joint_offset[n] = (int32_t)B.nj;
  contact_offset[n] = (int32_t)B.nc;
  halfspace_offset[n] = (int32_t)B.nh;
  return GPB_OK;
}
