// Host-side internals shared by the batch API (gpb_host.cpp) and the serving
// engine (gpb_serve.cpp): error reporting, device buffers, the context and
// batch objects, instance validation, and the code that writes one instance
// into one lane of a pack.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gpb.h"
#include "gpb_internal.h"

namespace gpb {

// Default DOF threshold of the block-cooperative packs (gpb_batch_set_coop).
constexpr int kDefaultCoopMinDof = 0;

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const std::string& msg);

#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess)                                                                \
      return ::gpb::fail(GPB_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, count * sizeof(T));
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t upload(const std::vector<T>& h, cudaStream_t s) {
    if (h.empty()) return cudaSuccess;
    return cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

// Validated shape of one instance of a gpb_model.
struct InstInfo {
  int32_t j0, nb, nq, nv, c0, nc, h0, nh, model, nu;
  int32_t mvs;  // velocity stepping: potential contacts (points × half-spaces + cuboid pairs)
  bool chain;
  int32_t kind;  // 0 general, 1 planar chain, 2 floating tree (PackDesc::kind)
  uint64_t sig;  // topology class
};

inline int joint_nq(int t) { return t == GPB_JOINT_FLOATING ? 7 : (t == GPB_JOINT_FIXED ? 0 : 1); }
inline int joint_nv(int t) { return t == GPB_JOINT_FLOATING ? 6 : (t == GPB_JOINT_FIXED ? 0 : 1); }

// Checks instance i of m against the documented limits and fills I
// (GPB_OK, or the error code with gpb_last_error set).
int inspect_instance(const gpb_model* m, int64_t i, InstInfo* I);

// Quaternion (x,y,z,w) → row-major rotation matrix (same formula as
// UnitQuaternion::to_rotation_matrix).
inline void quat_to_rot(const double* q, double* m) {
  double x = q[0], y = q[1], z = q[2], w = q[3];
  double xx = x * x, yy = y * y, zz = z * z, ww = w * w;
  double xy = x * y * 2, xz = x * z * 2, yz = y * z * 2, wx = w * x * 2, wy = w * y * 2,
         wz = w * z * 2;
  m[0] = ww + xx - yy - zz;
  m[1] = xy - wz;
  m[2] = xz + wy;
  m[3] = xy + wz;
  m[4] = ww - xx + yy - zz;
  m[5] = yz - wx;
  m[6] = xz - wy;
  m[7] = yz + wx;
  m[8] = ww - xx - yy + zz;
}

// Writes instance `inst` of m (shape I) into lane l of pack P.  Every element
// goes through the sink with its absolute index in the lane-interleaved
// arrays, so the batch builder (host vectors) and the serving engine (a
// device scatter list) lay an instance out identically.  `key` is the lane's
// instance number (the counter key of the open-loop torque draw); q_user,
// v_user and c_user are the instance's offsets in the caller's flat q, v and
// contact arrays (for the gather/scatter maps).
template <typename Sink>
void fill_lane(const gpb_model* m, int64_t inst, const InstInfo& I, const PackDesc& P, int l,
               int32_t key, int64_t q_user, int64_t v_user, int64_t c_user, Sink& S) {
  const int64_t L = LANES;
  const int64_t li = P.lane * L + l;
  S.li(li, key);
  S.li(li + 1 * L, I.nb);
  S.li(li + 2 * L, I.nq);
  S.li(li + 3 * L, I.nv);
  S.li(li + 4 * L, I.nc);
  S.li(li + 5 * L, I.nh);
  S.li(li + 6 * L, I.model);
  S.li(li + 7 * L, I.nu);
  // contacts sorted by body (stable), remembering the user order
  std::vector<int> corder(I.nc);
  std::iota(corder.begin(), corder.end(), 0);
  std::stable_sort(corder.begin(), corder.end(), [&](int a, int b) {
    return m->contact_body[I.c0 + a] < m->contact_body[I.c0 + b];
  });
  std::vector<int> cfirst(I.nb, 0), ccount(I.nb, 0);
  for (int k = 0; k < I.nc; ++k) {
    const int src = corder[k];
    const int body = m->contact_body[I.c0 + src] - 1;
    if (ccount[body] == 0) cfirst[body] = k;
    ccount[body]++;
    S.ci((P.ctc + k) * L + l, body | (src << 8));
    const double* cp = m->contact_params + 6 * (size_t)(I.c0 + src);
    for (int e = 0; e < CTC_D; ++e) S.cd((P.ctc * CTC_D + CTC_D * k + e) * L + l, cp[e]);
  }
  // the kernel writes contact forces by the contact's user-order index
  for (int k = 0; k < I.nc; ++k)
    for (int e = 0; e < 3; ++e) S.cmap((P.ctc * 3 + 3 * k + e) * L + l, 3 * (c_user + k) + e);
  for (int h = 0; h < I.nh; ++h) {
    const double* hp = m->halfspace_params + 8 * (size_t)(I.h0 + h);
    const double nn = std::sqrt(hp[3] * hp[3] + hp[4] * hp[4] + hp[5] * hp[5]);
    const double vals[8] = {hp[0], hp[1], hp[2], hp[3] / nn, hp[4] / nn, hp[5] / nn, hp[6], hp[7]};
    for (int e = 0; e < HS_D; ++e) S.hd((P.hs * HS_D + HS_D * h + e) * L + l, vals[e]);
  }
  // bodies
  std::vector<bool> branch(I.nb, false);
  for (int b = 0; b < I.nb; ++b) {
    const int par = m->joint_parent[I.j0 + b];  // 1-based
    if (par >= 1 && par != b) branch[par - 1] = true;
  }
  int qo = 0, vo = 0, slot = 0;
  for (int b = 0; b < I.nb; ++b) {
    const int j = I.j0 + b;
    const double* cub = m->body_cuboid ? m->body_cuboid + 3 * (size_t)j : nullptr;
    const bool has_cub = cub && !(cub[0] == 0.0 && cub[1] == 0.0 && cub[2] == 0.0);
    const int t = m->joint_type[j], par = m->joint_parent[j];
    const double* iso = m->joint_iso + 7 * (size_t)j;
    const double* ax = m->joint_axis + 3 * (size_t)j;
    const double* in = m->body_inertia + 10 * (size_t)j;
    const double sk = m->joint_spring ? m->joint_spring[2 * (size_t)j] : 0.0;
    const double sl = m->joint_spring ? m->joint_spring[2 * (size_t)j + 1] : 0.0;
    uint32_t flags = 0;
    double R[9];
    quat_to_rot(iso, R);
    if (iso[0] == 0.0 && iso[1] == 0.0 && iso[2] == 0.0 && iso[3] == 1.0) flags |= BF_INIT_ROT_IDENTITY;
    int nz = 0, idx = 0;
    for (int e = 0; e < 3; ++e)
      if (ax[e] != 0.0) {
        nz++;
        idx = e;
      }
    if ((t == GPB_JOINT_REVOLUTE) && nz == 1 && std::fabs(ax[idx]) == 1.0) {
      flags |= BF_AXIS_PRINCIPAL | ((uint32_t)idx << 2);
      if (ax[idx] < 0) flags |= BF_AXIS_NEG;
    }
    if (branch[b]) flags |= BF_BRANCH;
    if (t == GPB_JOINT_PRISMATIC && sk != 0.0) flags |= BF_SPRING;
    if (in[7] == 0.0 && in[8] == 0.0 && in[9] == 0.0) flags |= BF_DIAG_INERTIA;
    S.w(((P.topo + b) * 2) * L + l, (uint32_t)t | ((uint32_t)par << 4) | ((uint32_t)qo << 12) | ((uint32_t)vo << 22));
    // cuboid slots in body order: the pairs are then visited in the reference's
    // order (src/contact.rs:191-197)
    const uint32_t uslot = has_cub ? (uint32_t)(++slot) : 0u;
    S.w(((P.topo + b) * 2 + 1) * L + l, flags | ((uint32_t)cfirst[b] << 8) | ((uint32_t)ccount[b] << 16) |
                                             (uslot << W1_CUBOID_SHIFT));
    double vals[TOPO_D];
    for (int e = 0; e < 9; ++e) vals[TD_RINIT + e] = R[e];
    for (int e = 0; e < 3; ++e) vals[TD_TINIT + e] = iso[4 + e];
    for (int e = 0; e < 3; ++e) vals[TD_AXIS + e] = ax[e];
    for (int e = 0; e < 10; ++e) vals[TD_INERTIA + e] = in[e];
    vals[TD_SPRING] = sk;
    vals[TD_SPRING + 1] = sl;
    vals[TD_ARMATURE] = m->joint_armature ? m->joint_armature[j] : 0.0;
    for (int e = 0; e < 3; ++e) vals[TD_CUBOID + e] = has_cub ? cub[e] : 0.0;
    for (int e = 0; e < TOPO_D; ++e) S.td((P.topo * TOPO_D + TOPO_D * b + e) * L + l, vals[e]);
    // state maps and the zero state (identity pose for floating joints)
    for (int e = 0; e < joint_nq(t); ++e) S.qmap((P.q + qo + e) * L + l, q_user + qo + e);
    if (t == GPB_JOINT_FLOATING) S.q0((P.q + qo + 3) * L + l, 1.0);
    for (int e = 0; e < joint_nv(t); ++e) S.vmap((P.v + vo + e) * L + l, v_user + vo + e);
    qo += joint_nq(t);
    vo += joint_nv(t);
  }
}

}  // namespace gpb

// The opaque objects of gpb.h.
struct gpb_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // bracket the last simulate kernel
  bool timed = false;
};

struct gpb_batch {
  gpb_ctx* ctx = nullptr;
  int64_t n = 0;
  int32_t npacks = 0;
  int warps_per_sm = 0;  // resident warps per SM of the step kernel (0 = occupancy limit)
  int coop_min_dof = -1; // block-cooperative packs: DOF threshold (-1 = default, 0 = off)
  int lanes = 1;         // lanes per instance of GPB_FP64 steps (1, or 2..32: body-parallel chains)
  bool group_ok = false; // every instance is a serial chain of 1-DOF or fixed joints without colliders
  int nb_max = 0, nv_max = 0;
  int algorithm = GPB_ALGO_CRBA;
  double gravity = 9.81;  // src/lib.rs:39
  std::vector<int64_t> q_off, v_off, c_off;  // user layout, [n+1]
  int64_t nq_total = 0, nv_total = 0, nc_total = 0;
  std::vector<gpb::PackDesc> packs_h;
  int64_t q_slots = 0, v_slots = 0, c_slots = 0;
  int64_t scratch_words = 0;  // 8-byte words of per-instance scratch, all packs
  int64_t vs_rows = 0;        // rows of velocity-stepping scratch, all packs (allocated on first use)
  std::vector<int32_t> status_slot;  // user instance -> status slot (pack*32+lane)
  gpb::DBuf<gpb::PackDesc> packs;
  gpb::DBuf<uint32_t> topoW;
  gpb::DBuf<double> topoD, ctcD, hsD, q, v, tau_in, scratch, stage_q, stage_v, stage_c, hist, vscratch;
  gpb::DBuf<float> topoF, ctcF, hsF;
  gpb::DBuf<int32_t> ctcI, laneI, status, queue;
  gpb::DBuf<int64_t> qmap, vmap, cmap, done;
  gpb::DeviceBatch dev() const {
    gpb::DeviceBatch b;
    std::memset(&b, 0, sizeof(b));
    b.npacks = npacks;
    b.packs = packs.p;
    b.topoW = topoW.p;
    b.topoD = topoD.p;
    b.topoF = topoF.p;
    b.ctcI = ctcI.p;
    b.ctcD = ctcD.p;
    b.ctcF = ctcF.p;
    b.hsD = hsD.p;
    b.hsF = hsF.p;
    b.laneI = laneI.p;
    b.status = status.p;
    b.done = done.p;
    b.q = q.p;
    b.v = v.p;
    b.tau_in = tau_in.p;
    b.scratch = scratch.p;
    b.qmap = qmap.p;
    b.vmap = vmap.p;
    b.cmap = cmap.p;
    b.nq_total = nq_total;
    b.nv_total = nv_total;
    b.nc_total = nc_total;
    b.queue = queue.p;
    b.algorithm = algorithm;
    b.gravity = gravity;
    b.vscratch = vscratch.p;
    return b;
  }
  void release() {
    packs.free();
    topoW.free();
    topoD.free();
    ctcD.free();
    hsD.free();
    q.free();
    v.free();
    tau_in.free();
    scratch.free();
    vscratch.free();
    stage_q.free();
    stage_v.free();
    stage_c.free();
    hist.free();
    topoF.free();
    ctcF.free();
    hsF.free();
    ctcI.free();
    laneI.free();
    status.free();
    queue.free();
    qmap.free();
    vmap.free();
    cmap.free();
    done.free();
  }
};
