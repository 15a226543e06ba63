// Serving engine of include/gpb.h (gpb_server_*): continuous batching of
// independent simulation requests over a pool of lane slots kept resident on
// one GPU.
//
// The reference has no serving layer; each request here is the reference's
// `simulate` (src/simulate.rs:87-112) of one mechanism over its own horizon.
// Design:
//   * The pool is an ordinary lane-interleaved batch whose packs have fixed
//     capacities (one slot class per capacity).  A request is written into one
//     free lane by the same fill_lane code the batch builder uses, delivered
//     as a list of (array, element, word) entries that one scatter kernel
//     applies, so admission costs one upload and one launch per tick.
//   * Every slot carries a LaneJob (steps left, its own step counter, dt,
//     integrator, control law).  A tick launches the persistent step kernel
//     over the packs that hold active slots (largest class first); each lane
//     runs min(chunk, steps_left) steps and appends its slot to a finished
//     list when its job ends or fails.
//   * Retirement gathers the final q, v, status and steps left of the
//     finished slots in one pass and frees them.
// A lane reads nothing of its neighbours, and every scratch word a step reads
// is written earlier in the same step, so a request's trajectory is the same
// whatever else shares the pool.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#include "gpb.h"
#include "gpb_host_impl.h"
#include "gpb_internal.h"

using namespace gpb;

namespace {

// Scatter targets of the pool (index into ScatterTable::t).
enum Target { T_W, T_TD, T_TF, T_CI, T_CD, T_CF, T_HD, T_HF, T_LI, T_Q, T_V, T_TAU, T_STATUS, T_JOBS, T_COUNT };

struct ClassInfo {
  gpb_slot_class caps;
  int32_t first_pack = 0, npacks = 0;
  int32_t high = 0;  // packs [first_pack, first_pack + high) have held a request
  int64_t pack_bytes = 0;
  std::vector<int32_t> free_slots;  // stack
};

// One instance's model tables, owned by a queued request (a gpb_model of one
// instance pointing into these vectors).
struct OwnedModel {
  std::vector<int32_t> joint_offset{0, 0}, joint_type, joint_parent, contact_offset{0, 0}, contact_body,
      halfspace_offset{0, 0}, contact_model;
  std::vector<double> joint_iso, joint_axis, joint_spring, body_inertia, contact_params, halfspace_params,
      joint_armature, body_cuboid;
  gpb_model view() const {
    gpb_model m;
    std::memset(&m, 0, sizeof(m));
    m.n_instances = 1;
    m.joint_offset = joint_offset.data();
    m.joint_type = joint_type.data();
    m.joint_parent = joint_parent.data();
    m.joint_iso = joint_iso.data();
    m.joint_axis = joint_axis.data();
    m.joint_spring = joint_spring.data();
    m.body_inertia = body_inertia.data();
    m.contact_offset = contact_offset.data();
    m.contact_body = contact_body.data();
    m.contact_params = contact_params.data();
    m.halfspace_offset = halfspace_offset.data();
    m.halfspace_params = halfspace_params.data();
    m.contact_model = contact_model.data();
    m.joint_armature = joint_armature.data();
    m.body_cuboid = body_cuboid.data();
    return m;
  }
};

struct Request {
  uint64_t id = 0;
  int cls = 0;
  InstInfo info{};
  OwnedModel model;
  std::vector<double> q, v, tau;
  gpb_request req{};
  std::chrono::steady_clock::time_point t_submit;
  int64_t left = 0;   // steps not yet launched (host count, for gpb_server_stats.steps)
  int64_t chunk = 0;  // steps per tick of its class
};

struct Result {
  std::vector<double> q, v;
  int32_t status = 0;
  int64_t steps_done = 0;
  double latency_s = 0.0;
};

// Device bytes of one pack with these capacities (every per-slot array of the pool).
int64_t pack_bytes(const gpb_slot_class& c) {
  const int64_t L = LANES;
  const int64_t nb = c.max_bodies, nq = c.max_q, nv = c.max_v, nc = c.max_contacts, nh = c.max_halfspaces,
                nu = c.max_cuboids;
  int64_t b = 0;
  b += nb * 2 * L * 4;                                     // topology words
  b += nb * TOPO_D * L * (8 + 4);                          // topology reals (double + float)
  b += nc * L * 4 + nc * CTC_D * L * (8 + 4);              // contacts
  b += nh * HS_D * L * (8 + 4);                            // half-spaces
  b += LANE_I * L * 4;                                     // lane ints
  b += (nq + 2 * nv) * L * 8;                              // q, v, tau_in
  b += (int64_t)scratch_layout((int)nb, (int)nq, (int)nv, (int)nc, (int)nu).total * L * 8;  // scratch
  b += L * (4 + 8 + 4 + (int64_t)sizeof(LaneJob));         // status, done, finished, job
  b += (int64_t)sizeof(PackDesc) + 4;                      // descriptor, active-list entry
  return b;
}

int check_class(const gpb_slot_class& c) {
  if (c.max_bodies < 1 || c.max_bodies > GPB_MAX_BODIES || c.max_q < 0 || c.max_q > 7 * GPB_MAX_BODIES ||
      c.max_v < 0 || c.max_v > GPB_MAX_DOF || c.max_contacts < 0 || c.max_contacts > GPB_MAX_CONTACTS ||
      c.max_halfspaces < 0 || c.max_halfspaces > GPB_MAX_HALFSPACES || c.weight < 0.0 || c.packs < 0 ||
      c.chunk_steps < 0 || c.max_cuboids < 0 || c.max_cuboids > GPB_MAX_CUBOIDS)
    return fail(GPB_E_RANGE, "gpb_server: slot class capacity outside the documented limits");
  return GPB_OK;
}

}  // namespace

struct gpb_server {
  gpb_ctx* ctx = nullptr;
  gpb_server_opts opts{};
  std::vector<ClassInfo> classes;
  std::vector<int> class_order;  // classes by pack cost, largest first (queue order)
  gpb_batch pool;                // the resident slots
  DBuf<LaneJob> jobs;
  DBuf<int32_t> active, finished, nfinished;
  DBuf<uint64_t> skey, sbits;    // scatter entries
  DBuf<int64_t> gidx;            // gather indices
  DBuf<uint64_t> gout;           // gathered words
  uint64_t* h_key = nullptr;     // pinned staging
  uint64_t* h_bits = nullptr;
  size_t h_cap = 0;
  std::vector<int32_t> pack_class, pack_active;
  std::vector<uint64_t> slot_req;  // 0 = free
  std::deque<Request> pending;
  std::unordered_map<uint64_t, Request> running;
  std::unordered_map<uint64_t, Result> results;
  std::vector<uint64_t> unread;
  uint64_t next_id = 1;
  int64_t ticks = 0, completed = 0, pool_bytes = 0, steps_run = 0;
  ScatterTable table{};
};

extern "C" int gpb_server_plan(const gpb_server_opts* o, int32_t* packs_per_class, int64_t* bytes_per_pack) {
  if (!o || !o->classes) return fail(GPB_E_INVAL, "gpb_server_plan: NULL argument");
  if (o->n_classes < 1 || o->n_classes > 16) return fail(GPB_E_RANGE, "gpb_server_plan: 1..16 slot classes");
  double wsum = 0.0;
  for (int k = 0; k < o->n_classes; ++k) {
    if (int r = check_class(o->classes[k])) return r;
    wsum += o->classes[k].weight;
  }
  if (wsum > 0.0 && o->hbm_budget_bytes <= 0)
    return fail(GPB_E_INVAL, "gpb_server_plan: weighted classes need a positive hbm_budget_bytes");
  // classes with a fixed pack count are served first; weighted classes share the rest
  int64_t fixed = 0;
  for (int k = 0; k < o->n_classes; ++k)
    if (!(o->classes[k].weight > 0.0)) fixed += (int64_t)o->classes[k].packs * pack_bytes(o->classes[k]);
  const int64_t rest = o->hbm_budget_bytes - fixed;
  if (wsum > 0.0 && rest <= 0)
    return fail(GPB_E_RANGE, "gpb_server_plan: no budget left for the weighted classes");
  int64_t total = 0;
  for (int k = 0; k < o->n_classes; ++k) {
    const gpb_slot_class& c = o->classes[k];
    const int64_t pb = pack_bytes(c);
    int64_t np = c.packs;
    if (c.weight > 0.0) np = (int64_t)((double)rest * (c.weight / wsum) / (double)pb);
    if (np > (1 << 24)) np = 1 << 24;
    if (packs_per_class) packs_per_class[k] = (int32_t)np;
    if (bytes_per_pack) bytes_per_pack[k] = pb;
    total += np * pb;
  }
  if (o->hbm_budget_bytes > 0 && total > o->hbm_budget_bytes)
    return fail(GPB_E_RANGE, "gpb_server_plan: the classes' packs exceed hbm_budget_bytes");
  return GPB_OK;
}

static void release(gpb_server* S) {
  S->pool.release();
  S->jobs.free();
  S->active.free();
  S->finished.free();
  S->nfinished.free();
  S->skey.free();
  S->sbits.free();
  S->gidx.free();
  S->gout.free();
  if (S->h_key) cudaFreeHost(S->h_key);
  if (S->h_bits) cudaFreeHost(S->h_bits);
  S->h_key = S->h_bits = nullptr;
}

extern "C" int gpb_server_create(gpb_ctx* ctx, const gpb_server_opts* o, gpb_server** out) {
  if (!ctx || !o || !out) return fail(GPB_E_INVAL, "gpb_server_create: NULL argument");
  if (o->precision != GPB_FP64 && o->precision != GPB_MIXED && o->precision != GPB_MIXED_REFINED)
    return fail(GPB_E_INVAL, "gpb_server_create: unknown precision");
  if (o->chunk_steps < 1) return fail(GPB_E_INVAL, "gpb_server_create: chunk_steps must be >= 1");
  if (o->algorithm != GPB_ALGO_CRBA && o->algorithm != GPB_ALGO_ABA)
    return fail(GPB_E_INVAL, "gpb_server_create: unknown algorithm");
  std::vector<int32_t> np(o->n_classes > 0 && o->n_classes <= 16 ? o->n_classes : 1);
  std::vector<int64_t> pb(np.size());
  if (int r = gpb_server_plan(o, np.data(), pb.data())) return r;
  gpb_server* S = new gpb_server();
  S->ctx = ctx;
  S->opts = *o;
  S->opts.classes = nullptr;
  S->classes.resize(o->n_classes);
  int32_t npacks = 0;
  for (int k = 0; k < o->n_classes; ++k) {
    ClassInfo& C = S->classes[k];
    C.caps = o->classes[k];
    C.first_pack = npacks;
    C.npacks = np[k];
    C.pack_bytes = pb[k];
    npacks += np[k];
    S->pool_bytes += (int64_t)np[k] * pb[k];
  }
  S->class_order.resize(o->n_classes);
  std::iota(S->class_order.begin(), S->class_order.end(), 0);
  std::stable_sort(S->class_order.begin(), S->class_order.end(), [&](int a, int b) {
    return S->classes[a].pack_bytes > S->classes[b].pack_bytes;
  });
  // pack descriptors: capacities of the class, rows laid out pack after pack
  gpb_batch& B = S->pool;
  B.ctx = ctx;
  B.algorithm = o->algorithm;
  B.npacks = npacks;
  B.packs_h.resize(npacks);
  S->pack_class.assign(npacks, 0);
  S->pack_active.assign(npacks, 0);
  int64_t rt = 0, rc = 0, rh = 0, rq = 0, rv = 0, rl = 0, rs = 0;
  for (int k = 0; k < o->n_classes; ++k) {
    const ClassInfo& C = S->classes[k];
    for (int32_t p = C.first_pack; p < C.first_pack + C.npacks; ++p) {
      PackDesc& P = B.packs_h[p];
      std::memset(&P, 0, sizeof(P));
      P.count = LANES;
      P.nb = C.caps.max_bodies;
      P.nq = C.caps.max_q;
      P.nv = C.caps.max_v;
      P.nc = C.caps.max_contacts;
      P.nh = C.caps.max_halfspaces;
      P.nu = C.caps.max_cuboids;
      P.chain = 0;
      P.kind = C.caps.planar_only ? 1 : 0;
      P.topo = rt;
      P.ctc = rc;
      P.hs = rh;
      P.q = rq;
      P.v = rv;
      P.lane = rl;
      P.scr = rs;
      rt += P.nb;
      rc += P.nc;
      rh += P.nh;
      rq += P.nq;
      rv += P.nv;
      rl += LANE_I;
      rs += scratch_layout(P.nb, P.nq, P.nv, P.nc, P.nu).total;
      S->pack_class[p] = k;
    }
  }
  // free slots: lane 0 of the first pack on top of each class stack
  for (int k = 0; k < o->n_classes; ++k) {
    ClassInfo& C = S->classes[k];
    for (int64_t s = (int64_t)(C.first_pack + C.npacks) * LANES - 1; s >= (int64_t)C.first_pack * LANES; --s)
      C.free_slots.push_back((int32_t)s);
  }
  S->slot_req.assign((size_t)npacks * LANES, 0);
  const size_t L = LANES;
  cudaError_t e = cudaSetDevice(ctx->device);
  auto chk = [&](cudaError_t x) {
    if (x != cudaSuccess && e == cudaSuccess) e = x;
  };
  chk(B.packs.alloc(npacks));
  chk(B.topoW.alloc(rt * 2 * L));
  chk(B.topoD.alloc(rt * TOPO_D * L));
  chk(B.topoF.alloc(rt * TOPO_D * L));
  chk(B.ctcI.alloc(rc * L));
  chk(B.ctcD.alloc(rc * CTC_D * L));
  chk(B.ctcF.alloc(rc * CTC_D * L));
  chk(B.hsD.alloc(rh * HS_D * L));
  chk(B.hsF.alloc(rh * HS_D * L));
  chk(B.laneI.alloc(rl * L));
  chk(B.status.alloc(npacks * L));
  chk(B.done.alloc(npacks * L));
  chk(B.q.alloc(rq * L));
  chk(B.v.alloc(rv * L));
  chk(B.tau_in.alloc(rv * L));
  chk(B.scratch.alloc(rs * L));
  chk(B.queue.alloc(2));
  chk(S->jobs.alloc(npacks * L));
  chk(S->active.alloc(std::max<int32_t>(npacks, 1)));
  chk(S->finished.alloc(std::max<size_t>(npacks * L, 1)));
  chk(S->nfinished.alloc(1));
  if (e != cudaSuccess) {
    release(S);
    delete S;
    return fail(e == cudaErrorMemoryAllocation ? GPB_E_NOMEM : GPB_E_CUDA,
                std::string("gpb_server_create: ") + cudaGetErrorString(e));
  }
  cudaStream_t s = ctx->stream;
  chk(B.packs.upload(B.packs_h, s));
  auto zero = [&](void* p, size_t bytes) {
    if (bytes) chk(cudaMemsetAsync(p, 0, bytes, s));
  };
  zero(B.topoW.p, B.topoW.n * 4);
  zero(B.topoD.p, B.topoD.n * 8);
  zero(B.topoF.p, B.topoF.n * 4);
  zero(B.ctcI.p, B.ctcI.n * 4);
  zero(B.ctcD.p, B.ctcD.n * 8);
  zero(B.ctcF.p, B.ctcF.n * 4);
  zero(B.hsD.p, B.hsD.n * 8);
  zero(B.hsF.p, B.hsF.n * 4);
  zero(B.laneI.p, B.laneI.n * 4);
  zero(B.status.p, B.status.n * 4);
  zero(B.done.p, B.done.n * 8);
  zero(B.q.p, B.q.n * 8);
  zero(B.v.p, B.v.n * 8);
  zero(B.tau_in.p, B.tau_in.n * 8);
  zero(S->jobs.p, S->jobs.n * sizeof(LaneJob));  // steps_left = 0: every slot idle
  chk(cudaStreamSynchronize(s));
  if (e != cudaSuccess) {
    release(S);
    delete S;
    return fail(GPB_E_CUDA, std::string("gpb_server_create: ") + cudaGetErrorString(e));
  }
  ScatterTable& T = S->table;
  auto tgt = [&](int id, void* base, size_t count, int bytes) {
    T.t[id].base = base;
    T.t[id].count = (int64_t)count;
    T.t[id].bytes = bytes;
    T.t[id].pad = 0;
  };
  tgt(T_W, B.topoW.p, B.topoW.n, 4);
  tgt(T_TD, B.topoD.p, B.topoD.n, 8);
  tgt(T_TF, B.topoF.p, B.topoF.n, 4);
  tgt(T_CI, B.ctcI.p, B.ctcI.n, 4);
  tgt(T_CD, B.ctcD.p, B.ctcD.n, 8);
  tgt(T_CF, B.ctcF.p, B.ctcF.n, 4);
  tgt(T_HD, B.hsD.p, B.hsD.n, 8);
  tgt(T_HF, B.hsF.p, B.hsF.n, 4);
  tgt(T_LI, B.laneI.p, B.laneI.n, 4);
  tgt(T_Q, B.q.p, B.q.n, 8);
  tgt(T_V, B.v.p, B.v.n, 8);
  tgt(T_TAU, B.tau_in.p, B.tau_in.n, 8);
  tgt(T_STATUS, B.status.p, B.status.n, 4);
  tgt(T_JOBS, S->jobs.p, S->jobs.n * LANE_JOB_WORDS, 8);
  T.n = T_COUNT;
  *out = S;
  return GPB_OK;
}

extern "C" int gpb_server_destroy(gpb_server* S) {
  if (!S) return GPB_OK;
  cudaSetDevice(S->ctx->device);
  cudaStreamSynchronize(S->ctx->stream);
  release(S);
  delete S;
  return GPB_OK;
}

extern "C" int gpb_server_submit(gpb_server* S, const gpb_model* m, int64_t first, int64_t count,
                                 const double* q, const double* v, const double* tau,
                                 const gpb_request* reqs, uint64_t* ids) {
  if (!S || !m || !reqs || (count > 0 && (!q || !v))) return fail(GPB_E_INVAL, "gpb_server_submit: NULL argument");
  if (first < 0 || count < 0 || first + count > m->n_instances)
    return fail(GPB_E_INVAL, "gpb_server_submit: instance range outside the model");
  std::vector<Request> batch;
  batch.reserve(count);
  int64_t qo = 0, vo = 0;
  for (int64_t k = 0; k < count; ++k) {
    const int64_t i = first + k;
    Request R;
    if (int r = inspect_instance(m, i, &R.info)) return r;
    const gpb_request& rq = reqs[k];
    if (!(rq.dt > 0.0) || !std::isfinite(rq.dt) || rq.steps < 1 || rq.integrator < 0 || rq.integrator > 2 ||
        rq.control < 0 || rq.control > 2)
      return fail(GPB_E_INVAL, "gpb_server_submit: request " + std::to_string(k) +
                                   ": dt > 0, steps >= 1 and a known integrator / control are required "
                                   "(velocity stepping is not served)");
    // smallest class that fits; a planar chain takes a planar-only class first.
    // The choice depends on the request alone, so its path (and its bits) do too.
    int best = -1;
    for (int pass = R.info.kind == 1 ? 0 : 1; pass < 2 && best < 0; ++pass) {
      for (int c = 0; c < (int)S->classes.size(); ++c) {
        const gpb_slot_class& cap = S->classes[c].caps;
        if ((cap.planar_only != 0) != (pass == 0)) continue;
        if (S->classes[c].npacks == 0 || R.info.nb > cap.max_bodies || R.info.nq > cap.max_q ||
            R.info.nv > cap.max_v || R.info.nc > cap.max_contacts || R.info.nh > cap.max_halfspaces ||
            R.info.nu > cap.max_cuboids)
          continue;
        if (best < 0 || S->classes[c].pack_bytes < S->classes[best].pack_bytes) best = c;
      }
    }
    if (best < 0)
      return fail(GPB_E_RANGE, "gpb_server_submit: instance " + std::to_string(i) + " fits no slot class");
    R.cls = best;
    R.req = rq;
    // private copy of the instance's tables
    const InstInfo& I = R.info;
    OwnedModel& O = R.model;
    O.joint_offset = {0, I.nb};
    O.joint_type.assign(m->joint_type + I.j0, m->joint_type + I.j0 + I.nb);
    O.joint_parent.assign(m->joint_parent + I.j0, m->joint_parent + I.j0 + I.nb);
    O.joint_iso.assign(m->joint_iso + 7 * (size_t)I.j0, m->joint_iso + 7 * (size_t)(I.j0 + I.nb));
    O.joint_axis.assign(m->joint_axis + 3 * (size_t)I.j0, m->joint_axis + 3 * (size_t)(I.j0 + I.nb));
    if (m->joint_spring)
      O.joint_spring.assign(m->joint_spring + 2 * (size_t)I.j0, m->joint_spring + 2 * (size_t)(I.j0 + I.nb));
    else
      O.joint_spring.assign(2 * (size_t)I.nb, 0.0);
    O.body_inertia.assign(m->body_inertia + 10 * (size_t)I.j0, m->body_inertia + 10 * (size_t)(I.j0 + I.nb));
    if (m->joint_armature)
      O.joint_armature.assign(m->joint_armature + I.j0, m->joint_armature + I.j0 + I.nb);
    else
      O.joint_armature.assign((size_t)I.nb, 0.0);
    if (m->body_cuboid)
      O.body_cuboid.assign(m->body_cuboid + 3 * (size_t)I.j0, m->body_cuboid + 3 * (size_t)(I.j0 + I.nb));
    else
      O.body_cuboid.assign(3 * (size_t)I.nb, 0.0);
    O.contact_offset = {0, I.nc};
    if (I.nc) {
      O.contact_body.assign(m->contact_body + I.c0, m->contact_body + I.c0 + I.nc);
      O.contact_params.assign(m->contact_params + 6 * (size_t)I.c0, m->contact_params + 6 * (size_t)(I.c0 + I.nc));
    }
    O.halfspace_offset = {0, I.nh};
    if (I.nh)
      O.halfspace_params.assign(m->halfspace_params + 8 * (size_t)I.h0,
                                m->halfspace_params + 8 * (size_t)(I.h0 + I.nh));
    O.contact_model = {I.model};
    R.info.j0 = R.info.c0 = R.info.h0 = 0;  // indices into the private copy
    R.q.assign(q + qo, q + qo + I.nq);
    R.v.assign(v + vo, v + vo + I.nv);
    if (tau) R.tau.assign(tau + vo, tau + vo + I.nv);
    qo += I.nq;
    vo += I.nv;
    batch.push_back(std::move(R));
  }
  const auto now = std::chrono::steady_clock::now();
  for (int64_t k = 0; k < count; ++k) {
    batch[k].id = S->next_id++;
    batch[k].t_submit = now;
    if (ids) ids[k] = batch[k].id;
    S->pending.push_back(std::move(batch[k]));
  }
  return GPB_OK;
}

namespace {

// fill_lane sink that emits scatter entries into the pool.
struct ScatterSink {
  std::vector<uint64_t>& key;
  std::vector<uint64_t>& bits;
  void put(int t, int64_t e, uint64_t b) {
    key.push_back(((uint64_t)t << 56) | (uint64_t)e);
    bits.push_back(b);
  }
  static uint64_t dbits(double x) {
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
  }
  static uint64_t fbits(double x) {
    const float f = (float)x;
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
  }
  void li(int64_t i, int32_t x) { put(T_LI, i, (uint32_t)x); }
  void ci(int64_t i, int32_t x) { put(T_CI, i, (uint32_t)x); }
  void cd(int64_t i, double x) {
    put(T_CD, i, dbits(x));
    put(T_CF, i, fbits(x));
  }
  void hd(int64_t i, double x) {
    put(T_HD, i, dbits(x));
    put(T_HF, i, fbits(x));
  }
  void w(int64_t i, uint32_t x) { put(T_W, i, x); }
  void td(int64_t i, double x) {
    put(T_TD, i, dbits(x));
    put(T_TF, i, fbits(x));
  }
  void q0(int64_t, double) {}  // the request's own q is written instead
  void qmap(int64_t, int64_t) {}
  void vmap(int64_t, int64_t) {}
  void cmap(int64_t, int64_t) {}
};

int grow_staging(gpb_server* S, size_t n) {
  if (n <= S->h_cap) return GPB_OK;
  size_t cap = std::max<size_t>(n, 2 * S->h_cap);
  if (S->h_key) cudaFreeHost(S->h_key);
  if (S->h_bits) cudaFreeHost(S->h_bits);
  S->h_key = S->h_bits = nullptr;
  S->h_cap = 0;
  CUDA_TRY(cudaMallocHost(&S->h_key, cap * 8));
  CUDA_TRY(cudaMallocHost(&S->h_bits, cap * 8));
  CUDA_TRY(S->skey.alloc(cap));
  CUDA_TRY(S->sbits.alloc(cap));
  S->h_cap = cap;
  return GPB_OK;
}

}  // namespace

extern "C" int gpb_server_tick(gpb_server* S, int32_t* completed_now) {
  if (!S) return fail(GPB_E_INVAL, "gpb_server_tick: server is NULL");
  if (completed_now) *completed_now = 0;
  CUDA_TRY(cudaSetDevice(S->ctx->device));
  cudaStream_t s = S->ctx->stream;
  const int64_t L = LANES;
  // ---- admission (FIFO within each class) --------------------------------
  std::vector<uint64_t> key, bits;
  ScatterSink sink{key, bits};
  int32_t admitted = 0;
  for (auto it = S->pending.begin(); it != S->pending.end();) {
    if (S->opts.max_admit_per_tick > 0 && admitted >= S->opts.max_admit_per_tick) break;
    ClassInfo& C = S->classes[it->cls];
    if (C.free_slots.empty()) {
      ++it;
      continue;
    }
    const int32_t slot = C.free_slots.back();
    C.free_slots.pop_back();
    const int32_t pk = slot / LANES, l = slot % LANES;
    const PackDesc& P = S->pool.packs_h[pk];
    Request& R = *it;
    const gpb_model mv = R.model.view();
    fill_lane(&mv, 0, R.info, P, l, R.req.key, 0, 0, 0, sink);
    for (int e = 0; e < R.info.nq; ++e) sink.put(T_Q, (P.q + e) * L + l, ScatterSink::dbits(R.q[e]));
    for (int e = 0; e < R.info.nv; ++e) sink.put(T_V, (P.v + e) * L + l, ScatterSink::dbits(R.v[e]));
    for (int e = 0; e < R.info.nv; ++e)
      sink.put(T_TAU, (P.v + e) * L + l, ScatterSink::dbits(R.tau.empty() ? 0.0 : R.tau[e]));
    sink.put(T_STATUS, slot, 0);
    LaneJob j;
    std::memset(&j, 0, sizeof(j));
    j.steps_left = R.req.steps;
    j.step_index = 0;
    j.dt = R.req.dt;
    j.sigma = R.req.sigma;
    j.kp = R.req.kp;
    j.kd = R.req.kd;
    j.seed = R.req.seed;
    j.control = R.req.control;
    j.resample = R.req.resample_every > 0 ? R.req.resample_every : 1;
    j.integrator = R.req.integrator;
    j.tau_mode = (R.req.control == GPB_CONTROL_HOST_TAU && !R.tau.empty()) ? 1 : 0;
    j.chunk = C.caps.chunk_steps;
    R.left = R.req.steps;
    R.chunk = C.caps.chunk_steps > 0 ? C.caps.chunk_steps : S->opts.chunk_steps;
    uint64_t words[LANE_JOB_WORDS];
    std::memcpy(words, &j, sizeof(j));
    for (int w = 0; w < LANE_JOB_WORDS; ++w) sink.put(T_JOBS, (int64_t)slot * LANE_JOB_WORDS + w, words[w]);
    S->slot_req[slot] = R.id;
    S->pack_active[pk]++;
    C.high = std::max(C.high, pk - C.first_pack + 1);
    S->running.emplace(R.id, std::move(R));
    it = S->pending.erase(it);
    ++admitted;
  }
  if (!key.empty()) {
    // the kernel skips out-of-range entries; check here so a bad entry is an error
    for (size_t k = 0; k < key.size(); ++k) {
      const int t = (int)(key[k] >> 56);
      const int64_t e = (int64_t)(key[k] & 0xffffffffffffull);
      if (t >= S->table.n || e >= S->table.t[t].count)
        return fail(GPB_E_CUDA, "gpb_server_tick: internal scatter index out of range");
    }
    if (int r = grow_staging(S, key.size())) return r;
    std::memcpy(S->h_key, key.data(), key.size() * 8);
    std::memcpy(S->h_bits, bits.data(), bits.size() * 8);
    CUDA_TRY(cudaMemcpyAsync(S->skey.p, S->h_key, key.size() * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(S->sbits.p, S->h_bits, bits.size() * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(launch_scatter_words(S->table, S->skey.p, S->sbits.p, (int64_t)key.size(), s));
    S->ctx->launches++;
  }
  // ---- one chunk over the packs holding active slots ------------------------
  std::vector<int32_t> act;
  for (int c : S->class_order) {
    const ClassInfo& C = S->classes[c];
    for (int32_t p = C.first_pack; p < C.first_pack + C.high; ++p)  // slots are taken lowest first
      if (S->pack_active[p] > 0) act.push_back(p);
  }
  S->ticks++;
  if (act.empty()) {
    CUDA_TRY(cudaStreamSynchronize(s));
    return GPB_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(S->active.p, act.data(), act.size() * 4, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemsetAsync(S->nfinished.p, 0, 4, s));
  DeviceBatch db = S->pool.dev();
  db.jobs = S->jobs.p;
  db.active = S->active.p;
  db.nactive = (int32_t)act.size();
  db.finished = S->finished.p;
  db.nfinished = S->nfinished.p;
  StepParams p;
  std::memset(&p, 0, sizeof(p));
  p.K = S->opts.chunk_steps;
  p.precision = S->opts.precision;
  p.dt = 1.0;  // per-slot values come from the jobs
  for (auto& kv : S->running) {  // every admitted request runs min(chunk, left) steps
    Request& R = kv.second;
    const int64_t k = std::min(R.chunk, R.left);
    R.left -= k;
    S->steps_run += k;
  }
  CUDA_TRY(cudaEventRecord(S->ctx->ev0, s));
  CUDA_TRY(launch_simulate(db, p, S->ctx->num_sms, 0, s));
  CUDA_TRY(cudaEventRecord(S->ctx->ev1, s));
  S->ctx->timed = true;
  S->ctx->launches++;
  int32_t nfin = 0;
  CUDA_TRY(cudaMemcpyAsync(&nfin, S->nfinished.p, 4, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (nfin <= 0) return GPB_OK;
  std::vector<int32_t> fin(nfin);
  CUDA_TRY(cudaMemcpyAsync(fin.data(), S->finished.p, (size_t)nfin * 4, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  // ---- retirement: gather q, v, steps left and status of the finished slots --
  std::vector<int64_t> qi, vi, ji, si;
  // a slot is listed once per job end: its job is then idle until a new admission
  std::vector<int32_t> keep;
  keep.reserve(fin.size());
  for (int32_t slot : fin)
    if (slot >= 0 && (size_t)slot < S->slot_req.size() && S->running.count(S->slot_req[slot])) keep.push_back(slot);
  if (keep.size() != fin.size()) return fail(GPB_E_CUDA, "gpb_server_tick: finished list names an idle slot");
  for (int32_t slot : fin) {
    const int32_t pk = slot / LANES, l = slot % LANES;
    const PackDesc& P = S->pool.packs_h[pk];
    const Request& R = S->running.at(S->slot_req[slot]);
    for (int e = 0; e < R.info.nq; ++e) qi.push_back((P.q + e) * L + l);
    for (int e = 0; e < R.info.nv; ++e) vi.push_back((P.v + e) * L + l);
    ji.push_back((int64_t)slot * LANE_JOB_WORDS + 1);  // step_index (steps run) is word 1 of LaneJob
    si.push_back(slot);
  }
  const size_t nidx = qi.size() + vi.size() + ji.size() + si.size();
  if (S->gidx.n < nidx) CUDA_TRY(S->gidx.alloc(std::max(nidx, 2 * S->gidx.n)));
  if (S->gout.n < nidx) CUDA_TRY(S->gout.alloc(std::max(nidx, 2 * S->gout.n)));
  std::vector<int64_t> all;
  all.reserve(nidx);
  all.insert(all.end(), qi.begin(), qi.end());
  all.insert(all.end(), vi.begin(), vi.end());
  all.insert(all.end(), ji.begin(), ji.end());
  all.insert(all.end(), si.begin(), si.end());
  CUDA_TRY(cudaMemcpyAsync(S->gidx.p, all.data(), nidx * 8, cudaMemcpyHostToDevice, s));
  size_t o = 0;
  CUDA_TRY(launch_gather_words(S->pool.q.p, 8, S->gidx.p + o, (int64_t)qi.size(), S->gout.p + o, s));
  o += qi.size();
  CUDA_TRY(launch_gather_words(S->pool.v.p, 8, S->gidx.p + o, (int64_t)vi.size(), S->gout.p + o, s));
  o += vi.size();
  CUDA_TRY(launch_gather_words(S->jobs.p, 8, S->gidx.p + o, (int64_t)ji.size(), S->gout.p + o, s));
  o += ji.size();
  // status words are 4 bytes: gathered into the low halves of the last region
  CUDA_TRY(launch_gather_words(S->pool.status.p, 4, S->gidx.p + o, (int64_t)si.size(),
                               reinterpret_cast<uint32_t*>(S->gout.p + o), s));
  S->ctx->launches += 4;
  std::vector<uint64_t> outw(nidx);
  CUDA_TRY(cudaMemcpyAsync(outw.data(), S->gout.p, nidx * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  const auto now = std::chrono::steady_clock::now();
  const uint32_t* st32 = reinterpret_cast<const uint32_t*>(outw.data() + qi.size() + vi.size() + ji.size());
  size_t oq = 0, ov = qi.size(), oj = qi.size() + vi.size();
  for (int32_t k = 0; k < nfin; ++k) {
    const int32_t slot = fin[k];
    const uint64_t id = S->slot_req[slot];
    auto it = S->running.find(id);
    Request& R = it->second;
    Result res;
    res.q.resize(R.info.nq);
    res.v.resize(R.info.nv);
    std::memcpy(res.q.data(), outw.data() + oq, R.info.nq * 8);
    std::memcpy(res.v.data(), outw.data() + ov, R.info.nv * 8);
    oq += R.info.nq;
    ov += R.info.nv;
    std::memcpy(&res.steps_done, outw.data() + oj + k, 8);
    S->steps_run += res.steps_done - (R.req.steps - R.left);  // exact once retired (a failed job stops early)
    res.status = (int32_t)st32[k];
    res.latency_s = std::chrono::duration<double>(now - R.t_submit).count();
    S->results.emplace(id, std::move(res));
    S->unread.push_back(id);
    S->running.erase(it);
    S->slot_req[slot] = 0;
    const int32_t pk = slot / LANES;
    S->pack_active[pk]--;
    S->classes[S->pack_class[pk]].free_slots.push_back(slot);
    S->completed++;
  }
  if (completed_now) *completed_now = nfin;
  return GPB_OK;
}

extern "C" int gpb_server_completed(gpb_server* S, uint64_t* ids, int32_t max, int32_t* count) {
  if (!S || !count || (max > 0 && !ids)) return fail(GPB_E_INVAL, "gpb_server_completed: NULL argument");
  const int32_t n = (int32_t)std::min<size_t>(S->unread.size(), (size_t)std::max(max, 0));
  for (int32_t k = 0; k < n; ++k) ids[k] = S->unread[k];
  S->unread.erase(S->unread.begin(), S->unread.begin() + n);
  *count = n;
  return GPB_OK;
}

extern "C" int gpb_server_result(gpb_server* S, uint64_t id, double* q, double* v, int32_t* status,
                                 int64_t* steps_done, double* latency_s) {
  if (!S) return fail(GPB_E_INVAL, "gpb_server_result: server is NULL");
  auto it = S->results.find(id);
  if (it == S->results.end())
    return fail(GPB_E_STATE, "gpb_server_result: request " + std::to_string(id) + " has not finished (or was read)");
  const Result& r = it->second;
  if (q) std::memcpy(q, r.q.data(), r.q.size() * 8);
  if (v) std::memcpy(v, r.v.data(), r.v.size() * 8);
  if (status) *status = r.status;
  if (steps_done) *steps_done = r.steps_done;
  if (latency_s) *latency_s = r.latency_s;
  S->results.erase(it);
  return GPB_OK;
}

extern "C" int gpb_server_forget(gpb_server* S, const uint64_t* ids, int64_t count) {
  if (!S || (count > 0 && !ids)) return fail(GPB_E_INVAL, "gpb_server_forget: NULL argument");
  for (int64_t k = 0; k < count; ++k) S->results.erase(ids[k]);
  return GPB_OK;
}

extern "C" int gpb_server_stats_get(const gpb_server* S, gpb_server_stats* st) {
  if (!S || !st) return fail(GPB_E_INVAL, "gpb_server_stats_get: NULL argument");
  st->pending = (int64_t)S->pending.size();
  st->active = (int64_t)S->running.size();
  st->completed = S->completed;
  st->slots = (int64_t)S->slot_req.size();
  st->ticks = S->ticks;
  st->pool_bytes = S->pool_bytes;
  st->steps = S->steps_run;
  return GPB_OK;
}
