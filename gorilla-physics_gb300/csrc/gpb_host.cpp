// Host side of the batched rigid-body step: the C ABI of include/gpb.h.
//
// The reference keeps one MechanismState per mechanism (src/mechanism.rs:41-58)
// and steps it with `step` / `simulate` (src/simulate.rs:20-112).  Here a batch
// owns the structure-of-arrays tables of many mechanisms on one GPU: instances
// are sorted by size and topology class, grouped into packs of 32 (one warp,
// one lane per instance), and every per-instance array is lane-interleaved so
// that a warp's 32 lanes read 32 consecutive words.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gpb.h"
#include "gpb_host_impl.h"
#include "gpb_internal.h"

using namespace gpb;

// ---------------------------------------------------------------------------
// errors

static thread_local std::string g_last_error;

int gpb::fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

extern "C" int gpb_abi_version(void) { return GPB_ABI_VERSION; }
extern "C" const char* gpb_last_error(void) { return g_last_error.c_str(); }

extern "C" int gpb_create(int device, gpb_ctx** out) {
  if (!out) return fail(GPB_E_INVAL, "gpb_create: out is NULL");
  int count = 0;
  CUDA_TRY(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(GPB_E_INVAL, "gpb_create: no such CUDA device");
  CUDA_TRY(cudaSetDevice(device));
  gpb_ctx* c = new gpb_ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e != cudaSuccess) {
    delete c;
    return fail(GPB_E_CUDA, std::string("gpb_create: ") + cudaGetErrorString(e));
  }
  *out = c;
  return GPB_OK;
}

extern "C" int gpb_destroy(gpb_ctx* ctx) {
  if (!ctx) return GPB_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GPB_OK;
}

extern "C" double gpb_last_launch_ms(gpb_ctx* ctx) {
  if (!ctx || !ctx->timed) return -1.0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return -1.0;
  if (cudaEventSynchronize(ctx->ev1) != cudaSuccess) return -1.0;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) return -1.0;
  return (double)ms;
}

extern "C" int gpb_synchronize(gpb_ctx* ctx) {
  if (!ctx) return fail(GPB_E_INVAL, "gpb_synchronize: ctx is NULL");
  CUDA_TRY(cudaSetDevice(ctx->device));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GPB_OK;
}

extern "C" int64_t gpb_launch_count(const gpb_ctx* ctx) { return ctx ? ctx->launches : -1; }

// ---------------------------------------------------------------------------
// model validation and packing


int gpb::inspect_instance(const gpb_model* m, int64_t i, InstInfo* out) {
  InstInfo& I = *out;
  I.j0 = m->joint_offset[i];
  I.nb = m->joint_offset[i + 1] - I.j0;
  if (I.nb < 0 || I.nb > GPB_MAX_BODIES)
    return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": body count outside [0, 64]");
  I.nq = I.nv = 0;
  I.chain = true;
  bool planar_chain = true, floating_tree = I.nb > 0;
  uint64_t sig = 1469598103934665603ull;
  for (int b = 0; b < I.nb; ++b) {
    int t = m->joint_type[I.j0 + b], p = m->joint_parent[I.j0 + b];
    if (t < 0 || t > 3) return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": bad joint type");
    if (m->joint_armature && m->joint_armature[I.j0 + b] != 0.0 && t != GPB_JOINT_REVOLUTE)
      return fail(GPB_E_INVAL, "instance " + std::to_string(i) +
                                   ": armature is only supported on revolute joints");  // src/joint/mod.rs:105-109
    if (p < 0 || p > b)
      return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": joint " + std::to_string(b + 1) +
                                   " has parent " + std::to_string(p) + " (must be < its own number)");
    if (p != b) I.chain = false;
    {  // the kinds with their own instantiation of the articulated-body passes
      const double* iso = m->joint_iso + 7 * (size_t)(I.j0 + b);
      const double* ax = m->joint_axis + 3 * (size_t)(I.j0 + b);
      const int nz = (ax[0] != 0.0) + (ax[1] != 0.0) + (ax[2] != 0.0);
      const double amax = std::max(std::fabs(ax[0]), std::max(std::fabs(ax[1]), std::fabs(ax[2])));
      const bool ident = iso[0] == 0.0 && iso[1] == 0.0 && iso[2] == 0.0 && iso[3] == 1.0;
      const bool principal_revolute = t == GPB_JOINT_REVOLUTE && nz == 1 && amax == 1.0 && ident;
      if (!principal_revolute || p != b) planar_chain = false;
      if (b == 0 ? !(t == GPB_JOINT_FLOATING && p == 0 && ident) : !principal_revolute) floating_tree = false;
    }
    I.nq += joint_nq(t);
    I.nv += joint_nv(t);
    sig = (sig ^ (uint64_t)(t * 131 + p)) * 1099511628211ull;
  }
  if (I.nv > GPB_MAX_DOF) return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": more than 64 DOF");
  I.c0 = m->contact_offset ? m->contact_offset[i] : 0;
  I.nc = m->contact_offset ? m->contact_offset[i + 1] - I.c0 : 0;
  if (I.nc < 0 || I.nc > GPB_MAX_CONTACTS)
    return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": contact count outside [0, 64]");
  for (int k = 0; k < I.nc; ++k) {
    int bb = m->contact_body[I.c0 + k];
    if (bb < 1 || bb > I.nb) return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": contact on a missing body");
  }
  I.h0 = m->halfspace_offset ? m->halfspace_offset[i] : 0;
  I.nh = m->halfspace_offset ? m->halfspace_offset[i + 1] - I.h0 : 0;
  if (I.nh < 0 || I.nh > GPB_MAX_HALFSPACES)
    return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": half-space count outside [0, 4]");
  I.model = m->contact_model ? m->contact_model[i] : GPB_HUNT_CROSSLEY;
  if (I.model != GPB_HUNT_CROSSLEY && I.model != GPB_LINEAR_SPRING_DAMPER)
    return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": bad contact model");
  // cuboid colliders (src/rigid_body.rs:197-199): sizes all zero = none
  I.nu = 0;
  for (int b = 0; b < I.nb && m->body_cuboid; ++b) {
    const double* d = m->body_cuboid + 3 * (size_t)(I.j0 + b);
    if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) continue;
    if (!(d[0] > 0.0 && d[1] > 0.0 && d[2] > 0.0 && std::isfinite(d[0] + d[1] + d[2])))
      return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": cuboid sizes must be positive");
    if (++I.nu > GPB_MAX_CUBOIDS)
      return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": more than " +
                                   std::to_string(GPB_MAX_CUBOIDS) + " cuboid colliders");
  }
  I.mvs = I.nc * I.nh + I.nu * (I.nu - 1) / 2;
  bool springs = false;
  for (int b = 0; b < I.nb && m->joint_spring; ++b) springs = springs || m->joint_spring[2 * (size_t)(I.j0 + b)] != 0.0;
  if (I.nc > 0 || I.nu > 0 || springs) planar_chain = false;
  if (I.nu > 0 || springs) floating_tree = false;
  I.kind = planar_chain ? 1 : (floating_tree ? 2 : 0);
  sig = (sig ^ (uint64_t)(I.nc * 7 + I.nh + 1000 * I.nu)) * 1099511628211ull;
  I.sig = sig;
  return GPB_OK;
}

extern "C" int gpb_batch_create(gpb_ctx* ctx, const gpb_model* m, gpb_batch** out) {
  if (!ctx || !m || !out) return fail(GPB_E_INVAL, "gpb_batch_create: NULL argument");
  if (m->n_instances < 0) return fail(GPB_E_INVAL, "gpb_batch_create: negative instance count");
  if (!m->joint_offset || !m->joint_type || !m->joint_parent || !m->joint_iso || !m->joint_axis ||
      !m->body_inertia)
    return fail(GPB_E_INVAL, "gpb_batch_create: joint/body tables missing");
  const int64_t n = m->n_instances;
  std::vector<InstInfo> info(n);
  for (int64_t i = 0; i < n; ++i)
    if (int r = inspect_instance(m, i, &info[i])) return r;

  gpb_batch* B = new gpb_batch();
  B->ctx = ctx;
  B->n = n;
  B->q_off.assign(n + 1, 0);
  B->v_off.assign(n + 1, 0);
  B->c_off.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) {
    B->q_off[i + 1] = B->q_off[i] + info[i].nq;
    B->v_off[i + 1] = B->v_off[i] + info[i].nv;
    B->c_off[i + 1] = B->c_off[i] + info[i].nc;
  }
  B->nq_total = B->q_off[n];
  B->nv_total = B->v_off[n];
  B->nc_total = B->c_off[n];

  // the body-parallel mapping (serial chains of revolute, prismatic and fixed
  // joints, no cuboid colliders)
  B->group_ok = n > 0;
  for (int64_t i = 0; i < n; ++i) {
    const InstInfo& I = info[i];
    B->nb_max = std::max(B->nb_max, (int)I.nb);
    B->nv_max = std::max(B->nv_max, (int)I.nv);
    bool ok = I.chain && I.nu == 0;
    for (int b = 0; b < I.nb && ok; ++b) ok = m->joint_type[I.j0 + b] != GPB_JOINT_FLOATING;
    B->group_ok = B->group_ok && ok;
  }

  // sort: largest work first (the persistent queue then balances), same topology together
  std::vector<int64_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    const InstInfo &A = info[a], &Bq = info[b];
    if (A.nv != Bq.nv) return A.nv > Bq.nv;
    if (A.nb != Bq.nb) return A.nb > Bq.nb;
    if (A.nc != Bq.nc) return A.nc > Bq.nc;
    return A.sig < Bq.sig;
  });
  const int64_t npacks = (n + LANES - 1) / LANES;
  B->npacks = (int32_t)npacks;
  B->packs_h.resize(npacks);
  int64_t rt = 0, rc = 0, rh = 0, rq = 0, rv = 0, rl = 0, rs = 0, rvs = 0;
  for (int64_t p = 0; p < npacks; ++p) {
    PackDesc& P = B->packs_h[p];
    std::memset(&P, 0, sizeof(P));
    P.count = (int32_t)std::min<int64_t>(LANES, n - p * LANES);
    P.chain = 1;
    P.kind = -1;
    P.minnv = GPB_MAX_DOF;
    for (int l = 0; l < P.count; ++l) {
      const InstInfo& I = info[order[p * LANES + l]];
      P.nb = std::max(P.nb, I.nb);
      P.nq = std::max(P.nq, I.nq);
      P.nv = std::max(P.nv, I.nv);
      P.nc = std::max(P.nc, I.nc);
      P.nh = std::max(P.nh, I.nh);
      P.nu = std::max(P.nu, I.nu);
      P.mvs = std::max(P.mvs, I.mvs);
      P.minnv = std::min(P.minnv, I.nv);
      if (!I.chain) P.chain = 0;
      P.kind = (P.kind < 0 || P.kind == I.kind) ? I.kind : 0;
    }
    P.topo = rt;
    P.ctc = rc;
    P.hs = rh;
    P.q = rq;
    P.v = rv;
    P.lane = rl;
    P.scr = rs;
    P.vs = rvs;
    if (P.mvs <= GPB_MAX_VS_CONTACTS) rvs += vs_layout(P.nv, P.mvs).total;
    rt += P.nb;
    rc += P.nc;
    rh += P.nh;
    rq += P.nq;
    rv += P.nv;
    rl += LANE_I;
    rs += scratch_layout(P.nb, P.nq, P.nv, P.nc, P.nu).total;
  }
  // A special kind only for a batch of that kind alone: when its packs run
  // beside packs of other kinds, the instantiations share each SM's instruction
  // cache and the batch runs slower than with the general one (16,384
  // quadrupeds + 16,384 chains, mixed: 40.8 against 47.4 M instance-steps/s on
  // GB300 with the chains' packs specialised).
  int kind = npacks > 0 ? std::max(B->packs_h[0].kind, 0) : 0;
  for (const PackDesc& P : B->packs_h)
    if (P.kind != kind) kind = 0;
  for (PackDesc& P : B->packs_h) P.kind = kind;
  const size_t L = LANES;
  std::vector<uint32_t> W(rt * 2 * L, 0);
  std::vector<double> TD(rt * TOPO_D * L, 0.0), CD(rc * CTC_D * L, 0.0), HD(rh * HS_D * L, 0.0);
  std::vector<int32_t> CI(rc * L, 0), LI(rl * L, 0);
  std::vector<int64_t> qmap(rq * L, -1), vmap(rv * L, -1), cmap(rc * 3 * L, -1);
  std::vector<double> q0(rq * L, 0.0);
  B->status_slot.assign(n, 0);
  struct VectorSink {  // fill_lane into the host tables below
    std::vector<uint32_t>* W_;
    std::vector<double>*TD_, *CD_, *HD_, *Q0_;
    std::vector<int32_t>*CI_, *LI_;
    std::vector<int64_t>*QM_, *VM_, *CM_;
    void li(int64_t i, int32_t x) { (*LI_)[i] = x; }
    void ci(int64_t i, int32_t x) { (*CI_)[i] = x; }
    void cd(int64_t i, double x) { (*CD_)[i] = x; }
    void hd(int64_t i, double x) { (*HD_)[i] = x; }
    void w(int64_t i, uint32_t x) { (*W_)[i] = x; }
    void td(int64_t i, double x) { (*TD_)[i] = x; }
    void q0(int64_t i, double x) { (*Q0_)[i] = x; }
    void qmap(int64_t i, int64_t x) { (*QM_)[i] = x; }
    void vmap(int64_t i, int64_t x) { (*VM_)[i] = x; }
    void cmap(int64_t i, int64_t x) { (*CM_)[i] = x; }
  } sink{&W, &TD, &CD, &HD, &q0, &CI, &LI, &qmap, &vmap, &cmap};

  for (int64_t p = 0; p < npacks; ++p) {
    const PackDesc& P = B->packs_h[p];
    for (int l = 0; l < LANES; ++l) {
      int64_t li = P.lane * L + l;
      if (l >= P.count) {
        LI[li] = -1;
        continue;
      }
      const int64_t inst = order[p * LANES + l];
      B->status_slot[inst] = (int32_t)(p * LANES + l);
      fill_lane(m, inst, info[inst], P, l, (int32_t)inst, B->q_off[inst], B->v_off[inst], B->c_off[inst], sink);
    }
  }
  std::vector<float> TF(TD.begin(), TD.end()), CF(CD.begin(), CD.end()), HF(HD.begin(), HD.end());

  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSetDevice(ctx->device);
  auto chk = [&](cudaError_t x) {
    if (x != cudaSuccess && e == cudaSuccess) e = x;
  };
  B->scratch_words = rs * L;
  B->vs_rows = rvs;
  B->q_slots = rq * L;
  B->v_slots = rv * L;
  B->c_slots = rc * 3 * L;
  chk(B->packs.alloc(npacks));
  chk(B->topoW.alloc(W.size()));
  chk(B->topoD.alloc(TD.size()));
  chk(B->topoF.alloc(TF.size()));
  chk(B->ctcI.alloc(CI.size()));
  chk(B->ctcD.alloc(CD.size()));
  chk(B->ctcF.alloc(CF.size()));
  chk(B->hsD.alloc(HD.size()));
  chk(B->hsF.alloc(HF.size()));
  chk(B->laneI.alloc(LI.size()));
  chk(B->status.alloc(npacks * L));
  chk(B->done.alloc(npacks * L));
  chk(B->q.alloc(rq * L));
  chk(B->v.alloc(rv * L));
  chk(B->tau_in.alloc(rv * L));
  chk(B->scratch.alloc(rs * L));
  chk(B->qmap.alloc(qmap.size()));
  chk(B->vmap.alloc(vmap.size()));
  chk(B->cmap.alloc(cmap.size()));
  chk(B->stage_q.alloc(std::max<int64_t>(B->nq_total, 1)));
  chk(B->stage_v.alloc(std::max<int64_t>(B->nv_total, 1)));
  chk(B->stage_c.alloc(std::max<int64_t>(3 * B->nc_total, 1)));
  chk(B->queue.alloc(2));
  if (e != cudaSuccess) {
    B->release();
    delete B;
    return fail(e == cudaErrorMemoryAllocation ? GPB_E_NOMEM : GPB_E_CUDA,
                std::string("gpb_batch_create: ") + cudaGetErrorString(e));
  }
  chk(B->packs.upload(B->packs_h, s));
  chk(B->topoW.upload(W, s));
  chk(B->topoD.upload(TD, s));
  chk(B->topoF.upload(TF, s));
  chk(B->ctcI.upload(CI, s));
  chk(B->ctcD.upload(CD, s));
  chk(B->ctcF.upload(CF, s));
  chk(B->hsD.upload(HD, s));
  chk(B->hsF.upload(HF, s));
  chk(B->laneI.upload(LI, s));
  chk(B->qmap.upload(qmap, s));
  chk(B->vmap.upload(vmap, s));
  chk(B->cmap.upload(cmap, s));
  chk(B->q.upload(q0, s));
  if (B->v.n) chk(cudaMemsetAsync(B->v.p, 0, B->v.n * sizeof(double), s));
  if (B->tau_in.n) chk(cudaMemsetAsync(B->tau_in.p, 0, B->tau_in.n * sizeof(double), s));
  if (B->status.n) chk(cudaMemsetAsync(B->status.p, 0, B->status.n * sizeof(int32_t), s));
  if (B->done.n) chk(cudaMemsetAsync(B->done.p, 0, B->done.n * sizeof(int64_t), s));
  chk(cudaStreamSynchronize(s));  // host vectors go out of scope
  if (e != cudaSuccess) {
    B->release();
    delete B;
    return fail(GPB_E_CUDA, std::string("gpb_batch_create upload: ") + cudaGetErrorString(e));
  }
  *out = B;
  return GPB_OK;
}

extern "C" int gpb_batch_destroy(gpb_batch* b) {
  if (!b) return GPB_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  b->release();
  delete b;
  return GPB_OK;
}

extern "C" int gpb_batch_layout(const gpb_batch* b, int64_t* q_offset, int64_t* v_offset,
                                int64_t* nq_total, int64_t* nv_total) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_layout: batch is NULL");
  if (q_offset) std::memcpy(q_offset, b->q_off.data(), sizeof(int64_t) * (b->n + 1));
  if (v_offset) std::memcpy(v_offset, b->v_off.data(), sizeof(int64_t) * (b->n + 1));
  if (nq_total) *nq_total = b->nq_total;
  if (nv_total) *nv_total = b->nv_total;
  return GPB_OK;
}

extern "C" int gpb_batch_set_algorithm(gpb_batch* b, int algorithm) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_algorithm: batch is NULL");
  if (algorithm != GPB_ALGO_CRBA && algorithm != GPB_ALGO_ABA)
    return fail(GPB_E_INVAL, "gpb_batch_set_algorithm: GPB_ALGO_CRBA or GPB_ALGO_ABA");
  b->algorithm = algorithm;
  return GPB_OK;
}

extern "C" int gpb_batch_set_gravity(gpb_batch* b, double g) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_gravity: batch is NULL");
  if (!std::isfinite(g)) return fail(GPB_E_INVAL, "gpb_batch_set_gravity: g must be finite");
  b->gravity = g;
  return GPB_OK;
}

extern "C" int gpb_batch_set_coop(gpb_batch* b, int min_dof) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_coop: batch is NULL");
  if (min_dof < -1 || min_dof > GPB_MAX_DOF)
    return fail(GPB_E_INVAL, "gpb_batch_set_coop: min_dof must be -1 (default), 0 (off) or 1..64");
  b->coop_min_dof = min_dof;
  return GPB_OK;
}

// Packs at the front of the queue whose every instance has at least the
// block-cooperative threshold of DOF (packs are sorted by DOF, largest first).
static int32_t coop_packs(const gpb_batch* b, int precision) {
  if (precision == GPB_MIXED_REFINED || b->algorithm != GPB_ALGO_CRBA) return 0;
  int thr = b->coop_min_dof < 0 ? kDefaultCoopMinDof : b->coop_min_dof;
  if (thr <= 0) return 0;
  if (precision == GPB_MIXED) thr = std::max(thr, 13);  // the FP64-factor form of GPB_MIXED
  int32_t n = 0;
  while (n < b->npacks && b->packs_h[n].minnv >= thr) ++n;
  return n;
}

// Bodies per lane of the body-parallel mapping with `lanes` lanes per
// instance, 0 if the batch cannot run it that way.
static int group_bodies_per_lane(const gpb_batch* b, int lanes) {
  if (!b->group_ok) return 0;
  if (lanes == 4 * LANES) return 1;  // a 4-warp block per instance: one body per thread
  if (lanes < 2 || lanes > LANES || (lanes & (lanes - 1))) return 0;
  const int s = (b->nb_max + lanes - 1) / lanes;
  return s <= 1 ? 1 : (s == 2 ? 2 : 0);
}

extern "C" int gpb_batch_set_mapping(gpb_batch* b, int lanes_per_instance) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_mapping: batch is NULL");
  if (lanes_per_instance != 1 && !group_bodies_per_lane(b, lanes_per_instance)) {
    if (!b->group_ok)
      return fail(GPB_E_INVAL, "gpb_batch_set_mapping: several lanes per instance need a batch of serial chains "
                               "of revolute, prismatic and fixed joints without cuboid colliders");
    return fail(GPB_E_INVAL, "gpb_batch_set_mapping: lanes_per_instance must be 1, a power of two in [2, 32] "
                             "with at most two bodies per lane (this batch has chains of " +
                                 std::to_string(b->nb_max) + " bodies), or 128 (a 4-warp block per instance)");
  }
  b->lanes = lanes_per_instance;
  return GPB_OK;
}

extern "C" int gpb_batch_set_launch(gpb_batch* b, int warps_per_sm) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_launch: batch is NULL");
  if (warps_per_sm < 0 || warps_per_sm > 64 || warps_per_sm % 4 != 0)
    return fail(GPB_E_INVAL, "gpb_batch_set_launch: warps_per_sm must be 0 or a multiple of 4 up to 64");
  b->warps_per_sm = warps_per_sm;
  return GPB_OK;
}

static int upload_user(gpb_batch* b, const double* src, int64_t count, DBuf<double>& stage,
                       const DBuf<int64_t>& map, int64_t slots, DBuf<double>& dst) {
  cudaStream_t s = b->ctx->stream;
  if (count > 0) {
    CUDA_TRY(cudaMemcpyAsync(stage.p, src, count * sizeof(double), cudaMemcpyHostToDevice, s));
    CUDA_TRY(launch_scatter(map.p, slots, stage.p, dst.p, s));
    b->ctx->launches++;
  }
  return GPB_OK;
}

extern "C" int gpb_set_state(gpb_batch* b, const double* q, const double* v) {
  if (!b) return fail(GPB_E_INVAL, "gpb_set_state: batch is NULL");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  if (q) {
    int r = upload_user(b, q, b->nq_total, b->stage_q, b->qmap, b->q_slots, b->q);
    if (r) return r;
  }
  if (v) {
    int r = upload_user(b, v, b->nv_total, b->stage_v, b->vmap, b->v_slots, b->v);
    if (r) return r;
  }
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return GPB_OK;
}

extern "C" int gpb_get_state(gpb_batch* b, double* q, double* v) {
  if (!b) return fail(GPB_E_INVAL, "gpb_get_state: batch is NULL");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  if (q && b->nq_total) {
    CUDA_TRY(launch_gather(b->qmap.p, b->q_slots, b->q.p, b->stage_q.p, s));
    b->ctx->launches++;
    CUDA_TRY(cudaMemcpyAsync(q, b->stage_q.p, b->nq_total * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (v && b->nv_total) {
    CUDA_TRY(launch_gather(b->vmap.p, b->v_slots, b->v.p, b->stage_v.p, s));
    b->ctx->launches++;
    CUDA_TRY(cudaMemcpyAsync(v, b->stage_v.p, b->nv_total * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  return GPB_OK;
}

static int check_enums(int integrator, int precision) {
  if (integrator < 0 || integrator > 3) return fail(GPB_E_INVAL, "unknown integrator");
  if (precision != GPB_FP64 && precision != GPB_MIXED && precision != GPB_MIXED_REFINED)
    return fail(GPB_E_INVAL, "unknown precision");
  return GPB_OK;
}

extern "C" int gpb_dynamics(gpb_batch* b, const double* tau, int precision, double* qdd,
                            double* contact_force) {
  if (!b || !qdd) return fail(GPB_E_INVAL, "gpb_dynamics: NULL argument");
  if (int r = check_enums(0, precision)) return r;
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  StepParams p;
  std::memset(&p, 0, sizeof(p));
  p.precision = precision;
  p.tau_mode = tau ? 1 : 0;
  if (tau) {
    int r = upload_user(b, tau, b->nv_total, b->stage_v, b->vmap, b->v_slots, b->tau_in);
    if (r) return r;
  }
  p.qdd_out = b->stage_v.p;
  p.cforce_out = contact_force ? b->stage_c.p : nullptr;
  CUDA_TRY(launch_dynamics(b->dev(), p, s));
  b->ctx->launches++;
  if (b->nv_total)
    CUDA_TRY(cudaMemcpyAsync(qdd, b->stage_v.p, b->nv_total * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (contact_force && b->nc_total)
    CUDA_TRY(cudaMemcpyAsync(contact_force, b->stage_c.p, 3 * b->nc_total * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return GPB_OK;
}

extern "C" int gpb_free_velocity(gpb_batch* b, double dt, const double* tau, int precision, double* v_free) {
  if (!b || !v_free) return fail(GPB_E_INVAL, "gpb_free_velocity: NULL argument");
  if (int r = check_enums(0, precision)) return r;
  if (!std::isfinite(dt)) return fail(GPB_E_INVAL, "gpb_free_velocity: dt must be finite");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  StepParams p;
  std::memset(&p, 0, sizeof(p));
  p.precision = precision;
  p.tau_mode = tau ? 1 : 0;
  p.free_velocity = 1;
  p.vfree_dt = dt;
  if (tau) {
    int r = upload_user(b, tau, b->nv_total, b->stage_v, b->vmap, b->v_slots, b->tau_in);
    if (r) return r;
  }
  p.qdd_out = b->stage_v.p;
  DeviceBatch db = b->dev();
  db.plain = 1;
  CUDA_TRY(launch_dynamics(db, p, s));
  b->ctx->launches++;
  if (b->nv_total)
    CUDA_TRY(cudaMemcpyAsync(v_free, b->stage_v.p, b->nv_total * sizeof(double), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return GPB_OK;
}

static int run_simulate(gpb_batch* b, double dt, int64_t K, int64_t step0, int integrator,
                        int precision, const gpb_control_params* ctl, int64_t record_every,
                        double* history) {
  if (int r = check_enums(integrator, precision)) return r;
  if (K < 0) return fail(GPB_E_INVAL, "negative step count");
  if (integrator == GPB_VELOCITY_STEPPING) {  // FP64 only; its scratch on first use
    if (precision != GPB_FP64) return fail(GPB_E_INVAL, "velocity stepping runs in GPB_FP64 only");
    for (const PackDesc& P : b->packs_h)
      if (P.mvs > GPB_MAX_VS_CONTACTS)
        return fail(GPB_E_RANGE, "velocity stepping: an instance has more than " +
                                     std::to_string(GPB_MAX_VS_CONTACTS) +
                                     " potential contacts (contact points x half-spaces + cuboid pairs)");
    if (b->vs_rows > 0 && !b->vscratch.p) {
      CUDA_TRY(cudaSetDevice(b->ctx->device));
      if (b->vscratch.alloc((size_t)b->vs_rows * LANES) != cudaSuccess)
        return fail(GPB_E_NOMEM, "velocity stepping: scratch allocation failed");
    }
  }
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(GPB_E_INVAL, "dt must be positive and finite");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  StepParams p;
  std::memset(&p, 0, sizeof(p));
  p.dt = dt;
  p.K = K;
  p.step0 = step0;
  p.integrator = integrator;
  p.precision = precision;
  p.control = ctl ? ctl->mode : GPB_CONTROL_HOST_TAU;
  if (p.control < 0 || p.control > 2) return fail(GPB_E_INVAL, "unknown control mode");
  if (ctl) {
    p.seed = ctl->seed;
    p.resample = ctl->resample_every > 0 ? ctl->resample_every : 1;
    p.sigma = ctl->sigma;
    p.kp = ctl->kp;
    p.kd = ctl->kd;
  }
  const double* tau = ctl ? ctl->tau : nullptr;
  p.tau_mode = tau ? 1 : 0;
  if (tau) {
    int r = upload_user(b, tau, b->nv_total, b->stage_v, b->vmap, b->v_slots, b->tau_in);
    if (r) return r;
  } else if (p.control == GPB_CONTROL_PD && b->tau_in.n) {
    CUDA_TRY(cudaMemsetAsync(b->tau_in.p, 0, b->tau_in.n * sizeof(double), s));
  }
  int64_t rows = 0;
  if (history && record_every > 0) {
    rows = K / record_every;
    size_t need = (size_t)rows * (size_t)(b->nq_total + b->nv_total);
    if (b->hist.n < need) CUDA_TRY(b->hist.alloc(need));
    p.history = b->hist.p;
    p.record_every = record_every;
  }
  // body-parallel mapping (GPB_FP64 or GPB_MIXED steps of a chain batch), when
  // chosen; it factors H in FP64 whatever the algorithm setting, which
  // selects the one-lane route
  const int gs = (precision == GPB_FP64 || precision == GPB_MIXED) && integrator != GPB_VELOCITY_STEPPING &&
                         b->lanes > 1
                     ? group_bodies_per_lane(b, b->lanes)
                     : 0;
  p.ncoop = gs ? 0 : coop_packs(b, precision);
  p.group = gs ? b->lanes : 0;
  p.group_nvp = b->nv_max;
  if (b->npacks > 0 && K > 0) {
    CUDA_TRY(cudaEventRecord(b->ctx->ev0, s));
    if (gs)
      CUDA_TRY(launch_simulate_group(b->dev(), p, gs, b->ctx->num_sms, s));
    else
      CUDA_TRY(launch_simulate(b->dev(), p, b->ctx->num_sms, b->warps_per_sm, s));
    CUDA_TRY(cudaEventRecord(b->ctx->ev1, s));
    b->ctx->timed = true;
    b->ctx->launches++;
  }
  if (rows > 0)
    CUDA_TRY(cudaMemcpyAsync(history, b->hist.p, rows * (b->nq_total + b->nv_total) * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  return GPB_OK;
}

extern "C" int gpb_step(gpb_batch* b, double dt, const double* tau, int integrator, int precision) {
  if (!b) return fail(GPB_E_INVAL, "gpb_step: batch is NULL");
  gpb_control_params c;
  std::memset(&c, 0, sizeof(c));
  c.mode = GPB_CONTROL_HOST_TAU;
  c.tau = tau;
  int r = run_simulate(b, dt, 1, 0, integrator, precision, &c, 0, nullptr);
  if (r) return r;
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return GPB_OK;
}

// Launch-shape autotuner: short timed trials of the batch's own step from its
// current state (restored after every trial and at the end).
extern "C" int gpb_batch_autotune(gpb_batch* b, double dt, int integrator, int precision,
                                  const gpb_control_params* control, int trial_steps, int* warps_per_sm,
                                  int* coop_min_dof, int* lanes_per_instance) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_autotune: batch is NULL");
  if (int r = check_enums(integrator, precision)) return r;
  if (trial_steps < 1) return fail(GPB_E_INVAL, "gpb_batch_autotune: trial_steps must be >= 1");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t s = b->ctx->stream;
  DBuf<double> q0, v0, t0;
  DBuf<int32_t> st0;
  CUDA_TRY(q0.alloc(b->q.n));
  CUDA_TRY(v0.alloc(b->v.n));
  CUDA_TRY(t0.alloc(b->tau_in.n));
  CUDA_TRY(st0.alloc(b->status.n));
  auto copy = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s) : cudaSuccess;
  };
  auto save_restore = [&](bool save) -> cudaError_t {
    cudaError_t e = save ? copy(q0.p, b->q.p, b->q.n * 8) : copy(b->q.p, q0.p, b->q.n * 8);
    if (e == cudaSuccess) e = save ? copy(v0.p, b->v.p, b->v.n * 8) : copy(b->v.p, v0.p, b->v.n * 8);
    if (e == cudaSuccess)
      e = save ? copy(t0.p, b->tau_in.p, b->tau_in.n * 8) : copy(b->tau_in.p, t0.p, b->tau_in.n * 8);
    if (e == cudaSuccess)
      e = save ? copy(st0.p, b->status.p, b->status.n * 4) : copy(b->status.p, st0.p, b->status.n * 4);
    return e;
  };
  CUDA_TRY(save_restore(true));
  const int keep_w = b->warps_per_sm, keep_c = b->coop_min_dof, keep_l = b->lanes;
  struct Shape {
    int w, c, l;  // warps per SM, block-cooperative threshold, lanes per instance
  };
  // one lane per instance: 4 warps per SM and every further multiple of 4 the
  // kernel's registers leave room for, up to 16
  int wmax = 8;
  CUDA_TRY(simulate_max_warps_per_sm(precision, &wmax));
  std::vector<Shape> cand;
  for (int w = 4; w <= 16 && (w == 4 || w <= wmax); w += 4) {
    cand.push_back({w, 0, 1});
    if (precision != GPB_MIXED_REFINED && b->algorithm == GPB_ALGO_CRBA && b->npacks > 0 &&
        b->packs_h[0].minnv >= 32)
      for (int c : {40, 32}) cand.push_back({w, c, 1});
  }
  // body-parallel chains: the group sizes with one or two bodies per lane, and
  // a 4-warp block per instance for chains longer than 16 bodies in batches of
  // at most 4 instances per SM (beyond that the schedulers' FP64 units are
  // full and a warp per instance is ahead: 1,024 chains 4.9 against 2.6 M
  // instance-steps/s on GB300)
  if ((precision == GPB_FP64 || precision == GPB_MIXED) && integrator != GPB_VELOCITY_STEPPING) {
    for (int l = 2; l <= LANES; l *= 2)
      if (group_bodies_per_lane(b, l) && (l < 2 * b->nb_max || l == 2)) cand.push_back({0, 0, l});
    if (group_bodies_per_lane(b, 4 * LANES) && b->nb_max > LANES / 2 && b->n <= 4 * (int64_t)b->ctx->num_sms)
      cand.push_back({0, 0, 4 * LANES});
  }
  double best = 1e300;
  Shape pick{keep_w, keep_c, keep_l};
  int err = GPB_OK;
  for (const auto& cw : cand) {
    b->warps_per_sm = cw.w;
    b->coop_min_dof = cw.c;
    b->lanes = cw.l;
    CUDA_TRY(save_restore(false));
    // one untimed step, then the timed trial
    err = run_simulate(b, dt, 1, 0, integrator, precision, control, 0, nullptr);
    if (err == GPB_OK) err = run_simulate(b, dt, trial_steps, 1, integrator, precision, control, 0, nullptr);
    if (err != GPB_OK) break;
    const double ms = gpb_last_launch_ms(b->ctx);
    if (ms >= 0.0 && ms < best) {
      best = ms;
      pick = cw;
    }
  }
  b->warps_per_sm = err == GPB_OK ? pick.w : keep_w;
  b->coop_min_dof = err == GPB_OK ? pick.c : keep_c;
  b->lanes = err == GPB_OK ? pick.l : keep_l;
  CUDA_TRY(save_restore(false));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (err != GPB_OK) return err;
  if (warps_per_sm) *warps_per_sm = pick.w;
  if (coop_min_dof) *coop_min_dof = pick.c;
  if (lanes_per_instance) *lanes_per_instance = pick.l;
  return GPB_OK;
}

extern "C" int gpb_simulate(gpb_batch* b, double dt, int64_t K, int64_t step0, int integrator,
                            int precision, const gpb_control_params* control, int64_t record_every,
                            double* history) {
  if (!b) return fail(GPB_E_INVAL, "gpb_simulate: batch is NULL");
  int r = run_simulate(b, dt, K, step0, integrator, precision, control, record_every, history);
  if (r) return r;
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return GPB_OK;
}

extern "C" int64_t gpb_simulate_steps(double final_time, double dt) {
  if (!(dt > 0.0)) return -1;
  double t = 0.0;
  int64_t k = 0;
  while (t < final_time) {  // src/simulate.rs:102-109
    t += dt;
    ++k;
  }
  return k;
}

extern "C" int gpb_batch_status(gpb_batch* b, int32_t* status) {
  if (!b || !status) return fail(GPB_E_INVAL, "gpb_batch_status: NULL argument");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  std::vector<int32_t> slots(b->status.n);
  if (!slots.empty())
    CUDA_TRY(cudaMemcpyAsync(slots.data(), b->status.p, slots.size() * sizeof(int32_t),
                             cudaMemcpyDeviceToHost, b->ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  for (int64_t i = 0; i < b->n; ++i) status[i] = slots[b->status_slot[i]];
  return GPB_OK;
}

extern "C" int gpb_batch_steps_done(gpb_batch* b, int64_t* steps) {
  if (!b || !steps) return fail(GPB_E_INVAL, "gpb_batch_steps_done: NULL argument");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  std::vector<int64_t> slots(b->done.n);
  if (!slots.empty())
    CUDA_TRY(cudaMemcpyAsync(slots.data(), b->done.p, slots.size() * sizeof(int64_t),
                             cudaMemcpyDeviceToHost, b->ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  for (int64_t i = 0; i < b->n; ++i) steps[i] = slots[b->status_slot[i]];
  return GPB_OK;
}

extern "C" int gpb_batch_clear_status(gpb_batch* b) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_clear_status: batch is NULL");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  if (b->status.n) CUDA_TRY(cudaMemsetAsync(b->status.p, 0, b->status.n * sizeof(int32_t), b->ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return GPB_OK;
}

// q̈ from caller device buffers with the library's static scratch: no device
// memory is allocated or freed here (see gpb.h).
extern "C" int gpb_dynamics_static(gpb_batch* b, const double* q, const double* v,
                                   const double* tau, int precision, double* qdd, void* stream) {
  if (!b || !q || !v || !qdd) return fail(GPB_E_INVAL, "gpb_dynamics_static: NULL argument");
  if (int r = check_enums(0, precision)) return r;
  const int64_t limit = (int64_t)(GPB_STATIC_SCRATCH_BYTES / sizeof(double));
  if (b->scratch_words > limit)
    return fail(GPB_E_RANGE, "gpb_dynamics_static: the batch needs " +
                                 std::to_string(b->scratch_words * 8) + " bytes of scratch; the static array holds " +
                                 std::to_string((int64_t)GPB_STATIC_SCRATCH_BYTES) +
                                 " (use gpb_dynamics, or a smaller batch)");
  CUDA_TRY(cudaSetDevice(b->ctx->device));
  // A host pointer would make the kernel fault: accept device or managed memory only.
  const void* bufs[4] = {q, v, qdd, tau};
  const char* names[4] = {"q", "v", "qdd", "tau"};
  for (int k = 0; k < 4; ++k) {
    if (!bufs[k]) continue;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, bufs[k]) != cudaSuccess) {
      cudaGetLastError();  // clear the sticky-free error of an unknown pointer
      return fail(GPB_E_INVAL, std::string("gpb_dynamics_static: ") + names[k] + " is not a CUDA pointer");
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
      return fail(GPB_E_INVAL, std::string("gpb_dynamics_static: ") + names[k] +
                                   " must be device or managed memory");
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : b->ctx->stream;
  CUDA_TRY(launch_dynamics_static(b->dev(), b->ctx->device, b->scratch_words, precision, q, v, tau,
                                  qdd, s));
  b->ctx->launches++;
  return GPB_OK;
}

extern "C" int gpb_collide_cuboids_device(gpb_ctx* ctx, int64_t n, const double* pose_a, const double* size_a,
                                          const double* pose_b, const double* size_b, int32_t* result,
                                          double* cp_a, double* cp_b, void* stream) {
  if (!ctx || n < 0) return fail(GPB_E_INVAL, "gpb_collide_cuboids_device: bad argument");
  if (n == 0) return GPB_OK;
  if (!pose_a || !size_a || !pose_b || !size_b || !result || !cp_a || !cp_b)
    return fail(GPB_E_INVAL, "gpb_collide_cuboids_device: NULL buffer");
  CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  CUDA_TRY(launch_collide(n, pose_a, size_a, pose_b, size_b, result, cp_a, cp_b, ctx->num_sms, s));
  ctx->launches++;
  return GPB_OK;
}

extern "C" int gpb_collide_cuboids(gpb_ctx* ctx, int64_t n, const double* pose_a, const double* size_a,
                                   const double* pose_b, const double* size_b, int32_t* result, double* cp_a,
                                   double* cp_b) {
  if (!ctx || n < 0) return fail(GPB_E_INVAL, "gpb_collide_cuboids: bad argument");
  if (n == 0) return GPB_OK;
  if (!pose_a || !size_a || !pose_b || !size_b || !result || !cp_a || !cp_b)
    return fail(GPB_E_INVAL, "gpb_collide_cuboids: NULL buffer");
  CUDA_TRY(cudaSetDevice(ctx->device));
  // one allocation: poses (14 n), sizes (6 n), contact points (6 n), results (n int32)
  DBuf<double> d;
  if (d.alloc((size_t)n * 26 + ((size_t)n + 1) / 2) != cudaSuccess)
    return fail(GPB_E_NOMEM, "gpb_collide_cuboids: device allocation failed");
  double *pa = d.p, *pb = pa + 7 * n, *sa = pb + 7 * n, *sb = sa + 3 * n, *ca = sb + 3 * n, *cb = ca + 3 * n;
  int32_t* res = reinterpret_cast<int32_t*>(cb + 3 * n);
  cudaStream_t s = ctx->stream;
  int rc = GPB_OK;
  auto h2d = [&](double* dst, const double* src, int64_t k) {
    return cudaMemcpyAsync(dst, src, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, s);
  };
  cudaError_t e = h2d(pa, pose_a, 7 * n);
  if (e == cudaSuccess) e = h2d(pb, pose_b, 7 * n);
  if (e == cudaSuccess) e = h2d(sa, size_a, 3 * n);
  if (e == cudaSuccess) e = h2d(sb, size_b, 3 * n);
  if (e == cudaSuccess) e = launch_collide(n, pa, sa, pb, sb, res, ca, cb, ctx->num_sms, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cp_a, ca, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cp_b, cb, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(result, res, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) rc = fail(GPB_E_CUDA, std::string("gpb_collide_cuboids: ") + cudaGetErrorString(e));
  ctx->launches++;
  cudaStreamSynchronize(s);
  d.free();
  return rc;
}

extern "C" double gpb_open_loop_tau(uint32_t seed, int64_t instance, int64_t block, int32_t dof,
                                    double sigma) {
  return gpb::open_loop_tau(seed, instance, block, dof, sigma);
}
