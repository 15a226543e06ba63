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
#include "gpb_internal.h"

using namespace gpb;

// ---------------------------------------------------------------------------
// errors

static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess)                                                                \
      return fail(GPB_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));        \
  } while (0)

extern "C" int gpb_abi_version(void) { return GPB_ABI_VERSION; }
extern "C" const char* gpb_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// device buffers

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
  int mapping = 0;
  int warps_per_sm = 0;  // resident warps per SM of the step kernel (0 = occupancy limit)
  std::vector<int64_t> q_off, v_off, c_off;  // user layout, [n+1]
  int64_t nq_total = 0, nv_total = 0, nc_total = 0;
  std::vector<PackDesc> packs_h;
  int64_t q_slots = 0, v_slots = 0, c_slots = 0;
  int64_t scratch_words = 0;  // 8-byte words of per-instance scratch, all packs
  std::vector<int32_t> status_slot;  // user instance -> status slot (pack*32+lane)
  DBuf<PackDesc> packs;
  DBuf<uint32_t> topoW;
  DBuf<double> topoD, ctcD, hsD, q, v, tau_in, scratch, stage_q, stage_v, stage_c, hist;
  DBuf<float> topoF, ctcF, hsF;
  DBuf<int32_t> ctcI, laneI, status, queue;
  DBuf<int64_t> qmap, vmap, cmap, done;
  DeviceBatch dev() const {
    DeviceBatch b;
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

namespace {

struct InstInfo {
  int32_t j0, nb, nq, nv, c0, nc, h0, nh, model;
  bool chain;
  uint64_t sig;  // topology class
};

static int joint_nq(int t) { return t == GPB_JOINT_FLOATING ? 7 : (t == GPB_JOINT_FIXED ? 0 : 1); }
static int joint_nv(int t) { return t == GPB_JOINT_FLOATING ? 6 : (t == GPB_JOINT_FIXED ? 0 : 1); }

// Quaternion (x,y,z,w) → row-major rotation matrix (same formula as
// UnitQuaternion::to_rotation_matrix).
static void quat_to_rot(const double* q, double* m) {
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

}  // namespace

extern "C" int gpb_batch_create(gpb_ctx* ctx, const gpb_model* m, gpb_batch** out) {
  if (!ctx || !m || !out) return fail(GPB_E_INVAL, "gpb_batch_create: NULL argument");
  if (m->n_instances < 0) return fail(GPB_E_INVAL, "gpb_batch_create: negative instance count");
  if (!m->joint_offset || !m->joint_type || !m->joint_parent || !m->joint_iso || !m->joint_axis ||
      !m->body_inertia)
    return fail(GPB_E_INVAL, "gpb_batch_create: joint/body tables missing");
  const int64_t n = m->n_instances;
  std::vector<InstInfo> info(n);
  for (int64_t i = 0; i < n; ++i) {
    InstInfo& I = info[i];
    I.j0 = m->joint_offset[i];
    I.nb = m->joint_offset[i + 1] - I.j0;
    if (I.nb < 0 || I.nb > GPB_MAX_BODIES)
      return fail(GPB_E_RANGE, "instance " + std::to_string(i) + ": body count outside [0, 64]");
    I.nq = I.nv = 0;
    I.chain = true;
    uint64_t sig = 1469598103934665603ull;
    for (int b = 0; b < I.nb; ++b) {
      int t = m->joint_type[I.j0 + b], p = m->joint_parent[I.j0 + b];
      if (t < 0 || t > 3) return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": bad joint type");
      if (p < 0 || p > b)
        return fail(GPB_E_INVAL, "instance " + std::to_string(i) + ": joint " + std::to_string(b + 1) +
                                     " has parent " + std::to_string(p) + " (must be < its own number)");
      if (p != b) I.chain = false;
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
    sig = (sig ^ (uint64_t)(I.nc * 7 + I.nh)) * 1099511628211ull;
    I.sig = sig;
  }

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
  int64_t rt = 0, rc = 0, rh = 0, rq = 0, rv = 0, rl = 0, rs = 0;
  for (int64_t p = 0; p < npacks; ++p) {
    PackDesc& P = B->packs_h[p];
    std::memset(&P, 0, sizeof(P));
    P.count = (int32_t)std::min<int64_t>(LANES, n - p * LANES);
    P.chain = 1;
    for (int l = 0; l < P.count; ++l) {
      const InstInfo& I = info[order[p * LANES + l]];
      P.nb = std::max(P.nb, I.nb);
      P.nq = std::max(P.nq, I.nq);
      P.nv = std::max(P.nv, I.nv);
      P.nc = std::max(P.nc, I.nc);
      P.nh = std::max(P.nh, I.nh);
      if (!I.chain) P.chain = 0;
    }
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
    rs += scratch_layout(P.nb, P.nq, P.nv, P.nc).total;
  }
  const size_t L = LANES;
  std::vector<uint32_t> W(rt * 2 * L, 0);
  std::vector<double> TD(rt * TOPO_D * L, 0.0), CD(rc * CTC_D * L, 0.0), HD(rh * HS_D * L, 0.0);
  std::vector<int32_t> CI(rc * L, 0), LI(rl * L, 0);
  std::vector<int64_t> qmap(rq * L, -1), vmap(rv * L, -1), cmap(rc * 3 * L, -1);
  std::vector<double> q0(rq * L, 0.0);
  B->status_slot.assign(n, 0);
  for (int64_t p = 0; p < npacks; ++p) {
    const PackDesc& P = B->packs_h[p];
    for (int l = 0; l < LANES; ++l) {
      int64_t li = P.lane * L + l;
      if (l >= P.count) {
        LI[li] = -1;
        continue;
      }
      const int64_t inst = order[p * LANES + l];
      const InstInfo& I = info[inst];
      B->status_slot[inst] = (int32_t)(p * LANES + l);
      LI[li] = (int32_t)inst;
      LI[li + 1 * L] = I.nb;
      LI[li + 2 * L] = I.nq;
      LI[li + 3 * L] = I.nv;
      LI[li + 4 * L] = I.nc;
      LI[li + 5 * L] = I.nh;
      LI[li + 6 * L] = I.model;
      // contacts sorted by body (stable), remembering the user order
      std::vector<int> corder(I.nc);
      std::iota(corder.begin(), corder.end(), 0);
      std::stable_sort(corder.begin(), corder.end(), [&](int a, int b) {
        return m->contact_body[I.c0 + a] < m->contact_body[I.c0 + b];
      });
      std::vector<int> cfirst(I.nb, 0), ccount(I.nb, 0);
      for (int k = 0; k < I.nc; ++k) {
        int src = corder[k];
        int body = m->contact_body[I.c0 + src] - 1;
        if (ccount[body] == 0) cfirst[body] = k;
        ccount[body]++;
        CI[(P.ctc + k) * L + l] = body | (src << 8);
        const double* cp = m->contact_params + 6 * (size_t)(I.c0 + src);
        for (int e = 0; e < CTC_D; ++e) CD[((P.ctc) * CTC_D + CTC_D * k + e) * L + l] = cp[e];
      }
      // the kernel writes contact forces by the contact's user-order index
      for (int k = 0; k < I.nc; ++k)
        for (int e = 0; e < 3; ++e) cmap[(P.ctc * 3 + 3 * k + e) * L + l] = 3 * (B->c_off[inst] + k) + e;
      for (int h = 0; h < I.nh; ++h) {
        const double* hp = m->halfspace_params + 8 * (size_t)(I.h0 + h);
        double nn = std::sqrt(hp[3] * hp[3] + hp[4] * hp[4] + hp[5] * hp[5]);
        double vals[8] = {hp[0], hp[1], hp[2], hp[3] / nn, hp[4] / nn, hp[5] / nn, hp[6], hp[7]};
        for (int e = 0; e < HS_D; ++e) HD[(P.hs * HS_D + HS_D * h + e) * L + l] = vals[e];
      }
      // bodies
      std::vector<bool> branch(I.nb, false);
      for (int b = 0; b < I.nb; ++b) {
        int par = m->joint_parent[I.j0 + b];  // 1-based
        if (par >= 1 && par != b) branch[par - 1] = true;
      }
      int qo = 0, vo = 0;
      for (int b = 0; b < I.nb; ++b) {
        const int j = I.j0 + b;
        int t = m->joint_type[j], par = m->joint_parent[j];
        const double* iso = m->joint_iso + 7 * (size_t)j;
        const double* ax = m->joint_axis + 3 * (size_t)j;
        const double* in = m->body_inertia + 10 * (size_t)j;
        double sk = m->joint_spring ? m->joint_spring[2 * (size_t)j] : 0.0;
        double sl = m->joint_spring ? m->joint_spring[2 * (size_t)j + 1] : 0.0;
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
        W[((P.topo + b) * 2) * L + l] =
            (uint32_t)t | ((uint32_t)par << 4) | ((uint32_t)qo << 12) | ((uint32_t)vo << 22);
        W[((P.topo + b) * 2 + 1) * L + l] =
            flags | ((uint32_t)cfirst[b] << 8) | ((uint32_t)ccount[b] << 16);
        double vals[TOPO_D];
        for (int e = 0; e < 9; ++e) vals[TD_RINIT + e] = R[e];
        for (int e = 0; e < 3; ++e) vals[TD_TINIT + e] = iso[4 + e];
        for (int e = 0; e < 3; ++e) vals[TD_AXIS + e] = ax[e];
        for (int e = 0; e < 10; ++e) vals[TD_INERTIA + e] = in[e];
        vals[TD_SPRING] = sk;
        vals[TD_SPRING + 1] = sl;
        for (int e = 0; e < TOPO_D; ++e) TD[((P.topo) * TOPO_D + TOPO_D * b + e) * L + l] = vals[e];
        // state maps and the zero state (identity pose for floating joints)
        for (int e = 0; e < joint_nq(t); ++e) qmap[(P.q + qo + e) * L + l] = B->q_off[inst] + qo + e;
        if (t == GPB_JOINT_FLOATING) q0[(P.q + qo + 3) * L + l] = 1.0;
        for (int e = 0; e < joint_nv(t); ++e) vmap[(P.v + vo + e) * L + l] = B->v_off[inst] + vo + e;
        qo += joint_nq(t);
        vo += joint_nv(t);
      }
    }
  }
  std::vector<float> TF(TD.begin(), TD.end()), CF(CD.begin(), CD.end()), HF(HD.begin(), HD.end());

  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSetDevice(ctx->device);
  auto chk = [&](cudaError_t x) {
    if (x != cudaSuccess && e == cudaSuccess) e = x;
  };
  B->scratch_words = rs * L;
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
  chk(B->queue.alloc(1));
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

extern "C" int gpb_batch_set_mapping(gpb_batch* b, int lanes) {
  if (!b) return fail(GPB_E_INVAL, "gpb_batch_set_mapping: batch is NULL");
  if (lanes != 0 && lanes != 1) return fail(GPB_E_INVAL, "gpb_batch_set_mapping: lanes must be 0 or 1");
  b->mapping = lanes;
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
  if (integrator < 0 || integrator > 2) return fail(GPB_E_INVAL, "unknown integrator");
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

static int run_simulate(gpb_batch* b, double dt, int64_t K, int64_t step0, int integrator,
                        int precision, const gpb_control_params* ctl, int64_t record_every,
                        double* history) {
  if (int r = check_enums(integrator, precision)) return r;
  if (K < 0) return fail(GPB_E_INVAL, "negative step count");
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
  if (b->npacks > 0 && K > 0) {
    CUDA_TRY(cudaEventRecord(b->ctx->ev0, s));
    CUDA_TRY(launch_simulate(b->dev(), p, b->mapping, b->ctx->num_sms, b->warps_per_sm, s));
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
  cudaStream_t s = stream ? (cudaStream_t)stream : b->ctx->stream;
  CUDA_TRY(launch_dynamics_static(b->dev(), b->ctx->device, b->scratch_words, precision, q, v, tau,
                                  qdd, s));
  b->ctx->launches++;
  return GPB_OK;
}

extern "C" double gpb_open_loop_tau(uint32_t seed, int64_t instance, int64_t block, int32_t dof,
                                    double sigma) {
  return gpb::open_loop_tau(seed, instance, block, dof, sigma);
}
