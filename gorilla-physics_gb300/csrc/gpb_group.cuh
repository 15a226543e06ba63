// Body-parallel mapping of the step for serial chains (included by
// gpb_kernels.cu after the per-lane evaluators, make_ctx and control).
//
// G lanes of a warp (G = 2, 4, 8, 16 or 32) step one instance together, so a
// warp holds 32 / G instances of a pack; G = 32 is one warp per instance; or a
// whole 4-warp block does (G = 128, group_block_kernel: the warps' scan totals
// meet in shared memory and the barriers are block barriers).  Lane t of a
// group owns the S consecutive bodies t·S … t·S + S − 1 of the chain (S = 1 or
// 2, G·S ≥ bodies).  One dynamics evaluation
// (src/dynamics.rs:322-364) becomes:
//   outward   world poses are the prefix products X_1 X_2 … X_b of the joint
//             transforms; body velocities and bias accelerations are prefix
//             sums of S_a q̇_a and of V_{a−1} ×m S_a q̇_a, computed as one scan of
//             pairs with (V1, A1) ⊕ (V2, A2) = (V1 + V2, A1 + A2 + V1 ×m V2)
//             (associative because ×m is bilinear).  Each scan is a serial
//             pass over the lane's own bodies, then a Kogge–Stone scan of the
//             lane totals across the group by warp shuffles;
//   per body  the world inertia, the Newton–Euler force and the point
//             contacts, each on the lane that owns the body;
//   inward    composite inertias and joint forces are suffix sums along the
//             chain, the same scan in the other direction;
//   H         on a chain every body is an ancestor of the next, so
//             H_ij = (Ic_i S_i) · S_j for j ≤ i (src/mechanism.rs:592-696);
//             the lower triangle is filled in shared memory, its entries dealt
//             evenly to the lanes;
//   solve     Cholesky H = L Lᵀ, right-looking by 4-column panels (every lane
//             factors the diagonal block, the rows below it and the trailing
//             update's entries are dealt evenly to the lanes), then the two
//             triangular solves by the same panels (src/dynamics.rs:255-276
//             solves the same system by LU).
// It serves instances too few to fill the GPU one lane each, where the
// latency of one instance's step sets the rate.  The arithmetic is FP64 for
// GPB_FP64 and GPB_MIXED requests alike: a double-float version of this
// kernel (every sum and product on the FP32 pipes) measured no faster on
// GB300 — 1,024 chains 4.6 against 4.7 M instance-steps/s, a lone 48-body
// chain 166 against 188 µs a step — since one instance's chain of dependent
// operations and barriers, not the FP64 pipe's throughput, sets its step
// time.  Its sums run in another order than the one-lane sweeps, so the two
// mappings agree to rounding, not bit for bit.
//
// Every shuffle and __syncwarp of a group runs under the group's own mask and
// in control flow that depends only on the instance (never on the lane), so
// groups of one warp may diverge from each other (different instances).

#pragma once

namespace grp {

using gpb::M3;
using gpb::SI;
using gpb::SV;
using gpb::V3;

// Rigid transform (rotation, translation): x ↦ R x + p.
struct Xf {
  M3<double> R;
  V3<double> p;
};
__device__ __forceinline__ Xf identity() {
  Xf x;
#pragma unroll
  for (int k = 0; k < 9; ++k) x.R.a[k] = 0.0;
  x.R.a[0] = x.R.a[4] = x.R.a[8] = 1.0;
  x.p = {0.0, 0.0, 0.0};
  return x;
}
// a ∘ b: first b, then a
__device__ __forceinline__ Xf compose(const Xf& a, const Xf& b) {
  return {gpb::mul(a.R, b.R), a.p + gpb::mul(a.R, b.p)};
}

__device__ __forceinline__ double up(unsigned m, double x, int d, int G) { return __shfl_up_sync(m, x, d, G); }
__device__ __forceinline__ double dn(unsigned m, double x, int d, int G) { return __shfl_down_sync(m, x, d, G); }
__device__ __forceinline__ V3<double> up3(unsigned m, V3<double> x, int d, int G) {
  return {up(m, x.x, d, G), up(m, x.y, d, G), up(m, x.z, d, G)};
}
__device__ __forceinline__ V3<double> dn3(unsigned m, V3<double> x, int d, int G) {
  return {dn(m, x.x, d, G), dn(m, x.y, d, G), dn(m, x.z, d, G)};
}
__device__ __forceinline__ Xf up_xf(unsigned m, const Xf& x, int d, int G) {
  Xf y;
#pragma unroll
  for (int k = 0; k < 9; ++k) y.R.a[k] = up(m, x.R.a[k], d, G);
  y.p = up3(m, x.p, d, G);
  return y;
}
__device__ __forceinline__ SV<double> up_sv(unsigned m, const SV<double>& x, int d, int G) {
  return {up3(m, x.w, d, G), up3(m, x.v, d, G)};
}
__device__ __forceinline__ SV<double> dn_sv(unsigned m, const SV<double>& x, int d, int G) {
  return {dn3(m, x.w, d, G), dn3(m, x.v, d, G)};
}
__device__ __forceinline__ SI<double> dn_si(unsigned m, const SI<double>& x, int d, int G) {
  SI<double> y;
#pragma unroll
  for (int k = 0; k < 6; ++k) y.j[k] = dn(m, x.j[k], d, G);
  y.c = dn3(m, x.c, d, G);
  y.m = dn(m, x.m, d, G);
  return y;
}
__device__ __forceinline__ SV<double> sv_zero() { return {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}; }
__device__ __forceinline__ SI<double> si_zero() {
  SI<double> z;
#pragma unroll
  for (int k = 0; k < 6; ++k) z.j[k] = 0.0;
  z.c = {0.0, 0.0, 0.0};
  z.m = 0.0;
  return z;
}

// The values the three scans carry, their shuffles and combinations.
struct VA {  // (body velocity, bias acceleration) sums along the chain
  SV<double> V, A;
};
struct IFc {  // (composite inertia, joint force) sums from the tip
  SI<double> I;
  SV<double> F;
};
__device__ __forceinline__ Xf up1(unsigned m, const Xf& x, int d, int W) { return up_xf(m, x, d, W); }
__device__ __forceinline__ VA up1(unsigned m, const VA& x, int d, int W) {
  return {up_sv(m, x.V, d, W), up_sv(m, x.A, d, W)};
}
__device__ __forceinline__ IFc dn1(unsigned m, const IFc& x, int d, int W) {
  return {dn_si(m, x.I, d, W), dn_sv(m, x.F, d, W)};
}
// left-to-right combination: first a's segment of the chain, then b's
__device__ __forceinline__ Xf comb(const Xf& a, const Xf& b) { return compose(a, b); }
__device__ __forceinline__ VA comb(const VA& a, const VA& b) {
  return {a.V + b.V, a.A + b.A + gpb::crm(a.V, b.V)};
}
__device__ __forceinline__ IFc add(const IFc& a, const IFc& b) {
  IFc r = a;
  gpb::iadd(r.I, b.I);
  r.F = a.F + b.F;
  return r;
}

// Barrier and OR-reduction of a group: its lanes of one warp, or (BLK) the
// whole block, which then steps one instance.
template <bool BLK>
__device__ __forceinline__ void gsync(unsigned gm) {
  if constexpr (BLK)
    __syncthreads();
  else
    __syncwarp(gm);
}
template <bool BLK>
__device__ __forceinline__ unsigned gor(unsigned gm, unsigned v) {
  if constexpr (BLK) {  // __syncthreads_or answers any-nonzero, not the OR of the bits: one per status bit
    unsigned r = 0;
#pragma unroll
    for (int bit = 0; bit < 4; ++bit)
      if (__syncthreads_or((int)(v & (1u << bit)))) r |= 1u << bit;
    return r;
  } else {
    return __reduce_or_sync(gm, v);
  }
}

// Exclusive prefix scan of x over the group's lanes (the combination of the
// values of lanes 0 … t−1; ident for lane 0): Kogge–Stone by shuffles within
// a warp; with BLK the warps' totals then meet in shared memory (wsm, one
// slot per warp), each warp combining those of the warps before it.
template <bool BLK, typename T>
__device__ __forceinline__ T excl_prefix(T x, int t, int G, unsigned gm, const T& ident, T* wsm) {
  const int W = BLK ? 32 : G, lane = BLK ? (t & 31) : t;
  for (int d = 1; d < W; d <<= 1) {
    const T y = up1(gm, x, d, W);
    if (lane >= d) x = comb(y, x);
  }
  T pre = ident;
  if constexpr (BLK) {
    const int w = t >> 5;
    if (lane == W - 1) wsm[w] = x;
    __syncthreads();
    for (int u = 0; u < w; ++u) pre = comb(pre, wsm[u]);
    __syncthreads();  // the slots are reused by the next scan
    x = comb(pre, x);
  }
  T e = up1(gm, x, 1, W);
  if (lane == 0) e = pre;
  return e;
}
// Exclusive suffix sum over the group's lanes (lanes t+1 … G−1; zero for the
// last), the same way from the other end.
template <bool BLK>
__device__ __forceinline__ IFc excl_suffix(IFc x, int t, int G, unsigned gm, const IFc& zero, IFc* wsm) {
  const int W = BLK ? 32 : G, lane = BLK ? (t & 31) : t;
  for (int d = 1; d < W; d <<= 1) {
    const IFc y = dn1(gm, x, d, W);
    if (lane + d < W) x = add(x, y);
  }
  IFc post = zero;
  if constexpr (BLK) {
    const int w = t >> 5, nw = G >> 5;
    if (lane == 0) wsm[w] = x;
    __syncthreads();
    for (int u = nw - 1; u > w; --u) post = add(post, wsm[u]);
    __syncthreads();
    x = add(x, post);
  }
  IFc e = dn1(gm, x, 1, W);
  if (lane == W - 1) e = post;
  return e;
}

// Doubles of shared memory per instance for up to n DOF: packed lower
// triangle of H (row i at i(i+1)/2), the world motion subspaces and the
// columns Ic_i S_i (6 n each, component-major), the right-hand side, the
// intermediate vector of the solves and the reciprocal pivots (n each).
// The matrix is padded to whole 4×4 panels (identity rows beyond n).
__host__ __device__ inline int smem_words(int n) {
  const int m = (n + 3) & ~3;
  return m * (m + 1) / 2 + 15 * m;
}
// A block per instance also keeps its warps' scan totals: 4 warps × 16 doubles.
constexpr int BLK_WARPS = 4;
constexpr int BLK_SCAN_WORDS = BLK_WARPS * 16;

__device__ __forceinline__ int off(int i) { return (i * (i + 1)) >> 1; }

// One instance as seen by the lanes of its group.
template <int S>
struct Inst {
  int G, t;       // group size, lane in the group
  unsigned gm;    // the group's lanes
  int nb, nv, nc, nh, model;
  double grav;
  double* sm;     // this instance's shared memory (smem_words(nvp))
  int nvp;
  // tables of the instance (lane of the pack applied)
  const uint32_t* W;
  const double* T;
  const double* CD;
  const double* HD;
  // the lane's bodies
  int type[S], qo[S], vo[S];
  uint32_t w1[S];
  __device__ __forceinline__ double t_(int e) const { return __ldg(T + (size_t)e * gpb::LANES); }
  __device__ __forceinline__ double cd(int e) const { return __ldg(CD + (size_t)e * gpb::LANES); }
  __device__ __forceinline__ double hd(int e) const { return __ldg(HD + (size_t)e * gpb::LANES); }
  __device__ __forceinline__ int body(int s) const { return t * S + s; }
  __device__ __forceinline__ bool dof(int s) const { return type[s] == 1 || type[s] == 2; }
};

// Joint transform of body bb (parent frame ← body frame) at joint position qv:
// (Rinit Rot(axis, q), tinit) for a revolute joint, (Rinit, tinit + q Rinit axis)
// for a prismatic one (src/joint/revolute.rs, src/joint/prismatic.rs).
template <int S>
__device__ __forceinline__ Xf joint_xf(const Inst<S>& g, int s, double qv) {
  const int tb = gpb::TOPO_D * g.body(s);
  const uint32_t fl = g.w1[s] & 255u;
  Xf x;
  if (fl & gpb::BF_INIT_ROT_IDENTITY) {
    x = identity();
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) x.R.a[k] = g.t_(tb + gpb::TD_RINIT + k);
  }
  x.p = {g.t_(tb + gpb::TD_TINIT), g.t_(tb + gpb::TD_TINIT + 1), g.t_(tb + gpb::TD_TINIT + 2)};
  const V3<double> ax{g.t_(tb + gpb::TD_AXIS), g.t_(tb + gpb::TD_AXIS + 1), g.t_(tb + gpb::TD_AXIS + 2)};
  if (g.type[s] == 1) {
    double sn, co;
    sincos(qv, &sn, &co);
    if (fl & gpb::BF_AXIS_PRINCIPAL) {
      const int ai = gpb::bf_axis_index(fl);
      const double sg = (fl & gpb::BF_AXIS_NEG) ? -sn : sn;
      const int i1 = (ai + 1) % 3, i2 = (ai + 2) % 3;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const double a1 = x.R.a[3 * r + i1], a2 = x.R.a[3 * r + i2];
        x.R.a[3 * r + i1] = a1 * co + a2 * sg;
        x.R.a[3 * r + i2] = a2 * co - a1 * sg;
      }
    } else {
      // rows of Rinit Rot: r Rot = c r + s (r × a) + (1 − c)(r · a) a
      const double omc = 1.0 - co;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const V3<double> ar{x.R.a[3 * r], x.R.a[3 * r + 1], x.R.a[3 * r + 2]};
        const V3<double> cx = gpb::cross(ar, ax);
        const double d = gpb::dot(ar, ax) * omc;
        x.R.a[3 * r] = ar.x * co + cx.x * sn + ax.x * d;
        x.R.a[3 * r + 1] = ar.y * co + cx.y * sn + ax.y * d;
        x.R.a[3 * r + 2] = ar.z * co + cx.z * sn + ax.z * d;
      }
    }
  } else if (g.type[s] == 2) {
    x.p = x.p + gpb::mul(x.R, ax) * qv;
  }
  return x;
}

// Point contacts of body s against the instance's half-spaces
// (src/contact.rs:97-128, 260-338): subtracts each contact's wrench from f.
template <int S>
__device__ __forceinline__ void contacts(const Inst<S>& g, int s, const Xf& X, const SV<double>& Vb,
                                         SV<double>& f) {
  const int cb = (g.w1[s] >> 8) & 255, cn = (g.w1[s] >> 16) & 255;
  for (int k = cb; k < cb + cn; ++k) {
    const int cd = gpb::CTC_D * k;
    const V3<double> loc{g.cd(cd), g.cd(cd + 1), g.cd(cd + 2)};
    const double kp = g.cd(cd + 3), rad = g.cd(cd + 4), damp = g.cd(cd + 5);
    const V3<double> pw = gpb::mul(X.R, loc) + X.p;
    for (int h = 0; h < g.nh; ++h) {
      const int hd = gpb::HS_D * h;
      const V3<double> hp{g.hd(hd), g.hd(hd + 1), g.hd(hd + 2)};
      const V3<double> hn{g.hd(hd + 3), g.hd(hd + 4), g.hd(hd + 5)};
      const double al = g.hd(hd + 6), mu = g.hd(hd + 7);
      const double dist = gpb::dot(pw - hp, hn);
      V3<double> app = pw;
      double pen;
      if (rad > 0.0) {
        if (!(dist - rad <= 1e-8)) continue;
        pen = rad - dist;
        app = pw - hn * rad;
      } else {
        if (!(dist <= 1e-8)) continue;  // HalfSpace::has_inside (margin 1e-8)
        pen = -dist;
      }
      const V3<double> vel = Vb.v + gpb::cross(Vb.w, app);
      const V3<double> fc = gpb::contact_force<double>(g.model, pen, hn, vel, kp, damp, al, mu);
      f.w = f.w - gpb::cross(app, fc);
      f.v = f.v - fc;
    }
  }
}

// One dynamics evaluation of the group's instance: q, v, τ of the lane's
// bodies → q̈ of the lane's bodies.  Returns GPB status bits (the same in
// every lane of the group).
template <int S, bool BLK>
__device__ __noinline__ int eval(const Inst<S>& gin, const double (&qin)[S], const double (&vin)[S],
                                 const double (&tauin)[S], bool ht, bool springs, double (&qdd)[S]) {
  const Inst<S> g = gin;  // private copies: kept in registers, not read through the references
  double q[S], v[S], tau[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    q[s] = qin[s];
    v[s] = vin[s];
    tau[s] = tauin[s];
  }
  const int G = g.G, t = g.t;
  const unsigned gm = g.gm;
  // ---- poses: the lane's own prefix products, then the scan of lane totals
  Xf X[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const Xf J = g.body(s) < g.nb ? joint_xf(g, s, q[s]) : identity();
    X[s] = s == 0 ? J : compose(X[s - 1], J);
  }
  double* const wsm = g.sm + smem_words(g.nvp);  // BLK: the warps' scan totals
  {
    const Xf E = excl_prefix<BLK>(X[S - 1], t, G, gm, identity(), reinterpret_cast<Xf*>(wsm));
    if (t > 0) {
#pragma unroll
      for (int s = 0; s < S; ++s) X[s] = compose(E, X[s]);
    }
  }
  // ---- motion subspaces (world), joint velocities S q̇
  SV<double> Sw[S], V[S], A[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    Sw[s] = sv_zero();
    if (g.body(s) < g.nb && g.dof(s)) {
      const int tb = gpb::TOPO_D * g.body(s);
      const V3<double> ax{g.t_(tb + gpb::TD_AXIS), g.t_(tb + gpb::TD_AXIS + 1), g.t_(tb + gpb::TD_AXIS + 2)};
      const V3<double> aw = gpb::mul(X[s].R, ax);
      Sw[s] = g.type[s] == 1 ? SV<double>{aw, gpb::cross(X[s].p, aw)} : SV<double>{{0.0, 0.0, 0.0}, aw};
    }
    const SV<double> vj = gpb::scale(Sw[s], v[s]);
    if (s == 0) {
      V[0] = vj;
      A[0] = sv_zero();
    } else {
      A[s] = A[s - 1] + gpb::crm(V[s - 1], vj);
      V[s] = V[s - 1] + vj;
    }
  }
  // ---- (V, A) scan
  {
    const VA E = excl_prefix<BLK>(VA{V[S - 1], A[S - 1]}, t, G, gm, VA{sv_zero(), sv_zero()},
                                  reinterpret_cast<VA*>(wsm));
    const SV<double> EV = E.V, EA = E.A;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      A[s] = EA + A[s] + gpb::crm(EV, V[s]);
      A[s].v.z += g.grav;  // inverse gravity at the root (src/dynamics.rs:211-218)
      V[s] = EV + V[s];
    }
  }
  // ---- world inertias, Newton–Euler forces, contacts (src/dynamics.rs:41-100)
  SI<double> Ic[S];
  SV<double> F[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    Ic[s] = si_zero();
    F[s] = sv_zero();
    if (g.body(s) >= g.nb) continue;
    const int tb = gpb::TOPO_D * g.body(s);
    SI<double> Ib;
#pragma unroll
    for (int k = 0; k < 6; ++k) Ib.j[k] = g.t_(tb + gpb::TD_INERTIA + 4 + k);
    Ib.c = {g.t_(tb + gpb::TD_INERTIA + 1), g.t_(tb + gpb::TD_INERTIA + 2), g.t_(tb + gpb::TD_INERTIA + 3)};
    Ib.m = g.t_(tb + gpb::TD_INERTIA);
    Ic[s] = gpb::to_world(Ib, X[s].R, X[s].p, (g.w1[s] & gpb::BF_DIAG_INERTIA) != 0);
    F[s] = gpb::imul(Ic[s], A[s]) + gpb::crf(V[s], gpb::imul(Ic[s], V[s]));
    if (g.nc > 0) contacts(g, s, X[s], V[s], F[s]);
  }
  // ---- suffix sums: composite inertias and joint forces
#pragma unroll
  for (int s = S - 2; s >= 0; --s) {
    gpb::iadd(Ic[s], Ic[s + 1]);
    F[s] = F[s] + F[s + 1];
  }
  {
    const IFc E = excl_suffix<BLK>(IFc{Ic[0], F[0]}, t, G, gm, IFc{si_zero(), sv_zero()},
                                   reinterpret_cast<IFc*>(wsm));
    if (t + 1 < G) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
        gpb::iadd(Ic[s], E.I);
        F[s] = F[s] + E.F;
      }
    }
  }
  // ---- right-hand side, columns Ic S, diagonal of H
  const int n = g.nv, np = (g.nvp + 3) & ~3, n4 = (n + 3) & ~3;
  double* H = g.sm;
  double* Ssm = H + off(np);
  double* Fsm = Ssm + 6 * np;
  double* x = Fsm + 6 * np;
  double* z = x + np;
  double* dinv = z + np;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    if (g.body(s) >= g.nb || !g.dof(s)) continue;
    const int i = g.vo[s], tb = gpb::TOPO_D * g.body(s);
    const SV<double> Fi = gpb::imul(Ic[s], Sw[s]);
    const double sc[6] = {Sw[s].w.x, Sw[s].w.y, Sw[s].w.z, Sw[s].v.x, Sw[s].v.y, Sw[s].v.z};
    const double fc[6] = {Fi.w.x, Fi.w.y, Fi.w.z, Fi.v.x, Fi.v.y, Fi.v.z};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      Ssm[k * np + i] = sc[k];
      Fsm[k * np + i] = fc[k];
    }
    double rhs = ht ? tau[s] : 0.0;
    if (g.type[s] == 2 && (g.w1[s] & gpb::BF_SPRING) && springs)  // src/dynamics.rs:298-315
      rhs += -g.t_(tb + gpb::TD_SPRING) * (q[s] - g.t_(tb + gpb::TD_SPRING + 1));
    x[i] = rhs - gpb::sdot(Sw[s], F[s]);
    // (no armature: dynamics.rs's mass matrix has none; only free_velocity adds it)
    H[off(i) + i] = gpb::sdot2(Fi, Sw[s]);
  }
  gsync<BLK>(gm);
  // ---- strictly lower triangle of H, entry e = i(i−1)/2 + j to lane e mod G
  {
    int i = 1, j = t;
    while (j >= i) {
      j -= i;
      ++i;
    }
    while (i < n) {
      double h = 0.0;
#pragma unroll
      for (int k = 0; k < 6; ++k) h = fma(Fsm[k * np + i], Ssm[k * np + j], h);
      H[off(i) + j] = h;
      j += G;
      while (j >= i) {
        j -= i;
        ++i;
      }
    }
  }
  // padding rows n … n4−1: identity rows, zero right-hand side
  for (int i = n; i < n4; ++i) {
    for (int j = t; j <= i; j += G) H[off(i) + j] = j == i ? 1.0 : 0.0;
    if (t == 0) x[i] = 0.0;
  }
  // ---- Cholesky H = L Lᵀ in place, right-looking by 4-column panels: every
  // lane factors the 4×4 diagonal block in registers, the rows below it are
  // dealt to the lanes (each a 4-term triangular solve), then the trailing
  // block takes a rank-4 update entry by entry — two barriers per panel
  int st = 0;
  for (int k = 0; k < n4; k += 4) {
    gsync<BLK>(gm);
    double L[4][4], r[4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c <= a; ++c) L[a][c] = H[off(k + a) + k + c];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      double d = L[c][c];
#pragma unroll
      for (int e = 0; e < c; ++e) d = fma(-L[c][e], L[c][e], d);
      if (!(d > 0.0)) {
        st |= 2;  // GPB_ST_CHOL_FAIL; continue with a unit pivot, as the one-lane factor does
        d = 1.0;
      }
      r[c] = rsqrt(d);
      L[c][c] = d * r[c];
#pragma unroll
      for (int a = c + 1; a < 4; ++a) {
        double v = L[a][c];
#pragma unroll
        for (int e = 0; e < c; ++e) v = fma(-L[a][e], L[c][e], v);
        L[a][c] = v * r[c];
      }
    }
    for (int i = k + 4 + t; i < n4; i += G) {  // the panel's rows below the block
      double l[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double v = H[off(i) + k + c];
#pragma unroll
        for (int e = 0; e < c; ++e) v = fma(-l[e], L[c][e], v);
        l[c] = v * r[c];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) H[off(i) + k + c] = l[c];
    }
    gsync<BLK>(gm);
    if (t == 0) {  // the block's factor: no lane reads the block again in this panel
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int c = 0; c <= a; ++c) H[off(k + a) + k + c] = L[a][c];
        dinv[k + a] = r[a];
      }
    }
    // trailing block rows k+4 … n4−1, entry (a, c), c ≤ a, to lane (a(a+1)/2 + c) mod G
    const int m = n4 - k - 4;
    int a = 0, c = t;
    while (c > a) {
      c -= a + 1;
      ++a;
    }
    while (a < m) {
      const int i = k + 4 + a, j = k + 4 + c;
      const double* li = H + off(i) + k;
      const double* lj = H + off(j) + k;
      double h = H[off(i) + j];
      h = fma(-li[0], lj[0], h);
      h = fma(-li[1], lj[1], h);
      h = fma(-li[2], lj[2], h);
      h = fma(-li[3], lj[3], h);
      H[off(i) + j] = h;
      c += G;
      while (c > a) {
        c -= a + 1;
        ++a;
      }
    }
  }
  // ---- L y = rhs (y into z), then Lᵀ q̈ = y (into x), by the same panels:
  // every lane solves the 4×4 block, the other rows are dealt to the lanes
  for (int k = 0; k < n4; k += 4) {
    gsync<BLK>(gm);
    double y[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      double v = x[k + a];
#pragma unroll
      for (int e = 0; e < a; ++e) v = fma(-H[off(k + a) + k + e], y[e], v);
      y[a] = v * dinv[k + a];
    }
    for (int i = k + 4 + t; i < n4; i += G) {
      const double* li = H + off(i) + k;
      x[i] = fma(-li[3], y[3], fma(-li[2], y[2], fma(-li[1], y[1], fma(-li[0], y[0], x[i]))));
    }
    if (t == 0) {
#pragma unroll
      for (int a = 0; a < 4; ++a) z[k + a] = y[a];
    }
  }
  for (int k = n4 - 4; k >= 0; k -= 4) {
    gsync<BLK>(gm);
    double w[4];
#pragma unroll
    for (int a = 3; a >= 0; --a) {
      double v = z[k + a];
#pragma unroll
      for (int e = a + 1; e < 4; ++e) v = fma(-H[off(k + e) + k + a], w[e], v);
      w[a] = v * dinv[k + a];
    }
    for (int i = t; i < k; i += G)
      z[i] = fma(-H[off(k + 3) + i], w[3],
                 fma(-H[off(k + 2) + i], w[2], fma(-H[off(k + 1) + i], w[1], fma(-H[off(k) + i], w[0], z[i]))));
    if (t == 0) {
#pragma unroll
      for (int a = 0; a < 4; ++a) x[k + a] = w[a];
    }
  }
  gsync<BLK>(gm);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    qdd[s] = 0.0;
    if (g.body(s) < g.nb && g.dof(s)) {
      qdd[s] = x[g.vo[s]];
      if (!isfinite(qdd[s])) st |= 1;  // GPB_ST_NONFINITE
    }
  }
  gsync<BLK>(gm);  // the next evaluation overwrites x
  return (int)gor<BLK>(gm, (unsigned)st);
}

// All K steps of one instance (pack pk, lane l) by its group: the integrators
// of lane_step (src/integrators.rs:25-39,177-319) on the lane's own bodies.
template <int S, bool BLK>
__device__ void run_instance(const gpb::DeviceBatch& b, const gpb::StepParams& p, int pk, int l, int G, int t,
                             unsigned gm, double* sm) {
  using namespace gpb;
  const PackDesc pd = b.packs[pk];
  const int64_t slot = (int64_t)pk * LANES + l;
  const SlotParams lp = slot_params(b, p, slot);  // the launch's, or a serving job's
  const int64_t K = lp.K;
  if (K <= 0) return;
  const int32_t* li = b.laneI + pd.lane * LANES + l;
  Inst<S> g;
  g.G = G;
  g.t = t;
  g.gm = gm;
  g.nb = li[1 * LANES];
  g.nv = li[3 * LANES];
  g.nc = li[4 * LANES];
  g.nh = li[5 * LANES];
  g.model = li[6 * LANES];
  g.grav = b.gravity;
  g.sm = sm;
  g.nvp = p.group_nvp;
  g.W = b.topoW + pd.topo * 2 * LANES + l;
  g.T = b.topoD + pd.topo * TOPO_D * LANES + l;
  g.CD = b.ctcD + pd.ctc * CTC_D * LANES + l;
  g.HD = b.hsD + pd.hs * HS_D * LANES + l;
  const int64_t inst = li[0];
  double q[S], v[S], tin[S], tau[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const int bb = g.body(s);
    g.type[s] = 0;
    g.qo[s] = g.vo[s] = 0;
    g.w1[s] = 0;
    q[s] = v[s] = tin[s] = tau[s] = 0.0;
    if (bb < g.nb) {
      const uint32_t w0 = __ldg(g.W + (size_t)(2 * bb) * LANES);
      g.w1[s] = __ldg(g.W + (size_t)(2 * bb + 1) * LANES);
      g.type[s] = w0 & 15;
      g.qo[s] = (w0 >> 12) & 1023;
      g.vo[s] = (w0 >> 22) & 1023;
      if (g.dof(s)) {
        q[s] = b.q[(pd.q + g.qo[s]) * LANES + l];
        v[s] = b.v[(pd.v + g.vo[s]) * LANES + l];
        tin[s] = b.tau_in[(pd.v + g.vo[s]) * LANES + l];
      }
    }
  }
  int32_t status = b.status[slot];
  int64_t done = 0;
  const double dt = lp.dt;
  for (int64_t s = 0; s < K; ++s) {
    if (status) break;
    const int64_t sidx = lp.step0 + s;
    // control law before the step (as `control` of the one-lane mapping)
    bool ht;
    if (lp.control == 1) {  // open loop
      const int rs = lp.resample > 0 ? lp.resample : 1;
      if (s == 0 || sidx % rs == 0) {
        const int64_t block = sidx / rs;
#pragma unroll
        for (int k = 0; k < S; ++k)
          if (g.body(k) < g.nb && g.dof(k)) tau[k] = open_loop_tau(lp.seed, inst, block, g.vo[k], lp.sigma);
      }
      ht = true;
    } else if (lp.control == 2) {  // PD on 1-DOF joints
#pragma unroll
      for (int k = 0; k < S; ++k) tau[k] = lp.kp * (tin[k] - q[k]) + lp.kd * -v[k];
      ht = true;
    } else {
#pragma unroll
      for (int k = 0; k < S; ++k) tau[k] = tin[k];
      ht = lp.tau_mode != 0;
    }
    double k1[S];
    int st;
    if (lp.integrator == 0) {  // semi-implicit Euler
      st = eval<S, BLK>(g, q, v, tau, ht, true, k1);
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          v[k] = v[k] + k1[k] * dt;
          q[k] = q[k] + v[k] * dt;
        }
      }
    } else if (lp.integrator == 1) {  // RK2: every stage from (q0, v0), positions with v0
      double qs[S], vs[S];
      st = eval<S, BLK>(g, q, v, tau, ht, true, k1);
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          vs[k] = v[k] + k1[k] * (dt / 2.0);
          qs[k] = q[k] + v[k] * (dt / 2.0);
        }
        st = eval<S, BLK>(g, qs, vs, tau, ht, true, k1);
      }
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          q[k] = q[k] + v[k] * dt;
          v[k] = v[k] + k1[k] * dt;
        }
      }
    } else {  // RK4 as the reference writes it
      double qs[S], vs[S], f[S];
      st = eval<S, BLK>(g, q, v, tau, ht, true, k1);
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          f[k] = k1[k];
          vs[k] = v[k] + k1[k] * (dt / 2.0);
          qs[k] = q[k] + v[k] * (dt / 2.0);
        }
        st = eval<S, BLK>(g, qs, vs, tau, ht, true, k1);
      }
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          f[k] = f[k] + k1[k] * 2.0;
          vs[k] = v[k] + k1[k] * (dt / 2.0);
        }
        st = eval<S, BLK>(g, qs, vs, tau, ht, true, k1);
      }
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          f[k] = f[k] + k1[k] * 2.0;
          vs[k] = v[k] + k1[k] * dt;
          qs[k] = q[k] + v[k] * dt;
        }
        st = eval<S, BLK>(g, qs, vs, tau, ht, true, k1);
      }
      if (!st) {
#pragma unroll
        for (int k = 0; k < S; ++k) {
          f[k] = (f[k] + k1[k]) / 6.0;
          q[k] = q[k] + v[k] * dt;
          v[k] = v[k] + f[k] * dt;
        }
      }
    }
    if (st) {
      status = st;
      break;
    }
    unsigned bad = 0;
#pragma unroll
    for (int k = 0; k < S; ++k)
      if (!isfinite(q[k])) bad = 1;
    status |= (int32_t)gor<BLK>(gm, bad);
    done = s + 1;
    if (p.history && p.record_every > 0 && (s + 1) % p.record_every == 0) {
      double* row = p.history + ((s + 1) / p.record_every - 1) * (b.nq_total + b.nv_total);
#pragma unroll
      for (int k = 0; k < S; ++k) {
        if (g.body(k) >= g.nb || !g.dof(k)) continue;
        row[b.qmap[(pd.q + g.qo[k]) * LANES + l]] = q[k];
        row[b.nq_total + b.vmap[(pd.v + g.vo[k]) * LANES + l]] = v[k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < S; ++k) {
    if (g.body(k) >= g.nb || !g.dof(k)) continue;
    b.q[(pd.q + g.qo[k]) * LANES + l] = q[k];
    b.v[(pd.v + g.vo[k]) * LANES + l] = v[k];
  }
  if (t == 0) {
    b.status[slot] = status;
    b.done[slot] = done;
    if (b.jobs) {
      LaneJob& j = b.jobs[slot];
      j.steps_left -= done;
      j.step_index += done;
      if (status) j.steps_left = 0;  // a failed job ends here (step_index = steps run)
      if (j.steps_left == 0) b.finished[atomicAdd(b.nfinished, 1)] = (int32_t)slot;
    }
  }
}

}  // namespace grp

// Persistent step kernel of the group mapping: each warp takes work items
// (pack, sub-pack) from the device counter; an item is the 32 / G instances
// [j·32/G, (j+1)·32/G) of a pack, one per group.  Dynamic shared memory:
// 32 / G instances × smem_words(nvp) doubles per warp.
template <int S>
__global__ void __launch_bounds__(128) group_kernel(DeviceBatch b, StepParams p) {
  extern __shared__ double gsm[];
  const int G = p.group, P = LANES / G;
  const int lane = threadIdx.x & 31, gi = lane / G, t = lane % G;
  const unsigned gm = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (gi * G));
  double* sm = gsm + (size_t)((threadIdx.x >> 5) * P + gi) * grp::smem_words(p.group_nvp);
  const int64_t nwork = (int64_t)(b.active ? b.nactive : b.npacks) * G;
  while (true) {
    int w = 0;
    if (lane == 0) w = atomicAdd(b.queue, 1);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= nwork) break;
    const int pk = b.active ? b.active[w / G] : w / G;
    const int l = (w % G) * P + gi;
    if (l < b.packs[pk].count) grp::run_instance<S, false>(b, p, pk, l, G, t, gm, sm);
    __syncwarp();
  }
}

// The same step with a 4-warp block per instance (lanes per instance 128, one
// body per thread): each block takes one instance at a time from the device
// counter.  Dynamic shared memory: smem_words(nvp) + BLK_SCAN_WORDS doubles.
__global__ void __launch_bounds__(128) group_block_kernel(DeviceBatch b, StepParams p) {
  extern __shared__ double gsm[];
  __shared__ int s_w;
  const int t = threadIdx.x;
  const int64_t nwork = (int64_t)(b.active ? b.nactive : b.npacks) * LANES;
  while (true) {
    if (t == 0) s_w = atomicAdd(b.queue, 1);
    __syncthreads();
    const int w = s_w;
    __syncthreads();  // every thread has read s_w before thread 0 writes it again
    if (w >= nwork) break;
    const int pk = b.active ? b.active[w / LANES] : w / LANES;
    const int l = w % LANES;
    if (l < b.packs[pk].count) grp::run_instance<1, true>(b, p, pk, l, 32 * grp::BLK_WARPS, t, 0xffffffffu, gsm);
  }
}
