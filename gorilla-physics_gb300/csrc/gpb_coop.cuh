// Block-cooperative step for packs of large mechanisms (included by
// gpb_kernels.cu after the per-lane evaluators, make_ctx and control).
//
// A warp issues to one of the SM's four schedulers, and each scheduler has its
// own FP64 unit (0.5 DFMA lanes per clock), so one warp stepping a pack of
// 48-DOF chains is bounded by a quarter of the SM's FP64 rate: those packs set
// the critical path of a batch.  Here the four warps of a 128-thread block
// share one pack, lane l of every warp working on instance l:
//   warp 0      the outward / inward sweeps (serial along the tree), leaving the
//               composite inertias and the right-hand side in scratch; then the
//               triangular solves and the integrator;
//   all warps   the CRBA fill and the Cholesky factorisation, split by 4-row
//               tile rows (tile row I belongs to warp I mod 4), one barrier
//               per tile column.
// The sweeps, the fill (lane_fill) and every tile (chol_diag, chol_offdiag)
// are the same compiled functions the one-warp path calls, so the results are
// bit-identical to it.  The barrier sequence depends only on pack-wide values (K,
// the integrator's stage count, the pack's tile count), never on lane data.

#pragma once

constexpr int COOP_WARPS = 4;

// Named barrier of the block's 128 threads (non-aligned form: warp 0 and the
// helper warps reach it from different code).
__device__ __forceinline__ void coop_bar() { asm volatile("barrier.sync 1, 128;" ::: "memory"); }

// This warp's share of the factorisation: the tile rows it owns.  The owner
// of row J factors tile (J, J) right after its tile (J, J−1) (both its own
// work), so each column needs one barrier: after it, every warp computes its
// tiles (I, J), I > J.  nTp (the pack's largest tile count) fixes the barrier
// count; lanes with fewer tiles skip the work.
template <typename R, typename RC>
__device__ __noinline__ int coop_cholesky(const LaneCtx<R>& cin, int w, bool alive, int nTp) {
  const LaneCtx<R> c = cin;
  const int nT = (c.nv + 3) >> 2;
  int st = 0;
  if (alive && w == 0 && nT > 0) st |= chol_diag<R, RC>(cin, 0);
  for (int J = 0; J < nTp; ++J) {
    coop_bar();
    if (!alive || J >= nT) continue;
    for (int I = J + 1; I < nT; ++I) {
      if ((I & (COOP_WARPS - 1)) != w) continue;
      chol_offdiag<R, RC>(cin, I, J);
      if (I == J + 1) st |= chol_diag<R, RC>(cin, I);  // row J+1 is complete up to its diagonal
    }
  }
  return st;
}

// Per-block state shared by the four warps of a cooperative pack.
struct CoopShared {
  int32_t st[COOP_WARPS][LANES];
  int32_t alive[LANES];
};

// Evaluator of warp 0 (q, v, τ → q̈) and the matching helper-warp routine.
template <typename R, typename RC>
struct EvalCoop {
  LaneCtx<R> c;
  CoopShared* sh;
  int nTp;
  __device__ int run(Col<double> q, Col<double> v, Col<double> t, bool ht, Col<double> x, bool alive) const {
    Col<double> none{nullptr};
    int st = 0;
    if (alive) st |= lane_sweeps<R, RC>(c, q, v, t, ht, none, false);
    sh->alive[c.lane] = alive ? 1 : 0;
    coop_bar();  // A: sweeps done, composite inertias and rhs in scratch
    if (alive) {
      lane_fill<R, RC>(c, 0, COOP_WARPS);
      chol_pad<R, RC>(c, 0, COOP_WARPS);
    }
    coop_bar();  // B: H filled
    sh->st[0][c.lane] = coop_cholesky<R, RC>(c, 0, alive, nTp);
    coop_bar();  // C: factor complete
#pragma unroll
    for (int k = 0; k < COOP_WARPS; ++k) st |= sh->st[k][c.lane];
    if (alive) {  // as lane_cholesky_solve: the solve runs even after a failed pivot
      lane_solve<R, RC>(c);
      for (int i = 0; i < c.nv; ++i) {
        const double y = double(c.template x<RC>(c.L.rhs + i));
        x[i] = y;
        if (!isfinite(y)) st |= 1;  // GPB_ST_NONFINITE
      }
    }
    return st;
  }
};

template <typename R, typename RC>
__device__ void coop_helper_eval(const LaneCtx<R>& c, CoopShared* sh, int w, int nTp) {
  coop_bar();  // A
  const bool alive = sh->alive[c.lane] != 0;
  if (alive) {
    lane_fill<R, RC>(c, w, COOP_WARPS);
    chol_pad<R, RC>(c, w, COOP_WARPS);
  }
  coop_bar();  // B
  sh->st[w][c.lane] = coop_cholesky<R, RC>(c, w, alive, nTp);
  coop_bar();  // C
}

// lane_step for warp 0 of a cooperative pack: the same integrator arithmetic,
// but every stage's evaluation runs (and meets its barriers) even after a
// lane failed; a failed lane's q and v are left untouched.
template <typename E>
__device__ int coop_lane_step(const E& ev, Col<double> q, Col<double> v, Col<double> tau, bool have_tau,
                              double dt, int integrator, bool alive) {
  const auto& c = ev.c;
  const int nv = c.nv;
  Col<double> f{&c.d(c.L.facc)};
  Col<double> qs{&c.d(c.L.qs)}, vs{&c.d(c.L.vs)};
  Col<double> tmp{&c.d(c.L.v0)};
  int st = 0;
  if (integrator == 0) {  // semi-implicit Euler (src/integrators.rs:25-39,276-319)
    st |= ev.run(q, v, tau, have_tau, tmp, alive);
    if (!alive || st) return st;
    for (int i = 0; i < nv; ++i) v[i] = v[i] + tmp[i] * dt;
    advance_q(c, q, v, dt, q);
    return st;
  }
  Col<double> q0 = q;
  Col<double> k1{&c.d(c.L.v0)};
  st |= ev.run(q, v, tau, have_tau, k1, alive);
  bool ok = alive && !st;
  if (integrator == 1) {  // RK2
    if (ok) {
      for (int i = 0; i < nv; ++i) vs[i] = v[i] + k1[i] * (dt / 2.0);
      advance_q(c, q0, v, dt / 2.0, qs);
    }
    st |= ev.run(qs, vs, tau, have_tau, k1, ok);
    ok = ok && !st;
    if (!ok) return st;
    advance_q(c, q0, v, dt, q);
    for (int i = 0; i < nv; ++i) v[i] = v[i] + k1[i] * dt;
    return st;
  }
  // RK4
  if (ok) {
    for (int i = 0; i < nv; ++i) {
      f[i] = k1[i];
      vs[i] = v[i] + k1[i] * (dt / 2.0);
    }
    advance_q(c, q0, v, dt / 2.0, qs);
  }
  st |= ev.run(qs, vs, tau, have_tau, k1, ok);
  ok = ok && !st;
  if (ok) {
    for (int i = 0; i < nv; ++i) {
      f[i] = f[i] + k1[i] * 2.0;
      vs[i] = v[i] + k1[i] * (dt / 2.0);
    }
  }
  st |= ev.run(qs, vs, tau, have_tau, k1, ok);
  ok = ok && !st;
  if (ok) {
    for (int i = 0; i < nv; ++i) {
      f[i] = f[i] + k1[i] * 2.0;
      vs[i] = v[i] + k1[i] * dt;
    }
    advance_q(c, q0, v, dt, qs);
  }
  st |= ev.run(qs, vs, tau, have_tau, k1, ok);
  ok = ok && !st;
  if (!ok) return st;
  for (int i = 0; i < nv; ++i) f[i] = (f[i] + k1[i]) / 6.0;
  advance_q(c, q0, v, dt, q);
  for (int i = 0; i < nv; ++i) v[i] = v[i] + f[i] * dt;
  return st;
}

// All K steps of pack pk by the whole block (PREC 0: FP64; PREC 1: FP32 sweeps
// with the FP64 factorisation, as EvalMixed uses for n > 12).
template <int PREC>
__device__ void coop_pack(const DeviceBatch& b, const StepParams& p, int pk, CoopShared* sh) {
  using R = typename std::conditional<PREC == 0, double, float>::type;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const PackDesc pd = b.packs[pk];
  const bool in_pack = lane < pd.count;
  const int nTp = (pd.nv + 3) >> 2;
  const int nevals = p.integrator == 0 ? 1 : (p.integrator == 1 ? 2 : 4);
  EvalCoop<R, double> ev{make_ctx<R>(b, pd, lane), sh, nTp};
  const LaneCtx<R>& c = ev.c;
  if (w != 0) {
    for (int64_t s = 0; s < p.K; ++s)
      for (int e = 0; e < nevals; ++e) coop_helper_eval<R, double>(c, sh, w, nTp);
    return;
  }
  int32_t* status = b.status + (int64_t)pk * LANES + lane;
  const int64_t inst = in_pack ? b.laneI[pd.lane * LANES + lane] : 0;
  Col<double> q = col_at(b.q, pd.q, lane), v = col_at(b.v, pd.v, lane);
  Col<double> tin = col_at(b.tau_in, pd.v, lane);
  Col<double> tau{&c.d(c.L.tau)};
  int64_t done = 0;
  bool alive = in_pack && *status == 0;
  const SlotParams sp = slot_params(b, p, 0);  // batches only (no serving jobs)
  for (int64_t s = 0; s < p.K; ++s) {
    const int64_t sidx = p.step0 + s;
    bool ht = false;
    if (alive) ht = control(c, b, sp, inst, sidx, s == 0, q, v, tin, tau);
    Col<double> tsrc = p.control == 0 ? tin : tau;
    const int st = coop_lane_step(ev, q, v, tsrc, ht, p.dt, p.integrator, alive);
    if (!alive) continue;
    if (st) {
      *status = st;
      alive = false;
      continue;
    }
    for (int i = 0; i < c.nq; ++i)
      if (!isfinite(q[i])) *status |= 1;
    done = s + 1;
    if (*status) alive = false;
    if (p.history && p.record_every > 0 && (s + 1) % p.record_every == 0) {
      double* row = p.history + ((s + 1) / p.record_every - 1) * (b.nq_total + b.nv_total);
      const int64_t* qm = b.qmap + pd.q * LANES + lane;
      const int64_t* vm = b.vmap + pd.v * LANES + lane;
      for (int i = 0; i < c.nq; ++i) row[qm[(size_t)i * LANES]] = q[i];
      for (int i = 0; i < c.nv; ++i) row[b.nq_total + vm[(size_t)i * LANES]] = v[i];
    }
  }
  if (in_pack) b.done[(int64_t)pk * LANES + lane] = done;
}
