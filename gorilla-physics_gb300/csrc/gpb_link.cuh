// Link-coordinate dynamics (included by gpb_kernels.cu after LaneCtx, the
// column accessors, contact_force and the tiled Cholesky are defined).
//
// Featherstone's recursive Newton–Euler algorithm ("Rigid Body Dynamics
// Algorithms", Table 5.1) and composite-rigid-body algorithm (Table 6.2) in
// link coordinates: every body's velocity, acceleration, force and composite
// inertia live in its own frame, so no quantity grows with the distance from the
// world origin.  The world-frame sweep of lane_dynamics follows the reference's
// formulation (src/dynamics.rs:41-251, src/mechanism.rs:592-696); this one is
// the same mathematics in other coordinates.  It is used twice by the
// MIXED_REFINED mode:
//   SOLVE     in FP32: bias forces, mass matrix, Cholesky and solve (its rounding
//             error is 2-3× smaller than the world-frame sweep's in FP32,
//             because inertias about a far-away origin are dominated by m|p|²);
//   RESIDUAL  in FP64: τ + τ_spring − ID(q, q̇, ẍ) at a trial ẍ, with no mass
//             matrix — about a third of the FP64 work of a world-frame step.
// World poses are tracked only for instances with contacts.
#pragma once

// Rᵀ x for a row-major rotation R.
template <typename R>
__device__ __forceinline__ V3<R> mulT(const M3<R>& Rm, V3<R> x) {
  return {Rm.a[0] * x.x + Rm.a[3] * x.y + Rm.a[6] * x.z, Rm.a[1] * x.x + Rm.a[4] * x.y + Rm.a[7] * x.z,
          Rm.a[2] * x.x + Rm.a[5] * x.y + Rm.a[8] * x.z};
}
template <typename R>
__device__ __forceinline__ M3<R> eye3() {
  M3<R> m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.a[k] = (k % 4 == 0) ? R(1) : R(0);
  return m;
}
// Spatial force in a child frame → the parent frame (child → parent transform (Rr, t)).
template <typename R>
__device__ __forceinline__ SV<R> force_to_parent(const M3<R>& Rr, V3<R> t, const SV<R>& f) {
  const V3<R> fv = mul(Rr, f.v);
  return {mul(Rr, f.w) + cross(t, fv), fv};
}
// S_lᵀ F for DOF l of a joint, in the joint's child frame.
template <typename R>
__device__ __forceinline__ R s_dot(int type, V3<R> ax, int l, const SV<R>& F) {
  if (type == 1) return dot(ax, F.w);
  if (type == 2) return dot(ax, F.v);
  const V3<R> h = l < 3 ? F.w : F.v;  // selects, not an indexed local array
  const int m = l < 3 ? l : l - 3;
  return m == 0 ? h.x : (m == 1 ? h.y : h.z);
}

template <typename R>
__device__ __forceinline__ void load_rel(const LaneCtx<R>& c, int b, M3<R>& Rr, V3<R>& t) {
#pragma unroll
  for (int k = 0; k < 9; ++k) Rr.a[k] = c.r(c.L.I + 12 * b + k);
  t = {c.r(c.L.I + 12 * b + 9), c.r(c.L.I + 12 * b + 10), c.r(c.L.I + 12 * b + 11)};
}

// RESIDUAL = false: q̈ into qdd (returns status bits).  RESIDUAL = true: the
// residual at ẍ = xacc into the scratch rhs vector (in RC), returns the
// cuboid-collision status.
template <typename R, typename RC, bool RESIDUAL>
__device__ __noinline__ int lane_link(const LaneCtx<R>& cin, Col<double> q, Col<double> v,
                                      Col<double> tau, bool have_tau, Col<double> xacc,
                                      Col<double> qdd, Col<double> cf, bool want_cf) {
  const LaneCtx<R> c = cin;  // private copy: stores through scratch pointers cannot alias it
  using V = V3<R>;
  const bool contacts = c.nc > 0 || c.nu > 1;  // world poses (points or cuboid pairs)
  const V zero{R(0), R(0), R(0)};
  V pw_ = zero, pv_ = zero, pal_ = zero, pa_ = zero, ppos = zero;
  M3<R> pR = eye3<R>();
  // ---- outward: velocities, accelerations, Newton–Euler, contacts ------
  for (int b = 0; b < c.nb; ++b) {
    const uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    const int type = w0 & 15, parent = (w0 >> 4) & 255, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    const uint32_t fl = w1 & 255;
    V om, vl, al, ac, posw = zero;
    M3<R> Rw = eye3<R>();
    if (parent == 0) {
      om = zero;
      vl = zero;
      al = zero;
      ac = {R(0), R(0), R(c.grav)};  // inverse gravity (src/dynamics.rs:211-218)
    } else if (parent == b) {
      om = pw_;
      vl = pv_;
      al = pal_;
      ac = pa_;
      posw = ppos;
      Rw = pR;
    } else {
      const int pb = parent - 1;
      om = {c.r(c.L.V + 6 * pb), c.r(c.L.V + 6 * pb + 1), c.r(c.L.V + 6 * pb + 2)};
      vl = {c.r(c.L.V + 6 * pb + 3), c.r(c.L.V + 6 * pb + 4), c.r(c.L.V + 6 * pb + 5)};
      al = {c.r(c.L.A + 6 * pb), c.r(c.L.A + 6 * pb + 1), c.r(c.L.A + 6 * pb + 2)};
      ac = {c.r(c.L.A + 6 * pb + 3), c.r(c.L.A + 6 * pb + 4), c.r(c.L.A + 6 * pb + 5)};
      if (contacts) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Rw.a[k] = c.r(c.L.X + 12 * pb + k);
        posw = {c.r(c.L.X + 12 * pb + 9), c.r(c.L.X + 12 * pb + 10), c.r(c.L.X + 12 * pb + 11)};
      }
    }
    // joint transform child → parent: (Rr, t)
    const int tb = TOPO_D * b;
    V t{c.t(tb + TD_TINIT), c.t(tb + TD_TINIT + 1), c.t(tb + TD_TINIT + 2)};
    const bool rid = (fl & BF_INIT_ROT_IDENTITY) != 0;
    M3<R> Ri = eye3<R>();
    if (!rid) {
#pragma unroll
      for (int k = 0; k < 9; ++k) Ri.a[k] = c.t(tb + TD_RINIT + k);
    }
    V ax = zero;
    if (type == 1 || type == 2) ax = {c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
    M3<R> Rr;
    if (type == 1) {
      R s, co;
      sincos_q<R>(q[qo], &s, &co);
      const R omc = R(1) - co;  // Rot(a, q) = c 1 + s [a]× + (1 − c) a aᵀ
      M3<R> Ro;
      Ro.a[0] = co + ax.x * ax.x * omc;
      Ro.a[1] = ax.x * ax.y * omc - ax.z * s;
      Ro.a[2] = ax.x * ax.z * omc + ax.y * s;
      Ro.a[3] = ax.y * ax.x * omc + ax.z * s;
      Ro.a[4] = co + ax.y * ax.y * omc;
      Ro.a[5] = ax.y * ax.z * omc - ax.x * s;
      Ro.a[6] = ax.z * ax.x * omc - ax.y * s;
      Ro.a[7] = ax.z * ax.y * omc + ax.x * s;
      Ro.a[8] = co + ax.z * ax.z * omc;
      Rr = rid ? Ro : mul(Ri, Ro);
    } else if (type == 2) {
      Rr = Ri;
      t = t + mul(Ri, ax * R(q[qo]));
    } else if (type == 3) {
      const M3<R> Rq = quat_to_mat<R>(R(q[qo]), R(q[qo + 1]), R(q[qo + 2]), R(q[qo + 3]));
      const V tq{R(q[qo + 4]), R(q[qo + 5]), R(q[qo + 6])};
      Rr = rid ? Rq : mul(Ri, Rq);
      t = t + mul(Ri, tq);
    } else {
      Rr = Ri;
    }
    // parent motion in this frame: ω' = Rᵀω, v' = Rᵀ(v + ω × t); same for accelerations
    vl = mulT(Rr, vl + cross(om, t));
    om = mulT(Rr, om);
    ac = mulT(Rr, ac + cross(al, t));
    al = mulT(Rr, al);
    V jw = zero, jv = zero, xw = zero, xv = zero;
    if (type == 1) {
      jw = ax * R(v[vo]);
      if (RESIDUAL) xw = ax * R(xacc[vo]);
    } else if (type == 2) {
      jv = ax * R(v[vo]);
      if (RESIDUAL) xv = ax * R(xacc[vo]);
    } else if (type == 3) {
      jw = {R(v[vo]), R(v[vo + 1]), R(v[vo + 2])};
      jv = {R(v[vo + 3]), R(v[vo + 4]), R(v[vo + 5])};
      if (RESIDUAL) {
        xw = {R(xacc[vo]), R(xacc[vo + 1]), R(xacc[vo + 2])};
        xv = {R(xacc[vo + 3]), R(xacc[vo + 4]), R(xacc[vo + 5])};
      }
    }
    om = om + jw;
    vl = vl + jv;
    // a = X a_parent + S ẍ + v ×m (S q̇)
    al = al + xw + cross(om, jw);
    ac = ac + xv + (cross(om, jv) + cross(vl, jw));
    SI<R> I;
#pragma unroll
    for (int k = 0; k < 6; ++k) I.j[k] = c.t(tb + TD_INERTIA + 4 + k);
    I.c = {c.t(tb + TD_INERTIA + 1), c.t(tb + TD_INERTIA + 2), c.t(tb + TD_INERTIA + 3)};
    I.m = c.t(tb + TD_INERTIA);
    const SV<R> vb{om, vl};
    SV<R> f = imul(I, SV<R>{al, ac}) + crf(vb, imul(I, vb));
    if (contacts) {
      posw = posw + mul(Rw, t);
      Rw = mul(Rw, Rr);
      const int cb = (w1 >> 8) & 255, cn = (w1 >> 16) & 255;
      if (cn) {
        const V omw = mul(Rw, om), vw = mul(Rw, vl);
        for (int k = cb; k < cb + cn; ++k) {
          const int cd = CTC_D * k;
          const V loc{c.CD[(size_t)cd * LANES], c.CD[(size_t)(cd + 1) * LANES], c.CD[(size_t)(cd + 2) * LANES]};
          const R kp = c.CD[(size_t)(cd + 3) * LANES], rad = c.CD[(size_t)(cd + 4) * LANES],
                  damp = c.CD[(size_t)(cd + 5) * LANES];
          const V pw = mul(Rw, loc) + posw;
          V fsum = zero;
          for (int h = 0; h < c.nh; ++h) {
            const int hd = HS_D * h;
            const V hp{c.HD[(size_t)hd * LANES], c.HD[(size_t)(hd + 1) * LANES], c.HD[(size_t)(hd + 2) * LANES]};
            const V hn{c.HD[(size_t)(hd + 3) * LANES], c.HD[(size_t)(hd + 4) * LANES], c.HD[(size_t)(hd + 5) * LANES]};
            const R alh = c.HD[(size_t)(hd + 6) * LANES], mu = c.HD[(size_t)(hd + 7) * LANES];
            const R dist = dot(pw - hp, hn);
            V app = pw;
            R pen;
            if (rad > R(0)) {
              if (!(dist - rad <= R(1e-8))) continue;
              pen = rad - dist;
              app = pw - hn * rad;
            } else {
              if (!(dist <= R(1e-8))) continue;  // HalfSpace::has_inside (margin 1e-8)
              pen = -dist;
            }
            const V vel = vw + cross(omw, app - posw);
            const V fc = contact_force<R>(c.model, pen, hn, vel, kp, damp, alh, mu);
            const V fb = mulT(Rw, fc), rb = mulT(Rw, app - posw);
            f.w = f.w - cross(rb, fb);
            f.v = f.v - fb;
            fsum = fsum + fc;
          }
          if (want_cf) {
            const int orig = (c.CI[(size_t)k * LANES] >> 8) & 255;
            cf[3 * orig] = double(fsum.x);
            cf[3 * orig + 1] = double(fsum.y);
            cf[3 * orig + 2] = double(fsum.z);
          }
        }
      }
      const int uslot = (int)((w1 >> W1_CUBOID_SHIFT) & 15u);
      if (uslot && c.nu > 1) {  // cuboid record: world pose, world twist about the origin
        M3<double> Rd;
#pragma unroll
        for (int k = 0; k < 9; ++k) Rd.a[k] = double(Rw.a[k]);
        const V3<double> pd{double(posw.x), double(posw.y), double(posw.z)};
        const V3<double> omw = mul(Rd, V3<double>{double(om.x), double(om.y), double(om.z)});
        const V3<double> vlw = mul(Rd, V3<double>{double(vl.x), double(vl.y), double(vl.z)});
        store_cuboid(c, uslot - 1, b, Rd, pd, omw, vlw - cross(omw, pd));
      }
    }
    store_sv(c, c.L.F + 6 * b, f);
#pragma unroll
    for (int k = 0; k < 9; ++k) c.r(c.L.I + 12 * b + k) = Rr.a[k];
    c.r(c.L.I + 12 * b + 9) = t.x;
    c.r(c.L.I + 12 * b + 10) = t.y;
    c.r(c.L.I + 12 * b + 11) = t.z;
    if (fl & BF_BRANCH) {
      store_sv(c, c.L.V + 6 * b, SV<R>{om, vl});
      store_sv(c, c.L.A + 6 * b, SV<R>{al, ac});
      if (contacts) {
#pragma unroll
        for (int k = 0; k < 9; ++k) c.r(c.L.X + 12 * b + k) = Rw.a[k];
        c.r(c.L.X + 12 * b + 9) = posw.x;
        c.r(c.L.X + 12 * b + 10) = posw.y;
        c.r(c.L.X + 12 * b + 11) = posw.z;
      }
      if (!RESIDUAL) {  // composite inertia accumulator of a branch body
#pragma unroll
        for (int k = 0; k < 10; ++k) c.r(c.L.C + 10 * b + k) = R(0);
      }
    }
    pw_ = om;
    pv_ = vl;
    pal_ = al;
    pa_ = ac;
    ppos = posw;
    pR = Rw;
  }
  // ---- cuboid pairs: f −= W (body frame) ----------------------------
  int st = 0;
  if (c.nu > 1) {
    st = lane_cuboid_pairs(c);
    for (int b = 0; b < c.nb; ++b) {
      const int uslot = (int)((c.w(2 * b + 1) >> W1_CUBOID_SHIFT) & 15u);
      if (!uslot) continue;
      const SV<double> W = cuboid_wrench_body(c, uslot - 1);
      const SV<R> Wr{{R(W.w.x), R(W.w.y), R(W.w.z)}, {R(W.v.x), R(W.v.y), R(W.v.z)}};
      store_sv(c, c.L.F + 6 * b, load_sv(c, c.L.F + 6 * b) - Wr);
    }
  }
  // ---- inward: joint forces, composite inertias, mass-matrix fill ------
  const int nv = c.nv;
  if (!RESIDUAL && !c.chain) {  // clear the tiled triangle (fill-in of the previous factor)
    const int nT = (nv + 3) >> 2;
    const int nm = (nT * (nT + 1) >> 1) * 16;
    for (int e = 0; e < nm; ++e) c.template x<RC>(c.L.M + e) = RC(0);
  }
  SV<R> carry{zero, zero};
  SI<R> cI;
  int ctarget = -1;
  for (int b = c.nb - 1; b >= 0; --b) {
    const uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    const int type = w0 & 15, parent = (w0 >> 4) & 255, qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    const int tb = TOPO_D * b;
    SV<R> f = load_sv(c, c.L.F + 6 * b);
    SI<R> Ic;
    if (!RESIDUAL) {
#pragma unroll
      for (int k = 0; k < 6; ++k) Ic.j[k] = c.t(tb + TD_INERTIA + 4 + k);
      Ic.c = {c.t(tb + TD_INERTIA + 1), c.t(tb + TD_INERTIA + 2), c.t(tb + TD_INERTIA + 3)};
      Ic.m = c.t(tb + TD_INERTIA);
      if ((w1 & 255) & BF_BRANCH) iadd(Ic, load_si(c, c.L.C + 10 * b));
    }
    if (ctarget == b) {
      f = f + carry;
      if (!RESIDUAL) iadd(Ic, cI);
    }
    const int nvb = type == 3 ? 6 : (type == 0 ? 0 : 1);
    V ax = zero;
    if (type == 1 || type == 2) ax = {c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
    for (int k = 0; k < nvb; ++k) {
      double r = have_tau ? tau[vo + k] : 0.0;
      if (type == 2 && (w1 & BF_SPRING) && c.springs) {  // src/dynamics.rs:298-315
        r += -double(c.t(tb + TD_SPRING)) * (q[qo] - double(c.t(tb + TD_SPRING + 1)));
      }
      // free_velocity: revolute armature (src/hybrid/articulated/mod.rs:244-247)
      const double arm = type == 1 && c.armature ? double(c.t(tb + TD_ARMATURE)) : 0.0;
      if (RESIDUAL) {  // difference of nearly equal terms: form it in FP64
        c.template x<RC>(c.L.rhs + vo + k) = RC(r - double(s_dot<R>(type, ax, k, f)) - arm * xacc[vo + k]);
        continue;
      }
      c.template x<RC>(c.L.rhs + vo + k) = RC(RC(r) - RC(s_dot<R>(type, ax, k, f)));
      // CRBA: F = Ic S_k, then up the tree H(row, ·) = S_lᵀ F
      const int row = vo + k;
      SV<R> Sk{zero, zero};
      if (type == 1) Sk.w = ax;
      else if (type == 2) Sk.v = ax;
      else {
        const R e[3] = {R(k == 0 || k == 3), R(k == 1 || k == 4), R(k == 2 || k == 5)};
        if (k < 3) Sk.w = {e[0], e[1], e[2]};
        else Sk.v = {e[0], e[1], e[2]};
      }
      SV<R> F = imul(Ic, Sk);
      for (int l = 0; l <= k; ++l) {
        const R h = s_dot<R>(type, ax, l, F);
        c.template x<RC>(c.L.M + tix(row, vo + l)) = RC(l == k ? h + R(arm) : h);
      }
      int ch = b, a = parent;
      while (a != 0) {
        M3<R> Rr;
        V tt;
        load_rel(c, ch, Rr, tt);
        F = force_to_parent(Rr, tt, F);
        const uint32_t wa = c.w(2 * (a - 1));
        const int ta = wa & 15, voa = (wa >> 22) & 1023;
        const int nva = ta == 3 ? 6 : (ta == 0 ? 0 : 1);
        V axa = zero;
        if (ta == 1 || ta == 2) {
          const int tba = TOPO_D * (a - 1);
          axa = {c.t(tba + TD_AXIS), c.t(tba + TD_AXIS + 1), c.t(tba + TD_AXIS + 2)};
        }
        for (int l = 0; l < nva; ++l)
          c.template x<RC>(c.L.M + tix(row, voa + l)) = RC(s_dot<R>(ta, axa, l, F));
        ch = a - 1;
        a = (wa >> 4) & 255;
      }
    }
    if (parent != 0) {
      M3<R> Rr;
      V tt;
      load_rel(c, b, Rr, tt);
      const SV<R> fp = force_to_parent(Rr, tt, f);
      SI<R> Ip;
      if (!RESIDUAL) Ip = to_world(Ic, Rr, tt, false);  // composite inertia in the parent frame
      const int pb = parent - 1;
      if (pb == b - 1) {
        carry = fp;
        if (!RESIDUAL) cI = Ip;
        ctarget = pb;
      } else {
        store_sv(c, c.L.F + 6 * pb, load_sv(c, c.L.F + 6 * pb) + fp);
        if (!RESIDUAL) {
          SI<R> acc = load_si(c, c.L.C + 10 * pb);
          iadd(acc, Ip);
          store_si(c, c.L.C + 10 * pb, acc);
        }
        ctarget = -1;
      }
    } else {
      ctarget = -1;
    }
  }
  if (RESIDUAL) return st;
  return st | lane_cholesky_solve<R, RC>(cin, qdd);
}
