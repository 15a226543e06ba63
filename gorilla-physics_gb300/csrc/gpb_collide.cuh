// Cuboid–cuboid collision detection for one lane: GJK for the intersection
// test, then the expanding polytope algorithm (EPA) for the penetration and a
// contact point on each cuboid — gorilla-physics' CollisionDetector
// (src/collision/mod.rs:48-87; gjk.rs:14-125; epa.rs:69-254;
// polytope.rs:26-68; cuboid.rs:18-40,86-96).
//
// The query is a discrete algorithm: which support corner wins, which face is
// closest, when the expansion stops.  To make those decisions exactly the
// reference's, every floating-point operation is an IEEE-rounded intrinsic
// (no contraction into FMA) in the reference's order — dot products and
// matrix-vector products summed left to right, cross products component by
// component as a_y b_z − a_z b_y, …, norms as sqrt(x² + y² + z²) — and EPA's
// closest-face queue is a binary heap with the reference's sift rules
// (push: sift up; pop: move the last element to the root, sift it down along
// the larger children to the bottom, then up), because the face-visibility
// scan walks the heap in storage order, and that order fixes the numbering
// of new faces and so how later ties between equal distances break.
//
// Values the reference recomputes (a face's |w| and w·w, tests of |x| == 0)
// are computed once here, by the same operations, or tested as x·x == 0
// (equivalent under IEEE rounding, NaN included): the results are unchanged.
//
// Storage is fixed per lane (local memory): MAXV polytope vertices, MAXT
// faces ever created, MAXE horizon edges, GJK_MAX support evaluations.  Over
// 4·10⁵ random pairs (shallow face contacts and deep random overlaps) the
// largest counts seen were 23 vertices, 85 faces, 12 edges and 16 GJK
// iterations; a query that would exceed a bound reports CG_OVERFLOW (the
// instance stops with GPB_ST_COLLISION) instead of writing past it.
#pragma once

namespace gcol {

constexpr int MAXV = 48, MAXT = 160, MAXE = 32, GJK_MAX = 64;
enum { CG_HIT = 1, CG_NONE = 0, CG_PANIC = -1, CG_OVERFLOW = -2 };

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ double mu_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ad_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dv_(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ D3 add(D3 a, D3 b) { return {ad_(a.x, b.x), ad_(a.y, b.y), ad_(a.z, b.z)}; }
__device__ __forceinline__ D3 sub(D3 a, D3 b) { return {sb_(a.x, b.x), sb_(a.y, b.y), sb_(a.z, b.z)}; }
__device__ __forceinline__ D3 neg(D3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ D3 scale(double s, D3 a) { return {mu_(s, a.x), mu_(s, a.y), mu_(s, a.z)}; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return ad_(ad_(mu_(a.x, b.x), mu_(a.y, b.y)), mu_(a.z, b.z)); }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return {sb_(mu_(a.y, b.z), mu_(a.z, b.y)), sb_(mu_(a.z, b.x), mu_(a.x, b.z)), sb_(mu_(a.x, b.y), mu_(a.y, b.x))};
}
__device__ __forceinline__ double norm2(D3 a) { return dot(a, a); }
__device__ __forceinline__ double norm(D3 a) { return __dsqrt_rn(norm2(a)); }

// A cuboid's pose: row-major rotation, centre, sizes (w, d, h).
struct BoxPose {
  double R[9];
  double t[3];
  double dims[3];
};

// Rotation of a unit quaternion (x, y, z, w) (UnitQuaternion::to_rotation_matrix).
__device__ __forceinline__ void quat_to_matrix(double i, double j, double k, double w, double* R) {
  const double ww = mu_(w, w), ii = mu_(i, i), jj = mu_(j, j), kk = mu_(k, k);
  const double ij = mu_(mu_(i, j), 2.0), wk = mu_(mu_(w, k), 2.0), wj = mu_(mu_(w, j), 2.0);
  const double ik = mu_(mu_(i, k), 2.0), jk = mu_(mu_(j, k), 2.0), wi = mu_(mu_(w, i), 2.0);
  R[0] = sb_(sb_(ad_(ww, ii), jj), kk);
  R[1] = sb_(ij, wk);
  R[2] = ad_(wj, ik);
  R[3] = ad_(wk, ij);
  R[4] = sb_(ad_(sb_(ww, ii), jj), kk);
  R[5] = sb_(jk, wi);
  R[6] = sb_(ik, wj);
  R[7] = ad_(wi, jk);
  R[8] = ad_(sb_(sb_(ww, ii), jj), kk);
}

// Corner points R c + t, corner k = (±w/2, ±d/2, ±h/2) with the signs of bits
// 0, 1, 2 (cuboid.rs:22-31).
__device__ __forceinline__ void box_points(const BoxPose& b, D3 t, double* px, double* py, double* pz) {
  const double hw = dv_(b.dims[0], 2.0), hd = dv_(b.dims[1], 2.0), hh = dv_(b.dims[2], 2.0);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const double cx = (k & 1) ? -hw : hw, cy = (k & 2) ? -hd : hd, cz = (k & 4) ? -hh : hh;
    const D3 r{ad_(ad_(mu_(b.R[0], cx), mu_(b.R[1], cy)), mu_(b.R[2], cz)),
               ad_(ad_(mu_(b.R[3], cx), mu_(b.R[4], cy)), mu_(b.R[5], cz)),
               ad_(ad_(mu_(b.R[6], cx), mu_(b.R[7], cy)), mu_(b.R[8], cz))};
    px[k] = ad_(r.x, t.x);
    py[k] = ad_(r.y, t.y);
    pz[k] = ad_(r.z, t.z);
  }
}

// compute_support: the first corner of largest d·p.
__device__ __forceinline__ int support(const double* px, const double* py, const double* pz, D3 d) {
  int best = 0;
  double bv = dot(d, D3{px[0], py[0], pz[0]});
#pragma unroll
  for (int k = 1; k < 8; ++k) {
    const double v = dot(d, D3{px[k], py[k], pz[k]});
    if (v > bv) {
      bv = v;
      best = k;
    }
  }
  return best;
}

struct Shapes {  // the two cuboids' corners in the query frame
  double ax[8], ay[8], az[8], bx[8], by[8], bz[8];
  __device__ D3 a(int k) const { return {ax[k], ay[k], az[k]}; }
  __device__ D3 b(int k) const { return {bx[k], by[k], bz[k]}; }
};

struct PV {  // a vertex of the Minkowski difference A − B and its corners
  D3 v;
  int ia, ib;
};
__device__ __forceinline__ PV support_fn(const Shapes& S, D3 d) {
  const int ia = support(S.ax, S.ay, S.az, d), ib = support(S.bx, S.by, S.bz, neg(d));
  return {sub(S.a(ia), S.b(ib)), ia, ib};
}

// GJK: CG_HIT with the enclosing tetrahedron in s[0..3], CG_NONE, or an error.
__device__ __forceinline__ int gjk(const Shapes& S, D3 cA, D3 cB, PV* s) {
  const D3 origin{0.0, 0.0, 0.0};
  D3 dir = (cA.x == cB.x && cA.y == cB.y && cA.z == cB.z) ? D3{1.0, 0.0, 0.0} : sub(cA, cB);
  int n = 0;
  for (int it = 0; it < GJK_MAX; ++it) {
    const PV nv = support_fn(S, dir);
    if (nv.v.x == 0.0 && nv.v.y == 0.0 && nv.v.z == 0.0) return CG_NONE;  // touching
    if (dot(dir, nv.v) <= 0.0) return CG_NONE;  // not past the origin
    s[n++] = nv;
    if (n == 1) {
      dir = sub(origin, nv.v);
    } else if (n == 2) {
      const D3 v1 = s[0].v, v2 = s[1].v;
      const D3 v1v2 = sub(v2, v1);
      dir = cross(cross(v1, v2), v1v2);
      if (norm2(dir) == 0.0) {  // origin on the edge (|x| == 0 ⟺ x·x == 0, NaN in both)
        const D3 cand = cross(v1v2, D3{1.0, 0.0, 0.0});
        dir = norm2(cand) > 0.0 ? cand : cross(v1v2, D3{0.0, 1.0, 0.0});
      }
    } else if (n == 3) {
      const D3 v1 = s[0].v, v2 = s[1].v, v3 = s[2].v;
      dir = cross(sub(v3, v1), sub(v2, v1));
      if (dot(dir, sub(origin, v1)) < 0.0) {
        dir = neg(dir);
        const PV t = s[1];
        s[1] = s[2];
        s[2] = t;
      }
      if (norm2(dir) == 0.0) return CG_PANIC;  // colinear simplex
    } else {
      const PV p1 = s[0], p2 = s[1], p3 = s[2], p4 = s[3];
      const D3 v1 = p1.v, v2 = p2.v, v3 = p3.v, v4 = p4.v;
      const D3 v1v3 = sub(v3, v1), v1v2 = sub(v2, v1), v1v4 = sub(v4, v1);
      const D3 n143 = cross(v1v3, v1v4);
      if (dot(n143, v1v2) > 0.0) return CG_PANIC;
      if (dot(n143, v1) < 0.0) {
        dir = n143;
        s[1] = p4;  // (v1, v4, v3)
        n = 3;
        continue;
      }
      const D3 v2v3 = sub(v3, v2), v2v4 = sub(v4, v2), v2v1 = neg(v1v2);
      const D3 n234 = cross(v2v4, v2v3);
      if (dot(n234, v2v1) > 0.0) return CG_PANIC;
      if (dot(n234, v2) < 0.0) {
        dir = n234;
        s[0] = p2;  // (v2, v3, v4)
        s[1] = p3;
        s[2] = p4;
        n = 3;
        continue;
      }
      const D3 n124 = cross(v1v4, v1v2);
      if (dot(n124, v1v3) > 0.0) return CG_PANIC;
      if (dot(n124, v1) < 0.0) {
        dir = n124;
        s[2] = p4;  // (v1, v2, v4)
        n = 3;
        continue;
      }
      return CG_HIT;
    }
  }
  return CG_OVERFLOW;
}

// Barycentric coordinates of the origin's projection on the plane of
// (v1, v2, v3) and the plane normal (v2 − v1) × (v3 − v1) (area method).
__device__ __forceinline__ void lambda_area(D3 v1, D3 v2, D3 v3, double* l, D3* nrm) {
  const D3 v1v2 = sub(v2, v1), v1v3 = sub(v3, v1);
  const D3 n = cross(v1v2, v1v3);
  const double inv = dv_(1.0, norm2(n));
  const double b3 = mu_(dot(cross(v1, v1v2), n), inv);
  const double b2 = mu_(dot(cross(v1v3, v1), n), inv);
  l[0] = sb_(1.0, ad_(b2, b3));
  l[1] = b2;
  l[2] = b3;
  *nrm = n;
}
__device__ __forceinline__ D3 closest_area(D3 v1, D3 v2, D3 v3) {
  double l[3];
  D3 n;
  lambda_area(v1, v2, v3, l, &n);
  const D3 w = add(add(scale(l[0], v1), scale(l[1], v2)), scale(l[2], v3));
  const double s = dot(w, n), nn = norm2(n);
  return {dv_(mu_(s, n.x), nn), dv_(mu_(s, n.y), nn), dv_(mu_(s, n.z), nn)};
}

// EPA working set of one lane.
struct Poly {
  double vx[MAXV], vy[MAXV], vz[MAXV];
  uint8_t via[MAXV], vib[MAXV];
  double wx[MAXT], wy[MAXT], wz[MAXT];
  double dist[MAXT], wn2[MAXT];  // |w| (the heap key) and w·w, computed once per face
  uint8_t t0[MAXT], t1[MAXT], t2[MAXT], obs[MAXT];
  uint16_t heap[MAXT];
  uint8_t e0[MAXE], e1[MAXE];
  int nv, nt, nh, ne;
  __device__ D3 v(int i) const { return {vx[i], vy[i], vz[i]}; }
  __device__ D3 w(int i) const { return {wx[i], wy[i], wz[i]}; }
  // Heap order: Reverse((distance, face index)) — the smallest distance on
  // top, ties to the lowest index, NaN above every number.
  __device__ int cmp(int a, int b) const {
    const double x = dist[a], y = dist[b];
    const bool nx = isnan(x), ny = isnan(y);
    int c;
    if (nx || ny) c = nx == ny ? 0 : (nx ? 1 : -1);
    else c = x < y ? -1 : (x > y ? 1 : 0);
    return c ? c : (a < b ? -1 : (a > b ? 1 : 0));
  }
  __device__ bool le(int a, int b) const { return cmp(b, a) <= 0; }  // Reverse(a) <= Reverse(b)
  __device__ void sift_up(int start, int pos) {
    const int e = heap[pos];
    while (pos > start) {
      const int parent = (pos - 1) / 2;
      if (le(e, heap[parent])) break;
      heap[pos] = heap[parent];
      pos = parent;
    }
    heap[pos] = (uint16_t)e;
  }
  __device__ void push(int face) {
    heap[nh] = (uint16_t)face;
    ++nh;
    sift_up(0, nh - 1);
  }
  __device__ int pop() {  // nh > 0
    int item = heap[--nh];
    if (nh > 0) {
      const int top = heap[0];
      heap[0] = (uint16_t)item;
      item = top;
      const int end = nh, e = heap[0];
      int pos = 0, child = 1;
      while (child + 1 < end) {
        if (le(heap[child], heap[child + 1])) child += 1;
        heap[pos] = heap[child];
        pos = child;
        child = 2 * pos + 1;
      }
      if (child == end - 1) {
        heap[pos] = heap[child];
        pos = child;
      }
      heap[pos] = (uint16_t)e;
      sift_up(0, pos);
    }
    return item;
  }
  // addEdgeIfNotExisting (src/collision/mod.rs:21-35): drop the reverse edge
  // if present (keeping the order of the rest), else append.
  __device__ bool edge(int a, int b) {
    for (int k = 0; k < ne; ++k)
      if (e0[k] == b && e1[k] == a) {
        for (int m = k + 1; m < ne; ++m) {
          e0[m - 1] = e0[m];
          e1[m - 1] = e1[m];
        }
        --ne;
        return true;
      }
    if (ne >= MAXE) return false;
    e0[ne] = (uint8_t)a;
    e1[ne] = (uint8_t)b;
    ++ne;
    return true;
  }
  __device__ bool add_face(int a, int b, int c) {
    if (nt >= MAXT) return false;
    t0[nt] = (uint8_t)a;
    t1[nt] = (uint8_t)b;
    t2[nt] = (uint8_t)c;
    obs[nt] = 0;
    const D3 w = closest_area(v(a), v(b), v(c));
    wx[nt] = w.x;
    wy[nt] = w.y;
    wz[nt] = w.z;
    wn2[nt] = norm2(w);
    dist[nt] = __dsqrt_rn(wn2[nt]);  // = norm(w)
    push(nt);
    ++nt;
    return true;
  }
};

__device__ __forceinline__ int epa(const Shapes& S, const PV* s, Poly& P, D3* cpA, D3* cpB) {
  P.nv = 4;
  P.nt = 0;
  P.nh = 0;
  for (int i = 0; i < 4; ++i) {
    P.vx[i] = s[i].v.x;
    P.vy[i] = s[i].v.y;
    P.vz[i] = s[i].v.z;
    P.via[i] = (uint8_t)s[i].ia;
    P.vib[i] = (uint8_t)s[i].ib;
  }
  P.add_face(0, 1, 2);  // Polytope::from_simplex
  P.add_face(0, 3, 1);
  P.add_face(0, 2, 3);
  P.add_face(1, 3, 2);
  for (int guard = 0; guard < 4 * MAXT; ++guard) {
    if (P.nh == 0) return CG_PANIC;  // heap.pop().unwrap() on an empty heap
    const int index = P.pop();
    if (P.obs[index]) continue;
    P.obs[index] = 1;
    const int i1 = P.t0[index], i2 = P.t1[index], i3 = P.t2[index];
    const D3 w = P.w(index);
    const D3 v1 = P.v(i1), v2 = P.v(i2), v3 = P.v(i3);
    const D3 normal = cross(sub(v2, v1), sub(v3, v1));
    if (norm2(normal) == 0.0) return CG_PANIC;
    const D3 direction = normal;
    const PV v = support_fn(S, direction);
    const double v_dot_w = dot(v.v, w);
    const double wn2 = P.wn2[index], wn = P.dist[index];
    if (v_dot_w < sb_(wn2, 1e-8)) return CG_PANIC;  // below the face
    const double v_dot_d = dot(v.v, direction);
    if (v_dot_d < 0.0) return CG_PANIC;
    if (dv_(sb_(v_dot_w, wn2), wn) < 1e-6 || (wn == 0.0 && dv_(v_dot_d, norm(direction)) < 1e-6)) {
      double l[3];
      D3 n;
      lambda_area(v1, v2, v3, l, &n);
      *cpA = add(add(scale(l[0], S.a(P.via[i1])), scale(l[1], S.a(P.via[i2]))), scale(l[2], S.a(P.via[i3])));
      *cpB = add(add(scale(l[0], S.b(P.vib[i1])), scale(l[1], S.b(P.vib[i2]))), scale(l[2], S.b(P.vib[i3])));
      return CG_HIT;
    }
    // horizon: the popped face's edges, then every live face the new vertex sees
    P.ne = 3;
    P.e0[0] = (uint8_t)i1;
    P.e1[0] = (uint8_t)i2;
    P.e0[1] = (uint8_t)i2;
    P.e1[1] = (uint8_t)i3;
    P.e0[2] = (uint8_t)i3;
    P.e1[2] = (uint8_t)i1;
    for (int h = 0; h < P.nh; ++h) {
      const int i = P.heap[h];
      if (P.obs[i]) continue;
      const double wni = P.dist[i];
      bool seen = false;
      if (wni != 0.0 && dot(v.v, P.w(i)) > ad_(P.wn2[i], 0.0)) {
        seen = true;
      } else if (!(wni > 0.0)) {  // a face through the origin, seen along its normal
        const D3 a = P.v(P.t0[i]);
        const D3 tn = cross(sub(P.v(P.t1[i]), a), sub(P.v(P.t2[i]), a));
        seen = dot(v.v, tn) > 0.0;
      }
      if (!seen) continue;
      P.obs[i] = 1;
      if (!P.edge(P.t0[i], P.t1[i]) || !P.edge(P.t1[i], P.t2[i]) || !P.edge(P.t2[i], P.t0[i])) return CG_OVERFLOW;
    }
    if (P.nv >= MAXV) return CG_OVERFLOW;
    const int vi = P.nv++;
    P.vx[vi] = v.v.x;
    P.vy[vi] = v.v.y;
    P.vz[vi] = v.v.z;
    P.via[vi] = (uint8_t)v.ia;
    P.vib[vi] = (uint8_t)v.ib;
    for (int k = 0; k < P.ne; ++k) {
      const int a = P.e0[k], b = P.e1[k];
      const D3 ea = P.v(a), eb = P.v(b);
      const D3 tn = cross(sub(eb, ea), sub(v.v, ea));
      if (norm2(tn) == 0.0) return CG_PANIC;
      if (dot(tn, ea) < 0.0) return CG_PANIC;
      if (!P.add_face(a, b, vi)) return CG_OVERFLOW;
    }
  }
  return CG_OVERFLOW;
}

// CollisionDetector::new(A, B).gjk() then .epa(): both shapes moved by −t_A,
// the contact points moved back.  translate = false queries the shapes where
// they are.
__device__ __noinline__ int collide(const BoxPose& A, const BoxPose& B, bool translate, D3* cpA, D3* cpB) {
  D3 ta{A.t[0], A.t[1], A.t[2]}, tb{B.t[0], B.t[1], B.t[2]};
  const D3 off = ta;
  if (translate) {
    ta = add(ta, neg(off));
    tb = add(tb, neg(off));
  }
  Shapes S;
  box_points(A, ta, S.ax, S.ay, S.az);
  box_points(B, tb, S.bx, S.by, S.bz);
  PV s[4];
  const int g = gjk(S, ta, tb, s);
  if (g != CG_HIT) return g;
  Poly P;
  D3 ca, cb;
  const int e = epa(S, s, P, &ca, &cb);
  if (e != CG_HIT) return e;
  if (translate) {
    ca = add(ca, off);
    cb = add(cb, off);
  }
  *cpA = ca;
  *cpB = cb;
  return CG_HIT;
}

}  // namespace gcol
