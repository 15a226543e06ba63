// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// CPU restatement of gorilla-physics' cuboid–cuboid collision detection:
//   Cuboid::recompute_points / compute_support    src/collision/cuboid.rs:18-40,86-96
//   support_fn                                    src/collision/polytope.rs:59-68
//   gjk                                           src/collision/gjk.rs:14-125
//   Polytope::from_simplex                        src/collision/polytope.rs:26-39
//   solve_closest_point_{lambda_,}area_method     src/collision/epa.rs:69-96
//   epa                                           src/collision/epa.rs:108-254
//   addEdgeIfNotExisting, CollisionDetector       src/collision/mod.rs:21-87
// Vectors are growing std::vectors as in the reference; the heap follows Rust's
// std::collections::BinaryHeap (push = append + sift-up; pop = swap the last
// element to the root, sift it to the bottom along the larger children, then
// sift it up), because EPA's visibility loop walks the heap's array in storage
// order (epa.rs:177), and that order decides the order of the new triangles and
// so every later tie between equal distances.  Its element order is
// Reverse((OrderedFloat(distance), triangle index)): the smallest distance
// first, ties to the lowest index, NaN above every number.
//
// The arithmetic is written out in nalgebra's order for each operation (dot
// products and matrix-vector products summed left to right, the cross product
// as (a_y b_z − a_z b_y, a_z b_x − a_x b_z, a_x b_y − a_y b_x), norms as
// sqrt(x² + y² + z²)) and the file is compiled without floating-point
// contraction, so the GPU routine that computes the same operations in the same
// order with IEEE-rounded intrinsics agrees with it bit for bit.
//
// Loop bounds: the reference's GJK and EPA loops have none.  Here GJK stops
// after 1000 support evaluations and EPA after 1000 expansions (COL_*_LOOP),
// far above anything observed, so that a pathological input fails instead of
// hanging a test.

#include "collision.h"

#include <cmath>
#include <utility>
#include <vector>

namespace orc_col {
namespace {

// Operation count of the current query (the algorithmic work the throughput
// figures are measured against): add, sub, mul, div and sqrt count 1 each.
thread_local long long g_flops = 0;

struct V {
  double x, y, z;
};
inline V add(V a, V b) {
  g_flops += 3;
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
inline V sub(V a, V b) {
  g_flops += 3;
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
inline V neg(V a) { return {-a.x, -a.y, -a.z}; }
inline V scale(double s, V a) {
  g_flops += 3;
  return {s * a.x, s * a.y, s * a.z};
}
inline double dot(V a, V b) {
  g_flops += 5;
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
inline V cross(V a, V b) {
  g_flops += 9;
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm2(V a) {
  g_flops += 5;
  return a.x * a.x + a.y * a.y + a.z * a.z;
}
inline double norm(V a) {
  g_flops += 1;
  return std::sqrt(norm2(a));
}
inline bool is_zero(V a) { return a.x == 0.0 && a.y == 0.0 && a.z == 0.0; }

// Cuboid corner points in world (or detector) coordinates, in the order of
// cuboid.rs:22-31: x sign from bit 0, y sign from bit 1, z sign from bit 2.
struct Box {
  V p[8];
};
Box make_box(const double* R, V t, const double* dims) {
  Box b;
  const double hw = dims[0] / 2.0, hd = dims[1] / 2.0, hh = dims[2] / 2.0;
  g_flops += 3 + 8 * 15;  // half sizes; R c per corner (+ t counted by add)
  for (int k = 0; k < 8; ++k) {
    const V c{(k & 1) ? -hw : hw, (k & 2) ? -hd : hd, (k & 4) ? -hh : hh};
    const V r{R[0] * c.x + R[1] * c.y + R[2] * c.z, R[3] * c.x + R[4] * c.y + R[5] * c.z,
              R[6] * c.x + R[7] * c.y + R[8] * c.z};
    b.p[k] = add(r, t);
  }
  return b;
}
// compute_support: the first corner of largest d·p.
int support(const Box& b, V d) {
  int best = 0;
  double bv = dot(d, b.p[0]);
  for (int k = 1; k < 8; ++k) {
    const double v = dot(d, b.p[k]);
    if (v > bv) {
      bv = v;
      best = k;
    }
  }
  return best;
}

struct PV {  // PolytopeVertex
  V v;
  int ia, ib;
};
PV support_fn(const Box& A, const Box& B, V d) {
  const int ia = support(A, d), ib = support(B, neg(d));
  return {sub(A.p[ia], B.p[ib]), ia, ib};
}

int gjk(const Box& A, const Box& B, V cA, V cB, std::vector<PV>& simplex, Stats* st) {
  const V origin{0.0, 0.0, 0.0};
  V dir = (cA.x == cB.x && cA.y == cB.y && cA.z == cB.z) ? V{1.0, 0.0, 0.0} : sub(cA, cB);
  simplex.clear();
  for (int it = 1;; ++it) {
    if (it > 1000) return COL_GJK_LOOP;
    if (st && it > st->gjk_iters) st->gjk_iters = it;
    const PV nv = support_fn(A, B, dir);
    if (is_zero(nv.v)) return COL_NONE;        // origin is a vertex: touching
    if (dot(dir, nv.v) <= 0.0) return COL_NONE;  // not past the origin
    simplex.push_back(nv);
    switch (simplex.size()) {
      case 1:
        dir = sub(origin, nv.v);
        break;
      case 2: {
        const V v1 = simplex[0].v, v2 = simplex[1].v;
        const V v1v2 = sub(v2, v1);
        dir = cross(cross(v1, v2), v1v2);
        if (norm(dir) == 0.0) {  // origin on the edge
          const V cand = cross(v1v2, V{1.0, 0.0, 0.0});
          dir = norm(cand) > 0.0 ? cand : cross(v1v2, V{0.0, 1.0, 0.0});
        }
        break;
      }
      case 3: {
        const V v1 = simplex[0].v, v2 = simplex[1].v, v3 = simplex[2].v;
        dir = cross(sub(v3, v1), sub(v2, v1));
        if (dot(dir, sub(origin, v1)) < 0.0) {
          dir = neg(dir);
          std::swap(simplex[1], simplex[2]);
        }
        if (norm(dir) == 0.0) return COL_GJK_COLINEAR;
        break;
      }
      default: {  // 4
        const PV p1 = simplex[0], p2 = simplex[1], p3 = simplex[2], p4 = simplex[3];
        const V v1 = p1.v, v2 = p2.v, v3 = p3.v, v4 = p4.v;
        const V v1v3 = sub(v3, v1), v1v2 = sub(v2, v1), v1v4 = sub(v4, v1);
        const V n143 = cross(v1v3, v1v4);
        if (dot(n143, v1v2) > 0.0) return COL_GJK_ORIENTATION;
        if (dot(n143, v1) < 0.0) {
          dir = n143;
          simplex = {p1, p4, p3};
          continue;
        }
        const V v2v3 = sub(v3, v2), v2v4 = sub(v4, v2), v2v1 = neg(v1v2);
        const V n234 = cross(v2v4, v2v3);
        if (dot(n234, v2v1) > 0.0) return COL_GJK_ORIENTATION;
        if (dot(n234, v2) < 0.0) {
          dir = n234;
          simplex = {p2, p3, p4};
          continue;
        }
        const V n124 = cross(v1v4, v1v2);
        if (dot(n124, v1v3) > 0.0) return COL_GJK_ORIENTATION;
        if (dot(n124, v1) < 0.0) {
          dir = n124;
          simplex = {p1, p2, p4};
          continue;
        }
        return COL_HIT;  // the origin is inside the tetrahedron
      }
    }
  }
}

// Barycentric coordinates of the origin's projection on the plane of
// (v1, v2, v3), and the plane normal (v2 − v1) × (v3 − v1).
void lambda_area(V v1, V v2, V v3, double* lam, V* normal) {
  const V v1v2 = sub(v2, v1), v1v3 = sub(v3, v1);
  const V n = cross(v1v2, v1v3);
  const double inv = 1.0 / norm2(n);
  const double b3 = dot(cross(v1, v1v2), n) * inv;
  const double b2 = dot(cross(v1v3, v1), n) * inv;
  g_flops += 5;
  lam[0] = 1.0 - (b2 + b3);
  lam[1] = b2;
  lam[2] = b3;
  *normal = n;
}
V closest_area(V v1, V v2, V v3) {
  double l[3];
  V n;
  lambda_area(v1, v2, v3, l, &n);
  const V w = add(add(scale(l[0], v1), scale(l[1], v2)), scale(l[2], v3));
  const double s = dot(w, n), nn = norm2(n);
  g_flops += 6;
  return {s * n.x / nn, s * n.y / nn, s * n.z / nn};
}

// Rust's BinaryHeap<Reverse<(OrderedFloat<f64>, usize)>>.
struct Heap {
  struct E {
    double d;
    int i;
  };
  std::vector<E> a;
  // OrderedFloat: NaN equals NaN and exceeds every number.
  static int cmpf(double x, double y) {
    const bool nx = std::isnan(x), ny = std::isnan(y);
    if (nx || ny) return nx == ny ? 0 : (nx ? 1 : -1);
    return x < y ? -1 : (x > y ? 1 : 0);
  }
  static int cmp(const E& x, const E& y) {
    const int c = cmpf(x.d, y.d);
    return c ? c : (x.i < y.i ? -1 : (x.i > y.i ? 1 : 0));
  }
  // Reverse(x) <= Reverse(y)  ⟺  y <= x
  static bool le(const E& x, const E& y) { return cmp(y, x) <= 0; }
  void sift_up(size_t start, size_t pos) {
    const E e = a[pos];
    while (pos > start) {
      const size_t parent = (pos - 1) / 2;
      if (le(e, a[parent])) break;
      a[pos] = a[parent];
      pos = parent;
    }
    a[pos] = e;
  }
  void push(E e) {
    a.push_back(e);
    sift_up(0, a.size() - 1);
  }
  bool pop(E* out) {
    if (a.empty()) return false;
    E item = a.back();
    a.pop_back();
    if (!a.empty()) {
      std::swap(item, a[0]);
      // sift_down_to_bottom(0)
      const size_t end = a.size();
      size_t pos = 0;
      const E e = a[0];
      size_t child = 1;
      while (child + 1 < end) {  // child <= end.saturating_sub(2)
        if (le(a[child], a[child + 1])) child += 1;
        a[pos] = a[child];
        pos = child;
        child = 2 * pos + 1;
      }
      if (child == end - 1) {
        a[pos] = a[child];
        pos = child;
      }
      a[pos] = e;
      sift_up(0, pos);
    }
    *out = item;
    return true;
  }
};

void add_edge_if_not_existing(std::vector<std::pair<int, int>>& E, std::pair<int, int> e) {
  for (size_t k = 0; k < E.size(); ++k)
    if (E[k].first == e.second && E[k].second == e.first) {
      E.erase(E.begin() + (long)k);
      return;
    }
  E.push_back(e);
}

struct Tri {
  int a, b, c;
};

int epa(const std::vector<PV>& simplex, const Box& A, const Box& B, V* cpA, V* cpB, Stats* st) {
  std::vector<PV> verts = simplex;
  std::vector<Tri> tris = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
  std::vector<V> closest;
  std::vector<bool> obsolete(4, false);
  Heap heap;
  for (int i = 0; i < 4; ++i) {
    const Tri& t = tris[i];
    const V w = closest_area(verts[t.a].v, verts[t.b].v, verts[t.c].v);
    closest.push_back(w);
    heap.push({norm(w), i});
  }
  auto track = [&](size_t edges) {
    if (!st) return;
    if ((int)verts.size() > st->verts) st->verts = (int)verts.size();
    if ((int)tris.size() > st->tris) st->tris = (int)tris.size();
    if ((int)heap.a.size() > st->heap) st->heap = (int)heap.a.size();
    if ((int)edges > st->edges) st->edges = (int)edges;
  };
  track(0);
  for (int it = 0;; ++it) {
    if (it > 1000) return COL_EPA_LOOP;
    Heap::E el;
    if (!heap.pop(&el)) return COL_EPA_EMPTY;
    const int index = el.i;
    if (obsolete[index]) continue;
    obsolete[index] = true;
    const Tri tri = tris[index];
    const V w = closest[index];
    const PV p1 = verts[tri.a], p2 = verts[tri.b], p3 = verts[tri.c];
    const V normal = cross(sub(p2.v, p1.v), sub(p3.v, p1.v));
    if (norm(normal) == 0.0) return COL_EPA_DEGENERATE;
    const V direction = normal;
    const PV v = support_fn(A, B, direction);
    const double v_dot_w = dot(v.v, w);
    const double wn2 = norm2(w);
    g_flops += 4;  // the three explicit operations of the tests below (and a division)
    if (v_dot_w < wn2 - 1e-8) return COL_EPA_BELOW;
    if (dot(v.v, direction) < 0.0) return COL_EPA_OPPOSITE;
    if ((v_dot_w - wn2) / norm(w) < 1e-6 ||
        (norm(w) == 0.0 && dot(v.v, direction) / norm(direction) < 1e-6)) {
      double lam[3];
      V n;
      lambda_area(p1.v, p2.v, p3.v, lam, &n);
      *cpA = add(add(scale(lam[0], A.p[p1.ia]), scale(lam[1], A.p[p2.ia])), scale(lam[2], A.p[p3.ia]));
      *cpB = add(add(scale(lam[0], B.p[p1.ib]), scale(lam[1], B.p[p2.ib])), scale(lam[2], B.p[p3.ib]));
      if (st && it > st->epa_iters) st->epa_iters = it;
      return COL_HIT;
    }
    std::vector<std::pair<int, int>> edges = {{tri.a, tri.b}, {tri.b, tri.c}, {tri.c, tri.a}};
    for (const Heap::E& e : heap.a) {
      const int i = e.i;
      if (obsolete[i]) continue;
      const V wi = closest[i];
      const Tri& t = tris[i];
      if (norm(wi) != 0.0 && dot(v.v, wi) > norm2(wi) + 0.0) {
        obsolete[i] = true;  // the new vertex sees this face
        add_edge_if_not_existing(edges, {t.a, t.b});
        add_edge_if_not_existing(edges, {t.b, t.c});
        add_edge_if_not_existing(edges, {t.c, t.a});
        if (st && (int)edges.size() > st->edges) st->edges = (int)edges.size();
        continue;
      }
      if (norm(wi) > 0.0) continue;
      const V tn = cross(sub(verts[t.b].v, verts[t.a].v), sub(verts[t.c].v, verts[t.a].v));
      if (dot(v.v, tn) > 0.0) {  // face through the origin, seen along its normal
        obsolete[i] = true;
        add_edge_if_not_existing(edges, {t.a, t.b});
        add_edge_if_not_existing(edges, {t.b, t.c});
        add_edge_if_not_existing(edges, {t.c, t.a});
        if (st && (int)edges.size() > st->edges) st->edges = (int)edges.size();
      }
    }
    verts.push_back(v);
    const int vi = (int)verts.size() - 1;
    for (const auto& ed : edges) {
      const V e1 = verts[ed.first].v, e2 = verts[ed.second].v;
      const V tn = cross(sub(e2, e1), sub(v.v, e1));
      if (norm(tn) == 0.0) return COL_EPA_COLINEAR;
      if (dot(tn, e1) < 0.0) return COL_EPA_EDGE;
      tris.push_back({ed.first, ed.second, vi});
      const V wn = closest_area(e1, e2, v.v);
      closest.push_back(wn);
      obsolete.push_back(false);
      heap.push({norm(wn), (int)tris.size() - 1});
    }
    track(edges.size());
    if (st && it + 1 > st->epa_iters) st->epa_iters = it + 1;
  }
}

}  // namespace

void quat_to_matrix(const double* q, double* R) {
  const double i = q[0], j = q[1], k = q[2], w = q[3];
  const double ww = w * w, ii = i * i, jj = j * j, kk = k * k;
  const double ij = i * j * 2.0, wk = w * k * 2.0, wj = w * j * 2.0, ik = i * k * 2.0, jk = j * k * 2.0,
               wi = w * i * 2.0;
  R[0] = ww + ii - jj - kk;
  R[1] = ij - wk;
  R[2] = wj + ik;
  R[3] = wk + ij;
  R[4] = ww - ii + jj - kk;
  R[5] = jk - wi;
  R[6] = ik - wj;
  R[7] = wi + jk;
  R[8] = ww - ii - jj + kk;
}

int collide(const double* RA, const double* tA, const double* dA, const double* RB, const double* tB,
            const double* dB, bool translate, double* cp_a, double* cp_b, Stats* st) {
  g_flops = 0;
  V ta{tA[0], tA[1], tA[2]}, tb{tB[0], tB[1], tB[2]};
  const V off = ta;
  if (translate) {  // Isometry3::append_translation_mut(−t_A) on both shapes
    ta = add(ta, neg(off));
    tb = add(tb, neg(off));
  }
  const Box A = make_box(RA, ta, dA), B = make_box(RB, tb, dB);
  std::vector<PV> simplex;
  const int g = gjk(A, B, ta, tb, simplex, st);
  if (st) st->flops = g_flops;
  if (g != COL_HIT) return g;
  V ca, cb;
  const int e = epa(simplex, A, B, &ca, &cb, st);
  if (st) st->flops = g_flops;
  if (e != COL_HIT) return e;
  if (translate) {
    ca = add(ca, off);
    cb = add(cb, off);
  }
  if (st) st->flops = g_flops;
  cp_a[0] = ca.x;
  cp_a[1] = ca.y;
  cp_a[2] = ca.z;
  cp_b[0] = cb.x;
  cp_b[1] = cb.y;
  cp_b[2] = cb.z;
  return COL_HIT;
}

}  // namespace orc_col
