// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// Cuboid–cuboid collision of gorilla-physics (GJK + EPA, src/collision/gjk.rs,
// epa.rs, polytope.rs, mod.rs) restated on the CPU as the checker of the GPU
// library's collision routine.
#pragma once

namespace orc_col {

// High-water marks of one query (sizes of the reference's growing vectors).
struct Stats {
  int gjk_iters = 0;  // support evaluations of GJK
  int epa_iters = 0;  // EPA expansions (new vertices)
  int verts = 0;      // polytope vertices
  int tris = 0;       // triangles ever created
  int edges = 0;      // largest candidate edge list
  int heap = 0;       // largest heap
  long long flops = 0;  // FP64 operations of the restated algorithm (add, sub, mul, div, sqrt = 1)
};

// Outcome codes.  1: in collision (cp_a, cp_b written); 0: no collision;
// negative: a case where the reference panics (or a loop bound, see
// collision.cpp).
enum {
  COL_HIT = 1,
  COL_NONE = 0,
  COL_GJK_COLINEAR = -1,      // gjk.rs:70-72
  COL_GJK_ORIENTATION = -2,   // gjk.rs:86-88,98-100,110-112
  COL_GJK_LOOP = -3,          // iteration bound (the reference loops without one)
  COL_EPA_DEGENERATE = -4,    // epa.rs:141-143
  COL_EPA_BELOW = -5,         // epa.rs:150-155
  COL_EPA_OPPOSITE = -6,      // epa.rs:156-158
  COL_EPA_COLINEAR = -7,      // epa.rs:233-235
  COL_EPA_EDGE = -8,          // epa.rs:236-238
  COL_EPA_EMPTY = -9,         // heap.pop().unwrap() on an empty heap, epa.rs:127
  COL_EPA_LOOP = -10,         // iteration bound
};

// One query.  Each cuboid: row-major rotation R (9), centre t (3), sizes
// (w, d, h).  translate = true is CollisionDetector (src/collision/mod.rs:48-87:
// both shapes moved by −t_A, contact points moved back); false runs gjk / epa
// on the shapes where they are (the form of the reference's gjk/epa unit tests).
int collide(const double* RA, const double* tA, const double* dA, const double* RB, const double* tB,
            const double* dB, bool translate, double* cp_a, double* cp_b, Stats* st);

// UnitQuaternion::to_rotation_matrix for (x, y, z, w).
void quat_to_matrix(const double* q, double* R);

}  // namespace orc_col
