// Articulated-body algorithm (included by gpb_kernels.cu after gpb_link.cuh).
//
// Featherstone, "Rigid Body Dynamics Algorithms", Table 7.1: q̈ in three O(n)
// passes over the tree in link coordinates — velocities and bias terms
// outward, articulated inertias and bias forces inward, accelerations
// outward — instead of the reference's CRBA mass matrix and dense solve
// (src/dynamics.rs:255-276, src/mechanism.rs:592-696).  The same q̈ in exact
// arithmetic; no O(n²) fill and no O(n³) factorisation, so a 48-DOF chain
// costs about half the FP64 work and its critical path shrinks accordingly.
//
// Precision: kinematics, bias forces and the final accelerations run in R
// (double for GPB_FP64, float for GPB_MIXED).  The articulated inertias, the
// projections U = I^A S, D = Sᵀ U and the congruence X*ᵀ I^a X to the parent
// frame need more than FP32: that recursion subtracts U D⁻¹ Uᵀ from I^A and is
// where FP32 loses digits on long chains (FP32 everywhere gives q̈ errors up to
// 2e-5 of |q̈| on 48-DOF chains).  GPB_FP64 runs it in FP64; GPB_MIXED runs it
// in double-float (gpb_ff.cuh, about 48 bits) on the FP32 pipes, from the
// FP32-rounded model and the FP32 joint transforms of its kinematics — the
// exact recursion of a model perturbed by ≤ 6e-8 relative, which moves q̈ of
// the 48-DOF chains by less than 1e-6 of max |q̈|.  The q̈ solve of a 1-DOF
// joint, D⁻¹ (u − Uᵀ a), is double-float too; a floating joint's 6×6 solve
// stays FP64.  The poses that place contact points are computed in FP64
// whenever an instance has contacts (a penetration error ε·|p| becomes a force
// error k·ε·|p|).
#pragma once

// Symmetric 6×6 spatial inertia in blocks [[A, B], [Bᵀ, C]] acting on (ω, v):
// A, C symmetric (xx, yy, zz, xy, xz, yz), B row-major.  A rigid body's is
// A = J, B = [c]×, C = m·1 (the convention of imul).
struct ABI {
  double A[6], B[9], C[6];
};
constexpr int ABI_D = 21;

template <typename T>
__device__ __forceinline__ T symget(const T* S, int i, int j) {
  // (0,0)=0 (1,1)=1 (2,2)=2 (0,1)=3 (0,2)=4 (1,2)=5
  if (i == j) return S[i];
  const int a = i < j ? i : j, b = i < j ? j : i;
  return S[a == 0 ? (b == 1 ? 3 : 4) : 5];
}

template <typename R>
__device__ __forceinline__ void store_abi(const LaneCtx<R>& c, int base, const ABI& I) {
#pragma unroll
  for (int k = 0; k < 6; ++k) c.d(base + k) = I.A[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) c.d(base + 6 + k) = I.B[k];
#pragma unroll
  for (int k = 0; k < 6; ++k) c.d(base + 15 + k) = I.C[k];
}
template <typename R>
__device__ __forceinline__ ABI load_abi(const LaneCtx<R>& c, int base) {
  ABI I;
#pragma unroll
  for (int k = 0; k < 6; ++k) I.A[k] = c.d(base + k);
#pragma unroll
  for (int k = 0; k < 9; ++k) I.B[k] = c.d(base + 6 + k);
#pragma unroll
  for (int k = 0; k < 6; ++k) I.C[k] = c.d(base + 15 + k);
  return I;
}
__device__ __forceinline__ void abi_add(ABI& a, const ABI& b) {
#pragma unroll
  for (int k = 0; k < 6; ++k) a.A[k] += b.A[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) a.B[k] += b.B[k];
#pragma unroll
  for (int k = 0; k < 6; ++k) a.C[k] += b.C[k];
}

// Rigid-body inertia from the topology table (mass, m·com, J about the origin).
template <typename R>
__device__ __forceinline__ ABI body_abi(const LaneCtx<R>& c, int tb) {
  ABI I;
  const double m = c.td(tb + TD_INERTIA);
  const double cx = c.td(tb + TD_INERTIA + 1), cy = c.td(tb + TD_INERTIA + 2), cz = c.td(tb + TD_INERTIA + 3);
#pragma unroll
  for (int k = 0; k < 6; ++k) I.A[k] = c.td(tb + TD_INERTIA + 4 + k);
  I.B[0] = 0.0, I.B[1] = -cz, I.B[2] = cy;
  I.B[3] = cz, I.B[4] = 0.0, I.B[5] = -cx;
  I.B[6] = -cy, I.B[7] = cx, I.B[8] = 0.0;
  I.C[0] = I.C[1] = I.C[2] = m;
  I.C[3] = I.C[4] = I.C[5] = 0.0;
  return I;
}

// I·(w, v) = (A w + B v, Bᵀ w + C v).
__device__ __forceinline__ void abi_mul(const ABI& I, const double* w, const double* v, double* ow, double* ov) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ow[i] = symget(I.A, i, 0) * w[0] + symget(I.A, i, 1) * w[1] + symget(I.A, i, 2) * w[2] +
            I.B[3 * i] * v[0] + I.B[3 * i + 1] * v[1] + I.B[3 * i + 2] * v[2];
    ov[i] = I.B[i] * w[0] + I.B[3 + i] * w[1] + I.B[6 + i] * w[2] + symget(I.C, i, 0) * v[0] +
            symget(I.C, i, 1) * v[1] + symget(I.C, i, 2) * v[2];
  }
}

// S' = R S Rᵀ for symmetric S.
__device__ __forceinline__ void sym_rotate(const double* R, const double* S, double* out) {
  double P[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      P[3 * i + j] = R[3 * i] * symget(S, 0, j) + R[3 * i + 1] * symget(S, 1, j) + R[3 * i + 2] * symget(S, 2, j);
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k)
    out[k] = P[3 * ii[k]] * R[3 * jj[k]] + P[3 * ii[k] + 1] * R[3 * jj[k] + 1] + P[3 * ii[k] + 2] * R[3 * jj[k] + 2];
}
// B' = R B Rᵀ for general B.
__device__ __forceinline__ void gen_rotate(const double* R, const double* B, double* out) {
  double P[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) P[3 * i + j] = R[3 * i] * B[j] + R[3 * i + 1] * B[3 + j] + R[3 * i + 2] * B[6 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      out[3 * i + j] = P[3 * i] * R[3 * j] + P[3 * i + 1] * R[3 * j + 1] + P[3 * i + 2] * R[3 * j + 2];
}

// Three-way choice by a runtime axis index, written as selects: a small array
// indexed by a runtime value would be placed in local memory.
template <typename T>
__device__ __forceinline__ T pick3(int k, T x0, T x1, T x2) {
  return k == 0 ? x0 : (k == 1 ? x1 : x2);
}
// Rotation about principal axis e_k by (cos, sin): only the (k+1, k+2) plane
// (mod 3) turns.
template <typename T>
__device__ __forceinline__ M3<T> planar_rot(int k, T co, T si) {
  const T z = T(0), o = T(1);
  M3<T> R;
  R.a[0] = k == 0 ? o : co;
  R.a[1] = k == 2 ? -si : z;
  R.a[2] = k == 1 ? si : z;
  R.a[3] = k == 2 ? si : z;
  R.a[4] = k == 1 ? o : co;
  R.a[5] = k == 0 ? -si : z;
  R.a[6] = k == 1 ? -si : z;
  R.a[7] = k == 0 ? si : z;
  R.a[8] = k == 2 ? o : co;
  return R;
}

// One plane rotation of a pair: (co·a − si·b, si·a + co·b), in FP64 or in
// double-float with FP32 (cos, sin).
__device__ __forceinline__ void rot2(double a, double b, double co, double si, double& x, double& y) {
  x = co * a - si * b;
  y = si * a + co * b;
}
__device__ __forceinline__ void rot2(FF a, FF b, float co, float si, FF& x, FF& y) {
  x = ff_lin2(a, co, b, -si);
  y = ff_lin2(a, si, b, co);
}

// The rotation about principal axis k applied to the rows of a 3-column block
// (x_i1' = c x_i1 − s x_i2, x_i2' = s x_i1 + c x_i2 with i1 = k+1, i2 = k+2
// mod 3) or to its columns.
template <typename W, typename S>
__device__ __forceinline__ void planar_rows(W* M, int k, S co, S si) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    W x, y;
    rot2(pick3(k, M[3 + j], M[6 + j], M[j]), pick3(k, M[6 + j], M[j], M[3 + j]), co, si, x, y);
    M[j] = pick3(k, M[j], y, x);
    M[3 + j] = pick3(k, x, M[3 + j], y);
    M[6 + j] = pick3(k, y, x, M[6 + j]);
  }
}
template <typename W, typename S>
__device__ __forceinline__ void planar_cols(W* M, int k, S co, S si) {
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    W x, y;
    rot2(pick3(k, M[3 * r + 1], M[3 * r + 2], M[3 * r]), pick3(k, M[3 * r + 2], M[3 * r], M[3 * r + 1]), co, si,
         x, y);
    M[3 * r] = pick3(k, M[3 * r], y, x);
    M[3 * r + 1] = pick3(k, x, M[3 * r + 1], y);
    M[3 * r + 2] = pick3(k, y, x, M[3 * r + 2]);
  }
}
// R S Rᵀ for symmetric S and the rotation about principal axis k: only the
// plane block (a = S_i1i1, b = S_i2i2, d = S_i1i2) and the couplings to the
// axis (e1 = S_i1k, e2 = S_i2k) change.
__device__ __forceinline__ void sym_planar_terms(double a, double b, double d, double e1, double e2, double co,
                                                 double si, double& a2, double& b2, double& d2, double& f1,
                                                 double& f2) {
  const double c2 = co * co, s2 = si * si, cs = co * si;
  const double cs2d = 2.0 * cs * d;
  a2 = c2 * a + s2 * b - cs2d;
  b2 = s2 * a + c2 * b + cs2d;
  d2 = cs * (a - b) + (c2 - s2) * d;
  f1 = co * e1 - si * e2;
  f2 = si * e1 + co * e2;
}
// double-float: rows, then columns (M = R S, S' = M Rᵀ), each entry one ff_lin2
__device__ __forceinline__ void sym_planar_terms(FF a, FF b, FF d, FF e1, FF e2, float co, float si, FF& a2, FF& b2,
                                                 FF& d2, FF& f1, FF& f2) {
  FF m11, m21, m12, m22;
  rot2(a, d, co, si, m11, m21);
  rot2(d, b, co, si, m12, m22);
  rot2(m11, m12, co, si, a2, d2);
  b2 = ff_lin2(m21, si, m22, co);
  rot2(e1, e2, co, si, f1, f2);
}
// packed order xx yy zz xy xz yz
template <typename W, typename S>
__device__ __forceinline__ void sym_planar(W* P, int k, S co, S si) {
  W a2, b2, d2, f1, f2;
  sym_planar_terms(pick3(k, P[1], P[2], P[0]), pick3(k, P[2], P[0], P[1]), pick3(k, P[5], P[4], P[3]),
                   pick3(k, P[3], P[5], P[4]), pick3(k, P[4], P[3], P[5]), co, si, a2, b2, d2, f1, f2);
  P[0] = pick3(k, P[0], b2, a2);
  P[1] = pick3(k, a2, P[1], b2);
  P[2] = pick3(k, b2, a2, P[2]);
  P[3] = pick3(k, f1, f2, d2);
  P[4] = pick3(k, f2, d2, f1);
  P[5] = pick3(k, d2, f1, f2);
}

template <typename W>
__device__ __forceinline__ void sym_expand(const W* S, W* F) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[3 * i + j] = symget(S, i, j);
}
template <typename W>
__device__ __forceinline__ void sym_pack(const W* F, W* S) {
  S[0] = F[0], S[1] = F[4], S[2] = F[8], S[3] = F[1], S[4] = F[2], S[5] = F[5];
}

// General shift by t (T = [t]×): C_p = C', B_p = B' + T C',
// A_p = A' − B'T − (B'T)ᵀ − T C' T.
__device__ __forceinline__ void shift_general(const double* A, const double* B, const double* Cm, V3<double> t,
                                              ABI& o) {
  double W[9], BT[9];  // W = T C', BT = B' T
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    W[j] = -t.z * Cm[3 + j] + t.y * Cm[6 + j];
    W[3 + j] = t.z * Cm[j] - t.x * Cm[6 + j];
    W[6 + j] = -t.y * Cm[j] + t.x * Cm[3 + j];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    BT[3 * i] = B[3 * i + 1] * t.z - B[3 * i + 2] * t.y;
    BT[3 * i + 1] = -B[3 * i] * t.z + B[3 * i + 2] * t.x;
    BT[3 * i + 2] = B[3 * i] * t.y - B[3 * i + 1] * t.x;
  }
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int i = ii[k], j = jj[k];
    // (T C' T)_ij = (W T)_ij
    const double wt = j == 0 ? (W[3 * i + 1] * t.z - W[3 * i + 2] * t.y)
                             : (j == 1 ? (-W[3 * i] * t.z + W[3 * i + 2] * t.x) : (W[3 * i] * t.y - W[3 * i + 1] * t.x));
    o.A[k] = A[3 * i + j] - BT[3 * i + j] - BT[3 * j + i] - wt;
    o.C[k] = Cm[3 * i + j];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) o.B[k] = B[k] + W[k];
}

// Articulated inertia of a child, in the child frame, expressed in the parent
// frame: X*ᵀ I X for the child→parent transform (rotation Rr, child origin t):
// every block rotated (R S Rᵀ) — a planar rotation when `planar` ≥ 0 (the
// rotation about that principal axis by (co, si)) — then shifted by t.  One
// code path for every lane, so a mechanism's result does not depend on the
// mechanisms sharing its warp (lanes with different axes run it together).
__device__ __forceinline__ ABI abi_to_parent(const ABI& I, const double* Rr, V3<double> t, int planar, double co,
                                             double si) {
  double A[9], B[9], Cm[9];
  if (planar >= 0) {
    double a6[6], c6[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      a6[k] = I.A[k];
      c6[k] = I.C[k];
    }
    sym_planar(a6, planar, co, si);
    sym_planar(c6, planar, co, si);
    sym_expand(a6, A);
    sym_expand(c6, Cm);
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = I.B[k];
    planar_rows(B, planar, co, si);
    planar_cols(B, planar, co, si);
  } else {
    double a6[6], c6[6];
    sym_rotate(Rr, I.A, a6);
    sym_rotate(Rr, I.C, c6);
    gen_rotate(Rr, I.B, B);
    sym_expand(a6, A);
    sym_expand(c6, Cm);
  }
  ABI o;
  shift_general(A, B, Cm, t, o);
  return o;
}

// ---- double-float articulated inertias (GPB_MIXED) -------------------------
// The same blocks as ABI, each entry an FF pair; rotations and translations
// are the FP32 joint transforms of the sweep.
struct ABIF {
  FF A[6], B[9], C[6];
};

// FF view of an 8-byte scratch word (the pair is stored as hi, lo).
template <typename R>
__device__ __forceinline__ FF& ffw(const LaneCtx<R>& c, int e) {
  return *reinterpret_cast<FF*>(&c.d(e));
}
template <typename R>
__device__ __forceinline__ void store_abi_ff(const LaneCtx<R>& c, int base, const ABIF& I) {
#pragma unroll
  for (int k = 0; k < 6; ++k) ffw(c, base + k) = I.A[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) ffw(c, base + 6 + k) = I.B[k];
#pragma unroll
  for (int k = 0; k < 6; ++k) ffw(c, base + 15 + k) = I.C[k];
}
template <typename R>
__device__ __forceinline__ ABIF load_abi_ff(const LaneCtx<R>& c, int base) {
  ABIF I;
#pragma unroll
  for (int k = 0; k < 6; ++k) I.A[k] = ffw(c, base + k);
#pragma unroll
  for (int k = 0; k < 9; ++k) I.B[k] = ffw(c, base + 6 + k);
#pragma unroll
  for (int k = 0; k < 6; ++k) I.C[k] = ffw(c, base + 15 + k);
  return I;
}
__device__ __forceinline__ void abi_add(ABIF& a, const ABIF& b) {
#pragma unroll
  for (int k = 0; k < 6; ++k) a.A[k] = ff_add(a.A[k], b.A[k]);
#pragma unroll
  for (int k = 0; k < 9; ++k) a.B[k] = ff_add(a.B[k], b.B[k]);
#pragma unroll
  for (int k = 0; k < 6; ++k) a.C[k] = ff_add(a.C[k], b.C[k]);
}
__device__ __forceinline__ ABI abi_to_double(const ABIF& I) {
  ABI o;
#pragma unroll
  for (int k = 0; k < 6; ++k) o.A[k] = ff_to_double(I.A[k]);
#pragma unroll
  for (int k = 0; k < 9; ++k) o.B[k] = ff_to_double(I.B[k]);
#pragma unroll
  for (int k = 0; k < 6; ++k) o.C[k] = ff_to_double(I.C[k]);
  return o;
}
// Rigid-body inertia from the FP32 topology table.
template <typename R>
__device__ __forceinline__ ABIF body_abi_ff(const LaneCtx<R>& c, int tb) {
  ABIF I;
  const float m = c.t(tb + TD_INERTIA);
  const float cx = c.t(tb + TD_INERTIA + 1), cy = c.t(tb + TD_INERTIA + 2), cz = c.t(tb + TD_INERTIA + 3);
#pragma unroll
  for (int k = 0; k < 6; ++k) I.A[k] = ff(c.t(tb + TD_INERTIA + 4 + k));
  I.B[0] = ff(0.0f), I.B[1] = ff(-cz), I.B[2] = ff(cy);
  I.B[3] = ff(cz), I.B[4] = ff(0.0f), I.B[5] = ff(-cx);
  I.B[6] = ff(-cy), I.B[7] = ff(cx), I.B[8] = ff(0.0f);
  I.C[0] = I.C[1] = I.C[2] = ff(m);
  I.C[3] = I.C[4] = I.C[5] = ff(0.0f);
  return I;
}
// S' = R S Rᵀ (S symmetric) and B' = R B Rᵀ for an FP32 rotation R.
__device__ __forceinline__ void sym_rotate(const float* R, const FF* S, FF* out) {
  FF P[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      P[3 * i + j] = ff_dot3f(symget(S, 0, j), symget(S, 1, j), symget(S, 2, j), R[3 * i], R[3 * i + 1], R[3 * i + 2]);
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k)
    out[k] = ff_dot3f(P[3 * ii[k]], P[3 * ii[k] + 1], P[3 * ii[k] + 2], R[3 * jj[k]], R[3 * jj[k] + 1],
                      R[3 * jj[k] + 2]);
}
__device__ __forceinline__ void gen_rotate(const float* R, const FF* B, FF* out) {
  FF P[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      P[3 * i + j] = ff_dot3f(B[j], B[3 + j], B[6 + j], R[3 * i], R[3 * i + 1], R[3 * i + 2]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      out[3 * i + j] = ff_dot3f(P[3 * i], P[3 * i + 1], P[3 * i + 2], R[3 * j], R[3 * j + 1], R[3 * j + 2]);
}
// The shift of shift_general with an FP32 translation, in the equivalent form
// B_p = B' + T C', A_p = A' − B_p T − (B' T)ᵀ (B_p T = B'T + T C' T).
__device__ __forceinline__ void shift_general(const FF* A, const FF* B, const FF* Cm, V3<float> t, ABIF& o) {
  FF BT[9];  // B' T
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    BT[3 * i] = ff_lin2(B[3 * i + 1], t.z, B[3 * i + 2], -t.y);
    BT[3 * i + 1] = ff_lin2(B[3 * i], -t.z, B[3 * i + 2], t.x);
    BT[3 * i + 2] = ff_lin2(B[3 * i], t.y, B[3 * i + 1], -t.x);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    o.B[j] = ff_add(B[j], ff_lin2(Cm[3 + j], -t.z, Cm[6 + j], t.y));
    o.B[3 + j] = ff_add(B[3 + j], ff_lin2(Cm[j], t.z, Cm[6 + j], -t.x));
    o.B[6 + j] = ff_add(B[6 + j], ff_lin2(Cm[j], -t.y, Cm[3 + j], t.x));
  }
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int i = ii[k], j = jj[k];
    const FF bpt = j == 0 ? ff_lin2(o.B[3 * i + 1], t.z, o.B[3 * i + 2], -t.y)
                          : (j == 1 ? ff_lin2(o.B[3 * i], -t.z, o.B[3 * i + 2], t.x)
                                    : ff_lin2(o.B[3 * i], t.y, o.B[3 * i + 1], -t.x));
    o.A[k] = ff_sub(A[3 * i + j], ff_add(bpt, BT[3 * j + i]));
    o.C[k] = Cm[3 * i + j];
  }
}
// abi_to_parent in double-float, in place on packed blocks: the rotation of
// every block (a planar rotation when `planar` ≥ 0), then the shift by t with
// B_p = B' + T C', A_p = A' − B_p T − (B' T)ᵀ, C_p = C' (T = [t]×).  Fewer live
// values than expanding the symmetric blocks to 3×3.
__device__ __forceinline__ void abi_to_parent_inplace(ABIF& I, const M3<float>& Rr, V3<float> t, int planar,
                                                      float co, float si) {
  if (planar >= 0) {
    sym_planar(I.A, planar, co, si);
    sym_planar(I.C, planar, co, si);
    planar_rows(I.B, planar, co, si);
    planar_cols(I.B, planar, co, si);
  } else {
    FF a6[6], c6[6], B[9];
    sym_rotate(Rr.a, I.A, a6);
    sym_rotate(Rr.a, I.C, c6);
    gen_rotate(Rr.a, I.B, B);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      I.A[k] = a6[k];
      I.C[k] = c6[k];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) I.B[k] = B[k];
  }
  FF BT[9];  // B' T
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    BT[3 * i] = ff_lin2(I.B[3 * i + 1], t.z, I.B[3 * i + 2], -t.y);
    BT[3 * i + 1] = ff_lin2(I.B[3 * i], -t.z, I.B[3 * i + 2], t.x);
    BT[3 * i + 2] = ff_lin2(I.B[3 * i], t.y, I.B[3 * i + 1], -t.x);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    I.B[j] = ff_add(I.B[j], ff_lin2(symget(I.C, 1, j), -t.z, symget(I.C, 2, j), t.y));
    I.B[3 + j] = ff_add(I.B[3 + j], ff_lin2(symget(I.C, 0, j), t.z, symget(I.C, 2, j), -t.x));
    I.B[6 + j] = ff_add(I.B[6 + j], ff_lin2(symget(I.C, 0, j), -t.y, symget(I.C, 1, j), t.x));
  }
  const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int i = ii[k], j = jj[k];
    const FF bpt = j == 0 ? ff_lin2(I.B[3 * i + 1], t.z, I.B[3 * i + 2], -t.y)
                          : (j == 1 ? ff_lin2(I.B[3 * i], -t.z, I.B[3 * i + 2], t.x)
                                    : ff_lin2(I.B[3 * i], t.y, I.B[3 * i + 1], -t.x));
    I.A[k] = ff_sub(I.A[k], ff_add(bpt, BT[3 * j + i]));
  }
}
// I·(w, v) in FP32 from the rounded entries (the bias-force update needs only FP32).
__device__ __forceinline__ SV<float> abi_mul_hi(const ABIF& I, const SV<float>& x) {
  const float w[3] = {x.w.x, x.w.y, x.w.z}, v[3] = {x.v.x, x.v.y, x.v.z};
  float A[6], B[9], C[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    A[k] = ff_f(I.A[k]);
    C[k] = ff_f(I.C[k]);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] = ff_f(I.B[k]);
  float ow[3], ov[3];
  const int s[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ow[i] = A[s[i][0]] * w[0] + A[s[i][1]] * w[1] + A[s[i][2]] * w[2] + B[3 * i] * v[0] + B[3 * i + 1] * v[1] +
            B[3 * i + 2] * v[2];
    ov[i] = B[i] * w[0] + B[3 + i] * w[1] + B[6 + i] * w[2] + C[s[i][0]] * v[0] + C[s[i][1]] * v[1] +
            C[s[i][2]] * v[2];
  }
  return {{ow[0], ow[1], ow[2]}, {ov[0], ov[1], ov[2]}};
}

// ---- double-float bias forces (GPB_MIXED) ----------------------------------
// The bias force p = v ×* I v of each body and the inward recursion
// p^a = p^A + I^a c + U D⁻¹ u, carried to the parent frame, run in
// double-float from the FP32 velocities and the FP32 model.  In FP32 their
// rounding (≈ 6e-8 of the body forces, summed along the tree) reaches q̈
// through u = τ − Sᵀ p^A, where much of p^A cancels: on 2–48-DOF chains it
// moved q̈ of 0.3 % of the instances by more than 1e-5 of |q̈| (up to 3e-5);
// in double-float the largest error is about 2e-6.  The velocities, the bias
// accelerations c and the product I^a c stay FP32 (they move q̈ by ≤ 1e-6).
struct SVF {
  FF w[3], v[3];
};
template <typename R>
__device__ __forceinline__ SVF load_svf(const LaneCtx<R>& c, int base) {
  SVF s;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s.w[k] = ffw(c, base + k);
    s.v[k] = ffw(c, base + 3 + k);
  }
  return s;
}
template <typename R>
__device__ __forceinline__ void store_svf(const LaneCtx<R>& c, int base, const SVF& s) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ffw(c, base + k) = s.w[k];
    ffw(c, base + 3 + k) = s.v[k];
  }
}
__device__ __forceinline__ SVF svf_add(const SVF& a, const SVF& b) {
  SVF s;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s.w[k] = ff_add(a.w[k], b.w[k]);
    s.v[k] = ff_add(a.v[k], b.v[k]);
  }
  return s;
}
__device__ __forceinline__ SVF svf_zero() {
  SVF s;
#pragma unroll
  for (int k = 0; k < 3; ++k) s.w[k] = s.v[k] = ff(0.0f);
  return s;
}
__device__ __forceinline__ SVF svf_from_double(const SV<double>& d) {
  return {{ff_from_double(d.w.x), ff_from_double(d.w.y), ff_from_double(d.w.z)},
          {ff_from_double(d.v.x), ff_from_double(d.v.y), ff_from_double(d.v.z)}};
}

// p = v ×* I v for the FP32 body velocity (w, vl) and the FP32 inertia (J about
// the origin in the order xx yy zz xy xz yz, cross part cm = m·com, mass m),
// written as p_w = w × (J w) + cm × (w × vl), p_v = m (w × vl) − w × (cm × w):
// the same vector as (w × f_w + vl × f_v, w × f_v) with f = I v, with every
// product of two FP32 inputs exact.
__device__ __forceinline__ SVF bias_force_ff(const float* J, V3<float> cm, float m, V3<float> w, V3<float> vl,
                                             bool diag) {
  const FF g[3] = {ff_det2(w.y, vl.z, w.z, vl.y), ff_det2(w.z, vl.x, w.x, vl.z), ff_det2(w.x, vl.y, w.y, vl.x)};
  FF h[3];  // J w
  if (diag) {
    h[0] = two_prod(J[0], w.x);
    h[1] = two_prod(J[1], w.y);
    h[2] = two_prod(J[2], w.z);
  } else {
    h[0] = ff_add_prod(J[4], w.z, ff_add_prod(J[3], w.y, two_prod(J[0], w.x)));
    h[1] = ff_add_prod(J[5], w.z, ff_add_prod(J[1], w.y, two_prod(J[3], w.x)));
    h[2] = ff_add_prod(J[2], w.z, ff_add_prod(J[5], w.y, two_prod(J[4], w.x)));
  }
  const FF k[3] = {ff_det2(cm.y, w.z, cm.z, w.y), ff_det2(cm.z, w.x, cm.x, w.z),
                   ff_det2(cm.x, w.y, cm.y, w.x)};  // cm × w
  SVF p;
  p.w[0] = ff_add(ff_lin2(h[2], w.y, h[1], -w.z), ff_lin2(g[2], cm.y, g[1], -cm.z));
  p.w[1] = ff_add(ff_lin2(h[0], w.z, h[2], -w.x), ff_lin2(g[0], cm.z, g[2], -cm.x));
  p.w[2] = ff_add(ff_lin2(h[1], w.x, h[0], -w.y), ff_lin2(g[1], cm.x, g[0], -cm.y));
  p.v[0] = ff_fmaf(k[1], w.z, ff_lin2(g[0], m, k[2], -w.y));
  p.v[1] = ff_fmaf(k[2], w.x, ff_lin2(g[1], m, k[0], -w.z));
  p.v[2] = ff_fmaf(k[0], w.y, ff_lin2(g[2], m, k[1], -w.x));
  return p;
}

// A spatial force in the child frame → the parent frame, (Rr n + t × Rr f, Rr f),
// in double-float with the FP32 transform: a rotation about principal axis
// `planar` ≥ 0 by (co, si) turns one pair of components, otherwise Rr.
__device__ __forceinline__ SVF force_to_parent_ff(const M3<float>& Rr, V3<float> t, const SVF& f, int planar,
                                                  float co, float si) {
  FF fw[3], fv[3];
  if (planar >= 0) {
    const int k = planar;
    FF x, y;
    rot2(pick3(k, f.w[1], f.w[2], f.w[0]), pick3(k, f.w[2], f.w[0], f.w[1]), co, si, x, y);
    fw[0] = pick3(k, f.w[0], y, x);
    fw[1] = pick3(k, x, f.w[1], y);
    fw[2] = pick3(k, y, x, f.w[2]);
    rot2(pick3(k, f.v[1], f.v[2], f.v[0]), pick3(k, f.v[2], f.v[0], f.v[1]), co, si, x, y);
    fv[0] = pick3(k, f.v[0], y, x);
    fv[1] = pick3(k, x, f.v[1], y);
    fv[2] = pick3(k, y, x, f.v[2]);
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      fw[i] = ff_dot3f(f.w[0], f.w[1], f.w[2], Rr.a[3 * i], Rr.a[3 * i + 1], Rr.a[3 * i + 2]);
      fv[i] = ff_dot3f(f.v[0], f.v[1], f.v[2], Rr.a[3 * i], Rr.a[3 * i + 1], Rr.a[3 * i + 2]);
    }
  }
  SVF o;
  o.w[0] = ff_add(fw[0], ff_lin2(fv[2], t.y, fv[1], -t.z));
  o.w[1] = ff_add(fw[1], ff_lin2(fv[0], t.z, fv[2], -t.x));
  o.w[2] = ff_add(fw[2], ff_lin2(fv[1], t.x, fv[0], -t.y));
#pragma unroll
  for (int k = 0; k < 3; ++k) o.v[k] = fv[k];
  return o;
}

// Bias acceleration c = v ×m (S q̇) of a body from its velocity (w, vl) (which
// includes S q̇) and its joint velocity, as in the outward pass.
template <typename R>
__device__ __forceinline__ SV<R> bias_acc(int type, V3<R> ax, Col<double> v, int vo, V3<R> w, V3<R> vl) {
  const V3<R> zero{R(0), R(0), R(0)};
  V3<R> jw = zero, jv = zero;
  if (type == 1) {
    jw = ax * R(v[vo]);
  } else if (type == 2) {
    jv = ax * R(v[vo]);
  } else if (type == 3) {
    jw = {R(v[vo]), R(v[vo + 1]), R(v[vo + 2])};
    jv = {R(v[vo + 3]), R(v[vo + 4]), R(v[vo + 5])};
  }
  return {cross(w, jw), cross(w, jv) + cross(vl, jw)};
}

// 6×6 Cholesky of a spatial inertia (packed lower triangle L[21], reciprocal
// diagonal) and the solve L Lᵀ x = b.  Returns false for a non-positive pivot.
__device__ __forceinline__ int l6(int i, int j) { return (i * (i + 1) >> 1) + j; }
__device__ __forceinline__ bool chol6(const ABI& I, double* L, double* dinv) {
  double M6[21];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      double x;
      if (i < 3) x = symget(I.A, i, j);
      else if (j < 3) x = I.B[3 * j + (i - 3)];  // block (v, ω) = Bᵀ
      else x = symget(I.C, i - 3, j - 3);
      M6[l6(i, j)] = x;
    }
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      double x = M6[l6(i, j)];
#pragma unroll
      for (int k = 0; k < j; ++k) x -= L[l6(i, k)] * L[l6(j, k)];
      if (i == j) {
        if (!(x > 0.0)) {
          ok = false;
          x = 1.0;
        }
        L[l6(i, i)] = sqrt(x);
        dinv[i] = 1.0 / L[l6(i, i)];
      } else {
        L[l6(i, j)] = x * dinv[j];
      }
    }
  }
  return ok;
}
__device__ __forceinline__ void solve6(const double* L, const double* dinv, double* x) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double s = x[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= L[l6(i, k)] * x[k];
    x[i] = s * dinv[i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double s = x[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) s -= L[l6(k, i)] * x[k];
    x[i] = s * dinv[i];
  }
}

// The same factor and solve in double-float (the mixed form's floating
// joints): each pivot's 1/√x by ff_rsqrt after renormalising x, whose sign
// the test reads from hi.
__device__ __forceinline__ bool chol6_ff(const ABIF& I, FF* L, FF* dinv) {
  FF M6[21];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      FF x;
      if (i < 3) x = symget(I.A, i, j);
      else if (j < 3) x = I.B[3 * j + (i - 3)];  // block (v, ω) = Bᵀ
      else x = symget(I.C, i - 3, j - 3);
      M6[l6(i, j)] = x;
    }
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      FF x = M6[l6(i, j)];
#pragma unroll
      for (int k = 0; k < j; ++k) x = ff_fms(x, L[l6(i, k)], L[l6(j, k)]);
      if (i == j) {
        x = two_sum(x.hi, x.lo);
        if (!(x.hi > 0.0f)) {
          ok = false;
          x = ff(1.0f);
        }
        dinv[i] = ff_rsqrt(x);
        L[l6(i, i)] = ff_mul(x, dinv[i]);
      } else {
        L[l6(i, j)] = ff_mul(x, dinv[j]);
      }
    }
  }
  return ok;
}
__device__ __forceinline__ void solve6_ff(const FF* L, const FF* dinv, FF* x) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    FF s = x[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s = ff_fms(s, L[l6(i, k)], x[k]);
    x[i] = ff_mul(s, dinv[i]);
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    FF s = x[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) s = ff_fms(s, L[l6(k, i)], x[k]);
    x[i] = ff_mul(s, dinv[i]);
  }
}

// Per-DOF record of the inward pass (DU region, 11 words per DOF):
//   1-DOF joint: U (6), 1/D, u
//   floating joint (its 6 DOF slots, 66 words): L (21), 1/diag (6), u (6) —
//   FP64 words in the FP64 form, FF words in the mixed form
constexpr int DU_D = 11;

// I·(w, v) in the sweep precision R (the bias-force update needs only R).
template <typename R>
__device__ __forceinline__ SV<R> abi_mul_r(const ABI& I, const SV<R>& x) {
  R A[6], B[9], C[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    A[k] = R(I.A[k]);
    C[k] = R(I.C[k]);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] = R(I.B[k]);
  const R w[3] = {x.w.x, x.w.y, x.w.z}, v[3] = {x.v.x, x.v.y, x.v.z};
  R ow[3], ov[3];
  const int s[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ow[i] = A[s[i][0]] * w[0] + A[s[i][1]] * w[1] + A[s[i][2]] * w[2] + B[3 * i] * v[0] + B[3 * i + 1] * v[1] +
            B[3 * i + 2] * v[2];
    ov[i] = B[i] * w[0] + B[3 + i] * w[1] + B[6 + i] * w[2] + C[s[i][0]] * v[0] + C[s[i][1]] * v[1] +
            C[s[i][2]] * v[2];
  }
  return {{ow[0], ow[1], ow[2]}, {ov[0], ov[1], ov[2]}};
}

// (Rrel, t) of body b in the sweep precision: the FP64 record in the I
// region, or (R = float) its FP32 copy in RF.  A planar rotation about e_k
// (planar = k ≥ 0) is stored as (cos, sin) and rebuilt exactly; in the mixed
// form its translation, the joint frame's own, is read from the FP32
// topology table instead of a record (3 fewer words written per body).
template <typename R>
__device__ __forceinline__ void load_xf(const LaneCtx<R>& c, int b, int planar, M3<R>& Rr, V3<R>& t) {
  const int base = sizeof(R) == 8 ? c.L.I + 12 * b : c.L.RF + 12 * b;
  auto at = [&](int e) -> R { return sizeof(R) == 8 ? R(c.d(base + e)) : c.r(base + e); };
  if (planar >= 0) {
    Rr = planar_rot<R>(planar, at(0), at(1));
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) Rr.a[k] = at(k);
  }
  if (sizeof(R) == 4 && planar >= 0) {  // a planar joint's translation is its joint frame's
    const int tb = TOPO_D * b + TD_TINIT;
    t = {R(c.t(tb)), R(c.t(tb + 1)), R(c.t(tb + 2))};
  } else {
    t = {at(9), at(10), at(11)};
  }
}
// planar axis index of body b's joint (−1: not a planar rotation).
__device__ __forceinline__ int planar_axis(int type, uint32_t fl) {
  return (type == 1 && (fl & BF_INIT_ROT_IDENTITY) && (fl & BF_AXIS_PRINCIPAL)) ? (int)bf_axis_index(fl) : -1;
}

template <typename R>
__device__ __forceinline__ SV<double> sv_d(const SV<R>& s) {
  return {{double(s.w.x), double(s.w.y), double(s.w.z)}, {double(s.v.x), double(s.v.y), double(s.v.z)}};
}
template <typename R>
__device__ __forceinline__ SV<R> sv_r(const SV<double>& s) {
  return {{R(s.w.x), R(s.w.y), R(s.w.z)}, {R(s.v.x), R(s.v.y), R(s.v.z)}};
}
// Row of a contact mechanism's FP64 bias-force record: in the FP64 form region
// F, its bias force p − f_contact; in the mixed form region FD, only the
// contact term −f_contact (FP64), since F holds the mixed form's double-float
// branch accumulators (and, whatever a lane writes there, every lane of the
// pack must use the same element width: an FP32 row fills the first half of
// the bytes of the FP64 row of the same index, the elements of lanes 0-15).
// A body that can carry a contact wrench: contact points (count in bits 16-23
// of topology word 1) or a cuboid collider (slot in bits 24-27).
__device__ __forceinline__ bool has_wrench(uint32_t w1) {
  return ((w1 >> 16) & 255u) != 0 || ((w1 >> W1_CUBOID_SHIFT) & 15u) != 0;
}
template <typename R>
__device__ __forceinline__ int fd_row(const LaneCtx<R>& c) {
  return sizeof(R) == 8 ? c.L.F : c.L.FD;
}
template <typename R>
__device__ __forceinline__ SV<double> load_svd(const LaneCtx<R>& c, int base) {
  return {{c.d(base), c.d(base + 1), c.d(base + 2)}, {c.d(base + 3), c.d(base + 4), c.d(base + 5)}};
}
template <typename R>
__device__ __forceinline__ void store_svd(const LaneCtx<R>& c, int base, const SV<double>& s) {
  c.d(base) = s.w.x;
  c.d(base + 1) = s.w.y;
  c.d(base + 2) = s.w.z;
  c.d(base + 3) = s.v.x;
  c.d(base + 4) = s.v.y;
  c.d(base + 5) = s.v.z;
}

// ---- mechanism kinds with their own instantiation of the passes ------------
// KIND_GENERAL: any tree.  KIND_PLANAR_CHAIN: revolute joints about ±x/±y/±z
// with identity joint rotations, each body the child of the previous one, no
// contacts, colliders or springs.  KIND_FLOATING_TREE: a floating root and
// revolute joints about ±x/±y/±z below it, identity joint rotations, any tree,
// point / sphere contacts, no colliders or springs.  Joint type, parent (for a
// chain), axis kind and the absent cases are then constants: their code drops
// out of the loops, which shrinks the instruction stream the passes fetch.
constexpr int KIND_GENERAL = 0, KIND_PLANAR_CHAIN = 1, KIND_FLOATING_TREE = 2;
template <int KIND>
__device__ __forceinline__ int kind_type(uint32_t w0, int b) {
  return KIND == KIND_PLANAR_CHAIN ? 1 : (KIND == KIND_FLOATING_TREE ? (b == 0 ? 3 : 1) : (int)(w0 & 15));
}
template <int KIND>
__device__ __forceinline__ int kind_parent(uint32_t w0, int b) {
  return KIND == KIND_PLANAR_CHAIN ? b : (int)((w0 >> 4) & 255);
}
// flags: a planar chain has no branch bodies; both special kinds have identity
// joint rotations
template <int KIND>
__device__ __forceinline__ uint32_t kind_flags(uint32_t w1) {
  const uint32_t f = w1 & 255;
  if (KIND == KIND_PLANAR_CHAIN) return (f & ~(uint32_t)BF_BRANCH) | BF_INIT_ROT_IDENTITY;
  if (KIND == KIND_FLOATING_TREE) return f | BF_INIT_ROT_IDENTITY;
  return f;
}
// principal axis index of a planar joint, −1 for any other joint
template <int KIND>
__device__ __forceinline__ int kind_planar(int type, uint32_t fl, int b) {
  if (KIND == KIND_PLANAR_CHAIN) return (int)bf_axis_index(fl);
  if (KIND == KIND_FLOATING_TREE) return b == 0 ? -1 : (int)bf_axis_index(fl);
  return planar_axis(type, fl);
}

// Pass 2 of the mixed form: articulated inertias, U, D and the congruence to
// the parent in double-float, from the FP32 model and the FP32 transforms of
// pass 1; each body's bias force p = v ×* I v (from its FP32 velocity, plus
// the FP64 contact wrench of a contact mechanism) and the bias-force
// recursion in double-float; the bias acceleration c and I^a c in FP32.  A
// 1-DOF joint's DU record holds FF words (U, 1/D, u); a floating joint's holds
// the FP64 record of the FP64 form.
template <typename R, int KIND>
__device__ __forceinline__ int aba_inward_ff(const LaneCtx<R>& c, Col<double> q, Col<double> v, Col<double> tau,
                                             bool have_tau, bool contacts) {
  using V = V3<R>;
  int st = 0;
  ABIF carryI{};
  SVF carryP = svf_zero();
  int ctarget = -1;
  for (int b = c.nb - 1; b >= 0; --b) {
    const uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    const uint32_t fl = kind_flags<KIND>(w1);
    const int type = kind_type<KIND>(w0, b), parent = kind_parent<KIND>(w0, b);
    const int qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    const int tb = TOPO_D * b;
    const V ax{c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
    // bias terms from the body velocity of pass 1
    const SV<R> vb = load_sv(c, c.L.V + 6 * b);
    const SV<R> cb = bias_acc(type, ax, v, vo, vb.w, vb.v);
    SVF pA;
    {
      float J[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) J[k] = c.t(tb + TD_INERTIA + 4 + k);
      const V cm{c.t(tb + TD_INERTIA + 1), c.t(tb + TD_INERTIA + 2), c.t(tb + TD_INERTIA + 3)};
      pA = bias_force_ff(J, cm, c.t(tb + TD_INERTIA), vb.w, vb.v, (fl & BF_DIAG_INERTIA) != 0);
    }
    if (contacts && has_wrench(w1))  // − contact wrench (bodies with points or a cuboid collider)
      pA = svf_add(pA, svf_from_double(load_svd(c, fd_row(c) + 6 * b)));
    ABIF IA = body_abi_ff(c, tb);
    if (fl & BF_BRANCH) {
      abi_add(IA, load_abi_ff(c, c.L.AI + ABI_D * b));
      pA = svf_add(pA, load_svf(c, c.L.F + 6 * b));
    }
    if (ctarget == b) {
      abi_add(IA, carryI);
      pA = svf_add(pA, carryP);
    }
    SVF pa;
    const bool to_parent = parent != 0;
    const int planar = kind_planar<KIND>(type, fl, b);
    if (type == 1 || type == 2) {
      FF Uw[3], Uv[3], D;
      if (type == 1 && (KIND != KIND_GENERAL || (fl & BF_AXIS_PRINCIPAL))) {  // a = ±e_k: U = ±(A[:,k], row k of B), D = A_kk
        const int k = (int)bf_axis_index(fl);
        Uw[0] = pick3(k, IA.A[0], IA.A[3], IA.A[4]);
        Uw[1] = pick3(k, IA.A[3], IA.A[1], IA.A[5]);
        Uw[2] = pick3(k, IA.A[4], IA.A[5], IA.A[2]);
#pragma unroll
        for (int i = 0; i < 3; ++i) Uv[i] = pick3(k, IA.B[i], IA.B[3 + i], IA.B[6 + i]);
        if (fl & BF_AXIS_NEG) {
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            Uw[i] = ff_neg(Uw[i]);
            Uv[i] = ff_neg(Uv[i]);
          }
        }
        D = pick3(k, IA.A[0], IA.A[1], IA.A[2]);
      } else if (type == 1) {  // U = I (a, 0) = (A a, Bᵀ a)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Uw[i] = ff_dot3f(symget(IA.A, i, 0), symget(IA.A, i, 1), symget(IA.A, i, 2), ax.x, ax.y, ax.z);
          Uv[i] = ff_dot3f(IA.B[i], IA.B[3 + i], IA.B[6 + i], ax.x, ax.y, ax.z);
        }
        D = ff_dot3f(Uw[0], Uw[1], Uw[2], ax.x, ax.y, ax.z);
      } else {  // U = I (0, a) = (B a, C a)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Uw[i] = ff_dot3f(IA.B[3 * i], IA.B[3 * i + 1], IA.B[3 * i + 2], ax.x, ax.y, ax.z);
          Uv[i] = ff_dot3f(symget(IA.C, i, 0), symget(IA.C, i, 1), symget(IA.C, i, 2), ax.x, ax.y, ax.z);
        }
        D = ff_dot3f(Uv[0], Uv[1], Uv[2], ax.x, ax.y, ax.z);
      }
      // u = τ + τ_spring − Sᵀ p^A (the torque in FP64, split; Sᵀ p^A in double-float)
      double tt = have_tau ? tau[vo] : 0.0;
      if (KIND == KIND_GENERAL && type == 2 && (w1 & BF_SPRING) && c.springs)
        tt += -c.td(tb + TD_SPRING) * (q[qo] - c.td(tb + TD_SPRING + 1));
      const FF sp = type == 1 ? ff_dot3f(pA.w[0], pA.w[1], pA.w[2], ax.x, ax.y, ax.z)
                              : ff_dot3f(pA.v[0], pA.v[1], pA.v[2], ax.x, ax.y, ax.z);
      const FF uf = ff_sub(ff_from_double(tt), sp);
      if (type == 1 && c.armature) {  // free_velocity: revolute armature (src/hybrid/articulated/mod.rs:244-247)
        const float arm = c.t(tb + TD_ARMATURE);
        if (arm != 0.0f) D = ff_add(D, ff(arm));
      }
      D = two_sum(D.hi, D.lo);  // ff_rcp starts from D.hi
      if (!(D.hi > 0.0f)) st |= 2;  // GPB_ST_CHOL_FAIL
      const FF Dinv = ff_rcp(D);
      const int du = c.L.DU + DU_D * vo;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        ffw(c, du + i) = Uw[i];
        ffw(c, du + 3 + i) = Uv[i];
      }
      ffw(c, du + 6) = Dinv;
      ffw(c, du + 7) = uf;
      if (to_parent) {
        // I^a = I^A − U D⁻¹ Uᵀ ; p^a = p^A + I^a c + U D⁻¹ u
        FF Ww[3], Wv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          Ww[i] = ff_mul(Uw[i], Dinv);
          Wv[i] = ff_mul(Uv[i], Dinv);
        }
        const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          IA.A[k] = ff_fms(IA.A[k], Ww[ii[k]], Uw[jj[k]]);
          IA.C[k] = ff_fms(IA.C[k], Wv[ii[k]], Uv[jj[k]]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) IA.B[3 * i + j] = ff_fms(IA.B[3 * i + j], Ww[i], Uv[j]);
        const FF ud = ff_mul(uf, Dinv);
        const SV<R> iac = abi_mul_hi(IA, cb);
        const R iw[3] = {iac.w.x, iac.w.y, iac.w.z}, iv[3] = {iac.v.x, iac.v.y, iac.v.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          pa.w[i] = ff_add(pA.w[i], ff_fma(Uw[i], ud, ff(iw[i])));
          pa.v[i] = ff_add(pA.v[i], ff_fma(Uv[i], ud, ff(iv[i])));
        }
      }
    } else if (type == 3) {  // floating joint: the 6×6 factor of the FP64 form, in double-float
      FF L[21], dinv[6];
      if (!chol6_ff(IA, L, dinv)) st |= 2;
      const int du = c.L.DU + DU_D * vo;
#pragma unroll
      for (int k = 0; k < 21; ++k) ffw(c, du + k) = L[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) ffw(c, du + 21 + k) = dinv[k];
      const FF p6[6] = {pA.w[0], pA.w[1], pA.w[2], pA.v[0], pA.v[1], pA.v[2]};
      FF pa6[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const FF u = have_tau ? ff_sub(ff_from_double(tau[vo + k]), p6[k]) : ff_neg(p6[k]);
        ffw(c, du + 27 + k) = u;
        pa6[k] = ff_add(p6[k], u);  // floating joint: I^a = 0, p^a = p^A + u
      }
      pa = {{pa6[0], pa6[1], pa6[2]}, {pa6[3], pa6[4], pa6[5]}};
    } else {  // fixed joint: I^a = I^A, p^a = p^A + I^A c
      const SV<R> iac = abi_mul_hi(IA, cb);
      const R iw[3] = {iac.w.x, iac.w.y, iac.w.z}, iv[3] = {iac.v.x, iac.v.y, iac.v.z};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        pa.w[i] = ff_addf(pA.w[i], iw[i]);
        pa.v[i] = ff_addf(pA.v[i], iv[i]);
      }
    }
    if (to_parent) {
      const int pb = parent - 1;
      M3<R> RrR;
      V tr;
      load_xf(c, b, planar, RrR, tr);
      const R co = planar >= 0 ? c.r(c.L.RF + 12 * b) : R(1);
      const R si = planar >= 0 ? c.r(c.L.RF + 12 * b + 1) : R(0);
      // the bias force first: p^a is dead before the congruence's temporaries live
      const SVF fp = force_to_parent_ff(RrR, tr, pa, planar, co, si);
      if (pb == b - 1) {
        carryP = fp;
      } else {
        store_svf(c, c.L.F + 6 * pb, svf_add(load_svf(c, c.L.F + 6 * pb), fp));
        carryP = svf_zero();
      }
      if (type != 3) {
        abi_to_parent_inplace(IA, RrR, tr, planar, co, si);
        if (pb == b - 1) {
          carryI = IA;
        } else {
          ABIF acc = load_abi_ff(c, c.L.AI + ABI_D * pb);
          abi_add(acc, IA);
          store_abi_ff(c, c.L.AI + ABI_D * pb, acc);
          carryI = ABIF{};
        }
      } else {
        carryI = ABIF{};  // floating joint: I^a = 0
      }
      ctarget = pb == b - 1 ? pb : -1;
    } else {
      // every path writes both carries, so their previous values are dead once
      // read at the top of the iteration (not held in registers through it)
      carryI = ABIF{};
      carryP = svf_zero();
      ctarget = -1;
    }
  }
  return st;
}

// One dynamics evaluation by the articulated-body algorithm.  q̈ into qdd;
// GPB status bits (CHOL_FAIL for a non-positive articulated inertia D).
template <typename R, int KIND>
__device__ __noinline__ int lane_aba(const LaneCtx<R>& cin, Col<double> q, Col<double> v, Col<double> tau,
                                     bool have_tau, Col<double> qdd, Col<double> cf, bool want_cf) {
  const LaneCtx<R> c = cin;  // private copy: stores through scratch pointers cannot alias it
  using V = V3<R>;
  using VD = V3<double>;
  // world poses in FP64 (points or cuboid pairs)
  const bool contacts = KIND == KIND_PLANAR_CHAIN ? false
                        : (KIND == KIND_FLOATING_TREE ? c.nc > 0 : (c.nc > 0 || c.nu > 1));
  const bool wide = contacts || sizeof(R) == 8;  // FP64 joint transforms
  const V zero{R(0), R(0), R(0)};
  V pw_ = zero, pv_ = zero;                  // parent velocity (chain carry)
  // The mixed form of a contact mechanism propagates its body velocities in
  // FP64: the regularised friction divides the contact point's tangential
  // velocity by 1e-3, so an FP32 velocity recursion (errors ~1e-7 of the body
  // speeds along a leg) would become a ~1e-4 error in the friction force.
  const bool dvel = sizeof(R) == 4 && contacts;
  VD pwd_{0.0, 0.0, 0.0}, pvd_{0.0, 0.0, 0.0};  // its FP64 chain carry
  VD ppos{0.0, 0.0, 0.0};
  M3<double> pR = eye3<double>();            // parent world pose (contacts only)
  int st = 0;
  // ---- pass 1 (outward): transforms, velocities, bias terms, contacts ------
  for (int b = 0; b < c.nb; ++b) {
    const uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
    const int type = kind_type<KIND>(w0, b), parent = kind_parent<KIND>(w0, b);
    const int qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
    const uint32_t fl = kind_flags<KIND>(w1);
    V om = zero, vl = zero;
    VD omd{0.0, 0.0, 0.0}, vld{0.0, 0.0, 0.0};
    VD posw{0.0, 0.0, 0.0};
    M3<double> Rw = eye3<double>();
    if (parent == b && parent != 0) {
      om = pw_;
      vl = pv_;
      omd = pwd_;
      vld = pvd_;
      posw = ppos;
      Rw = pR;
    } else if (parent != 0) {
      const int pb = parent - 1;
      om = {c.r(c.L.V + 6 * pb), c.r(c.L.V + 6 * pb + 1), c.r(c.L.V + 6 * pb + 2)};
      vl = {c.r(c.L.V + 6 * pb + 3), c.r(c.L.V + 6 * pb + 4), c.r(c.L.V + 6 * pb + 5)};
      if (dvel) {
        omd = {c.d(c.L.VW + 6 * pb), c.d(c.L.VW + 6 * pb + 1), c.d(c.L.VW + 6 * pb + 2)};
        vld = {c.d(c.L.VW + 6 * pb + 3), c.d(c.L.VW + 6 * pb + 4), c.d(c.L.VW + 6 * pb + 5)};
      }
      if (contacts) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Rw.a[k] = c.d(c.L.X + 12 * pb + k);
        posw = {c.d(c.L.X + 12 * pb + 9), c.d(c.L.X + 12 * pb + 10), c.d(c.L.X + 12 * pb + 11)};
      }
    }
    // child → parent transform (Rr, t): FP64 record Rd / td; Rr, t in R
    const int tb = TOPO_D * b;
    const bool rid = (fl & BF_INIT_ROT_IDENTITY) != 0;
    const bool planar = kind_planar<KIND>(type, fl, b) >= 0 && rid;
    M3<double> Rd = eye3<double>();
    VD td{c.td(tb + TD_TINIT), c.td(tb + TD_TINIT + 1), c.td(tb + TD_TINIT + 2)};
    M3<R> Rr;
    double pco = 1.0, psi = 0.0;  // (cos, sin) of a planar joint, FP64 and in R
    R rco = R(1), rsi = R(0);
    if (planar) {  // rotation about ±e_k: only the (k+1, k+2) plane turns
      const int k = (int)bf_axis_index(fl);
      double co, si;
      R cor, sir;
      if (wide) {
        sincos(q[qo], &si, &co);
        cor = R(co);
        sir = R(si);
      } else {
        float sf, cfl;
        sincos_q<float>(q[qo], &sf, &cfl);
        cor = R(cfl);
        sir = R(sf);
        co = cfl;
        si = sf;
      }
      if (fl & BF_AXIS_NEG) {
        si = -si;
        sir = -sir;
      }
      Rd = planar_rot<double>(k, co, si);
      Rr = planar_rot<R>(k, cor, sir);
      pco = co;
      psi = si;
      rco = cor;
      rsi = sir;
    } else {
      M3<double> Rid = eye3<double>();
      if (!rid) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Rid.a[k] = c.td(tb + TD_RINIT + k);
      }
      VD axd{0.0, 0.0, 0.0};
      if (type == 1 || type == 2) axd = {c.td(tb + TD_AXIS), c.td(tb + TD_AXIS + 1), c.td(tb + TD_AXIS + 2)};
      if (type == 1) {
        double co, si;
        if (wide) {
          sincos(q[qo], &si, &co);
        } else {
          float sf, cfl;
          sincos_q<float>(q[qo], &sf, &cfl);
          si = sf;
          co = cfl;
        }
        const double omc = 1.0 - co;  // Rot(a, q) = c 1 + s [a]× + (1 − c) a aᵀ
        M3<double> Ro;
        Ro.a[0] = co + axd.x * axd.x * omc;
        Ro.a[1] = axd.x * axd.y * omc - axd.z * si;
        Ro.a[2] = axd.x * axd.z * omc + axd.y * si;
        Ro.a[3] = axd.y * axd.x * omc + axd.z * si;
        Ro.a[4] = co + axd.y * axd.y * omc;
        Ro.a[5] = axd.y * axd.z * omc - axd.x * si;
        Ro.a[6] = axd.z * axd.x * omc - axd.y * si;
        Ro.a[7] = axd.z * axd.y * omc + axd.x * si;
        Ro.a[8] = co + axd.z * axd.z * omc;
        Rd = rid ? Ro : mul(Rid, Ro);
      } else if (type == 2) {
        Rd = Rid;
        td = td + mul(Rid, axd * q[qo]);
      } else if (type == 3) {
        const M3<double> Rq = quat_to_mat<double>(q[qo], q[qo + 1], q[qo + 2], q[qo + 3]);
        const VD tq{q[qo + 4], q[qo + 5], q[qo + 6]};
        Rd = rid ? Rq : mul(Rid, Rq);
        td = td + mul(Rid, tq);
      } else {
        Rd = Rid;
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) Rr.a[k] = R(Rd.a[k]);
    }
    const V t{R(td.x), R(td.y), R(td.z)};
    // velocity: v = X v_p + S q̇ ; bias acceleration c = v ×m (S q̇)
    V jw = zero, jv = zero;
    if (dvel) {  // FP64 recursion, rounded for the FP32 bias terms
      if (parent != 0) {  // a body on the world starts from rest
        vld = mulT(Rd, vld + cross(omd, td));
        omd = mulT(Rd, omd);
      }
      VD jwd{0.0, 0.0, 0.0}, jvd{0.0, 0.0, 0.0};
      if (type == 1 || type == 2) {
        const VD axd{c.td(tb + TD_AXIS), c.td(tb + TD_AXIS + 1), c.td(tb + TD_AXIS + 2)};
        if (type == 1) jwd = axd * v[vo];
        else jvd = axd * v[vo];
      } else if (type == 3) {
        jwd = {v[vo], v[vo + 1], v[vo + 2]};
        jvd = {v[vo + 3], v[vo + 4], v[vo + 5]};
      }
      omd = omd + jwd;
      vld = vld + jvd;
      om = {R(omd.x), R(omd.y), R(omd.z)};
      vl = {R(vld.x), R(vld.y), R(vld.z)};
      jw = {R(jwd.x), R(jwd.y), R(jwd.z)};
      jv = {R(jvd.x), R(jvd.y), R(jvd.z)};
    } else {
      if (!(contacts && parent == 0)) {
        vl = mulT(Rr, vl + cross(om, t));
        om = mulT(Rr, om);
      }
      if (type == 1 || type == 2) {
        const V ax{c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
        if (type == 1) jw = ax * R(v[vo]);
        else jv = ax * R(v[vo]);
      } else if (type == 3) {
        jw = {R(v[vo]), R(v[vo + 1]), R(v[vo + 2])};
        jv = {R(v[vo + 3]), R(v[vo + 4]), R(v[vo + 5])};
      }
      om = om + jw;
      vl = vl + jv;
    }
    const SV<R> vb{om, vl};
    // bias acceleration c and bias force p = v ×* I v − f_contact (body frame);
    // the mixed form forms both in pass 2 from the stored velocity
    SV<R> cb, p;
    if constexpr (sizeof(R) == 8) {
      cb = {cross(om, jw), cross(om, jv) + cross(vl, jw)};
      SI<R> I;
#pragma unroll
      for (int k = 0; k < 6; ++k) I.j[k] = c.t(tb + TD_INERTIA + 4 + k);
      I.c = {c.t(tb + TD_INERTIA + 1), c.t(tb + TD_INERTIA + 2), c.t(tb + TD_INERTIA + 3)};
      I.m = c.t(tb + TD_INERTIA);
      p = crf(vb, imul(I, vb));
    }
    // contact wrench (body frame), FP64: stiff contacts make it the largest term
    // of the bias force, and the root's u = τ − p^A reads it directly
    SV<double> wc{{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    if (contacts) {
      if (parent == 0) {  // a body on the world: its joint transform is its world pose
        posw = td;
        Rw = Rd;
      } else {
        posw = posw + mul(Rw, td);
        Rw = mul(Rw, Rd);
      }
      const int cb0 = (w1 >> 8) & 255, cn = (w1 >> 16) & 255;
      if (cn) {
        // Poses and penetrations in FP64 (a penetration is a small difference
        // of O(1) positions, and k·δ becomes force), and so are the
        // contact-point velocity v + ω × r (it cancels for rolling or sticking
        // contacts) and its split into the approach speed ż = −v·n and the
        // tangential part v_t = v + n ż (which cancels for normal impacts, and
        // which the regularised friction divides by 1e-3).  The FP64 form
        // runs the force law and the wrench in FP64 too; the mixed form runs
        // them in FP32 from those FP64 differences (the law depends only on z,
        // ż and v_t), in the body frame.
        M3<R> RwR;
#pragma unroll
        for (int k = 0; k < 9; ++k) RwR.a[k] = R(Rw.a[k]);
        V ww = zero, wv = zero;  // the mixed form's wrench
        // the mixed form forms the first half-space's normal in the body frame
        // and the body origin's signed distance once per body: a point's
        // penetration is then one dot product
        VD nb0{0.0, 0.0, 0.0};
        double d00 = 0.0;
        if (sizeof(R) == 4 && c.nh > 0) {
          const VD hn0{c.hdd(3), c.hdd(4), c.hdd(5)};
          nb0 = mulT(Rw, hn0);
          d00 = dot(posw - VD{c.hdd(0), c.hdd(1), c.hdd(2)}, hn0);
        }
        for (int k = cb0; k < cb0 + cn; ++k) {
          const int cd = CTC_D * k;
          const VD locd{c.cdd(cd), c.cdd(cd + 1), c.cdd(cd + 2)};
          const V loc{c.CD[(size_t)cd * LANES], c.CD[(size_t)(cd + 1) * LANES], c.CD[(size_t)(cd + 2) * LANES]};
          const R kp = c.CD[(size_t)(cd + 3) * LANES], rad = c.CD[(size_t)(cd + 4) * LANES],
                  damp = c.CD[(size_t)(cd + 5) * LANES];
          const double radd = c.cdd(cd + 4);
          const VD pwc = sizeof(R) == 8 ? mul(Rw, locd) + posw : VD{0.0, 0.0, 0.0};
          V fsum = zero;
          for (int h = 0; h < c.nh; ++h) {
            const int hd = HS_D * h;
            const VD hp{c.hdd(hd), c.hdd(hd + 1), c.hdd(hd + 2)};
            const VD hnd{c.hdd(hd + 3), c.hdd(hd + 4), c.hdd(hd + 5)};
            const bool first = sizeof(R) == 4 && h == 0;
            const double dist = first ? d00 + dot(nb0, locd)
                                      : dot((sizeof(R) == 8 ? pwc : mul(Rw, locd) + posw) - hp, hnd);
            double pen;
            if (radd > 0.0) {
              if (!(dist - radd <= 1e-8)) continue;
              pen = radd - dist;
            } else {
              if (!(dist <= 1e-8)) continue;  // HalfSpace::has_inside (margin 1e-8)
              pen = -dist;
            }
            const double alh = c.hdd(hd + 6), mu = c.hdd(hd + 7);
            const VD nbd = first ? nb0 : mulT(Rw, hnd);  // normal in the body frame
            const V nb{R(nbd.x), R(nbd.y), R(nbd.z)};
            const V app = rad > R(0) ? loc - nb * rad : loc;  // application point (body frame)
            const VD appd = radd > 0.0 ? locd - nbd * radd : locd;
            // a floating root's body velocity is the state itself: read it
            // unrounded; the mixed form's other bodies carry FP64 velocities
            const bool root6 = type == 3 && parent == 0;
            const VD vlc = root6 ? VD{v[vo + 3], v[vo + 4], v[vo + 5]}
                                 : (dvel ? vld : VD{double(vl.x), double(vl.y), double(vl.z)});
            const VD omc = root6 ? VD{v[vo], v[vo + 1], v[vo + 2]}
                                 : (dvel ? omd : VD{double(om.x), double(om.y), double(om.z)});
            const VD vd = vlc + cross(omc, appd);
            V fb;
            if (sizeof(R) == 4) {
              const double zd = -dot(vd, nbd);
              const VD vtd = vd + nbd * zd;
              fb = contact_force_parts<R>(c.model, R(pen), R(zd), nb, V{R(vtd.x), R(vtd.y), R(vtd.z)}, kp, damp,
                                          R(alh), R(mu));
              ww = ww - cross(app, fb);
              wv = wv - fb;
            } else {
              const VD fbd = contact_force<double>(c.model, pen, nbd, vd, c.cdd(cd + 3), c.cdd(cd + 5), alh, mu);
              fb = V{R(fbd.x), R(fbd.y), R(fbd.z)};
              wc.w = wc.w - cross(appd, fbd);
              wc.v = wc.v - fbd;
            }
            fsum = fsum + fb;
          }
          if (want_cf) {
            const V fw = mul(RwR, fsum);
            const int orig = (c.CI[(size_t)k * LANES] >> 8) & 255;
            cf[3 * orig] = double(fw.x);
            cf[3 * orig + 1] = double(fw.y);
            cf[3 * orig + 2] = double(fw.z);
          }
        }
        if (sizeof(R) == 4) wc = {{double(ww.x), double(ww.y), double(ww.z)}, {double(wv.x), double(wv.y), double(wv.z)}};
      }
      const int uslot = (int)((w1 >> W1_CUBOID_SHIFT) & 15u);
      if (uslot && c.nu > 1) {  // cuboid record: world pose, world twist about the origin
        const bool root6 = type == 3 && parent == 0;
        const VD omc = root6 ? VD{v[vo], v[vo + 1], v[vo + 2]}
                             : (dvel ? omd : VD{double(om.x), double(om.y), double(om.z)});
        const VD vlc = root6 ? VD{v[vo + 3], v[vo + 4], v[vo + 5]}
                             : (dvel ? vld : VD{double(vl.x), double(vl.y), double(vl.z)});
        const VD omw = mul(Rw, omc);
        store_cuboid(c, uslot - 1, b, Rw, posw, omw, mul(Rw, vlc) - cross(omw, posw));
      }
    }
    // records for the inward and second outward passes: (Rrel, t) in R (the
    // FP64 form's FP64 record; the mixed form's FP32 record, which its
    // double-float inward pass reads too); a planar rotation keeps only its
    // (cos, sin) — the other entries are 0 and 1 — so the passes that read it
    // back touch 5 rows instead of 12
    if (sizeof(R) == 8) {
      if (planar) {
        c.d(c.L.I + 12 * b) = pco;
        c.d(c.L.I + 12 * b + 1) = psi;
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) c.d(c.L.I + 12 * b + k) = Rd.a[k];
      }
      c.d(c.L.I + 12 * b + 9) = td.x;
      c.d(c.L.I + 12 * b + 10) = td.y;
      c.d(c.L.I + 12 * b + 11) = td.z;
    } else {
      if (planar) {
        c.r(c.L.RF + 12 * b) = rco;
        c.r(c.L.RF + 12 * b + 1) = rsi;
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) c.r(c.L.RF + 12 * b + k) = Rr.a[k];
        c.r(c.L.RF + 12 * b + 9) = t.x;
        c.r(c.L.RF + 12 * b + 10) = t.y;
        c.r(c.L.RF + 12 * b + 11) = t.z;
      }
    }
    if constexpr (sizeof(R) == 8) {
      store_sv(c, c.L.A + 6 * b, cb);
      if (contacts) store_svd(c, fd_row(c) + 6 * b, sv_d(p) + wc);  // bias forces of contact mechanisms: FP64
      else store_sv(c, c.L.F + 6 * b, p);
    } else {
      store_sv(c, c.L.V + 6 * b, vb);  // passes 2 and 3 form c and p from it
      if (contacts && has_wrench(w1)) store_svd(c, fd_row(c) + 6 * b, wc);
    }
    if (fl & BF_BRANCH) {
      // accumulators for children other than b+1
      if (sizeof(R) == 8) {
        store_abi(c, c.L.AI + ABI_D * b, ABI{});
        store_sv(c, c.L.V + 6 * b, vb);
      } else {
        store_abi_ff(c, c.L.AI + ABI_D * b, ABIF{});
        store_svf(c, c.L.F + 6 * b, svf_zero());
      }
      if (dvel) store_svd(c, c.L.VW + 6 * b, SV<double>{omd, vld});
      if (contacts) {
#pragma unroll
        for (int k = 0; k < 9; ++k) c.d(c.L.X + 12 * b + k) = Rw.a[k];
        c.d(c.L.X + 12 * b + 9) = posw.x;
        c.d(c.L.X + 12 * b + 10) = posw.y;
        c.d(c.L.X + 12 * b + 11) = posw.z;
      }
    }
    pw_ = om;
    pv_ = vl;
    pwd_ = omd;
    pvd_ = vld;
    ppos = posw;
    pR = Rw;
  }
  // ---- cuboid pairs: p −= W (body frame, FP64 records of contact mechanisms)
  if (KIND == KIND_GENERAL && c.nu > 1) {
    st |= lane_cuboid_pairs(c);
    for (int b = 0; b < c.nb; ++b) {
      const int uslot = (int)((c.w(2 * b + 1) >> W1_CUBOID_SHIFT) & 15u);
      if (uslot) store_svd(c, fd_row(c) + 6 * b, load_svd(c, fd_row(c) + 6 * b) - cuboid_wrench_body(c, uslot - 1));
    }
  }
  // ---- pass 2 (inward): articulated inertias and bias forces --------------
  // A child that is the next body (every link of a chain) hands its terms to
  // the parent in registers; other children accumulate into the parent's slot.
  if constexpr (sizeof(R) == 4) {
    st |= aba_inward_ff<R, KIND>(c, q, v, tau, have_tau, contacts);
  } else {
    ABI carryI{};
    SV<R> carryP{zero, zero};
    int ctarget = -1;
    for (int b = c.nb - 1; b >= 0; --b) {
      const uint32_t w0 = c.w(2 * b), w1 = c.w(2 * b + 1);
      const uint32_t fl = kind_flags<KIND>(w1);
      const int type = kind_type<KIND>(w0, b), parent = kind_parent<KIND>(w0, b);
      const int qo = (w0 >> 12) & 1023, vo = (w0 >> 22) & 1023;
      const int tb = TOPO_D * b;
      ABI IA = body_abi(c, tb);
      SV<double> pAd;  // FP64 copy (contact mechanisms) for u
      SV<R> pA;
      if (contacts) {
        pAd = load_svd(c, fd_row(c) + 6 * b);
        if (ctarget == b) pAd = pAd + sv_d(carryP);
        pA = sv_r<R>(pAd);
      } else {
        pA = load_sv(c, c.L.F + 6 * b);
        if (ctarget == b) pA = pA + carryP;
      }
      if (fl & BF_BRANCH) abi_add(IA, load_abi(c, c.L.AI + ABI_D * b));
      if (ctarget == b) abi_add(IA, carryI);
      const SV<R> cb = load_sv(c, c.L.A + 6 * b);
      SV<R> pa;  // bias force handed to the parent
      const bool to_parent = parent != 0;
      if (type == 1 || type == 2) {
        double Uw[3], Uv[3], D;
        if (type == 1 && (KIND != KIND_GENERAL || (fl & BF_AXIS_PRINCIPAL))) {  // a = ±e_k: U = ±(A[:,k], row k of B), D = A_kk
          const int k = (int)bf_axis_index(fl);
          Uw[0] = pick3(k, IA.A[0], IA.A[3], IA.A[4]);
          Uw[1] = pick3(k, IA.A[3], IA.A[1], IA.A[5]);
          Uw[2] = pick3(k, IA.A[4], IA.A[5], IA.A[2]);
#pragma unroll
          for (int i = 0; i < 3; ++i) Uv[i] = pick3(k, IA.B[i], IA.B[3 + i], IA.B[6 + i]);
          if (fl & BF_AXIS_NEG) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              Uw[i] = -Uw[i];
              Uv[i] = -Uv[i];
            }
          }
          D = pick3(k, IA.A[0], IA.A[1], IA.A[2]);
        } else {
          const double ax[3] = {c.td(tb + TD_AXIS), c.td(tb + TD_AXIS + 1), c.td(tb + TD_AXIS + 2)};
          if (type == 1) {  // U = I (a, 0) = (A a, Bᵀ a)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              Uw[i] = symget(IA.A, i, 0) * ax[0] + symget(IA.A, i, 1) * ax[1] + symget(IA.A, i, 2) * ax[2];
              Uv[i] = IA.B[i] * ax[0] + IA.B[3 + i] * ax[1] + IA.B[6 + i] * ax[2];
            }
            D = ax[0] * Uw[0] + ax[1] * Uw[1] + ax[2] * Uw[2];
          } else {  // U = I (0, a) = (B a, C a)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              Uw[i] = IA.B[3 * i] * ax[0] + IA.B[3 * i + 1] * ax[1] + IA.B[3 * i + 2] * ax[2];
              Uv[i] = symget(IA.C, i, 0) * ax[0] + symget(IA.C, i, 1) * ax[1] + symget(IA.C, i, 2) * ax[2];
            }
            D = ax[0] * Uv[0] + ax[1] * Uv[1] + ax[2] * Uv[2];
          }
        }
        // u = τ + τ_spring − Sᵀ p^A
        const V axr{c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
        double u = have_tau ? tau[vo] : 0.0;
        if (KIND == KIND_GENERAL && type == 2 && (w1 & BF_SPRING) && c.springs)
          u += -c.td(tb + TD_SPRING) * (q[qo] - c.td(tb + TD_SPRING + 1));
        if (contacts) {
          const VD axd{c.td(tb + TD_AXIS), c.td(tb + TD_AXIS + 1), c.td(tb + TD_AXIS + 2)};
          u -= type == 1 ? dot(axd, pAd.w) : dot(axd, pAd.v);
        } else {
          u -= double(type == 1 ? dot(axr, pA.w) : dot(axr, pA.v));
        }
        if (type == 1 && c.armature)  // free_velocity: revolute armature (src/hybrid/articulated/mod.rs:244-247)
          D += c.td(tb + TD_ARMATURE);
        if (!(D > 0.0)) st |= 2;  // GPB_ST_CHOL_FAIL
        const double Dinv = 1.0 / D;
        const int du = c.L.DU + DU_D * vo;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          c.d(du + i) = Uw[i];
          c.d(du + 3 + i) = Uv[i];
        }
        c.d(du + 6) = Dinv;
        c.d(du + 7) = u;
        if (to_parent) {
          // I^a = I^A − U D⁻¹ Uᵀ (FP64) ; p^a = p^A + I^a c + U D⁻¹ u (R)
          double Ww[3], Wv[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            Ww[i] = Uw[i] * Dinv;
            Wv[i] = Uv[i] * Dinv;
          }
          const int ii[6] = {0, 1, 2, 0, 0, 1}, jj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            IA.A[k] -= Ww[ii[k]] * Uw[jj[k]];
            IA.C[k] -= Wv[ii[k]] * Uv[jj[k]];
          }
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) IA.B[3 * i + j] -= Ww[i] * Uv[j];
          const R ud = R(u * Dinv);
          const SV<R> Ur{{R(Uw[0]), R(Uw[1]), R(Uw[2])}, {R(Uv[0]), R(Uv[1]), R(Uv[2])}};
          pa = pA + abi_mul_r<R>(IA, cb) + scale(Ur, ud);
        }
      } else if (type == 3) {
        double L[21], dinv[6];
        if (!chol6(IA, L, dinv)) st |= 2;
        const int du = c.L.DU + DU_D * vo;
#pragma unroll
        for (int k = 0; k < 21; ++k) c.d(du + k) = L[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) c.d(du + 21 + k) = dinv[k];
        const SV<double> pp = contacts ? pAd : sv_d(pA);
        const double pv6[6] = {pp.w.x, pp.w.y, pp.w.z, pp.v.x, pp.v.y, pp.v.z};
        R pa6[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const double u = (have_tau ? tau[vo + k] : 0.0) - pv6[k];
          c.d(du + 27 + k) = u;
          pa6[k] = R(double(pv6[k]) + u);  // floating joint: I^a = 0, p^a = p^A + u
        }
        pa = {{pa6[0], pa6[1], pa6[2]}, {pa6[3], pa6[4], pa6[5]}};
      } else {  // fixed joint: I^a = I^A, p^a = p^A + I^A c
        pa = pA + abi_mul_r<R>(IA, cb);
      }
      if (to_parent) {
        const int pb = parent - 1;
        if (type != 3) {
          double Rr[9];
          const VD t{c.d(c.L.I + 12 * b + 9), c.d(c.L.I + 12 * b + 10), c.d(c.L.I + 12 * b + 11)};
          const int planar = kind_planar<KIND>(type, fl, b);
          double co = 1.0, si = 0.0;
          if (planar >= 0) {  // (cos, sin) record; abi_to_parent does not read Rr then
            co = c.d(c.L.I + 12 * b);
            si = c.d(c.L.I + 12 * b + 1);
#pragma unroll
            for (int k = 0; k < 9; ++k) Rr[k] = 0.0;
          } else {
#pragma unroll
            for (int k = 0; k < 9; ++k) Rr[k] = c.d(c.L.I + 12 * b + k);
          }
          const ABI Ip = abi_to_parent(IA, Rr, t, planar, co, si);
          if (pb == b - 1) {
            carryI = Ip;
          } else {
            ABI acc = load_abi(c, c.L.AI + ABI_D * pb);
            abi_add(acc, Ip);
            store_abi(c, c.L.AI + ABI_D * pb, acc);
            carryI = ABI{};
          }
        } else {
          carryI = ABI{};  // floating joint: I^a = 0
        }
        // force to the parent frame: (Rr n + t × Rr f, Rr f)
        M3<R> RrR;
        V tr;
        load_xf(c, b, kind_planar<KIND>(type, fl, b), RrR, tr);
        const SV<R> fp = force_to_parent(RrR, tr, pa);
        if (pb == b - 1) {
          carryP = fp;
          ctarget = pb;
        } else {
          if (contacts) store_svd(c, fd_row(c) + 6 * pb, load_svd(c, fd_row(c) + 6 * pb) + sv_d(fp));
          else store_sv(c, c.L.F + 6 * pb, load_sv(c, c.L.F + 6 * pb) + fp);
          carryP = SV<R>{zero, zero};
          ctarget = -1;
        }
      } else {
        // every path writes both carries: their previous values are dead once read
        carryI = ABI{};
        carryP = SV<R>{zero, zero};
        ctarget = -1;
      }
    }
  }
  // ---- pass 3 (outward): accelerations -------------------------------------
  SV<R> ap_{zero, zero};
  for (int b = 0; b < c.nb; ++b) {
    const uint32_t w0 = c.w(2 * b);
    const uint32_t w1 = (c.w(2 * b + 1) & ~(uint32_t)255) | kind_flags<KIND>(c.w(2 * b + 1));
    const int type = kind_type<KIND>(w0, b), parent = kind_parent<KIND>(w0, b);
    const int vo = (w0 >> 22) & 1023;
    const int tb = TOPO_D * b;
    SV<R> a;
    if (parent == 0) {
      a = {zero, {R(0), R(0), R(c.grav)}};  // inverse gravity (src/dynamics.rs:211-218)
    } else if (parent == b) {
      a = ap_;
    } else {
      a = load_sv(c, c.L.V + 6 * (parent - 1));  // pass 3 reuses V for branch accelerations
    }
    M3<R> Rr;
    V t;
    load_xf(c, b, kind_planar<KIND>(type, w1 & 255, b), Rr, t);
    const V ax{c.t(tb + TD_AXIS), c.t(tb + TD_AXIS + 1), c.t(tb + TD_AXIS + 2)};
    // a' = X a_p + c (the mixed form forms c again from the body velocity,
    // which a branch body's acceleration overwrites only below)
    SV<R> cb;
    if constexpr (sizeof(R) == 8) {
      cb = load_sv(c, c.L.A + 6 * b);
    } else {
      const SV<R> vb = load_sv(c, c.L.V + 6 * b);
      cb = bias_acc(type, ax, v, vo, vb.w, vb.v);
    }
    a.v = mulT(Rr, a.v + cross(a.w, t));
    a.w = mulT(Rr, a.w);
    a = a + cb;
    const int du = c.L.DU + DU_D * vo;
    if (type == 1 || type == 2) {
      double x;
      R xr;
      if constexpr (sizeof(R) == 4) {  // x = D⁻¹ (u − Uᵀ a') in double-float
        FF ua = ff_lin2(ffw(c, du), a.w.x, ffw(c, du + 1), a.w.y);
        ua = ff_fmaf(ffw(c, du + 2), a.w.z, ua);
        ua = ff_fmaf(ffw(c, du + 3), a.v.x, ua);
        ua = ff_fmaf(ffw(c, du + 4), a.v.y, ua);
        ua = ff_fmaf(ffw(c, du + 5), a.v.z, ua);
        const FF xf = ff_mul(ffw(c, du + 6), ff_sub(ffw(c, du + 7), ua));
        x = ff_to_double(xf);
        xr = ff_f(xf);
      } else {
        const double aw[3] = {double(a.w.x), double(a.w.y), double(a.w.z)};
        const double av[3] = {double(a.v.x), double(a.v.y), double(a.v.z)};
        double ua = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) ua += c.d(du + i) * aw[i] + c.d(du + 3 + i) * av[i];
        x = c.d(du + 6) * (c.d(du + 7) - ua);
        xr = R(x);
      }
      qdd[vo] = x;
      if (!isfinite(x)) st |= 1;  // GPB_ST_NONFINITE
      if (type == 1) a.w = a.w + ax * xr;
      else a.v = a.v + ax * xr;
    } else if (type == 3 && sizeof(R) == 4) {  // the mixed form's double-float record
      FF x[6], L[21], dinv[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) x[k] = ffw(c, du + 27 + k);
#pragma unroll
      for (int k = 0; k < 21; ++k) L[k] = ffw(c, du + k);
#pragma unroll
      for (int k = 0; k < 6; ++k) dinv[k] = ffw(c, du + 21 + k);
      solve6_ff(L, dinv, x);
      const float a6[6] = {float(a.w.x), float(a.w.y), float(a.w.z), float(a.v.x), float(a.v.y), float(a.v.z)};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double y = ff_to_double(ff_addf(x[k], -a6[k]));
        qdd[vo + k] = y;
        if (!isfinite(y)) st |= 1;
      }
      a = {{R(ff_f(x[0])), R(ff_f(x[1])), R(ff_f(x[2]))}, {R(ff_f(x[3])), R(ff_f(x[4])), R(ff_f(x[5]))}};
    } else if (type == 3) {
      // q̈ = D⁻¹ (u − Uᵀ a') with U = D = I^A, i.e. D⁻¹ u − a'; then a = D⁻¹ u
      double x[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) x[k] = c.d(du + 27 + k);
      double L[21], dinv[6];
#pragma unroll
      for (int k = 0; k < 21; ++k) L[k] = c.d(du + k);
#pragma unroll
      for (int k = 0; k < 6; ++k) dinv[k] = c.d(du + 21 + k);
      solve6(L, dinv, x);
      const double a6[6] = {double(a.w.x), double(a.w.y), double(a.w.z), double(a.v.x), double(a.v.y), double(a.v.z)};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double y = x[k] - a6[k];
        qdd[vo + k] = y;
        if (!isfinite(y)) st |= 1;
      }
      a = {{R(x[0]), R(x[1]), R(x[2])}, {R(x[3]), R(x[4]), R(x[5])}};
    }
    if ((w1 & 255) & BF_BRANCH) store_sv(c, c.L.V + 6 * b, a);
    ap_ = a;
  }
  return st;
}
