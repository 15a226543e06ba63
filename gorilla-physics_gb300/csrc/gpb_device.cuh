// Device spatial algebra for the batched rigid-body step (templated on the
// arithmetic type: double for the FP64 form, float for the mixed form's sweeps).
//
// Everything is expressed in the world frame, as in gorilla-physics'
// dynamics.rs / mechanism.rs, but restructured for the GPU:
//   - transforms are (rotation matrix, translation) pairs, not quaternion
//     isometries, so composing a revolute joint about a principal axis costs
//     12 multiplies;
//   - the Coriolis term is V_i ×m (S_i q̇_i) in the world frame, which equals the
//     reference's X_i[(X_i⁻¹ V_i) ×m (S_i^b q̇_i)] (src/dynamics.rs:143-192)
//     because the spatial motion cross product commutes with a rigid transform;
//   - the world-frame spatial inertia is built with the parallel-axis form
//     J_O = R J Rᵀ + m(|p|²1 − p pᵀ) + 2(c·p)1 − c pᵀ − p cᵀ,  c = R·(m com),
//     algebraically identical to SpatialInertia::transform (src/inertia.rs:106-134).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gpb {

template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R>
__device__ __forceinline__ V3<R> v3(R x, R y, R z) {
  return {x, y, z};
}
template <typename R>
__device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename R>
__device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename R>
__device__ __forceinline__ V3<R> operator*(V3<R> a, R s) {
  return {a.x * s, a.y * s, a.z * s};
}
template <typename R>
__device__ __forceinline__ R dot(V3<R> a, V3<R> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
__device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Row-major 3x3.
template <typename R>
struct M3 {
  R a[9];
};
template <typename R>
__device__ __forceinline__ V3<R> mul(const M3<R>& m, V3<R> v) {
  return {m.a[0] * v.x + m.a[1] * v.y + m.a[2] * v.z, m.a[3] * v.x + m.a[4] * v.y + m.a[5] * v.z,
          m.a[6] * v.x + m.a[7] * v.y + m.a[8] * v.z};
}
template <typename R>
__device__ __forceinline__ V3<R> col(const M3<R>& m, int c) {
  return {m.a[c], m.a[3 + c], m.a[6 + c]};
}
template <typename R>
__device__ __forceinline__ M3<R> mul(const M3<R>& x, const M3<R>& y) {
  M3<R> r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      r.a[3 * i + j] = x.a[3 * i] * y.a[j] + x.a[3 * i + 1] * y.a[3 + j] + x.a[3 * i + 2] * y.a[6 + j];
  return r;
}

// Spatial vector (angular, linear).
template <typename R>
struct SV {
  V3<R> w, v;
};
template <typename R>
__device__ __forceinline__ SV<R> operator+(const SV<R>& a, const SV<R>& b) {
  return {a.w + b.w, a.v + b.v};
}
template <typename R>
__device__ __forceinline__ SV<R> operator-(const SV<R>& a, const SV<R>& b) {
  return {a.w - b.w, a.v - b.v};
}
template <typename R>
__device__ __forceinline__ SV<R> scale(const SV<R>& a, R s) {
  return {a.w * s, a.v * s};
}
// motion cross product x ×m y (src/util.rs:44-53)
template <typename R>
__device__ __forceinline__ SV<R> crm(const SV<R>& x, const SV<R>& y) {
  return {cross(x.w, y.w), cross(x.w, y.v) + cross(x.v, y.w)};
}
// force cross product v ×* f (src/util.rs:62-66)
template <typename R>
__device__ __forceinline__ SV<R> crf(const SV<R>& x, const SV<R>& f) {
  return {cross(x.w, f.w) + cross(x.v, f.v), cross(x.w, f.v)};
}
template <typename R>
__device__ __forceinline__ R sdot(const SV<R>& a, const SV<R>& b) {
  return dot(a.w, b.w) + dot(a.v, b.v);
}

// Spatial inertia about the frame origin: symmetric moment (xx,yy,zz,xy,xz,yz),
// cross part c = m·com, mass.
template <typename R>
struct SI {
  R j[6];
  V3<R> c;
  R m;
};
template <typename R>
__device__ __forceinline__ V3<R> jmul(const R* j, V3<R> w) {
  return {j[0] * w.x + j[3] * w.y + j[4] * w.z, j[3] * w.x + j[1] * w.y + j[5] * w.z,
          j[4] * w.x + j[5] * w.y + j[2] * w.z};
}
// I · (w, v) = (J w + c × v, m v − c × w)   (src/util.rs:18-28)
template <typename R>
__device__ __forceinline__ SV<R> imul(const SI<R>& I, const SV<R>& s) {
  return {jmul(I.j, s.w) + cross(I.c, s.v), s.v * I.m - cross(I.c, s.w)};
}
template <typename R>
__device__ __forceinline__ void iadd(SI<R>& a, const SI<R>& b) {
#pragma unroll
  for (int k = 0; k < 6; ++k) a.j[k] += b.j[k];
  a.c = a.c + b.c;
  a.m += b.m;
}

// Body inertia (body frame) → world frame, given the body rotation Rm and
// origin p.  `diag` = the body-frame moment is diagonal (j[3..5] == 0).
template <typename R>
__device__ __forceinline__ SI<R> to_world(const SI<R>& Ib, const M3<R>& Rm, V3<R> p, bool diag) {
  SI<R> o;
  // R J Rᵀ
  if (diag) {
    V3<R> c0 = col(Rm, 0), c1 = col(Rm, 1), c2 = col(Rm, 2);
    R d0 = Ib.j[0], d1 = Ib.j[1], d2 = Ib.j[2];
    o.j[0] = d0 * c0.x * c0.x + d1 * c1.x * c1.x + d2 * c2.x * c2.x;
    o.j[1] = d0 * c0.y * c0.y + d1 * c1.y * c1.y + d2 * c2.y * c2.y;
    o.j[2] = d0 * c0.z * c0.z + d1 * c1.z * c1.z + d2 * c2.z * c2.z;
    o.j[3] = d0 * c0.x * c0.y + d1 * c1.x * c1.y + d2 * c2.x * c2.y;
    o.j[4] = d0 * c0.x * c0.z + d1 * c1.x * c1.z + d2 * c2.x * c2.z;
    o.j[5] = d0 * c0.y * c0.z + d1 * c1.y * c1.z + d2 * c2.y * c2.z;
  } else {
    // T = R J (3x3), then (T Rᵀ) upper triangle
    R t[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      V3<R> r{Rm.a[3 * i], Rm.a[3 * i + 1], Rm.a[3 * i + 2]};
      V3<R> tj = jmul(Ib.j, r);  // (R J)_i· = J r_i since J symmetric
      t[3 * i] = tj.x;
      t[3 * i + 1] = tj.y;
      t[3 * i + 2] = tj.z;
    }
    auto rr = [&](int i, int k) {
      return t[3 * i] * Rm.a[3 * k] + t[3 * i + 1] * Rm.a[3 * k + 1] + t[3 * i + 2] * Rm.a[3 * k + 2];
    };
    o.j[0] = rr(0, 0);
    o.j[1] = rr(1, 1);
    o.j[2] = rr(2, 2);
    o.j[3] = rr(0, 1);
    o.j[4] = rr(0, 2);
    o.j[5] = rr(1, 2);
  }
  V3<R> c = mul(Rm, Ib.c);
  R m = Ib.m;
  V3<R> mp = p * m;
  // m(|p|²1 − p pᵀ) + 2(c·p)1 − c pᵀ − p cᵀ
  R pp = dot(p, p);
  R cp2 = dot(c, p) * R(2);
  R dg = m * pp + cp2;
  o.j[0] += dg - mp.x * p.x - R(2) * c.x * p.x;
  o.j[1] += dg - mp.y * p.y - R(2) * c.y * p.y;
  o.j[2] += dg - mp.z * p.z - R(2) * c.z * p.z;
  o.j[3] += -mp.x * p.y - (c.x * p.y + p.x * c.y);
  o.j[4] += -mp.x * p.z - (c.x * p.z + p.x * c.z);
  o.j[5] += -mp.y * p.z - (c.y * p.z + p.y * c.z);
  o.c = c + mp;
  o.m = m;
  return o;
}

}  // namespace gpb
