// Double-float ("FF") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers with |lo| of the order of ulp(hi), about 48 significant bits.
//
// GB300 issues FP32 at 63× its FP64 rate (78 against 1.25 TFLOP/s measured),
// so a recursion that needs more than FP32's 24 bits but not all of FP64's 53
// is cheaper in pairs of FP32 numbers: an FF multiply-add is about 15 FP32
// instructions, an FP64 one occupies the FP64 pipe for as long as about 64.
//
// The building blocks are the published error-free transformations:
//   two_sum       Knuth, TAOCP vol. 2 §4.2.2 (s + e = a + b exactly, 6 adds);
//   fast_two_sum  Dekker 1971 (the same for |a| ≥ |b|, 3 adds);
//   the exact product with a fused multiply-add: p = a·b rounded,
//                 e = fma(a, b, −p), p + e = a·b exactly (2 ops);
// composed as in Dekker, "A floating-point technique for extending the
// available precision" (Numer. Math. 18, 1971) and Hida, Li & Bailey's
// double-double library (2001): the sum adds the low parts after an exact
// sum of the high parts, so its error is about 2^-47 of the larger operand
// (the same absolute bound as a cancelling FP64 subtraction scaled by 2^6).
//
// Every operation is an explicit round-to-nearest intrinsic: the compiler
// may neither contract a product into a following add nor reorder the sums,
// either of which breaks the exactness the transformations rely on.
//
// The products-and-sums (ff_fma, ff_fmaf, ff_lin2) return the exact sum of
// their leading terms plus the rounded sum of the small ones without the
// final renormalisation: |lo| may reach a few ulp(hi) instead of ½ — after a
// cancelling subtraction, more than |hi| — which every operation here
// accepts (hi + lo is the same value either way), and it saves 3 of their
// 12–14 instructions.  ff_add renormalises.  Where an FP32 approximation of a
// value is needed, ff_f rounds hi + lo (hi alone can be far off).
#pragma once

struct alignas(8) FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff(float x) { return {x, 0.0f}; }
// The FP32 value nearest hi + lo.
__device__ __forceinline__ float ff_f(FF a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.hi, -a.lo}; }

// s + e = a + b exactly (any a, b).
__device__ __forceinline__ FF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// s + e = a + b exactly when |a| ≥ |b| (or a = 0).
__device__ __forceinline__ FF fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// c + a·b and c − a·b (one exact sum of the leading terms, no intermediate
// normalisation of the product).
__device__ __forceinline__ FF ff_fma(FF a, FF b, FF c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const FF s = two_sum(p, c.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo))};
}
__device__ __forceinline__ FF ff_fms(FF c, FF a, FF b) { return ff_fma(ff_neg(a), b, c); }
// c + a·f for an FP32 factor f.
__device__ __forceinline__ FF ff_fmaf(FF a, float f, FF c) {
  const float p = __fmul_rn(a.hi, f);
  float e = __fmaf_rn(a.hi, f, -p);
  e = __fmaf_rn(a.lo, f, e);
  const FF s = two_sum(p, c.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo))};
}
// a·x + b·y for FP32 factors x, y (a plane rotation's or a cross product's term).
__device__ __forceinline__ FF ff_lin2(FF a, float x, FF b, float y) {
  const float p = __fmul_rn(a.hi, x);
  float e1 = __fmaf_rn(a.hi, x, -p);
  e1 = __fmaf_rn(a.lo, x, e1);
  const float r = __fmul_rn(b.hi, y);
  float e2 = __fmaf_rn(b.hi, y, -r);
  e2 = __fmaf_rn(b.lo, y, e2);
  const FF s = two_sum(p, r);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(e1, e2))};
}
// Σ a_i·x_i over three terms with FP32 factors.
__device__ __forceinline__ FF ff_dot3f(FF a0, FF a1, FF a2, float x0, float x1, float x2) {
  return ff_fmaf(a2, x2, ff_lin2(a0, x0, a1, x1));
}

// Exact products of FP32 operands.
__device__ __forceinline__ FF two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
// a·b − c·d for FP32 operands (a cross-product component): both products
// exact, their difference one exact sum of the leading terms.
__device__ __forceinline__ FF ff_det2(float a, float b, float c, float d) {
  const float p = __fmul_rn(a, b);
  const float e1 = __fmaf_rn(a, b, -p);
  const float r = __fmul_rn(c, d);
  const float e2 = __fmaf_rn(c, d, -r);
  const FF s = two_sum(p, -r);
  return {s.hi, __fadd_rn(s.lo, __fsub_rn(e1, e2))};
}
// c + a·b for FP32 a, b (the product exact).
__device__ __forceinline__ FF ff_add_prod(float a, float b, FF c) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const FF s = two_sum(p, c.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo))};
}
// a + f for an FP32 f.
__device__ __forceinline__ FF ff_addf(FF a, float f) {
  const FF s = two_sum(a.hi, f);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

// 1/d: the FP32 reciprocal refined by one Newton step, r + r·(1 − d·r), with
// the residual formed exactly from the FF product.
__device__ __forceinline__ FF ff_rcp(FF d) {
  const float r = __frcp_rn(d.hi);
  const float p = __fmul_rn(d.hi, r);
  float e = __fmaf_rn(d.hi, r, -p);
  e = __fmaf_rn(d.lo, r, e);
  const float res = __fsub_rn(__fsub_rn(1.0f, p), e);  // 1 − p is exact (p ≈ 1)
  return fast_two_sum(r, __fmul_rn(r, res));
}

// 1/√x for x > 0 (hi + lo normalised): the FP32 rsqrtf refined by one Newton
// step, y + y·(1 − x·y²)/2, with the residual 1 − x·y² formed from the exact
// square y² and an FF product.  rsqrtf's relative error δ (a few 2^-24) leaves
// 3δ²/2 after the step, below 1e-13.
__device__ __forceinline__ FF ff_rsqrt(FF x) {
  const float y = rsqrtf(x.hi);
  const FF r = ff_sub(ff(1.0f), ff_mul(x, two_prod(y, y)));
  return fast_two_sum(y, __fmul_rn(__fmul_rn(0.5f, y), ff_f(r)));
}

// Conversions (FP64 instructions: keep them out of inner loops).
__device__ __forceinline__ FF ff_from_double(double x) {
  const float hi = __double2float_rn(x);
  return {hi, __double2float_rn(x - (double)hi)};
}
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }
