// Double-float ("double-word") arithmetic on the FP32 pipes.
//
// GB300 runs FP64 FMA at ~1 TFLOP/s but FP32 FMA at ~72 TFLOP/s (measured on
// this part), so the gate kernels keep each real number as an unevaluated sum
// hi + lo of two floats (~48-bit significand) and use error-free transforms:
//   TwoSum (Knuth), Fast2Sum (Dekker), TwoProd via FMA,
// as analysed in M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic",
// ACM TOMS 44(2), 2017.  The products below accumulate the low-order cross
// terms in a float and renormalise once, which bounds the ABSOLUTE error of a
// k-term dot product by a small multiple of 2^-48 * sum |a_i b_i|; that is the
// bound that matters for unit-norm statevectors.
//
// Every operation is written with __fadd_rn/__fmul_rn/__fmaf_rn so that the
// compiler can neither contract nor reassociate the error-free transforms.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pqc {

struct df {
  float h, l;
};

// complex double-float amplitude: (re.h, re.l, im.h, im.l) = one float4
struct cdf {
  float rh, rl, ih, il;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

// a*x + b*y with a, b, x, y double-float.
__device__ __forceinline__ df dot2(df a, df x, df b, df y) {
  float p1 = __fmul_rn(a.h, x.h);
  float e1 = __fmaf_rn(a.h, x.h, -p1);
  float p2 = __fmul_rn(b.h, y.h);
  float e2 = __fmaf_rn(b.h, y.h, -p2);
  df s = two_sum(p1, p2);
  float lo = __fadd_rn(__fadd_rn(e1, e2), s.l);
  lo = __fmaf_rn(a.h, x.l, lo);
  lo = __fmaf_rn(a.l, x.h, lo);
  lo = __fmaf_rn(b.h, y.l, lo);
  lo = __fmaf_rn(b.l, y.h, lo);
  return fast_two_sum(s.h, lo);
}

// a*x + b*y + c*z + d*w.
__device__ __forceinline__ df dot4(df a, df x, df b, df y, df c, df z, df d, df w) {
  float p1 = __fmul_rn(a.h, x.h);
  float lo = __fmaf_rn(a.h, x.h, -p1);
  float p2 = __fmul_rn(b.h, y.h);
  lo = __fadd_rn(lo, __fmaf_rn(b.h, y.h, -p2));
  float p3 = __fmul_rn(c.h, z.h);
  lo = __fadd_rn(lo, __fmaf_rn(c.h, z.h, -p3));
  float p4 = __fmul_rn(d.h, w.h);
  lo = __fadd_rn(lo, __fmaf_rn(d.h, w.h, -p4));
  df s12 = two_sum(p1, p2);
  df s34 = two_sum(p3, p4);
  df s = two_sum(s12.h, s34.h);
  lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(s12.l, s34.l), s.l));
  lo = __fmaf_rn(a.h, x.l, lo);
  lo = __fmaf_rn(a.l, x.h, lo);
  lo = __fmaf_rn(b.h, y.l, lo);
  lo = __fmaf_rn(b.l, y.h, lo);
  lo = __fmaf_rn(c.h, z.l, lo);
  lo = __fmaf_rn(c.l, z.h, lo);
  lo = __fmaf_rn(d.h, w.l, lo);
  lo = __fmaf_rn(d.l, w.h, lo);
  return fast_two_sum(s.h, lo);
}

// The same dot products without the final Fast2Sum: the result stays an exact
// unevaluated sum hi + lo, but lo is not reduced below ulp(hi)/2 (it stays
// within a few ulps of hi).  Every later operation multiplies and adds both
// parts, so the absolute error bound is unchanged (2^-46 of the operands'
// magnitude instead of 2^-48); the gate kernels use these, 3 instructions
// cheaper per output.
__device__ __forceinline__ df dot2_lazy(df a, df x, df b, df y) {
  float p1 = __fmul_rn(a.h, x.h);
  float e1 = __fmaf_rn(a.h, x.h, -p1);
  float p2 = __fmul_rn(b.h, y.h);
  float e2 = __fmaf_rn(b.h, y.h, -p2);
  df s = two_sum(p1, p2);
  float lo = __fadd_rn(__fadd_rn(e1, e2), s.l);
  lo = __fmaf_rn(a.h, x.l, lo);
  lo = __fmaf_rn(a.l, x.h, lo);
  lo = __fmaf_rn(b.h, y.l, lo);
  lo = __fmaf_rn(b.l, y.h, lo);
  return {s.h, lo};
}

// x + t*y (one product): the same lazy form as dot2_lazy, 12 instructions.
__device__ __forceinline__ df axpy_lazy(df x, df t, df y) {
  const float p = __fmul_rn(t.h, y.h);
  const float e = __fmaf_rn(t.h, y.h, -p);
  const df s = two_sum(x.h, p);
  float lo = __fadd_rn(__fadd_rn(x.l, e), s.l);
  lo = __fmaf_rn(t.h, y.l, lo);
  lo = __fmaf_rn(t.l, y.h, lo);
  return {s.h, lo};
}

// a*b, renormalised
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}

// a*b without the final renormalisation (4 instructions)
__device__ __forceinline__ df df_mul_lazy(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return {p, e};
}

__device__ __forceinline__ df dneg(df a) { return {-a.h, -a.l}; }
__device__ __forceinline__ df dhalf(df a) { return {__fmul_rn(a.h, 0.5f), __fmul_rn(a.l, 0.5f)}; }

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.h, b.h);
  float lo = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return fast_two_sum(s.h, lo);
}

// split a double into hi + lo floats (uses two FP64-rate conversions; used
// only at sweep boundaries and for coefficients)
__device__ __forceinline__ df df_from_double(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return {h, l};
}

__device__ __forceinline__ double df_to_double(df a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ cdf cdf_from(double2 v) {
  df r = df_from_double(v.x), i = df_from_double(v.y);
  return {r.h, r.l, i.h, i.l};
}

__device__ __forceinline__ double2 cdf_to(cdf v) {
  return make_double2((double)v.rh + (double)v.rl, (double)v.ih + (double)v.il);
}

__device__ __forceinline__ df re(cdf v) { return {v.rh, v.rl}; }
__device__ __forceinline__ df im(cdf v) { return {v.ih, v.il}; }
__device__ __forceinline__ cdf mk(df r, df i) { return {r.h, r.l, i.h, i.l}; }

// complex multiply (a.r + i a.i)(x.r + i x.i)
__device__ __forceinline__ cdf cmul(df ar, df ai, cdf x) {
  df xr = re(x), xi = im(x);
  return mk(dot2(ar, xr, dneg(ai), xi), dot2(ar, xi, ai, xr));
}

// complex a*x + b*y
__device__ __forceinline__ cdf cdot2(df ar, df ai, cdf x, df br, df bi, cdf y) {
  df xr = re(x), xi = im(x), yr = re(y), yi = im(y);
  return mk(dot4(ar, xr, dneg(ai), xi, br, yr, dneg(bi), yi), dot4(ar, xi, ai, xr, br, yi, bi, yr));
}

__device__ __forceinline__ cdf cneg(cdf v) { return {-v.rh, -v.rl, -v.ih, -v.il}; }
// multiply by i
__device__ __forceinline__ cdf cmul_i(cdf v) { return {-v.ih, -v.il, v.rh, v.rl}; }
__device__ __forceinline__ cdf cscale_half(cdf v) {
  return {__fmul_rn(v.rh, 0.5f), __fmul_rn(v.rl, 0.5f), __fmul_rn(v.ih, 0.5f), __fmul_rn(v.il, 0.5f)};
}

__device__ __forceinline__ cdf cadd(cdf a, cdf b) {
  df r = df_add(re(a), re(b)), i = df_add(im(a), im(b));
  return mk(r, i);
}

}  // namespace pqc
