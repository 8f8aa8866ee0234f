// qt_arith.cuh -- complex arithmetic policies of the chain kernels.
//
// F64   complex128 on the FP64 pipe (double2).
// C32   complex64 arithmetic on the FP32 pipe in the DF64 storage layout
//       (below).
// DF64  complex numbers whose real and imaginary parts are each an
//       unevaluated sum of two floats, hi + lo ("double-float"), computed on
//       the FP32 pipe.  GB300 runs FP32 61x faster than FP64; a double-float
//       multiply-add costs 11 FP32 operations, so a complex multiply-add runs
//       ~5x faster than on the FP64 pipe.  Precision: products are exact up
//       to the dropped lo*lo term (2^-48 relative), sums use error-free
//       two-sums (Knuth), so a length-K dot product carries ~K * 2^-48
//       relative error -- far inside the 1e-12 parity bar.  Exponent range is
//       FP32's (|x| in 1e-38 .. 3e38).
//       Storage: float4 (re_hi, re_lo, im_hi, im_lo), 16 bytes like double2,
//       so both precisions share one arena layout.
//
// All error-free transformations use the _rn intrinsics, which the compiler
// never contracts into FMAs or reassociates.
#pragma once

#include <cuda_runtime.h>

namespace qt {

__device__ __forceinline__ double2 cz64() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double2 cmul64(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ void cfma64(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfmac64(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
__device__ __forceinline__ double2 cadd64(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}

struct F64 {
  typedef double2 S;  // storage / operand
  typedef double2 A;  // accumulator
  typedef double2 C;  // coefficient
  static __device__ __forceinline__ A zero() { return cz64(); }
  static __device__ __forceinline__ S ld(const S* p) { return __ldg(p); }
  static __device__ __forceinline__ void mac(A& acc, const S& a, const S& b) { cfma64(acc, a, b); }
  static __device__ __forceinline__ void macc(A& acc, const S& a, const S& b) { cfmac64(acc, a, b); }
  static __device__ __forceinline__ void add(A& acc, const S& b) { acc = cadd64(acc, b); }
  static __device__ __forceinline__ C coef(double2 c) { return c; }
  static __device__ __forceinline__ S fin(const A& a) { return a; }
  static __device__ __forceinline__ S scale(const C& c, const S& v) { return cmul64(c, v); }
  static __device__ __forceinline__ S plus(const S& a, const S& b) { return cadd64(a, b); }
  static __device__ __forceinline__ S mul(const S& a, const S& b) { return cmul64(a, b); }
  static __device__ __forceinline__ void cmac(A& acc, const C& c, const S& b) { cfma64(acc, c, b); }
  static __device__ __forceinline__ void norm(A&) {}
  // projector helpers: |x|^2, -x, 1/x
  static __device__ __forceinline__ double mag2(const S& x) { return x.x * x.x + x.y * x.y; }
  static __device__ __forceinline__ S neg(const S& x) { return make_double2(-x.x, -x.y); }
  static __device__ __forceinline__ S recip(const S& x) {
    const double den = x.x * x.x + x.y * x.y;
    return make_double2(x.x / den, -x.y / den);
  }
};

// ---- double-float helpers --------------------------------------------------
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void df_quick_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// (hi, lo) += (ah, al) * (bh, bl), lo left unnormalised
__device__ __forceinline__ void df_mac(float& hi, float& lo, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(err, e));
}
__device__ __forceinline__ void df_norm(float& hi, float& lo) {
  float s, e;
  df_quick_two_sum(hi, lo, s, e);
  hi = s;
  lo = e;
}
// (hi, lo) += (bh, bl)
__device__ __forceinline__ void df_add(float& hi, float& lo, float bh, float bl) {
  float s, e;
  df_two_sum(hi, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, bl));
  hi = s;
  lo = e;
}
__device__ __forceinline__ float2 df_split(double x) {
  const float h = __double2float_rn(x);
  const float l = __double2float_rn(x - (double)h);
  return make_float2(h, l);
}

struct DF64 {
  typedef float4 S;  // (re_hi, re_lo, im_hi, im_lo)
  typedef float4 A;
  typedef float4 C;
  static __device__ __forceinline__ A zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ S ld(const S* p) { return __ldg(p); }
  // acc += a * b
  static __device__ __forceinline__ void mac(A& acc, const S& a, const S& b) {
    df_mac(acc.x, acc.y, a.x, a.y, b.x, b.y);
    df_mac(acc.x, acc.y, -a.z, -a.w, b.z, b.w);
    df_mac(acc.z, acc.w, a.x, a.y, b.z, b.w);
    df_mac(acc.z, acc.w, a.z, a.w, b.x, b.y);
  }
  // acc += conj(a) * b
  static __device__ __forceinline__ void macc(A& acc, const S& a, const S& b) {
    df_mac(acc.x, acc.y, a.x, a.y, b.x, b.y);
    df_mac(acc.x, acc.y, a.z, a.w, b.z, b.w);
    df_mac(acc.z, acc.w, a.x, a.y, b.z, b.w);
    df_mac(acc.z, acc.w, -a.z, -a.w, b.x, b.y);
  }
  static __device__ __forceinline__ void add(A& acc, const S& b) {
    df_add(acc.x, acc.y, b.x, b.y);
    df_add(acc.z, acc.w, b.z, b.w);
  }
  static __device__ __forceinline__ C coef(double2 c) {
    const float2 r = df_split(c.x), i = df_split(c.y);
    return make_float4(r.x, r.y, i.x, i.y);
  }
  static __device__ __forceinline__ S fin(A a) {
    df_norm(a.x, a.y);
    df_norm(a.z, a.w);
    return a;
  }
  static __device__ __forceinline__ S mul(const S& a, const S& b) {
    A acc = zero();
    mac(acc, a, b);
    return fin(acc);
  }
  static __device__ __forceinline__ S scale(const C& c, const S& v) { return mul(c, v); }
  static __device__ __forceinline__ S plus(const S& a, const S& b) {
    A acc = a;
    add(acc, b);
    return fin(acc);
  }
  static __device__ __forceinline__ void cmac(A& acc, const C& c, const S& b) { mac(acc, c, b); }
  // renormalise (hi, lo) so that |lo| <= ulp(hi)/2: called every few
  // multiply-adds, it keeps the rounding of the lo additions at 2^-48 |hi|
  static __device__ __forceinline__ void norm(A& a) {
    df_norm(a.x, a.y);
    df_norm(a.z, a.w);
  }
  // projector helpers: |x|^2 (from the hi parts), -x, 1/x (complex128 reciprocal, split)
  static __device__ __forceinline__ double mag2(const S& x) {
    return (double)x.x * (double)x.x + (double)x.z * (double)x.z;
  }
  static __device__ __forceinline__ S neg(const S& x) { return make_float4(-x.x, -x.y, -x.z, -x.w); }
  static __device__ __forceinline__ S recip(const S& x) {
    const double re = (double)x.x + (double)x.y, im = (double)x.z + (double)x.w;
    const double den = re * re + im * im;
    const float2 r = df_split(re / den), i = df_split(-im / den);
    return make_float4(r.x, r.y, i.x, i.y);
  }
};

// ---- complex64 arithmetic ---------------------------------------------------
// C32: complex FP32 on the FP32 pipe (four FFMA per complex multiply-add).
// Storage stays the 16-byte float4 of DF64, (re, re_lo, im, im_lo): loads use
// the hi words only (a double-float input is rounded to FP32), results are
// written with zero lo words, so conversions and arenas are shared with DF64.
struct C32 {
  typedef float4 S;
  typedef float4 A;  // (re, 0, im, 0)
  typedef float4 C;
  static __device__ __forceinline__ A zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ S ld(const S* p) { return __ldg(p); }
  static __device__ __forceinline__ void mac(A& acc, const S& a, const S& b) {
    acc.x = __fmaf_rn(a.x, b.x, acc.x);
    acc.x = __fmaf_rn(-a.z, b.z, acc.x);
    acc.z = __fmaf_rn(a.x, b.z, acc.z);
    acc.z = __fmaf_rn(a.z, b.x, acc.z);
  }
  static __device__ __forceinline__ void macc(A& acc, const S& a, const S& b) {
    acc.x = __fmaf_rn(a.x, b.x, acc.x);
    acc.x = __fmaf_rn(a.z, b.z, acc.x);
    acc.z = __fmaf_rn(a.x, b.z, acc.z);
    acc.z = __fmaf_rn(-a.z, b.x, acc.z);
  }
  static __device__ __forceinline__ void add(A& acc, const S& b) {
    acc.x = __fadd_rn(acc.x, b.x);
    acc.z = __fadd_rn(acc.z, b.z);
  }
  static __device__ __forceinline__ C coef(double2 c) { return make_float4((float)c.x, 0.f, (float)c.y, 0.f); }
  static __device__ __forceinline__ S fin(const A& a) { return make_float4(a.x, 0.f, a.z, 0.f); }
  static __device__ __forceinline__ S mul(const S& a, const S& b) {
    A acc = zero();
    mac(acc, a, b);
    return fin(acc);
  }
  static __device__ __forceinline__ S scale(const C& c, const S& v) { return mul(c, v); }
  static __device__ __forceinline__ S plus(const S& a, const S& b) {
    return make_float4(__fadd_rn(a.x, b.x), 0.f, __fadd_rn(a.z, b.z), 0.f);
  }
  static __device__ __forceinline__ void cmac(A& acc, const C& c, const S& b) { mac(acc, c, b); }
  static __device__ __forceinline__ void norm(A&) {}
  static __device__ __forceinline__ double mag2(const S& x) {
    return (double)x.x * (double)x.x + (double)x.z * (double)x.z;
  }
  static __device__ __forceinline__ S neg(const S& x) { return make_float4(-x.x, 0.f, -x.z, 0.f); }
  static __device__ __forceinline__ S recip(const S& x) {
    const double re = x.x, im = x.z;
    const double den = re * re + im * im;
    return make_float4((float)(re / den), 0.f, (float)(-im / den), 0.f);
  }
};

}  // namespace qt
