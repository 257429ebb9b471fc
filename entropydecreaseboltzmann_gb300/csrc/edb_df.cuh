// Double-float arithmetic for the FP64-accurate kernels on the FP32 pipe.
//
// A value is an unevaluated sum hi + lo of two floats (about 48 significant
// bits).  Products are split exactly by the FMA two-product (p + e with
// e = fma(a, b, -p)) and sums are carried exactly by Knuth's two-sum; see
// edb_kernels_calq64x.cu for how a collision-sum term uses them.  Packed
// helpers work on f32x2 register pairs (two lanes, e.g. the real and
// imaginary parts of a complex value); scalar helpers on float2 {hi, lo}.
// The scalar helpers use the _rn intrinsics so no operation is contracted.
#pragma once

#include <cuda_runtime.h>

namespace edb {
namespace df {

typedef unsigned long long u64;

__device__ __forceinline__ u64 pk(float a, float b) {
  u64 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 upk(u64 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ u64 mul2(u64 a, u64 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 fma2(u64 a, u64 b, u64 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ u64 add2(u64 a, u64 b) {
  u64 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
  u64 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

struct DF2 {  // packed double-float pair: lanes (re, im)
  u64 h, l;
};

// acc += s * u for a real double-float scalar s (given as the pairs (s_h, s_h),
// (-s_h, -s_h), (-s_l, -s_l)) and u = -nu_h + uc.
__device__ __forceinline__ void df_axpy(DF2 &acc, u64 sh2, u64 nsh2, u64 nsl2, u64 nu_h, u64 uc) {
  // leading product s_h * u_h = s_h * (-nu_h): nph = -(s_h u_h) rounded, pe exact error
  const u64 nph = mul2(sh2, nu_h);       // = -rn(s_h u_h)
  const u64 pe = fma2(nsh2, nu_h, nph);  // = s_h u_h - rn(s_h u_h)
  // cross terms s_h * uc + s_l * u_h  (u_h = -nu_h, so s_l u_h = (-s_l) nu_h)
  const u64 pl = fma2(sh2, uc, fma2(nsl2, nu_h, pe));
  // two-sum of acc.h and p_h = -nph
  const u64 s = sub2(acc.h, nph);
  const u64 bb = sub2(s, acc.h);  // ~ p_h
  const u64 e = sub2(sub2(acc.h, sub2(s, bb)), add2(nph, bb));  // (acc.h - (s - bb)) + (p_h - bb)
  acc.h = s;
  acc.l = add2(acc.l, add2(e, pl));
}

// ---- scalar {hi, lo}
// a + b = s + e exactly (Knuth)
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
// a + b = s + e exactly when |a| >= |b| (Dekker); renormalises a hi, lo pair
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 sdf_add(float2 a, float2 b) {
  const float2 s = two_sum(a.x, b.x);
  return fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 sdf_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sdf_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e));
  return fast_two_sum(p, e);
}

}  // namespace df
}  // namespace edb
