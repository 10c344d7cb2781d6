// Float-float arithmetic on the FP32 pipe, for kernels that would otherwise be bound by
// GB300's FP64 pipe (about 2 FMA/clk/SM against 128 FP32 lanes).
//
// split_f64 turns an FP64 value into hi + lo floats by bit manipulation (no FP64
// instruction): hi keeps the sign, the exponent and the top 23 mantissa bits, lo the other
// 29 bits rounded to 24 — about 47 significant bits, 2^-47 relative.  Values below 2^-126
// in magnitude become zero and those below 2^-74 keep hi only (absolute error < 2^-97).
// ff_fma adds an error-free product of two such pairs (hi*hi with its FMA residual, plus
// the cross terms) to a float pair with TwoSum.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ float2 split_f64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0x7ff) return make_float2(__int_as_float((int)(sign | 0x7fc00000u)), 0.f);  // inf / nan -> nan
  if (e < 1023 - 126) return make_float2(__int_as_float((int)sign), 0.f);
  if (e > 1023 + 127) return make_float2(__int_as_float((int)(sign | 0x7f800000u)), 0.f);
  const unsigned mh = (unsigned)(b >> 29) & 0x7fffffu;
  const float hi = __int_as_float((int)(sign | ((unsigned)(e - 1023 + 127) << 23) | mh));
  const int el = e - 1075 + 127;  // biased exponent of 2^(e - 1075), the weight of lo's unit
  float lo = 0.f;
  if (el > 0) lo = __uint2float_rn((unsigned)(b & 0x1fffffffull)) * __int_as_float(el << 23);
  return make_float2(hi, sign ? -lo : lo);
}

// (sh, sl) += a * b, a and b float pairs
__device__ __forceinline__ void ff_fma(float &sh, float &sl, float2 a, float2 b) {
  const float ph = __fmul_rn(a.x, b.x);
  float pl = __fmaf_rn(a.x, b.x, -ph);
  pl = __fmaf_rn(a.x, b.y, pl);
  pl = __fmaf_rn(a.y, b.x, pl);
  const float t = __fadd_rn(sh, ph);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
  sl = __fadd_rn(sl, __fadd_rn(err, pl));
  sh = t;
}

__device__ __forceinline__ void ff_renorm(float &sh, float &sl) {
  const float t = __fadd_rn(sh, sl);
  sl = __fsub_rn(sl, __fsub_rn(t, sh));
  sh = t;
}
