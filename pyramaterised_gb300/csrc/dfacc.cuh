// Double-float accumulation helpers shared by the reduction kernels.
#pragma once
#include <cuda_runtime.h>

namespace pqc {

// double -> (hi, lo) floats with integer operations only: hi keeps the top 24
// significand bits (exact), lo the next 23; values below 2^-80 in magnitude
// keep only hi (absolute error < 2^-104) and below 2^-126 become 0; values beyond the float range (and
// inf, nan) convert as float.
__device__ __forceinline__ float2 split_double(double x) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
  if (e < 897) return make_float2(0.f, 0.f);
  if (e > 1150) return make_float2(__double2float_rn(x), 0.f);  // beyond float range, inf, nan
  const unsigned long long m = (unsigned long long)b & 0xfffffffffffffull;
  const float hi = __int_as_float((int)(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29)));
  float lo = 0.f;
  if (e >= 943) {
    const unsigned m23 = (unsigned)((m >> 6) & 0x7fffffu);
    const float f = __fsub_rn(__int_as_float((int)(0x4B000000u | m23)), 8388608.0f);  // exact: m23 < 2^23
    const float scale = __int_as_float((e - 1069 + 127) << 23);                        // 2^(e - 1075 + 6)
    lo = __int_as_float(__float_as_int(__fmul_rn(f, scale)) | (int)sign);
  }
  return make_float2(hi, lo);
}

struct Acc {
  float h, l;
};

// acc += x * y  (x, y double-float)
__device__ __forceinline__ void acc_mul(Acc& acc, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = __fmaf_rn(xh, yh, -p);
  const float s = __fadd_rn(acc.h, p);
  const float bb = __fsub_rn(s, acc.h);
  const float t = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.h = s;
  float l = __fmaf_rn(xh, yl, acc.l);
  l = __fmaf_rn(xl, yh, l);
  acc.l = __fadd_rn(__fadd_rn(l, e), t);
}

__device__ __forceinline__ void acc_add(Acc& acc, float xh, float xl) {
  const float s = __fadd_rn(acc.h, xh);
  const float bb = __fsub_rn(s, acc.h);
  const float t = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(xh, bb));
  acc.h = s;
  acc.l = __fadd_rn(acc.l, __fadd_rn(xl, t));
}

// Double-float sum over a warp (TwoSum at every butterfly step); lane 0 holds the result.
__device__ __forceinline__ Acc warp_sum_df(Acc a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, a.h, o);
    const float l = __shfl_xor_sync(0xffffffffu, a.l, o);
    acc_add(a, h, l);
  }
  return a;
}

}  // namespace pqc
