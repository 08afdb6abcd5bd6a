// Double-float arithmetic: values as unevaluated pairs hi + lo of floats (about 48
// significant bits), computed on the FP32 pipe.  The error-free transformations use
// the _rn intrinsics so that no FMA contraction can merge a product into the
// following sum.
#pragma once

#include <cuda_runtime.h>

namespace fi {

__device__ __forceinline__ float2 df_split(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}

__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// (a.x + a.y) + (b.x + b.y), renormalised
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  const float lo = __fadd_rn(__fadd_rn(a.y, b.y), err);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// (sh, sl) += b * z (the lo * lo term, 2^-48 relative, is dropped)
__device__ __forceinline__ void df_mac(float2 b, float2 z, float& sh, float& sl) {
  const float p = __fmul_rn(b.x, z.x);
  float e = __fmaf_rn(b.x, z.x, -p);
  e = __fmaf_rn(b.x, z.y, e);
  e = __fmaf_rn(b.y, z.x, e);
  const float t = __fadd_rn(sh, p);
  const float bb = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = t;
}

__device__ __forceinline__ float2 df_neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Two independent df_mac in the lanes of float2 pairs, with packed FP32x2
// instructions (each lane rounds exactly as df_mac):
// (sh.x, sl.x) += b * (zh.x + zl.x) and (sh.y, sl.y) += b * (zh.y + zl.y).
__device__ __forceinline__ void df_mac_x2(float2 b, float2 zh, float2 zl, float2& sh,
                                          float2& sl) {
  const float2 bh = make_float2(b.x, b.x), bl = make_float2(b.y, b.y);
  const float2 p = __fmul2_rn(bh, zh);
  float2 e = __ffma2_rn(bh, zh, df_neg2(p));
  e = __ffma2_rn(bh, zl, e);
  e = __ffma2_rn(bl, zh, e);
  const float2 t = __fadd2_rn(sh, p);
  const float2 bb = __fadd2_rn(t, df_neg2(sh));
  const float2 err = __fadd2_rn(__fadd2_rn(sh, df_neg2(__fadd2_rn(t, df_neg2(bb)))),
                                __fadd2_rn(p, df_neg2(bb)));
  sl = __fadd2_rn(sl, __fadd2_rn(err, e));
  sh = t;
}

}  // namespace fi
