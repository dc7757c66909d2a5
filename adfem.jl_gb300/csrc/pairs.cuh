// Double-float ("pair") arithmetic and conversions shared by the CG kernels and the
// assembly: a value as an unevaluated FP32 pair h + l (~48 bits).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace adfem {

// ---- double-float arithmetic: a value as an unevaluated FP32 pair h + l (~48 bits).
// Explicitly rounded intrinsics keep the compiler from fusing or reassociating the error
// terms.  Used where FP64 would put long chains of dependent FP64 instructions on the
// critical path: on GB300 an FP64 instruction has a long latency as well as a low rate,
// and the end-of-launch reduction of the banded iteration (one warp, then one thread)
// measured ~10 us per iteration with FP64 sums and divisions.
__device__ __forceinline__ float2 df_norm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  return df_norm(s, e);
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return df_norm(p, e);
}
__device__ __forceinline__ float2 df_div(float2 a, float2 b) {
  const float q1 = __fdiv_rn(a.x, b.x);
  const float2 r = df_add(a, df_neg(df_mul(make_float2(q1, 0.0f), b)));
  const float q2 = __fdiv_rn(r.x, b.x);
  return df_norm(q1, q2);
}
__device__ __forceinline__ double df_to_d(float2 a) { return (double)a.x + (double)a.y; }
// a <= b for normalised pairs (|l| at most half an ulp of h)
__device__ __forceinline__ bool df_le(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y <= b.y); }
__device__ __forceinline__ float2 d_to_df(double d) {
  const float h = (float)d;
  return make_float2(h, (float)(d - (double)h));
}

// ---- conversions between FP64 and pairs with integer instructions.  On GB300 the FP64
// pipe, which also executes the FP64<->FP32 conversion instructions, retires ~0.5 T lane
// operations per second against ~37-40 T for the FP32 and integer pipes (measured with a
// throughput probe), so a conversion instruction costs as much as an FP64 add.
//
// d2p: h is d with its significand truncated to 24 bits, l the next (up to 29) bits
// truncated to 24 (|l| < ulp(h), together ~48 bits).  Integer path for |d| in [2^-74, 2^128),
// where both parts are normal floats; zero is exact; anything else takes the conversion
// instructions.
__device__ __forceinline__ float2 d2p(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hw = (unsigned)(b >> 32);
  const unsigned e = (hw >> 20) & 0x7FFu;
  const unsigned sign = hw & 0x80000000u;
  if (e >= 949u && e <= 1150u) {
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;  // 52 fraction bits
    const float h = __uint_as_float(sign | ((e - 896u) << 23) | (unsigned)(m >> 29));
    const unsigned rem = (unsigned)m & 0x1FFFFFFFu;       // the low 29 fraction bits
    float l = 0.0f;
    if (rem != 0u) {
      const unsigned lz = (unsigned)__clz(rem) - 3u;       // rem < 2^29: leading one moved to bit 28
      const unsigned rm = rem << lz;
      l = __uint_as_float(sign | ((e - 920u - lz) << 23) | ((rm >> 5) & 0x7FFFFFu));
    }
    return make_float2(h, l);
  }
  if ((b << 1) == 0ull) return make_float2(__uint_as_float(sign), 0.0f);
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - (double)h));
}
// exact FP32 -> FP64 with integer instructions for normal floats and zero
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e != 0u && e != 255u)
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
  if ((u << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)(u & 0x80000000u) << 32));
  return (double)f;
}
// pair -> FP64: h and l converted exactly, one FP64 add
__device__ __forceinline__ double p2d(float2 a) { return f2d_int(a.x) + f2d_int(a.y); }

}  // namespace adfem
