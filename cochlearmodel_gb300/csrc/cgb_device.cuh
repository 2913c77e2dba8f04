// Device helpers shared by the solver kernels.
#pragma once

#include <cstdint>

namespace cgb {

constexpr unsigned kFull = 0xffffffffu;

// e^y for y >= 0 by Cody-Waite reduction y = k ln2 + r and a degree-8 Taylor
// polynomial of e^r; 2^k is assembled in the exponent field.  The order of
// every float operation is fixed (explicit fma, no contraction) so the CPU
// oracle, which evaluates the same sequence, rounds identically.
__device__ __forceinline__ float own_expf_pos(float y) {
  const float log2e = 1.44269504088896341f;
  const float ln2_hi = 0.693145751953125f;
  const float ln2_lo = 1.42860682030941723e-06f;
  float k = rintf(__fmul_rn(y, log2e));
  float r = __fmaf_rn(-k, ln2_hi, y);
  r = __fmaf_rn(-k, ln2_lo, r);
  float p = 1.0f / 40320.0f;
  p = __fmaf_rn(p, r, 1.0f / 5040.0f);
  p = __fmaf_rn(p, r, 1.0f / 720.0f);
  p = __fmaf_rn(p, r, 1.0f / 120.0f);
  p = __fmaf_rn(p, r, 1.0f / 24.0f);
  p = __fmaf_rn(p, r, 1.0f / 6.0f);
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  int ki = (int)k;
  float scale = __int_as_float((ki + 127) << 23);
  return __fmul_rn(p, scale);
}

// 1/d for a positive normal d without a branch: the classic bit-level seed
// 0x7EF311C3 - bits(d) (within ~12%) refined by three Newton steps
// r <- r + r(1 - d r); measured <= 0.5004 ulp over [1, 2) and across exponents.
__device__ __forceinline__ float own_rcpf(float d) {
  float r = __int_as_float(0x7EF311C3 - __float_as_int(d));
  r = __fmaf_rn(r, __fmaf_rn(-d, r, 1.0f), r);
  r = __fmaf_rn(r, __fmaf_rn(-d, r, 1.0f), r);
  r = __fmaf_rn(r, __fmaf_rn(-d, r, 1.0f), r);
  return r;
}

// tanh(x): odd Taylor series to x^21 below |x| = 0.55, 1 - 2/(e^{2|x|}+1)
// up to |x| = 20, +-1 beyond.  Both branches are evaluated and one is
// selected, so unrolled per-section calls keep their instruction-level
// parallelism (no divergent branch per section).
__device__ __forceinline__ float own_tanhf(float x) {
  const float ax = fabsf(x);
  const float x2 = __fmul_rn(x, x);
  float p = (float)(18888466084.0 / 194896477400625.0);
  p = __fmaf_rn(p, x2, (float)(-443861162.0 / 1856156927625.0));
  p = __fmaf_rn(p, x2, (float)(6404582.0 / 10854718875.0));
  p = __fmaf_rn(p, x2, (float)(-929569.0 / 638512875.0));
  p = __fmaf_rn(p, x2, (float)(21844.0 / 6081075.0));
  p = __fmaf_rn(p, x2, (float)(-1382.0 / 155925.0));
  p = __fmaf_rn(p, x2, (float)(62.0 / 2835.0));
  p = __fmaf_rn(p, x2, (float)(-17.0 / 315.0));
  p = __fmaf_rn(p, x2, (float)(2.0 / 15.0));
  p = __fmaf_rn(p, x2, (float)(-1.0 / 3.0));
  p = __fmul_rn(p, x2);
  const float tp = __fmaf_rn(p, x, x);
  const float e = own_expf_pos(__fmul_rn(2.0f, fminf(ax, 20.0f)));
  float te = __fmaf_rn(-2.0f, own_rcpf(__fadd_rn(e, 1.0f)), 1.0f);
  te = ax < 20.0f ? te : 1.0f;
  te = x < 0.0f ? -te : te;
  return ax < 0.55f ? tp : te;
}

// log10(x) for a positive normal x: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(s), s = (m-1)/(m+1), by its odd series to s^11, then
// log10 x = e log10(2) + ln(m) log10(e) (log10(2) split hi + lo).  <= 4 ulp.
__device__ __forceinline__ float own_log10f(float x) {
  const int ix = __float_as_int(x);
  int e = ((ix >> 23) & 0xff) - 127;
  float m = __int_as_float((ix & 0x7fffff) | 0x3f800000);
  const bool hi = m > 1.41421356f;
  m = hi ? __fmul_rn(m, 0.5f) : m;
  e += hi ? 1 : 0;
  const float f = __fsub_rn(m, 1.0f);
  const float s = __fmul_rn(f, own_rcpf(__fadd_rn(2.0f, f)));
  const float s2 = __fmul_rn(s, s);
  float p = 1.0f / 11.0f;
  p = __fmaf_rn(p, s2, 1.0f / 9.0f);
  p = __fmaf_rn(p, s2, 1.0f / 7.0f);
  p = __fmaf_rn(p, s2, 1.0f / 5.0f);
  p = __fmaf_rn(p, s2, 1.0f / 3.0f);
  const float two_s = __fmul_rn(2.0f, s);
  const float lnm = __fmaf_rn(__fmul_rn(two_s, s2), p, two_s);
  const float ef = (float)e;
  const float l2hi = 0.30102999566398120f;
  const float l2lo = (float)(0.30102999566398120 - (double)0.30102999566398120f);
  return __fmaf_rn(ef, l2hi, __fmaf_rn(ef, l2lo, __fmul_rn(lnm, 0.43429448190325182f)));
}

// Packed pairs of FP32 values: Blackwell's two-wide FP32 add / multiply /
// fma (add.rn.f32x2 and friends).  Every element rounds exactly like the
// scalar instruction, so a pair computation equals two scalar ones bit for
// bit; only the instruction count halves.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2b(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// a - b == a + (-b) exactly (negation is exact), signed zeros included
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 max2(float2 a, float2 b) {
  return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y));
}

// own_expf_pos on a pair: the same operation sequence per element.
__device__ __forceinline__ float2 own_expf_pos2(float2 y) {
  const float log2e = 1.44269504088896341f;
  const float ln2_hi = 0.693145751953125f;
  const float ln2_lo = 1.42860682030941723e-06f;
  const float2 kk = mul2(y, f2b(log2e));
  const float2 k = f2(rintf(kk.x), rintf(kk.y));
  float2 r = fma2(neg2(k), f2b(ln2_hi), y);
  r = fma2(neg2(k), f2b(ln2_lo), r);
  float2 p = f2b(1.0f / 40320.0f);
  p = fma2(p, r, f2b(1.0f / 5040.0f));
  p = fma2(p, r, f2b(1.0f / 720.0f));
  p = fma2(p, r, f2b(1.0f / 120.0f));
  p = fma2(p, r, f2b(1.0f / 24.0f));
  p = fma2(p, r, f2b(1.0f / 6.0f));
  p = fma2(p, r, f2b(0.5f));
  p = fma2(p, r, f2b(1.0f));
  p = fma2(p, r, f2b(1.0f));
  const float2 scale = f2(__int_as_float(((int)k.x + 127) << 23),
                          __int_as_float(((int)k.y + 127) << 23));
  return mul2(p, scale);
}

// own_rcpf on a pair.
__device__ __forceinline__ float2 own_rcpf2(float2 d) {
  float2 r = f2(__int_as_float(0x7EF311C3 - __float_as_int(d.x)),
                __int_as_float(0x7EF311C3 - __float_as_int(d.y)));
  const float2 nd = neg2(d);
  r = fma2(r, fma2(nd, r, f2b(1.0f)), r);
  r = fma2(r, fma2(nd, r, f2b(1.0f)), r);
  r = fma2(r, fma2(nd, r, f2b(1.0f)), r);
  return r;
}

// own_tanhf on a pair.
__device__ __forceinline__ float2 own_tanhf2(float2 x) {
  const float2 ax = abs2(x);
  const float2 x2 = mul2(x, x);
  float2 p = f2b((float)(18888466084.0 / 194896477400625.0));
  p = fma2(p, x2, f2b((float)(-443861162.0 / 1856156927625.0)));
  p = fma2(p, x2, f2b((float)(6404582.0 / 10854718875.0)));
  p = fma2(p, x2, f2b((float)(-929569.0 / 638512875.0)));
  p = fma2(p, x2, f2b((float)(21844.0 / 6081075.0)));
  p = fma2(p, x2, f2b((float)(-1382.0 / 155925.0)));
  p = fma2(p, x2, f2b((float)(62.0 / 2835.0)));
  p = fma2(p, x2, f2b((float)(-17.0 / 315.0)));
  p = fma2(p, x2, f2b((float)(2.0 / 15.0)));
  p = fma2(p, x2, f2b((float)(-1.0 / 3.0)));
  p = mul2(p, x2);
  const float2 tp = fma2(p, x, x);
  const float2 e = own_expf_pos2(mul2(f2b(2.0f), f2(fminf(ax.x, 20.0f), fminf(ax.y, 20.0f))));
  float2 te = fma2(f2b(-2.0f), own_rcpf2(add2(e, f2b(1.0f))), f2b(1.0f));
  te.x = ax.x < 20.0f ? te.x : 1.0f;
  te.y = ax.y < 20.0f ? te.y : 1.0f;
  te.x = x.x < 0.0f ? -te.x : te.x;
  te.y = x.y < 0.0f ? -te.y : te.y;
  return f2(ax.x < 0.55f ? tp.x : te.x, ax.y < 0.55f ? tp.y : te.y);
}

__device__ __forceinline__ float warp_sum_xor(float v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Maximum over the full warp in one instruction (redux.sync on f32, a
// Blackwell addition); callers pass no NaNs, so it equals the fmaxf
// butterfly exactly.
__device__ __forceinline__ float warp_max_xor(float v) {
  float r;
  asm volatile("redux.sync.max.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
  return r;
}

}  // namespace cgb
