// Device helpers shared by the solver kernels.
#pragma once

#include <cstdint>

namespace cgb {

constexpr unsigned kFull = 0xffffffffu;

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

// tanh(x) = x P(z) / Q(z), z = min(x^2, 9.5^2): P and Q of degree 4 in z (a
// minimax-relative rational fit on [0, 9], derived by
// cochlearmodel_gb300/fit_tanh.py), Horner in z, quotient as x P times
// own_rcpf(Q) (Q >= 1), result clamped to [-1, 1].  From |x| = 9.5 on,
// |x| P / Q exceeds 1, so the result saturates to +-1 exactly (also for
// infinite x; NaN gives -1).  One branch-free path, <= 6.1 ulp (every float
// in [0, 9.5] checked against double tanh); the CPU oracle evaluates the same
// sequence.
__device__ __forceinline__ float own_tanhf(float x) {
  const float z = fminf(__fmul_rn(x, x), 90.25f);
  float p = 1.335385846346071e-08f;
  p = __fmaf_rn(p, z, 2.0608504200936295e-05f);
  p = __fmaf_rn(p, z, 0.0034955532755702734f);
  p = __fmaf_rn(p, z, 0.13380996882915497f);
  p = __fmaf_rn(p, z, 1.0f);
  float q = 7.776229722367134e-07f;
  q = __fmaf_rn(q, z, 0.00032855774043127894f);
  q = __fmaf_rn(q, z, 0.02587684988975525f);
  q = __fmaf_rn(q, z, 0.46714311838150024f);
  q = __fmaf_rn(q, z, 1.0f);
  const float t = __fmul_rn(__fmul_rn(x, p), own_rcpf(q));
  return fminf(fmaxf(t, -1.0f), 1.0f);
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

// own_tanhf on a pair: the same operation sequence per element.
__device__ __forceinline__ float2 own_tanhf2(float2 x) {
  const float2 z0 = mul2(x, x);
  const float2 z = f2(fminf(z0.x, 90.25f), fminf(z0.y, 90.25f));
  float2 p = f2b(1.335385846346071e-08f);
  p = fma2(p, z, f2b(2.0608504200936295e-05f));
  p = fma2(p, z, f2b(0.0034955532755702734f));
  p = fma2(p, z, f2b(0.13380996882915497f));
  p = fma2(p, z, f2b(1.0f));
  float2 q = f2b(7.776229722367134e-07f);
  q = fma2(q, z, f2b(0.00032855774043127894f));
  q = fma2(q, z, f2b(0.02587684988975525f));
  q = fma2(q, z, f2b(0.46714311838150024f));
  q = fma2(q, z, f2b(1.0f));
  const float2 t = mul2(mul2(x, p), own_rcpf2(q));
  return f2(fminf(fmaxf(t.x, -1.0f), 1.0f), fminf(fmaxf(t.y, -1.0f), 1.0f));
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
