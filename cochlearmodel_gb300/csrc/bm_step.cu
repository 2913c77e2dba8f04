// BM/OHC adaptive-step solver: reference kernel 17
// (include/cochlea.cuh:13573-14245) and the default BMOHC_NEW_kernel
// (include/cochlea.cuh:3486-4324), launched by BMOHCNewKernel
// (src/cochlea.cu:1436-1493, 2298-2330).
//
// GB300 layout: one WARP owns one unit (one time block of one signal); lane l
// holds sections 8l..8l+7 of every state vector in registers, as four
// two-wide FP32 pairs.  Two Jacobi sweeps take one round of four shuffles
// for a two-section halo and, in the own order with four or more sweeps, one
// update over the second neighbours (three two-wide fmas per pair) -- no
// shared-memory round trip and no block barrier, where the reference spends
// two __syncthreads per sweep across 256 threads.  The
// Lipschitz/fault reductions are xor-butterflies, so every lane holds the
// full result and takes the same step decision.  Units come from a device
// work queue, so a persistent grid of warps drains batches of uneven-length
// signals.
//
// Step controller (CTL):
//   0  kernel 17: a step needs another iteration while the SUM over sections
//      of |v - v_ref| - max(mtt, v dt) is positive.  Kernel 17's warp-0
//      reduction leaves the full sum only in lane 0 and its other lanes race
//      on the shared decision slots; this kernel takes the lane-0 value.
//   1  BMOHC_NEW_kernel: another iteration while ANY section has
//      |v - v_ref| > max(mtt, v dt) (its fault count, cochlea.cuh:4080-4100).
// Arithmetic (ARITH):
//   0  own fixed order, reproduced bit for bit by the CPU oracle: explicit
//      __fmaf_rn, own tanh and reciprocal, the step-size tests as products
//      (no division), and an iteration's four or more Jacobi sweeps taken
//      two at a time as one update over the second neighbours (the same
//      iterates in exact arithmetic, three roundings per section instead
//      of four).
//   1  BMOHC_NEW_kernel's own operation order: its fmaf placement, CUDA's
//      tanhf, __fdividef where it divides, its shared-memory tree order for
//      the velocity-error sum and one Jacobi sweep at a time; checked bit for
//      bit against the reference's compiled kernel.  (CUDA's tanhf gives the
//      same bits under --fmad=false as under the reference's default
//      --fmad=true, checked on every float input.)
//   Both keep simulated time in a float accumulator, as the reference does.
//
// Floating-point order is fixed: the file is compiled with --fmad=false and
// every fused multiply-add is an explicit __fmaf_rn.

#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>

#include "cgb_device.cuh"
#include "cgb_internal.h"
#include "warmstart.cuh"

namespace cgb {

constexpr int kSPL = 8;  // sections per lane

struct BMArgs {
  const float* secp;   // [8][256]: 1/M, 1/m, R, S, Q, S_ohc, S_tm, R_tm
  const float* gamma;  // [P][256]
  const cgb_unit* units;
  int n_units;
  const float* in;
  float* out;
  // host mirror of out (pinned, mapped): its byte offset from out, or 0 for
  // none; a row's host address is its device address plus the offset
  long long host_delta;
  int32_t* failed;
  float* conv;  // [rows][3] mean dt, substeps, mean outer iterations per sample
  cgb_unit_stats* stats;
  int32_t* work;
  float ratio, nas, al, e1, e2, nw, ar, dx2, dxa0, na1, na2, gme, sow;
  float dt0, dtmin, dtmax;
  // the reference's float constants 1/Ts, 1/sigma_ow (each formed in double
  // and rounded, src/cochlea.cu:1099,1105) and time_step_out
  float fs_f, rsow, tout_f;
  // sigma_ow is a power of two (its reciprocal rsow is exact), so x / sigma_ow
  // is x * rsow bit for bit
  int ow_pow2;
  int jfast, jslow, max_outer, max_sub;
  // tolerance mode (jacobi_mode 2)
  float jtol;
  int jcap, guess, learn_every;
  const unsigned char* ws_blob;  // packed network weights (guess 2)
  float* log;                    // training records [6][256] (optional)
  long long log_cap;
  int log_every;
  int* log_count;
};

__device__ __forceinline__ void load8(const float* p, float (&r)[kSPL]) {
  const float4 a = reinterpret_cast<const float4*>(p)[0];
  const float4 b = reinterpret_cast<const float4*>(p)[1];
  r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
  r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
}

__device__ __forceinline__ void store8(float* p, const float (&r)[kSPL]) {
  reinterpret_cast<float4*>(p)[0] = make_float4(r[0], r[1], r[2], r[3]);
  reinterpret_cast<float4*>(p)[1] = make_float4(r[4], r[5], r[6], r[7]);
}

// Sections of a lane as four mirror pairs: pair j holds sections 8l+j (x)
// and 8l+7-j (y).  The Jacobi neighbours of pair j are whole pairs j-1 and
// j+1 (for the y half the two swap roles, and the sum p_{s-1} + p_{s+1} is
// the same); the halo of the lane, sections 8l-1 and 8l+8 (and 8l-2, 8l+9),
// arrives as one pair, and the lane's own edge sections 8l, 8l+1, 8l+6, 8l+7
// sit in pairs 0 and 1 only.  Pair 3 is its own neighbour, swapped.
__device__ __forceinline__ void load8p(const float* p, float2 (&r)[4]) {
  const float4 a = reinterpret_cast<const float4*>(p)[0];
  const float4 b = reinterpret_cast<const float4*>(p)[1];
  r[0] = f2(a.x, b.w);
  r[1] = f2(a.y, b.z);
  r[2] = f2(a.z, b.y);
  r[3] = f2(a.w, b.x);
}

__device__ __forceinline__ void store8p(float* p, const float2 (&r)[4]) {
  reinterpret_cast<float4*>(p)[0] = make_float4(r[0].x, r[1].x, r[2].x, r[3].x);
  reinterpret_cast<float4*>(p)[1] = make_float4(r[3].y, r[2].y, r[1].y, r[0].y);
}

// Shared-memory copies of per-section vectors are laid out [half][lane][4]:
// lane l's eight sections in pair order (0,7,1,6 | 2,5,3,4) as two 16-byte
// halves, the first halves of all lanes contiguous, then the second halves.
// Each of the two 16-byte loads of a warp reads one contiguous 512-byte span
// (no bank conflicts) and lands as two whole register pairs (no repacking).
// p points at the vector plus 4 * lane floats.
__device__ __forceinline__ int smem_pos(int s) {
  const int c = s & 7, pp = c < 4 ? 2 * c : 2 * (7 - c) + 1;
  return ((pp >> 2) << 7) | ((s >> 3) << 2) | (pp & 3);
}

__device__ __forceinline__ void load8q(const float* p, float2 (&r)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  const float4 b = *reinterpret_cast<const float4*>(p + 128);
  r[0] = f2(a.x, a.y);
  r[1] = f2(a.z, a.w);
  r[2] = f2(b.x, b.y);
  r[3] = f2(b.z, b.w);
}

__device__ __forceinline__ void store8q(float* p, const float2 (&r)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(r[0].x, r[0].y, r[1].x, r[1].y);
  *reinterpret_cast<float4*>(p + 128) = make_float4(r[2].x, r[2].y, r[3].x, r[3].y);
}

// pairs -> sections 8l..8l+7 in order
__device__ __forceinline__ void unpair(const float2 (&r)[4], float (&o)[kSPL]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    o[j] = r[j].x;
    o[7 - j] = r[j].y;
  }
}

// ((t0 + t1) + (t2 + t3)) + ((t4 + t5) + (t6 + t7)) on the pair layout (the
// y halves add as (t7 + t6) + (t5 + t4): the same values, addition commutes)
__device__ __forceinline__ float pair_sum8p(const float2 (&t)[4]) {
  const float2 s = add2(add2(t[0], t[1]), add2(t[2], t[3]));
  return __fadd_rn(s.x, s.y);
}

// The previous-step state (x, v, a, y, u, psi, psi') of a unit lives either
// in registers or, with PREV_SMEM, in the first 7 x 256 floats of the warp's
// slice of shared memory, which frees 56 registers per thread at the cost of
// reloading it on every outer iteration.
template <bool PREV_SMEM>
struct PrevState {
  float2 r[7][4];
  float* sm;  // this lane in the warp's [9][256] slice (PREV_SMEM only)
  __device__ __forceinline__ void init(float* slice, int qb) {
    sm = slice;
#pragma unroll
    for (int j = 0; j < 7; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) r[j][k] = f2b(0.0f);
    if (PREV_SMEM)
#pragma unroll
      for (int j = 0; j < 7; ++j) store8q(sm + j * 256 + qb, r[j]);
  }
  __device__ __forceinline__ void load(int j, int qb, float2 (&o)[4]) const {
    if (PREV_SMEM) {
      load8q(sm + j * 256 + qb, o);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k] = r[j][k];
    }
  }
  __device__ __forceinline__ void store(int j, int qb, const float2 (&o)[4]) {
    if (PREV_SMEM) {
      store8q(sm + j * 256 + qb, o);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) r[j][k] = o[k];
    }
  }
};

// G and P_tm between the phases of an outer iteration: registers, or (with
// the previous-step state in shared memory) two more 256-float slots of the
// warp's slice, which keeps the bounded-register shapes free of spills.
template <bool IN_SMEM>
struct SideVec {
  float2 r[4];
  float* sm;  // this lane's position in the slot (IN_SMEM only)
  __device__ __forceinline__ void init(float* slot) {
    sm = slot;
#pragma unroll
    for (int k = 0; k < 4; ++k) r[k] = f2b(0.0f);
    if (IN_SMEM) store8q(sm, r);
  }
  __device__ __forceinline__ void put(const float2 (&o)[4]) {
    if (IN_SMEM) {
      store8q(sm, o);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) r[k] = o[k];
    }
  }
  __device__ __forceinline__ void get(float2 (&o)[4]) const {
    if (IN_SMEM) {
      load8q(sm, o);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k] = r[k];
    }
  }
};

// CUDA's tanhf and __fdividef on a pair (ARITH 1).
__device__ __forceinline__ float2 tanhf2(float2 x) { return f2(tanhf(x.x), tanhf(x.y)); }
__device__ __forceinline__ float2 fdividef2(float2 a, float2 b) {
  return f2(__fdividef(a.x, b.x), __fdividef(a.y, b.y));
}

// Sum over the 256 sections in BMOHC_NEW_kernel's order (ARITH 1): its
// shared-memory tree adds element i + t into element i for t = 128, 64, ...,
// 1 (include/cochlea.cuh:4057-4066).  Section s = 8l + j sits in lane l, so
// the strides 128..8 pair lanes l and l + 16..1 element by element (an xor
// butterfly leaves the same value in both lanes, addition commutes), and
// strides 4, 2, 1 finish inside the lane.  Every lane returns the sum.
__device__ __forceinline__ float ref_tree_sum(const float2 (&t)[4]) {
  float e[kSPL];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    e[j] = t[j].x;
    e[7 - j] = t[j].y;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int j = 0; j < kSPL; ++j) e[j] = __fadd_rn(e[j], __shfl_xor_sync(kFull, e[j], o));
#pragma unroll
  for (int j = 0; j < 4; ++j) e[j] = __fadd_rn(e[j], e[j + 4]);
  e[0] = __fadd_rn(e[0], e[2]);
  e[1] = __fadd_rn(e[1], e[3]);
  return __fadd_rn(e[0], e[1]);
}

// One unit, executed by one full warp.  sp: shared [8][256] section
// parameters; sg / sgs: shared gamma and gamma*S_ohc of the unit's profile
// (all three in pair order, as are the previous-step slice and hist).
// The per-section arithmetic runs on section pairs (two-wide FP32), each
// element rounding as the scalar sequence the CPU oracle (ARITH 0) or the
// reference's BMOHC_NEW_kernel (ARITH 1) evaluates.  CTL and ARITH: see the
// head of this file.
//
// TOL 0: fixed sweep counts (the reference schedule).  TOL 1: tolerance
// mode; each solve sweeps in pairs until max|p2 - p1| <= jtol * max|p2|
// (jcap sweeps at most), and the first solve of a step starts from the
// previous step's pressure (guess 0) or from its linear extrapolation
// p1 + rho (p1 - p2), rho = dt / dt_prev (guess 1).  TOL 2: as 1, with the
// network's correction of the extrapolation every learn_every-th step.
// hist: two 256-float slots per warp holding the pressure at the start of
// the last two steps; ws_scratch / wblob: inference scratch and weights.
template <bool PREV_SMEM, int TOL, int CTL, int ARITH>
__device__ __forceinline__ void run_unit(const BMArgs& A, const cgb_unit& un,
                                         const float* __restrict__ sp,
                                         const float* __restrict__ sg,
                                         const float* __restrict__ sgs, float* prev_slice,
                                         float* hist, unsigned char* ws_scratch,
                                         const unsigned char* wblob, int lane,
                                         cgb_unit_stats* st) {
  const int base = lane * kSPL, qb = lane * 4;
  const bool first = lane == 0, last = lane == 31;
  float2 rm[4];
  load8q(sp + 1 * 256 + qb, rm);
  // 1/m of the halo sections 8l-1 and 8l+8 (used by the paired sweeps)
  float2 rmh = f2(__shfl_up_sync(kFull, rm[0].y, 1), __shfl_down_sync(kFull, rm[0].x, 1));
  // Boundary sections without per-sweep fix-ups (reference schedule and
  // tolerance mode with the previous or extrapolated guess).  There the
  // pressure of section 255 is +0 at every point: Y_255 = 0 and its update
  // only sees p_256 = 0.  So (a) the left halo is shuffled with wrap-around,
  // and lane 0 reads p_255 = +0 as p_{-1}; (b) lane 0's halo section -1 gets
  // coefficient 0 and right-hand side +0 (from Yrm_255), so its update is +0;
  // (c) section 255's coefficient is 0, so its update is +0 whatever its
  // (finite) neighbours; (d) section 254's lower neighbour enters through
  // fma(0, p_253, p_255) = +0 = p_255.  Each value equals the fixed-up
  // sequence bit for bit.  The learned guess can leave p_255 != 0 before the
  // first sweep, so it keeps the explicit fix-ups.
  constexpr bool kWrap = TOL != 2;
  const int src_l = (lane + 31) & 31;
  float2 lo1 = f2b(1.0f);  // lower-neighbour factor of pair 1 (section 254)
  if (kWrap) {
    if (first) rmh.x = 0.0f;
    if (last) {
      rm[0].y = 0.0f;
      lo1.y = 0.0f;
    }
  }

  PrevState<PREV_SMEM> prev;
  prev.init(prev_slice, qb);
  float2 x[4], v[4], a[4], y[4], u[4], ps[4], dp[4];
  float2 p[4], Yrm[4];
  SideVec<PREV_SMEM> Gs, Ps;  // G and P_tm
  Gs.init(prev_slice + 7 * 256 + qb);
  Ps.init(prev_slice + 8 * 256 + qb);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x[k] = v[k] = a[k] = y[k] = u[k] = ps[k] = dp[k] = f2b(0.0f);
    p[k] = Yrm[k] = f2b(0.0f);
  }
  float w0 = 0.f, wd0 = 0.f, wdd0 = 0.f, w = 0.f, wd = 0.f, wdd = 0.f;

  const float mtt = un.mtt, mmspt = un.mmspt;
  const float* inb = A.in + un.in_base;
  float* outb = A.out + un.out_base * 256;
  int32_t* fb = A.failed ? A.failed + un.out_base : nullptr;
  float* cb = A.conv ? A.conv + un.out_base * 3 : nullptr;

  float dt = A.dt0;
  // simulated time since the current sample: a float accumulator, as the
  // reference's curr_time_f (include/cochlea.cuh:13642,14230)
  float tau_f = 0.0f;
  int n = un.start;
  float sx0 = inb[n], sx1 = inb[n + 1];
  int fail_flag = 0;
  long long n_sub = 0, n_it = 0, n_sw = 0;
  int n_failed = 0, n_written = 0, status = 0, sub_in_sample = 0;
  float smp_dt = 0.0f, smp_sub = 0.0f, smp_it = 0.0f;  // per-sample sums
  float dt_prev = dt, rho = 1.0f;

  while (n < un.end) {
    if (++sub_in_sample > A.max_sub) {  // dt collapsed: stop this unit, flag it
      status = 1;
      break;
    }
    int out_loop = 0, reset = 1, another = 1;
    if (TOL) {
      // rotate the pressure history: slot (n_sub & 1) receives p at the start
      // of this step, the other slot holds the start of the previous one
      rho = __fdiv_rn(dt, dt_prev);
      dt_prev = dt;
      store8q(hist + (n_sub & 1) * 256 + qb, p);
    }
    // sx[9] = curr_time_f * Fs, sx[10] = 1 - sx[9]
    // (include/cochlea.cuh:3925-3927)
    const float delta = __fmul_rn(tau_f, A.fs_f);
    const float smp = __fmaf_rn(sx1, delta, __fmul_rn(sx0, __fsub_rn(1.0f, delta)));
    // (s * 0.5) * dt == s * (dt * 0.5) exactly, so each trapezoid update is
    // one fma with the half step
    const float hdt = __fmul_rn(dt, 0.5f);
    const float2 dt2 = f2b(dt), hdt2 = f2b(hdt);
    do {
      // Predictor.  The first iteration of a step (or one after a reset) is
      // Euler, which is the trapezoid rule with the new-derivative slots
      // holding the previous derivatives: (d0 + d0) * 0.5 == d0 exactly, so
      // one code path serves both.
      float2 x0[4], v0[4], a0[4], y0[4], u0[4], ps0[4], dp0[4];
      prev.load(0, qb, x0);
      prev.load(1, qb, v0);
      prev.load(2, qb, a0);
      prev.load(3, qb, y0);
      prev.load(4, qb, u0);
      prev.load(5, qb, ps0);
      prev.load(6, qb, dp0);
      if (__all_sync(kFull, out_loop == 0 || reset)) {
        out_loop = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          a[k] = a0[k];
          u[k] = u0[k];
          dp[k] = dp0[k];
        }
        wd = wd0;
        wdd = wdd0;
      }
      float2 dv[4], fl[4];
      const float2 mtt2 = f2b(mtt);
      bool fault = false;  // CTL 1: some section of this lane fails the speed test
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 vn = fma2(add2(a0[k], a[k]), hdt2, v0[k]);
        dv[k] = abs2(sub2(vn, v[k]));
        const float2 thr = max2(mtt2, mul2(vn, dt2));
        if (CTL == 0) fl[k] = sub2(dv[k], thr);
        else fault = fault || dv[k].x > thr.x || dv[k].y > thr.y;
        v[k] = vn;
        x[k] = fma2(add2(v0[k], vn), hdt2, x0[k]);
        y[k] = fma2(add2(u0[k], u[k]), hdt2, y0[k]);
        ps[k] = fma2(add2(dp0[k], dp[k]), hdt2, ps0[k]);
      }
      w = __fmaf_rn(__fadd_rn(wd0, wd), hdt, w0);
      wd = __fmaf_rn(__fadd_rn(wdd0, wdd), hdt, wd0);
      // The velocity-error sum (ARITH 1: in the reference's tree order) and,
      // for CTL 0, the summed margin.  The whole-warp reductions are issued
      // here, where nothing waits on them, so their shuffle latency overlaps
      // the TM update and the sweeps (the tester runs only when reset == 0,
      // a warp-uniform condition).
      float ev = 0.0f, Fsum = 0.0f;
      bool faulty = false;
      if (__all_sync(kFull, reset == 0)) {
        ev = ARITH ? ref_tree_sum(dv) : warp_sum_xor(pair_sum8p(dv));
        if (CTL == 0) Fsum = warp_sum_xor(pair_sum8p(fl));
        else faulty = __any_sync(kFull, fault);
      }

      // OHC / TM coupling, G and the right-hand side Y (scaled by 1/m).
      const bool tm_update = out_loop < 2;
      // the G/Y section tables are loaded here, so that their shared-memory
      // latency passes under the TM update (2% of the step against loading
      // them next to their use)
      float2 Rs[4], Ss[4], Qs[4];
      load8q(sp + 2 * 256 + qb, Rs);
      load8q(sp + 3 * 256 + qb, Ss);
      load8q(sp + 4 * 256 + qb, Qs);
      {
        // the TM tables are loaded next to their use (short live ranges)
        if (tm_update) {
          float2 Stm[4], Rtm[4], gs[4], gm[4], Ptm[4];
          load8q(sp + 6 * 256 + qb, Stm);
          load8q(sp + 7 * 256 + qb, Rtm);
          load8q(sgs + qb, gs);
          load8q(sg + qb, gm);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float2 d = sub2(y[k], x[k]);
            const float2 Pohc = mul2(gs[k], d);
            const float2 targ = mul2(f2b(A.ratio), ps[k]);
            const float2 t = ARITH ? tanhf2(targ) : own_tanhf2(targ);
            const float2 dL = mul2(f2b(A.nas), t);
            const float2 Aa = mul2(f2b(A.al), fma2(t, t, f2b(-1.0f)));
            // ARITH 1: -w psi, + eta_1 d, + eta_2 v (include/cochlea.cuh:3842-3844)
            const float2 N1 =
                ARITH ? fma2(f2b(A.e2), v[k], fma2(f2b(A.e1), d, mul2(f2b(A.nw), ps[k])))
                      : fma2(f2b(A.e1), d, fma2(f2b(A.e2), v[k], mul2(f2b(A.nw), ps[k])));
            const float2 N = fma2(Stm[k], dL, mul2(mul2(N1, Rtm[k]), Aa));
            const float2 Pp = fma2(Stm[k], y[k], Pohc);
            const float2 num = fma2(neg2(gm[k]), N, Pp);
            const float2 den = mul2(Rtm[k], fma2(mul2(gm[k], Aa), f2b(A.e2), f2b(-1.0f)));
            if (ARITH) {
              u[k] = fdividef2(num, den);
            } else {
              const float2 q = mul2(num, own_rcpf2(abs2(den)));
              u[k] = f2(den.x < 0.0f ? -q.x : q.x, den.y < 0.0f ? -q.y : q.y);
            }
            Ptm[k] = fma2(Rtm[k], u[k], mul2(Stm[k], y[k]));
          }
          Ps.put(Ptm);
        }
        float2 Ptm[4], G[4];
        Ps.get(Ptm);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float2 g = mul2(Rs[k], fma2(f2b(A.ar), mul2(v[k], v[k]), f2b(1.0f)));
          g = fma2(g, v[k], mul2(Ss[k], x[k]));
          G[k] = sub2(neg2(g), Ptm[k]);
          float2 Yk = mul2(mul2(f2b(A.dx2), G[k]), Qs[k]);
          if (k == 0 && first) {  // section 0
            if (ARITH)  // -a2 w' + -a1 w + Gme smp, then dx a0 (cochlea.cuh:3940-3943)
              Yk.x = __fmul_rn(A.dxa0, __fmaf_rn(A.gme, smp,
                                                 __fmaf_rn(A.na1, w, __fmul_rn(A.na2, wd))));
            else
              Yk.x = __fmul_rn(A.dxa0,
                               __fmaf_rn(A.na1, w, __fmaf_rn(A.na2, wd, __fmul_rn(A.gme, smp))));
          }
          if (k == 0 && last) Yk.y = 0.0f;  // section 255
          // ARITH 0 sweeps with Y/m formed once; ARITH 1 keeps Y (it sweeps
          // (Y - t) * (1/m), cochlea.cuh:3963-3965)
          Yrm[k] = ARITH ? Yk : mul2(Yk, rm[k]);
        }
        Gs.put(G);
      }

      // Jacobi sweeps on the pressure; p persists across iterations and steps.
      // Sweeps run in pairs: a lane fetches a halo of two sections on each
      // side, computes the first sweep on sections 8l-1..8l+8 (the two halo
      // sections duplicate exactly what the neighbours compute) and the
      // second on its own sections, so one shuffle round serves two sweeps.
      // Sections 254 and 255 carry no lower coefficient; p_{-1} = p_256 = 0.
      const int J = TOL ? A.jcap : (tm_update ? A.jslow : A.jfast);
      const float2 Yrmh = f2(kWrap ? __shfl_sync(kFull, Yrm[0].y, src_l)
                                   : __shfl_up_sync(kFull, Yrm[0].y, 1),
                             __shfl_down_sync(kFull, Yrm[0].x, 1));
      if (TOL && out_loop == 0 && n_sub >= 2) {
        float2 p2[4];
        load8q(hist + ((n_sub + 1) & 1) * 256 + qb, p2);
        if (A.log && n_sub % A.log_every == 0) {
          int idx = 0;
          if (lane == 0) idx = atomicAdd(A.log_count, 1);
          idx = __shfl_sync(kFull, idx, 0);
          if (idx < A.log_cap) {
            float* rec = A.log + (long long)idx * 6 * 256;
            store8p(rec + 0 * 256 + base, Yrm);
            store8p(rec + 1 * 256 + base, p);
            store8p(rec + 2 * 256 + base, p2);
            store8p(rec + 3 * 256 + base, v);
            store8p(rec + 4 * 256 + base, x);
            float meta[kSPL] = {lane == 0 ? rho : 0.0f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            store8(rec + 5 * 256 + base, meta);
          }
        }
        if (TOL == 2 && n_sub % A.learn_every == 0) {
          const float* wb = reinterpret_cast<const float*>(wblob + ws::kOffBias);
          float cY[kSPL], cp[kSPL], cp2[kSPL], cv[kSPL], cx[kSPL], crm[kSPL], pe[kSPL];
          unpair(Yrm, cY);
          unpair(p, cp);
          unpair(p2, cp2);
          unpair(v, cv);
          unpair(x, cx);
          unpair(rm, crm);
          const float nr = ws::make_features(cY, cp, cp2, cv, cx, crm, rho, wb[201], pe,
                                             ws_scratch, 8, lane);
          __syncwarp();
          ws::infer_unit(wblob, ws_scratch, lane);
          float2 o[4];
          load8p(reinterpret_cast<const float*>(ws_scratch + ws::kOffOut) + base, o);
          const float sc = __fmul_rn(nr, wb[200]);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            p[k] = fma2(f2b(sc), o[k], f2(pe[k], pe[7 - k]));
          n_sw += 1;  // the residual sweep of the features
          __syncwarp();
        } else if (A.guess >= 1) {
#pragma unroll
          for (int k = 0; k < 4; ++k) p[k] = fma2(f2b(rho), sub2(p[k], p2[k]), p[k]);
        }
      }
      // two sweeps with one shuffle round; q holds the first sweep's result
      float2 q[4];
      auto sweep_pair = [&]() {
        float2 T[4];
        // halo pairs: (8l-1, 8l+8) and (8l-2, 8l+9)
        float2 H, H2;
        if (kWrap) {
          H = f2(__shfl_sync(kFull, p[0].y, src_l), __shfl_down_sync(kFull, p[0].x, 1));
          H2 = f2(__shfl_sync(kFull, p[1].y, src_l), __shfl_down_sync(kFull, p[1].x, 1));
        } else {
          H = f2(__shfl_up_sync(kFull, p[0].y, 1), __shfl_down_sync(kFull, p[0].x, 1));
          H2 = f2(__shfl_up_sync(kFull, p[1].y, 1), __shfl_down_sync(kFull, p[1].x, 1));
          if (first) H.x = 0.0f;
        }
        // the first sweep on the halo sections 8l-1 and 8l+8
        float2 qh = fma2(neg2(add2(H2, p[0])), rmh, Yrmh);
        if (!kWrap) {
          if (first) qh.x = 0.0f;
          if (last) qh.y = 0.0f;
        }
        // t_s = p_{s-1} + p_{s+1} on the mirror pairs
        T[0] = add2(H, p[1]);
        T[1] = kWrap ? fma2(lo1, p[2], p[0]) : add2(p[2], p[0]);
        T[2] = add2(p[1], p[3]);
        T[3] = f2(__fadd_rn(p[2].x, p[3].y), __fadd_rn(p[2].y, p[3].x));
        if (!kWrap && last) {
          T[0].y = 0.0f;
          T[1].y = p[0].y;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = fma2(neg2(T[k]), rm[k], Yrm[k]);
        T[0] = add2(qh, q[1]);
        T[1] = kWrap ? fma2(lo1, q[2], q[0]) : add2(q[2], q[0]);
        T[2] = add2(q[1], q[3]);
        T[3] = f2(__fadd_rn(q[2].x, q[3].y), __fadd_rn(q[2].y, q[3].x));
        if (!kWrap && last) {
          T[0].y = 0.0f;
          T[1].y = q[0].y;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = fma2(neg2(T[k]), rm[k], Yrm[k]);
      };
      // Own order, four or more sweeps: pairs of sweeps as one update over
      // the second neighbours, p''_s = C_s + a_s p_{s-2} + b_s p_s + c_s p_{s+2}
      // (C = one sweep applied to Y/m; the coefficient rows are built per CTA
      // in bm_body).  Three fmas per section instead of two sweeps' four
      // operations, no halo sections, and one dependent fma after the
      // shuffles.  On the mirror pairs both second neighbours are whole
      // pairs: p[k-2] (the halos H2, H for k = 0, 1) holds the lower one of
      // the pair's x section and the upper one of its y section, p[k+2]
      // (p[3], p[2] swapped for k = 2, 3) the other two.  Row 8 multiplies
      // the first, row 9 the second, which is added first: sections
      // 8l..8l+3 add the upper term before the lower, 8l+4..8l+7 the lower
      // before the upper.  Beyond the ends the wrapped and clamped shuffles
      // deliver p_254, p_255 (below sections 0, 1) and p_248, p_249 (above
      // 254, 255), each times a zero coefficient.
      float2 C2[4], KL[4], KH[4], KB[4];
      auto two_step_setup = [&]() {
        load8q(sp + 8 * 256 + qb, KL);
        load8q(sp + 9 * 256 + qb, KH);
        load8q(sp + 10 * 256 + qb, KB);
        float2 T[4];
        T[0] = add2(Yrmh, Yrm[1]);
        T[1] = fma2(lo1, Yrm[2], Yrm[0]);
        T[2] = add2(Yrm[1], Yrm[3]);
        T[3] = f2(__fadd_rn(Yrm[2].x, Yrm[3].y), __fadd_rn(Yrm[2].y, Yrm[3].x));
#pragma unroll
        for (int k = 0; k < 4; ++k) C2[k] = fma2(neg2(T[k]), rm[k], Yrm[k]);
      };
      auto two_step = [&]() {
        const float2 H =
            f2(__shfl_sync(kFull, p[0].y, src_l), __shfl_down_sync(kFull, p[0].x, 1));
        const float2 H2 =
            f2(__shfl_sync(kFull, p[1].y, src_l), __shfl_down_sync(kFull, p[1].x, 1));
        float2 r[4];
        r[0] = fma2(KL[0], H2, fma2(KH[0], p[2], fma2(KB[0], p[0], C2[0])));
        r[1] = fma2(KL[1], H, fma2(KH[1], p[3], fma2(KB[1], p[1], C2[1])));
        r[2] = fma2(KL[2], p[0], fma2(KH[2], f2(p[3].y, p[3].x), fma2(KB[2], p[2], C2[2])));
        r[3] = fma2(KL[3], p[1], fma2(KH[3], f2(p[2].y, p[2].x), fma2(KB[3], p[3], C2[3])));
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = r[k];
      };
      int it = 0;
      if (ARITH) {
        // BMOHC_NEW_kernel's sweep, one at a time: p_s <- (Y_s - t_s) / m_s
        // with t_s = l_s p_{s-1} + p_{s+1} (l_s = 0 on 254, 255) and
        // p_{-1} = p_256 = 0 (include/cochlea.cuh:3958-3967)
        for (; it < J; ++it) {
          float2 H = f2(__shfl_up_sync(kFull, p[0].y, 1), __shfl_down_sync(kFull, p[0].x, 1));
          if (first) H.x = 0.0f;
          if (last) H.y = 0.0f;
          float2 T[4];
          T[0] = add2(H, p[1]);
          T[1] = add2(p[2], p[0]);
          T[2] = add2(p[1], p[3]);
          T[3] = f2(__fadd_rn(p[2].x, p[3].y), __fadd_rn(p[2].y, p[3].x));
          if (last) {
            T[0].y = H.y;
            T[1].y = p[0].y;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) p[k] = mul2(sub2(Yrm[k], T[k]), rm[k]);
        }
      } else if (!TOL && J == 20) {
        // the reference schedule's slow count, fully unrolled
        two_step_setup();
#pragma unroll
        for (int r = 0; r < 10; ++r) two_step();
        it = 20;
      } else if (!TOL && J == 2) {
        // and its fast count, one pair without the loop
        sweep_pair();
        it = 2;
      } else if (!TOL && J >= 4) {
        two_step_setup();
        for (; it + 1 < J; it += 2) two_step();
      } else {
#pragma unroll 2
        for (; it + 1 < J; it += 2) {
          sweep_pair();
          if (TOL) {
            float dm = 0.0f, pm = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const float2 e = abs2(sub2(p[k], q[k]));
              const float2 ap = abs2(p[k]);
              dm = fmaxf(dm, fmaxf(e.x, e.y));
              pm = fmaxf(pm, fmaxf(ap.x, ap.y));
            }
            dm = warp_max_xor(dm);
            pm = warp_max_xor(pm);
            if (__all_sync(kFull, dm <= __fmul_rn(A.jtol, pm))) {
              it += 2;
              break;
            }
          }
        }
      }
      if (!TOL && !ARITH && it < J) {
        float2 H = f2(__shfl_up_sync(kFull, p[0].y, 1), __shfl_down_sync(kFull, p[0].x, 1));
        if (first) H.x = 0.0f;
        if (last) H.y = 0.0f;
        float2 T[4];
        T[0] = add2(H, p[1]);
        T[1] = add2(p[2], p[0]);
        T[2] = add2(p[1], p[3]);
        T[3] = f2(__fadd_rn(p[2].x, p[3].y), __fadd_rn(p[2].y, p[3].x));
        if (last) {
          T[0].y = H.y;
          T[1].y = p[0].y;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = fma2(neg2(T[k]), rm[k], Yrm[k]);
      }
      n_sw += TOL ? it : J;

      const float p0 = __shfl_sync(kFull, p[0].x, 0);
      float2 da[4];
      {
        float2 invM[4];
        load8q(sp + 0 * 256 + qb, invM);
        float2 G[4];
        Gs.get(G);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float2 an = mul2(add2(p[k], G[k]), invM[k]);
          da[k] = abs2(sub2(a[k], an));
          a[k] = an;
          const float2 d = sub2(y[k], x[k]);
          if (ARITH)  // eta_2 (u - v), + eta_1 d, + -w psi (cochlea.cuh:4010-4013)
            dp[k] = fma2(f2b(A.nw), ps[k],
                         fma2(f2b(A.e1), d, mul2(f2b(A.e2), sub2(u[k], v[k]))));
          else
            dp[k] = fma2(f2b(A.e1), d,
                         fma2(f2b(A.e2), sub2(u[k], v[k]), mul2(f2b(A.nw), ps[k])));
        }
      }
      if (ARITH)  // oval window: (-a1 w + -a2 w') + (Gme smp + p_0), times 1/sigma_ow
        wdd = __fmul_rn(A.rsow, __fadd_rn(__fmaf_rn(A.na2, wd, __fmul_rn(A.na1, w)),
                                          __fmaf_rn(A.gme, smp, p0)));
      else {
        const float ws = __fmaf_rn(A.na1, w, __fmaf_rn(A.na2, wd, __fmaf_rn(A.gme, smp, p0)));
        wdd = A.ow_pow2 ? __fmul_rn(ws, A.rsow) : __fdiv_rn(ws, A.sow);
      }

      if (reset == 0) {
        const float2 m = max2(max2(da[0], da[1]), max2(da[2], da[3]));
        const float eap = fmaxf(0.0f, fmaxf(m.x, m.y));
        const float ea = warp_max_xor(eap);
        // CTL 0: the summed margin; CTL 1: any failing section
        if (CTL == 0) faulty = Fsum > 0.0f;
        const float num = __fmul_rn(ea, dt);
        // L = ea dt / ev (0 unless ev > mmspt).  ARITH 1 divides as the
        // reference does; ARITH 0 tests L > 6 as num > 6 ev and L < 0.5 as
        // num < 0.5 ev, with 6 ev rounded once (no division on the step's
        // critical path).
        const bool lcheck = ev > mmspt;
        const float L = lcheck && ARITH ? __fdividef(num, ev) : 0.0f;
        const bool l_big = ARITH ? L > 6.0f : lcheck && num > __fmul_rn(6.0f, ev);
        const bool l_small = ARITH ? L < 0.5f : !lcheck || num < __fmul_rn(0.5f, ev);
        // Step decisions are the same in every lane (they come from warp
        // reductions and uniform counters); taking them through a vote makes
        // that visible to the compiler, which then branches without
        // reconvergence barriers.
        if (__all_sync(kFull, l_big)) {
          dt = __fmul_rn(dt, 0.5f);
          if (dt < A.dtmin) dt = A.dtmin;
          another = 0;
          reset = 1;
        } else if (__all_sync(kFull, faulty)) {
          another = 1;
          reset = 0;
        } else if (__all_sync(kFull, l_small)) {
          dt = __fmul_rn(dt, 2.0f);
          if (dt > A.dtmax) dt = A.dtmax;
          another = 0;
          reset = 1;
        } else {
          another = 1;
          reset = 0;
        }
      } else {
        another = 1;
        reset = 0;
      }
      ++out_loop;
      if (out_loop >= A.max_outer) {
        another = 0;
        reset = 1;
        fail_flag = 1;
      }
    } while (__all_sync(kFull, another));
    ++n_sub;
    n_it += out_loop;
    smp_sub = __fadd_rn(smp_sub, 1.0f);
    smp_dt = __fadd_rn(smp_dt, dt);
    smp_it = __fadd_rn(smp_it, (float)out_loop);

    if (__all_sync(kFull, tau_f > A.tout_f)) {
      tau_f = __fsub_rn(tau_f, A.tout_f);
      sx0 = sx1;
      sx1 = inb[n + 2];
      if (__all_sync(kFull, n >= un.out_first)) {
        store8p(outb + (int64_t)n * 256 + base, v);
        if (A.host_delta)
          store8p(reinterpret_cast<float*>(reinterpret_cast<char*>(outb + (int64_t)n * 256 + base) +
                                           A.host_delta),
                  v);
        if (fb && lane == 0) fb[n] = fail_flag;
        if (cb && lane == 0) {
          cb[(int64_t)n * 3 + 0] = __fdiv_rn(smp_dt, smp_sub);
          cb[(int64_t)n * 3 + 1] = smp_sub;
          cb[(int64_t)n * 3 + 2] = __fdiv_rn(smp_it, smp_sub);
        }
        ++n_written;
        n_failed += fail_flag;
      }
      fail_flag = 0;
      sub_in_sample = 0;
      smp_dt = smp_sub = smp_it = 0.0f;
      ++n;
    }
    prev.store(0, qb, x);
    prev.store(1, qb, v);
    prev.store(2, qb, a);
    prev.store(3, qb, y);
    prev.store(4, qb, u);
    prev.store(5, qb, ps);
    prev.store(6, qb, dp);
    w0 = w;
    wd0 = wd;
    wdd0 = wdd;
    tau_f = __fadd_rn(tau_f, dt);
  }
  if (st && lane == 0) {
    st->substeps = n_sub;
    st->iterations = n_it;
    st->sweeps = n_sw;
    st->failed_samples = n_failed;
    st->written_samples = n_written;
    st->status = status;
  }
}

// Dynamic shared memory (TOL >= 1): per warp two 256-float history slots;
// TOL 2 adds the packed weights and the per-warp inference scratch.
template <int WARPS, int TOL>
constexpr int bm_dyn_smem() {
  return TOL == 0 ? 0
                  : WARPS * 2 * 256 * 4 +
                        (TOL == 2 ? ws::kBlobBytes + WARPS * ws::kWarpScratch : 0);
}

template <int WARPS, bool PREV_SMEM, int TOL, int CTL, int ARITH>
__device__ __forceinline__ void bm_body(const BMArgs& A) {
  // rows 0-7: the section vectors of d_secp; 8-10 (own order, fixed sweep
  // counts only): the two-step sweep coefficients derived from row 1 (1/m)
  constexpr bool kTwoStep = TOL == 0 && ARITH == 0;
  __shared__ __align__(16) float s_par[(kTwoStep ? 11 : 8) * 256];
  __shared__ __align__(16) float s_gam[WARPS][2][256];
  __shared__ __align__(16) float s_prev[PREV_SMEM ? WARPS : 1][PREV_SMEM ? 9 * 256 : 4];
  extern __shared__ __align__(16) unsigned char s_dyn[];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
    s_par[(i & ~255) | smem_pos(i & 255)] = A.secp[i];
  __syncthreads();
  // Two-step sweep coefficients (run_unit), each one FP32 product of 1/m
  // values: a_s = rm_s rm_{s-1} (2 <= s <= 253), c_s = rm_s rm_{s+1}
  // (s <= 253), b_s = rm_s (l_s rm_{s-1} + l_{s+1} rm_{s+1}) with l_s = 0 on
  // sections 254, 255 and rm_{-1} = rm_256 = 0.  Row 8 multiplies the
  // neighbour pair p[k-2], which holds the lower second neighbour of an x
  // section (s mod 8 < 4: a_s) and the upper one of a y section (c_s); row 9
  // the other one; row 10 b_s.
  for (int s = threadIdx.x; kTwoStep && s < 256; s += blockDim.x) {
    const float r = s_par[256 + smem_pos(s)];
    const float rl = s >= 1 ? s_par[256 + smem_pos(s - 1)] : 0.0f;
    const float ru = s <= 254 ? s_par[256 + smem_pos(s + 1)] : 0.0f;
    const float a = (s >= 2 && s <= 253) ? __fmul_rn(r, rl) : 0.0f;
    const float c = s <= 253 ? __fmul_rn(r, ru) : 0.0f;
    const float b =
        __fmul_rn(r, __fadd_rn((s >= 1 && s <= 253) ? rl : 0.0f, s <= 252 ? ru : 0.0f));
    const bool x_half = (s & 7) < 4;
    const int q = smem_pos(s);
    s_par[8 * 256 + q] = x_half ? a : c;
    s_par[9 * 256 + q] = x_half ? c : a;
    s_par[10 * 256 + q] = b;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* hist = nullptr;
  unsigned char* wblob = nullptr;
  unsigned char* scratch = nullptr;
  if (TOL) {
    hist = reinterpret_cast<float*>(s_dyn) + warp * 512;
    for (int i = lane; i < 512; i += 32) hist[i] = 0.0f;
  }
  if (TOL == 2) {
    wblob = s_dyn + WARPS * 2 * 256 * 4;
    scratch = wblob + ws::kBlobBytes + warp * ws::kWarpScratch;
    const uint4* src = reinterpret_cast<const uint4*>(A.ws_blob);
    uint4* dst = reinterpret_cast<uint4*>(wblob);
    for (int i = threadIdx.x; i < ws::kBlobBytes / 16; i += blockDim.x) dst[i] = src[i];
    // zero rows stay zero: feature rows outside the unit, hidden-buffer tails
    uint4* z = reinterpret_cast<uint4*>(scratch);
    for (int i = lane; i < ws::kWarpScratch / 16; i += 32) z[i] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  for (;;) {
    int uid = 0;
    if (lane == 0) uid = atomicAdd(A.work, 1);
    uid = __shfl_sync(kFull, uid, 0);
    if (uid >= A.n_units) break;
    const cgb_unit un = A.units[uid];
    const float* g = A.gamma + (int64_t)un.profile * 256;
#pragma unroll
    for (int k = 0; k < kSPL; ++k) {
      const int s = lane * kSPL + k, q = smem_pos(s);
      const float gm = g[s];
      s_gam[warp][0][q] = gm;
      s_gam[warp][1][q] = __fmul_rn(gm, s_par[5 * 256 + q]);
    }
    __syncwarp();
    run_unit<PREV_SMEM, TOL, CTL, ARITH>(A, un, s_par, s_gam[warp][0], s_gam[warp][1],
                             PREV_SMEM ? s_prev[warp] : nullptr, hist, scratch, wblob, lane,
                             A.stats ? A.stats + uid : nullptr);
    __syncwarp();
  }
}

template <int WARPS, int MINB, bool PREV_SMEM, int TOL, int CTL, int ARITH>
__global__ void __launch_bounds__(WARPS * 32, MINB) bm_warp_kernel(const BMArgs A) {
  bm_body<WARPS, PREV_SMEM, TOL, CTL, ARITH>(A);
}

// Launch shapes built: (warps per CTA, minimum resident CTAs per SM the
// register allocation is bounded for, previous-step state in shared
// memory).  Shape 0: registers only, up to 255 per thread (2 CTAs of 4 warps
// per SM); 1: bounded for 3 CTAs; 2, 3: the same with the previous-step
// state in shared memory.  (Tighter register caps spill and measure
// slower: 10 warps per SM at 200 registers 1.7x, 12 warps at 168 1.06x.)
struct LaunchShape {
  const void* fn;
  void (*launch)(unsigned, cudaStream_t, const BMArgs&);
  int dyn_smem;
  int warps;
};

template <int W, int M, bool PS, int TOL, int CTL, int ARITH>
void launch_shape(unsigned grid, cudaStream_t st, const BMArgs& A) {
  bm_warp_kernel<W, M, PS, TOL, CTL, ARITH><<<grid, W * 32, bm_dyn_smem<W, TOL>(), st>>>(A);
}

#define CGB_SHAPE(W, M, PS, TOL, CTL, ARITH)                                        \
  {reinterpret_cast<const void*>(bm_warp_kernel<W, M, PS, TOL, CTL, ARITH>),           \
   launch_shape<W, M, PS, TOL, CTL, ARITH>, bm_dyn_smem<W, TOL>(), W}

const LaunchShape kShapes[] = {
    CGB_SHAPE(4, 1, false, 0, 0, 0),
    CGB_SHAPE(4, 3, false, 0, 0, 0),
    CGB_SHAPE(4, 1, true, 0, 0, 0),
    CGB_SHAPE(4, 3, true, 0, 0, 0),
};
// Tolerance-mode kernels: plain / extrapolated guess, and the learned guess.
const LaunchShape kTolShape = CGB_SHAPE(4, 1, false, 1, 0, 0);
const LaunchShape kLearnedShape = CGB_SHAPE(4, 1, false, 2, 0, 0);
// BMOHC_NEW_kernel's controller, in the own order and in the reference's.
const LaunchShape kCountShape = CGB_SHAPE(4, 1, false, 0, 1, 0);
const LaunchShape kRefArithShape = CGB_SHAPE(4, 1, false, 0, 1, 1);
int g_shape = 0;

}  // namespace cgb

extern "C" int cgb_bm_set_launch_shape(int shape) {
  if (shape < 0 || shape >= (int)(sizeof(cgb::kShapes) / sizeof(cgb::kShapes[0])))
    return cgb::fail(CGB_ERR_ARG, "cgb_bm_set_launch_shape: unknown shape");
  cgb::g_shape = shape;
  return CGB_OK;
}

extern "C" int cgb_bm_launch_shape_count(void) {
  return (int)(sizeof(cgb::kShapes) / sizeof(cgb::kShapes[0]));
}

extern "C" int cgb_bm_run_dev(const float* d_secp, const float* d_gamma, int n_profiles,
                              const cgb_bm_scalars* sc, const cgb_unit* d_units, int n_units,
                              const float* d_in, int64_t in_len, float* d_out,
                              int64_t out_rows, int32_t* d_failed, float* d_conv,
                              cgb_unit_stats* d_stats,
                              int32_t* d_work, void* stream) {
  return cgb_bm_run_ex_dev(d_secp, d_gamma, n_profiles, sc, d_units, n_units, d_in, in_len, d_out,
                           out_rows, d_failed, d_conv, d_stats, d_work, nullptr, stream);
}

extern "C" int cgb_bm_run_ex_dev(const float* d_secp, const float* d_gamma, int n_profiles,
                                 const cgb_bm_scalars* sc, const cgb_unit* d_units, int n_units,
                                 const float* d_in, int64_t in_len, float* d_out,
                                 int64_t out_rows, int32_t* d_failed, float* d_conv,
                                 cgb_unit_stats* d_stats, int32_t* d_work,
                                 const cgb_bm_extras* ex, void* stream) {
  using namespace cgb;
  if (n_units == 0) return CGB_OK;  // an empty table enqueues nothing
  if (!d_secp || !d_gamma || !sc || !d_units || !d_in || !d_out || !d_work)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: null pointer argument");
  if (n_units < 0 || n_profiles <= 0 || in_len <= 0 || out_rows <= 0)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: bad sizes");
  if (sc->red_lanes != 32 || (sc->jacobi_mode != 0 && sc->jacobi_mode != 2))
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: only red_lanes=32, jacobi_mode 0 or 2 are built");
  if (sc->controller != 0 && sc->controller != 1)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: controller must be 0 (kernel 17) or 1 "
                             "(BMOHC_NEW_kernel)");
  if (sc->arith != 0 && sc->arith != 1)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: arith must be 0 (own order) or 1 (reference)");
  if (sc->arith == 1 && sc->controller != 1)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: arith 1 is built for controller 1 only");
  if (sc->controller == 1 && sc->jacobi_mode != 0)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: controller 1 is built for jacobi_mode 0 only");
  if (sc->jacobi_fast < 0 || sc->jacobi_slow < 0 || sc->max_outer < 1 ||
      sc->max_substeps_per_sample < 1)
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: bad loop counts");
  const bool tol = sc->jacobi_mode == 2;
  if (tol && (sc->jacobi_cap < 2 || (sc->jacobi_cap & 1) || !(sc->jacobi_tol >= 0.0f) ||
              sc->guess_mode < 0 || sc->guess_mode > 2))
    return fail(CGB_ERR_ARG,
                "cgb_bm_run_dev: jacobi_mode 2 needs an even jacobi_cap >= 2, jacobi_tol >= 0 "
                "and guess_mode 0, 1 or 2");
  const bool learned = tol && sc->guess_mode == 2;
  if (learned && (!ex || !ex->d_ws_blob || sc->learned_every < 1))
    return fail(CGB_ERR_ARG,
                "cgb_bm_run_dev: guess_mode 2 needs network weights and learned_every >= 1");
  if (ex && ex->d_log && (!tol || !ex->d_log_count || ex->log_every < 1 || ex->log_cap < 0))
    return fail(CGB_ERR_ARG,
                "cgb_bm_run_dev: logging needs jacobi_mode 2, a counter and log_every >= 1");
  if (learned && (reinterpret_cast<uintptr_t>(ex->d_ws_blob) & 15))
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: the weight blob must be 16-byte aligned");
  if ((reinterpret_cast<uintptr_t>(d_out) & 15) || (reinterpret_cast<uintptr_t>(d_secp) & 15))
    return fail(CGB_ERR_ARG, "cgb_bm_run_dev: d_out and d_secp must be 16-byte aligned");
  if (ex && ex->h_out) {
    if (ex->h_out_bytes < out_rows * 256 * (int64_t)sizeof(float))
      return fail(CGB_ERR_RANGE, "cgb_bm_run_dev: h_out is shorter than out_rows x 256 floats");
    const int rc = check_host_mirror(ex->h_out, "cgb_bm_run_dev: h_out");
    if (rc) return rc;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BMArgs A{};
  A.secp = d_secp;
  A.gamma = d_gamma;
  A.units = d_units;
  A.n_units = n_units;
  A.in = d_in;
  A.out = d_out;
  A.host_delta = ex && ex->h_out ? (long long)(reinterpret_cast<uintptr_t>(ex->h_out) -
                                               reinterpret_cast<uintptr_t>(d_out))
                                  : 0;
  A.failed = d_failed;
  A.conv = d_conv;
  A.stats = d_stats;
  A.work = d_work;
  const bool ref_arith = sc->arith == 1;
  // ARITH 1 takes alpha_L / alpha_s formed in double and rounded, as the
  // reference host does for the kernels' constant (src/cochlea.cu:1104)
  A.ratio = ref_arith ? (float)((double)sc->alpha_l / (double)sc->alpha_s)
                      : sc->alpha_l / sc->alpha_s;
  A.fs_f = (float)(1.0 / (double)sc->Ts);
  A.rsow = (float)(1.0 / (double)sc->sigma_ow);
  {
    int e = 0;
    const double m = std::frexp((double)sc->sigma_ow, &e);
    // a normal power of two whose reciprocal is normal too
    A.ow_pow2 = m == 0.5 && std::fpclassify(sc->sigma_ow) == FP_NORMAL &&
                std::fpclassify(A.rsow) == FP_NORMAL;
  }
  A.tout_f = sc->time_step_out;
  A.nas = -sc->alpha_s;
  A.al = sc->alpha_l;
  A.e1 = sc->eta_1;
  A.e2 = sc->eta_2;
  A.nw = -sc->w_ohc;
  A.ar = sc->alpha_r;
  A.dx2 = sc->delta_x * sc->delta_x;
  A.dxa0 = sc->delta_x * sc->a0;
  A.na1 = -sc->a1;
  A.na2 = -sc->a2;
  A.gme = sc->Gme;
  A.sow = sc->sigma_ow;
  A.dt0 = sc->time_step;
  A.dtmin = sc->dt_min;
  A.dtmax = sc->dt_max;
  A.jfast = sc->jacobi_fast;
  A.jslow = sc->jacobi_slow;
  A.max_outer = sc->max_outer;
  A.max_sub = sc->max_substeps_per_sample;
  A.jtol = sc->jacobi_tol;
  A.jcap = sc->jacobi_cap;
  A.guess = tol ? sc->guess_mode : 0;
  A.learn_every = sc->learned_every < 1 ? 1 : sc->learned_every;
  A.ws_blob = learned ? static_cast<const unsigned char*>(ex->d_ws_blob) : nullptr;
  A.log = ex && tol ? ex->d_log : nullptr;
  A.log_cap = ex ? ex->log_cap : 0;
  A.log_every = ex && ex->log_every > 0 ? ex->log_every : 1;
  A.log_count = ex ? ex->d_log_count : nullptr;

  int dev = 0, n_sm = 0, per_sm = 0;
  CGB_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  CGB_TRY_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev),
               "cudaDeviceGetAttribute");
  const LaunchShape& shape = learned               ? kLearnedShape
                             : tol                 ? kTolShape
                             : ref_arith           ? kRefArithShape
                             : sc->controller == 1 ? kCountShape
                                                   : kShapes[g_shape];
  if (shape.dyn_smem > 48 * 1024) {
    static int configured[64] = {};
    if (dev < 64 && !configured[dev]) {
      CGB_TRY_CUDA(cudaFuncSetAttribute(shape.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        shape.dyn_smem),
                   "cudaFuncSetAttribute(bm learned)");
      configured[dev] = 1;
    }
  }
  CGB_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, shape.fn,
                                                             shape.warps * 32, shape.dyn_smem),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  if (per_sm < 1) per_sm = 1;
  long long want = (n_units + shape.warps - 1) / shape.warps;
  long long grid = (long long)n_sm * per_sm;
  if (grid > want) grid = want;
  CGB_TRY_CUDA(cudaMemsetAsync(d_work, 0, sizeof(int32_t), st), "cudaMemsetAsync(work)");
  shape.launch((unsigned)grid, st, A);
  CGB_TRY_CUDA(cudaGetLastError(), "bm_warp_kernel launch");
  note_launch();
  (void)in_len;
  (void)out_rows;
  return CGB_OK;
}
