// Fused IHC + auditory-nerve rate (lambda) kernel: reference RunIHCKernel
// (src/cochlea.cu:3573-3644) = CudaUnifiedCalcIHC (:3431-3506) followed by
// CudaCalcLambda (:3365-3408), with the decoupled FIR look-back rule of
// DeviceCudaFIRFilter (:2712-2730).
//
// Per point (t, s) of a frame:
//   AC  = sum_{i<tu(t)} b_i v[t-i]          (AC low-pass, taps pre-scaled)
//   dS  = (scale v - AC)^2
//   DC  = sum_{i<tu(t)} d_i dS[t-i]         (DC moving average)
//         with uniform taps d (the reference's DC filter): d * S(t), S the
//         window sum, re-summed at every 32nd frame row (and where the
//         look-back rule restarts the window) and otherwise updated by
//         adding dS[t] and removing dS[t-tu]; all in compensated (TwoSum)
//         arithmetic
//   IHC = log10(max(10^ihc_s (eta_AC AC + eta_DC DC), 0) + 1e-20)
//   lambda_j = s ? min(SAT, max(A_js IHC, spont_j)) : spont_j,  j = 0..2
// in FP32, each FIR accumulated with a compensated dot product (Dot2).
//
// GB300 layout: one CTA = 32 sections x a run of consecutive TR-row tiles.
// Each tile's velocity window (TR rows plus the look-back) is staged into
// shared memory by TMA (cp.async.bulk.tensor.2d, 64-row boxes, completion on
// an mbarrier with a bounded wait), the next tile's while the current one
// finishes; AC and dS are computed from shared memory with 8-row register
// blocking, then DC, IHC and lambda, and the three lambda planes are written
// with coalesced 128-byte rows.

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "cgb_device.cuh"
#include "cgb_internal.h"

namespace cgb {
namespace {

constexpr int kSecTile = 32;   // sections per CTA (one per lane)
constexpr int kBoxRows = 64;   // rows per TMA box
constexpr int kIhcWarps = 16;
constexpr int kRB = 8;         // output rows per register block
// bound on one staging wait, in nanoseconds of the GPU's global timer
constexpr unsigned long long kWaitNs = 1000000000ull;
constexpr int kTilesPerRun = 8;  // consecutive tiles per CTA (short runs)

struct IHCArgs {
  const cgb_ihc_frame* frames;
  const int32_t* tile_prefix;  // [n_frames + 1] runs of tiles before each frame
  int n_frames;
  const float* taps;           // [n_ac] AC taps (x scale) then [n_dc] DC taps
  int n_ac, n_dc;
  float scale, eta_ac, eta_dc, sat;
  float spont0, spont1, spont2;
  const float* dmg;            // [P][256] 10^ihc
  const float* aihc;           // [3][256]
  float* lam;                  // [3][lam_plane_rows][256]
  float* lam_host;             // host mirror of lam (pinned, mapped), or null
  int64_t lam_plane_rows;
  float* ihc;                  // [lam rows][256] or null
  int TR, xrows;               // output rows per tile, staged rows (multiple of 64)
  int32_t* status;
  int dc_uniform;              // all DC taps equal: running window sum
  int ac_sym;                  // AC taps symmetric: FIR over tap pairs
  int run;                     // tiles per CTA (consecutive, one frame)
  const float* ac_ext;         // AC by velocity row (the IIR path), or null: the FIR
  int skip_first_copy;         // test-only: arm the first staging wait but issue no copy
  // RunIHCKernel's debug stage: 9 AC, 10 DC, 11 dS (0 none), stored by lambda
  // row into stage_out [lam rows][256]
  int stage;
  float* stage_out;
};

// Test-only fault injection (cgb_ihc_set_fault_injection): the next launches
// arm the first staging mbarrier without issuing its copies, so the bounded
// wait runs out with nothing in flight and the kernel reports status bit 1.
int g_fault_skip_copy = 0;

__device__ __forceinline__ int taps_used(int k, const cgb_ihc_frame& f, int taps) {
  const int sg = k < f.frdp - 1 ? f.seg : f.total;
  const int lim = (k + 1) % sg;
  return lim < taps ? lim : taps;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Compensated tap accumulation (Ogita-Rump-Oishi Dot2): the product error
// comes from one FMA, the sum error from TwoSum, and both are carried in c.
// The result equals the dot product evaluated in about twice the working
// precision and rounded once -- what the reference's double accumulators
// give after their float store -- at FP32 instruction rates.
struct Dot2 {
  float s, c;
  __device__ __forceinline__ void init() { s = c = 0.0f; }
  __device__ __forceinline__ void add(float b, float x) {
    const float p = __fmul_rn(b, x);
    const float q = __fmaf_rn(b, x, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, q));
  }
  // b (x1 + x2) for a symmetric tap pair: the pair sum by TwoSum, Dot2 on
  // its rounded value, b times its rounding error into c by one fma
  __device__ __forceinline__ void add_pair(float b, float x1, float x2) {
    const float sg = __fadd_rn(x1, x2);
    const float zz = __fsub_rn(sg, x1);
    const float ep = __fadd_rn(__fsub_rn(x1, __fsub_rn(sg, zz)), __fsub_rn(x2, zz));
    add(b, sg);
    c = __fmaf_rn(b, ep, c);
  }
  __device__ __forceinline__ float result() const { return __fadd_rn(s, c); }
};

// Dot2 on two independent sums at once (two-wide FP32); each element
// performs exactly the scalar Dot2 sequence.
struct Dot2x2 {
  float2 s, c;
  __device__ __forceinline__ void init() { s = c = f2b(0.0f); }
  __device__ __forceinline__ void add(float2 b, float2 x) {
    const float2 p = mul2(b, x);
    const float2 q = fma2(b, x, neg2(p));
    const float2 t = add2(s, p);
    const float2 z = sub2(t, s);
    const float2 e = add2(sub2(s, sub2(t, z)), sub2(p, z));
    s = t;
    c = add2(c, add2(e, q));
  }
  __device__ __forceinline__ void add_pair(float2 b, float2 x1, float2 x2) {
    const float2 sg = add2(x1, x2);
    const float2 zz = sub2(sg, x1);
    const float2 ep = add2(sub2(x1, sub2(sg, zz)), sub2(x2, zz));
    add(b, sg);
    c = fma2(b, ep, c);
  }
  __device__ __forceinline__ float2 result() const { return add2(s, c); }
};

// FIR of one 8-row block, rows kb..kb+7 all using `taps` taps.  src points at
// the staged row of output kb (lane's column); rows above it are older.  One
// shared-memory load feeds the eight rows' accumulators.  Rows r and r+4 form
// pair r, so the per-tap shift of the window moves whole pairs and only pair
// 0 is assembled from the newly loaded row.  The last step loads one row
// beyond the oldest tap (unused; the caller stages it).
__device__ __forceinline__ void fir_block8(const float* __restrict__ src,
                                           const float* __restrict__ b, int taps,
                                           float (&out)[kRB]) {
  float2 W[4];
  Dot2x2 acc[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    acc[j].init();
    W[j] = f2(src[j * kSecTile], src[(j + 4) * kSecTile]);
  }
#pragma unroll 4
  for (int i = 0; i < taps; ++i) {
    const float2 bi = f2b(b[i]);
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j].add(bi, W[j]);
    const float w3 = W[3].x;
    W[3] = W[2];
    W[2] = W[1];
    W[1] = W[0];
    W[0] = f2(src[-(i + 1) * kSecTile], w3);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float2 r = acc[j].result();
    out[j] = r.x;
    out[j + 4] = r.y;
  }
}

// fir_block8 for a symmetric (linear-phase) filter of n taps, b_k = b_{n-1-k}:
// for each tap pair k the rows t-k and t-(n-1)+k are added exactly first
// (Dot2::add_pair), then the centre tap of an odd filter.  Two windows move
// in opposite directions: W1 (rows t-k, as in fir_block8) and W2 (rows
// t-(n-1)+k), one shared-memory load each per tap pair.  The rows read lie
// in [kb - n + 1, kb + 7], inside the staged window.
__device__ __forceinline__ void fir_block8_sym(const float* __restrict__ src,
                                               const float* __restrict__ b, int n,
                                               float (&out)[kRB]) {
  float2 W1[4], W2[4];
  Dot2x2 acc[4];
  const int o2 = -(n - 1) * kSecTile;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    acc[j].init();
    W1[j] = f2(src[j * kSecTile], src[(j + 4) * kSecTile]);
    W2[j] = f2(src[o2 + j * kSecTile], src[o2 + (j + 4) * kSecTile]);
  }
  const int half = n / 2;
#pragma unroll 2
  for (int k = 0; k < half; ++k) {
    const float2 bk = f2b(b[k]);
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j].add_pair(bk, W1[j], W2[j]);
    const float w13 = W1[3].x;
    W1[3] = W1[2];
    W1[2] = W1[1];
    W1[1] = W1[0];
    W1[0] = f2(src[-(k + 1) * kSecTile], w13);
    const float w20 = W2[0].y;
    W2[0] = W2[1];
    W2[1] = W2[2];
    W2[2] = W2[3];
    W2[3] = f2(w20, src[o2 + (k + 8) * kSecTile]);
  }
  if (n & 1) {
    const float2 bc = f2b(b[half]);
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j].add(bc, W1[j]);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float2 r = acc[j].result();
    out[j] = r.x;
    out[j + 4] = r.y;
  }
}

// One row of a symmetric filter with all n taps (the order of fir_block8_sym).
__device__ __forceinline__ float fir_row_sym(const float* __restrict__ src,
                                             const float* __restrict__ b, int n) {
  Dot2 acc;
  acc.init();
  for (int k = 0; k < n / 2; ++k) acc.add_pair(b[k], src[-k * kSecTile], src[-(n - 1 - k) * kSecTile]);
  if (n & 1) acc.add(b[n / 2], src[-(n / 2) * kSecTile]);
  return acc.result();
}

// s + c += x exactly (Knuth's TwoSum; the rounding error goes to c).
__device__ __forceinline__ void two_sum_add(float& s, float& c, float x) {
  const float t = __fadd_rn(s, x);
  const float z = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z));
  s = t;
  c = __fadd_rn(c, e);
}

constexpr int kDcAnchor = 32;  // DC window re-summed at frame rows k % 32 == 0
constexpr int kEmitRows = 4;   // rows per warp in one IHC / lambda batch

__device__ __forceinline__ float fir_row(const float* __restrict__ src,
                                         const float* __restrict__ b, int tu) {
  Dot2 acc;
  acc.init();
  for (int i = 0; i < tu; ++i) acc.add(b[i], src[-i * kSecTile]);
  return acc.result();
}

// Stages velocity rows [y0, y0 + boxes * 64) of sections s0..s0+31 into X
// (TMA, completion on mbar).  Called by one thread after a block barrier that
// ends all reads of X; the proxy fence orders those generic-proxy reads
// before the asynchronous writes.
__device__ __forceinline__ void stage_rows(const CUtensorMap* vmap, float* X, uint64_t* mbar,
                                           int boxes, int y0, int s0, bool skip = false) {
  const uint32_t bytes = (uint32_t)boxes * kBoxRows * kSecTile * 4;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
  if (skip) return;  // test-only: the transaction count is never met
  for (int bxi = 0; bxi < boxes; ++bxi) {
    const int y = y0 + bxi * kBoxRows;  // may be negative or past the end: zero fill
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(X + (size_t)bxi * kBoxRows * kSecTile)),
        "l"(vmap), "r"(s0), "r"(y), "r"(smem_u32(mbar))
        : "memory");
  }
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait on phase `parity` of mbar by every thread, for at most kWaitNs of the
// global timer (each try_wait returns within a short system-defined time),
// then a block-wide vote so that all threads take the same branch.
__device__ __forceinline__ bool wait_stage(uint64_t* mbar, uint32_t parity) {
  uint32_t done = 0;
  const unsigned long long t_start = global_ns();
  while (!done) {
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    if (!done && global_ns() - t_start > kWaitNs) break;
  }
  return __syncthreads_and(done) != 0;
}

// One CTA = 32 sections x a run of up to A.run consecutive tiles of TR rows
// of one frame, processed in order.  The first tile of the run computes AC
// and dS on the DC filter's look-back rows as well; later tiles inherit those
// n_dc - 1 rows of dS from the previous tile (shifted down in shared memory)
// and stage only the AC filter's look-back (plus one row), the next tile's rows being copied
// by TMA while the current tile's DC/IHC/lambda phase runs.
__global__ void __launch_bounds__(kIhcWarps * 32)
    ihc_lambda_kernel(const __grid_constant__ CUtensorMap vmap, const IHCArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // layout: X [xrows][32] | dS [TR + n_dc][32] | AC [TR][32] | taps | mbarrier
  float* X = reinterpret_cast<float*>(smem_raw);
  float* DS = X + (size_t)A.xrows * kSecTile;
  float* ACb = DS + (size_t)(A.TR + A.n_dc) * kSecTile;
  float* TP = ACb + (size_t)A.TR * kSecTile;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(
      (reinterpret_cast<uintptr_t>(TP + A.n_ac + A.n_dc) + 15) & ~uintptr_t(15));

  // locate the frame and the run
  const int bx = blockIdx.x;
  int lo = 0, hi = A.n_frames;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (A.tile_prefix[mid] <= bx) lo = mid; else hi = mid;
  }
  const cgb_ihc_frame f = A.frames[lo];
  const int tiles = (f.lam_rows + A.TR - 1) / A.TR;
  const int t0 = (bx - A.tile_prefix[lo]) * A.run;
  const int t1 = min(t0 + A.run, tiles);
  const int s0 = blockIdx.y * kSecTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int boxes_first = A.xrows / kBoxRows;
  // later tiles stage rows from row0 - n_ac: the register-blocked FIR loads
  // one row beyond its oldest tap on its last step (a value it never uses),
  // and that row must lie inside the staged window
  const int boxes_next = (A.TR + A.n_ac + kBoxRows - 1) / kBoxRows;

  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  for (int i = threadIdx.x; i < A.n_ac + A.n_dc; i += blockDim.x) TP[i] = A.taps[i];
  __syncthreads();
  // staged rows of the first tile start one row below the oldest row either
  // filter reads; those of later tiles below the oldest row the AC filter reads
  if (threadIdx.x == 0)
    stage_rows(&vmap, X, mbar, boxes_first, (int)f.v_row0 + t0 * A.TR - A.n_ac - A.n_dc + 1, s0,
               A.skip_first_copy != 0);

  const float* bac = TP;
  const float* bdc = TP + A.n_ac;
  const float scale = A.scale;
  const int s = s0 + lane;
  const float dmg = A.dmg[(size_t)f.ihc_profile * 256 + s];
  const float a0 = A.aihc[0 * 256 + s], a1 = A.aihc[1 * 256 + s], a2 = A.aihc[2 * 256 + s];
  const bool sec0 = s == 0;

  for (int t = t0; t < t1; ++t) {
    const bool first = t == t0;
    const int row0 = t * A.TR;
    const int TRt = min(A.TR, f.lam_rows - row0);
    const int xbase = first ? row0 - A.n_ac - A.n_dc + 1 : row0 - A.n_ac;
    const int dsbase = row0 - A.n_dc;
    if (!wait_stage(mbar, (uint32_t)((t - t0) & 1))) {
      if (threadIdx.x == 0) atomicOr(A.status, 1);
      return;
    }
    if (!first) {
      // dS of rows row0 - n_dc + 1 .. row0 - 1 from the previous tile's buffer
      for (int i = 1 + warp; i < A.n_dc; i += kIhcWarps)
        DS[(size_t)i * kSecTile + lane] = DS[(size_t)(i + A.TR) * kSecTile + lane];
      __syncthreads();
    }

    // phase 1: AC and dS on rows [k_lo, row0 + TRt)
    const int k_lo = first ? max(0, row0 - A.n_dc + 1) : row0, k_hi = row0 + TRt;
    for (int kb = k_lo + warp * kRB; kb < k_hi; kb += kIhcWarps * kRB) {
      const int nr = min(kRB, k_hi - kb);
      bool fast = nr == kRB;
#pragma unroll
      for (int r = 0; r < kRB; ++r)
        fast = fast && taps_used(kb + r, f, A.n_ac) == A.n_ac;
      float acc[kRB];
      const float* src = X + (size_t)(kb - xbase) * kSecTile + lane;
      if (A.ac_ext) {
#pragma unroll
        for (int r = 0; r < kRB; ++r)
          acc[r] = r < nr ? A.ac_ext[((int64_t)f.v_row0 + kb + r) * 256 + s] : 0.0f;
      } else if (fast) {
        if (A.ac_sym)
          fir_block8_sym(src, bac, A.n_ac, acc);
        else
          fir_block8(src, bac, A.n_ac, acc);
      } else {
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
          const int tu = taps_used(kb + r, f, A.n_ac);
          acc[r] = r >= nr ? 0.0f
                   : (A.ac_sym && tu == A.n_ac ? fir_row_sym(src + r * kSecTile, bac, tu)
                                               : fir_row(src + r * kSecTile, bac, tu));
        }
      }
#pragma unroll
      for (int r = 0; r < kRB; ++r) {
        if (r < nr) {
          const int k = kb + r;
          const float ms = __fmaf_rn(src[r * kSecTile], scale, -acc[r]);
          const float ds = __fmul_rn(ms, ms);
          DS[(size_t)(k - dsbase) * kSecTile + lane] = ds;
          if (k >= row0) {
            ACb[(size_t)(k - row0) * kSecTile + lane] = acc[r];
            if (A.stage == 9 || A.stage == 11)
              A.stage_out[((int64_t)f.lam_row0 + k) * 256 + s] = A.stage == 9 ? acc[r] : ds;
          }
        }
      }
    }
    __syncthreads();
    // X is free: stage the next tile while this one finishes
    if (threadIdx.x == 0 && t + 1 < t1)
      stage_rows(&vmap, X, mbar, boxes_next, (int)f.v_row0 + (t + 1) * A.TR - A.n_ac, s0);

    // phase 2: DC, IHC and lambda on rows [row0, row0 + TRt).  Pass 1
    // computes each row's pre-synaptic value eta_AC * AC + eta_DC * DC and
    // leaves it in the row's ACb slot.  Pass 2 turns pre-synaptic values into
    // IHC and lambda, kEmitRows rows per warp at a time: their arithmetic is
    // branch-free and independent, so the rows' dependent chains (log10)
    // interleave; the stores follow, behind the uniform output branches.
    auto set_pre = [&](int k, float dc) {
      float& slot = ACb[(size_t)(k - row0) * kSecTile + lane];
      slot = __fmaf_rn(slot, A.eta_ac, __fmul_rn(dc, A.eta_dc));
      if (A.stage == 10) A.stage_out[((int64_t)f.lam_row0 + k) * 256 + s] = dc;
    };
    if (A.dc_uniform) {
      // tiles start on multiples of 32 rows, so every 32-row block opens on
      // an anchor row
      const float d = bdc[0];
      const float* col = DS + lane;
      for (int kb = row0 + warp * kDcAnchor; kb < k_hi; kb += kIhcWarps * kDcAnchor) {
        const int ke = min(kb + kDcAnchor, k_hi);
        float ws = 0.0f, wc = 0.0f;
        int tu_prev = -1;
        // taps_used(k) stepped from row to row: lim = (k + 1) mod sg(k)
        int sg = kb < f.frdp - 1 ? f.seg : f.total;
        int lim = (kb + 1) % sg;
#pragma unroll 4
        for (int k = kb; k < ke; ++k) {
          const int tu = lim < A.n_dc ? lim : A.n_dc;
          // both window ends lie inside DS for every tu <= n_dc, so they are
          // loaded ahead of the dependent sums
          const float x_new = col[(size_t)(k - dsbase) * kSecTile];
          const float x_old = col[(size_t)(k - tu - dsbase) * kSecTile];
          if (k == kb || (tu != tu_prev && tu != tu_prev + 1)) {
            ws = wc = 0.0f;
            for (int j = 0; j < tu; ++j)
              two_sum_add(ws, wc, col[(size_t)(k - j - dsbase) * kSecTile]);
          } else {
            two_sum_add(ws, wc, x_new);
            if (tu == tu_prev) two_sum_add(ws, wc, -x_old);
          }
          tu_prev = tu;
          if (k + 1 == f.frdp - 1) {
            sg = f.total;
            lim = (k + 2) % sg;
          } else if (++lim == sg) {
            lim = 0;
          }
          // d * (ws + wc), rounded once
          const float p = __fmul_rn(d, ws);
          const float q = __fmaf_rn(d, ws, -p);
          set_pre(k, __fadd_rn(p, __fmaf_rn(d, wc, q)));
        }
      }
    } else {
      for (int kb = row0 + warp * kRB; kb < k_hi; kb += kIhcWarps * kRB) {
        const int nr = min(kRB, k_hi - kb);
        bool fast = nr == kRB;
#pragma unroll
        for (int r = 0; r < kRB; ++r)
          fast = fast && taps_used(kb + r, f, A.n_dc) == A.n_dc;
        float acc[kRB];
        const float* src = DS + (size_t)(kb - dsbase) * kSecTile + lane;
        if (fast) {
          fir_block8(src, bdc, A.n_dc, acc);
        } else {
#pragma unroll
          for (int r = 0; r < kRB; ++r)
            acc[r] = r < nr ? fir_row(src + r * kSecTile, bdc, taps_used(kb + r, f, A.n_dc))
                            : 0.0f;
        }
#pragma unroll
        for (int r = 0; r < kRB; ++r)
          if (r < nr) set_pre(kb + r, acc[r]);
      }
    }
    __syncthreads();
    for (int kb = row0 + warp * kEmitRows; kb < k_hi; kb += kIhcWarps * kEmitRows) {
      float lg[kEmitRows], l0[kEmitRows], l1[kEmitRows], l2[kEmitRows];
#pragma unroll
      for (int r = 0; r < kEmitRows; ++r) {
        // rows past the tile repeat its last row; they are not stored
        const int k = min(kb + r, k_hi - 1);
        const float pre = ACb[(size_t)(k - row0) * kSecTile + lane];
        const float y = __fmul_rn(dmg, pre);
        lg[r] = own_log10f(__fadd_rn(fmaxf(y, 0.0f), 1e-20f));
        l0[r] = sec0 ? A.spont0 : fminf(A.sat, fmaxf(__fmul_rn(a0, lg[r]), A.spont0));
        l1[r] = sec0 ? A.spont1 : fminf(A.sat, fmaxf(__fmul_rn(a1, lg[r]), A.spont1));
        l2[r] = sec0 ? A.spont2 : fminf(A.sat, fmaxf(__fmul_rn(a2, lg[r]), A.spont2));
      }
#pragma unroll
      for (int r = 0; r < kEmitRows; ++r) {
        if (kb + r < k_hi) {
          const int64_t row = f.lam_row0 + kb + r;
          A.lam[(0 * A.lam_plane_rows + row) * 256 + s] = l0[r];
          A.lam[(1 * A.lam_plane_rows + row) * 256 + s] = l1[r];
          A.lam[(2 * A.lam_plane_rows + row) * 256 + s] = l2[r];
          if (A.ihc) A.ihc[row * 256 + s] = lg[r];
          if (A.lam_host) {
            A.lam_host[(0 * A.lam_plane_rows + row) * 256 + s] = l0[r];
            A.lam_host[(1 * A.lam_plane_rows + row) * 256 + s] = l1[r];
            A.lam_host[(2 * A.lam_plane_rows + row) * 256 + s] = l2[r];
          }
        }
      }
    }
    __syncthreads();
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

size_t smem_bytes(int TR, int xrows, int n_ac, int n_dc) {
  return ((size_t)xrows + TR + n_dc + TR) * kSecTile * 4 + (size_t)(n_ac + n_dc) * 4 + 32;
}

// Output rows per tile: a multiple of 32 (the DC anchor grid) whose staged
// window fits 227 KB of shared memory, at most 384.  Preferred: the largest
// such TR that is a multiple of kIhcWarps * kRB (every warp gets the same
// number of register blocks in phase 1) and >= n_dc (runs of tiles); else
// the largest that fits.  TR = 0: the filters are too long for one tile.
void pick_tile(int n_ac, int n_dc, int* TR, int* xrows) {
  *TR = *xrows = 0;
  int any = 0, ax = 0;
  for (int tr = 384; tr >= 32; tr -= 32) {
    const int xr = (tr + n_ac + n_dc - 1 + kBoxRows - 1) / kBoxRows * kBoxRows;
    if (smem_bytes(tr, xr, n_ac, n_dc) > 227 * 1024) continue;
    if (!any) {
      any = tr;
      ax = xr;
    }
    if (tr % (kIhcWarps * kRB) == 0 && tr >= n_dc) {
      *TR = tr;
      *xrows = xr;
      return;
    }
  }
  *TR = any;
  *xrows = ax;
}

// The AC taps as the kernel uses them (scaled in float) are symmetric,
// b_k == b_{n-1-k}: the FIR then runs over tap pairs (fir_block8_sym).
int ac_symmetric(const float* ac_taps, int n_ac, float scale) {
  if (n_ac < 2) return 0;
  for (int i = 0; i < n_ac / 2; ++i)
    if (ac_taps[i] * scale != ac_taps[n_ac - 1 - i] * scale) return 0;
  return 1;
}

// Tiles per CTA run.  A run's first tile recomputes the DC filter's n_dc - 1
// look-back rows, so longer runs cost less; the longest of 32 and 16 tiles
// that still leaves at least two CTAs per SM (eight section blocks per run),
// else 8.  Runs need TR >= n_dc (the look-back is inherited in place).  The
// choice depends only on the frame table and the device, so the upload and
// the launch of one table agree.
// Tiles per run forced by cgb_ihc_set_run_length (the autotuner), 0: the rule below.
int g_forced_run = 0;

// The run length each scratch buffer's tables were uploaded with: the tile
// prefix on the device depends on it, so a launch of uploaded tables must use
// the same run length whatever the setting is by then.
std::mutex g_upload_run_mu;
std::unordered_map<const void*, int> g_upload_run;

int pick_run(const cgb_ihc_frame* frames, int n_frames, int TR, int n_dc) {
  if (TR < n_dc) return 1;
  if (g_forced_run > 0) return g_forced_run;
  int dev = 0, n_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      n_sm < 1)
    n_sm = 1 << 20;  // unknown: keep the short runs
  for (int r : {32, 16}) {
    long long runs = 0;
    for (int i = 0; i < n_frames; ++i) {
      const long long tiles = ((long long)frames[i].lam_rows + TR - 1) / TR;
      runs += (tiles + r - 1) / r;
    }
    if (runs * (256 / kSecTile) >= 2LL * n_sm) return r;
  }
  return kTilesPerRun;
}

}  // namespace
}  // namespace cgb

namespace cgb {
// bytes of the per-call tables: frames, tile prefix, taps, each 256-aligned
constexpr int64_t ihc_table_bytes(int n_frames, int n_taps) {
  return ((int64_t)n_frames * (int64_t)sizeof(cgb_ihc_frame) + 255) / 256 * 256 +
         ((int64_t)(n_frames + 1) * 4 + 255) / 256 * 256 + ((int64_t)n_taps * 4 + 255) / 256 * 256;
}
}  // namespace cgb

extern "C" int64_t cgb_ihc_lambda_scratch_bytes(int n_frames, int n_ac, int n_dc) {
  return cgb::ihc_table_bytes(n_frames, n_ac + n_dc);
}

namespace cgb {
namespace {
constexpr int kUpload = 1, kLaunch = 2;

// Validates the frame table, then uploads the per-call tables (frames, tile
// prefix, taps) to the scratch buffer (kUpload) and/or launches the kernel
// on tables already there (kLaunch).  Upload and launch are separable so a
// CUDA graph can capture the launch alone.
int ihc_lambda_impl(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames, int n_frames,
                    const float* ac_taps, int n_ac, const float* dc_taps, int n_dc,
                    const cgb_ihc_params* prm, const float* d_dmg, int n_dmg_profiles,
                    const float* d_aihc, float* d_lam, int64_t lam_plane_rows, float* d_ihc,
                    void* d_scratch, int64_t scratch_bytes, int32_t* d_status, void* stream,
                    int mode,
                    const float* ac_ext = nullptr, float* lam_host = nullptr,
                    int32_t* stage_prefix = nullptr, float* stage_taps = nullptr,
                    int stage = 0, float* d_stage = nullptr) {
  if (n_frames == 0) return CGB_OK;
  if (!frames || n_frames < 0 || !ac_taps || !dc_taps || !prm || !d_scratch ||
      ((mode & kLaunch) && (!d_v || !d_dmg || !d_aihc || !d_lam || !d_status)))
    return fail(CGB_ERR_ARG, "cgb_ihc_lambda_dev: null pointer argument");
  if (n_ac < 1 || n_dc < 1 || n_ac > 1024 || n_dc > 1024)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_dev: filter lengths must be in [1, 1024]");
  if (scratch_bytes < cgb_ihc_lambda_scratch_bytes(n_frames, n_ac, n_dc))
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_dev: scratch buffer too small");
  if ((mode & kLaunch) && (reinterpret_cast<uintptr_t>(d_v) & 15))
    return fail(CGB_ERR_ARG, "cgb_ihc_lambda_dev: d_v must be 16-byte aligned");
  if (lam_host) {
    const int rc = check_host_mirror(lam_host, "cgb_ihc_lambda_dev: h_lam");
    if (rc) return rc;
  }
  if (stage != 0 && (stage < 9 || stage > 12 || ((mode & kLaunch) && !d_stage)))
    return fail(CGB_ERR_ARG, "cgb_ihc_lambda_stage_dev: stage must be 9-12 with an output buffer");
  if (v_rows > INT32_MAX)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_dev: more than 2^31-1 velocity rows");
  // host staging of the tile prefix and the taps: a vector, or the caller's
  // fixed arrays (stage_prefix: n_frames + 1 entries, stage_taps: n_ac + n_dc)
  std::vector<int32_t> prefix_v;
  int32_t* prefix = stage_prefix;
  if (!prefix) {
    prefix_v.assign(n_frames + 1, 0);
    prefix = prefix_v.data();
  }
  prefix[0] = 0;
  int TR = 0, xrows = 0;
  pick_tile(n_ac, n_dc, &TR, &xrows);
  if (TR < 32) return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_dev: filters too long for one tile");
  int run = pick_run(frames, n_frames, TR, n_dc);
  {
    std::lock_guard<std::mutex> lock(g_upload_run_mu);
    if (mode & kUpload) {
      g_upload_run[d_scratch] = run;
    } else {
      const auto it = g_upload_run.find(d_scratch);
      if (it != g_upload_run.end()) run = it->second;
    }
  }
  for (int i = 0; i < n_frames; ++i) {
    const cgb_ihc_frame& fr = frames[i];
    const bool ok = fr.v_row0 >= 0 && fr.lam_rows >= 0 && fr.lam_rows <= fr.rows &&
                    fr.v_row0 + fr.rows <= v_rows && fr.lam_row0 >= 0 &&
                    fr.lam_row0 + fr.lam_rows <= lam_plane_rows && fr.seg > 0 && fr.frdp > 0 &&
                    fr.total > 0 && fr.ihc_profile >= 0 && fr.ihc_profile < n_dmg_profiles;
    if (!ok)
      return fail(CGB_ERR_RANGE,
                  "cgb_ihc_lambda_dev: frame " + std::to_string(i) + " out of range");
    const int tiles = (fr.lam_rows + TR - 1) / TR;
    prefix[i + 1] = prefix[i] + (tiles + run - 1) / run;
  }
  const int n_tiles = prefix[n_frames];
  if (n_tiles == 0) return CGB_OK;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned char* sc = static_cast<unsigned char*>(d_scratch);
  const size_t fbytes = ((size_t)n_frames * sizeof(cgb_ihc_frame) + 255) / 256 * 256;
  const size_t pbytes = ((size_t)(n_frames + 1) * 4 + 255) / 256 * 256;
  if (mode & kUpload) {
    std::vector<float> taps_v;
    float* taps = stage_taps;
    if (!taps) {
      taps_v.resize(n_ac + n_dc);
      taps = taps_v.data();
    }
    for (int i = 0; i < n_ac; ++i) taps[i] = ac_taps[i] * prm->scale;
    for (int i = 0; i < n_dc; ++i) taps[n_ac + i] = dc_taps[i];
    CGB_TRY_CUDA(cudaMemcpyAsync(sc, frames, (size_t)n_frames * sizeof(cgb_ihc_frame),
                                 cudaMemcpyHostToDevice, st),
                 "upload frames");
    CGB_TRY_CUDA(cudaMemcpyAsync(sc + fbytes, prefix, (size_t)(n_frames + 1) * 4,
                                 cudaMemcpyHostToDevice, st),
                 "upload tile prefix");
    CGB_TRY_CUDA(cudaMemcpyAsync(sc + fbytes + pbytes, taps, (size_t)(n_ac + n_dc) * 4,
                                 cudaMemcpyHostToDevice, st),
                 "upload taps");
  }
  if (!(mode & kLaunch)) return CGB_OK;

  auto encode = get_encode();
  if (!encode) return fail(CGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap map;
  cuuint64_t dims[2] = {256, (cuuint64_t)v_rows};
  cuuint64_t strides[1] = {256 * 4};
  cuuint32_t box[2] = {(cuuint32_t)kSecTile, (cuuint32_t)kBoxRows};
  cuuint32_t estr[2] = {1, 1};
  CUresult cr = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(d_v), dims,
                       strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                       CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS)
    return fail(CGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)cr) + ")");

  IHCArgs A{};
  A.frames = reinterpret_cast<const cgb_ihc_frame*>(sc);
  A.tile_prefix = reinterpret_cast<const int32_t*>(sc + fbytes);
  A.n_frames = n_frames;
  A.taps = reinterpret_cast<const float*>(sc + fbytes + pbytes);
  A.n_ac = n_ac;
  A.n_dc = n_dc;
  A.scale = prm->scale;
  A.eta_ac = prm->eta_ac;
  A.eta_dc = prm->eta_dc;
  A.sat = prm->lambda_sat;
  A.spont0 = prm->spont[0];
  A.spont1 = prm->spont[1];
  A.spont2 = prm->spont[2];
  A.dmg = d_dmg;
  A.aihc = d_aihc;
  A.lam = d_lam;
  A.lam_host = lam_host;
  A.lam_plane_rows = lam_plane_rows;
  A.ihc = d_ihc;
  A.TR = TR;
  A.xrows = xrows;
  A.status = d_status;
  A.ac_ext = ac_ext;
  A.skip_first_copy = g_fault_skip_copy;
  A.stage = stage == 12 ? 11 : stage;  // the reference's 12 ("Shigh") is dS too
  A.stage_out = d_stage;
  A.run = run;
  A.dc_uniform = 1;
  for (int i = 1; i < n_dc; ++i) A.dc_uniform &= dc_taps[i] == dc_taps[0];
  A.ac_sym = ac_symmetric(ac_taps, n_ac, prm->scale);
  const size_t smem = smem_bytes(TR, xrows, n_ac, n_dc);
  CGB_TRY_CUDA(cudaFuncSetAttribute(ihc_lambda_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "cudaFuncSetAttribute(ihc smem)");
  dim3 grid((unsigned)n_tiles, 256 / kSecTile);
  ihc_lambda_kernel<<<grid, kIhcWarps * 32, smem, st>>>(map, A);
  CGB_TRY_CUDA(cudaGetLastError(), "ihc_lambda_kernel launch");
  note_launch();
  return CGB_OK;
}

}  // namespace
}  // namespace cgb

extern "C" int cgb_ihc_set_run_length(int tiles) {
  if (tiles < 0 || tiles > 64)
    return cgb::fail(CGB_ERR_ARG, "cgb_ihc_set_run_length: tiles must be 0 (automatic) or 1-64");
  cgb::g_forced_run = tiles;
  return CGB_OK;
}

extern "C" int cgb_ihc_set_fault_injection(int skip_first_copy) {
  cgb::g_fault_skip_copy = skip_first_copy ? 1 : 0;
  return CGB_OK;
}

extern "C" int cgb_ihc_lambda_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                                  int n_frames, const float* ac_taps, int n_ac,
                                  const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
                                  const float* d_dmg, int n_dmg_profiles, const float* d_aihc,
                                  float* d_lam, int64_t lam_plane_rows, float* d_ihc,
                                  void* d_scratch, int64_t scratch_bytes, int32_t* d_status,
                                  void* stream) {
  return cgb::ihc_lambda_impl(d_v, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc, prm,
                              d_dmg, n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc,
                              d_scratch, scratch_bytes, d_status, stream,
                              cgb::kUpload | cgb::kLaunch);
}

extern "C" int cgb_ihc_lambda_stage_dev(const float* d_v, int64_t v_rows,
                                        const cgb_ihc_frame* frames, int n_frames,
                                        const float* ac_taps, int n_ac, const float* dc_taps,
                                        int n_dc, const cgb_ihc_params* prm, const float* d_dmg,
                                        int n_dmg_profiles, const float* d_aihc, float* d_lam,
                                        int64_t lam_plane_rows, float* d_ihc, int stage,
                                        float* d_stage, void* d_scratch, int64_t scratch_bytes,
                                        int32_t* d_status, void* stream) {
  if (stage < 9 || stage > 12 || !d_stage)
    return cgb::fail(CGB_ERR_ARG,
                     "cgb_ihc_lambda_stage_dev: stage must be 9-12 with an output buffer");
  return cgb::ihc_lambda_impl(d_v, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc, prm,
                              d_dmg, n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc,
                              d_scratch, scratch_bytes, d_status, stream,
                              cgb::kUpload | cgb::kLaunch, nullptr, nullptr, nullptr, nullptr,
                              stage, d_stage);
}

extern "C" int cgb_ihc_lambda_upload_dev(const cgb_ihc_frame* frames, int n_frames,
                                         const float* ac_taps, int n_ac, const float* dc_taps,
                                         int n_dc, const cgb_ihc_params* prm, int64_t v_rows,
                                         int64_t lam_plane_rows, int n_dmg_profiles,
                                         void* d_scratch, int64_t scratch_bytes, void* stream) {
  return cgb::ihc_lambda_impl(nullptr, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc,
                              prm, nullptr, n_dmg_profiles, nullptr, nullptr, lam_plane_rows,
                              nullptr, d_scratch, scratch_bytes, nullptr, stream, cgb::kUpload);
}

extern "C" int cgb_ihc_lambda_launch_dev(const float* d_v, int64_t v_rows,
                                         const cgb_ihc_frame* frames, int n_frames,
                                         const float* ac_taps, int n_ac, const float* dc_taps,
                                         int n_dc, const cgb_ihc_params* prm,
                                         const float* d_dmg, int n_dmg_profiles,
                                         const float* d_aihc, float* d_lam,
                                         int64_t lam_plane_rows, float* d_ihc, void* d_scratch,
                                         int64_t scratch_bytes, int32_t* d_status, void* stream) {
  return cgb::ihc_lambda_impl(d_v, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc, prm,
                              d_dmg, n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc,
                              d_scratch, scratch_bytes, d_status, stream, cgb::kLaunch);
}

extern "C" int cgb_ihc_lambda_launch_mirror_dev(
    const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames, int n_frames,
    const float* ac_taps, int n_ac, const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
    const float* d_dmg, int n_dmg_profiles, const float* d_aihc, float* d_lam,
    int64_t lam_plane_rows, float* d_ihc, void* d_scratch, int64_t scratch_bytes,
    int32_t* d_status, float* h_lam, int64_t h_lam_bytes, void* stream) {
  if (!h_lam) return cgb::fail(CGB_ERR_ARG, "cgb_ihc_lambda_launch_mirror_dev: null h_lam");
  if (h_lam_bytes < 3 * lam_plane_rows * 256 * (int64_t)sizeof(float))
    return cgb::fail(CGB_ERR_RANGE, "cgb_ihc_lambda_launch_mirror_dev: h_lam is shorter than "
                                    "3 x lam_plane_rows x 256 floats");
  return cgb::ihc_lambda_impl(d_v, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc, prm,
                              d_dmg, n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc,
                              d_scratch, scratch_bytes, d_status, stream, cgb::kLaunch, nullptr,
                              h_lam);
}

// ---------------------------------------------------------------------------
// No-allocation variant of cgb_ihc_lambda_dev.
//
// The per-call tables (frames, tile prefix, filter taps) go to a file-scope
// __device__ array instead of caller scratch, for callers that cannot
// allocate device memory: a host that hands the library only the buffers it
// already owns, or a real-time audio thread that must not enter the device
// allocator (nor the host heap: the host-side staging of the prefix and taps
// is a pair of static arrays too).  The array is 192 KiB, holds at most
// kNoAllocMaxFrames frames and kNoAllocMaxTaps taps, and stays resident on
// every GPU that loads this library until the process exits.  All calls
// share it and the static staging, so calls must come from one host thread
// at a time and calls whose GPU work overlaps (different streams, or a
// second call enqueued before the first one ran) race on its contents;
// serialise them on one stream.  Each call rewrites every table byte it
// reads, so nothing needs clearing.  The tables are the same layout as the
// caller-scratch path's (frames, then the prefix, then the taps, each
// 256-byte aligned), sized for the maximum.
// ---------------------------------------------------------------------------
namespace cgb {
namespace {

constexpr int kNoAllocMaxFrames = 4096;
constexpr int kNoAllocMaxTaps = 2048;  // n_ac + n_dc
constexpr size_t kNoAllocBytes = 192 * 1024;
static_assert((size_t)ihc_table_bytes(kNoAllocMaxFrames, kNoAllocMaxTaps) <= kNoAllocBytes,
              "no-allocation scratch too small");

__device__ __align__(256) unsigned char g_ihc_noalloc_scratch[kNoAllocBytes];

// host staging of the tile prefix and the taps (no heap use per call)
int32_t g_noalloc_prefix[kNoAllocMaxFrames + 1];
float g_noalloc_taps[kNoAllocMaxTaps];

constexpr int kMaxDevices = 64;
std::atomic<void*> g_noalloc_ptr[kMaxDevices] = {};

// Device address of the array on the current device, looked up once per
// device (the host-side symbol is only a stand-in, not a device address).
// Concurrent first calls may both look it up; they store the same address.
// The cache is not cleared by cudaDeviceReset: after a reset, a process that
// calls this entry point again must be a new process.
int noalloc_scratch(void** out) {
  int dev = 0;
  CGB_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_noalloc_dev: device index beyond 63");
  void* p = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    CGB_TRY_CUDA(cudaGetSymbolAddress(&p, g_ihc_noalloc_scratch), "cudaGetSymbolAddress");
    g_noalloc_ptr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return CGB_OK;
}

}  // namespace
}  // namespace cgb

extern "C" int cgb_ihc_lambda_noalloc_dev(const float* d_v, int64_t v_rows,
                                          const cgb_ihc_frame* frames, int n_frames,
                                          const float* ac_taps, int n_ac, const float* dc_taps,
                                          int n_dc, const cgb_ihc_params* prm,
                                          const float* d_dmg, int n_dmg_profiles,
                                          const float* d_aihc, float* d_lam,
                                          int64_t lam_plane_rows, float* d_ihc,
                                          int32_t* d_status, void* stream) {
  using namespace cgb;
  if (n_frames == 0) return CGB_OK;
  if (n_frames > kNoAllocMaxFrames)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_noalloc_dev: more than 4096 frames (the fixed "
                               "scratch holds at most 4096)");
  if (n_ac < 1 || n_dc < 1 || n_ac > 1024 || n_dc > 1024 || n_ac + n_dc > kNoAllocMaxTaps)
    return fail(CGB_ERR_RANGE,
                "cgb_ihc_lambda_noalloc_dev: filter lengths must be in [1, 1024]");
  void* scratch = nullptr;
  if (int st = noalloc_scratch(&scratch)) return st;
  return ihc_lambda_impl(d_v, v_rows, frames, n_frames, ac_taps, n_ac, dc_taps, n_dc, prm,
                         d_dmg, n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc, scratch,
                         (int64_t)kNoAllocBytes, d_status, stream, kUpload | kLaunch, nullptr,
                         nullptr, g_noalloc_prefix, g_noalloc_taps);
}

// ---------------------------------------------------------------------------
// AC by IIR (the reference's is_ac_iir_filter path, DeviceCudaIIRFilter,
// src/cochlea.cu:2745-2775):
//   Y[k] = sum_{i<ob} b_i X[k-i] - sum_{1<=j<ob} a_j Y[k-j]
// with ob the FIR look-back bound.  The reference keeps Y in float (lambdaFloat)
// and adds each double-tap term in double before rounding back to float; the
// kernel performs those FP64 operations in the same order (products and sums
// rounded separately).  The recursion is sequential in time, so one CTA walks
// one segment of a frame -- rows between two points where the look-back rule
// gives zero taps, which start the recursion afresh -- with one thread per
// section.
// ---------------------------------------------------------------------------
namespace cgb {
namespace {

struct IIRSeg {
  int64_t v_row0;  // the frame's first velocity row
  int32_t k0, k1;  // frame rows [k0, k1)
  int32_t frame;
  int32_t pad;
};

__global__ void __launch_bounds__(256)
    iir_ac_kernel(const float* __restrict__ v, float* __restrict__ ac,
                  const IIRSeg* __restrict__ segs, const cgb_ihc_frame* __restrict__ frames,
                  const double* __restrict__ b, const double* __restrict__ a, int n) {
  const IIRSeg sg = segs[blockIdx.x];
  const cgb_ihc_frame f = frames[sg.frame];
  const int s = threadIdx.x;
  const float* x = v + sg.v_row0 * 256 + s;
  float* y = ac + sg.v_row0 * 256 + s;
  for (int k = sg.k0; k < sg.k1; ++k) {
    const int ob = taps_used(k, f, n);
    float yk = 0.0f;
    for (int i = 0; i < ob; ++i)
      yk = __double2float_rn(__dadd_rn((double)yk, __dmul_rn(b[i], (double)x[(int64_t)(k - i) * 256])));
    for (int j = 1; j < ob; ++j)
      yk = __double2float_rn(__dsub_rn((double)yk, __dmul_rn(a[j], (double)y[(int64_t)(k - j) * 256])));
    y[(int64_t)k * 256] = yk;
  }
}

constexpr int kMaxIIR = 64;

// Segments of every frame's lambda rows that the recursion can run
// independently: candidate starts are rows whose look-back bound is zero;
// a candidate is dropped when a later row's recursion reaches back across it
// (where the rule switches to the frame total, the bound can jump up).
std::vector<IIRSeg> iir_segments(const cgb_ihc_frame* frames, int n_frames, int n) {
  std::vector<IIRSeg> out;
  std::vector<int> starts;
  for (int fi = 0; fi < n_frames; ++fi) {
    const cgb_ihc_frame& f = frames[fi];
    starts.assign(1, 0);
    for (int k = 0; k < f.lam_rows; ++k) {
      const int sg = k < f.frdp - 1 ? f.seg : f.total;
      const int lim = (k + 1) % sg;
      const int ob = lim < n ? lim : n;
      if (ob == 0) {
        if (k > starts.back()) starts.push_back(k);
      } else if (ob >= 2) {
        const int lo = k - ob + 1;  // oldest output row this row reads
        while (starts.size() > 1 && starts.back() > lo) starts.pop_back();
      }
    }
    for (size_t i = 0; i < starts.size(); ++i) {
      const int k1 = i + 1 < starts.size() ? starts[i + 1] : f.lam_rows;
      if (k1 > starts[i]) out.push_back({f.v_row0, starts[i], k1, fi, 0});
    }
  }
  return out;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace cgb

extern "C" int64_t cgb_ihc_lambda_iir_scratch_bytes(const cgb_ihc_frame* frames, int n_frames,
                                                    int n_iir, int n_dc) {
  using namespace cgb;
  if (!frames || n_frames < 0 || n_iir < 1 || n_iir > kMaxIIR) return -1;
  const size_t segs = iir_segments(frames, n_frames, n_iir).size();
  return cgb_ihc_lambda_scratch_bytes(n_frames, 1, n_dc) +
         (int64_t)(align256(segs * sizeof(IIRSeg)) + align256((size_t)2 * n_iir * 8));
}

namespace cgb {
namespace {

int ihc_lambda_iir_impl(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                        int n_frames, const float* b_taps, const float* a_taps, int n_iir,
                        const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
                        const float* d_dmg, int n_dmg_profiles, const float* d_aihc,
                        float* d_lam, int64_t lam_plane_rows, float* d_ihc, float* d_ac,
                        void* d_scratch, int64_t scratch_bytes, int32_t* d_status, void* stream,
                        int stage, float* d_stage) {
  if (n_frames == 0) return CGB_OK;
  if (!frames || n_frames < 0 || !b_taps || !a_taps || !d_ac || !d_v || !prm || !d_scratch)
    return fail(CGB_ERR_ARG, "cgb_ihc_lambda_iir_dev: null pointer argument");
  if (n_iir < 1 || n_iir > kMaxIIR)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_iir_dev: IIR length must be in [1, 64]");
  const int64_t need = cgb_ihc_lambda_iir_scratch_bytes(frames, n_frames, n_iir, n_dc);
  if (scratch_bytes < need)
    return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_iir_dev: scratch buffer too small");
  for (int i = 0; i < n_frames; ++i) {
    const cgb_ihc_frame& fr = frames[i];
    if (fr.v_row0 < 0 || fr.lam_rows < 0 || fr.lam_rows > fr.rows || fr.v_row0 + fr.rows > v_rows ||
        fr.seg <= 0 || fr.frdp <= 0 || fr.total <= 0)
      return fail(CGB_ERR_RANGE, "cgb_ihc_lambda_iir_dev: frame outside the velocity rows");
  }
  const std::vector<IIRSeg> segs = iir_segments(frames, n_frames, n_iir);
  const int64_t base_bytes = cgb_ihc_lambda_scratch_bytes(n_frames, 1, n_dc);
  unsigned char* sc = static_cast<unsigned char*>(d_scratch) + base_bytes;
  const size_t seg_bytes = align256(segs.size() * sizeof(IIRSeg));
  std::vector<double> taps(2 * (size_t)n_iir);
  for (int i = 0; i < n_iir; ++i) {
    taps[i] = (double)b_taps[i] * (double)prm->scale;
    taps[n_iir + i] = (double)a_taps[i];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the fused kernel's tables first (its frame table is the IIR kernel's too)
  const float one = 1.0f;
  int rc = ihc_lambda_impl(d_v, v_rows, frames, n_frames, &one, 1, dc_taps, n_dc, prm, d_dmg,
                           n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc, d_scratch,
                           base_bytes, d_status, stream, kUpload);
  if (rc) return rc;
  if (!segs.empty()) {
    CGB_TRY_CUDA(cudaMemcpyAsync(sc, segs.data(), segs.size() * sizeof(IIRSeg),
                                 cudaMemcpyHostToDevice, st),
                 "upload IIR segments");
    CGB_TRY_CUDA(cudaMemcpyAsync(sc + seg_bytes, taps.data(), taps.size() * 8,
                                 cudaMemcpyHostToDevice, st),
                 "upload IIR taps");
    iir_ac_kernel<<<(unsigned)segs.size(), 256, 0, st>>>(
        d_v, d_ac, reinterpret_cast<const IIRSeg*>(sc),
        reinterpret_cast<const cgb_ihc_frame*>(d_scratch),
        reinterpret_cast<const double*>(sc + seg_bytes),
        reinterpret_cast<const double*>(sc + seg_bytes) + n_iir, n_iir);
    CGB_TRY_CUDA(cudaGetLastError(), "iir_ac_kernel launch");
    note_launch();
  }
  return ihc_lambda_impl(d_v, v_rows, frames, n_frames, &one, 1, dc_taps, n_dc, prm, d_dmg,
                         n_dmg_profiles, d_aihc, d_lam, lam_plane_rows, d_ihc, d_scratch,
                         base_bytes, d_status, stream, kLaunch, d_ac, nullptr, nullptr, nullptr,
                         stage, d_stage);
}

}  // namespace
}  // namespace cgb

extern "C" int cgb_ihc_lambda_iir_dev(const float* d_v, int64_t v_rows,
                                      const cgb_ihc_frame* frames, int n_frames,
                                      const float* b_taps, const float* a_taps, int n_iir,
                                      const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
                                      const float* d_dmg, int n_dmg_profiles, const float* d_aihc,
                                      float* d_lam, int64_t lam_plane_rows, float* d_ihc,
                                      float* d_ac, void* d_scratch, int64_t scratch_bytes,
                                      int32_t* d_status, void* stream) {
  return cgb::ihc_lambda_iir_impl(d_v, v_rows, frames, n_frames, b_taps, a_taps, n_iir, dc_taps,
                                  n_dc, prm, d_dmg, n_dmg_profiles, d_aihc, d_lam,
                                  lam_plane_rows, d_ihc, d_ac, d_scratch, scratch_bytes,
                                  d_status, stream, 0, nullptr);
}

extern "C" int cgb_ihc_lambda_iir_stage_dev(const float* d_v, int64_t v_rows,
                                            const cgb_ihc_frame* frames, int n_frames,
                                            const float* b_taps, const float* a_taps, int n_iir,
                                            const float* dc_taps, int n_dc,
                                            const cgb_ihc_params* prm, const float* d_dmg,
                                            int n_dmg_profiles, const float* d_aihc,
                                            float* d_lam, int64_t lam_plane_rows, float* d_ihc,
                                            float* d_ac, int stage, float* d_stage,
                                            void* d_scratch, int64_t scratch_bytes,
                                            int32_t* d_status, void* stream) {
  if (stage < 9 || stage > 12 || !d_stage)
    return cgb::fail(CGB_ERR_ARG,
                     "cgb_ihc_lambda_iir_stage_dev: stage must be 9-12 with an output buffer");
  return cgb::ihc_lambda_iir_impl(d_v, v_rows, frames, n_frames, b_taps, a_taps, n_iir, dc_taps,
                                  n_dc, prm, d_dmg, n_dmg_profiles, d_aihc, d_lam,
                                  lam_plane_rows, d_ihc, d_ac, d_scratch, scratch_bytes,
                                  d_status, stream, stage, d_stage);
}
