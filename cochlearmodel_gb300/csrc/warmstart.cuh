// Learned Jacobi warm start: the pieces shared by the BM kernel (inference,
// fused into the step) and the training kernels.
//
// Network: four 1-D convolutions over the 256 sections, kernel width 5,
// "same" zero padding, 8 -> 64 -> 64 -> 64 -> 1 channels, ReLU between
// layers.  Weights and activations are BF16, products accumulate in FP32 on
// the tensor cores (mma.sync m16n8k16, one warp per tile), biases are FP32.
//
// Input features at a step start (section s, all per-unit maxima taken over
// the 256 sections):
//   d    = p1 - p2                 (p1, p2: converged pressure of the last
//                                   two steps)
//   pe   = p1 + rho * d            (rho = dt / dt_prev; the extrapolated guess)
//   rt   = J(pe) - pe              (one Jacobi sweep's update from pe: the
//                                   residual scaled by 1/m_s)
//   f0 = rt / max|rt|, f1 = p1 / max|p1|, f2 = d / max|d|, f3 = Yrm / max|Yrm|,
//   f4 = (1/m_s) / max|1/m|, f5 = v / max|v|, f6 = x / max|x|, f7 = rho / 2.
// Output o_s; the guess is pe_s + max|rt| * s_out * o_s.
//
// Shared-memory layouts (bytes):
//   8-channel rows  : 16 B per row, row r at r * 16.
//   64-channel rows : 128 B per row; 16-byte chunk c of row r sits at chunk
//                     c ^ (r & 7), so eight consecutive rows read at the same
//                     chunk hit distinct banks (ldmatrix is conflict-free).
// Packed forward weights (one blob, copied to shared memory as is):
//   W1 [6 taps][64 out][8 in]   (tap 5 is zero: the tap pairs of the K loop)
//   W2 [5][64][64], W3 [5][64][64]  (64-channel rows, row = tap*64 + out)
//   W4 [5][8][64]                   (row = tap*8 + out; outputs 1..7 zero)
//   b1[64], b2[64], b3[64], b4[8] float; then s_out, rm_scale, 2 pad floats.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cgb_device.cuh"

namespace cgb {
namespace ws {

constexpr int kNS = 256;
constexpr int kC = 64;
constexpr int kTaps = 5;
constexpr int kW1Bytes = 6 * 64 * 8 * 2;      // 6144
constexpr int kW64Bytes = 5 * 64 * 64 * 2;    // 40960
constexpr int kW4Bytes = 5 * 8 * 64 * 2;      // 5120
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kW1Bytes;
constexpr int kOffW3 = kOffW2 + kW64Bytes;
constexpr int kOffW4 = kOffW3 + kW64Bytes;
constexpr int kOffBias = kOffW4 + kW4Bytes;   // 93184
constexpr int kBiasFloats = 64 + 64 + 64 + 8 + 4;
constexpr int kBlobBytes = kOffBias + kBiasFloats * 4;  // 94000
// Transposed weights for the backward pass (training only):
//   W4T [6][64][8] (layer-1 layout), W3T [5][64][64], W2T [5][64][64].
constexpr int kOffT4 = 0;
constexpr int kOffT3 = kOffT4 + kW1Bytes;
constexpr int kOffT2 = kOffT3 + kW64Bytes;
constexpr int kBlobTBytes = kOffT2 + kW64Bytes;  // 88064
constexpr int kParams = 5 * 64 * 8 + 64 + 5 * 64 * 64 + 64 + 5 * 64 * 64 + 64 + 5 * 64 + 1;

static_assert(kBlobBytes % 16 == 0, "blob must be a whole number of 16-byte chunks");

__host__ __device__ __forceinline__ int swz64(int row, int chunk) {
  return row * 128 + ((chunk ^ (row & 7)) << 4);
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(addr));
}
// D(16x8, f32) += A(16x16, bf16, row) * B(16x8, bf16, col)
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Round-to-nearest-even FP32 -> BF16 (bit pattern), and two packed.
__device__ __forceinline__ uint32_t bf16_bits(float f) {
  uint32_t u = __float_as_uint(f);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return u >> 16;
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  return bf16_bits(lo) | (bf16_bits(hi) << 16);
}
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// One 16-row output tile of a convolution whose input has 64 channels.
// in_base: shared address of the input buffer (64-channel rows); in_row0:
// input row of (output row 0, tap 0).  w_base: weights [tap][NT*8 out][64 in]
// as 64-channel rows.  acc[n][.] accumulates output channels n*8..n*8+7.
template <int NT>
__device__ __forceinline__ void conv64_tile(float (&acc)[NT][4], uint32_t in_base, int in_row0,
                                            uint32_t w_base, int lane) {
  const int q = lane >> 3, r = lane & 7;
#pragma unroll 1
  for (int tap = 0; tap < kTaps; ++tap) {
    const int arow = in_row0 + tap + r + 8 * (q & 1);
#pragma unroll
    for (int cb = 0; cb < 4; ++cb) {
      uint32_t a[4];
      ldsm_x4(a, in_base + swz64(arow, 2 * cb + (q >> 1)));
      if constexpr (NT == 1) {
        uint32_t b[2];
        ldsm_x2(b, w_base + swz64(tap * 8 + r, 2 * cb + (q & 1)));
        mma_bf16(acc[0], a, b[0], b[1]);
      } else {
#pragma unroll
        for (int np = 0; np < NT / 2; ++np) {
          uint32_t b[4];
          ldsm_x4(b, w_base + swz64(tap * NT * 8 + np * 16 + 8 * (q >> 1) + r, 2 * cb + (q & 1)));
          mma_bf16(acc[2 * np], a, b[0], b[1]);
          mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
        }
      }
    }
  }
}

// One 16-row output tile of a convolution whose input has 8 channels
// (16-byte rows).  The K loop runs over tap pairs (0,1), (2,3), (4,5); the
// weights of tap 5 are zero.  w_base: weights [6 taps][64 out][8 in].
__device__ __forceinline__ void conv8_tile(float (&acc)[8][4], uint32_t in_base, int in_row0,
                                           uint32_t w_base, int lane) {
  const int q = lane >> 3, r = lane & 7;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    uint32_t a[4];
    ldsm_x4(a, in_base + (in_row0 + 2 * j + (q >> 1) + r + 8 * (q & 1)) * 16);
#pragma unroll
    for (int np = 0; np < 4; ++np) {
      uint32_t b[4];
      ldsm_x4(b, w_base + ((2 * j + (q & 1)) * 64 + np * 16 + 8 * (q >> 1) + r) * 16);
      mma_bf16(acc[2 * np], a, b[0], b[1]);
      mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
    }
  }
}

template <int NT>
__device__ __forceinline__ void zero_acc(float (&acc)[NT][4]) {
#pragma unroll
  for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
}

// Epilogue of a hidden layer: bias, ReLU, BF16, stored to 64-channel rows
// out_row0.. of out (shared); rows whose position lies outside [0, 256) are
// stored as zero (the next layer's zero padding).  Fragment layout of
// mma m16n8k16: acc[n][0..1] = row g, columns n*8+2t..+1; acc[n][2..3] =
// row g+8.
__device__ __forceinline__ void store_hidden(const float (&acc)[8][4], unsigned char* out,
                                             int out_row0, int pos0, const float* bias, int lane) {
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int row = out_row0 + g + 8 * h, pos = pos0 + g + 8 * h;
    const bool in = pos >= 0 && pos < kNS;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int col = n * 8 + 2 * t;
      float lo = fmaxf(acc[n][2 * h] + bias[col], 0.0f);
      float hi = fmaxf(acc[n][2 * h + 1] + bias[col + 1], 0.0f);
      if (!in) lo = hi = 0.0f;
      *reinterpret_cast<uint32_t*>(out + swz64(row, col >> 3) + (col & 7) * 2) = pack_bf16(lo, hi);
    }
  }
}

// Features of one unit (lane l holds sections 8l..8l+7) into 8-channel rows
// feat_row0 + s of feat (shared).  pe receives the extrapolated guess; the
// return value is max|rt| (0: the guess needs no correction).  rmL/rmR and
// YrmL/YrmR are 1/m_s and Y_s/m_s of the halo sections 8l-1 and 8l+8.
__device__ __forceinline__ float make_features(const float (&Yrm)[8], const float (&p1)[8],
                                               const float (&p2)[8], const float (&v)[8],
                                               const float (&x)[8], const float (&rm)[8],
                                               float rho, float rm_scale, float (&pe)[8],
                                               unsigned char* feat, int feat_row0, int lane) {
  float d[8], rt[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    d[k] = __fsub_rn(p1[k], p2[k]);
    pe[k] = __fmaf_rn(rho, d[k], p1[k]);
  }
  const bool first = lane == 0, last = lane == 31;
  float left = __shfl_up_sync(kFull, pe[7], 1);
  float right = __shfl_down_sync(kFull, pe[0], 1);
  if (first) left = 0.0f;
  if (last) right = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float lo = k == 0 ? left : pe[k - 1];
    const float hi = k == 7 ? right : pe[k + 1];
    // sections 254 and 255 carry no lower coefficient
    const float t = (last && k >= 6) ? hi : __fadd_rn(lo, hi);
    rt[k] = __fsub_rn(__fmaf_rn(-t, rm[k], Yrm[k]), pe[k]);
  }
  float mr = 0.f, m1 = 0.f, md = 0.f, my = 0.f, mv = 0.f, mx = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    mr = fmaxf(mr, fabsf(rt[k]));
    m1 = fmaxf(m1, fabsf(p1[k]));
    md = fmaxf(md, fabsf(d[k]));
    my = fmaxf(my, fabsf(Yrm[k]));
    mv = fmaxf(mv, fabsf(v[k]));
    mx = fmaxf(mx, fabsf(x[k]));
  }
  mr = warp_max_xor(mr);
  m1 = warp_max_xor(m1);
  md = warp_max_xor(md);
  my = warp_max_xor(my);
  mv = warp_max_xor(mv);
  mx = warp_max_xor(mx);
  const float ir = mr > 0.f ? __fdiv_rn(1.0f, mr) : 0.f;
  const float i1 = m1 > 0.f ? __fdiv_rn(1.0f, m1) : 0.f;
  const float id = md > 0.f ? __fdiv_rn(1.0f, md) : 0.f;
  const float iy = my > 0.f ? __fdiv_rn(1.0f, my) : 0.f;
  const float iv = mv > 0.f ? __fdiv_rn(1.0f, mv) : 0.f;
  const float ix = mx > 0.f ? __fdiv_rn(1.0f, mx) : 0.f;
  const float f7 = __fmul_rn(rho, 0.5f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    uint4 w;
    w.x = pack_bf16(__fmul_rn(rt[k], ir), __fmul_rn(p1[k], i1));
    w.y = pack_bf16(__fmul_rn(d[k], id), __fmul_rn(Yrm[k], iy));
    w.z = pack_bf16(__fmul_rn(rm[k], rm_scale), __fmul_rn(v[k], iv));
    w.w = pack_bf16(__fmul_rn(x[k], ix), f7);
    *reinterpret_cast<uint4*>(feat + (feat_row0 + lane * 8 + k) * 16) = w;
  }
  return mr;
}

// Per-warp scratch of the fused inference, bytes: feature rows (position
// s at row s + 8; rows outside the unit stay zero), two hidden buffers of
// 88 64-channel rows (layer outputs for a 64-section chunk plus halo), and
// the output (256 floats).
constexpr int kFeatRows = 280;
constexpr int kHidRows = 88;
constexpr int kOffH1 = kFeatRows * 16;
constexpr int kOffH2 = kOffH1 + kHidRows * 128;
constexpr int kOffOut = kOffH2 + kHidRows * 128;
constexpr int kWarpScratch = kOffOut + kNS * 4;  // 28032

// Network output for the 256 sections of one unit, whose features sit in
// the warp's scratch (rows s + 8).  Sections are processed in chunks of 64
// with the halo each layer needs recomputed: layer 1 produces positions
// c0-6..c0+73, layer 2 c0-4..c0+75, layer 3 c0-2..c0+77, layer 4
// c0..c0+63 (the extra rows at the end of layers 1-3 are never consumed).
// wblob: the packed weights in shared memory.  The result is left in the
// scratch's output floats (index = section).
__device__ __forceinline__ void infer_unit(const unsigned char* wblob, unsigned char* scratch,
                                           int lane) {
  const uint32_t sW1 = smem_u32(wblob + kOffW1), sW2 = smem_u32(wblob + kOffW2),
                 sW3 = smem_u32(wblob + kOffW3), sW4 = smem_u32(wblob + kOffW4);
  const float* bias = reinterpret_cast<const float*>(wblob + kOffBias);
  unsigned char* h1 = scratch + kOffH1;
  unsigned char* h2 = scratch + kOffH2;
  float* outp = reinterpret_cast<float*>(scratch + kOffOut);
  const uint32_t sF = smem_u32(scratch), sH1 = smem_u32(h1), sH2 = smem_u32(h2);
  const int g = lane >> 2, t = lane & 3;
#pragma unroll 1
  for (int c0 = 0; c0 < kNS; c0 += 64) {
    float acc[8][4];
#pragma unroll 1
    for (int mt = 0; mt < 5; ++mt) {  // layer 1: feature row = pos + tap - 2 + 8
      zero_acc(acc);
      conv8_tile(acc, sF, c0 + 16 * mt, sW1, lane);
      store_hidden(acc, h1, 16 * mt, c0 - 6 + 16 * mt, bias, lane);
    }
    __syncwarp();
#pragma unroll 1
    for (int mt = 0; mt < 5; ++mt) {  // layer 2: h1 row = out row + tap
      zero_acc(acc);
      conv64_tile<8>(acc, sH1, 16 * mt, sW2, lane);
      store_hidden(acc, h2, 16 * mt, c0 - 4 + 16 * mt, bias + 64, lane);
    }
    __syncwarp();
#pragma unroll 1
    for (int mt = 0; mt < 5; ++mt) {  // layer 3: h2 row = out row + tap
      zero_acc(acc);
      conv64_tile<8>(acc, sH2, 16 * mt, sW3, lane);
      store_hidden(acc, h1, 16 * mt, c0 - 2 + 16 * mt, bias + 128, lane);
    }
    __syncwarp();
#pragma unroll 1
    for (int mt = 0; mt < 4; ++mt) {  // layer 4: one output channel
      float o[1][4];
      zero_acc(o);
      conv64_tile<1>(o, sH1, 16 * mt, sW4, lane);
      if (t == 0) {
        outp[c0 + 16 * mt + g] = o[0][0] + bias[192];
        outp[c0 + 16 * mt + g + 8] = o[0][2] + bias[192];
      }
    }
    __syncwarp();
  }
}
#endif

}  // namespace ws
}  // namespace cgb
