// Learned Jacobi warm start: training kernels and the standalone inference.
//
// The network and its feature vector are described in warmstart.cuh.  The
// training step is
//   prepare (once): features + exact pressure (FP64 tridiagonal solve) of
//                   logged step starts -> raw targets (p* - pe) / max|rt|
//   forward       : one CTA per record, the four layers in shared memory,
//                   hidden activations (BF16) kept for the backward pass
//   loss          : pred = s_out * o, MSE against the raw target; dL/do (BF16)
//   backward      : one CTA per record, the transposed convolutions with the
//                   ReLU masks -> pre-activation gradients (BF16)
//   weight grad   : per CTA, its records' dW = sum_pos dPre (x) input,
//                   accumulated in FP32 into the CTA's partial slot, then a
//                   fixed-order FP64 sum over the slots (deterministic)
//   adam          : FP32 master parameters, then re-packed to BF16.
// All products run on the tensor cores (mma.sync m16n8k16 BF16, FP32
// accumulate); ldmatrix (.trans for the weight gradients) feeds them.
#include <cuda_runtime.h>

#include <cstdint>

#include "cgb_device.cuh"
#include "cgb_internal.h"
#include "warmstart.cuh"

namespace cgb {
namespace ws {

// Canonical FP32 parameter offsets: W1[5][64][8], b1, W2[5][64][64], b2,
// W3[5][64][64], b3, W4[5][64], b4[1].
constexpr int oW1 = 0, ob1 = oW1 + 5 * 64 * 8, oW2 = ob1 + 64, ob2 = oW2 + 5 * 64 * 64,
              oW3 = ob2 + 64, ob3 = oW3 + 5 * 64 * 64, oW4 = ob3 + 64, ob4 = oW4 + 5 * 64;
static_assert(ob4 + 1 == kParams, "parameter layout");

constexpr int kRows = 272;            // 64-channel rows per record: position + 8
constexpr int kHBytes = kNS * 128;    // one stored hidden layer of one record
constexpr int kFeatBytes = kFeatRows * 16;

__device__ __forceinline__ uint16_t bf16_half(float f) { return (uint16_t)bf16_bits(f); }

// ---------------------------------------------------------------------------
// Packing: canonical FP32 -> BF16 blobs.
// ---------------------------------------------------------------------------
__global__ void pack_kernel(const float* __restrict__ prm, float s_out, float rm_scale,
                            unsigned char* __restrict__ blob, unsigned char* __restrict__ blobT) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  // W1 [6][64][8], tap 5 zero
  for (int i = tid; i < 6 * 64 * 8; i += nth) {
    const int tap = i / 512, co = (i / 8) % 64, ci = i % 8;
    const float w = tap < 5 ? prm[oW1 + (tap * 64 + co) * 8 + ci] : 0.0f;
    reinterpret_cast<uint16_t*>(blob + kOffW1)[i] = bf16_half(w);
  }
  // W2, W3 [5][64 out][64 in] as 64-channel rows (row = tap*64 + out)
  for (int i = tid; i < 2 * 5 * 64 * 64; i += nth) {
    const int l = i / (5 * 64 * 64), j = i % (5 * 64 * 64);
    const int row = j / 64, ci = j % 64;
    const float w = prm[(l ? oW3 : oW2) + j];
    *reinterpret_cast<uint16_t*>(blob + (l ? kOffW3 : kOffW2) + swz64(row, ci >> 3) +
                                 (ci & 7) * 2) = bf16_half(w);
  }
  // W4 [5][8 out][64 in]; outputs 1..7 zero
  for (int i = tid; i < 5 * 8 * 64; i += nth) {
    const int row = i / 64, ci = i % 64, tap = row / 8, co = row % 8;
    const float w = co == 0 ? prm[oW4 + tap * 64 + ci] : 0.0f;
    *reinterpret_cast<uint16_t*>(blob + kOffW4 + swz64(row, ci >> 3) + (ci & 7) * 2) =
        bf16_half(w);
  }
  float* bias = reinterpret_cast<float*>(blob + kOffBias);
  for (int i = tid; i < kBiasFloats; i += nth) {
    float b = 0.0f;
    if (i < 64) b = prm[ob1 + i];
    else if (i < 128) b = prm[ob2 + i - 64];
    else if (i < 192) b = prm[ob3 + i - 128];
    else if (i == 192) b = prm[ob4];
    else if (i == 200) b = s_out;
    else if (i == 201) b = rm_scale;
    bias[i] = b;
  }
  if (!blobT) return;
  // W4T [6 taps][64 out(=in of W4)][8 in(=out of W4)]: W4T[t][ci][co] = W4[4-t][co][ci]
  for (int i = tid; i < 6 * 64 * 8; i += nth) {
    const int tap = i / 512, ci = (i / 8) % 64, co = i % 8;
    const float w = (tap < 5 && co == 0) ? prm[oW4 + (4 - tap) * 64 + ci] : 0.0f;
    reinterpret_cast<uint16_t*>(blobT + kOffT4)[i] = bf16_half(w);
  }
  // W3T, W2T [5][64][64]: WT[t][ci][co] = W[4-t][co][ci]
  for (int i = tid; i < 2 * 5 * 64 * 64; i += nth) {
    const int l = i / (5 * 64 * 64), j = i % (5 * 64 * 64);
    const int tap = j / 4096, ci = (j / 64) % 64, co = j % 64;
    const float w = prm[(l ? oW2 : oW3) + ((4 - tap) * 64 + co) * 64 + ci];
    const int row = tap * 64 + ci;
    *reinterpret_cast<uint16_t*>(blobT + (l ? kOffT2 : kOffT3) + swz64(row, co >> 3) +
                                 (co & 7) * 2) = bf16_half(w);
  }
}

// ---------------------------------------------------------------------------
// Prepare: features, extrapolated guess, max|rt| and the raw target of each
// logged record (one warp per record).  Record: [6][256] = Y/m, p1, p2, v,
// x, {rho, ...}.  The exact pressure solves p_s + (1/m_s)(l_s p_{s-1} +
// p_{s+1}) = Y_s/m_s (the system the Jacobi sweep iterates) in FP64.
// ---------------------------------------------------------------------------
__global__ void prepare_kernel(const float* __restrict__ rec, int n, const float* __restrict__ rm_g,
                               float rm_scale, unsigned char* __restrict__ feat,
                               float* __restrict__ target, float* __restrict__ nr_out,
                               double* __restrict__ work) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= n) return;
  const float* r = rec + (int64_t)wid * 6 * 256;
  const int base = lane * 8;
  float Yrm[8], p1[8], p2[8], v[8], x[8], rm[8], pe[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    Yrm[k] = r[0 * 256 + base + k];
    p1[k] = r[1 * 256 + base + k];
    p2[k] = r[2 * 256 + base + k];
    v[k] = r[3 * 256 + base + k];
    x[k] = r[4 * 256 + base + k];
    rm[k] = rm_g[base + k];
  }
  const float rho = r[5 * 256];
  unsigned char* f = feat + (int64_t)wid * kFeatBytes;
  // rows outside the unit are zero
  for (int i = lane; i < 8; i += 32) {
    reinterpret_cast<uint4*>(f)[i] = make_uint4(0, 0, 0, 0);
  }
  for (int i = lane; i < kFeatRows - 264; i += 32)
    reinterpret_cast<uint4*>(f)[264 + i] = make_uint4(0, 0, 0, 0);
  const float nr = make_features(Yrm, p1, p2, v, x, rm, rho, rm_scale, pe, f, 8, lane);
  // exact solve (lane 0, FP64 Thomas); work: [n][2][256]
  double* c = work + (int64_t)wid * 512;
  double* y = c + 256;
  if (lane == 0) {
    // row s: lower a_s = rm_s * l_s (s >= 1), diag 1, upper b_s = rm_s
    double cp = 0.0, yp = 0.0;
    for (int s = 0; s < 256; ++s) {
      const double rs = (double)rm_g[s];
      const double a = (s >= 1 && s < 254) ? rs : 0.0;
      const double b = s < 255 ? rs : 0.0;
      const double den = 1.0 - a * cp;
      cp = b / den;
      yp = ((double)r[s] - a * yp) / den;
      c[s] = cp;
      y[s] = yp;
    }
    for (int s = 254; s >= 0; --s) y[s] -= c[s] * y[s + 1];
  }
  __syncwarp();
  const float inr = nr > 0.0f ? 1.0f / nr : 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    target[(int64_t)wid * 256 + base + k] = (float)((y[base + k] - (double)pe[k]) * (double)inr);
  if (lane == 0) nr_out[wid] = nr;
}

// ---------------------------------------------------------------------------
// Forward: one CTA (8 warps) per record.
// ---------------------------------------------------------------------------
constexpr int kFwdSmem = kBlobBytes + kFeatBytes + 2 * kRows * 128;

__device__ __forceinline__ void copy16(void* dst, const void* src, int bytes, int tid, int nth) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = tid; i < bytes / 16; i += nth) d[i] = s[i];
}
__device__ __forceinline__ void zero16(void* dst, int bytes, int tid, int nth) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = tid; i < bytes / 16; i += nth) d[i] = make_uint4(0, 0, 0, 0);
}

__global__ void __launch_bounds__(256) forward_kernel(const unsigned char* __restrict__ blob,
                                                      const unsigned char* __restrict__ feat,
                                                      int n, unsigned char* __restrict__ hid,
                                                      float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned char* sw = sm;
  unsigned char* sF = sw + kBlobBytes;
  unsigned char* sA = sF + kFeatBytes;
  unsigned char* sB = sA + kRows * 128;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  copy16(sw, blob, kBlobBytes, tid, 256);
  zero16(sA, 2 * kRows * 128, tid, 256);
  const float* bias = reinterpret_cast<const float*>(sw + kOffBias);
  const uint32_t uW1 = smem_u32(sw + kOffW1), uW2 = smem_u32(sw + kOffW2),
                 uW3 = smem_u32(sw + kOffW3), uW4 = smem_u32(sw + kOffW4);
  const uint32_t uF = smem_u32(sF), uA = smem_u32(sA), uB = smem_u32(sB);
  const int g = lane >> 2, t = lane & 3;
  for (int rec = blockIdx.x; rec < n; rec += gridDim.x) {
    __syncthreads();
    copy16(sF, feat + (int64_t)rec * kFeatBytes, kFeatBytes, tid, 256);
    __syncthreads();
    unsigned char* h = hid + (int64_t)rec * kHBytes;  // layer l at h + l * n * kHBytes
    float acc[8][4];
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv8_tile(acc, uF, 16 * mt + 6, uW1, lane);
      store_hidden(acc, sA, 8 + 16 * mt, 16 * mt, bias, lane);
    }
    __syncthreads();
    copy16(h, sA + 8 * 128, kHBytes, tid, 256);
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv64_tile<8>(acc, uA, 16 * mt + 6, uW2, lane);
      store_hidden(acc, sB, 8 + 16 * mt, 16 * mt, bias + 64, lane);
    }
    __syncthreads();
    copy16(h + (int64_t)n * kHBytes, sB + 8 * 128, kHBytes, tid, 256);
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv64_tile<8>(acc, uB, 16 * mt + 6, uW3, lane);
      store_hidden(acc, sA, 8 + 16 * mt, 16 * mt, bias + 128, lane);
    }
    __syncthreads();
    copy16(h + 2 * (int64_t)n * kHBytes, sA + 8 * 128, kHBytes, tid, 256);
    for (int mt = warp; mt < 16; mt += 8) {
      float o[1][4];
      zero_acc(o);
      conv64_tile<1>(o, uA, 16 * mt + 6, uW4, lane);
      if (t == 0) {
        out[(int64_t)rec * 256 + 16 * mt + g] = o[0][0] + bias[192];
        out[(int64_t)rec * 256 + 16 * mt + g + 8] = o[0][2] + bias[192];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Loss: pred = s_out * o; L = sum (pred - target)^2 / (n * 256);
// dL/do -> channel 0 of 8-channel rows (BF16), channels 1..7 zero.
// ---------------------------------------------------------------------------
__global__ void loss_kernel(const float* __restrict__ out, const float* __restrict__ target, int n,
                            float s_out, unsigned char* __restrict__ dout,
                            double* __restrict__ loss_part) {
  __shared__ double red[256];
  const int rec = blockIdx.x, s = threadIdx.x;
  const float e = s_out * out[(int64_t)rec * 256 + s] - target[(int64_t)rec * 256 + s];
  const float gsc = 2.0f * s_out / ((float)n * 256.0f);
  uint4 w = make_uint4(bf16_bits(gsc * e), 0, 0, 0);
  reinterpret_cast<uint4*>(dout + (int64_t)rec * 256 * 16)[s] = w;
  red[s] = (double)e * (double)e;
  __syncthreads();
  for (int o = 128; o >= 1; o >>= 1) {
    if (s < o) red[s] += red[s + o];
    __syncthreads();
  }
  if (s == 0) loss_part[rec] = red[0];
}

// ---------------------------------------------------------------------------
// Backward (data): one CTA per record.
//   dH3 = (W4^T * dO) . [H3 > 0], dH2 = (W3^T * dH3) . [H2 > 0],
//   dH1 = (W2^T * dH2) . [H1 > 0], each a convolution with the transposed,
//   tap-reversed weights.  Stored as BF16 64-channel rows (row = position).
// ---------------------------------------------------------------------------
constexpr int kBwdSmem = kBlobTBytes + kFeatBytes + 2 * kRows * 128;

__device__ __forceinline__ void store_masked(const float (&acc)[8][4], unsigned char* sout,
                                             int out_row0, int pos0,
                                             const unsigned char* __restrict__ mask,
                                             unsigned char* __restrict__ gout, int lane) {
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int pos = pos0 + g + 8 * h;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + 2 * t;
      const int off = swz64(pos, col >> 3) + (col & 7) * 2;
      const uint32_t m = *reinterpret_cast<const uint32_t*>(mask + off);
      const float lo = bf16_lo(m) > 0.0f ? acc[nt][2 * h] : 0.0f;
      const float hi = bf16_hi(m) > 0.0f ? acc[nt][2 * h + 1] : 0.0f;
      const uint32_t w = pack_bf16(lo, hi);
      if (sout) *reinterpret_cast<uint32_t*>(sout + swz64(out_row0 + g + 8 * h, col >> 3) +
                                             (col & 7) * 2) = w;
      *reinterpret_cast<uint32_t*>(gout + off) = w;
    }
  }
}

__global__ void __launch_bounds__(256) backward_kernel(const unsigned char* __restrict__ blobT,
                                                       const unsigned char* __restrict__ dout,
                                                       const unsigned char* __restrict__ hid,
                                                       int n, unsigned char* __restrict__ dpre) {
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned char* sw = sm;
  unsigned char* sO = sw + kBlobTBytes;
  unsigned char* sA = sO + kFeatBytes;
  unsigned char* sB = sA + kRows * 128;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  copy16(sw, blobT, kBlobTBytes, tid, 256);
  zero16(sO, kFeatBytes + 2 * kRows * 128, tid, 256);
  const uint32_t uT4 = smem_u32(sw + kOffT4), uT3 = smem_u32(sw + kOffT3),
                 uT2 = smem_u32(sw + kOffT2);
  const uint32_t uO = smem_u32(sO), uA = smem_u32(sA), uB = smem_u32(sB);
  for (int rec = blockIdx.x; rec < n; rec += gridDim.x) {
    __syncthreads();
    copy16(sO + 8 * 16, dout + (int64_t)rec * 256 * 16, 256 * 16, tid, 256);
    __syncthreads();
    const int64_t ro = (int64_t)rec * kHBytes, lo = (int64_t)n * kHBytes;
    float acc[8][4];
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv8_tile(acc, uO, 16 * mt + 6, uT4, lane);
      store_masked(acc, sA, 8 + 16 * mt, 16 * mt, hid + 2 * lo + ro, dpre + 2 * lo + ro, lane);
    }
    __syncthreads();
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv64_tile<8>(acc, uA, 16 * mt + 6, uT3, lane);
      store_masked(acc, sB, 8 + 16 * mt, 16 * mt, hid + lo + ro, dpre + lo + ro, lane);
    }
    __syncthreads();
    for (int mt = warp; mt < 16; mt += 8) {
      zero_acc(acc);
      conv64_tile<8>(acc, uB, 16 * mt + 6, uT2, lane);
      store_masked(acc, nullptr, 0, 16 * mt, hid + ro, dpre + ro, lane);
    }
  }
}

// ---------------------------------------------------------------------------
// Weight gradients.  CTA c handles records c, c + grid, ...; per record the
// inputs (features, H1..H3 at row position + 8) and the pre-activation
// gradients (dH1..dH3, dO at row position) are staged in shared memory and
// every (layer, tap, 16-output tile) task is one warp's 16 x Cin product over
// the 256 positions, added into the CTA's FP32 partial slot.
// ---------------------------------------------------------------------------
constexpr int kWgSmem = kFeatBytes + 3 * kRows * 128 + 3 * kNS * 128 + kNS * 16 + 128;

__device__ __forceinline__ void add_tile(float* __restrict__ part, int row_stride, int co0,
                                         int n_co, const float (&acc)[8][4], int nt_count,
                                         int lane) {
  const int g = lane >> 2, t = lane & 3;
  for (int nt = 0; nt < nt_count; ++nt) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = co0 + g + 8 * h;
      if (co >= n_co) continue;
      float* pr = part + co * row_stride + nt * 8 + 2 * t;
      pr[0] += acc[nt][2 * h];
      pr[1] += acc[nt][2 * h + 1];
    }
  }
}

__global__ void __launch_bounds__(256) wgrad_kernel(const unsigned char* __restrict__ feat,
                                                    const unsigned char* __restrict__ hid,
                                                    const unsigned char* __restrict__ dpre,
                                                    const unsigned char* __restrict__ dout, int n,
                                                    float* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned char* sF = sm;
  unsigned char* sH = sF + kFeatBytes;              // 3 x kRows rows (position + 8)
  unsigned char* sD = sH + 3 * kRows * 128;         // 3 x 256 rows (position)
  unsigned char* sO = sD + 3 * kNS * 128;           // 256 rows of 16 bytes
  unsigned char* sZ = sO + kNS * 16;                // 128 zero bytes
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int q = lane >> 3, r = lane & 7;
  zero16(sH, 3 * kRows * 128, tid, 256);
  zero16(sZ, 128, tid, 256);
  float* part = partial + (int64_t)blockIdx.x * kParams;
  for (int i = tid; i < kParams; i += 256) part[i] = 0.0f;
  const int64_t lo = (int64_t)n * kHBytes;
  for (int rec = blockIdx.x; rec < n; rec += gridDim.x) {
    __syncthreads();
    copy16(sF, feat + (int64_t)rec * kFeatBytes, kFeatBytes, tid, 256);
    for (int l = 0; l < 3; ++l) {
      copy16(sH + l * kRows * 128 + 8 * 128, hid + l * lo + (int64_t)rec * kHBytes, kHBytes, tid,
             256);
      copy16(sD + l * kNS * 128, dpre + l * lo + (int64_t)rec * kHBytes, kHBytes, tid, 256);
    }
    copy16(sO, dout + (int64_t)rec * kNS * 16, kNS * 16, tid, 256);
    __syncthreads();
    // tasks: layer 1: 20 (tap x 4 co tiles), layers 2, 3: 20 each, layer 4: 5
    for (int task = warp; task < 65; task += 8) {
      float acc[8][4];
      zero_acc(acc);
      if (task < 20) {  // layer 1: A = dH1^T (co), B = features (8 ci)
        const int tap = task >> 2, mt = task & 3;
        const uint32_t uD = smem_u32(sD), uF = smem_u32(sF);
        for (int kb = 0; kb < kNS; kb += 16) {
          uint32_t a[4], b[2];
          ldsm_x4_t(a, uD + swz64(kb + r + 8 * (q >> 1), 2 * mt + (q & 1)));
          ldsm_x2_t(b, uF + (kb + r + 8 * (q & 1) + tap + 6) * 16);
          mma_bf16(acc[0], a, b[0], b[1]);
        }
        __syncwarp();
        add_tile(part + oW1 + tap * 64 * 8, 8, 16 * mt, 64, acc, 1, lane);
      } else if (task < 60) {  // layers 2, 3: A = dH^T, B = previous hidden layer
        const int l = (task - 20) / 20, j = (task - 20) % 20, tap = j >> 2, mt = j & 3;
        const uint32_t uD = smem_u32(sD + (l + 1) * kNS * 128);
        const uint32_t uH = smem_u32(sH + l * kRows * 128);
        for (int kb = 0; kb < kNS; kb += 16) {
          uint32_t a[4];
          ldsm_x4_t(a, uD + swz64(kb + r + 8 * (q >> 1), 2 * mt + (q & 1)));
          const int brow = kb + r + 8 * (q & 1) + tap + 6;
#pragma unroll
          for (int np = 0; np < 4; ++np) {
            uint32_t b[4];
            ldsm_x4_t(b, uH + swz64(brow, 2 * np + (q >> 1)));
            mma_bf16(acc[2 * np], a, b[0], b[1]);
            mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
          }
        }
        __syncwarp();
        add_tile(part + (l ? oW3 : oW2) + tap * 64 * 64, 64, 16 * mt, 64, acc, 8, lane);
      } else {  // layer 4: A = dO^T (output 0; rows 8..15 of the tile read zeros)
        const int tap = task - 60;
        const uint32_t uO = smem_u32(sO), uZ = smem_u32(sZ);
        const uint32_t uH = smem_u32(sH + 2 * kRows * 128);
        for (int kb = 0; kb < kNS; kb += 16) {
          uint32_t a[4];
          ldsm_x4_t(a, (q & 1) ? uZ + r * 16 : uO + (kb + r + 8 * (q >> 1)) * 16);
          const int brow = kb + r + 8 * (q & 1) + tap + 6;
#pragma unroll
          for (int np = 0; np < 4; ++np) {
            uint32_t b[4];
            ldsm_x4_t(b, uH + swz64(brow, 2 * np + (q >> 1)));
            mma_bf16(acc[2 * np], a, b[0], b[1]);
            mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
          }
        }
        __syncwarp();
        add_tile(part + oW4 + tap * 64, 64, 0, 1, acc, 8, lane);
      }
    }
    // bias gradients: sums of the pre-activation gradients over positions
    if (tid < 193) {
      float sum = 0.0f;
      if (tid < 192) {
        const int l = tid >> 6, co = tid & 63;
        const unsigned char* d = sD + l * kNS * 128;
        for (int pos = 0; pos < kNS; ++pos) {
          const uint16_t hbits =
              *reinterpret_cast<const uint16_t*>(d + swz64(pos, co >> 3) + (co & 7) * 2);
          sum += __uint_as_float((uint32_t)hbits << 16);
        }
        part[(l == 0 ? ob1 : l == 1 ? ob2 : ob3) + co] += sum;
      } else {
        for (int pos = 0; pos < kNS; ++pos)
          sum += __uint_as_float((uint32_t)(*reinterpret_cast<const uint16_t*>(sO + pos * 16)) << 16);
        part[ob4] += sum;
      }
    }
  }
}

__global__ void reduce_kernel(const float* __restrict__ partial, int n_parts,
                              float* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  double s = 0.0;
  for (int c = 0; c < n_parts; ++c) s += (double)partial[(int64_t)c * kParams + i];
  grad[i] = (float)s;
}

__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ grad,
                            float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  prm[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Standalone inference through the BM kernel's fused routine: one warp per
// record, 4 warps per CTA sharing the weights.
constexpr int kInferSmem = kBlobBytes + 4 * kWarpScratch;

__global__ void __launch_bounds__(128) infer_kernel(const unsigned char* __restrict__ blob,
                                                    const unsigned char* __restrict__ feat, int n,
                                                    float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  copy16(sm, blob, kBlobBytes, tid, 128);
  unsigned char* scratch = sm + kBlobBytes + warp * kWarpScratch;
  for (int i = lane; i < kWarpScratch / 16; i += 32)
    reinterpret_cast<uint4*>(scratch)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for (int rec = blockIdx.x * 4 + warp; rec < n; rec += gridDim.x * 4) {
    const uint4* f = reinterpret_cast<const uint4*>(feat + (int64_t)rec * kFeatBytes);
    for (int i = lane; i < 256; i += 32) reinterpret_cast<uint4*>(scratch)[8 + i] = f[8 + i];
    __syncwarp();
    infer_unit(sm, scratch, lane);
    const float* o = reinterpret_cast<const float*>(scratch + kOffOut);
    for (int i = lane; i < 256; i += 32) out[(int64_t)rec * 256 + i] = o[i];
    __syncwarp();
  }
}

int grid_for(int n, int per) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long want = ((long long)n + per - 1) / per;
  long long cap = (long long)sms * 4;
  return (int)(want < cap ? (want < 1 ? 1 : want) : cap);
}

template <typename K>
int set_smem(K kernel, int bytes, const char* what) {
  CGB_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
               what);
  return CGB_OK;
}

}  // namespace ws
}  // namespace cgb

using namespace cgb;
using namespace cgb::ws;

extern "C" int cgb_ws_blob_bytes(void) { return kBlobBytes; }
extern "C" int cgb_ws_blobT_bytes(void) { return kBlobTBytes; }
extern "C" int cgb_ws_param_count(void) { return kParams; }

extern "C" int cgb_ws_pack_dev(const float* d_params, float s_out, float rm_scale, void* d_blob,
                               void* d_blobT, void* stream) {
  if (!d_params || !d_blob) return fail(CGB_ERR_ARG, "cgb_ws_pack_dev: null pointer");
  if ((reinterpret_cast<uintptr_t>(d_blob) & 15) || (reinterpret_cast<uintptr_t>(d_blobT) & 15))
    return fail(CGB_ERR_ARG, "cgb_ws_pack_dev: blobs must be 16-byte aligned");
  pack_kernel<<<64, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      d_params, s_out, rm_scale, static_cast<unsigned char*>(d_blob),
      static_cast<unsigned char*>(d_blobT));
  CGB_TRY_CUDA(cudaGetLastError(), "pack_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_prepare_dev(const float* d_rec, int n, const float* d_rm, float rm_scale,
                                  void* d_feat, float* d_target, float* d_nr, double* d_work,
                                  void* stream) {
  if (n == 0) return CGB_OK;
  if (n < 0 || !d_rec || !d_rm || !d_feat || !d_target || !d_nr || !d_work)
    return fail(CGB_ERR_ARG, "cgb_ws_prepare_dev: bad arguments");
  const int warps = 8;
  prepare_kernel<<<(n + warps - 1) / warps, warps * 32, 0,
                   reinterpret_cast<cudaStream_t>(stream)>>>(
      d_rec, n, d_rm, rm_scale, static_cast<unsigned char*>(d_feat), d_target, d_nr, d_work);
  CGB_TRY_CUDA(cudaGetLastError(), "prepare_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_forward_dev(const void* d_blob, const void* d_feat, int n, void* d_hid,
                                  float* d_out, void* stream) {
  if (n == 0) return CGB_OK;
  if (n < 0 || !d_blob || !d_feat || !d_hid || !d_out)
    return fail(CGB_ERR_ARG, "cgb_ws_forward_dev: bad arguments");
  if (set_smem(forward_kernel, kFwdSmem, "cudaFuncSetAttribute(forward)")) return CGB_ERR_CUDA;
  forward_kernel<<<grid_for(n, 1), 256, kFwdSmem, reinterpret_cast<cudaStream_t>(stream)>>>(
      static_cast<const unsigned char*>(d_blob), static_cast<const unsigned char*>(d_feat), n,
      static_cast<unsigned char*>(d_hid), d_out);
  CGB_TRY_CUDA(cudaGetLastError(), "forward_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_loss_dev(const float* d_out, const float* d_target, int n, float s_out,
                               void* d_dout, double* d_loss_part, void* stream) {
  if (n == 0) return CGB_OK;
  if (n < 0 || !d_out || !d_target || !d_dout || !d_loss_part)
    return fail(CGB_ERR_ARG, "cgb_ws_loss_dev: bad arguments");
  loss_kernel<<<n, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      d_out, d_target, n, s_out, static_cast<unsigned char*>(d_dout), d_loss_part);
  CGB_TRY_CUDA(cudaGetLastError(), "loss_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_backward_dev(const void* d_blobT, const void* d_dout, const void* d_hid,
                                   int n, void* d_dpre, void* stream) {
  if (n == 0) return CGB_OK;
  if (n < 0 || !d_blobT || !d_dout || !d_hid || !d_dpre)
    return fail(CGB_ERR_ARG, "cgb_ws_backward_dev: bad arguments");
  if (set_smem(backward_kernel, kBwdSmem, "cudaFuncSetAttribute(backward)")) return CGB_ERR_CUDA;
  backward_kernel<<<grid_for(n, 1), 256, kBwdSmem, reinterpret_cast<cudaStream_t>(stream)>>>(
      static_cast<const unsigned char*>(d_blobT), static_cast<const unsigned char*>(d_dout),
      static_cast<const unsigned char*>(d_hid), n, static_cast<unsigned char*>(d_dpre));
  CGB_TRY_CUDA(cudaGetLastError(), "backward_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_wgrad_dev(const void* d_feat, const void* d_hid, const void* d_dpre,
                                const void* d_dout, int n, float* d_partial, int n_parts,
                                float* d_grad, void* stream) {
  if (n < 0 || n_parts < 1 || !d_feat || !d_hid || !d_dpre || !d_dout || !d_partial || !d_grad)
    return fail(CGB_ERR_ARG, "cgb_ws_wgrad_dev: bad arguments");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (set_smem(wgrad_kernel, kWgSmem, "cudaFuncSetAttribute(wgrad)")) return CGB_ERR_CUDA;
  wgrad_kernel<<<n_parts, 256, kWgSmem, st>>>(
      static_cast<const unsigned char*>(d_feat), static_cast<const unsigned char*>(d_hid),
      static_cast<const unsigned char*>(d_dpre), static_cast<const unsigned char*>(d_dout), n,
      d_partial);
  CGB_TRY_CUDA(cudaGetLastError(), "wgrad_kernel launch");
  note_launch();
  reduce_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(d_partial, n_parts, d_grad);
  CGB_TRY_CUDA(cudaGetLastError(), "reduce_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_adam_dev(float* d_params, const float* d_grad, float* d_m, float* d_v,
                               int step, float lr, float beta1, float beta2, float eps,
                               void* stream) {
  if (!d_params || !d_grad || !d_m || !d_v || step < 1)
    return fail(CGB_ERR_ARG, "cgb_ws_adam_dev: bad arguments");
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<(kParams + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      d_params, d_grad, d_m, d_v, lr, beta1, beta2, eps, c1, c2);
  CGB_TRY_CUDA(cudaGetLastError(), "adam_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_ws_infer_dev(const void* d_blob, const void* d_feat, int n, float* d_out,
                                void* stream) {
  if (n == 0) return CGB_OK;
  if (n < 0 || !d_blob || !d_feat || !d_out)
    return fail(CGB_ERR_ARG, "cgb_ws_infer_dev: bad arguments");
  if (set_smem(infer_kernel, kInferSmem, "cudaFuncSetAttribute(infer)")) return CGB_ERR_CUDA;
  infer_kernel<<<grid_for(n, 4), 128, kInferSmem, reinterpret_cast<cudaStream_t>(stream)>>>(
      static_cast<const unsigned char*>(d_blob), static_cast<const unsigned char*>(d_feat), n,
      d_out);
  CGB_TRY_CUDA(cudaGetLastError(), "infer_kernel launch");
  note_launch();
  return CGB_OK;
}
