// Input generation (reference CudaGenerateInputFromProfile,
// src/cochlea.cu:4070-4103, normalisation :4165-4254) and the JND stage
// (CudaCalculateJND = GlobalCalculateMeanRate + GlobalCalculateJND,
// src/cochlea.cu:3741-3944, 3946-4065; final dB src/AudioGramCreator.cpp:454-508).

#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "cgb_device.cuh"
#include "cgb_internal.h"

namespace cgb {
namespace {

// x[p][n] = dA cos(2 pi f (n - head) / Fs) / norm_s + Wn (WN[n] - dc_w) / norm_w
// (signal_mode 0), or dA (S[n] - dc_s) / norm_s + ... (signal_mode 1), in
// double, stored as float.  2 pi is formed from the float constant PI of the
// reference (2 * 3.14159265f), as the reference does.
__global__ void input_gen_kernel(const cgb_profile* __restrict__ prof, int n_prof,
                                 const float* __restrict__ wn, const float* __restrict__ sig,
                                 int signal_mode, int interval_len, int head, float Fs,
                                 double wn_dc, double wn_norm, double sig_dc, double sig_norm,
                                 float* __restrict__ out) {
  const int p = blockIdx.y;
  const double two_pi = (double)(2.0f * 3.141592653589793f);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < interval_len;
       n += gridDim.x * blockDim.x) {
    const cgb_profile pr = prof[p];
    double sum;
    if (signal_mode) {
      sum = pr.dA * ((double)sig[n] - sig_dc) / sig_norm;
    } else {
      const double t = (double)(n - head) / (double)Fs;
      sum = pr.dA * cos(two_pi * pr.frequency * t) / sig_norm;
    }
    if (wn) sum = sum + pr.Wn * ((double)wn[n] - wn_dc) / wn_norm;
    out[(int64_t)p * interval_len + n] = (float)sum;
  }
}

// Hearing-aid shaping of generated input (CudaProcessSignalTroughHearingAID
// and ...IIR, src/cochlea.cu:4105-4150, applied at :4454-4503), per interval
// of length L, position n, as float fma chains in tap order:
//   aux[n] = sum_{i < min(n, Lf)} fir_i x[n-i]           (the first sample of
//            each interval gets no term: the reference bounds by n, not n+1)
//   out[n] = aux[n] + sum_{1 <= j < min(n+1, Li)} iir_j aux[n-j]
// The second stage reads aux only (not its own output).  Positions past the
// interval are not computed (the reference's grid can exceed the interval and
// then races into the next profile).
__global__ void hearing_aid_fir_kernel(const float* __restrict__ x, float* __restrict__ aux,
                                       int L, const float* __restrict__ fir, int fir_len) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= L) return;
  const int64_t base = (int64_t)blockIdx.y * L;
  const int back = min(n, fir_len);
  float acc = 0.0f;
  for (int i = 0; i < back; ++i) acc = __fmaf_rn(fir[i], x[base + n - i], acc);
  aux[base + n] = acc;
}

__global__ void hearing_aid_iir_kernel(const float* __restrict__ aux, float* __restrict__ out,
                                       int L, const float* __restrict__ iir, int iir_len) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= L) return;
  const int64_t base = (int64_t)blockIdx.y * L;
  const int back = min(n + 1, iir_len);
  float acc = aux[base + n];
  for (int j = 1; j < back; ++j) acc = __fmaf_rn(iir[j], aux[base + n - j], acc);
  out[base + n] = acc;
}

constexpr int kJndSections = 256;
constexpr int kJndGroups = 4;   // row groups per CTA (threads = 4 x 256)
constexpr int kJndThreads = kJndSections * kJndGroups;
constexpr int kJndRows = 8;     // rows per block of the walk

// A compensated FP32 sum (Kahan summation): s - c carries the sum of the
// added terms with an error of about 2 ulp of the total plus n eps^2 times
// the sum of |terms|; the terms here are never negative, so that is about
// 2 ulp of the total.
struct KahanF {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// The Fisher sums of one (interval, lambda plane): thread (g, s) walks the
// 8-row blocks b = g, g + 4, ... of the window of section s and of the same
// rows of the reference window, summing lambda and lambda_ref (the two mean
// rates) and (lambda - lambda_ref)^2 / lambda_ref (the AI term).  Each term
// is formed in FP32 and added to a compensated FP32 sum (KahanF), so the
// walk needs no FP64 operation (GB300's FP64 rate would bound it).  Rows past
// the last full block are added by the group that owns the next block.  The
// four groups' sums are then combined in FP64 in group order and the 256
// section terms reduced in FP64, so the result does not depend on
// scheduling.
__device__ __forceinline__ void jnd_interval(const float* __restrict__ lam, int64_t plane_rows,
                                             int j, int64_t row, int64_t ref_row, int len,
                                             double da, int out, int n_out,
                                             const double* __restrict__ nihc, double w,
                                             double Fs, double T, double* __restrict__ F_RA,
                                             double* __restrict__ F_AI,
                                             double* __restrict__ MR) {
  const int s = threadIdx.x & (kJndSections - 1), g = threadIdx.x / kJndSections;
  const float* c = lam + ((int64_t)j * plane_rows + row) * 256 + s;
  const float* rf = lam + ((int64_t)j * plane_rows + ref_row) * 256 + s;
  KahanF kc, kr, ka;
  const int nb = len / kJndRows;
  // two blocks per pass keep twice the loads in flight (same order of sums)
#pragma unroll 2
  for (int b = g; b < nb; b += kJndGroups) {
    const int t = b * kJndRows;
    float lc[kJndRows], lr[kJndRows];
#pragma unroll
    for (int k = 0; k < kJndRows; ++k) {
      lc[k] = c[(int64_t)(t + k) * 256];
      lr[k] = rf[(int64_t)(t + k) * 256];
    }
#pragma unroll
    for (int k = 0; k < kJndRows; ++k) {
      const float d = __fsub_rn(lc[k], lr[k]);
      kc.add(lc[k]);
      kr.add(lr[k]);
      ka.add(__fmul_rn(__fmul_rn(d, d), own_rcpf(lr[k])));
    }
  }
  if (g == nb % kJndGroups) {
    for (int t = nb * kJndRows; t < len; ++t) {
      const float lc = c[(int64_t)t * 256];
      const float lr = rf[(int64_t)t * 256];
      const float d = __fsub_rn(lc, lr);
      kc.add(lc);
      kr.add(lr);
      ka.add(__fmul_rn(__fmul_rn(d, d), own_rcpf(lr)));
    }
  }
  double sum_c = kc.value(), sum_r = kr.value(), sum_ai = ka.value();
  __shared__ double sh[3][kJndGroups][kJndSections];
  __shared__ double red[2][kJndSections / 32];
  sh[0][g][s] = sum_c;
  sh[1][g][s] = sum_r;
  sh[2][g][s] = sum_ai;
  __syncthreads();
  if (g == 0) {
    for (int k = 1; k < kJndGroups; ++k) {
      sum_c += sh[0][k][s];
      sum_r += sh[1][k][s];
      sum_ai += sh[2][k][s];
    }
    const double mr = sum_c / len, mrr = sum_r / len;
    if (MR) MR[((int64_t)j * n_out + out) * 256 + s] = mr;
    const double tl = (double)len / Fs;
    double rate = 0.0, ai = 0.0;
    if (da > 0.0) {
      const double dmr = (mr - mrr) / da;
      rate = nihc[s] * T * dmr * dmr / mrr;
      ai = nihc[s] * (T / tl) * sum_ai / (Fs * da * da);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      rate += __shfl_xor_sync(kFull, rate, o);
      ai += __shfl_xor_sync(kFull, ai, o);
    }
    if ((s & 31) == 0) {
      red[0][s >> 5] = rate;
      red[1][s >> 5] = ai;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ta = 0.0;
    for (int k = 0; k < kJndSections / 32; ++k) {
      tr += red[0][k];
      ta += red[1][k];
    }
    F_RA[(int64_t)j * n_out + out] = tr * w;
    F_AI[(int64_t)j * n_out + out] = ta * w;
  }
}

// Intervals of one run: interval i's window starts at row i * interval_nodes
// + head, its reference's at ref_of[i] * interval_nodes + head.
__global__ void __launch_bounds__(kJndThreads)
    jnd_kernel(const float* __restrict__ lam, int64_t plane_rows, int interval_nodes, int head,
               int len, const double* __restrict__ dA, const int32_t* __restrict__ ref_of,
               const double* __restrict__ nihc, double w0, double w1, double w2, double Fs,
               double T, double* __restrict__ F_RA, double* __restrict__ F_AI,
               double* __restrict__ MR, int n_int) {
  const int i = blockIdx.x, j = blockIdx.y;
  jnd_interval(lam, plane_rows, j, (int64_t)i * interval_nodes + head,
               (int64_t)ref_of[i] * interval_nodes + head, len, dA[i], i, n_int, nihc,
               j == 0 ? w0 : (j == 1 ? w1 : w2), Fs, T, F_RA, F_AI, MR);
}

// Intervals of any number of runs (groups of signals of different lengths)
// in one launch, from a descriptor table.
__global__ void __launch_bounds__(kJndThreads)
    jnd_batch_kernel(const float* __restrict__ lam, int64_t plane_rows,
                     const cgb_jnd_interval* __restrict__ iv, int n_out,
                     const double* __restrict__ nihc, double w0, double w1, double w2, double Fs,
                     double T, double* __restrict__ F_RA, double* __restrict__ F_AI,
                     double* __restrict__ MR) {
  // CTA b: descriptor b / 3, plane b % 3 (table order, planes together)
  const int b = (int)blockIdx.x, i = b / 3, j = b - 3 * i;
  const cgb_jnd_interval d = iv[i];
  jnd_interval(lam, plane_rows, j, d.row, d.ref_row, d.len, d.dA, d.out, n_out, nihc,
               j == 0 ? w0 : (j == 1 ? w1 : w2), Fs, T, F_RA, F_AI, MR);
}

}  // namespace
}  // namespace cgb

extern "C" int cgb_input_gen_dev(const cgb_profile* d_prof, int n_prof, const float* d_wn,
                                 const float* d_signal, int signal_mode, int interval_len,
                                 int head, float Fs, double wn_dc, double wn_norm, double sig_dc,
                                 double sig_norm, float* d_out, void* stream) {
  using namespace cgb;
  if (n_prof == 0 || interval_len == 0) return CGB_OK;
  if (!d_prof || !d_out || n_prof < 0 || interval_len < 0 || (signal_mode && !d_signal))
    return fail(CGB_ERR_ARG, "cgb_input_gen_dev: bad arguments");
  if (n_prof > 65535) return fail(CGB_ERR_RANGE, "cgb_input_gen_dev: more than 65535 profiles");
  if (!(wn_norm != 0.0) || !(sig_norm != 0.0))
    return fail(CGB_ERR_ARG, "cgb_input_gen_dev: zero normalisation factor");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int threads = 256;
  int bx = (interval_len + threads - 1) / threads;
  if (bx > 1024) bx = 1024;
  dim3 grid((unsigned)bx, (unsigned)n_prof);
  input_gen_kernel<<<grid, threads, 0, st>>>(d_prof, n_prof, d_wn, d_signal, signal_mode,
                                              interval_len, head, Fs, wn_dc, wn_norm, sig_dc,
                                              sig_norm, d_out);
  CGB_TRY_CUDA(cudaGetLastError(), "input_gen_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_jnd_dev(const float* d_lam, int64_t plane_rows, int n_int, int interval_nodes,
                           int head, int len, const double* d_dA, const int32_t* d_ref_of,
                           const double* d_nihc, const float* W, double Fs,
                           double delta_alpha_len_factor, double* d_F_RA, double* d_F_AI,
                           double* d_MR, void* stream) {
  using namespace cgb;
  if (n_int == 0) return CGB_OK;
  if (!d_lam || !d_dA || !d_ref_of || !d_nihc || !W || !d_F_RA || !d_F_AI || n_int < 0 ||
      len <= 0 || interval_nodes <= 0 || head < 0)
    return fail(CGB_ERR_ARG, "cgb_jnd_dev: bad arguments");
  if ((int64_t)n_int * interval_nodes > plane_rows || head + len > interval_nodes)
    return fail(CGB_ERR_RANGE, "cgb_jnd_dev: intervals reach outside the lambda planes");
  if (n_int > 2147483647 / 2) return fail(CGB_ERR_RANGE, "cgb_jnd_dev: too many intervals");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const double T = delta_alpha_len_factor / Fs;
  dim3 grid((unsigned)n_int, 3);
  jnd_kernel<<<grid, kJndThreads, 0, st>>>(d_lam, plane_rows, interval_nodes, head, len, d_dA,
                                           d_ref_of, d_nihc, (double)W[0], (double)W[1],
                                           (double)W[2], Fs, T, d_F_RA, d_F_AI, d_MR, n_int);
  CGB_TRY_CUDA(cudaGetLastError(), "jnd_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_hearing_aid_dev(float* d_in, int n_prof, int interval_len,
                                   const float* d_fir, int fir_len, const float* d_iir,
                                   int iir_len, float* d_aux, void* stream) {
  using namespace cgb;
  if (n_prof == 0 || interval_len == 0) return CGB_OK;
  if (!d_in || !d_aux || n_prof < 0 || interval_len < 0 || fir_len < 0 || iir_len < 0 ||
      (fir_len > 0 && !d_fir) || (iir_len > 0 && !d_iir))
    return fail(CGB_ERR_ARG, "cgb_hearing_aid_dev: bad arguments");
  if (n_prof > 65535) return fail(CGB_ERR_RANGE, "cgb_hearing_aid_dev: more than 65535 profiles");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid((unsigned)((interval_len + 255) / 256), (unsigned)n_prof);
  hearing_aid_fir_kernel<<<grid, 256, 0, st>>>(d_in, d_aux, interval_len, d_fir, fir_len);
  CGB_TRY_CUDA(cudaGetLastError(), "hearing_aid_fir_kernel launch");
  note_launch();
  if (iir_len > 0) {
    hearing_aid_iir_kernel<<<grid, 256, 0, st>>>(d_aux, d_in, interval_len, d_iir, iir_len);
    CGB_TRY_CUDA(cudaGetLastError(), "hearing_aid_iir_kernel launch");
  } else {
    CGB_TRY_CUDA(cudaMemcpyAsync(d_in, d_aux, (size_t)n_prof * interval_len * sizeof(float),
                                 cudaMemcpyDeviceToDevice, st),
                 "hearing aid copy-back");
  }
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_jnd_batch_dev(const float* d_lam, int64_t plane_rows,
                                 const cgb_jnd_interval* d_iv, int n_iv, int n_out,
                                 const double* d_nihc, const float* W, double Fs,
                                 double delta_alpha_len_factor, double* d_F_RA, double* d_F_AI,
                                 double* d_MR, void* stream) {
  using namespace cgb;
  if (n_iv == 0) return CGB_OK;
  if (!d_lam || !d_iv || !d_nihc || !W || !d_F_RA || !d_F_AI || n_iv < 0 || n_out <= 0 ||
      plane_rows <= 0)
    return fail(CGB_ERR_ARG, "cgb_jnd_batch_dev: bad arguments");
  if (n_iv > 2147483647 / 3) return fail(CGB_ERR_RANGE, "cgb_jnd_batch_dev: too many intervals");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const double T = delta_alpha_len_factor / Fs;
  dim3 grid((unsigned)(3 * n_iv));
  jnd_batch_kernel<<<grid, kJndThreads, 0, st>>>(d_lam, plane_rows, d_iv, n_out, d_nihc,
                                                 (double)W[0], (double)W[1], (double)W[2], Fs, T,
                                                 d_F_RA, d_F_AI, d_MR);
  CGB_TRY_CUDA(cudaGetLastError(), "jnd_batch_kernel launch");
  note_launch();
  return CGB_OK;
}

extern "C" int cgb_jnd_final(const double* F_RA, const double* F_AI, int n_int,
                             const int32_t* ref_of, double spl_ref, double max_db,
                             double* jnd_rate_db, double* jnd_ai_db) {
  if (!F_RA || !F_AI || !ref_of || !jnd_rate_db || !jnd_ai_db || n_int < 0)
    return cgb::fail(CGB_ERR_ARG, "cgb_jnd_final: bad arguments");
  const double max_pa = std::pow(10.0, max_db / 20.0) * spl_ref;
  auto to_db = [&](double sum) {
    const double pa = 1.0 / std::sqrt(sum);
    return (std::isinf(pa) || pa > max_pa) ? max_db : 20.0 * std::log10(pa / spl_ref);
  };
  for (int i = 0; i < n_int; ++i) {
    double ra = 0.0, ai = 0.0;
    for (int j = 0; j < 3; ++j) {
      ra += F_RA[(int64_t)j * n_int + i];
      ai += F_AI[(int64_t)j * n_int + i];
    }
    const bool is_ref = ref_of[i] == i;
    jnd_rate_db[i] = is_ref ? NAN : to_db(ra);
    jnd_ai_db[i] = is_ref ? NAN : to_db(ai);
  }
  return CGB_OK;
}

extern "C" int cgb_noise_normalization(const float* src, int normalize_type,
                                       double normalize_to_interval, double remove_dc,
                                       int start_dc, int end_dc, int start_norm, int end_norm,
                                       float Fs, double* dc, double* factor) {
  if (!dc || !factor) return cgb::fail(CGB_ERR_ARG, "cgb_noise_normalization: null output");
  // src == null: a pure tone (calculateDCANDNornalizationFactorPureTone)
  double d = 0.0, e;
  if (src) {
    if (end_dc <= start_dc || end_norm <= start_norm)
      return cgb::fail(CGB_ERR_ARG, "cgb_noise_normalization: empty window");
    d = src[start_dc];
    for (int i = start_dc + 1; i < end_dc; ++i) d = d + src[i];
    d = remove_dc * d / (double)(end_dc - start_dc);
    // the first term enters without the dc removed, as in the reference
    e = (double)src[start_norm] * (double)src[start_norm];
    for (int i = start_norm + 1; i < end_norm; ++i) e = e + ((src[i] - d) * (src[i] - d));
    e = std::sqrt(e);
  } else {
    e = std::sqrt(0.5 * (double)(end_norm - start_norm));
  }
  if (normalize_type == 1)
    e = e / std::sqrt((double)(end_norm - start_norm));
  else if (normalize_type == 2 && normalize_to_interval > 0)
    e = e / std::sqrt(Fs * normalize_to_interval);
  else if (normalize_type == 3)
    e = 1.0;
  *dc = d;
  *factor = e;
  return CGB_OK;
}
