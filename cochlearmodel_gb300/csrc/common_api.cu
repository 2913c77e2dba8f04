// The reference-named host API (include/cochlea_common.h) over the C ABI.
//
// Ownership and call semantics follow the reference's src/cochlea.cu:63-631:
// the library holds the device buffers of one run (velocity, lambda, JND
// intermediates), the caller passes host arrays that are copied
// synchronously, and every entry point returns with its GPU work finished.
// A failed CUDA call or a request this build does not provide raises
// std::runtime_error, as the reference's gpuAssert does.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "cgb_internal.h"
#include "cochlea_common.h"

namespace {

void gpu_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("cochlea_gb300: ") + what + ": " +
                             cudaGetErrorString(e));
}

void cgb_check(int status, const char* what) {
  if (status != CGB_OK)
    throw std::runtime_error(std::string("cochlea_gb300: ") + what + ": " + cgb_last_error());
}

template <class T>
void ensure(T*& p, size_t& have, size_t want, const char* what) {
  if (want <= have && p) return;
  if (p) gpu_check(cudaFree(p), what);
  p = nullptr;
  have = 0;
  if (want == 0) return;
  gpu_check(cudaMalloc(reinterpret_cast<void**>(&p), want * sizeof(T)), what);
  gpu_check(cudaMemset(p, 0, want * sizeof(T)), what);
  have = want;
}

template <class T>
void release(T*& p, size_t& have) {
  if (p) cudaFree(p);
  p = nullptr;
  have = 0;
}

// ---- per-unit statistics -> the reference's per-node / per-block arrays ----
__global__ void split_conv_kernel(const cgb_unit* units, int n_units, const float* conv,
                                  const cgb_unit_stats* stats, float* conv_time,
                                  float* conv_steps, float* conv_loops, float* blk_time,
                                  float* blk_steps, float* blk_loops, int* failed_blocks) {
  const int b = blockIdx.x;
  if (b >= n_units) return;
  const cgb_unit u = units[b];
  const int first = max(u.start, u.out_first);
  const float span = (float)(u.end - u.out_first);
  float st = 0.f, ss = 0.f, sl = 0.f;
  for (int n = first + threadIdx.x; n < u.end; n += blockDim.x) {
    const int64_t r = u.out_base + n;
    const float t = conv[r * 3 + 0], s = conv[r * 3 + 1], l = conv[r * 3 + 2];
    conv_time[r] = t;
    conv_steps[r] = s;
    conv_loops[r] = l;
    st += t / span;
    ss += s / span;
    sl += l / span;
  }
  for (int o = 16; o >= 1; o >>= 1) {
    st += __shfl_xor_sync(0xffffffffu, st, o);
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    sl += __shfl_xor_sync(0xffffffffu, sl, o);
  }
  __shared__ float acc[3][32];
  if ((threadIdx.x & 31) == 0) {
    acc[0][threadIdx.x >> 5] = st;
    acc[1][threadIdx.x >> 5] = ss;
    acc[2][threadIdx.x >> 5] = sl;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, c = 0.f, d = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += acc[0][w];
      c += acc[1][w];
      d += acc[2][w];
    }
    blk_time[b] = a;
    blk_steps[b] = c;
    blk_loops[b] = d;
    failed_blocks[b] = stats[b].failed_samples;
  }
}

// CUDAFIXJND_Lambda (src/cochlea.cu:4512-4532): lambda <- max(0, lambda - spont),
// buffer <- max(spont, lambda) when requested.
template <class T>
__global__ void fix_lambda_kernel(T* lam, T* buf, int64_t plane, float s0, float s1, float s2,
                                  int update_buffer) {
  const int j = blockIdx.y;
  const float sp = j == 0 ? s0 : (j == 1 ? s1 : s2);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < plane;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = (int64_t)j * plane + i;
    const float v = (float)lam[k];
    if (update_buffer) buf[k] = T(fmaxf(sp, v));
    lam[k] = T(fmaxf(0.0f, v - sp));
  }
}

// The JND's debug stages (GlobalCalculateJND's backup_stage,
// src/cochlea.cu:3773-3944), written into the stage buffer in the reference's
// layouts, for interval i of plane j (block (i, j)), section s (thread):
//   1 AvgMeanRate  out[j n + i] = mean over sections of MR
//   2 dMeanRate    out[(j n + i) 256 + s] = (MR - MR_ref) / dA
//   3 dLambda      out[j plane + 256 (i L + head + t) + s] = (l - l_ref) / dA
//                  (0 where dA <= 0), t < len
//   4 preFisherAI  same positions: dLambda^2 / (Fs l_ref)
//   5 preFisherAITimeReduced  out[(j n + i) 256 + s] =
//                  (T / Tlength) nIHC_s sum_t preFisherAI
//   6 CRLB_RA      out[(j n + i) 256 + s] = 1 / sqrt(T dMR^2 / MR_ref)
// MR is the JND kernel's (double) mean rate.  The hot JND kernel keeps its
// own order; these are for inspection and are computed separately.
__global__ void jnd_stage_kernel(int stage, const float* lam, int64_t plane, const double* MR,
                                 const double* dA, const int32_t* ref_of, const double* nihc,
                                 int n, int L, int head, int len, double Fs, double T,
                                 float* out) {
  const int i = blockIdx.x, j = blockIdx.y, s = threadIdx.x;
  const int r = ref_of[i];
  const double da = dA[i];
  const double mr = MR[((size_t)j * n + i) * 256 + s], mrr = MR[((size_t)j * n + r) * 256 + s];
  const double dmr = (mr - mrr) / da;
  const size_t mo = ((size_t)j * n + i) * 256 + s;
  if (stage == 1) {
    __shared__ double acc[256];
    acc[s] = mr;
    for (int t = 128; t >= 1; t >>= 1) {
      __syncthreads();
      if (s < t) acc[s] += acc[s + t];
    }
    if (s == 0) out[(size_t)j * n + i] = (float)(acc[0] / 256.0);
  } else if (stage == 2) {
    out[mo] = (float)dmr;
  } else if (stage == 6) {
    out[mo] = (float)(1.0 / sqrt(T * dmr * dmr / mrr));
  } else {
    const float* c = lam + (size_t)j * plane + 256 * ((size_t)i * L + head) + s;
    const float* rf = lam + (size_t)j * plane + 256 * ((size_t)r * L + head) + s;
    float* o = out + (size_t)j * plane + 256 * ((size_t)i * L + head) + s;
    double sum = 0.0;
    for (int t = 0; t < len; ++t) {
      const double dl = da > 0.0 ? ((double)c[(size_t)t * 256] - rf[(size_t)t * 256]) / da : 0.0;
      const double pre = dl * dl / (Fs * (double)rf[(size_t)t * 256]);
      if (stage == 3) o[(size_t)t * 256] = (float)dl;
      if (stage == 4) o[(size_t)t * 256] = (float)pre;
      sum += pre;
    }
    if (stage == 5) out[mo] = (float)((T / ((double)len / Fs)) * nihc[s] * sum);
  }
}

__global__ void to_float_kernel(const double* src, float* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// dA of each JND window: sqrt(max x^2) (cudaCalculateDA, src/cochlea.cu:3726-3738)
__global__ void calc_dA_kernel(const float* in, double* dA, int n_int, int interval_nodes,
                               int head, int len, int offset) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_int) return;
  float acc = 0.0f;
  const int s = offset + i * interval_nodes + head;
  for (int k = s; k < s + len; ++k) {
    const float c = in[k] * in[k];
    if (acc < c) acc = c;
  }
  dA[i] = (double)sqrtf(acc);
}

struct Holder {
  // model
  float* secp = nullptr;       size_t secp_n = 0;
  float* gamma = nullptr;      size_t gamma_n = 0;
  // BM run
  float* input = nullptr;      size_t input_n = 0;
  float* speeds = nullptr;     size_t speeds_n = 0;
  int32_t* failed = nullptr;   size_t failed_n = 0;
  float* conv = nullptr;       size_t conv_n = 0;
  float* conv_time = nullptr;  size_t conv_time_n = 0;
  float* conv_steps = nullptr; size_t conv_steps_n = 0;
  float* conv_loops = nullptr; size_t conv_loops_n = 0;
  float* blk_time = nullptr;   size_t blk_time_n = 0;
  float* blk_steps = nullptr;  size_t blk_steps_n = 0;
  float* blk_loops = nullptr;  size_t blk_loops_n = 0;
  int* failed_blocks = nullptr; size_t failed_blocks_n = 0;
  cgb_unit* units = nullptr;   size_t units_n = 0;
  cgb_unit_stats* stats = nullptr; size_t stats_n = 0;
  int32_t* work = nullptr;     size_t work_n = 0;
  std::vector<float> tol_mtt, tol_mmspt;  // per block, from setupToleranceProfile
  // Aihc
  std::vector<float> aihc;
  bool aihc_loaded = false;
  float* d_aihc = nullptr;     size_t d_aihc_n = 0;
  // IHC / lambda
  bool ihc_ready = false;
  std::vector<float> ac_taps, dc_taps, ac_a_taps;
  bool ac_iir = false;
  float* ac_buf = nullptr;     size_t ac_buf_n = 0;   // AC by velocity row (IIR path)
  cgb_ihc_params ihc_prm{};
  float W[3] = {0.61f, 0.23f, 0.16f};
  float* dmg = nullptr;        size_t dmg_n = 0;
  float* lam = nullptr;        size_t lam_n = 0;
  float* buffer1 = nullptr;    size_t buffer1_n = 0;
  unsigned char* scratch = nullptr; size_t scratch_n = 0;
  int32_t* status = nullptr;   size_t status_n = 0;
  int calc_time = 0, interval_nodes = 0, time_blocks = 0, decouple = 0, lambda_offset = 0;
  // JND
  double* mean_rate = nullptr; size_t mean_rate_n = 0;
  float* mean_rate_f = nullptr; size_t mean_rate_f_n = 0;
  double* nihc = nullptr;      size_t nihc_n = 0;
  double* dA = nullptr;        size_t dA_n = 0;
  int32_t* ref_of = nullptr;   size_t ref_of_n = 0;
  double* F = nullptr;         size_t F_n = 0;
  // input generation
  std::vector<device_jnd_params> profiles;
  cgb_profile* d_prof = nullptr; size_t d_prof_n = 0;
  float* wn = nullptr;         size_t wn_n = 0;
  float* sig = nullptr;        size_t sig_n = 0;
  double wn_dc = 0, wn_norm = 1, sig_dc = 0, sig_norm = 1;
} H;

}  // namespace

// ---------------------------------------------------------------- timing
extern "C" void cudaEventsCreate(cudaEvent_t& start, cudaEvent_t& stop, int condition) {
  if (condition) {
    gpu_check(cudaEventCreate(&start), "cudaEventCreate");
    gpu_check(cudaEventCreate(&stop), "cudaEventCreate");
  }
}
extern "C" void cudaEventsStartTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition) {
  (void)stop;
  if (condition) gpu_check(cudaEventRecord(start), "cudaEventRecord");
}
extern "C" void cudaEventsStopTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition) {
  (void)start;
  if (condition) gpu_check(cudaEventRecord(stop), "cudaEventRecord");
}
extern "C" float cudaEventsStopQueryTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition,
                                          const std::string& prefix) {
  cudaEventsStopTimer(start, stop, condition);
  float ms = 0.0f;
  if (condition) {
    gpu_check(cudaEventSynchronize(stop), "cudaEventSynchronize");
    gpu_check(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
    printf("%s : %.2f (msec) \n", prefix.c_str(), ms);
  }
  return ms;
}
extern "C" void viewGPUStatus(int flags, const std::string& prefix) {
  if (flags & 16) {
    size_t fr = 0, tot = 0;
    gpu_check(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    printf("%s : GPU Memory, Free(%d MB) / Total(%d MB)\n", prefix.c_str(),
           (int)(fr / (1024 * 1024)), (int)(tot / (1024 * 1024)));
  }
}

// ---------------------------------------------------------------- buffers
extern "C" JNDFloat* getCudaBuffer() { return H.buffer1; }
extern "C" JNDFloat* getCudaLambda() { return H.lam; }
extern "C" JNDFloat* getCudaMeanRate() { return H.mean_rate_f; }
extern "C" int* getCudaFailedTimeNodes() { return H.failed; }
extern "C" int* getCudaFailedBlocks() { return H.failed_blocks; }
extern "C" float* getCudaConvergeSpeedBlocks() { return H.blk_time; }
extern "C" float* getCudaConvergedTimeNodes() { return H.conv_steps; }
extern "C" float* getCudaConvergedBlocks() { return H.blk_steps; }
extern "C" float* getCudaConvergedJacobyLoopsPerIteration() { return H.conv_loops; }
extern "C" float* getCudaConvergedJacobyLoopsPerIterationBlocks() { return H.blk_loops; }

extern "C" void loadAihc(float* Aihc) {
  if (!H.aihc_loaded) {
    H.aihc.assign(Aihc, Aihc + 256 * LAMBDA_COUNT);
    ensure(H.d_aihc, H.d_aihc_n, (size_t)256 * LAMBDA_COUNT, "loadAihc");
    gpu_check(cudaMemcpy(H.d_aihc, Aihc, 256 * LAMBDA_COUNT * sizeof(float),
                         cudaMemcpyHostToDevice),
              "loadAihc");
    H.aihc_loaded = true;
  }
}
extern "C" void enableloadAihc() { H.aihc_loaded = false; }

extern "C" void allocateBuffer(const int size_in_nodes, int, cudaEvent_t&, cudaEvent_t&,
                               cudaDeviceProp) {
  ensure(H.buffer1, H.buffer1_n, (size_t)size_in_nodes, "allocateBuffer");
}
extern "C" void releaseBuffer(int, cudaEvent_t&, cudaEvent_t&, cudaDeviceProp) {
  release(H.buffer1, H.buffer1_n);
}
extern "C" void cudaMallocatingByMode(void** ptr, size_t bytes_num, bool disable_advanced_mode) {
  if (disable_advanced_mode)
    gpu_check(cudaMalloc(ptr, bytes_num), "cudaMalloc");
  else
    gpu_check(cudaMallocManaged(ptr, bytes_num), "cudaMallocManaged");
}

// ---------------------------------------------------------------- copies
extern "C" void GeneralKernel_Copy_Results(float* target, float* src, size_t size) {
  gpu_check(cudaMemcpy(target, src, size * sizeof(float), cudaMemcpyDeviceToHost), "copy");
}
extern "C" void GeneralKernel_Copy_Results_Double(double* target, double* src, size_t size) {
  gpu_check(cudaMemcpy(target, src, size * sizeof(double), cudaMemcpyDeviceToHost), "copy");
}
extern "C" void ReverseKernel_Copy_Results(float* src, size_t size) {
  gpu_check(cudaMemcpy(H.speeds, src, size * sizeof(float), cudaMemcpyHostToDevice), "copy");
}
extern "C" void BMOHCKernel_Copy_Results(float* target, size_t resultNodes, size_t offset) {
  gpu_check(cudaMemcpy(target, H.speeds + offset, resultNodes * sizeof(float),
                       cudaMemcpyDeviceToHost),
            "BMOHCKernel_Copy_Results");
}
extern "C" void BMOHCKernel_Copy_Lambda(JNDFloat* target, size_t lambdaNodes, int offset) {
  gpu_check(cudaMemcpy(target, H.buffer1 + offset, lambdaNodes * sizeof(JNDFloat),
                       cudaMemcpyDeviceToHost),
            "BMOHCKernel_Copy_Lambda");
}
extern "C" void extractConvergenceTimes(float* convergence_times, size_t nodes) {
  gpu_check(cudaMemcpy(convergence_times, H.conv_time, nodes * sizeof(float),
                       cudaMemcpyDeviceToHost),
            "extractConvergenceTimes");
}
extern "C" void BMOHCKernel_Wait_Threads() {
  gpu_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

template <class T>
void GeneralKernel_Copy_Results_Template(T* target, T* src, size_t size, size_t offset) {
  gpu_check(cudaMemcpy(target, src + offset, size * sizeof(T), cudaMemcpyDeviceToHost), "copy");
}
template <class T>
void GeneralKernel_Copy_Results_Template(T* target, T* src, size_t size) {
  GeneralKernel_Copy_Results_Template<T>(target, src, size, 0);
}
template <class T>
void ReverseKernel_Copy_Results_Template(T* cpu_src, T* cuda_target, size_t start_time_node,
                                         size_t time_nodes, int sections) {
  gpu_check(cudaMemcpy(cuda_target, &cpu_src[start_time_node * sections],
                       time_nodes * sections * sizeof(T), cudaMemcpyHostToDevice),
            "copy");
}
template <class T>
void updateCUDALambdaArray(T* lambda_array, T* cuda_buffer, size_t calc_time_nodes, int sections,
                           int, int, int cuda_buffer_update, Log&) {
  const int64_t plane = (int64_t)calc_time_nodes * sections;
  dim3 grid(1024, LAMBDA_COUNT);
  fix_lambda_kernel<T><<<grid, 256>>>(lambda_array, cuda_buffer, plane, H.ihc_prm.spont[0],
                                      H.ihc_prm.spont[1], H.ihc_prm.spont[2],
                                      cuda_buffer_update);
  gpu_check(cudaGetLastError(), "fix_lambda_kernel");
  gpu_check(cudaDeviceSynchronize(), "fix_lambda_kernel");
}
template void GeneralKernel_Copy_Results_Template<double>(double*, double*, size_t);
template void GeneralKernel_Copy_Results_Template<float>(float*, float*, size_t);
template void GeneralKernel_Copy_Results_Template<int>(int*, int*, size_t);
template void GeneralKernel_Copy_Results_Template<double>(double*, double*, size_t, size_t);
template void GeneralKernel_Copy_Results_Template<float>(float*, float*, size_t, size_t);
template void GeneralKernel_Copy_Results_Template<int>(int*, int*, size_t, size_t);
template void ReverseKernel_Copy_Results_Template<float>(float*, float*, size_t, size_t, int);
template void ReverseKernel_Copy_Results_Template<double>(double*, double*, size_t, size_t, int);
template void updateCUDALambdaArray<float>(float*, float*, size_t, int, int, int, int, Log&);
template void updateCUDALambdaArray<double>(double*, double*, size_t, int, int, int, int, Log&);

// ---------------------------------------------------------------- BM
extern "C" void BMOHCKernel_Init(float* gamma, float* mass, float* M, float* U, float* L,
                                 float* R, float* S, float* Q, float* S_ohc, float* S_tm,
                                 float* R_tm, float, float, size_t inputBufferNodes,
                                 size_t resultBufferNodes, size_t, bool, int, int, Log&) {
  (void)U;
  (void)L;  // kernel 17 uses 1/m only (the upper diagonal is all ones, the
            // lower one is 1 below row 254, include/cochlea.cuh:13736)
  float secp[8 * 256];
  for (int i = 0; i < 256; ++i) {
    secp[0 * 256 + i] = 1.0f / mass[i];
    secp[1 * 256 + i] = M[i];
    secp[2 * 256 + i] = R[i];
    secp[3 * 256 + i] = S[i];
    secp[4 * 256 + i] = Q[i];
    secp[5 * 256 + i] = S_ohc[i];
    secp[6 * 256 + i] = S_tm[i];
    secp[7 * 256 + i] = R_tm[i];
  }
  ensure(H.secp, H.secp_n, (size_t)8 * 256, "BMOHCKernel_Init");
  ensure(H.gamma, H.gamma_n, (size_t)256, "BMOHCKernel_Init");
  gpu_check(cudaMemcpy(H.secp, secp, sizeof(secp), cudaMemcpyHostToDevice), "upload model");
  gpu_check(cudaMemcpy(H.gamma, gamma, 256 * sizeof(float), cudaMemcpyHostToDevice),
            "upload gamma");
  ensure(H.input, H.input_n, inputBufferNodes + 4, "input buffer");
  ensure(H.speeds, H.speeds_n, std::max(resultBufferNodes, inputBufferNodes * 256), "speeds");
  const size_t rows = H.speeds_n / 256;
  ensure(H.failed, H.failed_n, rows, "failed nodes");
  ensure(H.conv, H.conv_n, rows * 3, "convergence");
  ensure(H.conv_time, H.conv_time_n, rows, "convergence");
  ensure(H.conv_steps, H.conv_steps_n, rows, "convergence");
  ensure(H.conv_loops, H.conv_loops_n, rows, "convergence");
  ensure(H.work, H.work_n, (size_t)4, "work queue");
}

extern "C" void BMOHCKernel_Free() {
  release(H.secp, H.secp_n);
  release(H.gamma, H.gamma_n);
  release(H.input, H.input_n);
  release(H.speeds, H.speeds_n);
  release(H.failed, H.failed_n);
  release(H.conv, H.conv_n);
  release(H.conv_time, H.conv_time_n);
  release(H.conv_steps, H.conv_steps_n);
  release(H.conv_loops, H.conv_loops_n);
  release(H.blk_time, H.blk_time_n);
  release(H.blk_steps, H.blk_steps_n);
  release(H.blk_loops, H.blk_loops_n);
  release(H.failed_blocks, H.failed_blocks_n);
  release(H.units, H.units_n);
  release(H.stats, H.stats_n);
  release(H.work, H.work_n);
}

// Kernel selection (src/cochlea.cu:1258-2331).  Run_Fast_BM_Calculation 0,
// the reference default (src/params.cpp:157), is BMOHC_NEW_kernel: this
// library runs it with the reference's own step controller and operation
// order (controller 1, arith 1).  17 is kernel 17, run with the full-sum
// value of its step controller (controller 0, own operation order).  Other
// variants are not built and raise.  BMOHC_Kernel_Configuration is only the
// reference's cudaFuncSetCacheConfig hint (0-3), which changes no result;
// the OHC nonlinearity and oval window are always on in both kernels, so
// enable_psi / enable_OW other than 1 raise rather than being ignored.
extern "C" void BMOHCNewKernel(
    float* input_samples, bool override_input_samples, float w_ohc, float time_step,
    float time_step_out, float delta_x, float alpha_r, int enable_psi, int enable_OW, int,
    float Ts,
    float _ohc_alpha_l, float _ohc_alpha_s, float model_Gme, float model_a0, float model_a1,
    float model_a2, float sigma_ow, float eta_1, float eta_2, float*, int Time_Blocks,
    int samplesBufferLengthP1, int overlap_nodes_for_block, long, int, float cuda_max_time_step,
    float cuda_min_time_step, int Decouple_Filter, float Max_M1_SP_Error_Parameter,
    float Max_Tolerance_Parameter, int Relative_Error_Parameters,
    int calculate_boundary_conditions, float M1_SP_Fix_Factor, float Tolerance_Fix_Factor,
    float SPLREfVal, int, int, int, int JACOBBY_Loops_Fast, int JACOBBY_Loops_Slow,
    int Cuda_Outern_Loops, int Run_Fast_BM_Calculation, int BMOHC_Kernel_Configuration,
    cudaEvent_t&, cudaEvent_t&, cudaDeviceProp, Log&) {
  if (!H.secp) throw std::runtime_error("cochlea_gb300: BMOHCNewKernel before BMOHCKernel_Init");
  if (Run_Fast_BM_Calculation != 0 && Run_Fast_BM_Calculation != 17)
    throw std::runtime_error("cochlea_gb300: Run_Fast_BM_Calculation " +
                             std::to_string(Run_Fast_BM_Calculation) +
                             " is not built (0: BMOHC_NEW_kernel, 17: kernel 17)");
  if (BMOHC_Kernel_Configuration < 0 || BMOHC_Kernel_Configuration > 3)
    throw std::runtime_error("cochlea_gb300: BMOHC_Kernel_Configuration must be 0-3");
  if (enable_psi != 1 || enable_OW != 1)
    throw std::runtime_error(
        "cochlea_gb300: enable_psi and enable_OW must be 1 (the reference's kernels 0 and 17 "
        "always run the OHC nonlinearity and the oval window)");
  if ((size_t)samplesBufferLengthP1 + 2 > H.input_n)
    throw std::runtime_error("cochlea_gb300: input longer than the BMOHCKernel_Init buffer");
  if (!override_input_samples)
    gpu_check(cudaMemcpy(H.input, input_samples, (size_t)samplesBufferLengthP1 * sizeof(float),
                         cudaMemcpyHostToDevice),
              "upload input");
  std::vector<int32_t> st(Time_Blocks), of(Time_Blocks), en(Time_Blocks);
  cgb_check(cgb_block_partition(Time_Blocks, samplesBufferLengthP1, overlap_nodes_for_block,
                                Decouple_Filter, st.data(), of.data(), en.data()),
            "block partition");
  // Per-block tolerances: setupToleranceProfile's table for generated input;
  // for file input with relative errors, the per-block power rule the
  // reference computes in calculateBoundariesForNonGeneratedInput
  // (src/cochlea.cu:919-963); otherwise the two constants.
  std::vector<float> mtt(Time_Blocks, Max_Tolerance_Parameter),
      mmspt(Time_Blocks, Max_M1_SP_Error_Parameter);
  if (calculate_boundary_conditions && Relative_Error_Parameters) {
    std::vector<float> host(samplesBufferLengthP1);
    gpu_check(cudaMemcpy(host.data(), H.input, host.size() * sizeof(float),
                         cudaMemcpyDeviceToHost),
              "read input");
    for (int b = 0; b < Time_Blocks; ++b) {
      float mx = 0.0f;
      for (int k = st[b]; k < en[b]; ++k) mx = std::max(mx, std::fabs(host[k]));
      const float pw = (1.0f / SPLREfVal) * mx;
      const float db = pw > 0.0f ? 20 * log10f(0.1f * pw) : 0.0f;
      mmspt[b] = Max_M1_SP_Error_Parameter * powf(10.0f, M1_SP_Fix_Factor * db);
      mtt[b] = Max_Tolerance_Parameter * powf(10.0f, Tolerance_Fix_Factor * db);
    }
  } else if (!calculate_boundary_conditions && (int)H.tol_mtt.size() >= Time_Blocks) {
    for (int b = 0; b < Time_Blocks; ++b) {
      mtt[b] = H.tol_mtt[b];
      mmspt[b] = H.tol_mmspt[b];
    }
  }
  std::vector<cgb_unit> units(Time_Blocks);
  for (int b = 0; b < Time_Blocks; ++b)
    units[b] = cgb_unit{0, 0, st[b], of[b], en[b], 0, mtt[b], mmspt[b]};
  const int64_t rows = (int64_t)(H.speeds_n / 256);
  cgb_check(cgb_check_units(units.data(), Time_Blocks, 1, (int64_t)H.input_n, rows),
            "unit table");
  ensure(H.units, H.units_n, (size_t)Time_Blocks, "units");
  ensure(H.stats, H.stats_n, (size_t)Time_Blocks, "stats");
  ensure(H.blk_time, H.blk_time_n, (size_t)Time_Blocks, "blocks");
  ensure(H.blk_steps, H.blk_steps_n, (size_t)Time_Blocks, "blocks");
  ensure(H.blk_loops, H.blk_loops_n, (size_t)Time_Blocks, "blocks");
  ensure(H.failed_blocks, H.failed_blocks_n, (size_t)Time_Blocks, "blocks");
  gpu_check(cudaMemcpy(H.units, units.data(), units.size() * sizeof(cgb_unit),
                       cudaMemcpyHostToDevice),
            "upload units");
  cgb_bm_scalars sc{};
  sc.w_ohc = w_ohc;
  sc.time_step = time_step;
  sc.time_step_out = time_step_out;
  sc.delta_x = delta_x;
  sc.alpha_r = alpha_r;
  sc.Ts = Ts;
  sc.alpha_l = _ohc_alpha_l;
  sc.alpha_s = _ohc_alpha_s;
  sc.Gme = model_Gme;
  sc.a0 = model_a0;
  sc.a1 = model_a1;
  sc.a2 = model_a2;
  sc.sigma_ow = sigma_ow;
  sc.eta_1 = eta_1;
  sc.eta_2 = eta_2;
  sc.dt_min = cuda_min_time_step;
  sc.dt_max = cuda_max_time_step;
  sc.jacobi_fast = JACOBBY_Loops_Fast;
  sc.jacobi_slow = JACOBBY_Loops_Slow;
  sc.max_outer = Cuda_Outern_Loops;
  sc.red_lanes = 32;
  sc.jacobi_mode = 0;
  sc.max_substeps_per_sample = 1 << 20;
  sc.controller = Run_Fast_BM_Calculation == 0 ? 1 : 0;
  sc.arith = Run_Fast_BM_Calculation == 0 ? 1 : 0;
  gpu_check(cudaMemset(H.failed, 0, H.failed_n * sizeof(int32_t)), "reset failed nodes");
  cgb_check(cgb_bm_run_dev(H.secp, H.gamma, 1, &sc, H.units, Time_Blocks, H.input,
                           (int64_t)H.input_n, H.speeds, rows, H.failed, H.conv, H.stats, H.work,
                           nullptr),
            "BM solver");
  split_conv_kernel<<<Time_Blocks, 256>>>(H.units, Time_Blocks, H.conv, H.stats, H.conv_time,
                                          H.conv_steps, H.conv_loops, H.blk_time, H.blk_steps,
                                          H.blk_loops, H.failed_blocks);
  gpu_check(cudaGetLastError(), "split_conv_kernel");
  gpu_check(cudaDeviceSynchronize(), "BM solver");
  std::vector<cgb_unit_stats> sts(Time_Blocks);
  gpu_check(cudaMemcpy(sts.data(), H.stats, sts.size() * sizeof(cgb_unit_stats),
                       cudaMemcpyDeviceToHost),
            "read stats");
  for (const auto& s : sts)
    if (s.status != 0)
      throw std::runtime_error("cochlea_gb300: a block stopped: its time step collapsed");
}

extern "C" void calculateBoundariesForNonGeneratedInput(int, int, int, float, float, float,
                                                        float, float, int, dim3) {
  // folded into BMOHCNewKernel, which sets the per-block tolerances itself
}

// ---------------------------------------------------------------- IHC / lambda
extern "C" void IHCNewKernel(double* IHC_Damage_Factor, float Nerves_Clusters[3 * LAMBDA_COUNT],
                             double* dc_filter, int order_of_dc_filter, double* ac_b_filter,
                             double* ac_a_filter, bool is_ac_iir_filter, int order_of_ac_filter,
                             int cochlea_sections, int time_blocks, double, float*, int,
                             int calcTime, int, int allocateTime, int intervalTimeNodes, int,
                             int lambda_offset, float Lambda_SAT, float eta_AC, float eta_DC, bool,
                             bool, bool, bool, bool, bool asMemoryHandlingOnly,
                             float scaleBMVelocityForLambdaCalculation, bool CalculateJNDOnGPU,
                             int maxJNDIntervals, int, int Decouple_Filter, int, Log&) {
  if (cochlea_sections != 256)
    throw std::runtime_error("cochlea_gb300: 256 cochlear sections are built");
  if (is_ac_iir_filter && (!ac_a_filter || order_of_ac_filter < 1 || order_of_ac_filter > 64))
    throw std::runtime_error("cochlea_gb300: IIR AC filter needs 1..64 a/b coefficients");
  if (lambda_offset != 0)
    throw std::runtime_error("cochlea_gb300: lambda_offset must be 0");
  ensure(H.lam, H.lam_n, (size_t)LAMBDA_COUNT * allocateTime * 256, "lambda buffer");
  if (asMemoryHandlingOnly) return;
  H.ac_taps.assign(order_of_ac_filter, 0.0f);
  for (int i = 0; i < order_of_ac_filter; ++i) H.ac_taps[i] = (float)ac_b_filter[i];
  H.ac_iir = is_ac_iir_filter;
  H.ac_a_taps.assign(is_ac_iir_filter ? order_of_ac_filter : 0, 0.0f);
  for (int i = 0; is_ac_iir_filter && i < order_of_ac_filter; ++i)
    H.ac_a_taps[i] = (float)ac_a_filter[i];
  H.dc_taps.assign(order_of_dc_filter, 0.0f);
  for (int i = 0; i < order_of_dc_filter; ++i) H.dc_taps[i] = (float)dc_filter[i];
  std::vector<float> dmg(256);
  for (int i = 0; i < 256; ++i) dmg[i] = (float)IHC_Damage_Factor[i];
  ensure(H.dmg, H.dmg_n, (size_t)256, "IHC damage");
  gpu_check(cudaMemcpy(H.dmg, dmg.data(), 256 * sizeof(float), cudaMemcpyHostToDevice),
            "upload IHC damage");
  H.ihc_prm.scale = scaleBMVelocityForLambdaCalculation;
  H.ihc_prm.eta_ac = eta_AC;
  H.ihc_prm.eta_dc = eta_DC;
  H.ihc_prm.lambda_sat = Lambda_SAT;
  for (int j = 0; j < 3; ++j) {
    H.ihc_prm.spont[j] = Nerves_Clusters[j];
    H.W[j] = Nerves_Clusters[2 * LAMBDA_COUNT + j];
  }
  H.calc_time = calcTime;
  H.interval_nodes = intervalTimeNodes;
  H.time_blocks = time_blocks;
  H.decouple = Decouple_Filter;
  H.lambda_offset = lambda_offset;
  ensure(H.status, H.status_n, (size_t)4, "status");
  if (CalculateJNDOnGPU) {
    const size_t mean = (size_t)maxJNDIntervals * LAMBDA_COUNT * 256;
    ensure(H.mean_rate, H.mean_rate_n, mean, "mean rate");
    ensure(H.mean_rate_f, H.mean_rate_f_n, mean, "mean rate");
  }
  H.ihc_ready = true;
}

extern "C" void RunIHCKernel(JNDFloat* host_backup, int, int save_lambda, int backup_stage, int,
                             Log&) {
  if (!H.ihc_ready) throw std::runtime_error("cochlea_gb300: RunIHCKernel before IHCNewKernel");
  if (!H.d_aihc) throw std::runtime_error("cochlea_gb300: RunIHCKernel before loadAihc");
  // debug stages (CudaUnifiedCalcIHC, src/cochlea.cu:3431-3506): 9 AC, 10 DC,
  // 11 and 12 dS, 13 and 14 IHC, each copied to host_backup
  const bool want_ihc = backup_stage == 13 || backup_stage == 14;
  const bool want_stage = backup_stage >= 9 && backup_stage <= 12;
  const int64_t v_rows = (int64_t)(H.speeds_n / 256);
  cgb_ihc_frame fr{};
  fr.v_row0 = 0;
  fr.lam_row0 = 0;
  fr.rows = (int32_t)std::min<int64_t>(v_rows, H.calc_time);
  fr.lam_rows = H.interval_nodes * H.time_blocks;
  fr.seg = H.decouple > 0 ? H.interval_nodes * H.decouple : H.calc_time;
  fr.frdp = H.interval_nodes * H.time_blocks;
  fr.total = H.calc_time;
  fr.ihc_profile = 0;
  if (fr.lam_rows > fr.rows)
    throw std::runtime_error("cochlea_gb300: lambda rows exceed the velocity buffer");
  const int64_t need =
      H.ac_iir ? cgb_ihc_lambda_iir_scratch_bytes(&fr, 1, (int)H.ac_taps.size(),
                                                  (int)H.dc_taps.size())
               : cgb_ihc_lambda_scratch_bytes(1, (int)H.ac_taps.size(), (int)H.dc_taps.size());
  if (need < 0) throw std::runtime_error("cochlea_gb300: bad IIR filter");
  ensure(H.scratch, H.scratch_n, (size_t)need, "IHC scratch");
  float* ihc = nullptr;
  float* stage_buf = nullptr;
  if (want_ihc || want_stage) {
    ensure(H.buffer1, H.buffer1_n, (size_t)H.calc_time * 256, "IHC stage buffer");
    gpu_check(cudaMemset(H.buffer1, 0, (size_t)H.calc_time * 256 * sizeof(float)),
              "clear stage buffer");
    (want_ihc ? ihc : stage_buf) = H.buffer1;
  }
  gpu_check(cudaMemset(H.status, 0, sizeof(int32_t)), "reset status");
  if (H.ac_iir) {
    ensure(H.ac_buf, H.ac_buf_n, (size_t)v_rows * 256, "AC buffer");
    const int rc =
        want_stage
            ? cgb_ihc_lambda_iir_stage_dev(H.speeds, v_rows, &fr, 1, H.ac_taps.data(),
                                           H.ac_a_taps.data(), (int)H.ac_taps.size(),
                                           H.dc_taps.data(), (int)H.dc_taps.size(), &H.ihc_prm,
                                           H.dmg, 1, H.d_aihc, H.lam, H.calc_time, ihc,
                                           H.ac_buf, backup_stage, stage_buf, H.scratch,
                                           (int64_t)H.scratch_n, H.status, nullptr)
            : cgb_ihc_lambda_iir_dev(H.speeds, v_rows, &fr, 1, H.ac_taps.data(),
                                     H.ac_a_taps.data(), (int)H.ac_taps.size(),
                                     H.dc_taps.data(), (int)H.dc_taps.size(), &H.ihc_prm, H.dmg,
                                     1, H.d_aihc, H.lam, H.calc_time, ihc, H.ac_buf, H.scratch,
                                     (int64_t)H.scratch_n, H.status, nullptr);
    cgb_check(rc, "IHC/lambda (IIR AC)");
  } else {
    const int rc =
        want_stage
            ? cgb_ihc_lambda_stage_dev(H.speeds, v_rows, &fr, 1, H.ac_taps.data(),
                                       (int)H.ac_taps.size(), H.dc_taps.data(),
                                       (int)H.dc_taps.size(), &H.ihc_prm, H.dmg, 1, H.d_aihc,
                                       H.lam, H.calc_time, ihc, backup_stage, stage_buf,
                                       H.scratch, (int64_t)H.scratch_n, H.status, nullptr)
            : cgb_ihc_lambda_dev(H.speeds, v_rows, &fr, 1, H.ac_taps.data(),
                                 (int)H.ac_taps.size(), H.dc_taps.data(), (int)H.dc_taps.size(),
                                 &H.ihc_prm, H.dmg, 1, H.d_aihc, H.lam, H.calc_time, ihc,
                                 H.scratch, (int64_t)H.scratch_n, H.status, nullptr);
    cgb_check(rc, "IHC/lambda");
  }
  gpu_check(cudaDeviceSynchronize(), "IHC/lambda");
  int32_t status = 0;
  gpu_check(cudaMemcpy(&status, H.status, sizeof(int32_t), cudaMemcpyDeviceToHost), "status");
  if (status) throw std::runtime_error("cochlea_gb300: IHC staging copy timed out");
  if ((want_ihc || want_stage) && host_backup)
    gpu_check(cudaMemcpy(host_backup, H.buffer1, (size_t)H.calc_time * 256 * sizeof(float),
                         cudaMemcpyDeviceToHost),
              "IHC stage backup");
  if (save_lambda && !want_ihc && !want_stage) {
    const size_t n = (size_t)LAMBDA_COUNT * H.calc_time * 256;
    ensure(H.buffer1, H.buffer1_n, n, "lambda buffer");
    gpu_check(cudaMemcpy(H.buffer1, H.lam, n * sizeof(float), cudaMemcpyDeviceToDevice),
              "save lambda");
  }
}

extern "C" void IHCKernel_Free() {
  release(H.lam, H.lam_n);
  release(H.ac_buf, H.ac_buf_n);
  release(H.dmg, H.dmg_n);
  release(H.scratch, H.scratch_n);
  release(H.status, H.status_n);
  release(H.mean_rate, H.mean_rate_n);
  release(H.mean_rate_f, H.mean_rate_f_n);
  release(H.nihc, H.nihc_n);
  release(H.dA, H.dA_n);
  release(H.ref_of, H.ref_of_n);
  release(H.F, H.F_n);
  release(H.d_aihc, H.d_aihc_n);
  H.aihc_loaded = false;
  H.ihc_ready = false;
}

// ---------------------------------------------------------------- input generation
extern "C" void InputProfilesArrayInitialization(int maxJNDIntervals, int wn_length,
                                                 int signal_length, int signal_mode, int) {
  ensure(H.d_prof, H.d_prof_n, (size_t)std::max(maxJNDIntervals, 1), "profiles");
  if (wn_length > 0) ensure(H.wn, H.wn_n, (size_t)wn_length, "noise buffer");
  if (signal_mode && signal_length > 0) ensure(H.sig, H.sig_n, (size_t)signal_length, "signal");
}
extern "C" void InputProfilesArrayTermination() {
  release(H.d_prof, H.d_prof_n);
  release(H.wn, H.wn_n);
  release(H.sig, H.sig_n);
  H.profiles.clear();
}
extern "C" void uploadProfiles(device_jnd_params* profiles, int numOfProfiles,
                               bool profilesLoaded) {
  if (profilesLoaded) return;
  H.profiles.assign(profiles, profiles + numOfProfiles);
  std::vector<cgb_profile> p(numOfProfiles);
  for (int i = 0; i < numOfProfiles; ++i)
    p[i] = cgb_profile{profiles[i].dA, profiles[i].Wn, profiles[i].frequency};
  ensure(H.d_prof, H.d_prof_n, (size_t)std::max(numOfProfiles, 1), "profiles");
  gpu_check(cudaMemcpy(H.d_prof, p.data(), p.size() * sizeof(cgb_profile),
                       cudaMemcpyHostToDevice),
            "upload profiles");
}
extern "C" void setupToleranceProfile(device_jnd_params* profiles, bool, float Max_M1,
                                      float Max_Tol, int Relative_Error_Parameters,
                                      float M1_SP_Fix_Factor, float Tolerance_Fix_Factor,
                                      int Blocks_Per_Interval, int from_profile_index,
                                      int calculatedProfiles) {
  // src/cochlea.cu:4256-4287
  H.tol_mtt.assign((size_t)Blocks_Per_Interval * calculatedProfiles, Max_Tol);
  H.tol_mmspt.assign((size_t)Blocks_Per_Interval * calculatedProfiles, Max_M1);
  for (int i = 0; i < calculatedProfiles; ++i) {
    float m1f = 1.0f, tf = 1.0f;
    if (Relative_Error_Parameters > 0) {
      const float db = (float)profiles[from_profile_index + i].dBSPLSignal;
      m1f = powf(10.0f, M1_SP_Fix_Factor * db);
      tf = powf(10.0f, Tolerance_Fix_Factor * db);
    }
    for (int j = 0; j < Blocks_Per_Interval; ++j) {
      H.tol_mmspt[(size_t)Blocks_Per_Interval * i + j] = Max_M1 * m1f;
      H.tol_mtt[(size_t)Blocks_Per_Interval * i + j] = Max_Tol * tf;
    }
  }
}

extern "C" void generateInputFromProfile(
    device_jnd_params* profiles, float* WN, int wn_length, float* Signal, int signal_length,
    int signal_mode, int Normalize_Sigma_Type, int Normalize_Sigma_Type_Signal,
    double Normalize_Noise_Energy_To_Given_Interval, double Remove_Generated_Noise_DC,
    int start_dc_expected, int end_dc_expected, int start_dc_normalized, int end_dc_normalized,
    int numOfProfiles, bool profilesLoaded, int from_profile_index, int calculatedProfiles,
    int, int IntervalLength, int JND_Interval_Head, int, float Fs, int Show_Generated_Input,
    float* target_input, bool, bool is_first_time_for_parameters_set, float Max_M1,
    float Max_Tol, int Relative_Error_Parameters, float M1_SP_Fix_Factor,
    float Tolerance_Fix_Factor, int Blocks_Per_Interval, int, float* fir_transfer_function,
    int fir_len, float* iir_transfer_function, int iir_len, Log&) {
  const bool fir_on = fir_len > 1 || (fir_len > 0 && fir_transfer_function[0] != 1);
  const bool iir_on = iir_len > 1 || (iir_len > 0 && iir_transfer_function[0] != 1);
  uploadProfiles(profiles, numOfProfiles, profilesLoaded);
  if (end_dc_expected == 0) end_dc_expected = IntervalLength;
  if (end_dc_normalized == 0) end_dc_normalized = IntervalLength;
  if (wn_length < IntervalLength || (signal_mode && signal_length < IntervalLength))
    throw std::runtime_error("cochlea_gb300: noise/signal shorter than one interval");
  ensure(H.wn, H.wn_n, (size_t)wn_length, "noise buffer");
  gpu_check(cudaMemcpy(H.wn, WN, (size_t)wn_length * sizeof(float), cudaMemcpyHostToDevice),
            "upload noise");
  if (signal_mode) {
    ensure(H.sig, H.sig_n, (size_t)signal_length, "signal buffer");
    gpu_check(cudaMemcpy(H.sig, Signal, (size_t)signal_length * sizeof(float),
                         cudaMemcpyHostToDevice),
              "upload signal");
  }
  if (is_first_time_for_parameters_set) {
    cgb_check(cgb_noise_normalization(WN, Normalize_Sigma_Type,
                                      Normalize_Noise_Energy_To_Given_Interval,
                                      Remove_Generated_Noise_DC, start_dc_expected,
                                      end_dc_expected, start_dc_normalized, end_dc_normalized,
                                      Fs, &H.wn_dc, &H.wn_norm),
              "noise normalisation");
    cgb_check(cgb_noise_normalization(signal_mode ? Signal : nullptr, Normalize_Sigma_Type_Signal,
                                      Normalize_Noise_Energy_To_Given_Interval,
                                      Remove_Generated_Noise_DC, start_dc_expected,
                                      end_dc_expected, start_dc_normalized, end_dc_normalized,
                                      Fs, &H.sig_dc, &H.sig_norm),
              "signal normalisation");
  }
  setupToleranceProfile(profiles, is_first_time_for_parameters_set, Max_M1, Max_Tol,
                        Relative_Error_Parameters, M1_SP_Fix_Factor, Tolerance_Fix_Factor,
                        Blocks_Per_Interval, from_profile_index, calculatedProfiles);
  if ((size_t)calculatedProfiles * IntervalLength + 2 > H.input_n)
    throw std::runtime_error("cochlea_gb300: generated input exceeds the input buffer");
  cgb_check(cgb_input_gen_dev(H.d_prof + from_profile_index, calculatedProfiles, H.wn, H.sig,
                              signal_mode, IntervalLength, JND_Interval_Head, Fs, H.wn_dc,
                              H.wn_norm, H.sig_dc, H.sig_norm, H.input, nullptr),
            "input generation");
  if (fir_on || iir_on) {
    // the reference runs the FIR stage whenever either function is active
    // (src/cochlea.cu:4454-4503); the taps live in temporary device buffers
    float* d_fir = nullptr;
    float* d_iir = nullptr;
    float* d_aux = nullptr;
    const size_t n = (size_t)calculatedProfiles * IntervalLength;
    gpu_check(cudaMalloc(&d_fir, std::max(fir_len, 1) * sizeof(float)), "hearing aid taps");
    gpu_check(cudaMalloc(&d_iir, std::max(iir_len, 1) * sizeof(float)), "hearing aid taps");
    gpu_check(cudaMalloc(&d_aux, n * sizeof(float)), "hearing aid buffer");
    if (fir_len > 0)
      gpu_check(cudaMemcpy(d_fir, fir_transfer_function, fir_len * sizeof(float),
                           cudaMemcpyHostToDevice),
                "upload hearing aid FIR");
    if (iir_on)
      gpu_check(cudaMemcpy(d_iir, iir_transfer_function, iir_len * sizeof(float),
                           cudaMemcpyHostToDevice),
                "upload hearing aid IIR");
    const int rc = cgb_hearing_aid_dev(H.input, calculatedProfiles, IntervalLength, d_fir,
                                       fir_len, d_iir, iir_on ? iir_len : 0, d_aux, nullptr);
    gpu_check(cudaDeviceSynchronize(), "hearing aid");
    cudaFree(d_fir);
    cudaFree(d_iir);
    cudaFree(d_aux);
    cgb_check(rc, "hearing aid");
  }
  gpu_check(cudaDeviceSynchronize(), "input generation");
  if (Show_Generated_Input & 1 && target_input)
    gpu_check(cudaMemcpy(target_input, H.input,
                         (size_t)calculatedProfiles * IntervalLength * sizeof(float),
                         cudaMemcpyDeviceToHost),
              "copy generated input");
}

// ---------------------------------------------------------------- JND
extern "C" void CudaCalculateJND(
    bool calculate_ai, bool calculate_rms, int, int fisher_size, double, double Fs, double,
    double* nIHC, int*, int, int* JND_Refrence_Intervals, int numOFJNDReferences,
    int handeledIntervalsJND, int JNDIntervalsFull, int JNDIntervals, int JNDIntervalHeadNodes,
    int overlapNodes, int JNDIntervalNodes, int lengthOffset, int* JND_Serial_Intervals_Positions,
    int* JND_Interval_To_Reference, JNDFloat* F_RA, JNDFloat* FisherAISum, int,
    int calculatedMatrixSize, double JND_Delta_Alpha_Length_Factor, int, int, bool calcdA, bool,
    int backup_stage, Log&) {
  if (!H.lam) throw std::runtime_error("cochlea_gb300: CudaCalculateJND before IHCNewKernel");
  // backup_stage 1-6 are the JND's debug stages (into getCudaBuffer); the
  // reference's JND kernel writes nothing for the others (8 is JND_Lambda,
  // read from the lambda buffer; 9-14 belong to RunIHCKernel)
  // reference interval of each interval of this chunk (src/cochlea.cu:3818-3840)
  std::vector<int32_t> ref(JNDIntervals);
  for (int i = 0; i < JNDIntervals; ++i) {
    const int g = i + handeledIntervalsJND;
    bool is_ref = false;
    for (int k = 0; k < numOFJNDReferences; ++k) is_ref |= JND_Refrence_Intervals[k] == g;
    const int gr = is_ref ? g : JND_Interval_To_Reference[JND_Serial_Intervals_Positions[g]];
    ref[i] = gr - handeledIntervalsJND;
    if (ref[i] < 0 || ref[i] >= JNDIntervals)
      throw std::runtime_error("cochlea_gb300: a JND reference interval lies outside this chunk");
  }
  std::vector<double> dA(JNDIntervals);
  ensure(H.dA, H.dA_n, (size_t)JNDIntervals, "dA");
  if (calcdA) {
    calc_dA_kernel<<<(JNDIntervals + 127) / 128, 128>>>(H.input, H.dA, JNDIntervals,
                                                         JNDIntervalNodes, JNDIntervalHeadNodes,
                                                         lengthOffset, overlapNodes);
    gpu_check(cudaGetLastError(), "dA kernel");
  } else {
    for (int i = 0; i < JNDIntervals; ++i)
      dA[i] = H.profiles.at((size_t)(i + handeledIntervalsJND)).dA;
    gpu_check(cudaMemcpy(H.dA, dA.data(), dA.size() * sizeof(double), cudaMemcpyHostToDevice),
              "upload dA");
  }
  ensure(H.ref_of, H.ref_of_n, (size_t)JNDIntervals, "reference map");
  gpu_check(cudaMemcpy(H.ref_of, ref.data(), ref.size() * sizeof(int32_t),
                       cudaMemcpyHostToDevice),
            "upload reference map");
  ensure(H.nihc, H.nihc_n, (size_t)256, "nIHC");
  gpu_check(cudaMemcpy(H.nihc, nIHC, 256 * sizeof(double), cudaMemcpyHostToDevice),
            "upload nIHC");
  ensure(H.F, H.F_n, (size_t)6 * JNDIntervals, "Fisher sums");
  const size_t mean = (size_t)LAMBDA_COUNT * JNDIntervals * 256;
  ensure(H.mean_rate, H.mean_rate_n, mean, "mean rate");
  ensure(H.mean_rate_f, H.mean_rate_f_n, mean, "mean rate");
  const int64_t plane_rows = calculatedMatrixSize / 256;
  cgb_check(cgb_jnd_dev(H.lam, plane_rows, JNDIntervals, JNDIntervalNodes, JNDIntervalHeadNodes,
                        lengthOffset, H.dA, H.ref_of, H.nihc, H.W, Fs,
                        JND_Delta_Alpha_Length_Factor, H.F, H.F + 3 * JNDIntervals,
                        H.mean_rate, nullptr),
            "JND");
  to_float_kernel<<<256, 256>>>(H.mean_rate, H.mean_rate_f, (int64_t)mean);
  gpu_check(cudaGetLastError(), "mean-rate conversion");
  if (backup_stage >= 1 && backup_stage <= 6) {
    const size_t need = (backup_stage == 3 || backup_stage == 4)
                            ? (size_t)LAMBDA_COUNT * plane_rows * 256
                            : (backup_stage == 1 ? (size_t)LAMBDA_COUNT * JNDIntervals : mean);
    ensure(H.buffer1, H.buffer1_n, need, "JND stage buffer");
    if (backup_stage == 3 || backup_stage == 4)
      gpu_check(cudaMemset(H.buffer1, 0, need * sizeof(float)), "clear JND stage buffer");
    const double T = JND_Delta_Alpha_Length_Factor / Fs;
    jnd_stage_kernel<<<dim3((unsigned)JNDIntervals, LAMBDA_COUNT), 256>>>(
        backup_stage, H.lam, (int64_t)plane_rows * 256, H.mean_rate, H.dA, H.ref_of, H.nihc,
        JNDIntervals, JNDIntervalNodes, JNDIntervalHeadNodes, lengthOffset, Fs, T, H.buffer1);
    gpu_check(cudaGetLastError(), "JND stage kernel");
  }
  std::vector<double> Fh((size_t)6 * JNDIntervals);
  gpu_check(cudaMemcpy(Fh.data(), H.F, Fh.size() * sizeof(double), cudaMemcpyDeviceToHost),
            "read Fisher sums");
  for (int j = 0; j < LAMBDA_COUNT; ++j)
    for (int i = 0; i < JNDIntervals; ++i) {
      const size_t dst = (size_t)j * JNDIntervalsFull + i + handeledIntervalsJND;
      if ((int)dst >= fisher_size) continue;
      if (calculate_rms) F_RA[dst] = (JNDFloat)Fh[(size_t)j * JNDIntervals + i];
      if (calculate_ai) FisherAISum[dst] = (JNDFloat)Fh[(size_t)(3 + j) * JNDIntervals + i];
    }
}
