// Test infrastructure: a launcher for the REFERENCE's own CUDA kernels.
//
// oracle/build_ref_gpu.sh compiles the reference's device code
// (src/cochlea.cu with include/cochlea.cuh, unmodified) into
// oracle/_ref/cochlea_ref.cubin for sm_103a.  This file is our own host side:
// it loads that cubin through the CUDA driver API, fills the reference's
// __constant__ symbols and launch arguments the way the reference's host
// functions do (each step cites the lines it restates), launches the
// reference's kernels and copies their results back.  It is the parity reference
// for the product's reference-arithmetic BM mode and reports the reference's
// FP32 results for the error tables; nothing in the product links or loads it.
//
// Everything is synchronous and uses the device's primary context (the one the
// CUDA runtime, and therefore torch, uses).

#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;
CUmodule g_mod = nullptr;
float g_bm_ms = 0.0f;  // device time of the last BM launch (CUDA events)
CUcontext g_ctx = nullptr;

int fail(const std::string& m) {
  g_err = m;
  return 1;
}

#define RG_TRY(call, what)                                                      \
  do {                                                                          \
    CUresult rc_ = (call);                                                      \
    if (rc_ != CUDA_SUCCESS) {                                                  \
      const char* s_ = nullptr;                                                 \
      cuGetErrorString(rc_, &s_);                                               \
      return fail(std::string(what) + ": " + (s_ ? s_ : "CUDA driver error"));  \
    }                                                                           \
  } while (0)

// Finds a kernel of the module by the start of its mangled name.
CUfunction find_fn(const std::string& prefix) {
  unsigned n = 0;
  if (cuModuleGetFunctionCount(&n, g_mod) != CUDA_SUCCESS) return nullptr;
  std::vector<CUfunction> fns(n);
  if (cuModuleEnumerateFunctions(fns.data(), n, g_mod) != CUDA_SUCCESS) return nullptr;
  for (CUfunction f : fns) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name &&
        std::strncmp(name, prefix.c_str(), prefix.size()) == 0)
      return f;
  }
  return nullptr;
}

std::string mangled(const char* name) {
  return "_Z" + std::to_string(std::strlen(name)) + name;
}

// A zero-filled device buffer freed on scope exit.
struct DBuf {
  CUdeviceptr p = 0;
  size_t bytes = 0;
  ~DBuf() {
    if (p) cuMemFree(p);
  }
  int alloc(size_t n) {
    bytes = n ? n : 16;
    if (cuMemAlloc(&p, bytes) != CUDA_SUCCESS) return fail("cuMemAlloc");
    if (cuMemsetD8(p, 0, bytes) != CUDA_SUCCESS) return fail("cuMemsetD8");
    return 0;
  }
  int up(const void* h, size_t n) {
    if (n > bytes) return fail("upload larger than buffer");
    return cuMemcpyHtoD(p, h, n) == CUDA_SUCCESS ? 0 : fail("cuMemcpyHtoD");
  }
  int down(void* h, size_t n) const {
    if (n > bytes) return fail("download larger than buffer");
    return cuMemcpyDtoH(h, p, n) == CUDA_SUCCESS ? 0 : fail("cuMemcpyDtoH");
  }
};

int set_symbol(const char* name, const void* h, size_t n) {
  CUdeviceptr d = 0;
  size_t bytes = 0;
  RG_TRY(cuModuleGetGlobal(&d, &bytes, g_mod, name), std::string("symbol ") + name);
  if (n > bytes) return fail(std::string("symbol ") + name + " is smaller than its data");
  RG_TRY(cuMemcpyHtoD(d, h, n), std::string("upload ") + name);
  return 0;
}

constexpr int kSections = 256;
constexpr int kMaxBlocks = 65536;  // MAX_NUMBER_OF_BLOCKS, include/const.h:363

}  // namespace

extern "C" {

// The BMOHCNewKernel arguments that reach the kernels (src/cochlea.cu:990-1042),
// as CSolver::Run_Cuda passes them (src/solver.cpp:629-659).
typedef struct {
  float w_ohc, time_step, time_step_out, delta_x, alpha_r;
  int enable_psi, enable_OW;
  float Ts, alpha_l, alpha_s, Gme, a0, a1, a2, sigma_ow, eta_1, eta_2;
  int Time_Blocks, samplesBufferLengthP1, overlap_nodes_for_block;
  long long overlapTimeMicroSec;
  int show_transient;
  float cuda_max_time_step, cuda_min_time_step;
  int Decouple_Filter;
  float Max_M1_SP_Error_Parameter, Max_Tolerance_Parameter;
  int Relative_Error_Parameters;
  float M1_SP_Fix_Factor, Tolerance_Fix_Factor, SPLREfVal;
  int JACOBBY_Loops_Fast, JACOBBY_Loops_Slow, Cuda_Outern_Loops;
} refgpu_bm_params;

const char* refgpu_last_error(void) { return g_err.c_str(); }

// Device time in ms of the last refgpu_bm_run launch, taken by CUDA events
// recorded on the launch stream on either side of the kernel.
float refgpu_last_bm_ms(void) { return g_bm_ms; }

// Loads the reference cubin into the primary context of device 0.
int refgpu_load(const char* cubin_path) {
  if (g_mod) return 0;
  RG_TRY(cuInit(0), "cuInit");
  CUdevice dev;
  RG_TRY(cuDeviceGet(&dev, 0), "cuDeviceGet");
  RG_TRY(cuDevicePrimaryCtxRetain(&g_ctx, dev), "cuDevicePrimaryCtxRetain");
  RG_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
  RG_TRY(cuModuleLoad(&g_mod, cubin_path), std::string("cuModuleLoad ") + cubin_path);
  return 0;
}

// Runs the reference's BM kernel `variant` over one Run_Cuda parameter set:
//   variant 0  : BMOHC_NEW_kernel (Run_Fast_BM_Calculation = 0, the default;
//                include/cochlea.cuh:3486-4324, dispatched at src/cochlea.cu:2298-2330)
//   variant 17 : BMOHC_FAST_Pre_fmaf_No_Constants_kernel_4B_Optimized_triple_aggregations
//                (include/cochlea.cuh:13573-14245, dispatched at src/cochlea.cu:1436-1493)
// sections: gamma, mass, rsM (= 1/m), U, L, R, S, Q, S_ohc, S_tm, R_tm, each
// float[256] as Run_Cuda casts them (src/solver.cpp:357-376).  mtt / mmspt:
// the per-block throw and m1-sp tolerances (setupToleranceProfile,
// src/cochlea.cu:4256-4287), Time_Blocks entries each.  input: the sample
// buffer (input_len >= samplesBufferLengthP1).  Outputs: saved_speeds
// float[out_rows][256], failed_nodes int[out_rows] and failed_blocks
// int[Time_Blocks] (the last two may be null).
int refgpu_bm_run(int variant, const refgpu_bm_params* p, const float* const* sections,
                  const float* mtt, const float* mmspt, const float* input, long long input_len,
                  float* saved_speeds, long long out_rows, int* failed_nodes,
                  int* failed_blocks) {
  if (!g_mod) return fail("refgpu_bm_run: refgpu_load first");
  if (!p || !sections || !mtt || !mmspt || !input || !saved_speeds)
    return fail("refgpu_bm_run: null argument");
  const int TB = p->Time_Blocks;
  if (TB < 1 || TB > kMaxBlocks) return fail("refgpu_bm_run: Time_Blocks out of range");
  if (input_len < p->samplesBufferLengthP1 || out_rows < p->samplesBufferLengthP1)
    return fail("refgpu_bm_run: buffers shorter than samplesBufferLengthP1");
  CUfunction fn = nullptr;
  if (variant == 0)
    fn = find_fn(mangled("BMOHC_NEW_kernel"));
  else if (variant == 17)
    fn = find_fn(mangled("BMOHC_FAST_Pre_fmaf_No_Constants_kernel_4B_Optimized_triple_aggregations"));
  else
    return fail("refgpu_bm_run: variant must be 0 or 17");
  if (!fn) return fail("refgpu_bm_run: kernel not found in the cubin");
  RG_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");

  // Constant packing, src/cochlea.cu:1098-1147.
  float c[64] = {};
  int ci[16] = {};
  long long cl[8] = {};
  c[0] = p->Ts;
  c[1] = static_cast<float>(1.0 / static_cast<double>(p->Ts));
  c[2] = p->alpha_l;
  c[3] = p->alpha_s;
  c[4] = -1.0f * p->alpha_l;
  c[5] = -1.0f * p->alpha_s;
  c[6] = static_cast<float>(static_cast<double>(p->alpha_l) / static_cast<double>(p->alpha_s));
  c[7] = static_cast<float>(1.0 / static_cast<double>(p->sigma_ow));
  c[8] = p->delta_x;
  c[9] = p->delta_x * p->delta_x;
  c[10] = p->a0;
  c[11] = p->a1;
  c[12] = p->a2;
  c[13] = p->eta_1;
  c[14] = p->eta_2;
  c[15] = p->Gme;
  c[16] = p->enable_OW * p->Gme;
  c[17] = (1 - p->enable_OW) * p->Gme;
  c[18] = -p->w_ohc;
  c[19] = p->time_step;
  c[20] = p->time_step_out;
  c[21] = p->cuda_min_time_step;
  c[22] = p->cuda_max_time_step;
  c[23] = p->Max_M1_SP_Error_Parameter;
  c[24] = p->Max_Tolerance_Parameter;
  c[25] = p->alpha_r;
  c[26] = c[8] * c[10];
  c[31] = -p->a1;
  c[32] = -p->a2;
  c[33] = p->SPLREfVal;
  c[34] = 1.0f / p->SPLREfVal;
  c[35] = p->M1_SP_Fix_Factor;
  c[36] = p->Tolerance_Fix_Factor;
  ci[0] = p->Decouple_Filter;
  ci[1] = p->enable_OW;
  ci[2] = p->enable_psi;
  ci[3] = TB;
  ci[4] = p->samplesBufferLengthP1;
  ci[5] = p->overlap_nodes_for_block;
  ci[6] = p->show_transient;
  ci[7] = p->Relative_Error_Parameters;
  ci[8] = (p->samplesBufferLengthP1 - p->overlap_nodes_for_block) / (TB + 1);
  ci[9] = p->JACOBBY_Loops_Fast;
  ci[10] = p->JACOBBY_Loops_Slow;
  ci[11] = p->Cuda_Outern_Loops;
  cl[0] = p->overlapTimeMicroSec;

  // Block partition, src/cochlea.cu:1152-1176.
  std::vector<int> out_idx(kMaxBlocks, 0), end_idx(kMaxBlocks, 0);
  const int D = ci[0], N = ci[8], ov = ci[5];
  for (int b = 0; b < TB; ++b) {
    const int transient_offset = (b > 0 && (D == 0 || (D != 1 && b % D != 0)));
    const int preDecoupled = D > 0 && (D == 1 || ((b + 1) % D == 0)) && b != TB - 1;
    const int postDecoupled = D > 0 && (b % D == 0);
    const int input_sample = b * N;
    out_idx[b] = input_sample + std::max(1 - transient_offset - postDecoupled, 0) * ov;
    const int block_length = N + (1 - preDecoupled) * ov;
    end_idx[b] = input_sample + block_length;
    if (b > 0) out_idx[b] = std::max(out_idx[b], end_idx[b - 1]);
  }
  if (set_symbol("model_constants", c, sizeof(c))) return 1;
  if (set_symbol("model_constants_integers", ci, sizeof(ci))) return 1;
  if (set_symbol("model_constants_longs", cl, sizeof(cl))) return 1;

  // Buffers.  The kernels read input_samples[input_sample + 2] at most up to
  // the block end and write saved_speeds / failure rows below it; both are
  // padded.
  const long long rows = out_rows + 4;
  DBuf d_in, d_out, d_fn, d_fb, d_sec[11], d_mtt, d_mmspt, d_oi, d_ei, d_conv[6];
  if (d_in.alloc((size_t)(input_len + 16) * 4) || d_in.up(input, (size_t)input_len * 4)) return 1;
  if (d_out.alloc((size_t)rows * kSections * 4) || d_fn.alloc((size_t)rows * 4) ||
      d_fb.alloc((size_t)kMaxBlocks * 4))
    return 1;
  for (int i = 0; i < 11; ++i) {
    if (!sections[i]) return fail("refgpu_bm_run: null section vector");
    if (d_sec[i].alloc(kSections * 4) || d_sec[i].up(sections[i], kSections * 4)) return 1;
  }
  if (d_mtt.alloc(kMaxBlocks * 4) || d_mtt.up(mtt, (size_t)TB * 4)) return 1;
  if (d_mmspt.alloc(kMaxBlocks * 4) || d_mmspt.up(mmspt, (size_t)TB * 4)) return 1;
  if (d_oi.alloc(kMaxBlocks * 4) || d_oi.up(out_idx.data(), kMaxBlocks * 4)) return 1;
  if (d_ei.alloc(kMaxBlocks * 4) || d_ei.up(end_idx.data(), kMaxBlocks * 4)) return 1;
  // convergence statistics: per node (0, 2, 4) and per block (1, 3, 5)
  for (int i = 0; i < 6; ++i)
    if (d_conv[i].alloc((size_t)((i & 1) ? kMaxBlocks : rows) * 4)) return 1;

  // Argument order of the dispatch, src/cochlea.cu:2303-2327 / 1442-1490;
  // the kernels take mass, rsM, U, L, R, S, Q, gamma, S_ohc, S_tm, R_tm.
  CUdeviceptr ptrs[25] = {d_in.p,      d_out.p,     d_fn.p,      d_fb.p,      d_sec[1].p,
                          d_sec[2].p,  d_sec[3].p,  d_sec[4].p,  d_sec[5].p,  d_sec[6].p,
                          d_sec[7].p,  d_sec[0].p,  d_sec[8].p,  d_sec[9].p,  d_sec[10].p,
                          d_mtt.p,     d_mmspt.p,   d_oi.p,      d_ei.p,      d_conv[0].p,
                          d_conv[1].p, d_conv[2].p, d_conv[3].p, d_conv[4].p, d_conv[5].p};
  std::vector<void*> args;
  for (auto& q : ptrs) args.push_back(&q);
  float base_time = 0.0f;
  float s_w = p->w_ohc, s_ts = p->time_step, s_tso = p->time_step_out, s_dx = p->delta_x,
        s_ar = p->alpha_r, s_Ts = p->Ts, s_al = p->alpha_l, s_as = p->alpha_s, s_g = p->Gme,
        s_a0 = p->a0, s_a1 = p->a1, s_a2 = p->a2, s_sow = p->sigma_ow, s_e1 = p->eta_1,
        s_e2 = p->eta_2, s_dtmin = p->cuda_min_time_step, s_dtmax = p->cuda_max_time_step;
  int s_psi = p->enable_psi, s_ow = p->enable_OW, s_len = p->samplesBufferLengthP1,
      s_ov = p->overlap_nodes_for_block;
  if (variant == 17) {
    void* extra[] = {&s_w,  &s_ts, &s_tso, &s_dx, &s_ar, &s_psi, &s_ow,    &base_time,
                     &s_Ts, &s_al, &s_as,  &s_g,  &s_a0, &s_a1,  &s_a2,    &s_sow,
                     &s_e1, &s_e2, &s_len, &s_ov, &s_dtmin, &s_dtmax};
    for (void* e : extra) args.push_back(e);
  }
  CUevent ev[2] = {nullptr, nullptr};
  RG_TRY(cuEventCreate(&ev[0], CU_EVENT_DEFAULT), "cuEventCreate");
  RG_TRY(cuEventCreate(&ev[1], CU_EVENT_DEFAULT), "cuEventCreate");
  RG_TRY(cuEventRecord(ev[0], nullptr), "cuEventRecord");
  RG_TRY(cuLaunchKernel(fn, (unsigned)TB, 1, 1, kSections, 1, 1, 0, nullptr, args.data(),
                        nullptr),
         "cuLaunchKernel (reference BM)");
  RG_TRY(cuEventRecord(ev[1], nullptr), "cuEventRecord");
  RG_TRY(cuCtxSynchronize(), "reference BM kernel");
  RG_TRY(cuEventElapsedTime(&g_bm_ms, ev[0], ev[1]), "cuEventElapsedTime");
  cuEventDestroy(ev[0]);
  cuEventDestroy(ev[1]);
  if (d_out.down(saved_speeds, (size_t)out_rows * kSections * 4)) return 1;
  if (failed_nodes && d_fn.down(failed_nodes, (size_t)out_rows * 4)) return 1;
  if (failed_blocks && d_fb.down(failed_blocks, (size_t)TB * 4)) return 1;
  return 0;
}

// The reference's device_params (include/cochlea_common.h:31-49) and
// vectors_sum_linear_coefficents (:50-54), the structs its IHC and lambda
// kernels read from global memory; the layout must be the reference's.
typedef struct {
  int filter_b_start_index, filter_a_start_index, cochlea_sections, calcTime, writeTime;
  int time_blocks, order_of_dc_filter, order_of_ac_filter, lambda_count, time_block;
  int lambda_offset, ovelapNodes, FilterDecoupledMode;
  double Lambda_SAT;
  int intervalTimeNodes;
  float reverseSQRTScaleBMVelocityForLambdaCalculation;
  int Decouple_Filter;
} refgpu_device_params;

typedef struct {
  double A_coefficent, B_coefficent;
  int reverseCoefficents;
} refgpu_sum_coefficients;

// Runs the reference's IHC and lambda stage of one Run_Cuda chunk: the
// unified CudaUnifiedCalcIHC<float> (src/cochlea.cu:3431-3506) on the grid
// RunIHCKernel uses with Decouple_Unified_IHC_Factor = 0, the default
// (src/cochlea.cu:3578-3594, src/params.cpp:195), then CudaCalcLambda
// (src/cochlea.cu:3365-3408) on its setDecoupledRun grid (:3563-3571,
// 3630-3632).  Parameters and constants are packed as IHCNewKernel packs them
// (src/cochlea.cu:2485-2593).  In a FIR run RunIHCKernel first launches the
// IIR kernel as well (:3587-3590); CudaUnifiedCalcIHC overwrites every
// element that kernel writes before reading it, so it is not launched here.
//   v            float[calcTime][256] BM velocity (cuda_saved_speeds)
//   calc_time    rows of the chunk (calcTime; a multiple of 64 in Run_Cuda)
//   interval     block nodes (intervalTimeNodes); time_blocks, decouple as
//                Time_Blocks / Decouple_Filter (time_blocks % decouple == 0)
//   ac, n_ac     AC FIR taps (double), multiplied by `scale` here as
//                IHCNewKernel does; dc, n_dc the DC taps
//   ihc_damage   double[256]; nerves float[9] (spont x3, unused x3, W x3);
//                aihc float[3][256]
// Outputs ihc float[calcTime][256] (written in place of the velocity) and
// lam float[3][calcTime][256] (rows below interval * time_blocks valid).
int refgpu_ihc_lambda(const float* v, int calc_time, int interval, int time_blocks,
                      int decouple, const double* ac, int n_ac, const double* dc, int n_dc,
                      double scale, double eta_ac, double eta_dc, double lambda_sat,
                      const double* ihc_damage, const float* nerves, const float* aihc,
                      float* ihc, float* lam) {
  if (!g_mod) return fail("refgpu_ihc_lambda: refgpu_load first");
  if (!v || !ac || !dc || !ihc_damage || !nerves || !aihc || !ihc || !lam)
    return fail("refgpu_ihc_lambda: null argument");
  if (calc_time < 1 || interval < 1 || time_blocks < 1 || decouple < 0 ||
      (decouple > 0 && time_blocks % decouple) || interval * time_blocks > calc_time)
    return fail("refgpu_ihc_lambda: bad sizes");
  if (n_ac < 1 || n_dc < 1 || n_ac + n_dc + 2 > 1024)
    return fail("refgpu_ihc_lambda: filters exceed DEVICE_MAX_FILTER_ORDER");
  CUfunction f_ihc = find_fn("_Z18CudaUnifiedCalcIHCIfE");
  CUfunction f_lam = find_fn("_Z14CudaCalcLambdaIffE");
  if (!f_ihc || !f_lam) return fail("refgpu_ihc_lambda: kernels not found in the cubin");
  RG_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");

  // device_time_filter: [n_dc, dc..., n_ac, ac * scale...] (src/cochlea.cu:2485-2503)
  std::vector<double> filt(1024, 0.0);
  filt[0] = n_dc;
  for (int i = 0; i < n_dc; ++i) filt[1 + i] = dc[i];
  const int ac_b = n_dc + 1;
  filt[ac_b] = n_ac;
  for (int i = 0; i < n_ac; ++i) filt[ac_b + 1 + i] = scale * ac[i];
  if (set_symbol("device_time_filter", filt.data(), filt.size() * sizeof(double))) return 1;
  if (set_symbol("CUDA_IHC_DAMAGE", ihc_damage, kSections * sizeof(double))) return 1;
  if (set_symbol("CUDA_Nerves_Clusters", nerves, 9 * sizeof(float))) return 1;
  if (set_symbol("model_Aihc", aihc, 3 * kSections * sizeof(float))) return 1;

  // device params and sum coefficients (src/cochlea.cu:2550-2590)
  refgpu_device_params prm[2] = {};
  prm[0].Decouple_Filter = decouple;
  prm[0].cochlea_sections = kSections;
  prm[0].intervalTimeNodes = interval;
  prm[0].time_blocks = time_blocks;
  prm[0].ovelapNodes = 0;
  prm[0].lambda_offset = 0;
  prm[0].order_of_dc_filter = n_dc;
  prm[0].order_of_ac_filter = n_ac;
  prm[0].lambda_count = 3;
  prm[0].time_block = calc_time / time_blocks;
  prm[0].FilterDecoupledMode = decouple > 0;
  prm[0].reverseSQRTScaleBMVelocityForLambdaCalculation = 1.0f / sqrtf((float)scale);
  prm[0].Lambda_SAT = (float)lambda_sat;
  prm[0].calcTime = calc_time;
  prm[0].writeTime = calc_time;
  prm[0].filter_b_start_index = ac_b;
  prm[0].filter_a_start_index = -1;
  prm[1] = prm[0];
  prm[1].filter_b_start_index = 0;
  prm[1].filter_a_start_index = -1;
  refgpu_sum_coefficients coef[2] = {{scale, -1.0, 0}, {eta_ac, eta_dc, 0}};

  const size_t plane = (size_t)calc_time * kSections;
  DBuf d_v, d_lam, d_buf1, d_prm, d_coef;
  if (d_v.alloc(plane * 4) || d_v.up(v, plane * 4)) return 1;
  if (d_lam.alloc(3 * plane * 4) || d_buf1.alloc(3 * plane * 4)) return 1;
  if (d_prm.alloc(sizeof(prm)) || d_prm.up(prm, sizeof(prm))) return 1;
  if (d_coef.alloc(sizeof(coef)) || d_coef.up(coef, sizeof(coef))) return 1;

  CUdeviceptr b2 = d_lam.p, b3 = d_lam.p + plane * 4, b4 = d_lam.p + 2 * plane * 4;
  int backup_stage = 0;
  void* a1[] = {&d_v.p, &b2, &b3, &b4, &d_buf1.p, &d_prm.p, &d_coef.p, &backup_stage};
  // IHC_FILTER_BLOCK x (SECTIONS_PER_IHC_FILTER_BLOCK, THREADS_PER_IHC_FILTER_SECTION)
  RG_TRY(cuLaunchKernel(f_ihc, kSections / 16, 1, 1, 16, 64, 1, 0, nullptr, a1, nullptr),
         "cuLaunchKernel (reference CudaUnifiedCalcIHC)");
  const int dfilter = decouple > 0 ? decouple : time_blocks;
  int save_lambda = 1;
  void* a2[] = {&d_v.p, &d_buf1.p, &d_lam.p, &d_prm.p, &save_lambda};
  RG_TRY(cuLaunchKernel(f_lam, 3 * time_blocks / dfilter, dfilter, 1, kSections, 1, 1, 0, nullptr,
                        a2, nullptr),
         "cuLaunchKernel (reference CudaCalcLambda)");
  RG_TRY(cuCtxSynchronize(), "reference IHC/lambda kernels");
  if (d_v.down(ihc, plane * 4) || d_lam.down(lam, 3 * plane * 4)) return 1;
  return 0;
}

// The reference's device_jnd_params (include/cochlea_common.h:56-66).
typedef struct {
  double dA, recipdA, dBSPLSignal, dBSPLNoise, Wn;
  bool isReference;
  int calculateIndexPosition, referenceIndex;
  double frequency;
} refgpu_jnd_params;

// Runs the reference's GlobalCalculateMeanRate and GlobalCalculateJND
// (src/cochlea.cu:3741-3944) on the grid CudaCalculateJND uses
// (src/cochlea.cu:4009-4010), over every interval of one run
// (handeledIntervalsJND = 0, both the AI and the rate JND, dA given).
//   lam        float[3][plane_rows][256] lambda (cuda_JND_Lambda)
//   n_int      intervals; interval_nodes, head, length: JNDIntervalLength,
//              JNDIntervalHeadNodes, lengthOffset
//   dA         double[n_int]; ref_of int[n_int]: each interval's reference
//              interval (ref_of[i] == i for a reference)
//   nihc       double[256]; W float[3]; Fs; factor (JND_Delta_Alpha_Length_Factor)
// Outputs F_RA and F_AI float[3][n_int] (the references' entries are left 0).
int refgpu_jnd(const float* lam, int plane_rows, int n_int, int interval_nodes, int head,
               int length, const double* dA, const int* ref_of, const double* nihc,
               const float* W, double Fs, double factor, float* F_RA, float* F_AI) {
  if (!g_mod) return fail("refgpu_jnd: refgpu_load first");
  if (!lam || !dA || !ref_of || !nihc || !W || !F_RA || !F_AI)
    return fail("refgpu_jnd: null argument");
  if (n_int < 1 || length < 1 || head < 0 ||
      (long long)(n_int - 1) * interval_nodes + head + length > plane_rows)
    return fail("refgpu_jnd: windows outside the lambda planes");
  CUfunction f_mr = find_fn(mangled("GlobalCalculateMeanRate"));
  CUfunction f_jnd = find_fn(mangled("GlobalCalculateJND"));
  if (!f_mr || !f_jnd) return fail("refgpu_jnd: kernels not found in the cubin");
  RG_TRY(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent");
  float nerves[9] = {};
  for (int j = 0; j < 3; ++j) nerves[6 + j] = W[j];
  if (set_symbol("CUDA_Nerves_Clusters", nerves, sizeof(nerves))) return 1;

  // interval tables as the host JND setup forms them: references, the tested
  // intervals in order, each interval's position among the tested ones and
  // each tested position's reference
  std::vector<refgpu_jnd_params> prm(n_int);
  std::vector<int> refs, calc, serial(n_int, 0), to_ref;
  for (int i = 0; i < n_int; ++i) {
    prm[i] = refgpu_jnd_params{};
    prm[i].dA = dA[i];
    prm[i].recipdA = dA[i] != 0.0 ? 1.0 / dA[i] : 0.0;
    prm[i].isReference = ref_of[i] == i;
    if (ref_of[i] < 0 || ref_of[i] >= n_int) return fail("refgpu_jnd: bad reference index");
    if (ref_of[i] == i) {
      refs.push_back(i);
    } else {
      serial[i] = (int)calc.size();
      calc.push_back(i);
      to_ref.push_back(ref_of[i]);
    }
  }
  if (refs.empty()) refs.push_back(-1);
  if (calc.empty()) {
    calc.push_back(0);
    to_ref.push_back(0);
  }
  const size_t plane = (size_t)plane_rows * kSections;
  DBuf d_prm, d_lam, d_mr, d_buf, d_nihc, d_refs, d_calc, d_serial, d_toref, d_fra, d_fai, d_gp;
  if (d_prm.alloc(prm.size() * sizeof(refgpu_jnd_params)) ||
      d_prm.up(prm.data(), prm.size() * sizeof(refgpu_jnd_params)))
    return 1;
  if (d_lam.alloc(3 * plane * 4) || d_lam.up(lam, 3 * plane * 4)) return 1;
  if (d_mr.alloc((size_t)3 * n_int * kSections * 4) || d_buf.alloc(3 * plane * 4)) return 1;
  if (d_nihc.alloc(kSections * 8) || d_nihc.up(nihc, kSections * 8)) return 1;
  if (d_refs.alloc(refs.size() * 4) || d_refs.up(refs.data(), refs.size() * 4)) return 1;
  if (d_calc.alloc(calc.size() * 4) || d_calc.up(calc.data(), calc.size() * 4)) return 1;
  if (d_serial.alloc(serial.size() * 4) || d_serial.up(serial.data(), serial.size() * 4)) return 1;
  if (d_toref.alloc(to_ref.size() * 4) || d_toref.up(to_ref.data(), to_ref.size() * 4)) return 1;
  if (d_fra.alloc((size_t)3 * n_int * 4) || d_fai.alloc((size_t)3 * n_int * 4)) return 1;
  if (d_gp.alloc(2 * sizeof(refgpu_device_params))) return 1;

  int calc_matrix = (int)plane, write_matrix = (int)plane, overlap = 0;
  int jnd_intervals = n_int, jnd_full = n_int, use_spont = 0;
  void* a1[] = {&d_prm.p, &d_lam.p, &d_mr.p, &length, &calc_matrix, &jnd_intervals,
                &interval_nodes, &head, &overlap, &use_spont};
  RG_TRY(cuLaunchKernel(f_mr, n_int, 3, 1, kSections, 1, 1, 0, nullptr, a1, nullptr),
         "cuLaunchKernel (reference GlobalCalculateMeanRate)");
  bool calc_ai = true, calc_rms = true;
  double scale = 1.0;
  int n_calc = (int)calc.size(), n_refs = refs[0] < 0 ? 0 : (int)refs.size(), handled = 0;
  int is_da_calced = 0, backup_stage = 0;
  void* a2[] = {&calc_ai,   &calc_rms,   &d_prm.p,     &d_lam.p,    &d_mr.p,       &d_buf.p,
                &d_nihc.p,  &Fs,         &scale,       &write_matrix, &calc_matrix, &overlap,
                &head,      &interval_nodes, &length,  &jnd_intervals, &jnd_full,  &d_calc.p,
                &n_calc,    &d_refs.p,   &n_refs,      &handled,    &d_serial.p,   &d_toref.p,
                &d_fra.p,   &d_fai.p,    &factor,      &d_gp.p,     &is_da_calced, &use_spont,
                &backup_stage};
  RG_TRY(cuLaunchKernel(f_jnd, n_int, 3, 1, kSections, 1, 1, 0, nullptr, a2, nullptr),
         "cuLaunchKernel (reference GlobalCalculateJND)");
  RG_TRY(cuCtxSynchronize(), "reference JND kernels");
  if (d_fra.down(F_RA, (size_t)3 * n_int * 4) || d_fai.down(F_AI, (size_t)3 * n_int * 4))
    return 1;
  return 0;
}

}  // extern "C"
