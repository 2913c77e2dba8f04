/*
 * cochlea_gb300.h -- plain C ABI of the GB300-native cochlear solver.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (CGB_OK == 0); the message of the last failure is in cgb_last_error().
 * Functions whose name ends in _dev take DEVICE pointers and a CUDA stream
 * (passed as void*), enqueue work and return without synchronising.  The
 * reference-named drop-in layer (include/cochlea_common.h) is built on top of
 * this ABI.
 *
 * Reference interfaces replaced (YonatanKoral/CochlearModel):
 *   cgb_model_setup        CModel ctor + CSolver::Init_Tri_Matrix
 *                          (src/model.cpp:18-86, src/solver.cpp:155-176)
 *   cgb_block_partition    the per-block start/output/end table built inside
 *                          BMOHCNewKernel (src/cochlea.cu:1148-1176)
 *   cgb_bm_run_dev         the kernel launch of BMOHCNewKernel, variant 17
 *                          (src/cochlea.cu:1436-1493,
 *                           include/cochlea.cuh:13573-14245)
 *   cgb_ihc_lambda_dev     RunIHCKernel: CudaUnifiedCalcIHC + CudaCalcLambda
 *                          (src/cochlea.cu:3573-3644, 3431-3506, 3365-3408)
 *   cgb_jnd_dev            CudaCalculateJND: GlobalCalculateMeanRate +
 *                          GlobalCalculateJND (src/cochlea.cu:3946-4065)
 *   cgb_input_gen_dev      generateInputFromProfile's kernel
 *                          CudaGenerateInputFromProfile (src/cochlea.cu:4070-4103)
 *   cgb_noise_normalization calculateDCANDNornalizationFactor /
 *                          ...PureTone (src/cochlea.cu:4165-4254)
 */
#ifndef COCHLEA_GB300_H
#define COCHLEA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGB_SECTIONS 256
#define CGB_LAMBDA_COUNT 3

enum {
  CGB_OK = 0,
  CGB_ERR_ARG = 1,    /* invalid argument (null pointer, bad size)        */
  CGB_ERR_CUDA = 2,   /* a CUDA runtime call failed                       */
  CGB_ERR_RANGE = 3,  /* a size beyond a documented maximum               */
  CGB_ERR_STATE = 4   /* call out of order (drop-in layer)                */
};

/* One unit of BM work: one time block of one signal, simulated from zero
 * state (reference: one CUDA block of BMOHCNewKernel).  Coordinates are in
 * samples of the unit's frame; the frame's sample 0 sits at input index
 * in_base and at output row out_base (rows of 256 floats). */
typedef struct cgb_unit {
  int64_t in_base;
  int64_t out_base;
  int32_t start;      /* first input sample simulated                     */
  int32_t out_first;  /* first sample whose velocity row is written       */
  int32_t end;        /* one past the last sample simulated               */
  int32_t profile;    /* OHC (gamma) profile row                          */
  float mtt;          /* throw tolerance   (Max_Tolerance)                */
  float mmspt;        /* m1_sp tolerance   (Max_M1_SP_Error)              */
} cgb_unit;

/* Per-unit counters written by the BM kernel. */
typedef struct cgb_unit_stats {
  int64_t substeps;        /* accepted + rejected time steps               */
  int64_t iterations;      /* outer (predictor/corrector) iterations       */
  int64_t sweeps;          /* Jacobi sweeps                                */
  int32_t failed_samples;  /* written samples with a non-converged step    */
  int32_t written_samples;
  int32_t status;          /* 0 ok; 1 stopped: a sample needed more than
                              max_substeps_per_sample steps (dt collapsed) */
  int32_t pad_;
} cgb_unit_stats;

/* Scalars of the BM/OHC step (the float arguments of BMOHCNewKernel). */
typedef struct cgb_bm_scalars {
  float w_ohc, time_step, time_step_out, delta_x, alpha_r, Ts;
  float alpha_l, alpha_s, Gme, a0, a1, a2, sigma_ow, eta_1, eta_2;
  float dt_min, dt_max;
  int32_t jacobi_fast;  /* sweeps on outer iterations >= 2 (JACOBBY_Loops_Fast) */
  int32_t jacobi_slow;  /* sweeps on outer iterations 0-1 (JACOBBY_Loops_Slow)  */
  int32_t max_outer;    /* Cuda_Outern_Loops                                   */
  int32_t red_lanes;    /* reduction tree width; must be 32                    */
  int32_t jacobi_mode;  /* 0: fixed sweeps (reference semantics);
                           2: sweep pairs until max|dp| <= jacobi_tol * max|p|
                              or jacobi_cap sweeps                            */
  int32_t max_substeps_per_sample; /* guard against a collapsed dt (>= 1)       */
  float jacobi_tol;     /* mode 2 stopping tolerance (relative, infinity norm) */
  int32_t jacobi_cap;   /* mode 2 sweep cap per solve (even, >= 2)             */
  int32_t guess_mode;   /* mode 2 first-solve guess of a step: 0 previous
                           pressure, 1 linear extrapolation of the last two,
                           2 extrapolation + the network's correction        */
  int32_t learned_every;/* guess 2: network every n-th step (others: 1)      */
  int32_t controller;   /* step controller: 0 kernel 17 (another iteration
                           while the summed margin sum(|dv| - max(mtt, v dt))
                           is positive; include/cochlea.cuh:14021-14105),
                           1 BMOHC_NEW_kernel, the reference default (while
                           any section fails |dv| <= max(mtt, v dt);
                           include/cochlea.cuh:4080-4120); 1 needs
                           jacobi_mode 0                                   */
  int32_t arith;        /* 0: own floating-point order (double time
                           accumulator), mirrored by the CPU oracle;
                           1: BMOHC_NEW_kernel's operation order (tanhf,
                           __fdividef, float time), needs controller 1    */
} cgb_bm_scalars;

/* Optional inputs of cgb_bm_run_ex_dev. */
typedef struct cgb_bm_extras {
  const void* d_ws_blob;  /* packed network weights (cgb_ws_pack_dev), guess 2 */
  float* d_log;           /* training records float[log_cap][6][256]: Y/m, p,
                             p_prev, v, x, {rho, 0...}; NULL: no logging     */
  int64_t log_cap;
  int32_t log_every;      /* record every n-th step start of each unit       */
  int32_t pad_;
  int32_t* d_log_count;   /* records claimed (may exceed log_cap)            */
  int64_t h_out_bytes;    /* size of h_out in bytes; at least out_rows * 256 * 4
                             when h_out is set (checked before the launch)  */
  float* h_out;           /* host mirror of d_out, or NULL: pinned host memory
                             mapped at the same address on the device, 16-byte
                             aligned, out_rows x 256 floats.  The kernel stores
                             every velocity row there too, as it writes it, so
                             the rows reach the host while the solve runs;
                             rows no unit writes are left as they are. */
} cgb_bm_extras;

/* One frame of the IHC/lambda stage: a run of consecutive velocity rows that
 * the reference filters as one buffer (one Run_Cuda chunk, or one signal of a
 * batch).  FIR look-back at row k of the frame uses
 *   min((k+1) % (k < frdp-1 ? seg : total), taps) taps
 * (DeviceCudaFIRFilter, src/cochlea.cu:2712-2730). */
typedef struct cgb_ihc_frame {
  int64_t v_row0;      /* first velocity row of the frame                     */
  int64_t lam_row0;    /* first row of the frame in each lambda plane         */
  int32_t rows;        /* velocity rows available to the frame                */
  int32_t lam_rows;    /* rows for which IHC and lambda are produced (<= rows) */
  int32_t seg;         /* decoupled interval length: block nodes x Decouple_Filter */
  int32_t frdp;        /* block nodes x Time_Blocks                           */
  int32_t total;       /* calcTime: rows rounded up to 64                      */
  int32_t ihc_profile; /* row of the 10^IHC damage table                      */
} cgb_ihc_frame;

typedef struct cgb_ihc_params {
  float scale;       /* scaleBMVelocityForLambdaCalculation (AC taps are scaled) */
  float eta_ac;      /* IHC AC coupling                                          */
  float eta_dc;      /* IHC DC coupling                                          */
  float lambda_sat;  /* Lambda_SAT                                               */
  float spont[3];    /* spontaneous rates of the high/medium/low fibres          */
  int32_t pad_;
} cgb_ihc_params;

/* One generated input interval (the fields of device_jnd_params the input
 * kernel reads, include/cochlea_common.h:56-66). */
typedef struct cgb_profile {
  double dA;         /* tone amplitude (dyn/cm^2), 0 for a noise-only interval */
  double Wn;         /* noise amplitude                                          */
  double frequency;  /* tone frequency (Hz)                                      */
} cgb_profile;

const char* cgb_last_error(void);
int cgb_abi_version(void);

/* Model vectors.  Outputs (double, 256 each): M, R, S, Q, S_ohc, S_tm, R_tm and
 * the pressure-system diagonals m, l, u.  scal (double[16]): w_ohc, dx,
 * alpha_r, alpha_L, alpha_s, Gme, a0, a1, a2, sigma_ow, eta_1, eta_2, w_ow,
 * Cme, ratio_K, psi0. */
int cgb_model_setup(double* M, double* R, double* S, double* Q, double* S_ohc,
                    double* S_tm, double* R_tm, double* diag_m, double* diag_l,
                    double* diag_u, double* scal);

/* Packs the float section parameters the BM kernel reads:
 * secp = float[8][256]: 1/M, 1/m, R, S, Q, S_ohc, S_tm, R_tm, from the float
 * casts the reference host makes (src/solver.cpp:357-376). */
int cgb_pack_sections(const double* M, const double* diag_m, const double* R,
                      const double* S, const double* Q, const double* S_ohc,
                      const double* S_tm, const double* R_tm, float* secp);

/* Fills the reference block partition for one run of `time_blocks` blocks
 * over a buffer of samples_p1 samples (totalTimeNodesP1). */
int cgb_block_partition(int time_blocks, int64_t samples_p1, int overlap, int decouple,
                        int32_t* start, int32_t* out_first, int32_t* end);

/* BM/OHC solver over n_units units (device pointers).
 *   d_secp   float[8][256]     section parameters (cgb_pack_sections)
 *   d_gamma  float[P][256]     OHC profiles
 *   d_units  cgb_unit[n_units]
 *   d_in     float[in_len]     input samples; each unit reads up to
 *                              in_base+end+1
 *   d_out    float[out_rows][256] velocity rows
 *   d_failed int32[out_rows]   1 where a written sample had a step that hit
 *                              max_outer (may be null)
 *   d_conv   float[out_rows][3] per written sample: mean dt, steps, mean outer
 *                              iterations per step (may be null)
 *   d_stats  cgb_unit_stats[n_units] (may be null)
 *   d_work   int32[1] scratch: the work-queue counter (reset in-stream)
 * Units are taken from a device work queue by a persistent grid of warps. */
int cgb_bm_run_dev(const float* d_secp, const float* d_gamma, int n_profiles,
                   const cgb_bm_scalars* sc, const cgb_unit* d_units, int n_units,
                   const float* d_in, int64_t in_len, float* d_out, int64_t out_rows,
                   int32_t* d_failed, float* d_conv, cgb_unit_stats* d_stats, int32_t* d_work,
                   void* stream);

/* cgb_bm_run_dev with the tolerance-mode extras (jacobi_mode 2): the network
 * weights of guess_mode 2 and the logging of training records.  ex may be
 * NULL.  No counterpart in the reference (it runs fixed sweep counts). */
int cgb_bm_run_ex_dev(const float* d_secp, const float* d_gamma, int n_profiles,
                      const cgb_bm_scalars* sc, const cgb_unit* d_units, int n_units,
                      const float* d_in, int64_t in_len, float* d_out, int64_t out_rows,
                      int32_t* d_failed, float* d_conv, cgb_unit_stats* d_stats,
                      int32_t* d_work, const cgb_bm_extras* ex, void* stream);

/* Learned Jacobi warm start: training and inference of the 4-layer 1-D
 * convolution network (8 -> 64 -> 64 -> 64 -> 1 channels, width 5, BF16
 * weights and activations, FP32 accumulation on the tensor cores).  No
 * counterpart in the reference.
 *   params   float[cgb_ws_param_count()] canonical FP32 parameters:
 *            W1[5][64][8], b1[64], W2[5][64][64], b2[64], W3[5][64][64],
 *            b3[64], W4[5][64], b4[1]   (W[tap][out][in])
 *   blob     packed BF16 forward weights (cgb_ws_blob_bytes(), 16-B aligned)
 *   blobT    transposed weights for the backward pass (cgb_ws_blobT_bytes())
 *   records  float[n][6][256] logged by cgb_bm_run_ex_dev
 *   feat     BF16 [n][280][8] features (section s at row s + 8)
 *   target   float[n][256] (p* - pe) / max|rt|; nr float[n] = max|rt|
 *   hid      BF16 [3][n][256][64] hidden activations (64-channel rows)
 *   dout     BF16 [n][256][8] dL/d(output); dpre BF16 [3][n][256][64]
 *   partial  float[n_parts][cgb_ws_param_count()]; grad float[param_count] */
int cgb_ws_blob_bytes(void);
int cgb_ws_blobT_bytes(void);
int cgb_ws_param_count(void);
int cgb_ws_pack_dev(const float* d_params, float s_out, float rm_scale, void* d_blob,
                    void* d_blobT, void* stream);
int cgb_ws_prepare_dev(const float* d_records, int n, const float* d_rm, float rm_scale,
                       void* d_feat, float* d_target, float* d_nr, double* d_work, void* stream);
int cgb_ws_forward_dev(const void* d_blob, const void* d_feat, int n, void* d_hid, float* d_out,
                       void* stream);
int cgb_ws_loss_dev(const float* d_out, const float* d_target, int n, float s_out, void* d_dout,
                    double* d_loss_part, void* stream);
int cgb_ws_backward_dev(const void* d_blobT, const void* d_dout, const void* d_hid, int n,
                        void* d_dpre, void* stream);
int cgb_ws_wgrad_dev(const void* d_feat, const void* d_hid, const void* d_dpre,
                     const void* d_dout, int n, float* d_partial, int n_parts, float* d_grad,
                     void* stream);
int cgb_ws_adam_dev(float* d_params, const float* d_grad, float* d_m, float* d_v, int step,
                    float lr, float beta1, float beta2, float eps, void* stream);
int cgb_ws_infer_dev(const void* d_blob, const void* d_feat, int n, float* d_out, void* stream);

/* IHC + lambda over n_frames frames (host frame table, device buffers).
 *   d_v      float[v_rows][256]  BM velocity (16-byte aligned)
 *   ac_taps / dc_taps  host float taps (AC taps are multiplied by scale)
 *   d_dmg    float[P][256]       10^IHC damage factors
 *   d_aihc   float[3][256]       A of the three fibre groups
 *   d_lam    float[3][lam_plane_rows][256] output
 *   d_ihc    float[lam_plane_rows][256] IHC output (may be null)
 *   d_scratch  device scratch of cgb_ihc_lambda_scratch_bytes() bytes
 *   d_status int32: bit 0 set if a staged copy did not complete in time
 * Filters of 1..1024 taps. */
int64_t cgb_ihc_lambda_scratch_bytes(int n_frames, int n_ac, int n_dc);
int cgb_ihc_lambda_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                       int n_frames, const float* ac_taps, int n_ac, const float* dc_taps,
                       int n_dc, const cgb_ihc_params* prm, const float* d_dmg,
                       int n_dmg_profiles, const float* d_aihc, float* d_lam,
                       int64_t lam_plane_rows, float* d_ihc, void* d_scratch,
                       int64_t scratch_bytes, int32_t* d_status, void* stream);

/* The two halves of cgb_ihc_lambda_dev, for CUDA-graph capture: the upload
 * call copies the frame table, tile prefix and taps into d_scratch (host to
 * device, not capturable); the launch call, given the same frames and taps,
 * only launches the kernel on the tables already in d_scratch. */
int cgb_ihc_lambda_upload_dev(const cgb_ihc_frame* frames, int n_frames, const float* ac_taps,
                              int n_ac, const float* dc_taps, int n_dc,
                              const cgb_ihc_params* prm, int64_t v_rows, int64_t lam_plane_rows,
                              int n_dmg_profiles, void* d_scratch, int64_t scratch_bytes,
                              void* stream);
int cgb_ihc_lambda_launch_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                              int n_frames, const float* ac_taps, int n_ac, const float* dc_taps,
                              int n_dc, const cgb_ihc_params* prm, const float* d_dmg,
                              int n_dmg_profiles, const float* d_aihc, float* d_lam,
                              int64_t lam_plane_rows, float* d_ihc, void* d_scratch,
                              int64_t scratch_bytes, int32_t* d_status, void* stream);
/* cgb_ihc_lambda_launch_dev with a host mirror of d_lam: h_lam is pinned host
 * memory mapped at the same address on the device (16-byte aligned, the
 * layout of d_lam), h_lam_bytes long, at least 3 * lam_plane_rows * 256 * 4
 * (CGB_ERR_RANGE otherwise).  The kernel stores every lambda value there
 * too, so the three planes reach the host while the stage runs, with no copy
 * after it. */
int cgb_ihc_lambda_launch_mirror_dev(const float* d_v, int64_t v_rows,
                                     const cgb_ihc_frame* frames, int n_frames,
                                     const float* ac_taps, int n_ac, const float* dc_taps,
                                     int n_dc, const cgb_ihc_params* prm, const float* d_dmg,
                                     int n_dmg_profiles, const float* d_aihc, float* d_lam,
                                     int64_t lam_plane_rows, float* d_ihc, void* d_scratch,
                                     int64_t scratch_bytes, int32_t* d_status, float* h_lam,
                                     int64_t h_lam_bytes,
                                     void* stream);

/* IHC + lambda with the AC stage by IIR (the reference's is_ac_iir_filter
 * path, DeviceCudaIIRFilter src/cochlea.cu:2745-2775):
 *   AC[k] = sum_{i<ob} b_i v[k-i] - sum_{1<=j<ob} a_j AC[k-j]
 * with ob the FIR look-back bound, in the reference's arithmetic (float
 * accumulator, each double-tap term added in double and rounded).  b_taps
 * are multiplied by prm->scale; a_taps[0] is not used.  The recursion runs
 * per section along independent segments of each frame, then the fused
 * kernel continues from d_ac.
 *   d_ac     float[v_rows][256] scratch receiving AC (by velocity row)
 *   scratch  cgb_ihc_lambda_iir_scratch_bytes(frames, n_frames, n_iir, n_dc)
 * IIR lengths 1..64. */
int64_t cgb_ihc_lambda_iir_scratch_bytes(const cgb_ihc_frame* frames, int n_frames, int n_iir,
                                         int n_dc);
int cgb_ihc_lambda_iir_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                           int n_frames, const float* b_taps, const float* a_taps, int n_iir,
                           const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
                           const float* d_dmg, int n_dmg_profiles, const float* d_aihc,
                           float* d_lam, int64_t lam_plane_rows, float* d_ihc, float* d_ac,
                           void* d_scratch, int64_t scratch_bytes, int32_t* d_status,
                           void* stream);

/* RunIHCKernel's debug stages (backup_stage 9-12 of CudaUnifiedCalcIHC,
 * src/cochlea.cu:3431-3506): cgb_ihc_lambda_dev and cgb_ihc_lambda_iir_dev
 * that also store one intermediate plane of every lambda row into d_stage,
 * laid out as d_ihc ([lam_plane_rows][256] floats):
 *   stage 9   AC, the AC filter's output
 *   stage 10  DC, the DC filter's output
 *   stage 11, 12  dS = (scale v - AC)^2 (the reference's "dS" and "Shigh"
 *             stages both copy dS)
 * The values are the kernel's own (the AC and dS that feed lambda, the DC
 * of the pre-synaptic sum); lambda and IHC are computed as without a stage.
 * Other stage values, or a null d_stage, return CGB_ERR_ARG. */
int cgb_ihc_lambda_stage_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                             int n_frames, const float* ac_taps, int n_ac, const float* dc_taps,
                             int n_dc, const cgb_ihc_params* prm, const float* d_dmg,
                             int n_dmg_profiles, const float* d_aihc, float* d_lam,
                             int64_t lam_plane_rows, float* d_ihc, int stage, float* d_stage,
                             void* d_scratch, int64_t scratch_bytes, int32_t* d_status,
                             void* stream);
int cgb_ihc_lambda_iir_stage_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                                 int n_frames, const float* b_taps, const float* a_taps,
                                 int n_iir, const float* dc_taps, int n_dc,
                                 const cgb_ihc_params* prm, const float* d_dmg,
                                 int n_dmg_profiles, const float* d_aihc, float* d_lam,
                                 int64_t lam_plane_rows, float* d_ihc, float* d_ac, int stage,
                                 float* d_stage, void* d_scratch, int64_t scratch_bytes,
                                 int32_t* d_status, void* stream);

/* Tiles each IHC/lambda CTA walks in a run (the DC look-back is recomputed
 * once per run): 0 restores the automatic choice (32 or 16 tiles while at
 * least two CTAs per SM remain, else 8); 1-64 forces that run length.  It
 * takes effect at the next upload of the per-call tables (cgb_ihc_lambda_dev,
 * _upload_dev, _noalloc_dev): a launch of tables uploaded earlier keeps the
 * run length they were uploaded with.  Every choice gives the same results
 * bit for bit; the autotuner times them. */
int cgb_ihc_set_run_length(int tiles);

/* Test-only fault injection for the IHC/lambda kernel's bounded staging
 * wait -- no counterpart in the reference.  With skip_first_copy = 1, later
 * launches arm each CTA's first staging mbarrier but issue none of its copies,
 * so the wait runs out after about one second with no copy in flight and the
 * kernel sets bit 1 of *d_status; 0 restores normal launches. */
int cgb_ihc_set_fault_injection(int skip_first_copy);

/* IHC + lambda without any device allocation -- no counterpart in the
 * reference.  For callers that cannot allocate device memory (a host that
 * gives the library only buffers it already owns, a real-time audio thread
 * that must not enter the device allocator or the host heap): the same
 * computation as cgb_ihc_lambda_dev, but the per-call tables live in a fixed
 * 192 KiB __device__ array inside the library instead of caller scratch, and
 * their host-side staging in static arrays (no stack or heap use per call).
 * Limits: at most 4096 frames and n_ac + n_dc <= 2048 taps (CGB_ERR_RANGE
 * beyond).  The array stays resident on every GPU that loads the library
 * until exit and is shared by all calls: call from one host thread at a
 * time, and serialise the calls on one stream (calls whose GPU work
 * overlaps race on the array).  Each call copies its frame table from
 * `frames` with cudaMemcpyAsync on `stream`: a pinned `frames` buffer must
 * stay valid until the stream has run that copy.  The first call on a device
 * looks the array's device address up (cudaGetSymbolAddress) and keeps it
 * for the process (not refreshed after cudaDeviceReset); make that first
 * call before any stream capture. */
int cgb_ihc_lambda_noalloc_dev(const float* d_v, int64_t v_rows, const cgb_ihc_frame* frames,
                               int n_frames, const float* ac_taps, int n_ac,
                               const float* dc_taps, int n_dc, const cgb_ihc_params* prm,
                               const float* d_dmg, int n_dmg_profiles, const float* d_aihc,
                               float* d_lam, int64_t lam_plane_rows, float* d_ihc,
                               int32_t* d_status, void* stream);

/* Input generation: d_out[p*interval_len + n] for n < interval_len,
 *   signal_mode 0: dA cos(2 pi f (n-head)/Fs)/sig_norm + Wn (wn[n]-wn_dc)/wn_norm
 *   signal_mode 1: dA (signal[n]-sig_dc)/sig_norm    + Wn (wn[n]-wn_dc)/wn_norm
 * in double, stored as float; d_wn may be null (no noise term). */
int cgb_input_gen_dev(const cgb_profile* d_prof, int n_prof, const float* d_wn,
                      const float* d_signal, int signal_mode, int interval_len, int head,
                      float Fs, double wn_dc, double wn_norm, double sig_dc, double sig_norm,
                      float* d_out, void* stream);

/* DC and energy normalisation of a noise (or signal) array over the given
 * windows; src == null gives the pure-tone factor sqrt(0.5 * window). */
int cgb_noise_normalization(const float* src, int normalize_type, double normalize_to_interval,
                            double remove_dc, int start_dc, int end_dc, int start_norm,
                            int end_norm, float Fs, double* dc, double* factor);

/* JND Fisher sums per interval and lambda plane (Eq. 17-24).
 *   d_lam   float[3][plane_rows][256]; interval i occupies rows
 *           [i*interval_nodes, (i+1)*interval_nodes), its window starts at +head
 *           and is len rows long
 *   d_dA    double[n_int] tone amplitude of each interval
 *   d_ref_of int32[n_int] the noise-only reference interval of each interval
 *           (ref_of[i] == i marks a reference)
 *   d_nihc  double[256] nerve fibres per section; W: host float[3]
 *   d_F_RA, d_F_AI  double[3][n_int] rate and all-information Fisher sums
 *   d_MR    double[3][n_int][256] mean rates over the window (may be null)
 * Time sums are compensated FP32 (Kahan) over FP32 terms; group and
 * section sums are FP64. */
int cgb_jnd_dev(const float* d_lam, int64_t plane_rows, int n_int, int interval_nodes, int head,
                int len, const double* d_dA, const int32_t* d_ref_of, const double* d_nihc,
                const float* W, double Fs, double delta_alpha_len_factor, double* d_F_RA,
                double* d_F_AI, double* d_MR, void* stream);

/* Hearing-aid shaping of the generated input (the reference's
 * CudaProcessSignalTroughHearingAID / ...IIR, src/cochlea.cu:4105-4150), in
 * place on d_in float[n_prof][interval_len], per interval position n:
 *   aux[n] = sum_{i < min(n, fir_len)} fir_i x[n-i]
 *   out[n] = aux[n] + sum_{1 <= j < min(n+1, iir_len)} iir_j aux[n-j]
 * (iir_len 0: out = aux).  d_fir / d_iir are device taps; d_aux is a
 * scratch of the same size as d_in.  The reference runs this only when a
 * transfer function is not the identity; the caller decides that. */
int cgb_hearing_aid_dev(float* d_in, int n_prof, int interval_len, const float* d_fir,
                        int fir_len, const float* d_iir, int iir_len, float* d_aux, void* stream);

/* One interval of cgb_jnd_batch_dev (rows index each lambda plane). */
typedef struct cgb_jnd_interval {
  int64_t row;      /* first row of the interval's window                   */
  int64_t ref_row;  /* first row of its reference interval's window         */
  double dA;        /* tone amplitude; <= 0 gives zero Fisher terms         */
  int32_t len;      /* window rows                                          */
  int32_t out;      /* output slot in F_RA / F_AI / MR                      */
} cgb_jnd_interval;

/* cgb_jnd_dev over intervals of any number of runs (signal groups of
 * different lengths) in one launch; d_iv is a device table of n_iv
 * descriptors, outputs are double[3][n_out] (MR double[3][n_out][256]).
 * Same arithmetic as cgb_jnd_dev.  The work is issued in table order, each
 * descriptor's three lambda planes together: a table sorted by len, longest
 * first, balances the GPU.  No counterpart in the reference, which runs one
 * interval length per call. */
int cgb_jnd_batch_dev(const float* d_lam, int64_t plane_rows, const cgb_jnd_interval* d_iv,
                      int n_iv, int n_out, const double* d_nihc, const float* W, double Fs,
                      double delta_alpha_len_factor, double* d_F_RA, double* d_F_AI,
                      double* d_MR, void* stream);

/* Equiripple low-pass FIR for the AC filter (the design problem the
 * reference hands to firpm in SubModel::calcFIRPM, src/SubModel.cpp:147-149):
 * Parks-McClellan / Remez exchange over the pass band [0, omega_c] (weight
 * weight_pass) and stop band [omega_c + transition, 1] (weight weight_stop),
 * frequencies normalised to Nyquist = 1; num_taps odd or even (3..4096);
 * taps double[num_taps] scaled to unit DC gain (fixDCGain).  delta_out:
 * the weighted ripple; iterations: exchanges used (both may be null). */
int cgb_design_equiripple_lowpass(int num_taps, double omega_c, double transition,
                                  double weight_pass, double weight_stop, double* taps,
                                  double* delta_out, int* iterations);

/* Complex-JND aggregation (ComplexJNDProfile, src/ComplexJNDProfile.cpp:19-100):
 * per profile, the JND values of its intervals across the tested power levels
 * (intervals int32[n_profiles][n_levels]: indexes into values/failed, the
 * calculated intervals) reduce to one value -- method 0: the last strict
 * interior local minimum (else a lower boundary value, warning 1); method 1:
 * the first value whose successor exceeds it by more than eps (else the
 * first, warning 1).  Outputs per profile: value (NaN where the reference
 * has none), warning, failed-convergence count of the chosen interval. */
int cgb_complex_jnd(const double* values, int n_values, const int32_t* failed,
                    const int32_t* intervals, int n_profiles, int n_levels, int method,
                    float eps, float* out_value, int32_t* out_warning, int32_t* out_failed);

/* Final JND in dB SPL per interval from the Fisher sums (host arrays):
 * 20 log10((1/sqrt(sum_j F_j)) / spl_ref), bounded at max_db; NaN for
 * reference intervals. */
int cgb_jnd_final(const double* F_RA, const double* F_AI, int n_int, const int32_t* ref_of,
                  double spl_ref, double max_db, double* jnd_rate_db, double* jnd_ai_db);

/* Host-side validation of a unit table against buffer sizes (the checks
 * cgb_bm_run_dev relies on); returns CGB_ERR_RANGE on the first bad unit. */
int cgb_check_units(const cgb_unit* units, int n_units, int n_profiles, int64_t in_len,
                    int64_t out_rows);

/* Launch shape of the BM kernel (register bound / CTAs per SM); 0 is the
 * default, cgb_bm_launch_shape_count() shapes are built.  Results do not
 * depend on the shape. */
int cgb_bm_set_launch_shape(int shape);
int cgb_bm_launch_shape_count(void);

/* Number of BM kernel launches enqueued by this process (for accounting). */
int64_t cgb_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* COCHLEA_GB300_H */
