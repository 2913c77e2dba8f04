// Test infrastructure: the CPU oracle of the cochlear-solver hot path.
//
// This file is NOT part of the product.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline / reference arm may load it, and only as the
// checker or as the timed CPU implementation -- never as the thing shipped.
//
// It restates, in plain C++, the arithmetic of the reference path
// (YonatanKoral/CochlearModel):
//   * model vectors            src/model.cpp:72-86, include/const.h:216-297
//   * tridiagonal diagonals    src/solver.cpp:155-176
//   * Thomas solve             src/tridiag.cpp:67-106
//   * block partition          src/cochlea.cu:1148-1176
//   * BM/OHC adaptive step     include/cochlea.cuh:13573-14245 (kernel 17)
//   * IHC + lambda             src/cochlea.cu:2712-2730, 2980-2988, 3291-3317,
//                              3365-3408, 3431-3506
//   * JND (Eq. 17-24)          src/cochlea.cu:3741-3944,
//                              src/AudioGramCreator.cpp:454-508
//   * input generation         src/cochlea.cu:4070-4103, 4165-4254
//
// Parity pinning: the reference publishes no tests, fixtures or golden
// vectors, and its host path cannot be built here (Windows/MFC/MATLAB).  Its
// Thomas solve (src/tridiag.cpp) and constants header (include/const.h)
// compile on their own; oracle/build_ref.sh builds them into oracle/_ref/ and
// tests/test_oracle_pins.py checks this restatement against them.  Its device
// code compiles too (oracle/build_ref_gpu.sh, launched by oracle/ref_gpu.cpp):
// on a GPU the IHC/lambda restatement in the reference's mixed precision
// equals the reference's own kernels bit for bit, the JND sums agree with
// them, and the product's reference-order BM mode equals BMOHC_NEW_kernel bit
// for bit (tests/test_ref_gpu_parity.py).
//
// FP32 mode fixes the order of every floating-point operation (explicit
// fmaf, IEEE division, a fixed reduction tree, the own-order pairs of Jacobi
// sweeps as one update over the second neighbours) so that the CUDA kernels,
// which follow the same order, agree with it bit for bit.  FP64 mode runs the
// reference algorithm (plain sweeps) in double and is the accuracy
// yardstick.
//
// Build: oracle/build.sh (g++ -O2 -ffp-contract=off, no fast-math).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

constexpr int NS = 256;  // cochlear sections (include/const.h:19)

// ---------------------------------------------------------------------------
// tanh in float.  The reference calls CUDA's tanhf; this project uses its own
// tanh on both sides so the GPU and the oracle round identically:
//   x P(z) / Q(z), z = min(x^2, 9.5^2), P and Q of degree 4 in z (a
//   minimax-relative rational fit on [0, 9], cochlearmodel_gb300/fit_tanh.py),
//   Horner in z, quotient as x P times own_rcpf(Q), result clamped to
//   [-1, 1]: from |x| = 9.5 on it saturates to +-1 exactly.
// Within 6.1 ulp of tanh (every float in [0, 9.5] checked); the GPU kernels evaluate the same sequence
// (cochlearmodel_gb300/csrc/cgb_device.cuh).
// ---------------------------------------------------------------------------
// 1/d for a positive normal d: bit-level seed 0x7EF311C3 - bits(d), then
// three Newton steps r <- r + r(1 - d r).
float own_rcpf(float d) {
  uint32_t bits;
  std::memcpy(&bits, &d, 4);
  bits = 0x7EF311C3u - bits;
  float r;
  std::memcpy(&r, &bits, 4);
  r = fmaf(r, fmaf(-d, r, 1.0f), r);
  r = fmaf(r, fmaf(-d, r, 1.0f), r);
  r = fmaf(r, fmaf(-d, r, 1.0f), r);
  return r;
}

float own_tanhf(float x) {
  const float z = fminf(x * x, 90.25f);
  float p = 1.335385846346071e-08f;
  p = fmaf(p, z, 2.0608504200936295e-05f);
  p = fmaf(p, z, 0.0034955532755702734f);
  p = fmaf(p, z, 0.13380996882915497f);
  p = fmaf(p, z, 1.0f);
  float q = 7.776229722367134e-07f;
  q = fmaf(q, z, 0.00032855774043127894f);
  q = fmaf(q, z, 0.02587684988975525f);
  q = fmaf(q, z, 0.46714311838150024f);
  q = fmaf(q, z, 1.0f);
  const float t = (x * p) * own_rcpf(q);
  return fminf(fmaxf(t, -1.0f), 1.0f);
}

// log10 of a positive normal float: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh((m-1)/(m+1)) by its odd series to s^11.
float own_log10f(float x) {
  uint32_t ix;
  std::memcpy(&ix, &x, 4);
  int e = (int)((ix >> 23) & 0xff) - 127;
  uint32_t mb = (ix & 0x7fffffu) | 0x3f800000u;
  float m;
  std::memcpy(&m, &mb, 4);
  bool hi = m > 1.41421356f;
  if (hi) {
    m = m * 0.5f;
    e += 1;
  }
  float f = m - 1.0f;
  float s = f * own_rcpf(2.0f + f);
  float s2 = s * s;
  float p = 1.0f / 11.0f;
  p = fmaf(p, s2, 1.0f / 9.0f);
  p = fmaf(p, s2, 1.0f / 7.0f);
  p = fmaf(p, s2, 1.0f / 5.0f);
  p = fmaf(p, s2, 1.0f / 3.0f);
  float two_s = 2.0f * s;
  float lnm = fmaf(two_s * s2, p, two_s);
  float ef = (float)e;
  const float l2hi = 0.30102999566398120f;
  const float l2lo = (float)(0.30102999566398120 - (double)0.30102999566398120f);
  return fmaf(ef, l2hi, fmaf(ef, l2lo, lnm * 0.43429448190325182f));
}

template <typename T> struct Ar;
template <> struct Ar<float> {
  // n/d as n * (1/|d|) with the sign of d (the kernels' division-free form)
  static float div(float n, float d) {
    float q = n * own_rcpf(fabsf(d));
    return d < 0.0f ? -q : q;
  }
  static float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static float tanh(float x) { return own_tanhf(x); }
  static float abs(float x) { return fabsf(x); }
  static float max(float a, float b) { return fmaxf(a, b); }
  static float min(float a, float b) { return fminf(a, b); }
};
template <> struct Ar<double> {
  static double div(double n, double d) { return n / d; }
  static double fma(double a, double b, double c) { return std::fma(a, b, c); }
  static double tanh(double x) { return std::tanh(x); }
  static double abs(double x) { return std::fabs(x); }
  static double max(double a, double b) { return std::fmax(a, b); }
  static double min(double a, double b) { return std::fmin(a, b); }
};

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Shared record layouts (the product declares identical ones in
// include/cochlea_gb300.h).
// ---------------------------------------------------------------------------
typedef struct {
  int64_t in_base;    // input index of frame sample 0
  int64_t out_base;   // output row of frame sample 0
  int32_t start;      // first input sample simulated (frame coords)
  int32_t out_first;  // first sample whose velocity row is written
  int32_t end;        // one past the last sample simulated
  int32_t profile;    // OHC (gamma) profile index
  float mtt;          // throw tolerance  (Max_Tolerance)
  float mmspt;        // m1_sp tolerance  (Max_M1_SP_Error)
} orc_unit;

typedef struct {
  int64_t substeps;
  int64_t iterations;
  int64_t sweeps;
  int32_t failed_samples;
  int32_t written_samples;
  int32_t status;
  int32_t pad_;
} orc_unit_stats;

typedef struct {
  float w_ohc, time_step, time_step_out, delta_x, alpha_r, Ts;
  float alpha_l, alpha_s, Gme, a0, a1, a2, sigma_ow, eta_1, eta_2;
  float dt_min, dt_max;
  int32_t jacobi_fast, jacobi_slow, max_outer;
  int32_t red_lanes;   // reduction tree width (sections per lane = 256/red_lanes)
  int32_t jacobi_mode; // 0 fixed sweeps (reference), 1 exact tridiagonal solve,
                       // 2 sweep pairs to a tolerance
  int32_t max_substeps_per_sample;  // a unit stops (status 1) past this many steps in a sample
  float jacobi_tol;    // mode 2: stop when max|p2 - p1| <= jacobi_tol * max|p2|
  int32_t jacobi_cap;  // mode 2: at most this many sweeps per solve (even)
  int32_t guess_mode;  // mode 2 first-solve guess: 0 previous pressure, 1 extrapolated
                       // (2, the network's guess, is GPU-only and treated as 1 here)
  int32_t learned_every;
  int32_t controller;  // 0 kernel 17 (summed margin), 1 BMOHC_NEW_kernel (any faulty section)
  int32_t arith;       // the FP32 oracle evaluates the own order (0) only; FP64 ignores it
} orc_bm_scalars;

float orc_tanhf(float x) { return own_tanhf(x); }
float orc_log10f(float x) { return own_log10f(x); }

// ---------------------------------------------------------------------------
// Model vectors in FP64 from the reference's float-valued constants
// (src/model.cpp:18-86, include/const.h:216-297) and the pressure system's
// diagonals (src/solver.cpp:155-176).  Outputs are 256-long arrays.
// scal_out (double[16]): w_ohc, dx, alpha_r, alpha_L, alpha_s, Gme, a0, a1,
// a2, sigma_ow, eta_1, eta_2, w_ow, Cme, ratio_K, psi0.
// ---------------------------------------------------------------------------
void orc_model_setup(double* M, double* R, double* S, double* Q, double* S_ohc,
                     double* S_tm, double* R_tm, double* diag_m, double* diag_l,
                     double* diag_u, double* scal_out) {
  const float PIf = 3.141592653589793f;
  // macro expansions evaluated in float, left to right, as the C++ compiler
  // does for the reference's #defines.
  float w_ohc_f = 2 * PIf * 1000.0f;                        // W_OHC
  float eta1_f = (1.0f) / (2e-6f) * 2 * PIf * 1000.0f;      // ETA_1
  float w_ow_f = 2 * PIf * 1500;                             // W_OW
  float cme_f = (2 * PIf * 1340) * (2 * PIf * 1340) * 0.059f / (0.49f * 1.4f);  // C_ME
  float bc0_f = ((2.0f * (1.0f) * (6e-3f)) / (0.5f));
  float bc1_f = ((0.5f) * (2 * PIf * 1500 * 2 * PIf * 1500) +
                 (2 * PIf * 1340) * (2 * PIf * 1340) * 0.059f / (0.49f * 1.4f) * (21.4f));
  float bc2_f = (0.5f) * (20e3f);
  float dx_f = (3.5f) / NS;

  const double dx = dx_f, area = 0.5f, rho = 1.0f, beta = 0.003f;
  const double w_ohc = w_ohc_f, ratio_K = 1e-3f;
  const double M0 = 1.286e-6f, M1 = 1.5f, R0 = 0.25f, R1 = -0.06f, S0 = 1.282e4f,
               S1 = -1.5f;
  const double a0 = bc0_f;
  for (int i = 0; i < NS; ++i) {
    M[i] = M0 * std::exp(M1 * dx * i);
    R[i] = R0 * std::exp(R1 * dx * i);
    S[i] = S0 * std::exp(S1 * dx * i);
    double wcf2 = S[i] / M[i];
    R_tm[i] = R[i];
    S_tm[i] = R[i] * wcf2 / w_ohc;
    S_ohc[i] = ratio_K * S_tm[i];
    Q[i] = 2 * rho * beta / (area * M[i]);
  }
  double dx2 = dx * dx;
  for (int i = 0; i < NS; ++i) {
    diag_u[i] = 1.0;
    diag_l[i] = 1.0;
    diag_m[i] = -1.0 * (2.0 + dx2 * Q[i]);
  }
  diag_m[0] = -1.0 * (1.0 + dx * a0);
  diag_m[NS - 1] = 1.0;
  diag_l[NS - 1] = 0.0;
  diag_l[NS - 2] = 0.0;
  double sc[16] = {w_ohc, dx, 0.0f /*BM_ALPHA_R*/, 2e-6f, 1e-6f, 21.4f, a0, bc1_f, bc2_f,
                   0.5f, eta1_f, 0.0 /*ETA_2*/, w_ow_f, cme_f, ratio_K, 70e-3f};
  std::memcpy(scal_out, sc, sizeof(sc));
}

// Thomas solve restated from src/tridiag.cpp:67-106: row i uses sub-diagonal
// l[i-1], diagonal m[i], super-diagonal u[i].
void orc_thomas(const double* m, const double* l, const double* u, const double* v,
                double* res, int n) {
  std::vector<double> k(n), h(n), p(n);
  k[0] = m[0];
  h[0] = u[0] / k[0];
  for (int i = 1; i < n; ++i) {
    k[i] = m[i] - l[i - 1] * h[i - 1];
    h[i] = u[i] / k[i];
  }
  p[0] = v[0] / m[0];
  for (int i = 1; i < n; ++i) p[i] = (v[i] - l[i - 1] * p[i - 1]) / k[i];
  res[n - 1] = p[n - 1];
  for (int j = n - 2; j >= 0; --j) res[j] = p[j] - res[j + 1] * h[j];
}

// Block partition of one run (src/cochlea.cu:1148-1176).  Writes
// start/out_first/end for each of `time_blocks` blocks.  out_first is the
// first sample the block owns; the reference also writes sample
// out_first-1, which the previous block owns (a cross-block write race).
void orc_block_partition(int time_blocks, int64_t samples_p1, int overlap, int decouple,
                         int32_t* start, int32_t* out_first, int32_t* end) {
  int64_t N = (samples_p1 - overlap) / (time_blocks + 1);
  for (int b = 0; b < time_blocks; ++b) {
    int transient_offset = (b > 0 && (decouple == 0 || (decouple != 1 && b % decouple != 0)));
    int pre = decouple > 0 && (decouple == 1 || ((b + 1) % decouple == 0)) && b != time_blocks - 1;
    int post = decouple > 0 && (b % decouple == 0);
    int64_t s = b * N;
    int64_t of = s + std::max(1 - transient_offset - post, 0) * (int64_t)overlap;
    int64_t len = N + (1 - pre) * (int64_t)overlap;
    int64_t e = s + len;
    if (b > 0) of = std::max<int64_t>(of, end[b - 1]);
    start[b] = (int32_t)s;
    out_first[b] = (int32_t)of;
    end[b] = (int32_t)e;
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// BM/OHC adaptive step of one unit (kernel 17 semantics, reference
// include/cochlea.cuh:13573-14245).  Decisions taken on the full block
// reduction (the reference's warp-0 lane-0 value; its other lanes race).
// ---------------------------------------------------------------------------
namespace {

template <typename T>
struct BMModel {
  T invM[NS], rm[NS], R[NS], S[NS], Q[NS], S_ohc[NS], S_tm[NS], R_tm[NS];
  // two-step sweep coefficients (FP32 own order): the lower / upper
  // neighbour's coefficient a_s / c_s and the centre's b_s
  T k2a[NS], k2c[NS], k2b[NS];
};

// Two sweeps p -> q -> p'' (q_s = Yrm_s - rm_s (l_s p_{s-1} + p_{s+1}), with
// l_s = 0 on sections 254 and 255 and the boundary values p_{-1} = p_256 =
// q_{-1} = q_256 = 0) fold into one update over the second neighbours:
//   p''_s = C_s + a_s p_{s-2} + b_s p_s + c_s p_{s+2},
//   C_s = Yrm_s - rm_s (l_s Yrm_{s-1} + Yrm_{s+1})   (one sweep applied to Y/m),
//   a_s = rm_s rm_{s-1}                 for 2 <= s <= 253, else 0,
//   c_s = rm_s rm_{s+1}                 for s <= 253, else 0,
//   b_s = rm_s (l_s rm_{s-1} + l_{s+1} rm_{s+1})  (rm_{-1} = rm_256 = 0).
// Each coefficient is one FP32 product (b_s of an FP32 sum).  In exact
// arithmetic p'' is the result of the two sweeps; in FP32 it takes three
// roundings per section instead of four.
template <typename T>
void two_step_coefficients(BMModel<T>& md) {
  for (int s = 0; s < NS; ++s) {
    const T r = md.rm[s];
    md.k2a[s] = (s >= 2 && s <= NS - 3) ? r * md.rm[s - 1] : (T)0;
    md.k2c[s] = s <= NS - 3 ? r * md.rm[s + 1] : (T)0;
    const T lo = (s >= 1 && s <= NS - 3) ? md.rm[s - 1] : (T)0;
    const T up = s + 1 <= NS - 3 ? md.rm[s + 1] : (T)0;
    md.k2b[s] = r * (lo + up);
  }
}

template <typename T>
T pair_sum(const T* t, int n) {
  return n == 1 ? t[0] : pair_sum(t, n / 2) + pair_sum(t + n / 2, n / 2);
}

// Sum over the 256 sections in the kernels' order: a pairwise tree over the
// sections of each lane, then an xor-butterfly across the lanes.
template <typename T>
T tree_sum(const T* term, int lanes) {
  int chunk = NS / lanes;
  T part[NS];
  for (int l = 0; l < lanes; ++l) part[l] = pair_sum(term + l * chunk, chunk);
  for (int o = lanes / 2; o >= 1; o /= 2) {
    T nxt[NS];
    for (int l = 0; l < lanes; ++l) nxt[l] = part[l] + part[l ^ o];
    for (int l = 0; l < lanes; ++l) part[l] = nxt[l];
  }
  return part[0];
}

// One Jacobi sweep, src -> dst: dst_s = fma(-(l_s src_{s-1} + src_{s+1}), 1/m_s, Y_s/m_s)
// with l_s = 0 on sections 254 and 255 and src_{-1} = src_256 = 0.
template <typename T>
void jacobi_sweep(const T* src, T* dst, const T* Yrm, const T* rm) {
  using A = Ar<T>;
  for (int s = 0; s < NS; ++s) {
    T pm1 = s > 0 ? src[s - 1] : (T)0;
    T pp1 = s < NS - 1 ? src[s + 1] : (T)0;
    T t = s < NS - 2 ? pm1 + pp1 : pp1;
    dst[s] = A::fma(-t, rm[s], Yrm[s]);
  }
}

template <typename T>
void exact_solve(const T* Y, const T* rm, T* p) {
  // kernel matrix: row s: l_s p_{s-1} + m_s p_s + p_{s+1} = Y_s,
  // l_s = 1 for s < 254 else 0 (reference include/cochlea.cuh:13736).
  double m[NS], l[NS], u[NS], v[NS], r[NS];
  for (int s = 0; s < NS; ++s) {
    m[s] = 1.0 / (double)rm[s];
    u[s] = 1.0;
    v[s] = (double)Y[s];
  }
  // tridiag.cpp convention: row i uses l[i-1]
  for (int s = 0; s < NS; ++s) l[s] = (s + 1 < NS - 2) ? 1.0 : 0.0;
  orc_thomas(m, l, u, v, r, NS);
  for (int s = 0; s < NS; ++s) p[s] = (T)r[s];
}

template <typename T, typename TO>
void bm_unit(const BMModel<T>& md, const T* gam, const T* gs, const orc_bm_scalars& sc,
             const orc_unit& un, const float* in, TO* out, int32_t* failed, float* conv,
             orc_unit_stats* st) {
  using A = Ar<T>;
  T x0[NS] = {}, v0[NS] = {}, a0[NS] = {}, y0[NS] = {}, u0[NS] = {}, ps0[NS] = {}, dp0[NS] = {};
  T x[NS] = {}, v[NS] = {}, a[NS] = {}, y[NS] = {}, u[NS] = {}, ps[NS] = {}, dp[NS] = {};
  T Ptm[NS] = {}, p[NS] = {}, Y[NS] = {}, G[NS] = {}, aref[NS] = {}, dv[NS] = {},
    flt[NS] = {}, tmp[NS] = {}, Yrm[NS] = {};
  T w0 = 0, wd0 = 0, wdd0 = 0, w = 0, wd = 0, wdd = 0;
  const T ratio = (T)(sc.alpha_l / sc.alpha_s);  // float division as the host does it
  const T nas = -(T)sc.alpha_s, al = (T)sc.alpha_l;
  const T e1 = (T)sc.eta_1, e2 = (T)sc.eta_2, nw = -(T)sc.w_ohc;
  const T ar = (T)sc.alpha_r;
  const T dx = (T)sc.delta_x;
  const T dx2 = dx * dx, dxa0 = dx * (T)sc.a0;
  const T na1 = -(T)sc.a1, na2 = -(T)sc.a2, Gme = (T)sc.Gme, sow = (T)sc.sigma_ow;
  const T mtt = (T)un.mtt, mmspt = (T)un.mmspt;
  const T dtmin = (T)sc.dt_min, dtmax = (T)sc.dt_max;
  const double Tout = (double)sc.time_step_out;
  const double invTs = 1.0 / (double)sc.Ts;
  const float* inb = in + un.in_base;
  TO* outb = out ? out + un.out_base * (int64_t)NS : nullptr;
  int32_t* fb = failed ? failed + un.out_base : nullptr;
  float* cb = conv ? conv + un.out_base * 3 : nullptr;
  float smp_dt = 0.0f, smp_sub = 0.0f, smp_it = 0.0f;

  T dt = (T)sc.time_step;
  // simulated time since the current sample: FP32 keeps it in a float
  // accumulator as the kernels (and the reference's curr_time_f) do, with
  // 1/Ts formed in double and rounded; the FP64 method in double
  constexpr bool kF32 = std::is_same<T, float>::value;
  double tau = 0.0;
  float tau_f = 0.0f;
  const float fs_f = (float)(1.0 / (double)sc.Ts), tout_f = sc.time_step_out;
  int64_t n = un.start;
  // tolerance mode: pressure at the start of the last two steps, dt ratio
  T hist[2][NS] = {};
  T dt_prev = dt, rho = (T)1;
  T sx0 = (T)inb[n], sx1 = (T)inb[n + 1];
  int fail_flag = 0;
  int64_t sub_in_sample = 0;
  orc_unit_stats S = {};
  while (n < un.end) {
    if (++sub_in_sample > sc.max_substeps_per_sample) {
      S.status = 1;
      break;
    }
    int out_loop = 0, reset = 1, another = 1;
    if (sc.jacobi_mode == 2) {
      rho = dt / dt_prev;
      dt_prev = dt;
      for (int s = 0; s < NS; ++s) hist[S.substeps & 1][s] = p[s];
    }
    const T delta = kF32 ? (T)(tau_f * fs_f) : (T)(tau * invTs);
    const T smp = A::fma(sx1, delta, sx0 * ((T)1 - delta));
    // (s * 0.5) * dt == s * (dt * 0.5) exactly (power-of-two scaling), so
    // each trapezoid update is one fma with the half step
    const T hdt = dt * (T)0.5;
    while (another) {
      for (int s = 0; s < NS; ++s) aref[s] = a[s];
      if (out_loop == 0 || reset) {
        out_loop = 0;
        for (int s = 0; s < NS; ++s) {
          y[s] = A::fma(u0[s], dt, y0[s]);
          T vn = A::fma(a0[s], dt, v0[s]);
          dv[s] = A::abs(vn - v[s]);
          v[s] = vn;
          x[s] = A::fma(v0[s] + vn, hdt, x0[s]);
          ps[s] = A::fma(dp0[s], dt, ps0[s]);
        }
        w = A::fma(wd0, dt, w0);
        wd = A::fma(wdd0, dt, wd0);
      } else {
        for (int s = 0; s < NS; ++s) {
          T vn = A::fma(a0[s] + a[s], hdt, v0[s]);
          dv[s] = A::abs(vn - v[s]);
          v[s] = vn;
          x[s] = A::fma(v0[s] + vn, hdt, x0[s]);
          y[s] = A::fma(u0[s] + u[s], hdt, y0[s]);
          ps[s] = A::fma(dp0[s] + dp[s], hdt, ps0[s]);
        }
        w = A::fma(wd0 + wd, hdt, w0);
        wd = A::fma(wdd0 + wdd, hdt, wd0);
      }
      for (int s = 0; s < NS; ++s) {
        T d = y[s] - x[s];
        T Pohc = gs[s] * d;
        if (out_loop < 2) {
          T t = A::tanh(ratio * ps[s]);
          T dL = nas * t;
          T Aa = al * A::fma(t, t, (T)-1);
          T N1 = A::fma(e1, d, A::fma(e2, v[s], nw * ps[s]));
          T N = A::fma(md.S_tm[s], dL, (N1 * md.R_tm[s]) * Aa);
          T Pp = A::fma(md.S_tm[s], y[s], Pohc);
          T num = A::fma(-gam[s], N, Pp);
          T den = md.R_tm[s] * A::fma(gam[s] * Aa, e2, (T)-1);
          u[s] = A::div(num, den);
          Ptm[s] = A::fma(md.R_tm[s], u[s], md.S_tm[s] * y[s]);
        }
        T g = md.R[s] * A::fma(ar, v[s] * v[s], (T)1);
        g = A::fma(g, v[s], md.S[s] * x[s]);
        G[s] = -g - Ptm[s];
        if (s == 0) {
          Y[s] = dxa0 * A::fma(na1, w, A::fma(na2, wd, Gme * smp));
        } else if (s == NS - 1) {
          Y[s] = 0;
        } else {
          Y[s] = (dx2 * G[s]) * md.Q[s];
        }
      }
      int J = out_loop < 2 ? sc.jacobi_slow : sc.jacobi_fast;
      if (sc.jacobi_mode == 1) {
        exact_solve<T>(Y, md.rm, p);
      } else if (sc.jacobi_mode == 2) {
        // Tolerance mode: sweeps run in pairs; after each pair the update of
        // the second sweep and the pressure are measured in the infinity
        // norm, and the solve stops when max|p2 - p1| <= tol * max|p2| or at
        // the sweep cap.  The GPU kernel checks at the same points.
        for (int s = 0; s < NS; ++s) Yrm[s] = Y[s] * md.rm[s];
        if (out_loop == 0 && S.substeps >= 2 && sc.guess_mode >= 1) {
          // p1 + rho (p1 - p2): linear extrapolation of the last two steps
          const T* p2 = hist[(S.substeps + 1) & 1];
          for (int s = 0; s < NS; ++s) p[s] = A::fma(rho, p[s] - p2[s], p[s]);
        }
        const T tol = (T)sc.jacobi_tol;
        int done = 0;
        while (done < sc.jacobi_cap) {
          jacobi_sweep<T>(p, tmp, Yrm, md.rm);
          jacobi_sweep<T>(tmp, p, Yrm, md.rm);
          done += 2;
          T dmax = 0, pmax = 0;
          for (int s = 0; s < NS; ++s) {
            dmax = A::max(dmax, A::abs(p[s] - tmp[s]));
            pmax = A::max(pmax, A::abs(p[s]));
          }
          if (dmax <= tol * pmax) break;
        }
        S.sweeps += done;
      } else if (kF32 && J >= 4) {
        // Own FP32 order with four or more sweeps: C = one sweep applied to
        // Y/m, then J/2 two-step updates (two_step_coefficients), then a
        // last single sweep if J is odd.  The kernel holds sections 8l+j and
        // 8l+7-j (j < 4) of lane l as one register pair and adds the two
        // neighbour terms in the pair's order: sections with s mod 8 < 4 add
        // the upper term, then the lower; the others the lower, then the
        // upper.  Beyond the ends the neighbour values are those the warp
        // shuffles deliver, each times a zero coefficient: p_254, p_255 below
        // sections 0 and 1, p_248, p_249 above sections 254 and 255.
        for (int s = 0; s < NS; ++s) Yrm[s] = Y[s] * md.rm[s];
        T C2[NS];
        jacobi_sweep<T>(Yrm, C2, Yrm, md.rm);
        int it = 0;
        for (; it + 1 < J; it += 2) {
          for (int s = 0; s < NS; ++s) {
            const T lo = s >= 2 ? p[s - 2] : p[s + NS - 2];
            const T hi = s <= NS - 3 ? p[s + 2] : p[s - 6];
            T r = A::fma(md.k2b[s], p[s], C2[s]);
            if ((s & 7) < 4) {
              r = A::fma(md.k2c[s], hi, r);
              r = A::fma(md.k2a[s], lo, r);
            } else {
              r = A::fma(md.k2a[s], lo, r);
              r = A::fma(md.k2c[s], hi, r);
            }
            tmp[s] = r;
          }
          for (int s = 0; s < NS; ++s) p[s] = tmp[s];
        }
        if (it < J) {
          jacobi_sweep<T>(p, tmp, Yrm, md.rm);
          for (int s = 0; s < NS; ++s) p[s] = tmp[s];
        }
        S.sweeps += J;
      } else {
        // p_s <- (Y_s - (l_s p_{s-1} + p_{s+1})) / m_s, evaluated as
        // fma(-t, 1/m_s, Y_s/m_s) with Y_s/m_s formed once per iteration.
        for (int s = 0; s < NS; ++s) Yrm[s] = Y[s] * md.rm[s];
        for (int it = 0; it < J; ++it) {
          for (int s = 0; s < NS; ++s) {
            T pm1 = s > 0 ? p[s - 1] : (T)0;
            T pp1 = s < NS - 1 ? p[s + 1] : (T)0;
            T t = s < NS - 2 ? pm1 + pp1 : pp1;
            tmp[s] = A::fma(-t, md.rm[s], Yrm[s]);
          }
          for (int s = 0; s < NS; ++s) p[s] = tmp[s];
        }
        S.sweeps += J;
      }
      for (int s = 0; s < NS; ++s) {
        a[s] = (p[s] + G[s]) * md.invM[s];
        T d = y[s] - x[s];
        dp[s] = A::fma(e1, d, A::fma(e2, u[s] - v[s], nw * ps[s]));
      }
      // (the kernels multiply by 1/sigma_ow where sigma_ow is a power of two:
      // the same value)
      wdd = A::fma(na1, w, A::fma(na2, wd, A::fma(Gme, smp, p[0]))) / sow;
      if (reset == 0) {
        T ea = 0;
        bool any_fault = false;
        for (int s = 0; s < NS; ++s) {
          ea = A::max(ea, A::abs(aref[s] - a[s]));
          const T thr = A::max(mtt, v[s] * dt);
          flt[s] = dv[s] - thr;
          any_fault = any_fault || dv[s] > thr;
        }
        T ev = tree_sum<T>(dv, sc.red_lanes);
        // controller 0 (kernel 17): the summed margin is positive;
        // controller 1 (BMOHC_NEW_kernel, include/cochlea.cuh:4080-4100):
        // some section fails the speed test (its fault count is positive)
        const bool faulty =
            sc.controller == 1 ? any_fault : tree_sum<T>(flt, sc.red_lanes) > (T)0;
        // L = ea dt / ev (0 unless ev > mmspt).  In FP32 the kernels test
        // L > 6 as ea dt > 6 ev and L < 0.5 as ea dt < 0.5 ev (6 ev rounded
        // once); the FP64 method divides.
        const T num = ea * dt;
        const bool lcheck = ev > mmspt;
        bool l_big, l_small;
        if (std::is_same<T, float>::value) {
          l_big = lcheck && num > (T)6 * ev;
          l_small = !lcheck || num < (T)0.5 * ev;
        } else {
          const T L = lcheck ? num / ev : (T)0;
          l_big = L > (T)6;
          l_small = L < (T)0.5;
        }
        if (l_big) {
          dt = dt * (T)0.5;
          if (dt < dtmin) dt = dtmin;
          another = 0;
          reset = 1;
        } else if (faulty) {
          another = 1;
          reset = 0;
        } else if (l_small) {
          dt = dt * (T)2;
          if (dt > dtmax) dt = dtmax;
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
      if (out_loop >= sc.max_outer) {
        another = 0;
        reset = 1;
        fail_flag = 1;
      }
    }
    S.substeps += 1;
    S.iterations += out_loop;
    smp_sub = smp_sub + 1.0f;
    smp_dt = smp_dt + (float)dt;
    smp_it = smp_it + (float)out_loop;
    if (kF32 ? tau_f > tout_f : tau > Tout) {
      if (kF32)
        tau_f = tau_f - tout_f;
      else
        tau -= Tout;
      sx0 = sx1;
      sx1 = (T)inb[n + 2];
      if (n >= un.out_first) {
        if (outb)
          for (int s = 0; s < NS; ++s) outb[n * NS + s] = (TO)v[s];
        if (fb) fb[n] = fail_flag;
        if (cb) {
          cb[n * 3 + 0] = smp_dt / smp_sub;
          cb[n * 3 + 1] = smp_sub;
          cb[n * 3 + 2] = smp_it / smp_sub;
        }
        S.written_samples += 1;
        S.failed_samples += fail_flag;
      }
      fail_flag = 0;
      sub_in_sample = 0;
      smp_dt = smp_sub = smp_it = 0.0f;
      ++n;
    }
    for (int s = 0; s < NS; ++s) {
      x0[s] = x[s];
      v0[s] = v[s];
      a0[s] = a[s];
      ps0[s] = ps[s];
      dp0[s] = dp[s];
      u0[s] = u[s];
      y0[s] = y[s];
    }
    w0 = w;
    wd0 = wd;
    wdd0 = wdd;
    if (kF32)
      tau_f = tau_f + (float)dt;
    else
      tau += (double)dt;
  }
  if (st) *st = S;
}

template <typename T, typename TO>
void bm_run(const float* secp, const float* gamma, const orc_bm_scalars* sc,
            const orc_unit* units, int n_units, const float* in, TO* out, int32_t* failed,
            float* conv, orc_unit_stats* stats, int n_threads) {
  // secp: float[8][256] = invM, rm, R, S, Q, S_ohc, S_tm, R_tm
  BMModel<T> md;
  for (int s = 0; s < NS; ++s) {
    md.invM[s] = (T)secp[0 * NS + s];
    md.rm[s] = (T)secp[1 * NS + s];
    md.R[s] = (T)secp[2 * NS + s];
    md.S[s] = (T)secp[3 * NS + s];
    md.Q[s] = (T)secp[4 * NS + s];
    md.S_ohc[s] = (T)secp[5 * NS + s];
    md.S_tm[s] = (T)secp[6 * NS + s];
    md.R_tm[s] = (T)secp[7 * NS + s];
  }
  two_step_coefficients(md);
  std::atomic<int> next(0);
  auto worker = [&]() {
    T gam[NS], gs[NS];
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= n_units) break;
      const orc_unit& un = units[i];
      for (int s = 0; s < NS; ++s) {
        gam[s] = (T)gamma[(int64_t)un.profile * NS + s];
        gs[s] = gam[s] * md.S_ohc[s];
      }
      bm_unit<T, TO>(md, gam, gs, *sc, un, in, out, failed, conv, stats ? stats + i : nullptr);
    }
  };
  n_threads = std::max(1, n_threads);
  if (n_threads == 1) {
    worker();
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t) th.emplace_back(worker);
    for (auto& t : th) t.join();
  }
}

}  // namespace

extern "C" {

void orc_bm_run_f32(const float* secp, const float* gamma, const orc_bm_scalars* sc,
                    const orc_unit* units, int n_units, const float* in, float* out,
                    int32_t* failed, float* conv, orc_unit_stats* stats, int n_threads) {
  bm_run<float, float>(secp, gamma, sc, units, n_units, in, out, failed, conv, stats, n_threads);
}

void orc_bm_run_f64(const float* secp, const float* gamma, const orc_bm_scalars* sc,
                    const orc_unit* units, int n_units, const float* in, double* out,
                    int32_t* failed, float* conv, orc_unit_stats* stats, int n_threads) {
  bm_run<double, double>(secp, gamma, sc, units, n_units, in, out, failed, conv, stats, n_threads);
}

// ---------------------------------------------------------------------------
// IHC + lambda of one frame, reference mixed precision (double taps and
// accumulators, float buffers): src/cochlea.cu:2712-2730 (FIR with the
// decoupled look-back limit), 2980-2988 (dS), 3291-3317 (IHC log),
// 3365-3408 (lambda).
//   v       : float [rows][256] BM velocity of the frame
//   seg     : decoupled interval length (Time_Block_Length nodes x Decouple_Filter)
//   frdp    : Time_Block_Length nodes x Time_Blocks (final_regular_division_position)
//   total   : rows rounded up to 64 (calcTime)
//   lam_rows: rows for which lambda is produced (Time_Block_Length nodes x Time_Blocks)
//   ihc     : float [rows][256] IHC output; lam: float [3][lam_stride][256]
// ---------------------------------------------------------------------------
static inline int fir_taps_used(int k, int seg, int frdp, int total, int taps) {
  int sg = k / (frdp - 1);
  sg = sg * total + (1 - sg) * seg;
  int lim = (k + 1) % sg;
  return lim < taps ? lim : taps;
}

// ac_in: AC already computed (the IIR path), else the AC FIR runs.
static void ihc_lambda_impl(const float* v, int rows, int seg, int frdp, int total, int lam_rows,
                            const double* ac_taps, int n_ac, const double* dc_taps, int n_dc,
                            double scale, double eta_ac, double eta_dc, const double* ihc_damage,
                            const float* aihc, const float* spont, double lambda_sat, float* ihc,
                            float* lam, int64_t lam_stride, int mode, const float* ac_in,
                            int stage = 0, float* stage_out = nullptr) {
  // stage 9 AC, 10 DC, 11 dS of every lambda row into stage_out [rows][256]
  auto put_stage = [&](int which, int k, int s, double val) {
    if (stage_out && stage == which && k < lam_rows) stage_out[(size_t)k * NS + s] = (float)val;
  };
  if (mode == 2) {
    // The GB300 kernel's arithmetic: float taps (AC taps pre-scaled), each
    // FIR summed over taps in order with the compensated dot product Dot2
    // (Ogita, Rump, Oishi 2005) -- for symmetric AC taps and rows with the
    // whole filter, over tap pairs (dot2s) -- own log10, float lambda.
    auto dot2 = [](const float* b, const float* x, int tu) {
      float s = 0.0f, c = 0.0f;
      for (int i = 0; i < tu; ++i) {
        float p = b[i] * x[-(int64_t)i * NS];
        float q = fmaf(b[i], x[-(int64_t)i * NS], -p);
        float t = s + p;
        float z = t - s;
        float e = (s - (t - z)) + (p - z);
        s = t;
        c = c + (e + q);
      }
      return s + c;
    };
    // Linear-phase (symmetric) taps, rows with the whole filter: the pair
    // x_{t-k} + x_{t-n+1+k} is formed exactly by TwoSum, Dot2 takes b_k
    // times its rounded sum, and b_k times the sum's rounding error goes into
    // the compensation with one fma; the centre tap of an odd filter last.
    auto dot2s = [](const float* b, const float* x, int n) {
      float s = 0.0f, c = 0.0f;
      auto step = [&](float bb, float xx) {
        float p = bb * xx;
        float q = fmaf(bb, xx, -p);
        float t = s + p;
        float z = t - s;
        float e = (s - (t - z)) + (p - z);
        s = t;
        c = c + (e + q);
      };
      for (int k = 0; k < n / 2; ++k) {
        const float x1 = x[-(int64_t)k * NS], x2 = x[-(int64_t)(n - 1 - k) * NS];
        const float sg = x1 + x2;
        const float zz = sg - x1;
        const float ep = (x1 - (sg - zz)) + (x2 - zz);
        step(b[k], sg);
        c = fmaf(b[k], ep, c);
      }
      if (n & 1) step(b[n / 2], x[-(int64_t)(n / 2) * NS]);
      return s + c;
    };
    std::vector<float> acf((size_t)rows * NS), dsf((size_t)rows * NS);
    std::vector<float> bt(n_ac), dt(n_dc);
    for (int i = 0; i < n_ac; ++i) bt[i] = (float)(ac_taps[i] * scale);
    for (int i = 0; i < n_dc; ++i) dt[i] = (float)dc_taps[i];
    bool ac_sym = n_ac > 1;
    for (int i = 0; i < n_ac / 2; ++i) ac_sym = ac_sym && bt[i] == bt[n_ac - 1 - i];
    const float sc = (float)scale, ea = (float)eta_ac, ed = (float)eta_dc;
    for (int k = 0; k < lam_rows; ++k) {
      int tu = fir_taps_used(k, seg, frdp, total, n_ac);
      for (int s = 0; s < NS; ++s) {
        float acc = ac_in ? ac_in[(size_t)k * NS + s]
                          : (ac_sym && tu == n_ac ? dot2s(bt.data(), v + (size_t)k * NS + s, tu)
                                                  : dot2(bt.data(), v + (size_t)k * NS + s, tu));
        acf[(size_t)k * NS + s] = acc;
        float ms = fmaf(v[(size_t)k * NS + s], sc, -acc);
        dsf[(size_t)k * NS + s] = ms * ms;
        put_stage(9, k, s, acc);
        put_stage(11, k, s, dsf[(size_t)k * NS + s]);
      }
    }
    // DC with uniform taps d: d * (window sum), the window re-summed at
    // rows k % 32 == 0 and where the look-back rule restarts it, otherwise
    // updated by +dS[k] (and -dS[k-tu] once full), in TwoSum arithmetic.
    bool uniform = true;
    for (int i = 1; i < n_dc; ++i) uniform = uniform && dt[i] == dt[0];
    auto two_sum_add = [](float& ws, float& wc, float x) {
      float t = ws + x;
      float z = t - ws;
      float e = (ws - (t - z)) + (x - z);
      ws = t;
      wc = wc + e;
    };
    std::vector<float> wsum(NS, 0.0f), wcomp(NS, 0.0f);
    int tu_prev = -1;
    for (int k = 0; k < lam_rows; ++k) {
      int tu = fir_taps_used(k, seg, frdp, total, n_dc);
      const bool anchor = k % 32 == 0 || (tu != tu_prev && tu != tu_prev + 1);
      for (int s = 0; s < NS; ++s) {
        float acc;
        if (uniform) {
          float& ws = wsum[s];
          float& wc = wcomp[s];
          if (anchor) {
            ws = wc = 0.0f;
            for (int j = 0; j < tu; ++j) two_sum_add(ws, wc, dsf[(size_t)(k - j) * NS + s]);
          } else {
            two_sum_add(ws, wc, dsf[(size_t)k * NS + s]);
            if (tu == tu_prev) two_sum_add(ws, wc, -dsf[(size_t)(k - tu) * NS + s]);
          }
          const float d = dt[0];
          const float p = d * ws;
          const float q = fmaf(d, ws, -p);
          acc = p + fmaf(d, wc, q);
        } else {
          acc = dot2(dt.data(), dsf.data() + (size_t)k * NS + s, tu);
        }
        put_stage(10, k, s, acc);
        float pre = fmaf(acf[(size_t)k * NS + s], ea, acc * ed);
        float y = (float)ihc_damage[s] * pre;
        float lg = own_log10f(fmaxf(y, 0.0f) + 1e-20f);
        if (ihc) ihc[(size_t)k * NS + s] = lg;
        for (int j = 0; j < 3; ++j) {
          float val = s != 0 ? fminf((float)lambda_sat, fmaxf(aihc[j * NS + s] * lg, spont[j]))
                             : spont[j];
          lam[(size_t)j * lam_stride * NS + (size_t)k * NS + s] = val;
        }
      }
      tu_prev = tu;
    }
    return;
  }
  int fp64 = mode == 1;
  std::vector<double> ac((size_t)rows * NS), ds((size_t)rows * NS);
  for (int k = 0; k < rows; ++k) {
    int tu = fir_taps_used(k, seg, frdp, total, n_ac);
    for (int s = 0; s < NS; ++s) {
      double acc = 0.0;
      if (ac_in)
        acc = (double)ac_in[(size_t)k * NS + s];
      else
        for (int i = 0; i < tu; ++i)
          acc = acc + ac_taps[i] * scale * (double)v[(size_t)(k - i) * NS + s];
      if (fp64) {
        ac[(size_t)k * NS + s] = acc;
        double ms = (double)v[(size_t)k * NS + s] * scale - acc;
        ds[(size_t)k * NS + s] = ms * ms;
      } else {
        float acf = (float)acc;
        ac[(size_t)k * NS + s] = acf;
        float ms = fmaf(v[(size_t)k * NS + s], (float)scale, -acf);
        ds[(size_t)k * NS + s] = (double)(ms * ms);
      }
      put_stage(9, k, s, ac[(size_t)k * NS + s]);
      put_stage(11, k, s, ds[(size_t)k * NS + s]);
    }
  }
  for (int k = 0; k < rows; ++k) {
    int tu = fir_taps_used(k, seg, frdp, total, n_dc);
    for (int s = 0; s < NS; ++s) {
      double acc = 0.0;
      for (int i = 0; i < tu; ++i) acc = acc + dc_taps[i] * ds[(size_t)(k - i) * NS + s];
      put_stage(10, k, s, acc);
      double pre;
      if (fp64) {
        pre = ac[(size_t)k * NS + s] * eta_ac + acc * eta_dc;
      } else {
        float dcf = (float)acc;
        pre = (double)fmaf((float)ac[(size_t)k * NS + s], (float)eta_ac,
                           (float)((double)dcf * eta_dc));
      }
      double lg = std::log10(std::fmax(ihc_damage[s] * pre, 0.0) + 1e-20);
      if (ihc && k < lam_rows) ihc[(size_t)k * NS + s] = (float)lg;
      if (k < lam_rows) {
        for (int j = 0; j < 3; ++j) {
          double sp = (double)spont[j];
          double A = (double)aihc[j * NS + s];
          double base = std::fmin(lambda_sat, std::fmax(A * (fp64 ? lg : (double)(float)lg), sp));
          double val = s != 0 ? base : sp;
          lam[(size_t)j * lam_stride * NS + (size_t)k * NS + s] = (float)val;
        }
      }
    }
  }
}

void orc_ihc_lambda(const float* v, int rows, int seg, int frdp, int total, int lam_rows,
                    const double* ac_taps, int n_ac, const double* dc_taps, int n_dc,
                    double scale, double eta_ac, double eta_dc, const double* ihc_damage,
                    const float* aihc /*[3][256]*/, const float* spont /*[3]*/,
                    double lambda_sat, float* ihc, float* lam, int64_t lam_stride,
                    int mode /*0: reference mixed precision, 1: all double, 2: kernel FP32*/) {
  ihc_lambda_impl(v, rows, seg, frdp, total, lam_rows, ac_taps, n_ac, dc_taps, n_dc, scale,
                  eta_ac, eta_dc, ihc_damage, aihc, spont, lambda_sat, ihc, lam, lam_stride, mode,
                  nullptr);
}

// Hearing-aid shaping (CudaProcessSignalTroughHearingAID and ...IIR,
// src/cochlea.cu:4105-4150): per interval of length L,
//   aux[n] = fma chain over i < min(n, fir_len) of fir[i] x[n-i], from 0;
//   out[n] = fma chain over 1 <= j < min(n+1, iir_len) of iir[j] aux[n-j],
//            from aux[n]  (iir_len 0: out = aux).
void orc_hearing_aid(const float* x, int n_prof, int L, const float* fir, int fir_len,
                     const float* iir, int iir_len, float* out) {
  std::vector<float> aux((size_t)n_prof * L);
  for (int p = 0; p < n_prof; ++p)
    for (int n = 0; n < L; ++n) {
      const float* xs = x + (size_t)p * L;
      const int back = std::min(n, fir_len);
      float acc = 0.0f;
      for (int i = 0; i < back; ++i) acc = fmaf(fir[i], xs[n - i], acc);
      aux[(size_t)p * L + n] = acc;
    }
  for (int p = 0; p < n_prof; ++p)
    for (int n = 0; n < L; ++n) {
      const float* as = aux.data() + (size_t)p * L;
      float acc = as[n];
      if (iir_len > 0) {
        const int back = std::min(n + 1, iir_len);
        for (int j = 1; j < back; ++j) acc = fmaf(iir[j], as[n - j], acc);
      }
      out[(size_t)p * L + n] = acc;
    }
}

// AC by the reference's IIR recursion (DeviceCudaIIRFilter, src/cochlea.cu:2745-2775):
//   Y[k] = sum_{i<ob} b_i X[k-i] - sum_{1<=j<ob} a_j Y[k-j],  ob = the FIR look-back
// bound, accumulated in float with each term added in double and rounded
// (the reference's float accumulator with double taps; products and sums kept
// as separate roundings).  b taps are multiplied by scale once, as the host
// does; a_0 is not used (normalised).
void orc_iir_ac(const float* v, int rows, int seg, int frdp, int total, const double* b,
                const double* a, int n, double scale, float* ac) {
  std::vector<double> bs(n);
  for (int i = 0; i < n; ++i) bs[i] = b[i] * scale;
  for (int k = 0; k < rows; ++k) {
    const int ob = fir_taps_used(k, seg, frdp, total, n);
    for (int s = 0; s < NS; ++s) {
      float y = 0.0f;
      for (int i = 0; i < ob; ++i) y = (float)((double)y + bs[i] * (double)v[(size_t)(k - i) * NS + s]);
      for (int j = 1; j < ob; ++j) y = (float)((double)y - a[j] * (double)ac[(size_t)(k - j) * NS + s]);
      ac[(size_t)k * NS + s] = y;
    }
  }
}

// IHC + lambda with the AC stage by the IIR recursion; mode as orc_ihc_lambda
// (the AC itself is the reference arithmetic in every mode).
void orc_ihc_lambda_iir(const float* v, int rows, int seg, int frdp, int total, int lam_rows,
                        const double* b, const double* a, int n_iir, const double* dc_taps,
                        int n_dc, double scale, double eta_ac, double eta_dc,
                        const double* ihc_damage, const float* aihc, const float* spont,
                        double lambda_sat, float* ihc, float* lam, int64_t lam_stride, int mode,
                        float* ac_out) {
  std::vector<float> ac((size_t)rows * NS);
  orc_iir_ac(v, rows, seg, frdp, total, b, a, n_iir, scale, ac.data());
  if (ac_out) std::copy(ac.begin(), ac.end(), ac_out);
  ihc_lambda_impl(v, rows, seg, frdp, total, lam_rows, b, n_iir, dc_taps, n_dc, scale, eta_ac,
                  eta_dc, ihc_damage, aihc, spont, lambda_sat, ihc, lam, lam_stride, mode,
                  ac.data());
}

// orc_ihc_lambda that also stores one intermediate plane of every lambda row
// into stage_out [lam_rows][256]: stage 9 AC, 10 DC, 11 dS (RunIHCKernel's
// backup stages, src/cochlea.cu:3431-3506), in `mode`'s arithmetic.
void orc_ihc_lambda_stage(const float* v, int rows, int seg, int frdp, int total, int lam_rows,
                          const double* ac_taps, int n_ac, const double* dc_taps, int n_dc,
                          double scale, double eta_ac, double eta_dc, const double* ihc_damage,
                          const float* aihc, const float* spont, double lambda_sat, float* ihc,
                          float* lam, int64_t lam_stride, int mode, int stage,
                          float* stage_out) {
  ihc_lambda_impl(v, rows, seg, frdp, total, lam_rows, ac_taps, n_ac, dc_taps, n_dc, scale,
                  eta_ac, eta_dc, ihc_damage, aihc, spont, lambda_sat, ihc, lam, lam_stride, mode,
                  nullptr, stage, stage_out);
}

// IHC + lambda from a given AC stage (ac: rows x 256 floats) in place of the
// FIR; everything after the AC stage as orc_ihc_lambda in `mode`.  Accuracy
// studies of other AC arithmetic feed their AC through it, and the IIR path's
// debug stages are checked with it (stage / stage_out as orc_ihc_lambda_stage;
// stage 0 for none).
void orc_ihc_lambda_ac(const float* v, const float* ac, int rows, int seg, int frdp, int total,
                       int lam_rows, const double* dc_taps, int n_dc, double scale,
                       double eta_ac, double eta_dc, const double* ihc_damage, const float* aihc,
                       const float* spont, double lambda_sat, float* ihc, float* lam,
                       int64_t lam_stride, int mode, int stage, float* stage_out) {
  const double one = 1.0;
  ihc_lambda_impl(v, rows, seg, frdp, total, lam_rows, &one, 1, dc_taps, n_dc, scale, eta_ac,
                  eta_dc, ihc_damage, aihc, spont, lambda_sat, ihc, lam, lam_stride, mode, ac,
                  stage, stage_out);
}

// ---------------------------------------------------------------------------
// JND (Eq. 17-24): src/cochlea.cu:3741-3944 and
// src/AudioGramCreator.cpp:454-508.  lam: float [3][lam_stride][256] with
// interval i starting at row i*interval_nodes.  ref_of[i] is the reference
// interval of i (== i for a reference interval).  Outputs (double) F_RA and
// FisherAI_sum [3][n_int].  mode 0: reference float arithmetic; 1: FP64 sums.
// ---------------------------------------------------------------------------
void orc_jnd(const float* lam, int64_t lam_stride, int n_int, int interval_nodes, int head,
             int len, const double* dA, const int32_t* ref_of, const double* nIHC,
             const float* W, double Fs, double delta_alpha_len_factor, double* F_RA,
             double* F_AI, int mode) {
  std::vector<double> MR((size_t)3 * n_int * NS);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < n_int; ++i)
      for (int s = 0; s < NS; ++s) {
        const float* base = lam + (size_t)j * lam_stride * NS +
                            ((size_t)i * interval_nodes + head) * NS + s;
        double acc = base[0];
        for (int t = 1; t < len; ++t) acc = acc + base[(size_t)t * NS];
        if (mode == 0)
          MR[((size_t)j * n_int + i) * NS + s] = (double)((float)acc / (float)len);
        else
          MR[((size_t)j * n_int + i) * NS + s] = acc / (double)len;
      }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < n_int; ++i) {
      int r = ref_of[i];
      if (mode == 0) {
        float T = (float)(delta_alpha_len_factor / Fs);
        float Tl = (float)((double)(float)len / Fs);
        float dAf = (float)dA[i];
        float ai[NS], ra[NS];
        for (int s = 0; s < NS; ++s) {
          float mr = (float)MR[((size_t)j * n_int + i) * NS + s];
          float mrr = (float)MR[((size_t)j * n_int + r) * NS + s];
          float dMR = (mr - mrr) / dAf;
          const float* c = lam + (size_t)j * lam_stride * NS + ((size_t)i * interval_nodes + head) * NS + s;
          const float* rf = lam + (size_t)j * lam_stride * NS + ((size_t)r * interval_nodes + head) * NS + s;
          float acc = 0.0f;
          for (int t = 0; t < len; ++t) {
            float rl = rf[(size_t)t * NS], cl = c[(size_t)t * NS];
            float dl = dAf > 0 ? (cl - rl) / dAf : 0.0f;
            float pre = (float)((double)(dl * dl) / (Fs * (double)rl));
            acc += pre;
          }
          float rs = 1.0f / sqrtf(acc);
          ai[s] = (float)((double)(T / Tl) * nIHC[s] / (double)(rs * rs));
          float crlb = 1.0f / sqrtf(((T / mrr) * dMR) * dMR);
          ra[s] = (float)(nIHC[s] / (double)(crlb * crlb));
        }
        for (int t = NS / 2; t >= 1; t >>= 1)
          for (int s = 0; s < t; ++s) {
            ai[s] = ai[s] + ai[s + t];
            ra[s] = ra[s] + ra[s + t];
          }
        F_AI[(size_t)j * n_int + i] = (double)(ai[0] * W[j]);
        F_RA[(size_t)j * n_int + i] = (double)(ra[0] * W[j]);
      } else {
        double T = delta_alpha_len_factor / Fs;
        double Tl = (double)len / Fs;
        double dAd = dA[i];
        double sai = 0.0, sra = 0.0;
        for (int s = 0; s < NS; ++s) {
          double mr = MR[((size_t)j * n_int + i) * NS + s];
          double mrr = MR[((size_t)j * n_int + r) * NS + s];
          double dMR = (mr - mrr) / dAd;
          const float* c = lam + (size_t)j * lam_stride * NS + ((size_t)i * interval_nodes + head) * NS + s;
          const float* rf = lam + (size_t)j * lam_stride * NS + ((size_t)r * interval_nodes + head) * NS + s;
          double acc = 0.0;
          for (int t = 0; t < len; ++t) {
            double rl = rf[(size_t)t * NS], cl = c[(size_t)t * NS];
            double dl = dAd > 0 ? (cl - rl) / dAd : 0.0;
            acc += dl * dl / (Fs * rl);
          }
          sai += (T / Tl) * nIHC[s] * acc;
          sra += nIHC[s] * (T / mrr) * dMR * dMR;
        }
        F_AI[(size_t)j * n_int + i] = sai * (double)W[j];
        F_RA[(size_t)j * n_int + i] = sra * (double)W[j];
      }
    }
}

// Final JND in dB (src/AudioGramCreator.cpp:478-504, include/params.h:328-331).
double orc_jnd_db(double fisher_sum, double spl_ref, double max_db) {
  double pa = 1.0 / std::sqrt(fisher_sum);
  double max_pa = std::pow(10.0, max_db / 20.0) * spl_ref;
  if (std::isinf(pa) || pa > max_pa) return max_db;
  return 20.0 * std::log10(pa / spl_ref);
}

// ---------------------------------------------------------------------------
// Input generation (src/cochlea.cu:4070-4103): x[p][n] for n < interval_len.
// prof: double[n_prof][3] = dA, Wn, frequency.
// ---------------------------------------------------------------------------
void orc_input_gen(const double* prof, int n_prof, const float* wn, int interval_len,
                   int head, float Fs, double wn_dc, double wn_norm, double sig_norm,
                   float* out) {
  const float PIf = 3.141592653589793f;
  const float two_pi = 2 * PIf;
  for (int p = 0; p < n_prof; ++p) {
    double dA = prof[p * 3 + 0], Wn = prof[p * 3 + 1], f = prof[p * 3 + 2];
    for (int n = 0; n < interval_len; ++n) {
      double t = (double)(n - head) / (double)Fs;
      double cut = (double)two_pi * f * t;
      double sum = dA * std::cos(cut) / sig_norm;
      sum = sum + Wn * ((double)wn[n] - wn_dc) / wn_norm;
      out[(size_t)p * interval_len + n] = (float)sum;
    }
  }
}

}  // extern "C"
