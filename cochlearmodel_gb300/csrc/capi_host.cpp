// Host side of the C ABI: error reporting, model vectors, the block
// partition and unit-table validation.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "cgb_internal.h"

namespace cgb {

namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};
}  // namespace

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_check(int cuda_status, const char* what) {
  return fail(CGB_ERR_CUDA, std::string(what) + ": " +
                                cudaGetErrorString(static_cast<cudaError_t>(cuda_status)));
}

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int check_host_mirror(const void* p, const char* what) {
  if (reinterpret_cast<uintptr_t>(p) & 15)
    return fail(CGB_ERR_ARG, std::string(what) + ": the host mirror must be 16-byte aligned");
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(CGB_ERR_ARG, std::string(what) + ": the host mirror is not a known pointer");
  }
  if (at.type != cudaMemoryTypeHost || at.hostPointer != p || at.devicePointer != p)
    return fail(CGB_ERR_ARG, std::string(what) +
                                 ": the host mirror must be pinned host memory mapped at the "
                                 "same address on the device");
  return 0;
}

// Physical constants of the model as the reference's #defines produce them
// (include/const.h:216-297): each macro is a float expression evaluated left
// to right; CModel stores the result in a double (src/model.cpp:18-55).
struct PhysConsts {
  float pi = 3.141592653589793f;
  float w_ohc() const { return 2 * pi * 1000.0f; }                     // W_OHC
  float eta_1() const { return (1.0f) / (2e-6f) * 2 * pi * 1000.0f; }  // ETA_1
  float w_ow() const { return 2 * pi * 1500; }                         // W_OW
  float c_me() const {                                                 // C_ME
    return (2 * pi * 1340) * (2 * pi * 1340) * 0.059f / (0.49f * 1.4f);
  }
  float bc0() const { return ((2.0f * (1.0f) * (6e-3f)) / (0.5f)); }  // BC_0
  float bc1() const {                                                 // BC_1
    return ((0.5f) * (2 * pi * 1500 * 2 * pi * 1500) +
            (2 * pi * 1340) * (2 * pi * 1340) * 0.059f / (0.49f * 1.4f) * (21.4f));
  }
  float bc2() const { return (0.5f) * (20e3f); }  // BC_2
  float dx() const { return (3.5f) / 256; }        // COCHLEA_LEN / SECTIONS
};

}  // namespace cgb

extern "C" {

const char* cgb_last_error(void) { return cgb::g_last_error.c_str(); }

int cgb_abi_version(void) { return 4; }

int64_t cgb_kernel_launch_count(void) { return cgb::g_launches.load(); }

int cgb_model_setup(double* M, double* R, double* S, double* Q, double* S_ohc, double* S_tm,
                    double* R_tm, double* diag_m, double* diag_l, double* diag_u,
                    double* scal) {
  if (!M || !R || !S || !Q || !S_ohc || !S_tm || !R_tm || !diag_m || !diag_l || !diag_u || !scal)
    return cgb::fail(CGB_ERR_ARG, "cgb_model_setup: null pointer argument");
  const cgb::PhysConsts c;
  const double dx = c.dx();
  const double area = 0.5f, rho = 1.0f, beta = 0.003f;  // COCHLEA_AREA, LIQUID_RHO, BM_WIDTH
  const double w_ohc = c.w_ohc();
  const double ratio_K = 1e-3f;                          // RATIO_K
  // BM mass, resistance and stiffness: M0 e^{M1 dx i} etc. (src/model.cpp:72-86)
  for (int i = 0; i < CGB_SECTIONS; ++i) {
    const double xi = dx * i;
    M[i] = (double)1.286e-6f * std::exp((double)1.5f * xi);
    R[i] = (double)0.25f * std::exp((double)-0.06f * xi);
    S[i] = (double)1.282e4f * std::exp((double)-1.5f * xi);
    const double w_cf2 = S[i] / M[i];
    R_tm[i] = R[i];
    S_tm[i] = R[i] * w_cf2 / w_ohc;
    S_ohc[i] = ratio_K * S_tm[i];
    Q[i] = 2 * rho * beta / (area * M[i]);
  }
  // Pressure-system diagonals (src/solver.cpp:155-176).
  const double dx2 = dx * dx;
  for (int i = 0; i < CGB_SECTIONS; ++i) {
    diag_u[i] = 1.0;
    diag_l[i] = 1.0;
    diag_m[i] = -1.0 * (2.0 + dx2 * Q[i]);
  }
  diag_m[0] = -1.0 * (1.0 + dx * (double)c.bc0());
  diag_m[CGB_SECTIONS - 1] = 1.0;
  diag_l[CGB_SECTIONS - 1] = 0.0;
  diag_l[CGB_SECTIONS - 2] = 0.0;
  const double sv[16] = {w_ohc,          dx,          0.0f,     2e-6f,     1e-6f,   21.4f,
                         c.bc0(),        c.bc1(),     c.bc2(),  0.5f,      c.eta_1(), 0.0,
                         c.w_ow(),       c.c_me(),    ratio_K,  70e-3f};
  std::memcpy(scal, sv, sizeof(sv));
  return CGB_OK;
}

int cgb_pack_sections(const double* M, const double* diag_m, const double* R, const double* S,
                      const double* Q, const double* S_ohc, const double* S_tm,
                      const double* R_tm, float* secp) {
  if (!M || !diag_m || !R || !S || !Q || !S_ohc || !S_tm || !R_tm || !secp)
    return cgb::fail(CGB_ERR_ARG, "cgb_pack_sections: null pointer argument");
  for (int i = 0; i < CGB_SECTIONS; ++i) {
    // the host casts each vector to float (src/solver.cpp:357-376); the
    // kernel forms 1/M in float (include/cochlea.cuh:13725)
    const float mass = static_cast<float>(M[i]);
    secp[0 * CGB_SECTIONS + i] = 1.0f / mass;
    secp[1 * CGB_SECTIONS + i] = 1.0f / static_cast<float>(diag_m[i]);
    secp[2 * CGB_SECTIONS + i] = static_cast<float>(R[i]);
    secp[3 * CGB_SECTIONS + i] = static_cast<float>(S[i]);
    secp[4 * CGB_SECTIONS + i] = static_cast<float>(Q[i]);
    secp[5 * CGB_SECTIONS + i] = static_cast<float>(S_ohc[i]);
    secp[6 * CGB_SECTIONS + i] = static_cast<float>(S_tm[i]);
    secp[7 * CGB_SECTIONS + i] = static_cast<float>(R_tm[i]);
  }
  return CGB_OK;
}

int cgb_block_partition(int time_blocks, int64_t samples_p1, int overlap, int decouple,
                        int32_t* start, int32_t* out_first, int32_t* end) {
  if (time_blocks <= 0 || !start || !out_first || !end || overlap < 0 || decouple < 0)
    return cgb::fail(CGB_ERR_ARG, "cgb_block_partition: bad arguments");
  if (samples_p1 - overlap < time_blocks + 1)
    return cgb::fail(CGB_ERR_ARG, "cgb_block_partition: buffer shorter than one node per block");
  if (samples_p1 > INT32_MAX)
    return cgb::fail(CGB_ERR_RANGE, "cgb_block_partition: buffer longer than 2^31-1 samples");
  // N nodes per block; block b starts at b*N from zero state.  A block that
  // opens a decoupled group writes from its start; the others spend the
  // overlap as warm-up.  The last block of a group stops at (b+1)*N, the
  // others run an overlap past it (src/cochlea.cu:1148-1176).
  const int64_t N = (samples_p1 - overlap) / (time_blocks + 1);
  int64_t prev_end = 0;
  for (int b = 0; b < time_blocks; ++b) {
    const bool opens_group = decouple > 0 && (b % decouple == 0);
    const bool mid_transient = b > 0 && (decouple == 0 || (decouple != 1 && b % decouple != 0));
    const bool closes_group =
        decouple > 0 && (decouple == 1 || ((b + 1) % decouple == 0)) && b != time_blocks - 1;
    const int64_t s = b * N;
    const int warm = std::max(1 - (int)mid_transient - (int)opens_group, 0);
    int64_t first = s + (int64_t)warm * overlap;
    const int64_t e = s + N + (closes_group ? 0 : overlap);
    if (b > 0) first = std::max(first, prev_end);
    start[b] = (int32_t)s;
    out_first[b] = (int32_t)first;
    end[b] = (int32_t)e;
    prev_end = e;
  }
  return CGB_OK;
}

int cgb_check_units(const cgb_unit* units, int n_units, int n_profiles, int64_t in_len,
                    int64_t out_rows) {
  if (n_units < 0 || (n_units > 0 && !units))
    return cgb::fail(CGB_ERR_ARG, "cgb_check_units: bad unit table");
  for (int i = 0; i < n_units; ++i) {
    const cgb_unit& u = units[i];
    const bool ok = u.start >= 0 && u.end > u.start && u.out_first >= u.start &&
                    u.in_base >= 0 && u.in_base + u.end + 1 < in_len && u.out_base >= 0 &&
                    u.out_base + u.end <= out_rows && u.profile >= 0 &&
                    u.profile < n_profiles && u.mtt == u.mtt && u.mmspt == u.mmspt;
    if (!ok)
      return cgb::fail(CGB_ERR_RANGE, "cgb_check_units: unit " + std::to_string(i) +
                                          " reaches outside its buffers");
  }
  return CGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Complex-JND aggregation (ComplexJNDProfile::calculateMinValue and
// ::calculateGradientMinMaxValue, src/ComplexJNDProfile.cpp:19-100, run by
// AudioGramCreator::calcComplexJND, src/AudioGramCreator.cpp:548-571).  Each
// profile lists, per tested power level, the index of its interval among the
// calculated intervals; its JND values across the levels are reduced to one:
//   method 0: the last strict local minimum inside the sequence; with none,
//             the first value if it is below the second, else the last if it
//             is below the one before (warning 1);
//   method 1: the first value whose successor exceeds it by more than eps;
//             with none, the first value (warning 1).
// failed: per calculated interval, its failed-convergence count; out_failed
// receives the count of the chosen interval.  Where the reference reads
// outside its vectors (no minimum captured: an empty vector; one level: the
// second element) or leaves a stale value (no boundary below its neighbour),
// this returns the count at the chosen index, takes a single level as its
// own value (warning 1), and returns NaN (warning 1) respectively.
// ---------------------------------------------------------------------------
extern "C" int cgb_complex_jnd(const double* values, int n_values, const int32_t* failed,
                               const int32_t* intervals, int n_profiles, int n_levels,
                               int method, float eps, float* out_value, int32_t* out_warning,
                               int32_t* out_failed) {
  using namespace cgb;
  if (!values || !intervals || !out_value || !out_warning || !out_failed || n_values < 0 ||
      n_profiles < 0 || n_levels < 1 || (method != 0 && method != 1))
    return fail(CGB_ERR_ARG, "cgb_complex_jnd: bad arguments");
  std::vector<double> rel(n_levels);
  std::vector<int32_t> fl(n_levels);
  for (int p = 0; p < n_profiles; ++p) {
    for (int l = 0; l < n_levels; ++l) {
      const int idx = intervals[(size_t)p * n_levels + l];
      if (idx < 0 || idx >= n_values)
        return fail(CGB_ERR_RANGE, "cgb_complex_jnd: interval index outside the values");
      rel[l] = values[idx];
      fl[l] = failed ? failed[idx] : 0;
    }
    float value = NAN;
    int32_t warning = 0, fc = 0;
    if (method == 0) {
      int chosen = -1;
      for (int i = 1; i + 1 < n_levels; ++i)
        if (rel[i] < rel[i - 1] && rel[i] < rel[i + 1]) chosen = i;  // keeps the last
      if (chosen < 0) {
        warning = 1;
        if (n_levels == 1) chosen = 0;
        else if (rel[0] < rel[1]) chosen = 0;
        else if (rel[n_levels - 1] < rel[n_levels - 2]) chosen = n_levels - 1;
      }
      if (chosen >= 0) {
        value = (float)rel[chosen];
        fc = fl[chosen];
      }
    } else {
      int chosen = -1;
      for (int i = 0; i + 1 < n_levels; ++i)
        if (rel[i + 1] - rel[i] > (double)eps) {
          chosen = i;
          break;
        }
      if (chosen < 0) {
        chosen = 0;
        warning = 1;
      }
      value = (float)rel[chosen];
      fc = fl[chosen];
    }
    out_value[p] = value;
    out_warning[p] = warning;
    out_failed[p] = fc;
  }
  return CGB_OK;
}
