// Test infrastructure: a shim that exposes pieces of the REFERENCE's own
// source, compiled from its files (include/const.h, src/tridiag.cpp), so the
// oracle's restatement can be checked against them.  Built by
// oracle/build_ref.sh into oracle/_ref/ where the reference tree is present.

#include <cmath>
#include <vector>

#include "const.h"    // the reference's constants header
#include "tridiag.h"  // the reference's tridiagonal solver (src/tridiag.cpp)

extern "C" {

// The reference's #define expressions, evaluated by the compiler exactly as
// CModel's initialiser list receives them (src/model.cpp:18-55).
void ref_consts(double* out) {
  out[0] = W_OHC;
  out[1] = COCHLEA_LEN / SECTIONS;
  out[2] = BM_ALPHA_R;
  out[3] = ALPHA_L;
  out[4] = ALPHA_S;
  out[5] = G_ME;
  out[6] = BC_0;
  out[7] = BC_1;
  out[8] = BC_2;
  out[9] = SIGMA_OW;
  out[10] = ETA_1;
  out[11] = ETA_2;
  out[12] = W_OW;
  out[13] = C_ME;
  out[14] = RATIO_K;
  out[15] = OHC_PSI_0;
  out[16] = M0;
  out[17] = M1;
  out[18] = R0;
  out[19] = R1;
  out[20] = S0;
  out[21] = S1Cochlear;
  out[22] = COCHLEA_AREA;
  out[23] = LIQUID_RHO;
  out[24] = BM_WIDTH;
  out[25] = CUDA_MAX_TIME_STEP;
  out[26] = CUDA_MIN_TIME_STEP;
  out[27] = MAX_M1_SP_ERROR;
  out[28] = MAX_TOLERANCE;
  out[29] = _CUDA_JACOBBY_LOOPS1;
  out[30] = _CUDA_JACOBBY_LOOPS2;
  out[31] = _CUDA_OUTERN_LOOPS;
  out[32] = CUDA_AUX_TM_LOOPS;
  out[33] = SPLRef;
  out[34] = RSAT;
  out[35] = AMP_AC;
  out[36] = AMP_DC;
  out[37] = Tdc;
  out[38] = SPONT_HIGH_RATE;
  out[39] = SPONT_MEDIUM_RATE;
  out[40] = SPONT_LOW_RATE;
  out[41] = HIGH_FREQ_NERVE;
  out[42] = MEDIUM_FREQ_NERVE;
  out[43] = LOW_FREQ_NERVE;
  out[44] = FIBER_HIGH_DIST;
  out[45] = FIBER_MEDIUM_DIST;
  out[46] = FIBER_LOW_DIST;
  out[47] = AN_FIBERS;
  out[48] = SECTIONS;
  out[49] = EPS;
}

// CTriDiag::SolveFor on the given diagonals (src/tridiag.cpp:67-106).
void ref_thomas(const double* m, const double* l, const double* u, const double* v,
                double* res, int n) {
  CTriDiag t(n);
  t.SetLowerDiag(std::vector<double>(l, l + n));
  t.SetUpperDiag(std::vector<double>(u, u + n));
  t.SetMidDiag(std::vector<double>(m, m + n));
  std::vector<double> r = t.SolveFor(std::vector<double>(v, v + n));
  for (int i = 0; i < n; ++i) res[i] = r[i];
}

}  // extern "C"
