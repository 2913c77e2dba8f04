// Linux host harness for the reference-named API (include/cochlea_common.h).
//
// Replays the call order the reference's CSolver::Run_Cuda uses in profile
// mode (src/solver.cpp:234-962; AudioGramCreator::runInCuda/calcJND,
// src/AudioGramCreator.cpp:261-313, 829-974): model setup, profile grid,
// BMOHCKernel_Init, input generation on the GPU, BMOHCNewKernel, velocity
// copy-back, IHCNewKernel + RunIHCKernel, lambda copy-back, CudaCalculateJND
// and the final JND in dB.  Parameters come from a key = value file in the
// grammar of the reference's .par files (src/ConfigFileHandler.cpp:31-59).
//
// Outputs:
// - Output_File (this harness's container, little-endian): int64 header
//   {rows, lam_rows, n_intervals, n_ac}, float velocity[rows][256], float
//   lambda[3][lam_rows][256], float F_RA[3][n], float FisherAI[3][n], double
//   jnd_rate_db[n], double jnd_ai_db[n].
// - Output_Result and JND_File_Name (the reference's own keys): the raw
//   float32 files Run_Cuda writes through OutputBuffer<float>, in its
//   write_vector order, selected by Allowed_Outputs / Discard_* and
//   Calculate_JND_Types as the reference selects them.
//
// usage: run_cuda_harness <params.par>

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cochlea_common.h"
#include "cochlea_gb300.h"

class Log {};  // the caller's logger; the library never dereferences it

namespace {

std::map<std::string, std::string> parse_par(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::map<std::string, std::string> m;
  const std::regex kv("^\\s*([_[:alnum:]]+)\\s*=\\s*(\"(.*)\"|([^\"\\r\\n]+))$");
  std::string line;
  while (std::getline(f, line)) {
    std::smatch s;
    if (std::regex_match(line, s, kv)) m[s[1]] = s[3].matched ? s[3].str() : s[4].str();
  }
  return m;
}

std::vector<double> numbers(const std::string& v) {
  std::string t = v;
  for (char& c : t)
    if (c == ',' || c == '[' || c == ']' || c == ';') c = ' ';
  std::istringstream is(t);
  std::vector<double> out;
  double x;
  while (is >> x) out.push_back(x);
  return out;
}

struct Par {
  std::map<std::string, std::string> m;
  bool has(const std::string& k) const { return m.count(k) > 0; }
  double num(const std::string& k, double def) const {
    auto it = m.find(k);
    return it == m.end() ? def : std::stod(it->second);
  }
  std::vector<double> vec(const std::string& k, std::vector<double> def) const {
    auto it = m.find(k);
    return it == m.end() ? def : numbers(it->second);
  }
  std::string str(const std::string& k, const std::string& def) const {
    auto it = m.find(k);
    return it == m.end() ? def : it->second;
  }
};

// expandVectorToSize (include/cvector.cpp:609-623)
std::vector<float> expand(const std::vector<double>& v, size_t n) {
  std::vector<float> out;
  const size_t times = n / v.size(), rem = n % v.size();
  for (size_t i = 0; i < v.size(); ++i) {
    for (size_t k = 0; k < times; ++k) out.push_back((float)v[i]);
    if (i < rem) out.push_back((float)v[i]);
  }
  return out;
}

std::vector<float> read_f32(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::vector<char> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<float> v(b.size() / 4);
  std::memcpy(v.data(), b.data(), v.size() * 4);
  return v;
}

double spl2pa(double db, double ref) { return db == 1111.0 ? 0.0 : 10.0 * std::pow(10.0, db / 20.0) * ref; }

// The reference's binary output target: OutputBuffer<float> opened for
// writing (include/OutputBuffer.h:47-110) behind ConfigFileHandler::write_vector
// (src/ConfigFileHandler.cpp:124-131).  It holds raw float32 values with no
// header, appended in the order of the write_vector calls; values of other
// types are cast to float first (castVector).
class RawTarget {
 public:
  explicit RawTarget(const std::string& path) : f_(path, std::ios::binary | std::ios::trunc) {
    if (!f_) throw std::runtime_error("cannot open Target file " + path);
  }
  template <class T>
  void append(const T* src, size_t length) {
    std::vector<float> buf(length);
    for (size_t i = 0; i < length; ++i) buf[i] = (float)src[i];
    f_.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)(length * 4));
  }

 private:
  std::ofstream f_;
};

// transposeVector(v, column_size) (include/cvector.cpp:520-530)
std::vector<float> transpose(const std::vector<float>& v, size_t column_size) {
  std::vector<float> out(v.size());
  const size_t row_size = v.size() / column_size;
  for (size_t i = 0; i < v.size(); ++i) out[(i % row_size) * column_size + i / row_size] = v[i];
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <params.par>\n", argv[0]);
    return 2;
  }
  try {
    Par P{parse_par(argv[1])};
    Log log;
    const long Fs = (long)P.num("Fs", 100000);
    const float tbl = (float)P.num("Time_Block_Length", 0.01);
    const int D = (int)P.num("Decouple_Filter", 1);
    const double ov_time = P.num("Overlap_Time", 0.005);
    const double spl_ref = P.num("SPLRef", 2e-5);
    const bool calc_jnd = P.num("Calculate_JND", 0) != 0;
    const auto freqs = P.vec("testedFrequencies", {1000.0});
    const auto powers = P.vec("testedPowerLevels", {60.0});
    const auto noises = P.vec("testedNoises", {1111.0});
    const auto ohc = expand(P.vec("OHC_Vector", {0.5}), 256);
    const auto ihcv = expand(P.vec("IHC_Vector", {8.0}), 256);

    // node counts (include/params.h:288-395)
    const long ov_us = (long)(std::round(ov_time * 1000) * 1000);
    const int overlap = (int)(ov_us * Fs / 1000000);
    const int N = (int)std::ceil((float)Fs * tbl);
    const int L = N * D;

    // profile grid (src/params.cpp:661-782), one reference per noise level
    std::vector<device_jnd_params> prof;
    std::vector<int> ref_pos;
    for (double nl : noises) {
      const double wn = spl2pa(nl, spl_ref);
      for (double pl : powers)
        for (double f : freqs) {
          device_jnd_params p{};
          p.dBSPLSignal = pl;
          p.dBSPLNoise = nl != 1111.0 ? nl : 0.0;
          p.dA = spl2pa(pl, spl_ref);
          p.recipdA = p.dA > 0 ? 1.0 / p.dA : 0.0;
          p.Wn = wn;
          p.frequency = f;
          p.calculateIndexPosition = (int)prof.size();
          prof.push_back(p);
        }
      if (calc_jnd) {
        device_jnd_params p{};
        p.dBSPLNoise = nl != 1111.0 ? nl : 0.0;
        p.Wn = wn;
        p.isReference = true;
        p.referenceIndex = (int)prof.size();
        p.calculateIndexPosition = -1;
        ref_pos.push_back((int)prof.size());
        prof.push_back(p);
      }
    }
    const int n_int = (int)prof.size();
    const int TB = n_int * D;
    const int64_t samples_p1 = (int64_t)overlap + (int64_t)N * (TB + 1);
    const int64_t total_nodes = (int64_t)overlap + (int64_t)N * TB;

    // model (src/solver.cpp:357-376)
    double M[256], R[256], S[256], Q[256], So[256], St[256], Rt[256], dm[256], dl[256], du[256],
        sc[16];
    if (cgb_model_setup(M, R, S, Q, So, St, Rt, dm, dl, du, sc) != CGB_OK)
      throw std::runtime_error(cgb_last_error());
    std::vector<float> gamma(ohc), mass(256), rsm(256), uu(256), ll(256), Rf(256), Sf(256),
        Qf(256), Sof(256), Stf(256), Rtf(256);
    for (int i = 0; i < 256; ++i) {
      mass[i] = (float)M[i];
      rsm[i] = 1.0f / (float)dm[i];
      uu[i] = (float)du[i];
      ll[i] = (float)dl[i];
      Rf[i] = (float)R[i];
      Sf[i] = (float)S[i];
      Qf[i] = (float)Q[i];
      Sof[i] = (float)So[i];
      Stf[i] = (float)St[i];
      Rtf[i] = (float)Rt[i];
    }
    BMOHCKernel_Init(gamma.data(), mass.data(), rsm.data(), uu.data(), ll.data(), Rf.data(),
                     Sf.data(), Qf.data(), Sof.data(), Stf.data(), Rtf.data(), 1.0f, 0.0f,
                     (size_t)samples_p1 + 4, (size_t)(samples_p1 + 4) * 256, 0, true, 0, 0, log);

    // input generation on the GPU
    std::vector<float> noise(L, 0.0f);
    const std::string nf = P.str("Input_Noise_File", "");
    if (!nf.empty()) {
      auto v = read_f32(nf);
      for (int i = 0; i < L && i < (int)v.size(); ++i) noise[i] = v[i];
    }
    std::vector<float> signal(L, 0.0f);
    // hearing-aid transfer functions (src/params.cpp:1401-1413: the IIR vector
    // is stored negated with element 0 = 1)
    std::vector<float> ha_fir(1, 1.0f), ha_iir(1, 1.0f);
    {
      const auto fv = P.vec("Hearing_AID_FIR_Transfer_Function", {});
      if (!fv.empty()) ha_fir.assign(fv.begin(), fv.end());
      const auto iv = P.vec("Hearing_AID_IIR_Transfer_Function", {});
      if (!iv.empty()) {
        ha_iir.assign(iv.size(), 0.0f);
        for (size_t i = 0; i < iv.size(); ++i) ha_iir[i] = -1.0f * (float)iv[i];
        ha_iir[0] = 1.0f;
      }
    }
    InputProfilesArrayInitialization(n_int, L, L, 0, 0);
    generateInputFromProfile(prof.data(), noise.data(), L, signal.data(), L, 0,
                             (int)P.num("Normalize_Sigma_Type", 3),
                             (int)P.num("Normalize_Sigma_Type_Signal", 3), 0.16, 0.0, 0, 0, 0, 0,
                             n_int, false, 0, n_int, overlap, L, 0, L, (float)Fs, 0, nullptr,
                             false, true, (float)P.num("MAX_M1_SP_ERROR", 1e-15),
                             (float)P.num("MAX_TOLERANCE", 1e-10),
                             (int)P.num("RELATIVE_ERRORS", 0),
                             (float)P.num("M1_SP_Fix_Factor", 0.0),
                             (float)P.num("Tolerance_Fix_Factor", 0.0), D, 0,
                             ha_fir.data(), (int)ha_fir.size(), ha_iir.data(),
                             (int)ha_iir.size(), log);

    // BM solver
    cudaEvent_t e0{}, e1{};
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, 0);
    const float time_step = 1e-6f;
    const int iters = (int)(1.0f / ((float)Fs * 1e-6f));
    const float time_step_out = time_step * (float)iters;
    float tres = 0.0f;
    BMOHCNewKernel(nullptr, true, (float)sc[0], time_step, time_step_out, (float)sc[1],
                   (float)sc[2], 1, 1, 0, (float)(1.0 / (double)Fs), (float)sc[3], (float)sc[4],
                   (float)sc[5], (float)sc[6], (float)sc[7], (float)sc[8], (float)sc[9],
                   (float)sc[10], (float)sc[11], &tres, TB, (int)samples_p1, overlap, ov_us, 1,
                   1e-6f, 1e-18f, D, (float)P.num("MAX_M1_SP_ERROR", 1e-15),
                   (float)P.num("MAX_TOLERANCE", 1e-10), (int)P.num("RELATIVE_ERRORS", 0), 0,
                   (float)P.num("M1_SP_Fix_Factor", 0.0),
                   (float)P.num("Tolerance_Fix_Factor", 0.0), (float)spl_ref, 0, 0,
                   0, (int)P.num("JACOBBY_Loops_Fast", 2), (int)P.num("JACOBBY_Loops_Slow", 20),
                   (int)P.num("Cuda_Outern_Loops", 10),
                   // kernel selection and cache hint, with the reference's
                   // defaults (src/params.cpp:157,188)
                   (int)P.num("Run_Fast_BM_Calculation", 0),
                   (int)P.num("BMOHC_Kernel_Configuration", 2), e0, e1, prop, log);
    std::vector<float> v((size_t)total_nodes * 256);
    BMOHCKernel_Copy_Results(v.data(), v.size(), 0);

    // IHC + lambda (AudioGramCreator::runInCuda)
    const auto ac = read_f32(P.str("AC_Filter_File", ""));
    std::vector<double> acd(ac.begin(), ac.end());
    // AC_Filter_A_File (raw float32 a coefficients, a[0] = 1) makes the AC
    // filter an IIR of the same length (is_ac_iir_filter)
    const std::string a_file = P.str("AC_Filter_A_File", "");
    const bool ac_iir = !a_file.empty();
    std::vector<double> acd_a = acd;
    if (ac_iir) {
      const auto aa = read_f32(a_file);
      if (aa.size() != ac.size()) throw std::runtime_error("AC_Filter_A_File length != AC_Filter_File");
      acd_a.assign(aa.begin(), aa.end());
    }
    const int dc_n = (int)std::round((float)Fs * 2e-3f);
    std::vector<double> dcd(dc_n, (double)(1.0f / ((float)Fs * 2e-3f)));
    std::vector<double> dmg(256);
    for (int i = 0; i < 256; ++i) dmg[i] = std::pow(10.0, (double)ihcv[i]);
    std::vector<float> aihc = expand({70.0, 50.0, 30.0}, 768);
    float clusters[9] = {60.0f, 3.0f, 0.1f, 70.0f, 50.0f, 30.0f, 0.61f, 0.23f, 0.16f};
    const int write_time = (int)total_nodes;
    const int calc_time = (write_time + 63) / 64 * 64;
    enableloadAihc();
    loadAihc(aihc.data());
    IHCNewKernel(dmg.data(), clusters, dcd.data(), dc_n, acd.data(), acd_a.data(), ac_iir,
                 (int)acd.size(), 256, TB, spl_ref, nullptr, 0, calc_time, write_time,
                 (int)(samples_p1 + 4), N, 0, 0, 500.0f, 1.0f, 100.0f, true, true, false, true,
                 false, false, 1.0f, calc_jnd, n_int, overlap, D, 0, log);
    allocateBuffer(LAMBDA_COUNT * calc_time * 256, 0, e0, e1, prop);
    // harness-only test key (not a reference key): make the IHC kernel's
    // staging wait run out, to exercise the drop-in's error path
    if (P.num("Test_Fault_IHC_Staging", 0) != 0) cgb_ihc_set_fault_injection(1);
    // the reference's test output (TEST_File_Target + Type_TEST_Output,
    // default MeanRate; src/AudioGramCreator.cpp:877-892,913-970, stage
    // names src/params.cpp:165-187), written as raw floats, the first run of
    // a set truncating the file:
    //  - an IHC stage, RunIHCKernel's backup of AC (9), DC (10), dS (11),
    //    Shigh (12, dS as well), IHC (13) or PRE_IHC (14): write_time x 256;
    //  - MeanRate, the JND's mean rates [3][intervals][256] (getCudaMeanRate);
    //  - JND_Lambda, the three lambda planes (3 x calc_time x 256), or
    //    JND_Lambda(k) plane k alone (calc_time x 256);
    //  - the JND's debug stages, passed to CudaCalculateJND as backup_stage
    //    and read from getCudaBuffer: AvgMeanRate (1, 3 x intervals),
    //    dMeanRate (2) and CRLB_RA (6) and preFisherAITimeReduced (5)
    //    [3][intervals][256], dLambda (3) and preFisherAI (4) 3 x calc_time x
    //    256, dLambda(k) plane k.  (The reference writes a stage buffer for
    //    dMeanRate, dLambda and CRLB_RA; for 1, 4 and 5 it writes the buffer it
    //    last filled, so these files are this build's.)
    const std::string test_target = P.str("TEST_File_Target", "");
    const std::string test_type = P.str("Type_TEST_Output", "MeanRate");
    int backup_stage = -1;
    const bool test_mean_rate = !test_target.empty() && test_type == "MeanRate";
    int test_lambda = -2;  // -1: all planes, 0..: one plane
    int jnd_stage = -1, jnd_plane = -1;
    std::smatch lam_m;
    {
      const char* jnames[] = {"AvgMeanRate", "dMeanRate", "dLambda", "preFisherAI",
                              "preFisherAITimeReduced", "CRLB_RA"};
      for (int k = 0; k < 6; ++k)
        if (!test_target.empty() && test_type == jnames[k]) jnd_stage = 1 + k;
      if (!test_target.empty() &&
          std::regex_match(test_type, lam_m, std::regex("dLambda\\(([[:digit:]])\\)"))) {
        jnd_stage = 3;
        jnd_plane = std::stoi(lam_m[1]);
        if (jnd_plane >= LAMBDA_COUNT)
          throw std::runtime_error("index of lambda must be smaller than 3, you chose " +
                                   lam_m[1].str());
      }
      if (jnd_stage > 0 && !calc_jnd)
        throw std::runtime_error("Type_TEST_Output " + test_type + " needs Calculate_JND");
    }
    if (!test_target.empty() && test_type == "JND_Lambda") test_lambda = -1;
    if (!test_target.empty() &&
        std::regex_match(test_type, lam_m, std::regex("JND_Lambda\\(([[:digit:]])\\)"))) {
      test_lambda = std::stoi(lam_m[1]);
      if (test_lambda >= LAMBDA_COUNT)
        throw std::runtime_error("index of lambda must be smaller than 3, you chose " +
                                 lam_m[1].str());
    }
    if (!test_target.empty() && !test_mean_rate && test_lambda == -2 && jnd_stage < 0) {
      const char* names[] = {"AC", "DC", "dS", "Shigh", "IHC", "PRE_IHC"};
      for (int k = 0; k < 6; ++k)
        if (test_type == names[k]) backup_stage = 9 + k;
      if (backup_stage < 0)
        throw std::runtime_error("Type_TEST_Output " + test_type +
                                 " is not served");
    }
    if (test_mean_rate && !calc_jnd)
      throw std::runtime_error("Type_TEST_Output MeanRate needs Calculate_JND");
    std::vector<float> backup(backup_stage > 0 ? (size_t)calc_time * 256 : 0);
    RunIHCKernel(backup_stage > 0 ? backup.data() : nullptr, 0, 1, backup_stage, 0, log);
    if (backup_stage > 0) {
      FILE* tf = std::fopen(test_target.c_str(), "wb");
      if (!tf) throw std::runtime_error("cannot open TEST_File_Target " + test_target);
      const size_t n = (size_t)write_time * 256;
      const bool ok = std::fwrite(backup.data(), sizeof(float), n, tf) == n;
      std::fclose(tf);
      if (!ok) throw std::runtime_error("short write to TEST_File_Target " + test_target);
    }
    std::vector<float> lam((size_t)LAMBDA_COUNT * calc_time * 256);
    BMOHCKernel_Copy_Lambda(lam.data(), lam.size(), 0);
    if (test_lambda != -2) {
      const size_t plane = (size_t)calc_time * 256;
      const float* src = lam.data() + (test_lambda < 0 ? 0 : (size_t)test_lambda * plane);
      const size_t n = test_lambda < 0 ? (size_t)LAMBDA_COUNT * plane : plane;
      FILE* tf = std::fopen(test_target.c_str(), "wb");
      if (!tf) throw std::runtime_error("cannot open TEST_File_Target " + test_target);
      const bool ok = std::fwrite(src, sizeof(float), n, tf) == n;
      std::fclose(tf);
      if (!ok) throw std::runtime_error("short write to TEST_File_Target " + test_target);
    }
    const int lam_rows = N * TB;

    // JND (AudioGramCreator::calcJND / calcJNDFinal)
    std::vector<float> FRA(3 * n_int, 0.0f), FAI(3 * n_int, 0.0f);
    std::vector<double> jr(n_int, NAN), ja(n_int, NAN);
    std::vector<int> serial(n_int), calc_pos, to_ref;
    if (calc_jnd) {
      const int head = (int)std::round((float)Fs * (float)P.num("JND_Interval_Head", 0.014));
      const int tail = (int)std::round((float)Fs * (float)P.num("JND_Interval_Tail", 0.002));
      const int len = L - head - tail;
      int ci = 0;
      for (int i = 0; i < n_int; ++i) {
        const int rr = i * (int)ref_pos.size() / n_int;
        bool isref = false;
        for (int r : ref_pos) isref |= r == i;
        if (!isref) {
          serial[i] = ci++;
          calc_pos.push_back(i);
          to_ref.push_back(ref_pos[rr]);
        } else {
          serial[i] = rr;
        }
      }
      std::vector<double> nihc(256, (double)(30000.0f / 256.0f));
      CudaCalculateJND(true, true, n_int * 3 * 256, 3 * n_int, spl_ref, (double)Fs, 1.0,
                       nihc.data(), calc_pos.data(), (int)calc_pos.size(), ref_pos.data(),
                       (int)ref_pos.size(), 0, n_int, n_int, head, overlap, L, len,
                       serial.data(), to_ref.data(), FRA.data(), FAI.data(), write_time * 256,
                       calc_time * 256, 0.2 * (double)Fs, 1, 0, false, false,
                       jnd_stage > 0 ? jnd_stage : backup_stage, log);
      for (int i = 0; i < n_int; ++i) {
        bool isref = false;
        for (int r : ref_pos) isref |= r == i;
        if (isref) continue;
        double ra = 0, ai = 0;
        for (int j = 0; j < 3; ++j) {
          ra += FRA[j * n_int + i];
          ai += FAI[j * n_int + i];
        }
        const double max_pa = std::pow(10.0, 150.0 / 20.0) * spl_ref;
        auto db = [&](double s) {
          const double pa = 1.0 / std::sqrt(s);
          return (std::isinf(pa) || pa > max_pa) ? 150.0 : 20.0 * std::log10(pa / spl_ref);
        };
        jr[i] = db(ra);
        ja[i] = db(ai);
      }
      if (jnd_stage > 0) {
        const size_t plane = (size_t)calc_time * 256, mean = (size_t)3 * n_int * 256;
        size_t n = mean, off = 0;
        if (jnd_stage == 1) n = (size_t)3 * n_int;
        if (jnd_stage == 3 || jnd_stage == 4) n = 3 * plane;
        if (jnd_plane >= 0) {
          n = plane;
          off = (size_t)jnd_plane * plane;
        }
        std::vector<float> st(n);
        GeneralKernel_Copy_Results_Template<float>(st.data(), getCudaBuffer(), n, off);
        FILE* tf = std::fopen(test_target.c_str(), "wb");
        if (!tf) throw std::runtime_error("cannot open TEST_File_Target " + test_target);
        const bool ok = std::fwrite(st.data(), sizeof(float), n, tf) == n;
        std::fclose(tf);
        if (!ok) throw std::runtime_error("short write to TEST_File_Target " + test_target);
      }
      if (test_mean_rate) {
        const size_t n = (size_t)3 * n_int * 256;  // getMeanNodes()
        std::vector<float> mr(n);
        GeneralKernel_Copy_Results_Template<float>(mr.data(), getCudaMeanRate(), n);
        FILE* tf = std::fopen(test_target.c_str(), "wb");
        if (!tf) throw std::runtime_error("cannot open TEST_File_Target " + test_target);
        const bool ok = std::fwrite(mr.data(), sizeof(float), n, tf) == n;
        std::fclose(tf);
        if (!ok) throw std::runtime_error("short write to TEST_File_Target " + test_target);
      }
    }

    // The reference's own output files, written when the .par names them.
    // One Run_Cuda pass in profile mode (src/solver.cpp:704-830,
    // AudioGramCreator::saveLambdas src/AudioGramCreator.cpp:202-212): the
    // transient is shown (Decouple_Filter > 0 requires it) and its tail removed
    // (Remove_Transient_Tail = 1 for generated profiles), so every stream
    // starts at node 0 and holds writeTime - overlap = N * Time_Blocks nodes.
    // write_vector calls whose name has no registered target go to the
    // Output_Result file (VirtualHandler::write_vector, include/VirtualHandler.h:
    // 156-173); jnd_ai and jnd_rms are registered to the raw JND file
    // (src/params.cpp:1636-1646).
    const std::string out_result = P.str("Output_Result", "");
    const std::string jnd_file = P.str("JND_File_Name", "");
    if (!out_result.empty() || (calc_jnd && !jnd_file.empty())) {
      // Allowed_Outputs (src/params.cpp:820-832): bit 0 velocity, bits 1-3 the
      // lambdas; the Discard_* keys set them unless Allowed_Outputs is given
      unsigned allowed = 0;
      if (P.has("Discard_BM_Velocity_Output") && P.num("Discard_BM_Velocity_Output", 0) != 1)
        allowed |= 1u;
      if (P.has("Discard_Lambdas_Output") && P.num("Discard_Lambdas_Output", 0) != 1)
        allowed |= 14u;
      if (P.has("Allowed_Outputs")) allowed = (unsigned)P.num("Allowed_Outputs", 0);
      const unsigned jnd_types = P.has("Calculate_JND_Types")
                                     ? (unsigned)P.num("Calculate_JND_Types", 0)
                                     : (1u << 16) - 1;
      const bool jnd_rms = (jnd_types & 1u) != 0, jnd_ai = (jnd_types & 2u) != 0;
      const size_t nodes = (size_t)N * TB;  // writeTime - overlap
      std::vector<int> failed_nodes((size_t)total_nodes), failed_blocks(TB);
      GeneralKernel_Copy_Results_Template<int>(failed_nodes.data(), getCudaFailedTimeNodes(),
                                               (size_t)total_nodes);
      GeneralKernel_Copy_Results_Template<int>(failed_blocks.data(), getCudaFailedBlocks(),
                                               (size_t)TB);
      std::unique_ptr<RawTarget> main_out;
      if (!out_result.empty()) main_out.reset(new RawTarget(out_result));
      if (main_out) {
        main_out->append(failed_nodes.data(), nodes);
        main_out->append(failed_blocks.data(), (size_t)TB);
        if (allowed & 1u) main_out->append(v.data(), nodes * 256);
        for (int j = 0; j < LAMBDA_COUNT; ++j)
          if (allowed & (2u << j))
            main_out->append(lam.data() + (size_t)j * calc_time * 256, nodes * 256);
      }
      if (calc_jnd) {
        // calcJNDFinal (src/AudioGramCreator.cpp:454-508): per tested
        // interval, its blocks' failed samples and the bounded JND in dB
        const size_t n_calc = calc_pos.size();
        std::vector<float> failed_signals(n_calc, 0.0f), ai(n_calc), rate(n_calc);
        for (size_t k = 0; k < n_calc; ++k) {
          const int i = calc_pos[k];
          for (int b = 0; b < D; ++b) failed_signals[k] += (float)failed_blocks[(size_t)i * D + b];
          ai[k] = (float)ja[i];
          rate[k] = (float)jr[i];
        }
        // column layout of the raw JND vectors (src/solver.cpp:763-767), for
        // generated tones (JND_Signal_Source 0)
        const size_t n_pow = powers.size(), n_freq = freqs.size();
        const size_t rms_m = n_calc / (n_pow * n_freq);
        const size_t mcols = rms_m * n_pow;
        std::unique_ptr<RawTarget> raw;
        if (!jnd_file.empty()) raw.reset(new RawTarget(jnd_file));
        if (main_out) main_out->append(failed_signals.data(), n_calc);
        if (jnd_ai) {
          if (main_out) main_out->append(ai.data(), n_calc);  // jnd_ai_power
          if (raw) raw->append(transpose(ai, mcols).data(), n_calc);
        }
        if (jnd_rms) {
          if (main_out) main_out->append(rate.data(), n_calc);  // jnd_rms_power
          if (raw) raw->append(transpose(rate, mcols).data(), n_calc);
        }
      }
    }

    std::ofstream out(P.str("Output_File", "harness_out.bin"), std::ios::binary);
    const int64_t hdr[4] = {total_nodes, lam_rows, n_int, (int64_t)acd.size()};
    out.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    out.write(reinterpret_cast<const char*>(v.data()), v.size() * 4);
    for (int j = 0; j < 3; ++j)
      out.write(reinterpret_cast<const char*>(lam.data() + (size_t)j * calc_time * 256),
                (size_t)lam_rows * 256 * 4);
    out.write(reinterpret_cast<const char*>(FRA.data()), FRA.size() * 4);
    out.write(reinterpret_cast<const char*>(FAI.data()), FAI.size() * 4);
    out.write(reinterpret_cast<const char*>(jr.data()), jr.size() * 8);
    out.write(reinterpret_cast<const char*>(ja.data()), ja.size() * 8);
    IHCKernel_Free();
    BMOHCKernel_Free();
    InputProfilesArrayTermination();
    std::printf("harness ok: %lld rows, %d intervals\n", (long long)total_nodes, n_int);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "harness failed: %s\n", e.what());
    return 1;
  }
  return 0;
}
