// CPU oracle of the learned Jacobi warm-start network -- TEST
// INFRASTRUCTURE ONLY.  It restates the network the GPU kernels train and
// run (cochlearmodel_gb300/csrc/warmstart.cuh, warmstart.cu) in FP64: four
// 1-D convolutions over the 256 sections, width 5, zero padding,
// 8 -> 64 -> 64 -> 64 -> 1 channels, ReLU between layers, MSE loss on
// s_out * output.  The reference has no learned component; the network is
// checked against this restatement (gradient check) and the restatement
// against finite differences.
//
// round_bf16 = 1 rounds at the points where the GPU path stores BF16
// (weights, hidden activations, dL/d(output), pre-activation gradients), so
// the two agree up to FP32-versus-FP64 accumulation; round_bf16 = 0 is the
// exact FP64 network (for finite differences).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int NS = 256, C = 64, K = 5;
constexpr int oW1 = 0, ob1 = oW1 + K * C * 8, oW2 = ob1 + C, ob2 = oW2 + K * C * C,
              oW3 = ob2 + C, ob3 = oW3 + K * C * C, oW4 = ob3 + C, ob4 = oW4 + K * C;
constexpr int kParams = ob4 + 1;

// FP32 -> BF16 -> FP32, round to nearest even (the bit-level method: add
// 0x7FFF plus the lowest kept bit, truncate).
double bf(double x, int on) {
  if (!on) return x;
  float f = (float)x;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  std::memcpy(&f, &u, 4);
  return (double)f;
}

// out[pos][co] = b[co] + sum_tap sum_ci W[tap][co][ci] in[pos+tap-2][ci]
void conv(const double* in, int cin, const double* W, const double* b, int cout, double* out) {
  for (int pos = 0; pos < NS; ++pos)
    for (int co = 0; co < cout; ++co) {
      double a = 0.0;
      for (int tap = 0; tap < K; ++tap) {
        const int ip = pos + tap - 2;
        if (ip < 0 || ip >= NS) continue;
        const double* w = W + (tap * cout + co) * cin;
        const double* x = in + ip * cin;
        for (int ci = 0; ci < cin; ++ci) a += w[ci] * x[ci];
      }
      out[pos * cout + co] = a + (b ? b[co] : 0.0);
    }
}

// din[pos][ci] = sum_tap sum_co W[tap][co][ci] d[pos-tap+2][co]
void conv_t(const double* d, int cout, const double* W, int cin, double* din) {
  for (int pos = 0; pos < NS; ++pos)
    for (int ci = 0; ci < cin; ++ci) {
      double a = 0.0;
      for (int tap = 0; tap < K; ++tap) {
        const int op = pos - tap + 2;
        if (op < 0 || op >= NS) continue;
        for (int co = 0; co < cout; ++co) a += W[(tap * cout + co) * cin + ci] * d[op * cout + co];
      }
      din[pos * cin + ci] = a;
    }
}

// gW[tap][co][ci] += sum_pos d[pos][co] in[pos+tap-2][ci]; gb[co] += sum_pos d[pos][co]
void wgrad(const double* d, int cout, const double* in, int cin, double* gW, double* gb) {
  for (int tap = 0; tap < K; ++tap)
    for (int co = 0; co < cout; ++co)
      for (int ci = 0; ci < cin; ++ci) {
        double a = 0.0;
        for (int pos = 0; pos < NS; ++pos) {
          const int ip = pos + tap - 2;
          if (ip < 0 || ip >= NS) continue;
          a += d[pos * cout + co] * in[ip * cin + ci];
        }
        gW[(tap * cout + co) * cin + ci] += a;
      }
  for (int co = 0; co < cout; ++co) {
    double a = 0.0;
    for (int pos = 0; pos < NS; ++pos) a += d[pos * cout + co];
    gb[co] += a;
  }
}

}  // namespace

extern "C" {

int orc_ws_param_count(void) { return kParams; }

// params float[kParams] (canonical layout W1[5][64][8], b1, W2[5][64][64],
// b2, W3, b3, W4[5][64], b4); feat float[n][256][8]; target float[n][256].
// Writes out[n][256] (network output o, before s_out), *loss = mean of
// (s_out o - target)^2, grad[kParams] (may be null).
void orc_ws_forward_backward(const float* params, const float* feat, const float* target, int n,
                             float s_out, int round_bf16, double* out, double* loss,
                             double* grad) {
  const int rb = round_bf16;
  std::vector<double> P(kParams);
  for (int i = 0; i < kParams; ++i) {
    const bool is_bias = (i >= ob1 && i < oW2) || (i >= ob2 && i < oW3) ||
                         (i >= ob3 && i < oW4) || i == ob4;
    P[i] = is_bias ? (double)params[i] : bf((double)params[i], rb);
  }
  std::vector<double> g(kParams, 0.0);
  std::vector<double> x(NS * 8), h1(NS * C), h2(NS * C), h3(NS * C), o(NS), d4(NS), d3(NS * C),
      d2(NS * C), d1(NS * C);
  double L = 0.0;
  const double s = (double)s_out;
  for (int r = 0; r < n; ++r) {
    for (int i = 0; i < NS * 8; ++i) x[i] = (double)feat[(int64_t)r * NS * 8 + i];
    conv(x.data(), 8, &P[oW1], &P[ob1], C, h1.data());
    for (auto& v : h1) v = bf(v > 0.0 ? v : 0.0, rb);
    conv(h1.data(), C, &P[oW2], &P[ob2], C, h2.data());
    for (auto& v : h2) v = bf(v > 0.0 ? v : 0.0, rb);
    conv(h2.data(), C, &P[oW3], &P[ob3], C, h3.data());
    for (auto& v : h3) v = bf(v > 0.0 ? v : 0.0, rb);
    conv(h3.data(), C, &P[oW4], &P[ob4], 1, o.data());
    for (int pos = 0; pos < NS; ++pos) {
      if (rb) o[pos] = (double)(float)o[pos];
      out[(int64_t)r * NS + pos] = o[pos];
      const double e = s * o[pos] - (double)target[(int64_t)r * NS + pos];
      L += e * e;
      d4[pos] = bf(2.0 * s * e / ((double)n * NS), rb);
    }
    if (!grad) continue;
    conv_t(d4.data(), 1, &P[oW4], C, d3.data());
    for (int i = 0; i < NS * C; ++i) d3[i] = bf(h3[i] > 0.0 ? d3[i] : 0.0, rb);
    conv_t(d3.data(), C, &P[oW3], C, d2.data());
    for (int i = 0; i < NS * C; ++i) d2[i] = bf(h2[i] > 0.0 ? d2[i] : 0.0, rb);
    conv_t(d2.data(), C, &P[oW2], C, d1.data());
    for (int i = 0; i < NS * C; ++i) d1[i] = bf(h1[i] > 0.0 ? d1[i] : 0.0, rb);
    wgrad(d4.data(), 1, h3.data(), C, &g[oW4], &g[ob4]);
    wgrad(d3.data(), C, h2.data(), C, &g[oW3], &g[ob3]);
    wgrad(d2.data(), C, h1.data(), C, &g[oW2], &g[ob2]);
    wgrad(d1.data(), C, x.data(), 8, &g[oW1], &g[ob1]);
  }
  *loss = L / ((double)n * NS);
  if (grad)
    for (int i = 0; i < kParams; ++i) grad[i] = g[i];
}

}  // extern "C"
