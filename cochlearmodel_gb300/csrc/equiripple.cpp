// Equiripple low-pass FIR design for the AC filter: the Remez exchange
// algorithm of Parks and McClellan (IEEE Trans. Circuit Theory, 1972), in the
// form given by Oppenheim & Schafer (Discrete-Time Signal Processing, the
// Parks-McClellan algorithm section).  The reference designs its AC filter
// with firpm (vendored, src/firpm) through SubModel::calcFIRPM
// (src/SubModel.cpp:147-149: bands {0, wc, wc + tw, 1}, desired {1, 1, 0, 0},
// weights {wpass, wstop}) followed by fixDCGain; this file is an independent
// implementation of the same design problem.
//
// Linear-phase FIR of N taps:
//   N odd  (type I):  A(w) = sum_{k=0}^{L} a_k cos(k w),            L = (N-1)/2
//   N even (type II): A(w) = cos(w/2) sum_{k=0}^{L} b_k cos(k w),   L = N/2 - 1
// minimising max_w W(w) |D(w) - A(w)| over the pass band [0, wc] (D = 1,
// W = wpass) and the stop band [wc + tw, pi] (D = 0, W = wstop).  Each
// exchange solves for the r + 1 extremal frequencies (r = L + 1 cosine
// coefficients) the alternation equations by barycentric Lagrange
// interpolation in x = cos(w), evaluates the weighted error on a dense grid,
// and takes the next extremal set from its alternating local extrema.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cgb_internal.h"

namespace cgb {
namespace {

struct Grid {
  std::vector<double> w, D, W;  // frequency (0..pi), desired, weight (type-adjusted)
};

Grid make_grid(int r, double wc, double ws, double wpass, double wstop, bool type2) {
  const double pi = 3.14159265358979323846;
  const int density = 16;
  const double total = wc + (pi - ws);
  const int n = std::max(density * r, 64);
  Grid g;
  const int np = std::max(2, (int)std::lround(n * wc / total));
  const int ns = std::max(2, n - np);
  const double wend = type2 ? pi - 1e-6 : pi;  // type II has a zero at pi
  for (int i = 0; i < np; ++i) {
    const double w = wc * i / (np - 1);
    g.w.push_back(w);
    g.D.push_back(1.0);
    g.W.push_back(wpass);
  }
  for (int i = 0; i < ns; ++i) {
    const double w = ws + (wend - ws) * i / (ns - 1);
    g.w.push_back(w);
    g.D.push_back(0.0);
    g.W.push_back(wstop);
  }
  if (type2)
    for (size_t i = 0; i < g.w.size(); ++i) {
      const double c = std::cos(g.w[i] / 2);
      g.D[i] /= c;
      g.W[i] *= c;
    }
  return g;
}

// Barycentric weights of the nodes x[0..m-1] (scaled products avoid overflow).
std::vector<double> bary(const std::vector<double>& x) {
  const size_t m = x.size();
  std::vector<double> b(m, 1.0);
  for (size_t i = 0; i < m; ++i)
    for (size_t j = 0; j < m; ++j)
      if (j != i) b[i] *= 2.0 * (x[i] - x[j]);
  for (size_t i = 0; i < m; ++i) b[i] = 1.0 / b[i];
  return b;
}

}  // namespace
}  // namespace cgb

extern "C" int cgb_design_equiripple_lowpass(int num_taps, double omega_c, double transition,
                                             double weight_pass, double weight_stop,
                                             double* taps, double* delta_out, int* iterations) {
  using namespace cgb;
  const double pi = 3.14159265358979323846;
  if (!taps || num_taps < 3 || num_taps > 4096 || !(omega_c > 0) || !(transition > 0) ||
      omega_c + transition >= 1.0 || !(weight_pass > 0) || !(weight_stop > 0))
    return fail(CGB_ERR_ARG, "cgb_design_equiripple_lowpass: bad arguments");
  const bool type2 = (num_taps % 2) == 0;
  const int L = type2 ? num_taps / 2 - 1 : (num_taps - 1) / 2;
  const int r = L + 1;  // unknown cosine coefficients
  const double wc = omega_c * pi, ws = (omega_c + transition) * pi;
  const Grid g = make_grid(r, wc, ws, weight_pass, weight_stop, type2);
  const int G = (int)g.w.size();
  if (G < r + 2) return fail(CGB_ERR_ARG, "cgb_design_equiripple_lowpass: grid too coarse");
  std::vector<double> xg(G);
  for (int i = 0; i < G; ++i) xg[i] = std::cos(g.w[i]);
  // initial extremal set: r + 1 grid points spread evenly
  std::vector<int> ext(r + 1);
  for (int i = 0; i <= r; ++i) ext[i] = (int)std::lround((double)i * (G - 1) / r);
  std::vector<double> A(G), E(G);
  double delta = 0.0;
  int it = 0;
  for (; it < 100; ++it) {
    std::vector<double> x(r + 1);
    for (int i = 0; i <= r; ++i) x[i] = xg[ext[i]];
    const std::vector<double> b = bary(x);
    double num = 0.0, den = 0.0;
    for (int i = 0; i <= r; ++i) {
      num += b[i] * g.D[ext[i]];
      den += b[i] * ((i & 1) ? -1.0 : 1.0) / g.W[ext[i]];
    }
    delta = num / den;
    // interpolate A through the first r extremal points with values
    // c_i = D_i - (-1)^i delta / W_i
    std::vector<double> xr(x.begin(), x.begin() + r), c(r);
    for (int i = 0; i < r; ++i) c[i] = g.D[ext[i]] - ((i & 1) ? -1.0 : 1.0) * delta / g.W[ext[i]];
    const std::vector<double> br = bary(xr);
    for (int k = 0; k < G; ++k) {
      double sn = 0.0, sd = 0.0;
      int hit = -1;
      for (int i = 0; i < r; ++i) {
        const double d = xg[k] - xr[i];
        if (d == 0.0) {
          hit = i;
          break;
        }
        sn += br[i] * c[i] / d;
        sd += br[i] / d;
      }
      A[k] = hit >= 0 ? c[hit] : sn / sd;
      E[k] = g.W[k] * (g.D[k] - A[k]);
    }
    // local extrema of E within each band (band edges included: a missing
    // neighbour never wins), then enforce alternation of sign
    std::vector<int> cand;
    for (int k = 0; k < G; ++k) {
      const double e = E[k];
      if (e == 0.0) continue;
      const bool has_l = k > 0 && g.D[k - 1] == g.D[k];
      const bool has_r = k + 1 < G && g.D[k + 1] == g.D[k];
      const bool ok = e > 0 ? ((!has_l || e >= E[k - 1]) && (!has_r || e >= E[k + 1]))
                            : ((!has_l || e <= E[k - 1]) && (!has_r || e <= E[k + 1]));
      if (ok) cand.push_back(k);
    }
    std::vector<int> alt;
    for (int k : cand) {
      if (!alt.empty() && (E[alt.back()] > 0) == (E[k] > 0)) {
        if (std::fabs(E[k]) > std::fabs(E[alt.back()])) alt.back() = k;
      } else {
        alt.push_back(k);
      }
    }
    while ((int)alt.size() > r + 1) {
      if (std::fabs(E[alt.front()]) < std::fabs(E[alt.back()])) alt.erase(alt.begin());
      else alt.pop_back();
    }
    if ((int)alt.size() < r + 1) break;  // degenerate; keep the current solution
    double emax = 0.0;
    for (int k : alt) emax = std::max(emax, std::fabs(E[k]));
    const bool same = alt == ext;
    ext = alt;
    if (same || (emax - std::fabs(delta)) <= 1e-9 * std::fabs(delta)) {
      ++it;
      break;
    }
  }
  // cosine-series coefficients from A sampled at w_m = 2 pi m / (2L + 1)
  // (type I) -- the inverse DFT of the symmetric frequency response
  {
    std::vector<double> xr(r), c(r);
    std::vector<double> x(r + 1);
    for (int i = 0; i <= r; ++i) x[i] = xg[ext[i]];
    const std::vector<double> b = bary(x);
    double num = 0.0, den = 0.0;
    for (int i = 0; i <= r; ++i) {
      num += b[i] * g.D[ext[i]];
      den += b[i] * ((i & 1) ? -1.0 : 1.0) / g.W[ext[i]];
    }
    delta = num / den;
    for (int i = 0; i < r; ++i) {
      xr[i] = x[i];
      c[i] = g.D[ext[i]] - ((i & 1) ? -1.0 : 1.0) * delta / g.W[ext[i]];
    }
    const std::vector<double> br = bary(xr);
    auto evalA = [&](double w) {
      const double xx = std::cos(w);
      double sn = 0.0, sd = 0.0;
      for (int i = 0; i < r; ++i) {
        const double d = xx - xr[i];
        if (std::fabs(d) < 1e-15) return c[i];
        sn += br[i] * c[i] / d;
        sd += br[i] / d;
      }
      return sn / sd;
    };
    // P(w) = sum_{k=0}^{L} p_k cos(k w) from M = 2L + 1 samples
    const int M = 2 * L + 1;
    std::vector<double> P(M), p(L + 1);
    for (int m = 0; m < M; ++m) P[m] = evalA(2.0 * pi * m / M);
    for (int k = 0; k <= L; ++k) {
      double s = 0.0;
      for (int m = 0; m < M; ++m) s += P[m] * std::cos(2.0 * pi * k * m / M);
      p[k] = (k == 0 ? 1.0 : 2.0) * s / M;
    }
    if (!type2) {
      // h[L +- k] = p_k / 2 (k > 0), h[L] = p_0
      taps[L] = p[0];
      for (int k = 1; k <= L; ++k) taps[L - k] = taps[L + k] = p[k] / 2.0;
    } else {
      // cos(w/2) sum b_k cos(k w) = sum_{n} h[n] e^{-jw(n - (N-1)/2)}:
      //   h[N/2 - 1 - k] = h[N/2 + k] = (b_k + b_{k+1}) / 4 (k >= 1),
      //   h[N/2 - 1] = h[N/2] = (2 b_0 + b_1) / 4, b_{L+1} = 0
      const int h0 = num_taps / 2;
      for (int k = 0; k <= L; ++k) {
        const double bk = p[k], bk1 = k + 1 <= L ? p[k + 1] : 0.0;
        const double v = k == 0 ? (2.0 * bk + bk1) / 4.0 : (bk + bk1) / 4.0;
        taps[h0 - 1 - k] = taps[h0 + k] = v;
      }
    }
  }
  // unit DC gain (the reference's fixDCGain)
  double sum = 0.0;
  for (int i = 0; i < num_taps; ++i) sum += taps[i];
  for (int i = 0; i < num_taps; ++i) taps[i] /= sum;
  if (delta_out) *delta_out = std::fabs(delta);
  if (iterations) *iterations = it;
  return CGB_OK;
}
