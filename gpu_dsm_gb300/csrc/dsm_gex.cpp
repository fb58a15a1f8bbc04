// Background molecular-weight distribution of a polydisperse melt (the
// reference's PD_flag = 1, polydisp.dat "a b mp Mk"; common/gamma.cpp:174-263,
// common/main_cuda.cu:95-103).  The generalised exponential (GEX) law
// W(m) ~ m^a exp(-m^b) of m = M/mp has the cumulative number fraction of
// chain mass P(m) = P_gamma((a+1)/b, m^b).  Two inverse tables, equidistant
// in probability, give the mass of the partner chain of a new entanglement:
//   M[j]:  P(M[j]) = j * step          (partner of an SD-created entanglement
//                                       and of the initial ones)
//   Md[j]: the same law weighted by the partner's mean CD destruction rate
//          normdt(N_K) (partner of a CD-created entanglement)
// and the CD creation prefactor is step * sum_j normdt(N_K(M[j])) / beta
// (common/ensemble.cu:137-146).  Published algorithms restated here: the
// regularised incomplete gamma function by its series and its continued
// fraction (modified Lentz), as in Press et al., Numerical Recipes 6.2; the
// lower branch W_-1 of Lambert's function by Halley's iteration from the
// branch-point series (K. Briggs).  Arithmetic is float where the reference
// tabulates in float, so the tables agree with it to float rounding.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/dsm.h"
#include "dsm_host.h"

namespace dsm {
namespace {

constexpr int kItMax = 300;
constexpr float kEps = 3.0e-7f;
constexpr float kFpMin = 1.0e-30f;
constexpr int kGrid = 1000000;  // points of the forward table in m

// P(a, x) by its series, x < a + 1
float gamma_series(float a, float x) {
  if (x <= 0.0f) return 0.0f;
  const float gln = (float)std::lgamma((double)a);
  float ap = a, del = 1.0f / a, sum = del;
  for (int n = 1; n <= kItMax; ++n) {
    ap += 1.0f;
    del *= x / ap;
    sum += del;
    if (std::fabs(del) < std::fabs(sum) * kEps) break;
  }
  return sum * (float)std::exp((double)(-x + a * std::log(x) - gln));
}

// Q(a, x) = 1 - P(a, x) by the continued fraction, x >= a + 1
float gamma_cfrac(float a, float x) {
  const float gln = (float)std::lgamma((double)a);
  float b = x + 1.0f - a, c = 1.0f / kFpMin, d = 1.0f / b, h = d;
  for (int i = 1; i <= kItMax; ++i) {
    const float an = -(float)i * ((float)i - a);
    b += 2.0f;
    d = an * d + b;
    if (std::fabs(d) < kFpMin) d = kFpMin;
    c = b + an / c;
    if (std::fabs(c) < kFpMin) c = kFpMin;
    d = 1.0f / d;
    const float del = d * c;
    h *= del;
    if (std::fabs(del - 1.0f) < kEps) break;
  }
  return (float)std::exp((double)(-x + a * std::log(x) - gln)) * h;
}

float gamma_p(float a, float x) {
  if (x < 0.0f || a <= 0.0f) return -1.0f;
  return (x < a + 1.0f) ? gamma_series(a, x) : 1.0f - gamma_cfrac(a, x);
}

// Lambert W, branch -1, for -1/e <= z < 0
double lambert_wm1(double z) {
  const double em1 = 0.36787944117144233, e = 2.718281828459045;
  if (!(z >= -em1 && z < 0.0)) return NAN;
  double p = 1.0, w;
  if (z < -1e-6) {  // series about the branch point -1/e
    p = -std::sqrt(2.0 * (e * z + 1.0));
    w = -1.0 + p * (1.0 + p * (-1.0 / 3.0 + p * (11.0 / 72.0)));
  } else {  // asymptotic expansion near 0
    const double l1 = std::log(-z), l2 = std::log(-l1);
    w = l1 - l2 + l2 / l1;
  }
  if (std::fabs(p) < 1e-4) return w;
  for (int i = 0; i < 10; ++i) {  // Halley
    const double ew = std::exp(w);
    double t = w * ew - z;
    const double q = w + 1.0;
    t /= ew * q - 0.5 * (q + 1.0) * t / q;
    w -= t;
    if (std::fabs(t) < 4e-16 * (1.0 + std::fabs(w))) break;
  }
  return w;
}

// m in [lb, rb] with P_gamma((a+1)/b, m^b) = y (false position, then
// bisection-style bracketing)
float root(float ag, float b, float lb, float rb, float y, float eps) {
  auto F = [&](float m) { return gamma_p(ag, std::pow(m, b)); };
  float fl = F(lb), fr = F(rb);
  float delta = (y - fl) / (fr - fl);
  float c = lb * (1.0f - delta) + rb * delta;
  for (int it = 0; it < 200; ++it) {
    const float fc = F(c);
    if (std::fabs(fc - y) <= eps) break;
    if (fc > y) { rb = c; fr = fc; } else { lb = c; fl = fc; }
    delta = (y - fl) / (fr - fl);
    c = lb * (1.0f - delta) + rb * delta;
  }
  return c;
}

}  // namespace

int make_gex_table(float a, float b, float mp, float mk, double beta, GexTable* out) {
  if (!out || !(a > -1.0f) || !(b > 0.0f) || !(mp > 0.0f) || !(mk > 0.0f)) return DSM_ERR_INVALID;
  const float ag = (a + 1.0f) / b;
  const double g1 = std::exp(std::lgamma((double)ag));
  // mass cutoff where W(m)/m falls to 1e-3 of its maximum
  const double m_max = std::pow((double)a / b, 1.0 / b);
  const double w_max = b / g1 * std::pow(m_max, (double)a) * std::exp(-std::pow(m_max, (double)b));
  const double cut = 0.001 * w_max;
  const double wm1 = lambert_wm1(-(double)b / a * std::pow(cut * g1 / b, (double)b / a));
  if (!std::isfinite(wm1)) return DSM_ERR_INVALID;
  const float cutoff = (float)std::pow(-(double)a / b * wm1, 1.0 / b);
  // forward table on an even grid in m; the step in P is 4x its largest increment
  std::vector<float> gm(kGrid), gp(kGrid);
  float step = 0.0f;
  for (int i = 0; i < kGrid; ++i) {
    gm[i] = (float)i * cutoff / (float)(kGrid - 1);
    gp[i] = gamma_p(ag, std::pow(gm[i], b));
    if (i > 0) step = std::max(step, std::fabs(gp[i] - gp[i - 1]));
  }
  step *= 4.0f;
  // inverse table M[j], P(M[j]) = j * step, extended past the cutoff up to P = 1
  std::vector<float> M;
  const float tol = 1.0e-5f;
  for (int i = 0; i < kGrid; ++i) {
    const float y = step * (float)M.size();
    if (gp[i] >= y) M.push_back(i == 0 ? gm[0] : root(ag, b, gm[i - 1], gm[i], y, tol));
  }
  float m_hi = M.empty() ? cutoff : M.back();
  const float dm = cutoff / (float)(kGrid - 1);
  for (int guard = 0; (float)M.size() < 1.0f / step && guard < 100 * kGrid; ++guard) {
    const float m_lo = m_hi;
    m_hi += dm;
    const float y = step * (float)M.size();
    if (gamma_p(ag, std::pow(m_hi, b)) >= y) M.push_back(root(ag, b, m_lo, m_hi, y, tol));
  }
  if (M.size() < 2) return DSM_ERR_INVALID;
  // CD-weighted law: cumulative normdt(N_K(M[k])) in float, as tabulated in
  // the reference, inverted on an even grid
  std::vector<float> cw(M.size());
  float norm = 0.0f;
  double pre = 0.0;
  for (size_t k = 0; k < M.size(); ++k) {
    const float nd = (float)make_pcd(beta, (double)M[k] * mp / mk).normdt;
    cw[k] = (k > 0) ? nd + cw[k - 1] : nd;
    norm += nd;
    if ((float)(k + 1) < 1.0f / step) pre += nd;  // ensemble.cu:139-143: i + 1 < 1/step
  }
  float step_d = 0.0f;
  for (size_t k = 0; k < M.size(); ++k) {
    cw[k] = cw[k] / norm;
    if (k > 0) step_d = std::max(step_d, cw[k] - cw[k - 1]);
  }
  // inverse of the CD-weighted law, one entry per probability step, at most
  // one per source entry (the last threshold may round above 1: stop at the end)
  std::vector<float> Md;
  for (size_t k = 0; k < M.size() && (float)Md.size() < 1.0f / step_d; ++k)
    if (cw[k] >= step_d * (float)Md.size()) Md.push_back(M[k]);
  out->M = M;
  out->Md = Md;
  out->step = step;
  out->step_d = step_d;
  out->mp = mp;
  out->mk = mk;
  out->prefact = (double)step * pre / beta;  // ensemble.cu:137-146
  return DSM_OK;
}

}  // namespace dsm

extern "C" int dsm_gex_table(float a, float b, float mp, float mk, double beta, float* m, int32_t* n, float* md,
                             int32_t* n_d, double* info) {
  if (!n || !n_d) return DSM_ERR_INVALID;
  dsm::GexTable t;
  const int rc = dsm::make_gex_table(a, b, mp, mk, beta, &t);
  if (rc != DSM_OK) return rc;
  const int32_t cap = *n, cap_d = *n_d;
  *n = (int32_t)t.M.size();
  *n_d = (int32_t)t.Md.size();
  if (info) { info[0] = t.step; info[1] = t.step_d; info[2] = t.prefact; }
  if (m) for (int32_t i = 0; i < std::min(cap, *n); ++i) m[i] = t.M[i];
  if (md) for (int32_t i = 0; i < std::min(cap_d, *n_d); ++i) md[i] = t.Md[i];
  return DSM_OK;
}
