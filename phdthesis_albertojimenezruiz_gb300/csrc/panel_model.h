// Two-terminal single-diode PV panel, FP64, shared by host and device code.
//
// The reference models a panel with an internal diode node plus series and
// shunt resistors as separate MNA elements (PVPP_Plant_Simulator/
// 003_create_electric_system.cpp:89-126).  Here the series resistance is
// condensed into the element, so a panel adds no internal unknown: its
// terminal current I(V) solves the implicit single-diode equation
//
//     I = Iph - I0 * (exp((V + I*Rs) / a) - 1) - (V + I*Rs) / Rsh,
//     a = n * Ncells * Vt,
//
// with the explicit Lambert-W form
//
//     I = (Rsh*(Iph + I0) - V) / (Rs + Rsh) - (a / Rs) * W(theta),
//     theta = Rs*Rsh*I0 / (a*(Rs + Rsh)) * exp(Rsh*(Rs*(Iph + I0) + V) / (a*(Rs + Rsh))).
//
// W is evaluated with Halley's iteration, in log form for large arguments so
// that no exponential overflows for any terminal voltage.
//
// Every operation here is a correctly rounded IEEE add, multiply or divide,
// and the exponential and logarithm are this file's own (pvglu_exp,
// pvglu_log), so host code built without FMA contraction
// (-ffp-contract=off) and device code built with --fmad=false produce
// bit-identical results.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PVGLU_HD __host__ __device__ __forceinline__
#else
#define PVGLU_HD static inline
#endif

typedef struct {
  double i0;    // diode saturation current [A]
  double a;     // modified ideality voltage n * Ncells * Vt [V]
  double rs;    // series resistance [ohm]
  double rsh;   // shunt resistance [ohm]
} pvglu_panel_params;

PVGLU_HD int64_t pvglu_bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

PVGLU_HD double pvglu_from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// 2^k for -1022 <= k <= 1023.
PVGLU_HD double pvglu_pow2(int k) { return pvglu_from_bits((int64_t)(k + 1023) << 52); }

// exp(x): Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split
// into ln2_hi (21 significant bits, so k * ln2_hi is exact) and ln2_lo, then
// the degree-13 Taylor polynomial of exp(r) (remainder < 5e-18 relative) in
// Horner form, scaled by 2^k.  A few ulps from the correctly rounded value.
PVGLU_HD double pvglu_exp(double x) {
  if (x != x) return x;
  if (x > 709.782712893384) return INFINITY;
  if (x < -745.2) return 0.0;
  const double ln2_hi = 0.6931471824645996;      // float(ln 2), 0x3FE62E4300000000
  const double ln2_lo = -1.904654299957768e-09;  // ln 2 - ln2_hi
  const double inv_ln2 = 1.4426950408889634;
  const int k = (int)floor(x * inv_ln2 + 0.5);
  const double r = (x - k * ln2_hi) - k * ln2_lo;
  double p = 1.6059043836821613e-10;  // 1/13!
  p = p * r + 2.08767569878681e-09;   // 1/12!
  p = p * r + 2.505210838544172e-08;
  p = p * r + 2.755731922398589e-07;
  p = p * r + 2.7557319223985893e-06;
  p = p * r + 2.48015873015873e-05;
  p = p * r + 0.0001984126984126984;
  p = p * r + 0.001388888888888889;
  p = p * r + 0.008333333333333333;
  p = p * r + 0.041666666666666664;
  p = p * r + 0.16666666666666666;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  if (k > 1023) return (p * 2.0) * pvglu_pow2(k - 1);
  if (k < -1021) return (p * pvglu_pow2(k + 1000)) * pvglu_pow2(-1000);
  return p * pvglu_pow2(k);
}

// log(x): x = 2^e m with m in [sqrt(1/2), sqrt(2)), then
// log(m) = 2 atanh(s) = 2 (s + s^3/3 + ... + s^27/27), s = (m - 1)/(m + 1),
// |s| <= 0.1716 (remainder < 1e-19 relative); m - 1 is exact.  A few ulps
// from the correctly rounded value.
PVGLU_HD double pvglu_log(double x) {
  if (x != x || x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (x == INFINITY) return x;
  int e = 0;
  if (x < 2.2250738585072014e-308) {  // subnormal: scale into the normal range
    x *= 18014398509481984.0;         // 2^54
    e = -54;
  }
  const int64_t b = pvglu_bits(x);
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = pvglu_from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (m > 1.4142135623730951) {
    m *= 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double z = s * s;
  double p = 0.037037037037037035;  // 1/27
  p = p * z + 0.04;
  p = p * z + 0.043478260869565216;
  p = p * z + 0.047619047619047616;
  p = p * z + 0.05263157894736842;
  p = p * z + 0.058823529411764705;
  p = p * z + 0.06666666666666667;
  p = p * z + 0.07692307692307693;
  p = p * z + 0.09090909090909091;
  p = p * z + 0.1111111111111111;
  p = p * z + 0.14285714285714285;
  p = p * z + 0.2;
  p = p * z + 0.3333333333333333;
  p = p * z + 1.0;
  const double ln2_hi = 0.6931471824645996;
  const double ln2_lo = -1.904654299957768e-09;
  return e * ln2_hi + ((2.0 * s) * p + e * ln2_lo);
}

// Principal branch W0(theta) for theta = exp(log_theta) >= 0.  Halley's
// iteration converges cubically; it stops once a step is below 1e-15
// relative (the next one would be at the rounding level).
PVGLU_HD double pvglu_lambert_w0_exp(double log_theta) {
  double w;
  if (log_theta < 1.0) {
    // Solve w * exp(w) = theta directly.
    const double theta = pvglu_exp(log_theta);
    w = theta < 0.1 ? theta * (1.0 - theta)
                    : 0.5 * pvglu_log(1.0 + theta) + 0.25 * theta / (1.0 + theta);
    for (int it = 0; it < 16; it++) {
      const double ew = pvglu_exp(w);
      const double f = w * ew - theta;
      const double wp1 = w + 1.0;
      const double denom = ew * wp1 - (w + 2.0) * f / (2.0 * wp1);
      const double dw = f / denom;
      w -= dw;
      if (fabs(dw) <= 1e-15 * fabs(w)) break;
    }
  } else {
    // Solve h(w) = w + log(w) - log_theta = 0 (Halley on h).
    w = log_theta - pvglu_log(log_theta);
    if (w < 0.5) w = 0.5;
    for (int it = 0; it < 16; it++) {
      const double h = w + pvglu_log(w) - log_theta;
      const double h1 = 1.0 + 1.0 / w;
      const double h2 = -1.0 / (w * w);
      const double dw = h / (h1 - 0.5 * h * h2 / h1);
      w -= dw;
      if (fabs(dw) <= 1e-15 * w) break;
    }
  }
  return w;
}

// Terminal current I(V) (out of the + terminal), dI/dV and dI/dIph.
PVGLU_HD void pvglu_panel_iv3(const pvglu_panel_params* p, double iph, double v,
                              double* current, double* didv, double* didiph) {
  const double rs = p->rs, rsh = p->rsh, a = p->a, i0 = p->i0;
  const double rsum = rs + rsh;
  const double log_theta = pvglu_log(rs * rsh * i0 / (a * rsum)) +
                           rsh * (rs * (iph + i0) + v) / (a * rsum);
  const double w = pvglu_lambert_w0_exp(log_theta);
  const double i = (rsh * (iph + i0) - v) / rsum - (a / rs) * w;
  // Implicit derivatives: with gd = dIdiode/dVd + 1/Rsh at Vd = V + I*Rs,
  // dI/dV = -gd / (1 + Rs*gd) and dI/dIph = 1 / (1 + Rs*gd).
  const double vd = v + i * rs;
  const double gd = i0 / a * pvglu_exp(vd / a) + 1.0 / rsh;
  *current = i;
  *didv = -gd / (1.0 + rs * gd);
  *didiph = 1.0 / (1.0 + rs * gd);
}

// Terminal current I(V) (out of the + terminal) and dI/dV.
PVGLU_HD void pvglu_panel_iv(const pvglu_panel_params* p, double iph, double v,
                             double* current, double* didv) {
  double didiph;
  pvglu_panel_iv3(p, iph, v, current, didv, &didiph);
}
