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
// W is evaluated in log form, w + log(w) = log(theta), so that no
// exponential overflows for any terminal voltage.
//
// Every operation here is a correctly rounded IEEE add, multiply, divide or
// explicit fused multiply-add (fma(), one rounding on every host and on the
// device), and the exponential and logarithm are this file's own (pvglu_exp,
// pvglu_log), so host code built without FMA contraction (-ffp-contract=off)
// and device code built with --fmad=false produce bit-identical results.
// FP64 is scarce on GB300, so the evaluation is written to few FP64
// instructions: fma() in the polynomials, no special-case tests where the
// argument is known to be positive and normal.
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
// Horner form with fused multiply-adds, scaled by 2^k.  A few ulps from the
// correctly rounded value.
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
  p = fma(p, r, 2.08767569878681e-09);   // 1/12!
  p = fma(p, r, 2.505210838544172e-08);
  p = fma(p, r, 2.755731922398589e-07);
  p = fma(p, r, 2.7557319223985893e-06);
  p = fma(p, r, 2.48015873015873e-05);
  p = fma(p, r, 0.0001984126984126984);
  p = fma(p, r, 0.001388888888888889);
  p = fma(p, r, 0.008333333333333333);
  p = fma(p, r, 0.041666666666666664);
  p = fma(p, r, 0.16666666666666666);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  if (k > 1023) return (p * 2.0) * pvglu_pow2(k - 1);
  if (k < -1021) return (p * pvglu_pow2(k + 1000)) * pvglu_pow2(-1000);
  return p * pvglu_pow2(k);
}

// log(x) for positive, normal, finite x: x = 2^e m with m in
// [sqrt(1/2), sqrt(2)), then log(m) = 2 atanh(s) = 2 (s + s^3/3 + ... +
// s^21/21), s = (m - 1)/(m + 1), |s| <= 0.1716, so s^2 <= 0.0295 and the
// first omitted term is below 7e-19 relative; m - 1 is exact.  Horner form
// with fused multiply-adds.  A few ulps from the correctly rounded value.
PVGLU_HD double pvglu_log_normal(double x) {
  const int64_t b = pvglu_bits(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = pvglu_from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (m > 1.4142135623730951) {
    m *= 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double z = s * s;
  double p = 0.047619047619047616;  // 1/21
  p = fma(p, z, 0.05263157894736842);
  p = fma(p, z, 0.058823529411764705);
  p = fma(p, z, 0.06666666666666667);
  p = fma(p, z, 0.07692307692307693);
  p = fma(p, z, 0.09090909090909091);
  p = fma(p, z, 0.1111111111111111);
  p = fma(p, z, 0.14285714285714285);
  p = fma(p, z, 0.2);
  p = fma(p, z, 0.3333333333333333);
  p = fma(p, z, 1.0);
  const double ln2_hi = 0.6931471824645996;
  const double ln2_lo = -1.904654299957768e-09;
  const double ed = (double)e;
  return fma(ed, ln2_hi, fma(2.0 * s, p, ed * ln2_lo));
}

// log(x) for every double: NaN, negative, zero, infinity and subnormal
// arguments handled, the rest by pvglu_log_normal.
PVGLU_HD double pvglu_log(double x) {
  if (x != x || x < 0.0) return NAN;
  if (x == 0.0) return -INFINITY;
  if (x == INFINITY) return x;
  if (x < 2.2250738585072014e-308)  // subnormal: scale into the normal range
    return pvglu_log_normal(x * 18014398509481984.0) - 54.0 * 0.6931471805599453;
  return pvglu_log_normal(x);
}

// FP32 counterparts of pvglu_exp / pvglu_log (same methods, fewer terms:
// degree-7 Taylor polynomial, atanh series to s^11/11), for the starting
// guess of the Lambert-W iteration.  Arguments within the normal float range.
PVGLU_HD float pvglu_expf(float x) {
  if (x > 88.0f) return INFINITY;
  if (x < -80.0f) return 0.0f;
  const float ln2_hi = 0.693115234375f;       // ln 2 to 12 bits (0x3F317000)
  const float ln2_lo = 3.194618329871446e-05f;
  const int k = (int)floorf(x * 1.4426950216293335f + 0.5f);
  const float r = (x - k * ln2_hi) - k * ln2_lo;
  float p = 0.00019841270113829523f;  // 1/7!
  p = p * r + 0.0013888889225199819f;
  p = p * r + 0.008333333767950535f;
  p = p * r + 0.0416666679084301f;
  p = p * r + 0.1666666716337204f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  unsigned int u;
  const unsigned int e = (unsigned int)(k + 127) << 23;
  memcpy(&u, &p, sizeof u);
  u += e - (127u << 23);
  float out;
  memcpy(&out, &u, sizeof out);
  return out;
}

PVGLU_HD float pvglu_logf(float x) {
  unsigned int b;
  memcpy(&b, &x, sizeof b);
  int e = (int)((b >> 23) & 0xff) - 127;
  const unsigned int mb = (b & 0x7fffffu) | 0x3f800000u;
  float m;
  memcpy(&m, &mb, sizeof m);
  if (m > 1.4142135381698608f) {
    m *= 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float p = 0.09090909361839294f;  // 1/11
  p = p * z + 0.1111111119389534f;
  p = p * z + 0.1428571492433548f;
  p = p * z + 0.20000000298023224f;
  p = p * z + 0.3333333432674408f;
  p = p * z + 1.0f;
  return e * 0.693115234375f + ((2.0f * s) * p + e * 3.194618329871446e-05f);
}

// Principal branch W0(theta) for theta = exp(L).  W solves w + log(w) = L.
// Below L = -40, W(theta) = theta (1 - theta + ...) equals theta to double
// precision.  Otherwise an FP32 estimate (Winitzki's approximation or the
// asymptotic series, then three Halley steps on h(w) = w + log(w) - L) is
// finished by one FP64 Halley step, which takes the FP32 error (~1e-7)
// below the FP64 rounding (cubic convergence).  The FP64 work is one
// logarithm of a positive normal number and one division.
PVGLU_HD double pvglu_lambert_w0_exp(double L) {
  if (L < -40.0) return pvglu_exp(L);
  const float lf = (float)L;
  float w;
  if (lf < 1.0f) {
    const float theta = pvglu_expf(lf);
    if (theta < 1e-3f) {
      w = theta * (1.0f - theta);
    } else {
      const float l1 = pvglu_logf(1.0f + theta);  // log(1 + theta)
      w = l1 * (1.0f - pvglu_logf(1.0f + l1) / (2.0f + l1));
    }
  } else {
    const float ll = pvglu_logf(lf);
    w = lf - ll + ll / lf;
  }
  for (int it = 0; it < 3; it++) {
    const float h = w + pvglu_logf(w) - lf;
    const float wp1 = w + 1.0f;
    w = w - 2.0f * h * w * wp1 / (2.0f * wp1 * wp1 + h);
  }
  // w > 0 and normal here (W(e^-40) is about 4e-18), or NaN from a NaN L,
  // which h carries on.
  const double wd = (double)w;
  const double h = (wd + pvglu_log_normal(wd)) - L;
  const double wp1 = wd + 1.0;
  return wd - (2.0 * h * wd * wp1) / fma(2.0 * wp1, wp1, h);
}

// Constants of the panel law, computed once per parameter set.
typedef struct {
  double log_c;      // log(Rs Rsh I0 / (a (Rs + Rsh)))
  double k_l0;       // Rsh / (a (Rs + Rsh))
  double rs_iph;     // Rs (multiplies Iph + I0 in the exponent)
  double i0;
  double rsh_rsum;   // Rsh / (Rs + Rsh)
  double inv_rsum;   // 1 / (Rs + Rsh)
  double a_over_rs;
  double k_gd;       // (Rs + Rsh) / (Rs Rsh)
  double inv_rsh;
  double rs;
} pvglu_panel_const;

PVGLU_HD void pvglu_panel_prepare(const pvglu_panel_params* p, pvglu_panel_const* c) {
  const double rsum = p->rs + p->rsh;
  c->log_c = pvglu_log(p->rs * p->rsh * p->i0 / (p->a * rsum));
  c->k_l0 = p->rsh / (p->a * rsum);
  c->rs_iph = p->rs;
  c->i0 = p->i0;
  c->rsh_rsum = p->rsh / rsum;
  c->inv_rsum = 1.0 / rsum;
  c->a_over_rs = p->a / p->rs;
  c->k_gd = rsum / (p->rs * p->rsh);
  c->inv_rsh = 1.0 / p->rsh;
  c->rs = p->rs;
}

// Terminal current I(V) (out of the + terminal), dI/dV and dI/dIph.  With
// w = W(theta) = Rs Rsh I0 / (a (Rs + Rsh)) * exp(Vd / a), Vd = V + I Rs:
//   I = Rsh (Iph + I0) / (Rs + Rsh) - V / (Rs + Rsh) - (a / Rs) w,
//   gd = dIdiode/dVd + 1/Rsh = w (Rs + Rsh) / (Rs Rsh) + 1/Rsh,
//   dI/dV = -gd / (1 + Rs gd),  dI/dIph = 1 / (1 + Rs gd).
PVGLU_HD void pvglu_panel_eval(const pvglu_panel_const* c, double iph, double v,
                               double* current, double* didv, double* didiph) {
  const double ip = iph + c->i0;
  const double log_theta = fma(c->k_l0, fma(c->rs_iph, ip, v), c->log_c);
  const double w = pvglu_lambert_w0_exp(log_theta);
  const double i = fma(-c->a_over_rs, w, fma(c->rsh_rsum, ip, -v * c->inv_rsum));
  const double gd = fma(w, c->k_gd, c->inv_rsh);
  const double q = 1.0 / fma(c->rs, gd, 1.0);
  *current = i;
  *didv = -gd * q;
  *didiph = q;
}

PVGLU_HD void pvglu_panel_iv3(const pvglu_panel_params* p, double iph, double v,
                              double* current, double* didv, double* didiph) {
  pvglu_panel_const c;
  pvglu_panel_prepare(p, &c);
  pvglu_panel_eval(&c, iph, v, current, didv, didiph);
}

// Terminal current I(V) (out of the + terminal) and dI/dV.
PVGLU_HD void pvglu_panel_iv(const pvglu_panel_params* p, double iph, double v,
                             double* current, double* didv) {
  double didiph;
  pvglu_panel_iv3(p, iph, v, current, didv, &didiph);
}

// Irradiance [W/m^2] at panel position (x, y) [m] and time t [s] under
// `count` Gaussian shadows drifting with constant velocity, clamped at 0:
//   G = g_clear - sum_k depth_k exp(-((x - cx_k - vx_k t)^2 + (y - cy_k - vy_k t)^2) / (2 sigma_k^2)).
// Shadow k is sh[6k .. 6k+5] = cx, cy, vx, vy, depth, sigma.  The clouds of
// the reference are painted as opacity canvases moving at constant speed
// (001_clouds.cu:55-62, :96-137); this is the synthetic field of the
// benchmark configurations, shared by the host generator and the device.
PVGLU_HD double pvglu_shadow_irradiance(double x, double y, const double* sh, int count, double t,
                                        double g_clear) {
  double g = g_clear;
  for (int k = 0; k < count; k++) {
    const double* c = sh + 6 * k;
    const double dx = x - (c[0] + c[2] * t);
    const double dy = y - (c[1] + c[3] * t);
    g -= c[4] * pvglu_exp(-(dx * dx + dy * dy) / (2.0 * c[5] * c[5]));
  }
  return g > 0.0 ? g : 0.0;
}
