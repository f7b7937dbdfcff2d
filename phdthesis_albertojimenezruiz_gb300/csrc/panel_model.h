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
#pragma once
#include <math.h>

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

// Principal branch W0(theta) for theta = exp(log_theta) >= 0.
PVGLU_HD double pvglu_lambert_w0_exp(double log_theta) {
  double w;
  if (log_theta < 1.0) {
    // Solve w * exp(w) = theta directly.
    const double theta = exp(log_theta);
    w = theta < 0.1 ? theta * (1.0 - theta) : 0.5 * log1p(theta) + 0.25 * theta / (1.0 + theta);
    for (int it = 0; it < 40; it++) {
      const double ew = exp(w);
      const double f = w * ew - theta;
      const double wp1 = w + 1.0;
      const double denom = ew * wp1 - (w + 2.0) * f / (2.0 * wp1);
      const double dw = f / denom;
      w -= dw;
      if (fabs(dw) <= 1e-17 * (fabs(w) + 1e-300)) break;
    }
  } else {
    // Solve h(w) = w + log(w) - log_theta = 0 (Halley on h).
    w = log_theta - log(log_theta);
    if (w < 0.5) w = 0.5;
    for (int it = 0; it < 40; it++) {
      const double h = w + log(w) - log_theta;
      const double h1 = 1.0 + 1.0 / w;
      const double h2 = -1.0 / (w * w);
      const double dw = h / (h1 - 0.5 * h * h2 / h1);
      w -= dw;
      if (fabs(dw) <= 1e-16 * w) break;
    }
  }
  return w;
}

// Terminal current I(V) (out of the + terminal), dI/dV and dI/dIph.
PVGLU_HD void pvglu_panel_iv3(const pvglu_panel_params* p, double iph, double v,
                              double* current, double* didv, double* didiph) {
  const double rs = p->rs, rsh = p->rsh, a = p->a, i0 = p->i0;
  const double rsum = rs + rsh;
  const double log_theta = log(rs * rsh * i0 / (a * rsum)) +
                           rsh * (rs * (iph + i0) + v) / (a * rsum);
  const double w = pvglu_lambert_w0_exp(log_theta);
  const double i = (rsh * (iph + i0) - v) / rsum - (a / rs) * w;
  // Implicit derivatives: with gd = dIdiode/dVd + 1/Rsh at Vd = V + I*Rs,
  // dI/dV = -gd / (1 + Rs*gd) and dI/dIph = 1 / (1 + Rs*gd).
  const double vd = v + i * rs;
  const double gd = i0 / a * exp(vd / a) + 1.0 / rsh;
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
