// Synthetic PV plant: inverters x parallel strings x series panels.
//
// Topology per inverter v (all negative terminals on ground):
//   string s, panel p sits between node(v,s,p-1) (ground for p = 0) and
//   node(v,s,p); node(v,s,last) -- 0.05 ohm -- combiner bus C_v
//   -- 0.02 ohm -- inverter terminal T_v; a fixed-voltage MPPT sink
//   (an MNA voltage source, extra unknown I_v) holds T_v at 0.8 * Voc_string.
// Unknown order per inverter: string nodes (string-major), C_v, T_v, I_v.
//
// MNA stamp conventions follow PVPP_Plant_Simulator/002b_sistema_electrico_
// base_matriz.cpp: admittance (:5-38), voltage source with its extra row
// (:110-125), current source (:99-108) and the companion model of a nonlinear
// element G = f'(V), Ieq = f(V) - G*V (:183-197).
#pragma once
#include <cstdint>
#include <vector>

#include "panel_model.h"

namespace pvglu {

struct PlantConfig {
  int n_inverters = 4, n_strings = 8, n_series = 20;
  double iph_stc = 8.5;       // A at 1000 W/m^2 (Iph = 8.5 * G / 1000)
  double i0 = 1e-9;
  double ideality = 1.3;
  int cells = 60;
  double vt = 0.0257;
  double rs = 0.3, rsh = 300.0;
  double r_string = 0.05, r_combiner = 0.02;
  double mppt_fraction = 0.8;
  double pitch = 2.0;         // panel grid [m]
};

struct ShadowConfig {
  int min_shadows = 3, max_shadows = 3;
  double min_depth = 300.0, max_depth = 800.0;   // W/m^2
  double min_sigma = 20.0, max_sigma = 80.0;     // m
  double min_speed = 5.0, max_speed = 15.0;      // m/s
  double g_clear = 1000.0;
};

struct Plant {
  PlantConfig cfg;
  int n = 0, n_panels = 0;
  pvglu_panel_params panel{};
  double voc_panel = 0, v_mppt = 0;
  // Jacobian pattern, original order, CSR with sorted rows.
  std::vector<int> rowptr, colidx;
  std::vector<double> a_lin;        // linear part of every A entry
  std::vector<double> b_lin;        // RHS of the linear part (source rows)
  // Panels: terminals (unknown id or -1 for ground) and panel position.
  std::vector<int> pan_hi, pan_lo;
  std::vector<double> pan_x, pan_y;
  // A entry e receives sum over c in [contrib_ptr[e], contrib_ptr[e+1]) of
  // contrib_sign[c] * g[contrib_panel[c]].
  std::vector<int> contrib_ptr, contrib_panel;
  std::vector<signed char> contrib_sign;
  // Node incidence of panels for the KCL mismatch: node i gets
  // sum over c of inc_sign[c] * f[inc_panel[c]] (f = current hi -> lo).
  std::vector<int> inc_ptr, inc_panel;
  std::vector<signed char> inc_sign;
  std::vector<int> inv_terminal, inv_current, inv_combiner;
  double extent_x = 0, extent_y = 0;
};

int build_plant(const PlantConfig& cfg, Plant& out);

// The seeded Gaussian shadows of one scenario: 6 values per shadow (cx, cy,
// vx, vy, depth, sigma; see pvglu_shadow_irradiance).
void plant_shadows(const Plant& p, const ShadowConfig& sc, uint64_t seed,
                   std::vector<double>& params);

// Per-panel irradiance G for one scenario at time t (seeded Gaussian shadows
// drifting with constant velocity; G clamped at 0).
void plant_irradiance(const Plant& p, const ShadowConfig& sc, uint64_t seed,
                      double t, double* g_out);

// Open-circuit voltage of one panel at photocurrent iph.
double panel_voc(const pvglu_panel_params& pp, double iph);

}  // namespace pvglu
