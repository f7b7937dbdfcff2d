/*
 * pvglu plant API: the synthetic PV plant whose Newton Jacobians feed the
 * hot path (inverters x parallel strings x series panels, fixed-voltage MPPT
 * sinks), its seeded Gaussian-shadow irradiance, and the device-side
 * Jacobian assembly and Newton iteration.
 *
 * Reference counterparts (AlbertoJimenezRuiz/PhdThesis_AlbertoJimenezRuiz,
 * PVPP_Plant_Simulator/): create_full_electric_system
 * (003_create_electric_system.cpp:314-382) builds the circuit,
 * basic_electric_circuit::create_matrix_and_vector (002b:141-240) assembles
 * J and b every iteration, calculate_new_iteration (011:37-110) damps the
 * update, PVPP_Simulator (000:95-259) drives the loop.
 */
#ifndef PVGLU_PLANT_H
#define PVGLU_PLANT_H

#include <stdint.h>

#include "pvglu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Builds the plant (host).  Panel constants, cable resistances and the MPPT
 * fraction take the defaults of the synthetic configurations: Iph = 8.5*G/1000,
 * I0 = 1e-9, n = 1.3, 60 cells, Vt = 25.7 mV, Rs = 0.3, Rsh = 300,
 * 0.05 / 0.02 ohm cables, V_mppt = 0.8 * Voc_string, 2 m panel grid. */
int pvglu_plant_create(int n_inverters, int n_strings, int n_series, pvglu_plant** out);
int pvglu_plant_destroy(pvglu_plant* p);

typedef struct {
  int n;             /* unknowns */
  int n_panels;
  int64_t nnz_a;
  int n_inverters, n_strings, n_series;
  double voc_panel, v_mppt, extent_x, extent_y;
  double panel_i0, panel_a, panel_rs, panel_rsh, iph_stc;
} pvglu_plant_info;
int pvglu_plant_get_info(const pvglu_plant* p, pvglu_plant_info* info);

/* Integer arrays: rowptr, colidx (Jacobian pattern), pan_hi, pan_lo (panel
 * terminals, -1 = ground), contrib_ptr, contrib_panel, inc_ptr, inc_panel,
 * inv_terminal, inv_current, inv_combiner.  Signed-char arrays are exposed as
 * int: contrib_sign, inc_sign.  Double arrays: a_lin, b_lin, pan_x, pan_y. */
int pvglu_plant_get_iarray(const pvglu_plant* p, const char* name, const int** data,
                           int64_t* len);
int pvglu_plant_get_darray(const pvglu_plant* p, const char* name, const double** data,
                           int64_t* len);

/* Irradiance [W/m^2] per panel for one scenario at time t: 1000 minus
 * `n_shadows` in [min_shadows, max_shadows] seeded Gaussian shadows (depth
 * U[min_depth, max_depth], sigma U[20, 80] m, drift 5-15 m/s), clamped >= 0. */
int pvglu_plant_irradiance(const pvglu_plant* p, int min_shadows, int max_shadows,
                           double min_depth, double max_depth, uint64_t seed, double t,
                           double* g_out);

/* The seeded shadows behind pvglu_plant_irradiance for one scenario:
 * *count shadows (at most max_shadows), params[6k .. 6k+5] = centre x, y
 * [m] at t = 0, velocity x, y [m/s], depth [W/m^2], sigma [m].  For the
 * device field of pvglu_newton_set_field. */
int pvglu_plant_shadows(const pvglu_plant* p, int min_shadows, int max_shadows,
                        double min_depth, double max_depth, uint64_t seed, int* count,
                        double* params);

/* Host evaluation of the panel model: current out of the + terminal and its
 * derivative for `count` (photocurrent, terminal voltage) pairs. */
int pvglu_plant_panel_iv(const pvglu_plant* p, int count, const double* iph,
                         const double* v, double* current, double* didv);

/* The panel model's own exponential and logarithm (the same code runs on
 * the device), for accuracy checks: exp_out[i] = exp(x[i]),
 * log_out[i] = log(x[i]); either output may be NULL. */
int pvglu_plant_exp_log(int count, const double* x, double* exp_out, double* log_out);

#ifdef __cplusplus
}
#endif
#endif /* PVGLU_PLANT_H */
