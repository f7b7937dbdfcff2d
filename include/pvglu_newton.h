/*
 * pvglu Newton driver: the per-iteration loop of the PV plant simulator on
 * the device, around the hot path of pvglu.h.
 *
 * One iteration, for every scenario still running, is
 *   companion model of every nonlinear element at its voltage iterate
 *     (002b_sistema_electrico_base_matriz.cpp:183-202: G = f'(V),
 *      Ieq = f(V) - G*V, convergence conductance gmin while it is > 0),
 *   right-hand side b = b_lin - incidence * Ieq (002b:196, current source
 *     stamp :100-110),
 *   scatter from the registered stamps, refactor, solve (pvglu.h (a)-(c);
 *     FP32 handles refine in FP64, pvglu_refine),
 *   damped update of every element voltage: the step to the new voltage drop
 *     is halved per element while it moves the voltage by more than 1 V or
 *     gives NaN (011_calculate_new_iteration.cpp:37-90), diff = sum of
 *     |change|,
 * and the scenario moves to the next gmin stage once diff < tol
 * (000_PVPP_simulator.cpp:163-236: stages {100, 10, ..., 0.05, -1},
 * tol = 1e-6 * n, at most 5000 iterations).  Scenarios are independent:
 * each follows its own stage and stops on its own.
 *
 * The element law is the two-terminal single-diode panel of panel_model.h
 * (constants per handle, photocurrent per element and scenario).
 *
 * Vectors are device FP64 arrays [count * ld], scenario fastest
 * (ld = pvglu_numeric_ld).  All calls are asynchronous on `stream` unless
 * stated otherwise; a handle is not thread-safe.
 */
#ifndef PVGLU_NEWTON_H
#define PVGLU_NEWTON_H

#include "pvglu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pvglu_newton pvglu_newton;

/* The circuit around the Jacobian pattern of the symbolic handle.  Host
 * arrays, copied at creation. */
typedef struct {
  int n_elems;            /* nonlinear two-terminal elements (panels) */
  const int* elem_hi;     /* [n_elems] unknown of the + terminal, -1 = ground */
  const int* elem_lo;     /* [n_elems] unknown of the - terminal, -1 = ground */
  const double* a_lin;    /* [nnz_a] linear part of A, caller CSR order */
  const double* b_lin;    /* [n] right-hand side of the linear part */
  double i0, a, rs, rsh;  /* element constants (panel_model.h) */
} pvglu_circuit;

/* Per-scenario outcome (pvglu_newton_results). */
enum {
  PVGLU_NEWTON_CONVERGED = 0,
  PVGLU_NEWTON_RUNNING = 1,
  PVGLU_NEWTON_MAX_ITERATIONS = 2, /* the reference aborts ("Did not converge") */
  PVGLU_NEWTON_DAMPING = 3         /* step halved below 1e-13 ("Convergence error") */
};

/* Binds a Newton driver to a numeric handle (FP64, or FP32 with FP64
 * refinement).  Registers the circuit's stamps on `num`
 * (pvglu_numeric_set_stamps); every element terminal pair must be in the
 * Jacobian pattern (PVGLU_ERR_STRUCTURAL otherwise).  `num` must outlive the
 * driver. */
int pvglu_newton_create(pvglu_numeric* num, const pvglu_circuit* c, pvglu_newton** out);
int pvglu_newton_destroy(pvglu_newton* nw);

/* Photocurrent of every element and scenario, device [n_elems * ld]. */
int pvglu_newton_set_iph(pvglu_newton* nw, const double* iph, void* stream);
/* Voltage iterate of every element and scenario, device [n_elems * ld]
 * (the flat start, or a previous solution). */
int pvglu_newton_set_voltages(pvglu_newton* nw, const double* v, void* stream);

/* Irradiance field on the device (the per-time-step input of the simulator:
 * the reference paints moving cloud canvases, 001_clouds.cu:55-62, :96-137,
 * and reads one value per panel, 003_create_electric_system.cpp:162-201).
 * Host arrays, copied: panel positions elem_x, elem_y [n_elems] (m), and per
 * scenario counts[s] <= max_shadows Gaussian shadows, shadows[(s *
 * max_shadows + k) * 6 + j] = centre x, y, velocity x, y, depth, sigma
 * (pvglu_plant_shadows gives them for the synthetic plant). */
int pvglu_newton_set_field(pvglu_newton* nw, const double* elem_x, const double* elem_y,
                           int max_shadows, const int* counts, const double* shadows,
                           const double* t_offset, double g_clear, double iph_per_g);
/* t_offset (host [S] or NULL): scenario s sees the field at time t +
 * t_offset[s] (time steps of one field solved as one batch).
 * Photocurrents of every element and scenario at time t from the field,
 * iph = iph_per_g * G (pvglu_shadow_irradiance), straight into the driver's
 * photocurrent buffer: no host traffic per time step.  g_out (device
 * [n_elems * ld]) receives G, or NULL. */
int pvglu_newton_field_iph(pvglu_newton* nw, double t, double* g_out, void* stream);

/* Broken panels.  The reference replaces a broken panel by a wire of
 * resistance 1e-5 ohm between the same nodes (003_create_electric_system.cpp:
 * 248-260, main.h:76): the Jacobian pattern does not change, so no new
 * analysis is needed -- the flagged elements (host [n_elems], nonzero =
 * broken; NULL clears) switch to that linear law on the device (conductance
 * 1/r_wire, no current source, no damping, not part of the Newton diff, no
 * irradiance sensitivity). */
int pvglu_newton_set_broken(pvglu_newton* nw, const int* broken, double r_wire);

/* Iteration of FP32 handles: refinement tolerance and sweep limit of each
 * linear solve (defaults 1e-12, 8).  Each Newton step solves for the node
 * voltages themselves, not for a correction, so this tolerance bounds the
 * accuracy of the converged operating point. */
int pvglu_newton_set_refinement(pvglu_newton* nw, double tol, int max_sweeps);

/* Runs the damped Newton iteration from the current voltage iterate over the
 * convergence-conductance schedule gmin[0..n_stages-1] (host, at most 16
 * stages; a value <= 0 adds nothing), stage tolerance `tol` on the summed
 * absolute voltage change, at most max_iterations iterations per scenario.
 * Launches the iteration body as a CUDA graph where the stream capture
 * succeeds, in groups of `check_every` (>= 1) between host reads of the
 * converged count; returns when every scenario has stopped or after
 * max_iterations bodies.  Synchronizes `stream`. */
int pvglu_newton_run(pvglu_newton* nw, const double* gmin, int n_stages, double tol,
                     int max_iterations, int check_every, void* stream);

/* Host arrays [S] (any may be NULL): iterations, outcome (PVGLU_NEWTON_*),
 * last diff.  Synchronous. */
int pvglu_newton_results(pvglu_newton* nw, int* iterations, int* outcome, double* diff);

/* Device pointers owned by the driver: element voltage iterate
 * [n_elems * ld]. */
const double* pvglu_newton_voltages(const pvglu_newton* nw);
/* Node solution of each scenario's last linear solve, caller order, into
 * device x [n * ld]. */
int pvglu_newton_solution(pvglu_newton* nw, double* x, void* stream);
/* Kirchhoff current mismatch of each scenario at its node solution x:
 * max_i |(A_lin x)_i + sum of the element currents at V = x[hi] - x[lo]
 * leaving node i - b_lin_i| [A], the convergence measure of the synthetic
 * configurations (||mismatch||_inf < 1e-9 A).  Host out [S].  Synchronous;
 * uses the driver's companion buffer as scratch (the next iteration rebuilds
 * it). */
int pvglu_newton_mismatch(pvglu_newton* nw, double* out);
/* Number of iteration bodies launched by the last pvglu_newton_run and
 * whether they ran as a graph (1) or as direct launches (0). */
int pvglu_newton_last_run(const pvglu_newton* nw, int* bodies, int* graph);

/* Adjoint sensitivity of a linear objective P = dpdx . x at the current
 * iterate (every scenario): the Jacobian is rebuilt at the voltage iterate
 * without convergence conductance, refactored, and J^T lambda = dpdx solved
 * (FP32 handles: refined); then
 *   dP/dIph[k] = dI_k/dIph_k * (lambda[hi_k] - lambda[lo_k])
 * for every element (ground terms 0).  dpdx: device [n * ld] caller order;
 * dpdiph: device [n_elems * ld].  Overwrites the handle's factors.  No
 * counterpart in the reference (its simulator computes no sensitivities). */
int pvglu_newton_adjoint(pvglu_newton* nw, const double* dpdx, double* dpdiph, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PVGLU_NEWTON_H */
