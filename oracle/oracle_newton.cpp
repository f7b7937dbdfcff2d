// ORACLE — test infrastructure only.
//
// CPU restatement of the PV plant simulator's Newton loop, one scenario at a
// time, over the oracle's own symbolic analysis and sequential GLU
// (oracle_glu.cpp):
//   stages of convergence conductance, a stage ends once diff < tol
//     (PVPP_Plant_Simulator/000_PVPP_simulator.cpp:163-236),
//   A and b assembled entry by entry as create_matrix_and_vector does
//     (002b_sistema_electrico_base_matriz.cpp:141-240: linear part, then per
//     nonlinear element the admittance G, the current source -Ieq and, while
//     positive, the convergence admittance),
//   permutation, scatter, GLU, substitution, unpermutation (000:193-233),
//   damped update with a global halving loop (011_calculate_new_iteration.cpp:
//   37-90) and a long double diff.
// The element law is the plant's own definition (panel_model.h), an input of
// the check like the plant's pattern and linear part.
#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <vector>

#include "panel_model.h"

extern "C" {
int oracle_get(void* h, const char* name, const int** ptr, long long* len);
int oracle_scatter_refactor_solve(void* h, const double* a_vals, double* lu_out, double* b,
                                  int sequential);
int oracle_scatter(void* h, const double* a_vals, double* csc_vals);
int oracle_refactor_sequential(void* h, double* v, int* bad_col);
int oracle_solve_transposed(void* h, const double* v, double* b);
}

namespace {

using Row = std::map<int, double>;

struct Circuit {
  int n, n_elems;
  const int *rowptr, *colidx, *hi, *lo;
  const double *a_lin, *b_lin;
  pvglu_panel_params panel;
  const int* broken;  // [n_elems] or NULL: panels replaced by a wire
  double g_wire;
};

bool is_broken(const Circuit& c, int k) { return c.broken && c.broken[k]; }

// 002b:5-38 (admittance between n1 and n2, ground = -1).
void add_admittance(std::vector<Row>& A, int n1, int n2, double g) {
  if (n1 >= 0) A[n1][n1] += g;
  if (n1 >= 0 && n2 >= 0) {
    A[n1][n2] += -g;
    A[n2][n1] += -g;
  }
  if (n2 >= 0) A[n2][n2] += g;
}

// 002b:100-110 (current source val from n1 to n2).
void add_current_source(std::vector<double>& b, int n1, int n2, double val) {
  if (n1 >= 0) b[n1] += val;
  if (n2 >= 0) b[n2] -= val;
}

// create_matrix_and_vector at the voltage iterate v; A's values returned in
// the pattern's CSR order.  Returns false if a stamp falls outside it.
bool assemble(const Circuit& c, const double* iph, const double* v, double gmin,
              std::vector<double>& a_vals, std::vector<double>& b, std::vector<double>* didiph) {
  std::vector<Row> A(c.n);
  for (int i = 0; i < c.n; i++)
    for (int p = c.rowptr[i]; p < c.rowptr[i + 1]; p++) A[i][c.colidx[p]] = c.a_lin[p];
  b.assign(c.b_lin, c.b_lin + c.n);
  for (int k = 0; k < c.n_elems; k++) {
    if (is_broken(c, k)) {  // 003_create_electric_system.cpp:252-255: a linear wire
      add_admittance(A, c.hi[k], c.lo[k], c.g_wire);
      if (didiph) (*didiph)[k] = 0.0;
      continue;
    }
    double cur, didv, dphi;
    pvglu_panel_iv3(&c.panel, iph[k], v[k], &cur, &didv, &dphi);
    const double f = -cur, G = -didv;
    const double ieq = f - G * v[k];
    add_admittance(A, c.hi[k], c.lo[k], G);
    add_current_source(b, c.hi[k], c.lo[k], -ieq);
    if (gmin > 0) add_admittance(A, c.hi[k], c.lo[k], gmin);
    if (didiph) (*didiph)[k] = dphi;
  }
  a_vals.assign(c.rowptr[c.n], 0.0);
  size_t count = 0;
  for (int i = 0; i < c.n; i++) {
    count += A[i].size();
    for (int p = c.rowptr[i]; p < c.rowptr[i + 1]; p++) a_vals[p] = A[i][c.colidx[p]];
  }
  return count == (size_t)c.rowptr[c.n];
}

}  // namespace

extern "C" {

// Outcome: 0 converged, 2 iteration limit, 3 damping below 1e-13, 4 pivot
// failure, 5 stamp outside the pattern.  v: element voltages in/out; x: the
// last linear solution (caller order); iterations and the last diff out.
int oracle_newton(void* sym, int n, const int* rowptr, const int* colidx, const double* a_lin,
                  const double* b_lin, int n_elems, const int* hi, const int* lo, double i0,
                  double a, double rs, double rsh, const int* broken, double r_wire,
                  const double* iph, double* v, const double* gmin, int n_stages, double tol,
                  int max_iterations, double* x, int* iterations, double* last_diff) {
  const Circuit c{n,     n_elems, rowptr, colidx, hi, lo, a_lin, b_lin, {i0, a, rs, rsh},
                  broken, 1.0 / r_wire};
  const int* csc_row = nullptr;
  long long nnz_lu = 0;
  oracle_get(sym, "csc_row", &csc_row, &nnz_lu);
  std::vector<double> lu(nnz_lu), a_vals, b, sol(n, 0.0);
  std::vector<double> movement(n_elems), cand(n_elems), newv(n_elems);
  int it = 0;
  long double diff = 0;
  for (int stage = 0; stage < n_stages; stage++) {
    diff = 1e10L;
    for (;;) {
      if (diff < (long double)tol) break;
      if (++it > max_iterations) {
        *iterations = it - 1;
        *last_diff = (double)diff;
        return 2;
      }
      if (!assemble(c, iph, v, gmin[stage], a_vals, b, nullptr)) return 5;
      if (oracle_scatter_refactor_solve(sym, a_vals.data(), lu.data(), b.data(), 1)) {
        *iterations = it;
        return 4;
      }
      sol = b;
      for (int k = 0; k < n_elems; k++) {
        newv[k] = (hi[k] >= 0 ? sol[hi[k]] : 0.0) - (lo[k] >= 0 ? sol[lo[k]] : 0.0);
        movement[k] = 1.0;
      }
      // A wire is not a nonlinear element: it takes its new voltage drop and
      // is not part of the damping or of diff (011:37-90 only walks the
      // nonlinear sources).
      auto nonlinear = [&](int k) { return !is_broken(c, k); };
      for (;;) {
        for (int k = 0; k < n_elems; k++)
          cand[k] = nonlinear(k) ? v[k] * (1.0 - movement[k]) + newv[k] * movement[k] : newv[k];
        for (int k = 0; k < n_elems; k++)
          if (nonlinear(k) && movement[k] < 1e-13) {
            *iterations = it;
            for (int i = 0; i < n; i++) x[i] = sol[i];
            return 3;
          }
        bool reduce = false;
        for (int k = 0; k < n_elems; k++) {
          const bool ok = !nonlinear(k) || (!std::isnan(v[k]) && !std::isnan(cand[k]) &&
                                            !(std::fabs(v[k] - cand[k]) > 1.0));
          if (ok) continue;
          movement[k] /= 2.0;
          reduce = true;
        }
        if (!reduce) break;
      }
      diff = 0;
      for (int k = 0; k < n_elems; k++) {
        if (nonlinear(k)) diff += std::fabs(cand[k] - v[k]);
        v[k] = cand[k];
      }
    }
  }
  for (int i = 0; i < n; i++) x[i] = sol[i];
  *iterations = it;
  *last_diff = (double)diff;
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Central difference of a linear objective P = dpdx . x with respect to the
// photocurrent of element k, in extended precision (long double: a 64-bit
// significand on x86-64, 113 bits on aarch64).
//
// FP64 cannot resolve such a difference to 1e-6 at small steps: node
// voltages near 1 kV are quantised at 2.3e-13 V, which through a 0.02 ohm
// cable is 1.1e-11 A of inverter current, 1.2e-8 W at the inverter voltage,
// while one panel's 1e-3 W/m^2 step moves the plant power by about 5e-4 W.
// So the two perturbed operating points are solved here with the node
// voltages held in long double: Newton in correction form, the nonlinear
// residual b_lin - A_lin x - incidence f(V) evaluated in long double with the
// panel law solved in long double, the correction solved with the FP64
// Jacobian through the oracle's GLU.  That converges to the long double
// solution whenever FP64 factors of J give a contraction (cond(J) eps64 < 1).
// Start: the FP64 element voltages v0 (e.g. a converged FP64 operating
// point).  Outputs the difference quotient (P(+delta) - P(-delta)) / (2 delta),
// the Newton iterations of each side and the largest final residual [A].
// Returns 0, 4 (pivot failure), 5 (stamp outside the pattern) or 6 (no
// convergence within max_iter).

namespace {

using ld_t = long double;

// I(V) of the single-diode panel (panel_model.h) solved in long double by
// Newton on g(I) = Iph - I0 (exp((V + I Rs) / a) - 1) - (V + I Rs) / Rsh - I,
// from the start value *cur (the previous solution of this element, or the
// FP64 law's value); also dI/dV.  Stops when a step is within a few ulps of
// long double or stops shrinking.
void panel_iv_ext(const pvglu_panel_params& p, ld_t iph, ld_t v, ld_t* cur, ld_t* didv) {
  const ld_t eps = std::numeric_limits<ld_t>::epsilon();
  const ld_t i0 = p.i0, a = p.a, rs = p.rs, rsh = p.rsh;
  ld_t i = *cur, e = 0, last = 1e300L;
  for (int it = 0; it < 60; it++) {
    const ld_t vd = v + i * rs;
    e = expl(vd / a);
    const ld_t g = iph - i0 * (e - 1.0L) - vd / rsh - i;
    const ld_t dg = -i0 * e * rs / a - rs / rsh - 1.0L;
    const ld_t step = g / dg;
    i -= step;
    const ld_t mag = fabsl(step);
    if (mag <= 4.0L * eps * (fabsl(i) + 1.0L) || mag >= last) break;
    last = mag;
  }
  e = expl((v + i * rs) / a);
  const ld_t gd = i0 * e / a + 1.0L / rsh;  // -dI/dVd
  *cur = i;
  *didv = -gd / (1.0L + rs * gd);
}

}  // namespace

extern "C" int oracle_fd_ext(void* sym, int n, const int* rowptr, const int* colidx,
                             const double* a_lin, const double* b_lin, int n_elems,
                             const int* hi, const int* lo, double i0, double a, double rs,
                             double rsh, const double* iph, const double* v0, const double* dpdx,
                             int k, double delta, int max_iter, double* fd_out,
                             int* iterations_out, double* resid_out) {
  const Circuit c{n, n_elems, rowptr, colidx, hi, lo, a_lin, b_lin, {i0, a, rs, rsh}, nullptr, 0};
  const int* csc_row = nullptr;
  long long nnz_lu = 0;
  oracle_get(sym, "csc_row", &csc_row, &nnz_lu);
  std::vector<double> lu(nnz_lu), a_vals, b, vd(n_elems), iphd(iph, iph + n_elems);
  std::vector<ld_t> x(n), r(n), icur(n_elems);
  ld_t P[2] = {0, 0};
  double worst = 0.0;
  for (int side = 0; side < 2; side++) {
    const ld_t sign = side == 0 ? 1.0L : -1.0L;
    const ld_t iph_k = (ld_t)iph[k] + sign * (ld_t)delta;
    // Start: one FP64 linear solve at v0.
    for (int e = 0; e < n_elems; e++) vd[e] = v0[e];
    if (!assemble(c, iphd.data(), vd.data(), -1.0, a_vals, b, nullptr)) return 5;
    if (oracle_scatter_refactor_solve(sym, a_vals.data(), lu.data(), b.data(), 1)) return 4;
    for (int i = 0; i < n; i++) x[i] = b[i];
    for (int e = 0; e < n_elems; e++) {
      double cur64, didv64, dphi64;
      pvglu_panel_iv3(&c.panel, iph[e], v0[e], &cur64, &didv64, &dphi64);
      icur[e] = cur64;
    }
    ld_t best = 1e300L;
    int stall = 0, it = 0;
    bool done = false;
    for (it = 1; it <= max_iter && !done; it++) {
      // Residual in long double, the linear part in branch form:
      // sum_j a_ij x_j = (sum_j a_ij) x_i + sum_{j != i} a_ij (x_j - x_i).
      // Node rows of pure conductances have a zero row sum, so no product
      // of a large conductance sum with a 1 kV voltage is formed and the
      // floor is that of the branch currents themselves.
      for (int i = 0; i < n; i++) {
        ld_t rowsum = 0, acc = 0;
        for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
          rowsum += (ld_t)a_lin[p];
          if (colidx[p] != i) acc += (ld_t)a_lin[p] * (x[colidx[p]] - x[i]);
        }
        r[i] = ((ld_t)b_lin[i] - rowsum * x[i]) - acc;
      }
      for (int e = 0; e < n_elems; e++) {
        const ld_t ve = (hi[e] >= 0 ? x[hi[e]] : 0.0L) - (lo[e] >= 0 ? x[lo[e]] : 0.0L);
        ld_t didv;
        panel_iv_ext(c.panel, e == k ? iph_k : (ld_t)iph[e], ve, &icur[e], &didv);
        const ld_t f = -icur[e];  // element current hi -> lo
        if (hi[e] >= 0) r[hi[e]] -= f;
        if (lo[e] >= 0) r[lo[e]] += f;
        vd[e] = (double)ve;
      }
      ld_t rmax = 0;
      for (int i = 0; i < n; i++) rmax = fmaxl(rmax, fabsl(r[i]));
      if (rmax < best * 0.5L) {
        best = rmax;
        stall = 0;
      } else if (++stall >= 3) {
        done = true;  // at the long double floor
        break;
      }
      // Correction with the FP64 Jacobian at the current voltages.
      if (!assemble(c, iphd.data(), vd.data(), -1.0, a_vals, b, nullptr)) return 5;
      for (int i = 0; i < n; i++) b[i] = (double)r[i];
      if (oracle_scatter_refactor_solve(sym, a_vals.data(), lu.data(), b.data(), 1)) return 4;
      for (int i = 0; i < n; i++) x[i] += b[i];
    }
    if (!done) return 6;
    worst = std::max(worst, (double)best);
    iterations_out[side] = it;
    ld_t pv = 0;
    for (int i = 0; i < n; i++) pv += (ld_t)dpdx[i] * x[i];
    P[side] = pv;
  }
  *fd_out = (double)((P[0] - P[1]) / (2.0L * (ld_t)delta));
  *resid_out = worst;
  return 0;
}

extern "C" {

// Adjoint check: J at the iterate v without convergence conductance,
// J^T lambda = dpdx through the oracle's factors and permutations, then
// dP/dIph[k] = dI/dIph * (lambda[hi] - lambda[lo]).  Returns 0, 4 (pivot) or 5.
int oracle_adjoint(void* sym, int n, const int* rowptr, const int* colidx, const double* a_lin,
                   const double* b_lin, int n_elems, const int* hi, const int* lo, double i0,
                   double a, double rs, double rsh, const int* broken, double r_wire,
                   const double* iph, const double* v, const double* dpdx, double* dpdiph) {
  const Circuit c{n,     n_elems, rowptr, colidx, hi, lo, a_lin, b_lin, {i0, a, rs, rsh},
                  broken, 1.0 / r_wire};
  const int *csc_row = nullptr, *perm_amd = nullptr, *perm_rows = nullptr;
  long long nnz_lu = 0, len = 0;
  oracle_get(sym, "csc_row", &csc_row, &nnz_lu);
  oracle_get(sym, "perm_amd", &perm_amd, &len);
  oracle_get(sym, "perm_rows", &perm_rows, &len);
  std::vector<double> lu(nnz_lu), a_vals, b, dphi(n_elems);
  if (!assemble(c, iph, v, -1.0, a_vals, b, &dphi)) return 5;
  oracle_scatter(sym, a_vals.data(), lu.data());
  int bad = -1;
  if (oracle_refactor_sequential(sym, lu.data(), &bad)) return 4;
  // J x = b is M y = R b, x = C y (x[perm_amd[i]] = y[i]); so J^T l = g is
  // M^T z = C^T g with l = R^T z.
  std::vector<int> perm_amd_rev(n);
  for (int i = 0; i < n; i++) perm_amd_rev[perm_amd[i]] = i;
  std::vector<double> w(n), t(n), lam(n);
  for (int i = 0; i < n; i++) w[i] = dpdx[perm_amd[i]];
  oracle_solve_transposed(sym, lu.data(), w.data());
  for (int i = 0; i < n; i++) t[i] = w[perm_rows[i]];
  for (int i = 0; i < n; i++) lam[i] = t[perm_amd_rev[i]];
  for (int k = 0; k < n_elems; k++) {
    const double lh = hi[k] >= 0 ? lam[hi[k]] : 0.0;
    const double ll = lo[k] >= 0 ? lam[lo[k]] : 0.0;
    dpdiph[k] = dphi[k] * (lh - ll);
  }
  return 0;
}

}  // extern "C"
