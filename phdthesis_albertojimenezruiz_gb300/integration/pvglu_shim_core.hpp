// Core of the drop-in shim (pvglu_shim.cpp): the reference's two GPU hot-path
// entry points, factorize_electrical_system_CUDA and
// triangular_substitution_LU_CUDA (PVPP_Plant_Simulator/
// factorize_electrical_system.h:136-145), expressed as C-ABI call sequences
// on libpvglu.
//
// Written against the members of the reference's struct_CPU_CUDA_arrays that
// the two entry points use, so any type with those members works:
//   int n;
//   std::vector<int> mat_A_CSR_start_rows, mat_A_CSR_position_columns;
//   std::vector<double> mat_A_CSC_values;
// In the reference these hold the Jacobian AFTER prepare_matrices
// (000_PVPP_simulator.cpp:10-93): reordered by P, rows exchanged for zero
// diagonals, fill added, CSC values scattered.  The pvglu analysis is
// therefore built from that filled, permuted pattern with the identity
// ordering: it finds no zero diagonal and no new fill, so its CSC slots,
// levels and chains are the reference's, and the values and solution
// vectors pass through in the reference's own (permuted) order.
//
// The handles are created on the first call and kept; a call with arrays of
// another pattern (different n or number of entries, or another
// mat_A_CSR_start_rows buffer) builds new ones.
#pragma once
#include <cstddef>
#include <vector>

#include "pvglu.h"

namespace pvglu_shim {

struct State {
  pvglu_symbolic* sym = nullptr;
  pvglu_numeric* num = nullptr;
  int n = -1;
  size_t nnz = 0;
  const int* rows = nullptr;
};

inline void release(State& st) {
  if (st.num) pvglu_numeric_destroy(st.num);
  if (st.sym) pvglu_symbolic_destroy(st.sym);
  st = State();
}

// Handles for the arrays' pattern, created when missing or stale.
template <class Arrays>
int ensure(State& st, const Arrays& a) {
  const int n = a.n;
  const size_t nnz = a.mat_A_CSR_position_columns.size();
  if (st.num && st.n == n && st.nnz == nnz && st.rows == a.mat_A_CSR_start_rows.data())
    return PVGLU_OK;
  release(st);
  if (n <= 0 || a.mat_A_CSR_start_rows.size() != (size_t)n + 1 ||
      a.mat_A_CSC_values.size() != nnz)
    return PVGLU_ERR_BAD_ARG;
  std::vector<int> identity(n);
  for (int i = 0; i < n; i++) identity[i] = i;
  int rc = pvglu_symbolic_create(n, a.mat_A_CSR_start_rows.data(),
                                 a.mat_A_CSR_position_columns.data(), identity.data(), &st.sym);
  if (rc == PVGLU_OK) rc = pvglu_numeric_create(st.sym, 1, PVGLU_FP64, &st.num);
  // One launch per level, as the reference's own GPU path runs them
  // (factorize_electrical_system_CUDA.cu:67-115).
  if (rc == PVGLU_OK) rc = pvglu_numeric_set_schedule(st.num, PVGLU_SCHED_LEVELS);
  if (rc != PVGLU_OK) {
    release(st);
    return rc;
  }
  st.n = n;
  st.nnz = nnz;
  st.rows = a.mat_A_CSR_start_rows.data();
  return PVGLU_OK;
}

// factorize_electrical_system_CUDA: the host CSC values are factorized in
// place (combined L and U, the reference's layout), host in, host out.
template <class Arrays>
int factorize(State& st, Arrays& a) {
  const int rc = ensure(st, a);
  return rc != PVGLU_OK ? rc : pvglu_refactor_host(st.num, a.mat_A_CSC_values.data());
}

// triangular_substitution_LU_CUDA: `solution` holds the permuted right-hand
// side on entry and the permuted solution on return, with the factors of the
// last factorize().
template <class Arrays>
int solve(State& st, Arrays& a, double* solution) {
  const int rc = ensure(st, a);
  return rc != PVGLU_OK ? rc : pvglu_solve_host(st.num, solution);
}

}  // namespace pvglu_shim
