// ORACLE — test infrastructure only (builds only where the reference sources
// are present; never shipped, never linked by the product).
//
// A C entry layer around the reference's OWN source code, compiled from where
// it lies by oracle/Makefile.ref into oracle/_ref/libpvref.so.  It runs the
// reference's symbolic pipeline (prepare_matrices, PVPP_Plant_Simulator/
// 000_PVPP_simulator.cpp:10-93) and numeric CPU path (000:193-230) on a
// caller-given pattern and values, so that the CPU restatement in
// oracle_glu.cpp and the product can be checked against the reference itself.
//
// The reference computes the fill-in on the GPU (005a_obtain_fillin_matrix_
// CUDA.cu:18-236).  Its kernels are plain per-thread functions, so this file
// includes their headers with the CUDA qualifiers defined away and replays the
// host loop of 005a sequentially, one "thread" at a time: within a launch each
// thread only writes its own row (or benign identical flags), so the
// sequential replay computes what the GPU computes.
#include "main.h"
#include "matrix_functions.h"
#include "sparse_matrix.h"

#include <cstdint>
#include <numeric>
#include <string>

#define __host__
#define __device__
#define __global__
namespace {
struct FakeDim {
  unsigned int x, y, z;
};
FakeDim blockIdx{0, 0, 0}, blockDim{1, 1, 1}, threadIdx{0, 0, 0};
}  // namespace
#include "calculate_new_temporary_memory_size_CUDA.cuh"
#include "check_possible_new_nonzeros_CUDA.h"
#include "get_rows_and_columns_to_be_processed_CUDA.cuh"
#include "kernel_calculate_new_sizes.cuh"
#include "put_new_values_matrix_CUDA.cuh"

// Reference functions defined in sources without a shared header.
void algorithm_amd_cpp(Sparse_Matrix<FLOATING_TYPE>& matrix,
                       std::vector<int>& interchanges_position_row_columns);
void remove_zeros_diagonal(Sparse_Matrix<FLOATING_TYPE>& input_output,
                           std::vector<int>& interchanges_position_row_columns,
                           bool move_only_rows);

namespace {

// One "launch": every thread index in [0, threads) in order.
template <typename F>
void launch(int threads, F f) {
  for (int t = 0; t < threads; t++) {
    threadIdx.x = (unsigned)t;
    f();
  }
}

// Inclusive prefix sum; what call_cumsum_CUDA (005b_cumsum_CUDA.cu:23-31)
// computes with its blocked doubling launches.
void cumsum(std::vector<int>& a) { std::partial_sum(a.begin(), a.end(), a.begin()); }

// Host replay of obtain_fillin_matrix_CUDA (005a:18-236).
vector<vector<int>> obtain_fillin_host(Sparse_Matrix<FLOATING_TYPE>& m) {
  const int n = (int)m.m;
  int *sr = nullptr, *pc = nullptr;
  create_csr_boolean(m.convert_to_boolean_equivalent_rowmajor(), sr, pc);
  std::vector<int> start(sr, sr + n + 1), pos(pc, pc + sr[n]);
  free(sr);
  free(pc);
  std::vector<int> new_start(n + 1, 0), written(n, 0);
  std::vector<uint8_t> rows_p(n, 1), cols_p(n, 1), added_r(n, 0), added_c(n, 0);
  std::vector<int> row_tmp(n + 1, 0), new_row_tmp(n + 1, 0);
  std::vector<int> data_tmp(row_tmp[n]);
  bool added_zero = false, must_alloc = false;
  for (;;) {
    for (;;) {
      std::fill(written.begin(), written.end(), 0);
      std::fill(added_r.begin(), added_r.end(), 0);
      std::fill(added_c.begin(), added_c.end(), 0);
      added_zero = false;
      must_alloc = false;
      int* dt = data_tmp.empty() ? nullptr : data_tmp.data();
      launch(n, [&] {
        check_possible_new_nonzeros_CUDA(start.data(), pos.data(), n, dt,
                                         row_tmp.data(), written.data(),
                                         rows_p.data(), cols_p.data(),
                                         added_r.data(), added_c.data(),
                                         &added_zero, &must_alloc);
      });
      if (!must_alloc) break;
      launch(n, [&] {
        calculate_new_temporary_memory_size(n, row_tmp.data(), new_row_tmp.data(),
                                            written.data());
      });
      cumsum(new_row_tmp);
      std::swap(row_tmp, new_row_tmp);
      data_tmp.assign(row_tmp[n], 0);
    }
    launch(n, [&] {
      calculate_new_matrix_sizes_only_row_length_CUDA(n, start.data(), written.data(),
                                                      new_start.data());
    });
    cumsum(new_start);
    std::vector<int> new_pos(new_start[n]);
    const int* dt = data_tmp.empty() ? nullptr : data_tmp.data();
    launch(n, [&] {
      put_new_values_matrix_CUDA(n, start.data(), pos.data(), new_start.data(),
                                 new_pos.data(), row_tmp.data(), dt, written.data());
    });
    launch(n, [&] {
      get_rows_and_columns_to_be_processed(n, rows_p.data(), cols_p.data(),
                                           added_r.data(), added_c.data(),
                                           pos.data(), start.data());
    });
    std::swap(start, new_start);
    pos = new_pos;
    if (!added_zero) break;
  }
  vector<vector<int>> res(n);
  for (int i = 0; i < n; i++) res[i].assign(pos.begin() + start[i], pos.begin() + start[i + 1]);
  return res;
}

struct Ref {
  int n = 0;
  Sparse_Matrix<FLOATING_TYPE> a;  // original pattern + values of the last scatter
  std::vector<int> a_rowptr, a_colidx;
  std::vector<int> perm_amd, perm_amd_rev, perm_rows, perm_rows_rev;
  std::vector<int> fill_rowptr, fill_col;
  std::vector<int> lu_sl, lu_sc, lu_cols, l_sl, l_sc, l_cols, u_sl, u_sc, u_cols;
  std::vector<int> max_elements_per_column;
  std::vector<int> csr_rowptr, csr_col, csc_colptr, csc_row, csr_to_csc, csc_to_csr,
      csr_diag_start, csc_diag_start;
  std::vector<FLOATING_TYPE> csr_vals, csc_vals;
};

}  // namespace

extern "C" {

// prepare_matrices (000:10-93).  perm == nullptr runs the reference's own
// reorder_matrix (AMD + row exchanges, 004d:27-47); otherwise P is taken from
// the caller and only the row exchanges of 004b run.
void* ref_symbolic(int n, const int* rowptr, const int* colidx, const int* perm) {
  auto* r = new Ref();
  r->n = n;
  r->a_rowptr.assign(rowptr, rowptr + n + 1);
  r->a_colidx.assign(colidx, colidx + rowptr[n]);
  r->a = Sparse_Matrix<FLOATING_TYPE>(n, n);
  for (int i = 0; i < n; i++)
    for (int p = rowptr[i]; p < rowptr[i + 1]; p++) r->a.write(i, colidx[p], 1.0);
  Sparse_Matrix<FLOATING_TYPE> m;
  if (!perm) {
    m = reorder_matrix(r->a, r->perm_amd, r->perm_rows);
  } else {
    r->perm_amd.assign(perm, perm + n);
    std::vector<int> pinv = invert_permutation(r->perm_amd);
    m = r->a.interchange_row_columns(pinv.data());
    r->perm_rows.resize(n);
    for (int i = 0; i < n; i++) r->perm_rows[i] = i;
    remove_zeros_diagonal(m, r->perm_rows, true);
  }
  r->perm_amd_rev = invert_permutation(r->perm_amd);
  r->perm_rows_rev = invert_permutation(r->perm_rows);
  auto nz = obtain_fillin_host(m);
  fill_fillins(nz, m);
  r->fill_rowptr.assign(1, 0);
  for (int i = 0; i < n; i++) {
    r->fill_col.insert(r->fill_col.end(), nz[i].begin(), nz[i].end());
    r->fill_rowptr.push_back((int)r->fill_col.size());
  }
  auto lu = convert_dependence_list_in_chains_of_columns(get_dependencies_GLU_3_0(n, nz));
  auto l = convert_dependence_list_in_chains_of_columns(get_dependencies_matrix_L(n, nz));
  auto u = convert_dependence_list_in_chains_of_columns(get_dependencies_matrix_U(n, nz));
  r->max_elements_per_column = get_max_numbers_per_column(lu, nz);
  convert_chains_columns_levels_into_vector(lu, r->lu_sl, r->lu_sc, r->lu_cols);
  convert_chains_columns_levels_into_vector(l, r->l_sl, r->l_sc, r->l_cols);
  convert_chains_columns_levels_into_vector(u, r->u_sl, r->u_sc, r->u_cols);
  create_CSR_CSC_matrices(m, r->csr_rowptr, r->csr_col, r->csr_vals, r->csc_colptr,
                          r->csc_row, r->csc_vals, r->csr_to_csc, r->csc_to_csr,
                          r->csr_diag_start, r->csc_diag_start);
  return r;
}

void ref_free(void* h) { delete static_cast<Ref*>(h); }

int ref_get(void* h, const char* name, const int** ptr, long long* len) {
  auto* o = static_cast<Ref*>(h);
  const std::vector<int>* v = nullptr;
  const std::string s(name);
#define PVG(x) if (s == #x) v = &o->x;
  PVG(perm_amd) PVG(perm_rows) PVG(fill_rowptr) PVG(fill_col)
  PVG(lu_sl) PVG(lu_sc) PVG(lu_cols) PVG(l_sl) PVG(l_sc) PVG(l_cols)
  PVG(u_sl) PVG(u_sc) PVG(u_cols) PVG(max_elements_per_column) PVG(csr_rowptr)
  PVG(csr_col) PVG(csc_colptr) PVG(csc_row) PVG(csr_to_csc) PVG(csc_to_csr)
  PVG(csr_diag_start) PVG(csc_diag_start)
#undef PVG
  if (!v) return 1;
  *ptr = v->data();
  *len = (long long)v->size();
  return 0;
}

// Newton-iteration value path (000:193-210): permute A, exchange rows,
// fill_values_CSC_only (010:142-155).
int ref_scatter(void* h, const double* a_vals, double* csc_vals) {
  auto* r = static_cast<Ref*>(h);
  Sparse_Matrix<FLOATING_TYPE> a(r->n, r->n);
  for (int i = 0; i < r->n; i++)
    for (int p = r->a_rowptr[i]; p < r->a_rowptr[i + 1]; p++)
      a.write(i, r->a_colidx[p], a_vals[p]);
  a = a.interchange_row_columns(r->perm_amd_rev.data());
  a = a.exchange_rows(r->perm_rows.data());
  std::vector<FLOATING_TYPE> v(r->csc_row.size());
  fill_values_CSC_only(a, r->csc_colptr, r->csc_row, v);
  std::copy(v.begin(), v.end(), csc_vals);
  return 0;
}

// factorize_all_chains_of_columns_in_level_GLU_CSC_CPU over every LU level
// (GLU_CSC_CPU_levels_strings.cpp:65-106).  The reference asserts on a tiny
// pivot; callers only pass non-singular matrices.
int ref_refactor_levels(void* h, double* v) {
  auto* r = static_cast<Ref*>(h);
  for (int lv = 0; lv + 1 < (int)r->lu_sl.size(); lv++)
    factorize_all_chains_of_columns_in_level_GLU_CSC_CPU(
        r->lu_sl.data(), lv, r->lu_sc.data(), r->lu_cols.data(), r->csr_rowptr.data(),
        r->csr_col.data(), r->csr_to_csc.data(), r->csc_colptr.data(),
        r->csc_row.data(), v, r->csr_diag_start.data(), r->csc_diag_start.data());
  return 0;
}

// GLU_CSC_CPU_sequential (GLU_CSC_CPU_levels_strings.cpp:108-132).
int ref_refactor_sequential(void* h, double* v) {
  auto* r = static_cast<Ref*>(h);
  GLU_CSC_CPU_sequential(r->n, r->csr_rowptr.data(), r->csr_col.data(),
                         r->csr_to_csc.data(), r->csc_colptr.data(), r->csc_row.data(),
                         v, r->csr_diag_start.data(), r->csc_diag_start.data());
  return 0;
}

// Substitute_LU_Vector_b_CSC_CPU (GLU_CSC_CPU_Triangular.cpp:27-43).
int ref_solve(void* h, const double* v, double* b) {
  auto* r = static_cast<Ref*>(h);
  Substitute_LU_Vector_b_CSC_CPU((unsigned)r->n, r->csc_colptr.data(), r->csc_row.data(),
                                 v, r->csc_diag_start.data(), b);
  return 0;
}

}  // extern "C"
