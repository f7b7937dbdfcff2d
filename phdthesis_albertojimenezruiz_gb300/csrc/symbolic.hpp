// Host-side symbolic analysis of the PV-plant Jacobian pattern.
//
// One `Symbolic` object is built once per plant topology and then shared by
// every numeric refactorization / solve of that topology (any number of
// scenarios).  It reproduces the reference's symbolic pipeline, step by step:
//
//   ordering  : PVPP_Plant_Simulator/004a_algorithm_amd_function.cpp:10-50
//               (AMD is third-party code; the caller may pass its permutation,
//               otherwise a minimum-degree ordering of our own is used)
//   row swaps : 004b_remove_zeros_diagonal.cpp:12-100 (move_only_rows=true)
//   fill-in   : 005a_obtain_fillin_matrix_CUDA.cu:18-236 + 005c:4-14
//   deps      : 006_get_dependencies_GLU.cpp:5-77
//   levels    : 007_convert_dependencies_in_levels.cpp:4-210
//   flatten   : 008_convert_chains_columns_levels_into_vector.cpp:4-30
//   max nnz   : 009_get_max_numbers_per_column.cpp:3-31
//   CSR/CSC   : 010_create_CSR_CSC.cpp:15-128
//
// and adds the GB300 execution structures (value-slot maps, left-looking
// update targets, row-gather solve lists, transposed-solve levels).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pvglu {

// Level -> chain -> column lists in the reference's flattened form
// (008_convert_chains_columns_levels_into_vector.cpp:4-30).
struct LevelSet {
  std::vector<int> start_levels;   // [#levels + 1] index into start_chains
  std::vector<int> start_chains;   // [#chains + 1] index into columns
  std::vector<int> columns;        // [n] column ids, chain after chain
  int num_levels() const { return (int)start_levels.size() - 1; }
  int num_chains() const { return (int)start_chains.size() - 1; }
};

struct SymbolicOptions {
  int compute_transposed_levels = 1;  // levels for the L^T backward solve
};

struct Symbolic {
  int n = 0;
  int64_t nnz_a = 0;   // entries of the input pattern
  int64_t nnz_lu = 0;  // entries after fill

  // Input pattern, original unknown order, rows sorted.
  std::vector<int> a_rowptr, a_colidx;

  // Orderings, reference semantics:
  //   perm_amd  == interchanges_position_row_columns        (P, 004a:40-42)
  //   perm_rows == interchanges_position_row_columns_only_rows (Q, 004b:94-95)
  // LU matrix M(r, c) = A(row_orig[r], col_orig[c]) with
  //   row_orig[r] = P[Q[r]], col_orig[c] = P[c].
  std::vector<int> perm_amd, perm_rows, row_orig, col_orig;
  int row_swaps = 0;
  int perm_rows_is_involution = 1;  // 1 when the reference's Newton-loop row
                                    // exchange (000:196) equals the symbolic one

  // Filled pattern by rows (reference `nonzero_values`, 005a:205-223).
  std::vector<int> fill_rowptr, fill_col;

  // 010: CSR / CSC of the filled matrix and cross maps.
  std::vector<int> csr_rowptr, csr_col, csc_colptr, csc_row;
  std::vector<int> csr_to_csc, csc_to_csr;
  std::vector<int> csr_diag_start, csc_diag_start;  // first strictly off-diag

  // 006/007/008 level sets: LU refactor, L solve, U solve; plus the level
  // set of the transposed-L solve (deps {i > j : L(i,j) != 0}), which the
  // reference does not need (no adjoint there).
  LevelSet lu, l, u, lt;
  std::vector<int> max_elements_per_column;  // 009, one per LU level

  // ---- GB300 execution structures ----
  std::vector<int> diag_slot;      // [n] CSC slot of M(j,j)
  std::vector<int> slot_src;       // [nnz_lu] index into A's CSR values or -1
  // Left-looking refactor: for every U slot p (row j < column k) the target
  // slots in column k of the |L_j| updates A(i,k) -= L(i,j) * U(j,k),
  // i running over column j's L rows in CSC order.
  std::vector<int64_t> upd_ptr;    // [nnz_lu + 1] (only U slots non-empty)
  std::vector<int> upd_tgt;        // [sum_j |L_j| * |U_j|]
  // Row-gather lists for the forward solves.
  std::vector<int> lrow_ptr, lrow_slot, lrow_col;  // strictly lower, by rows
  std::vector<int> urow_ptr, urow_slot, urow_col;  // strictly upper, by rows
  int64_t update_count = 0;        // sum_j |L_j| * |U_j|
  double flops_refactor = 0;       // sum_j (|L_j| + 2 |L_j| |U_j|)

  // Dependence hazards of the reference's right-looking level schedule:
  // pairs (j', j) with L(j, j') != 0 and some U(j', k), U(j, k) != 0 where
  // j' is not scheduled before j.  Reported, never acted on: the left-looking
  // kernels here only need the U-column dependencies, which 006 provides.
  int64_t right_looking_hazards = 0;
};

// Status codes shared with the C ABI.
enum Status : int {
  OK = 0,
  ERR_BAD_ARG = 1,
  ERR_STRUCTURAL = 2,   // no row to swap into a zero diagonal (004b:82)
  ERR_ZERO_PIVOT = 3,
  ERR_NONFINITE = 4,
  ERR_CUDA = 5,
  ERR_BARRIER_TIMEOUT = 6,
  ERR_NOT_CONVERGED = 7,
  ERR_NO_MEMORY = 8,
  ERR_TOO_LARGE = 9,
};

// Builds the full symbolic analysis.  `perm` (length n) is P in the
// reference's semantics, or nullptr for the built-in minimum-degree ordering.
int build_symbolic(int n, const int* rowptr, const int* colidx, const int* perm,
                   const SymbolicOptions& opt, Symbolic& out, std::string& err);

// Dump format of a complete analysis (symbolic_io.cpp).
int save_symbolic(const Symbolic& s, const char* path, std::string& err);
int load_symbolic(const char* path, Symbolic& s, std::string& err);

// Minimum-degree ordering of the pattern of A + A^T (exact degrees on the
// explicit elimination graph; ties broken by the smallest index).
void minimum_degree_order(int n, const std::vector<int>& rowptr,
                          const std::vector<int>& colidx, std::vector<int>& perm);

// 007 restated: dependency lists (ascending) -> chains of columns per level.
void build_levels(const std::vector<std::vector<int>>& deps, LevelSet& out);

}  // namespace pvglu
