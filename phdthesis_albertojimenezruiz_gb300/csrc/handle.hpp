// Internal handle layout shared by the translation units of libpvglu
// (capi.cu: hot path; newton.cu: structured Jacobians, Newton, adjoint).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pvglu.h"
#include "kernels.cuh"
#include "persistent.cuh"
#include "symbolic.hpp"

namespace pvglu {
// Records the message returned by pvglu_last_error() and passes `code` on.
int fail(int code, const std::string& msg);
}  // namespace pvglu
using pvglu::fail;

#define PVGLU_CUDA(call)                                                       \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return fail(PVGLU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int upload(const std::vector<T>& h, T** d) {
  *d = nullptr;
  const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
  PVGLU_CUDA(cudaMalloc((void**)d, bytes));
  if (!h.empty()) PVGLU_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return PVGLU_OK;
}

struct pvglu_symbolic {
  pvglu::Symbolic s;
};

struct pvglu_numeric {
  const pvglu_symbolic* sym = nullptr;
  int n = 0, nnz = 0, nnz_a = 0;
  int S = 0, ld = 0, precision = PVGLU_FP64;
  int device = 0;               // CUDA device the handle's memory lives on
  int schedule = PVGLU_SCHED_LEVELS;
  double pivot_tol = 1e-8;
  pvglu::DevStruct d{};
  std::vector<void*> allocs;
  void* values = nullptr;       // [nnz * ld] T
  void* work = nullptr;         // [n * ld] T
  double* work64 = nullptr;     // [nnz_a * ld] staging / [n * ld] vectors
  double* b64 = nullptr;        // [n * ld]
  double* x64 = nullptr;        // [n * ld]
  double* g64 = nullptr;        // [n_elems * ld] conductances of pvglu_refine_stamps_host
  size_t g64_count = 0;
  int* col_pos = nullptr;       // inverse of col_orig
  int* row_pos = nullptr;       // inverse of row_orig
  pvglu::DevStatus* status = nullptr;
  int* ir_done = nullptr;
  unsigned long long* ir_max_dx = nullptr;
  unsigned long long* ir_max_x = nullptr;
  double* ir_prev_dx = nullptr;  // max|dx| of the previous sweep
  int* ir_sweeps_done = nullptr;  // sweep counter of the graph-replayed refinement
  // Refinement replayed from a graph whose sweeps run under a conditional
  // while node (run_refine); rebuilt when its launch arguments change.
  struct RefineKey {
    pvglu::AValues A;
    const double* b;
    double* x;
    int* sweeps_out;
    const int* init_done;
    double tol;
    int transpose, max_sweeps, schedule;
    bool operator==(const RefineKey& o) const {
      return A.a == o.A.a && A.base == o.A.base && A.ptr == o.A.ptr && A.elem == o.A.elem &&
             A.sign == o.A.sign && A.g == o.A.g && A.gmin == o.A.gmin && A.linear == o.A.linear &&
             b == o.b && x == o.x && sweeps_out == o.sweeps_out && init_done == o.init_done &&
             tol == o.tol && transpose == o.transpose && max_sweeps == o.max_sweeps &&
             schedule == o.schedule;
    }
  };
  RefineKey ir_key{};
  cudaGraphExec_t ir_graph = nullptr;
  cudaStream_t ir_cap[2] = {nullptr, nullptr};  // capture streams: outer, loop body
  bool ir_graph_failed = false;
  // Host copies of the level starts (launch ranges).
  std::vector<int> lu_sl, l_sl, u_sl, lt_sl;
  // Chain programs: refactor, L, U, U^T, L^T (programs.hpp).
  bool batch = false;              // ld > 1: lane = scenario
  int sm_count = 1;
  int resid_blocks = 1;             // resident blocks of k_residual_rows
  int max_locals = 0;               // table budget of levels with many chains
  int table_max = 0;                // widest table of any level (shared memory size)
  std::vector<int> prog_level_ml[5];  // table budget per phase and level
  pvglu::ProgSetDev progs{};
  std::vector<int> prog_level_chain[5];
  std::vector<int> prog_level_wide_len[5];  // per program level: 0, or (WIDE level) its
                                            // widest unit, for the launch's shared memory
  int prog_max_chains = 1;
  int prog_grid = 0;               // co-resident blocks of k_prog_persistent
  size_t smem_optin = 48 * 1024;   // shared memory a block may opt in to
  int64_t prog_ops = 0, prog_loads = 0, prog_wide_units = 0, prog_wide_levels = 0;
  unsigned int* barrier = nullptr;  // [2]: count, generation
  // A^T by rows (caller order): entries at_ptr[j]..at_ptr[j+1] of column j
  // of A, in row order, with their row and A-entry index.
  int* at_ptr = nullptr;
  int* at_row = nullptr;
  int* at_entry = nullptr;
  // Structured Jacobian (pvglu_numeric_set_stamps); n_elems = 0 until set.
  int n_elems = 0;
  std::vector<void*> stamp_allocs;
  double* st_base = nullptr;
  int* st_ptr = nullptr;
  int* st_elem = nullptr;
  int* st_sign = nullptr;
  pvglu::AValues stamps(const double* g, const double* gmin,
                        const int* linear = nullptr) const {
    return pvglu::AValues{nullptr, st_base, st_ptr, st_elem, st_sign, g, gmin, linear};
  }
  ~pvglu_numeric() {
    if (ir_graph) cudaGraphExecDestroy(ir_graph);
    for (cudaStream_t c : ir_cap)
      if (c) cudaStreamDestroy(c);
    for (void* p : allocs) cudaFree(p);
    for (void* p : stamp_allocs) cudaFree(p);
  }
  template <typename T>
  int put(const std::vector<T>& h, const T** out) {
    T* d = nullptr;
    int st = upload(h, &d);
    if (st) return st;
    allocs.push_back(d);
    *out = d;
    return PVGLU_OK;
  }
  template <typename T>
  int alloc(size_t count, T** out) {
    PVGLU_CUDA(cudaMalloc((void**)out, std::max<size_t>(count, 1) * sizeof(T)));
    allocs.push_back(*out);
    return PVGLU_OK;
  }
};


// Launch sequences of capi.cu shared with newton.cu.  All are asynchronous on
// `st`; vectors are [n x ld] in pivot order ("perm") or the caller's order.
namespace pvglu {
int run_scatter(pvglu_numeric* h, const AValues& A, const int* ndone, cudaStream_t st);
// skip.ndone (or NULL): nothing runs once every scenario is done; the
// refactorization itself never skips single scenarios.
int run_refactor(pvglu_numeric* h, cudaStream_t st, SkipDone skip = SkipDone{nullptr, nullptr});
// Scatter + refactor from A's FP64 values (one pass where the programs allow).
int run_scatter_refactor(pvglu_numeric* h, const double* a, cudaStream_t st);
// Solve in pivot order in place (x: T = double or float per the handle).
int run_solve_perm(pvglu_numeric* h, void* x, bool transpose, SkipDone skip, cudaStream_t st);
// Refactor + pivot-order solve; one persistent launch where the schedule has it.
int run_refactor_solve_perm(pvglu_numeric* h, void* x, bool transpose, SkipDone skip,
                            cudaStream_t st);
// FP32 factors + FP64 refinement of J x = b (J^T x = b): x, b in caller order.
// init_done (or NULL): scenarios flagged there are left alone, x included.
int run_refine(pvglu_numeric* h, const AValues& A, const double* b, double* x, bool transpose,
               double tol, int max_sweeps, int* sweeps_out, cudaStream_t st,
               const int* init_done = nullptr);
}  // namespace pvglu
