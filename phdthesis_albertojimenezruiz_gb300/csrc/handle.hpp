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
  int schedule = PVGLU_SCHED_LEVELS;
  double pivot_tol = 1e-8;
  pvglu::DevStruct d{};
  std::vector<void*> allocs;
  void* values = nullptr;       // [nnz * ld] T
  void* work = nullptr;         // [n * ld] T
  double* work64 = nullptr;     // [nnz_a * ld] staging / [n * ld] vectors
  double* b64 = nullptr;        // [n * ld]
  double* x64 = nullptr;        // [n * ld]
  int* col_pos = nullptr;       // inverse of col_orig
  int* row_pos = nullptr;       // inverse of row_orig
  pvglu::DevStatus* status = nullptr;
  int* ir_done = nullptr;
  unsigned long long* ir_max_dx = nullptr;
  unsigned long long* ir_max_x = nullptr;
  // Host copies of the level starts (launch ranges).
  std::vector<int> lu_sl, l_sl, u_sl, lt_sl;
  // Chain programs: refactor, L, U, U^T, L^T (programs.hpp).
  bool batch = false;              // ld > 1: lane = scenario
  int max_locals = 0;
  pvglu::ProgSetDev progs{};
  std::vector<int> prog_level_chain[5];
  int prog_max_chains = 1;
  int prog_grid = 0;               // co-resident blocks of k_prog_persistent
  int64_t prog_ops = 0, prog_loads = 0, prog_direct = 0;
  unsigned int* barrier = nullptr;  // [2]: count, generation
  // Structured Jacobian (pvglu_numeric_set_stamps): entry e of A is
  // st_base[e] + sum over c in [st_ptr[e], st_ptr[e+1]) of st_sign[c] * g[st_elem[c]].
  int n_elems = 0;
  const double* st_base = nullptr;
  const int* st_ptr = nullptr;
  const int* st_elem = nullptr;
  const int* st_sign = nullptr;
  ~pvglu_numeric() {
    for (void* p : allocs) cudaFree(p);
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

