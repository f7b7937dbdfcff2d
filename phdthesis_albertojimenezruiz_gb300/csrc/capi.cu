// C ABI of the hot path (include/pvglu.h): handles, device structure upload,
// scatter / refactor / solve launch sequences, the mixed-precision refinement
// (replayed from a CUDA graph whose sweep loop is a conditional while node),
// the host-buffer steps, size-class groups and the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "handle.hpp"

namespace pvglu {
namespace {
thread_local std::string g_err;
}
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
}  // namespace pvglu
using pvglu::g_err;

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Chain merging of pvglu_numeric_create(_ex) and pvglu_autotune: the level
// set's own chains, or ladder merging where that removes at least half of
// the execution levels (the U solve of the reference's own plant topology
// goes from 100 levels to 2).  Where no level is removed, regrouping can
// only lengthen a narrow level's chains.
int default_merge(const pvglu::Symbolic& s) {
  int own = 0, ladder = 0;
  for (int kind = -1; kind <= 1; kind++) {
    own += pvglu::execution_level_count(s, kind, 0);
    ladder += pvglu::execution_level_count(s, kind, 2);
  }
  return 2 * ladder <= own ? 2 : 0;
}

int launch_blocks(int64_t threads, int block) {
  int64_t b = (threads + block - 1) / block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 1 << 30));
}

template <typename T>
int refactor_levels(pvglu_numeric* h, cudaStream_t st, const int* ndone) {
  T* v = static_cast<T*>(h->values);
  for (size_t lv = 0; lv + 1 < h->lu_sl.size(); lv++) {
    const int cb = h->lu_sl[lv], ce = h->lu_sl[lv + 1];
    const int64_t threads = (int64_t)(ce - cb) * h->ld;
    pvglu::k_refactor_level<T><<<launch_blocks(threads, 128), 128, 0, st>>>(
        h->d, v, h->ld, h->S, cb, ce, h->pivot_tol, h->status, ndone);
  }
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

template <typename T, int KIND>
void solve_phase(pvglu_numeric* h, const std::vector<int>& sl, T* x, const int* done,
                 cudaStream_t st) {
  const T* v = static_cast<const T*>(h->values);
  for (size_t lv = 0; lv + 1 < sl.size(); lv++) {
    const int cb = sl[lv], ce = sl[lv + 1];
    const int64_t threads = (int64_t)(ce - cb) * h->ld;
    pvglu::k_solve_level<T, KIND><<<launch_blocks(threads, 128), 128, 0, st>>>(
        h->d, v, x, h->ld, h->S, cb, ce, done);
  }
}

// Kernel attributes (dynamic shared memory above 48 KB) and the persistent
// grid size of the chain-program kernels of one handle.
template <typename T, bool B>
int prog_prepare(pvglu_numeric* h) {
  const void* fns[] = {(const void*)pvglu::k_prog_level<T, -1, B>,
                       (const void*)pvglu::k_prog_level<T, 0, B>,
                       (const void*)pvglu::k_prog_level<T, 1, B>,
                       (const void*)pvglu::k_prog_level<T, 2, B>,
                       (const void*)pvglu::k_prog_level<T, 3, B>,
                       (const void*)pvglu::k_wide_level<T, -1, B>,
                       (const void*)pvglu::k_wide_level<T, 0, B>,
                       (const void*)pvglu::k_wide_level<T, 1, B>,
                       (const void*)pvglu::k_wide_level<T, 2, B>,
                       (const void*)pvglu::k_wide_level<T, 3, B>};
  for (const void* f : fns)
    if (pvglu::allow_max_dynamic_smem(f) != cudaSuccess) return 1;
  if constexpr (B) {
    const void* half[] = {(const void*)pvglu::k_wide_level<T, -1, B, 1>,
                          (const void*)pvglu::k_wide_level<T, 0, B, 1>,
                          (const void*)pvglu::k_wide_level<T, 1, B, 1>,
                          (const void*)pvglu::k_wide_level<T, 2, B, 1>,
                          (const void*)pvglu::k_wide_level<T, 3, B, 1>};
    for (const void* f : half)
      if (pvglu::allow_max_dynamic_smem(f) != cudaSuccess) return 1;
    if constexpr (std::is_same<T, double>::value) {
      const void* half_prog[] = {(const void*)pvglu::k_prog_level<T, -1, B, 1>,
                                 (const void*)pvglu::k_prog_level<T, 0, B, 1>,
                                 (const void*)pvglu::k_prog_level<T, 1, B, 1>,
                                 (const void*)pvglu::k_prog_level<T, 2, B, 1>,
                                 (const void*)pvglu::k_prog_level<T, 3, B, 1>};
      for (const void* f : half_prog)
        if (pvglu::allow_max_dynamic_smem(f) != cudaSuccess) return 1;
    }
  }
  if constexpr (B) {
    const void* from_a[] = {(const void*)pvglu::k_prog_refactor_from_a<T, 2>,
                            (const void*)pvglu::k_prog_refactor_from_a<T, 1>,
                            (const void*)pvglu::k_prog_refactor_from_a<T, 2, true>,
                            (const void*)pvglu::k_prog_refactor_from_a<T, 1, true>};
    for (const void* f : from_a)
      if (pvglu::allow_max_dynamic_smem(f) != cudaSuccess) return 1;
  }
  h->prog_grid = pvglu::prog_persistent_grid<T, B>(h->table_max);
  return 0;
}

// Threads per block of a WIDE level launch: a block per item (unit and
// scenario group); levels with fewer items than SMs get larger blocks (more
// chains of a column, and more producers of an ordered sum, at a time).
int wide_threads(const pvglu_numeric* h, int64_t items) {
  int threads = pvglu::kProgBlock;
  while (threads < pvglu::kWideBlockMax && items * (threads * 2 / pvglu::kProgBlock) <= h->sm_count)
    threads *= 2;
  return threads;
}

// Shared memory of a WIDE level launch: the ordered-sum scratch, and in
// single mode the level's widest column staged beside it when it fits.
template <typename T, bool B>
size_t wide_smem(const pvglu_numeric* h, int ph, int lv, int threads) {
  const size_t scratch = pvglu::wide_scratch_bytes<T, B>(threads);
  if (B || ph != 0) return scratch;
  const size_t want = scratch + (size_t)h->prog_level_wide_len[ph][lv] * sizeof(T);
  return std::min(want, h->smem_optin);
}

// One WIDE level launch: a block per item (a unit and a group of 32 * LW
// scenarios).  Batched levels with at most a quarter as many 64-scenario
// items as SMs run with LW = 1: twice the items, each with half the
// scenarios, still in blocks of 512 threads.  (With more items the blocks
// would shrink, and that measured slower: 7 bus columns at 512 scenarios,
// 3.25 against 3.12 ms per step; at 64 scenarios LW = 1 gives 1.29 against
// 1.54 ms.)
template <typename T, int KIND, bool B>
void launch_wide(pvglu_numeric* h, int ph, int lv, int cb, int ce, T* x, const int* done,
                 const int* ndone, cudaStream_t st) {
  int64_t items = (int64_t)(ce - cb) * (B ? h->ld / pvglu::kGroup : 1);
  const bool half = B && items * 4 <= h->sm_count;
  if (half) items *= 2;
  const int threads = wide_threads(h, items);
  const size_t smem = wide_smem<T, B>(h, ph, lv, threads);
  T* v = static_cast<T*>(h->values);
  if constexpr (B) {
    if (half) {
      pvglu::k_wide_level<T, KIND, B, 1><<<launch_blocks(items, 1), threads, smem, st>>>(
          h->progs.p[ph], h->d, cb, ce, v, x, h->ld, h->S, (T)h->pivot_tol, h->status, done,
          ndone, (int)smem);
      return;
    }
  }
  pvglu::k_wide_level<T, KIND, B, 2><<<launch_blocks(items, 1), threads, smem, st>>>(
      h->progs.p[ph], h->d, cb, ce, v, x, h->ld, h->S, (T)h->pivot_tol, h->status, done, ndone,
      (int)smem);
}

// One phase of chain programs with one launch per level.  a (batched
// refactorization without WIDE levels, or NULL): the caller's FP64 values,
// read by the levels in place of a scatter (k_prog_refactor_from_a).
template <typename T, bool B, int KIND>
void prog_levels(pvglu_numeric* h, T* x, const int* done, const int* ndone, cudaStream_t st,
                 const double* a = nullptr) {
  const int ph = KIND + 1;
  const auto& lc = h->prog_level_chain[ph];
  const int groups = B ? h->ld / pvglu::kGroup : 1;
  for (size_t lv = 0; lv + 1 < lc.size(); lv++) {
    const int cb = lc[lv], ce = lc[lv + 1];
    const int64_t items = (int64_t)(ce - cb) * groups;
    if (h->prog_level_wide_len[ph][lv] > 0) {  // a WIDE level: a block per unit and group
      launch_wide<T, KIND, B>(h, ph, (int)lv, cb, ce, x, done, ndone, st);
      continue;
    }
    const int table = h->prog_level_ml[ph][lv];
    if constexpr (B && std::is_same<T, double>::value) {
      // FP64 levels with few items run with one scenario per lane: twice the
      // warps, each with half the FP64 work.  Solves: up to a quarter of the
      // resident warps.  Refactorization (FP64-heavier): only while the
      // doubled items fit one block per SM; past that some SMs get two blocks
      // and the level is no faster (347 string chains at 64 scenarios: 220
      // against 166 us).
      const int64_t limit = KIND < 0 ? (int64_t)h->sm_count * pvglu::kProgWarps / 2
                                     : (int64_t)h->sm_count * pvglu::prog_min_blocks<T>() *
                                           pvglu::kProgWarps / 4;
      if (items <= limit) {
        const size_t smem = pvglu::prog_smem_bytes<T, B, 1>(table, pvglu::kProgWarps);
        if constexpr (KIND < 0) {
          if (a) {
            const auto k = items * 2 <= (int64_t)h->sm_count * pvglu::kProgWarps
                               ? pvglu::k_prog_refactor_from_a<T, 1, true>
                               : pvglu::k_prog_refactor_from_a<T, 1>;
            k<<<launch_blocks(items * 2, pvglu::kProgWarps), pvglu::kProgBlock, smem, st>>>(
                h->progs.p[ph], table, h->d, cb, ce, static_cast<T*>(h->values), a, h->ld, h->S,
                h->pivot_tol, h->status);
            continue;
          }
        }
        pvglu::k_prog_level<T, KIND, B, 1>
            <<<launch_blocks(items * 2, pvglu::kProgWarps), pvglu::kProgBlock, smem, st>>>(
                h->progs.p[ph], table, h->d, cb, ce, static_cast<T*>(h->values), x, h->ld,
                h->S, h->pivot_tol, h->status, done, ndone);
        continue;
      }
    }
    const size_t smem = pvglu::prog_smem_bytes<T, B>(table, pvglu::kProgWarps);
    if constexpr (KIND < 0 && B) {
      if (a) {
        // Narrow levels (at most one block of items per SM) keep more own
        // rows in flight.
        const auto k = items <= (int64_t)h->sm_count * pvglu::kProgWarps
                           ? pvglu::k_prog_refactor_from_a<T, 2, true>
                           : pvglu::k_prog_refactor_from_a<T, 2>;
        k<<<launch_blocks(items, pvglu::kProgWarps), pvglu::kProgBlock, smem, st>>>(
            h->progs.p[ph], table, h->d, cb, ce, static_cast<T*>(h->values), a, h->ld, h->S,
            h->pivot_tol, h->status);
        continue;
      }
    }
    pvglu::k_prog_level<T, KIND, B>
        <<<launch_blocks(items, pvglu::kProgWarps), pvglu::kProgBlock, smem, st>>>(
            h->progs.p[ph], table, h->d, cb, ce, static_cast<T*>(h->values), x, h->ld, h->S,
            h->pivot_tol, h->status, done, ndone);
  }
}

template <typename T, bool B>
int prog_dispatch(pvglu_numeric* h, int phases, T* x, pvglu::SkipDone skip, cudaStream_t st) {
  if (h->schedule == PVGLU_SCHED_PERSISTENT) {
    if (pvglu::launch_prog_persistent<T, B>(h->progs, h->prog_max_chains, h->d,
                                            static_cast<T*>(h->values), x, h->ld, h->S,
                                            h->pivot_tol, h->status, h->barrier, h->prog_grid,
                                            phases, st, skip))
      return fail(PVGLU_ERR_CUDA, std::string("persistent launch failed: ") +
                                      cudaGetErrorString(cudaGetLastError()));
    return PVGLU_OK;
  }
  if (phases & pvglu::PHASE_REFACTOR) prog_levels<T, B, -1>(h, x, nullptr, skip.ndone, st);
  if (phases & pvglu::PHASE_SOLVE) {
    prog_levels<T, B, 0>(h, x, skip.done, skip.ndone, st);
    prog_levels<T, B, 1>(h, x, skip.done, skip.ndone, st);
  }
  if (phases & pvglu::PHASE_SOLVE_T) {
    prog_levels<T, B, 2>(h, x, skip.done, skip.ndone, st);
    prog_levels<T, B, 3>(h, x, skip.done, skip.ndone, st);
  }
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

template <typename T>
int run_phases(pvglu_numeric* h, int phases, T* x, cudaStream_t st,
               pvglu::SkipDone skip = pvglu::SkipDone{nullptr, nullptr}) {
  // Batched chain programs move rows with TMA bulk copies: 16-byte alignment.
  if (h->batch && x && (reinterpret_cast<uintptr_t>(x) & 15))
    return fail(PVGLU_ERR_BAD_ARG, "solution vector must be 16-byte aligned");
  return h->batch ? prog_dispatch<T, true>(h, phases, x, skip, st)
                  : prog_dispatch<T, false>(h, phases, x, skip, st);
}

// skip: per-scenario convergence flags of iterative refinement (or none).
template <typename T>
int solve_permuted(pvglu_numeric* h, T* x, bool transpose, cudaStream_t st,
                   pvglu::SkipDone skip = pvglu::SkipDone{nullptr, nullptr}) {
  if (h->schedule != PVGLU_SCHED_THREAD_CHAIN)
    return run_phases<T>(h, transpose ? pvglu::PHASE_SOLVE_T : pvglu::PHASE_SOLVE, x, st, skip);
  if (!transpose) {
    solve_phase<T, 0>(h, h->l_sl, x, skip.done, st);
    solve_phase<T, 1>(h, h->u_sl, x, skip.done, st);
  } else {
    solve_phase<T, 2>(h, h->lu_sl, x, skip.done, st);
    solve_phase<T, 3>(h, h->lt_sl, x, skip.done, st);
  }
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

template <typename TI, typename TO>
void permute(pvglu_numeric* h, const int* perm, const TI* x, TO* y, bool gather,
             cudaStream_t st) {
  if (gather && h->ld % 64 == 0 &&
      !((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15)) {
    const int vb = std::min(pvglu::rows_grid(h->n, h->ld, 256), h->sm_count * 8);
    pvglu::k_rows_vec<TI, TO><<<vb, 256, 0, st>>>(perm, h->n, h->ld, h->S, x, y, nullptr);
    return;
  }
  pvglu::k_permute<TI, TO><<<pvglu::rows_grid(h->n, h->ld, 256), 256, 0, st>>>(
      perm, h->n, h->ld, h->S, x, y, gather ? 1 : 0);
}

template <typename T>
int solve_any(pvglu_numeric* h, T* x, int flags, cudaStream_t st) {
  const bool tr = (flags & PVGLU_SOLVE_TRANSPOSE) != 0;
  if (!(flags & PVGLU_SOLVE_ORIGINAL)) return solve_permuted<T>(h, x, tr, st);
  T* w = static_cast<T*>(h->work);
  // J x = b:   w = b[row_orig], solve M y = w, x[col_orig] = y
  // J^T x = b: w = b[col_orig], solve M^T z = w, x[row_orig] = z
  const int* in_perm = tr ? h->d.col_orig : h->d.row_orig;
  const int* out_perm = tr ? h->d.row_orig : h->d.col_orig;
  permute<T, T>(h, in_perm, x, w, true, st);
  int rc = solve_permuted<T>(h, w, tr, st);
  if (rc) return rc;
  permute<T, T>(h, out_perm, w, x, false, st);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

}  // namespace

namespace pvglu {

int run_scatter(pvglu_numeric* h, const AValues& A, const int* ndone, cudaStream_t st) {
  if (A.a && h->ld % 64 == 0 && !(reinterpret_cast<uintptr_t>(A.a) & 15)) {
    const int vb = std::min(rows_grid(h->nnz, h->ld, 256), h->sm_count * 8);
    if (h->precision == PVGLU_FP64)
      k_rows_vec<double, double><<<vb, 256, 0, st>>>(h->d.slot_src, h->nnz, h->ld, h->S, A.a,
                                                     (double*)h->values, ndone);
    else
      k_rows_vec<double, float><<<vb, 256, 0, st>>>(h->d.slot_src, h->nnz, h->ld, h->S, A.a,
                                                    (float*)h->values, ndone);
    PVGLU_CUDA(cudaGetLastError());
    return PVGLU_OK;
  }
  const int blocks = rows_grid(h->nnz, h->ld, 256);
  if (h->precision == PVGLU_FP64)
    k_scatter<double><<<blocks, 256, 0, st>>>(h->d.slot_src, h->nnz, h->ld, h->S, A,
                                              (double*)h->values, ndone);
  else
    k_scatter<float><<<blocks, 256, 0, st>>>(h->d.slot_src, h->nnz, h->ld, h->S, A,
                                             (float*)h->values, ndone);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

// Scatter and refactorization in one pass (k_prog_refactor_from_a): batched
// handles on the per-level schedule whose refactorization has no WIDE level,
// with 16-byte aligned values.  Otherwise the scatter, then the refactor.
int run_scatter_refactor(pvglu_numeric* h, const double* a, cudaStream_t st) {
  bool one_pass = h->batch && h->schedule == PVGLU_SCHED_LEVELS && h->ld % 64 == 0 &&
                  !(reinterpret_cast<uintptr_t>(a) & 15);
  for (const int w : h->prog_level_wide_len[0]) one_pass = one_pass && w == 0;
  if (!one_pass) {
    const AValues A{a, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const int rc = run_scatter(h, A, nullptr, st);
    return rc ? rc : run_refactor(h, st, SkipDone{nullptr, nullptr});
  }
  if (h->precision == PVGLU_FP64)
    prog_levels<double, true, -1>(h, nullptr, nullptr, nullptr, st, a);
  else
    prog_levels<float, true, -1>(h, nullptr, nullptr, nullptr, st, a);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

int run_refactor(pvglu_numeric* h, cudaStream_t st, SkipDone skip) {
  if (h->schedule == PVGLU_SCHED_THREAD_CHAIN)
    return h->precision == PVGLU_FP64 ? refactor_levels<double>(h, st, skip.ndone)
                                      : refactor_levels<float>(h, st, skip.ndone);
  return h->precision == PVGLU_FP64
             ? run_phases<double>(h, PHASE_REFACTOR, (double*)nullptr, st, skip)
             : run_phases<float>(h, PHASE_REFACTOR, (float*)nullptr, st, skip);
}

int run_solve_perm(pvglu_numeric* h, void* x, bool transpose, SkipDone skip, cudaStream_t st) {
  return h->precision == PVGLU_FP64 ? solve_permuted<double>(h, (double*)x, transpose, st, skip)
                                    : solve_permuted<float>(h, (float*)x, transpose, st, skip);
}

int run_refactor_solve_perm(pvglu_numeric* h, void* x, bool transpose, SkipDone skip,
                            cudaStream_t st) {
  if (h->schedule != PVGLU_SCHED_PERSISTENT) {
    const int rc = run_refactor(h, st, skip);
    return rc ? rc : run_solve_perm(h, x, transpose, skip, st);
  }
  const int phases = PHASE_REFACTOR | (transpose ? PHASE_SOLVE_T : PHASE_SOLVE);
  return h->precision == PVGLU_FP64 ? run_phases<double>(h, phases, (double*)x, st, skip)
                                    : run_phases<float>(h, phases, (float*)x, st, skip);
}

namespace {

// One refinement's arguments and the launch pieces it is made of.
struct Refine {
  pvglu_numeric* h;
  AValues A;
  const double* b;
  double* x;
  bool transpose;
  double tol;
  int max_sweeps;
  int* sweeps_out;
  const int* init_done;
  float* w;
  int* ndone;
  // J x = b:   w = b[row_orig], M y = w, x[col_orig] = y, residual rows by A.
  // J^T x = b: w = b[col_orig], M^T z = w, x[row_orig] = z, rows by A^T.
  const int *in_perm, *out_perm, *r_ptr, *r_idx, *r_ent, *r_pos;
  bool vec16;  // 16-byte vector loads in the batched residual
  dim3 grd, blk;
  int rgrid;

  Refine(pvglu_numeric* h_, const AValues& A_, const double* b_, double* x_, bool tr, double tol_,
         int ms, int* so, const int* init)
      : h(h_), A(A_), b(b_), x(x_), transpose(tr), tol(tol_), max_sweeps(ms), sweeps_out(so),
        init_done(init) {
    w = static_cast<float*>(h->work);
    ndone = h->ir_done + h->ld;
    in_perm = tr ? h->d.col_orig : h->d.row_orig;
    out_perm = tr ? h->d.row_orig : h->d.col_orig;
    r_ptr = tr ? h->at_ptr : h->d.a_rowptr;
    r_idx = tr ? h->at_row : h->d.a_colidx;
    r_ent = tr ? h->at_entry : nullptr;
    r_pos = tr ? h->col_pos : h->row_pos;
    vec16 = !((reinterpret_cast<uintptr_t>(A.a) | reinterpret_cast<uintptr_t>(b) |
               reinterpret_cast<uintptr_t>(x)) & 15);
    // About one full SM of threads per SM: the launches after every scenario
    // has converged (ndone == S) then cost little.
    blk = dim3(32, 8);
    const int gy = (h->ld + 31) / 32;
    const int fill = std::max(1, h->sm_count * 8);
    grd = dim3((unsigned)std::max(1, std::min((h->n + 7) / 8, (fill + gy - 1) / gy)),
               (unsigned)gy);
    rgrid = std::min(rows_grid(h->n, h->ld, 256), h->resid_blocks);
  }

  // Bookkeeping reset, and w = b in pivot order (x = 0: the first residual is b).
  int start(cudaStream_t st) const {
    if (init_done) {
      PVGLU_CUDA(cudaMemsetAsync(ndone, 0, sizeof(int), st));
      k_ir_init<<<rows_grid(h->n, h->ld, 256), 256, 0, st>>>(h->n, h->ld, h->S, init_done,
                                                             h->ir_done, ndone, x);
    } else {
      // x needs no clearing: the first sweep assigns it (k_ir_update, first).
      PVGLU_CUDA(cudaMemsetAsync(h->ir_done, 0, (h->ld + 1) * sizeof(int), st));
    }
    PVGLU_CUDA(cudaMemsetAsync(h->ir_max_dx, 0, h->ld * sizeof(unsigned long long), st));
    PVGLU_CUDA(cudaMemsetAsync(h->ir_max_x, 0, h->ld * sizeof(unsigned long long), st));
    if (sweeps_out) PVGLU_CUDA(cudaMemsetAsync(sweeps_out, 0, h->ld * sizeof(int), st));
    permute<double, float>(h, in_perm, b, w, true, st);
    PVGLU_CUDA(cudaGetLastError());
    return PVGLU_OK;
  }

  // dx = M^-1 w (FP32) and x += dx (FP64) for the scenarios still refining.
  int correct(bool first, cudaStream_t st) const {
    const int rc = solve_permuted<float>(h, w, transpose, st, SkipDone{h->ir_done, ndone});
    if (rc) return rc;
    k_ir_update<<<grd, blk, 0, st>>>(out_perm, h->n, h->ld, h->S, w, x, h->ir_done, ndone,
                                     h->ir_max_dx, h->ir_max_x, first ? 1 : 0);
    PVGLU_CUDA(cudaGetLastError());
    return PVGLU_OK;
  }

  // w = b - A x (FP64, rounded to FP32) in pivot order for the scenarios
  // still refining.
  int residual(cudaStream_t st) const {
    if (A.a && h->ld % 64 == 0 && vec16)
      k_residual_rows<<<rgrid, 256, 0, st>>>(r_ptr, r_idx, r_ent, h->n, h->ld, h->S, A.a, b, x,
                                             h->ir_done, ndone, w, r_pos);
    else
      k_residual<<<rows_grid(h->n, h->ld, 256), 256, 0, st>>>(
          r_ptr, r_idx, r_ent, h->n, h->ld, h->S, A, b, x, h->ir_done, ndone, w, r_pos);
    PVGLU_CUDA(cudaGetLastError());
    return PVGLU_OK;
  }

  int check_loop(cudaGraphConditionalHandle loop, cudaStream_t st) const {
    const int threads = std::min(1024, (h->S + 31) / 32 * 32);
    k_ir_check_loop<<<1, threads, 0, st>>>(h->S, max_sweeps, tol, h->ir_done, ndone, sweeps_out,
                                           h->ir_max_dx, h->ir_max_x, h->ir_prev_dx,
                                           h->ir_sweeps_done, loop);
    PVGLU_CUDA(cudaGetLastError());
    return PVGLU_OK;
  }
};

// Builds (or finds) the graph of a refinement: the first sweep, then a
// conditional while node whose body is residual, correction and check; the
// check's block decides whether the body runs again, so no launch is spent
// on sweeps after convergence.  Returns false when the graph cannot be built
// (the refinement then stays on direct launches for this handle).
bool refine_graph(const Refine& R) {
  pvglu_numeric* h = R.h;
  const pvglu_numeric::RefineKey key{R.A,    R.b,         R.x,          R.sweeps_out,
                                     R.init_done, R.tol, R.transpose ? 1 : 0, R.max_sweeps,
                                     h->schedule};
  if (h->ir_graph && h->ir_key == key) return true;
  if (h->ir_graph) {
    cudaGraphExecDestroy(h->ir_graph);
    h->ir_graph = nullptr;
  }
  if (h->ir_graph_failed) return false;
  for (cudaStream_t& c : h->ir_cap)
    if (!c && cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      h->ir_graph_failed = true;
      return false;
    }
  cudaStream_t outer = h->ir_cap[0], inner = h->ir_cap[1];
  cudaGraph_t g = nullptr, cg = nullptr, tmp = nullptr;
  cudaGraphExec_t ex = nullptr;
  bool ok = cudaStreamBeginCapture(outer, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  const bool outer_open = ok;
  bool inner_open = false;
  cudaGraphConditionalHandle loop = 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaGraphNode_t* deps = nullptr;
  size_t n_deps = 0;
  cudaGraphNode_t node = nullptr;
  cudaGraph_t body = nullptr;
  ok = ok && cudaMemsetAsync(h->ir_sweeps_done, 0, sizeof(int), outer) == cudaSuccess;
  ok = ok && R.start(outer) == PVGLU_OK && R.correct(true, outer) == PVGLU_OK;
  ok = ok && cudaStreamGetCaptureInfo(outer, &cs, nullptr, &cg) == cudaSuccess && cg &&
       cudaGraphConditionalHandleCreate(&loop, cg, 0, cudaGraphCondAssignDefault) == cudaSuccess;
  ok = ok && R.check_loop(loop, outer) == PVGLU_OK;
  ok = ok && cudaStreamGetCaptureInfo(outer, &cs, nullptr, &cg, &deps, nullptr, &n_deps) ==
                 cudaSuccess;
  if (ok) {
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    ok = cudaGraphAddNode(&node, cg, deps, nullptr, n_deps, &np) == cudaSuccess;
    if (ok) body = np.conditional.phGraph_out[0];
    ok = ok && cudaStreamUpdateCaptureDependencies(outer, &node, nullptr, 1,
                                                   cudaStreamSetCaptureDependencies) ==
                   cudaSuccess;
  }
  if (ok) {
    inner_open = cudaStreamBeginCaptureToGraph(inner, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    ok = inner_open && R.residual(inner) == PVGLU_OK && R.correct(false, inner) == PVGLU_OK &&
         R.check_loop(loop, inner) == PVGLU_OK;
  }
  if (inner_open) ok = (cudaStreamEndCapture(inner, &tmp) == cudaSuccess) && ok;
  if (outer_open) ok = (cudaStreamEndCapture(outer, &g) == cudaSuccess) && ok && g;
  ok = ok && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    h->ir_graph_failed = true;
    return false;
  }
  h->ir_graph = ex;
  h->ir_key = key;
  return true;
}

}  // namespace

// Mixed-precision refinement on factors already in the handle: x0 = 0, then
// per sweep dx = M^-1 r (FP32), x += dx (FP64), r = b - A x (FP64), until
// max|dx| <= tol * max|x| per scenario or max_sweeps.  Converged scenarios
// drop out of every later kernel (done flags; the whole launch once all are).
// Replayed from a graph with a conditional loop when the stream is not being
// captured and the schedule launches no cooperative kernel, otherwise
// launched sweep by sweep.
int run_refine(pvglu_numeric* h, const AValues& A, const double* b, double* x, bool transpose,
               double tol, int max_sweeps, int* sweeps_out, cudaStream_t st,
               const int* init_done) {
  if (h->precision != PVGLU_FP32) return fail(PVGLU_ERR_BAD_ARG, "needs an FP32 handle");
  const Refine R(h, A, b, x, transpose, tol, max_sweeps, sweeps_out, init_done);
  // PVGLU_REFINE_GRAPH=0: the same kernels launched one by one, for
  // profilers that do not list the kernels of conditional graph bodies.
  static const bool graph_on = [] {
    const char* e = std::getenv("PVGLU_REFINE_GRAPH");
    return !(e && e[0] == '0');
  }();
  if (graph_on && max_sweeps > 1 && h->schedule != PVGLU_SCHED_PERSISTENT) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PVGLU_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusNone && refine_graph(R)) {
      PVGLU_CUDA(cudaGraphLaunch(h->ir_graph, st));
      return PVGLU_OK;
    }
  }
  int rc = R.start(st);
  for (int sweep = 1; !rc && sweep <= max_sweeps; sweep++) {
    rc = R.correct(sweep == 1, st);
    if (rc) break;
    k_ir_check<<<(h->S + 127) / 128, 128, 0, st>>>(h->S, sweep, max_sweeps, tol, h->ir_done,
                                                   R.ndone, sweeps_out, h->ir_max_dx,
                                                   h->ir_max_x, h->ir_prev_dx);
    if (sweep < max_sweeps) rc = R.residual(st);
  }
  if (rc) return rc;
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

}  // namespace pvglu

extern "C" {

const char* pvglu_last_error(void) { return g_err.c_str(); }
const char* pvglu_version(void) { return "pvglu 0.1 (sm_103a)"; }

int pvglu_symbolic_create(int n, const int* rowptr, const int* colidx, const int* perm,
                          pvglu_symbolic** out) {
  if (!out) return fail(PVGLU_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  auto* h = new pvglu_symbolic();
  std::string err;
  pvglu::SymbolicOptions opt;
  const int st = pvglu::build_symbolic(n, rowptr, colidx, perm, opt, h->s, err);
  if (st) {
    delete h;
    return fail(st, err);
  }
  *out = h;
  return PVGLU_OK;
}

int pvglu_symbolic_save(const pvglu_symbolic* h, const char* path) {
  if (!h || !path) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  std::string err;
  const int st = pvglu::save_symbolic(h->s, path, err);
  return st ? fail(st, err) : PVGLU_OK;
}

int pvglu_symbolic_load(const char* path, pvglu_symbolic** out) {
  if (!path || !out) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  *out = nullptr;
  auto* h = new pvglu_symbolic();
  std::string err;
  const int st = pvglu::load_symbolic(path, h->s, err);
  if (st) {
    delete h;
    return fail(st, err);
  }
  *out = h;
  return PVGLU_OK;
}

int pvglu_symbolic_destroy(pvglu_symbolic* s) {
  delete s;
  return PVGLU_OK;
}

int pvglu_symbolic_get_info(const pvglu_symbolic* h, pvglu_symbolic_info* info) {
  if (!h || !info) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  const auto& s = h->s;
  info->n = s.n;
  info->nnz_a = s.nnz_a;
  info->nnz_lu = s.nnz_lu;
  info->update_count = s.update_count;
  info->lu_levels = s.lu.num_levels();
  info->l_levels = s.l.num_levels();
  info->u_levels = s.u.num_levels();
  info->lt_levels = s.lt.num_levels();
  info->lu_chains = s.lu.num_chains();
  info->l_chains = s.l.num_chains();
  info->u_chains = s.u.num_chains();
  info->lt_chains = s.lt.num_chains();
  info->row_swaps = s.row_swaps;
  info->perm_rows_is_involution = s.perm_rows_is_involution;
  info->right_looking_hazards = s.right_looking_hazards;
  info->flops_refactor = s.flops_refactor;
  return PVGLU_OK;
}

int pvglu_symbolic_get_array(const pvglu_symbolic* h, const char* name, const int** data,
                             int64_t* len) {
  if (!h || !name || !data || !len) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  const auto& s = h->s;
  const std::string k(name);
  const std::vector<int>* v = nullptr;
#define PVG(key, member) if (k == key) v = &s.member;
  PVG("perm_amd", perm_amd) PVG("perm_rows", perm_rows) PVG("row_orig", row_orig)
  PVG("col_orig", col_orig) PVG("fill_rowptr", fill_rowptr) PVG("fill_col", fill_col)
  PVG("csr_rowptr", csr_rowptr) PVG("csr_col", csr_col) PVG("csc_colptr", csc_colptr)
  PVG("csc_row", csc_row) PVG("csr_to_csc", csr_to_csc) PVG("csc_to_csr", csc_to_csr)
  PVG("csr_diag_start", csr_diag_start) PVG("csc_diag_start", csc_diag_start)
  PVG("lu_sl", lu.start_levels) PVG("lu_sc", lu.start_chains) PVG("lu_cols", lu.columns)
  PVG("l_sl", l.start_levels) PVG("l_sc", l.start_chains) PVG("l_cols", l.columns)
  PVG("u_sl", u.start_levels) PVG("u_sc", u.start_chains) PVG("u_cols", u.columns)
  PVG("lt_sl", lt.start_levels) PVG("lt_sc", lt.start_chains) PVG("lt_cols", lt.columns)
  PVG("max_elements_per_column", max_elements_per_column) PVG("slot_src", slot_src)
  PVG("diag_slot", diag_slot) PVG("a_rowptr", a_rowptr) PVG("a_colidx", a_colidx)
#undef PVG
  if (!v) return fail(PVGLU_ERR_BAD_ARG, std::string("unknown array ") + name);
  *data = v->data();
  *len = (int64_t)v->size();
  return PVGLU_OK;
}

int pvglu_numeric_create(const pvglu_symbolic* sym, int n_scenarios, int precision,
                         pvglu_numeric** out) {
  return pvglu_numeric_create_ex(sym, n_scenarios, precision, 0, out);
}

int pvglu_numeric_create_ex(const pvglu_symbolic* sym, int n_scenarios, int precision,
                            int max_locals, pvglu_numeric** out) {
  if (!sym) return fail(PVGLU_ERR_BAD_ARG, "symbolic handle is NULL");
  const pvglu_tuning t{max_locals, 0, default_merge(sym->s), PVGLU_SCHED_LEVELS};
  return pvglu_numeric_create_tuned(sym, n_scenarios, precision, &t, out);
}

int pvglu_numeric_create_tuned(const pvglu_symbolic* sym, int n_scenarios, int precision,
                               const pvglu_tuning* tuning, pvglu_numeric** out) {
  if (!sym || !out || !tuning || n_scenarios <= 0 ||
      (precision != PVGLU_FP64 && precision != PVGLU_FP32) || tuning->max_locals < 0 ||
      tuning->max_locals > pvglu::kMaxLocals || tuning->wide_threshold < 0 ||
      tuning->merge_chains < 0 || tuning->merge_chains > 2 ||
      (tuning->schedule != PVGLU_SCHED_LEVELS && tuning->schedule != PVGLU_SCHED_PERSISTENT &&
       tuning->schedule != PVGLU_SCHED_THREAD_CHAIN))
    return fail(PVGLU_ERR_BAD_ARG, "bad numeric_create arguments");
  const int max_locals = tuning->max_locals;
  if (max_locals > 0 && max_locals < 8)
    return fail(PVGLU_ERR_BAD_ARG, "max_locals must be 0 (default) or >= 8");
  *out = nullptr;
  const auto& s = sym->s;
  if (s.update_count > 0x7fffffffLL) return fail(PVGLU_ERR_TOO_LARGE, "update list > 2^31");
  {
    // The chain programs address values with 32-bit offsets.
    const int64_t ld_max = n_scenarios == 1 ? 1 : ((n_scenarios + 63) / 64) * 64;
    if (s.nnz_lu * ld_max >= 0x7fffffffLL || (int64_t)s.n * ld_max >= 0x7fffffffLL ||
        s.nnz_a * ld_max >= 0x7fffffffLL)
      return fail(PVGLU_ERR_TOO_LARGE, "nnz x scenarios exceeds 2^31 values per handle");
  }
  auto* h = new pvglu_numeric();
  h->sym = sym;
  h->n = s.n;
  h->nnz = (int)s.nnz_lu;
  h->nnz_a = (int)s.nnz_a;
  h->S = n_scenarios;
  // Scenario stride: one 64-scenario group per warp item in batched mode.
  h->ld = n_scenarios == 1 ? 1 : ((n_scenarios + 63) / 64) * 64;
  h->precision = precision;
  h->lu_sl = s.lu.start_levels;
  h->l_sl = s.l.start_levels;
  h->u_sl = s.u.start_levels;
  h->lt_sl = s.lt.start_levels;
  auto& d = h->d;
  d.n = s.n;
  d.nnz = (int)s.nnz_lu;
  std::vector<int> upd_ptr32(s.upd_ptr.begin(), s.upd_ptr.end());
  std::vector<int> row_pos(s.n);
  for (int r = 0; r < s.n; r++) row_pos[s.row_orig[r]] = r;
  int rc = 0;
  rc |= h->put(s.csc_colptr, &d.colptr);
  rc |= h->put(s.csc_row, &d.csc_row);
  rc |= h->put(s.diag_slot, &d.diag);
  rc |= h->put(s.slot_src, &d.slot_src);
  rc |= h->put(upd_ptr32, &d.upd_ptr);
  rc |= h->put(s.upd_tgt, &d.upd_tgt);
  rc |= h->put(s.lrow_ptr, &d.lrow_ptr);
  rc |= h->put(s.lrow_slot, &d.lrow_slot);
  rc |= h->put(s.lrow_col, &d.lrow_col);
  rc |= h->put(s.urow_ptr, &d.urow_ptr);
  rc |= h->put(s.urow_slot, &d.urow_slot);
  rc |= h->put(s.urow_col, &d.urow_col);
  rc |= h->put(s.row_orig, &d.row_orig);
  rc |= h->put(s.col_orig, &d.col_orig);
  rc |= h->put(s.a_rowptr, &d.a_rowptr);
  rc |= h->put(s.a_colidx, &d.a_colidx);
  rc |= h->put(s.lu.start_chains, &d.lu_sc);
  rc |= h->put(s.lu.columns, &d.lu_cols);
  rc |= h->put(s.l.start_chains, &d.l_sc);
  rc |= h->put(s.l.columns, &d.l_cols);
  rc |= h->put(s.u.start_chains, &d.u_sc);
  rc |= h->put(s.u.columns, &d.u_cols);
  rc |= h->put(s.lt.start_chains, &d.lt_sc);
  rc |= h->put(s.lt.columns, &d.lt_cols);
  {
    const int* rp = nullptr;
    rc |= h->put(row_pos, &rp);
    h->row_pos = const_cast<int*>(rp);
  }
  const size_t es = precision == PVGLU_FP64 ? sizeof(double) : sizeof(float);
  rc |= h->alloc((size_t)h->nnz * h->ld * es, (char**)&h->values);
  rc |= h->alloc((size_t)h->n * h->ld * es, (char**)&h->work);
  rc |= h->alloc((size_t)std::max(h->nnz_a, h->n) * h->ld, &h->work64);
  rc |= h->alloc((size_t)h->n * h->ld, &h->b64);
  rc |= h->alloc((size_t)h->n * h->ld, &h->x64);
  {
    // A^T by rows: counting sort of A's entries by column.
    std::vector<int> at_ptr(s.n + 1, 0), at_row(s.nnz_a), at_entry(s.nnz_a);
    for (int64_t p = 0; p < s.nnz_a; p++) at_ptr[s.a_colidx[p] + 1]++;
    for (int j = 0; j < s.n; j++) at_ptr[j + 1] += at_ptr[j];
    std::vector<int> fillp(at_ptr.begin(), at_ptr.end() - 1);
    for (int i = 0; i < s.n; i++)
      for (int p = s.a_rowptr[i]; p < s.a_rowptr[i + 1]; p++) {
        const int q = fillp[s.a_colidx[p]]++;
        at_row[q] = i;
        at_entry[q] = p;
      }
    const int *a0 = nullptr, *a1 = nullptr, *a2 = nullptr;
    rc |= h->put(at_ptr, &a0);
    rc |= h->put(at_row, &a1);
    rc |= h->put(at_entry, &a2);
    h->at_ptr = const_cast<int*>(a0);
    h->at_row = const_cast<int*>(a1);
    h->at_entry = const_cast<int*>(a2);
  }
  {
    std::vector<int> col_pos(s.n);
    for (int c = 0; c < s.n; c++) col_pos[s.col_orig[c]] = c;
    const int* cp = nullptr;
    rc |= h->put(col_pos, &cp);
    h->col_pos = const_cast<int*>(cp);
  }
  rc |= h->alloc(1, &h->status);
  rc |= h->alloc((size_t)h->ld + 1, &h->ir_done);  // [ld] flags + converged count
  rc |= h->alloc((size_t)h->ld, &h->ir_max_dx);
  rc |= h->alloc((size_t)h->ld, &h->ir_max_x);
  rc |= h->alloc((size_t)h->ld, &h->ir_prev_dx);
  rc |= h->alloc((size_t)1, &h->ir_sweeps_done);
  rc |= h->alloc(4, &h->barrier);
  if (rc) {
    const std::string e = g_err;
    delete h;
    return fail(PVGLU_ERR_NO_MEMORY, "device allocation failed: " + e);
  }
  if (cudaMemset(h->status, 0, sizeof(pvglu::DevStatus)) != cudaSuccess ||
      cudaMemset(h->barrier, 0, 4 * sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(h->values, 0, (size_t)h->nnz * h->ld * es) != cudaSuccess) {
    delete h;
    return fail(PVGLU_ERR_CUDA, "cudaMemset failed");
  }
  // Chain programs for the shared-memory schedules.  Table budget: a warp's
  // tile is max_locals x 32 scenarios (batched) or max_locals (single).
  h->batch = h->ld > 1;
  {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    h->device = dev;
    if (
        cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      h->sm_count = 1;
    // One resident wave of the batched residual (its grid-stride loop covers
    // the rows): no tail wave, and cheap launches after convergence.
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pvglu::k_residual_rows, 256, 0) !=
            cudaSuccess ||
        per_sm <= 0)
      per_sm = 4;
    h->resid_blocks = per_sm * h->sm_count;
  }
  h->max_locals = max_locals > 0 ? max_locals
                                 : (h->batch ? (precision == PVGLU_FP32 ? 64 : 40)
                                             : pvglu::kMaxLocals);
  {
    const size_t smem = precision == PVGLU_FP64
                            ? (h->batch ? pvglu::prog_smem_bytes<double, true>(h->max_locals,
                                                                               pvglu::kProgWarps)
                                        : pvglu::prog_smem_bytes<double, false>(
                                              h->max_locals, pvglu::kProgWarps))
                            : (h->batch ? pvglu::prog_smem_bytes<float, true>(h->max_locals,
                                                                              pvglu::kProgWarps)
                                        : pvglu::prog_smem_bytes<float, false>(
                                              h->max_locals, pvglu::kProgWarps));
    if (smem > 227 * 1024) {
      delete h;
      return fail(PVGLU_ERR_BAD_ARG, "max_locals too large for shared memory");
    }
  }
  // Levels with at most one warp item per resident warp slot of a one-block-
  // per-SM launch get the widest table that fits: their chains then run in
  // fewer segments, and the occupancy a wide table costs is not used anyway.
  const size_t elem = precision == PVGLU_FP64 ? sizeof(double) : sizeof(float);
  const int group = h->batch ? pvglu::kGroup : 1;
  const int wide = std::min<int>(
      pvglu::kMaxLocals,
      (int)((227 * 1024 - pvglu::kProgWarps * sizeof(unsigned long long)) /
            ((size_t)pvglu::kProgWarps * group * elem)));
  const int groups = h->batch ? h->ld / pvglu::kGroup : 1;
  h->table_max = 0;
  for (int ph = 0; ph < 5; ph++) {
    pvglu::ChainProgram prog;
    pvglu::ProgramOptions opt;
    opt.max_locals = h->max_locals;
    opt.wide_locals = wide;
    opt.narrow_chains = (int)((int64_t)h->sm_count * pvglu::kProgWarps / groups);
    opt.merge = tuning->merge_chains;
    opt.wide_threshold = tuning->wide_threshold;
    pvglu::build_chain_program(s, ph - 1, opt, prog);
    h->prog_level_ml[ph] = prog.level_max_locals;
    h->table_max = std::max(h->table_max, prog.max_locals);
    std::vector<int4> seg(prog.seg.size()), ops(prog.ops.size() / 4), carry(prog.seg.size());
    for (size_t i = 0; i < seg.size(); i++) {
      const auto& g = prog.seg[i];
      seg[i] = make_int4(g.load_begin,
                         g.n_load < 0 ? -1
                                      : (g.n_load | (g.n_own << 16) | (g.n_carry << 26) |
                                         (g.reads_own_chain << 30)),
                         g.op_begin, g.n_op);
      carry[i] = make_int4(g.carry[0], g.carry[1], g.carry[2], g.carry[3]);
    }
    std::memcpy(ops.data(), prog.ops.data(), ops.size() * sizeof(int4));
    pvglu::ProgDev& P = h->progs.p[ph];
    rc |= h->put(prog.level_chain, &P.level_chain);
    rc |= h->put(prog.chain_seg, &P.chain_seg);
    rc |= h->put(seg, &P.seg);
    rc |= h->put(carry, &P.carry);
    rc |= h->put(prog.loads, &P.loads);
    P.load_src = nullptr;
    if (ph == 0) {
      // One pass from A: the A entry of every own row's slot (-1 at fill).
      std::vector<int> src(prog.loads.size(), -1);
      for (const auto& sg : prog.seg)
        for (int l = 0; l < std::max(sg.n_own, 0); l++)
          src[sg.load_begin + l] = s.slot_src[prog.loads[sg.load_begin + l]];
      rc |= h->put(src, &P.load_src);
    }
    rc |= h->put(ops, &P.ops);
    rc |= h->put(prog.op_col, &P.op_col);
    std::vector<int> lwide(prog.level_wide.begin(), prog.level_wide.end());
    rc |= h->put(lwide, &P.level_wide);
    rc |= h->put(prog.wide.unit, &P.w_unit);
    rc |= h->put(prog.wide.lvl, &P.w_lvl);
    rc |= h->put(prog.wide.lv_chain, &P.lv_chain);
    rc |= h->put(prog.wide.ch_tgt, &P.ch_tgt);
    {
      std::vector<int4> rec(prog.wide.targets());
      for (size_t t = 0; t < rec.size(); t++)
        rec[t] = make_int4(prog.wide.tg_rec[4 * t], prog.wide.tg_rec[4 * t + 1],
                           prog.wide.tg_rec[4 * t + 2], prog.wide.tg_rec[4 * t + 3]);
      rc |= h->put(rec, &P.tg_rec);
    }
    rc |= h->put(prog.wide.pr_q, &P.pr_q);
    rc |= h->put(prog.wide.pr_p, &P.pr_p);
    P.n_levels = (int)prog.level_chain.size() - 1;
    h->prog_level_chain[ph] = prog.level_chain;
    // Per program level: 0, or for a WIDE level its widest unit (column
    // length for the refactorization, entries for a solve row), for the
    // shared memory of its launch.
    h->prog_level_wide_len[ph].assign(P.n_levels, 0);
    for (int lv = 0; lv < P.n_levels; lv++) {
      h->prog_max_chains = std::max(h->prog_max_chains,
                                    prog.level_chain[lv + 1] - prog.level_chain[lv]);
      if (!prog.level_wide[lv]) continue;
      int widest = 1;
      for (int c = prog.level_chain[lv]; c < prog.level_chain[lv + 1]; c++) {
        const int u = prog.units[prog.chain_unit[c]];
        widest = std::max(widest, s.csc_colptr[u + 1] - s.csc_colptr[u]);
      }
      h->prog_level_wide_len[ph][lv] = widest;
    }
    h->prog_ops += (int64_t)prog.ops.size();
    h->prog_loads += (int64_t)prog.loads.size();
    h->prog_wide_units += prog.wide_units;
    h->prog_wide_levels += prog.wide_levels;
  }
  // Wide levels of the persistent kernel use the warps' tables as scratch:
  // at least the smallest ordered-sum buffers (wide.cuh) must fit.
  if (h->prog_wide_levels > 0) {
    const size_t need = precision == PVGLU_FP64
                            ? (h->batch ? pvglu::wide_scratch_min<double, true>(pvglu::kProgBlock)
                                        : pvglu::wide_scratch_min<double, false>(pvglu::kProgBlock))
                            : (h->batch ? pvglu::wide_scratch_min<float, true>(pvglu::kProgBlock)
                                        : pvglu::wide_scratch_min<float, false>(pvglu::kProgBlock));
    const size_t per_row = (size_t)pvglu::kProgWarps * group * elem;
    h->table_max = std::max<int>(h->table_max, (int)((need + per_row - 1) / per_row));
  }
  {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) ==
            cudaSuccess)
      h->smem_optin = (size_t)optin - 1024;
    else
      cudaGetLastError();
  }
  if (rc) {
    delete h;
    return fail(PVGLU_ERR_NO_MEMORY, "chain program upload failed");
  }
  // The persistent kernel lays out one table size for every phase and level.
  for (int ph = 0; ph < 5; ph++) h->progs.p[ph].max_locals = h->table_max;
  const int smem_rc = precision == PVGLU_FP64
                          ? (h->batch ? prog_prepare<double, true>(h) : prog_prepare<double, false>(h))
                          : (h->batch ? prog_prepare<float, true>(h) : prog_prepare<float, false>(h));
  if (smem_rc) {
    delete h;
    return fail(PVGLU_ERR_CUDA, "cannot configure the chain-program kernels");
  }
  if (tuning->schedule == PVGLU_SCHED_PERSISTENT && h->prog_grid <= 0) {
    delete h;
    return fail(PVGLU_ERR_CUDA, "cooperative launch unavailable on this device");
  }
  h->schedule = tuning->schedule;
  *out = h;
  return PVGLU_OK;
}

int pvglu_numeric_destroy(pvglu_numeric* h) {
  delete h;
  return PVGLU_OK;
}

int pvglu_numeric_get_info(const pvglu_numeric* h, pvglu_numeric_info* info) {
  if (!h || !info) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  info->program_levels = 0;
  for (int ph = 0; ph < 5; ph++)
    info->program_levels += std::max(0, (int)h->prog_level_chain[ph].size() - 1);
  info->wide_levels = (int)h->prog_wide_levels;
  info->wide_units = (int)h->prog_wide_units;
  info->table_max = h->table_max;
  info->ops = h->prog_ops;
  info->loads = h->prog_loads;
  return PVGLU_OK;
}

int pvglu_numeric_ld(const pvglu_numeric* h) { return h ? h->ld : 0; }
int pvglu_numeric_max_locals(const pvglu_numeric* h) { return h ? h->max_locals : 0; }
void* pvglu_numeric_values(pvglu_numeric* h) { return h ? h->values : nullptr; }

int pvglu_numeric_set_schedule(pvglu_numeric* h, int schedule) {
  if (!h || (schedule != PVGLU_SCHED_LEVELS && schedule != PVGLU_SCHED_PERSISTENT &&
             schedule != PVGLU_SCHED_THREAD_CHAIN))
    return fail(PVGLU_ERR_BAD_ARG, "bad schedule");
  if (schedule == PVGLU_SCHED_PERSISTENT && h->prog_grid <= 0)
    return fail(PVGLU_ERR_CUDA, "cooperative launch unavailable on this device");
  h->schedule = schedule;
  return PVGLU_OK;
}

int pvglu_numeric_set_pivot_tol(pvglu_numeric* h, double tol) {
  if (!h || !(tol >= 0.0)) return fail(PVGLU_ERR_BAD_ARG, "bad pivot tolerance");
  h->pivot_tol = tol;
  return PVGLU_OK;
}

int pvglu_scatter(pvglu_numeric* h, const double* a_values, void* stream) {
  if (!h || !a_values) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  const pvglu::AValues A{a_values, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  return pvglu::run_scatter(h, A, nullptr, as_stream(stream));
}

int pvglu_numeric_set_stamps(pvglu_numeric* h, int n_elems, const double* base,
                             const int* entry_ptr, const int* entry_elem,
                             const int* entry_sign) {
  if (!h || n_elems < 0 || !base || !entry_ptr || (entry_ptr[h->nnz_a] > 0 && (!entry_elem || !entry_sign)))
    return fail(PVGLU_ERR_BAD_ARG, "bad set_stamps arguments");
  const int nnz_a = h->nnz_a;
  if (entry_ptr[0] != 0) return fail(PVGLU_ERR_BAD_ARG, "entry_ptr[0] must be 0");
  for (int e = 0; e < nnz_a; e++)
    if (entry_ptr[e + 1] < entry_ptr[e]) return fail(PVGLU_ERR_BAD_ARG, "entry_ptr not monotone");
  const int nc = entry_ptr[nnz_a];
  for (int c = 0; c < nc; c++) {
    if (entry_elem[c] < 0 || entry_elem[c] >= n_elems)
      return fail(PVGLU_ERR_BAD_ARG, "stamp element out of range");
    if (entry_sign[c] != 1 && entry_sign[c] != -1)
      return fail(PVGLU_ERR_BAD_ARG, "stamp sign must be +1 or -1");
  }
  for (void* p : h->stamp_allocs) cudaFree(p);
  h->stamp_allocs.clear();
  h->n_elems = 0;
  std::vector<double> vb(base, base + nnz_a);
  std::vector<int> vp(entry_ptr, entry_ptr + nnz_a + 1), ve(entry_elem, entry_elem + nc),
      vs(entry_sign, entry_sign + nc);
  int rc = 0;
  double* db = nullptr;
  int *dp = nullptr, *de = nullptr, *ds = nullptr;
  rc |= upload(vb, &db);
  h->stamp_allocs.push_back(db);
  rc |= upload(vp, &dp);
  h->stamp_allocs.push_back(dp);
  rc |= upload(ve, &de);
  h->stamp_allocs.push_back(de);
  rc |= upload(vs, &ds);
  h->stamp_allocs.push_back(ds);
  if (rc) return fail(PVGLU_ERR_NO_MEMORY, "stamp upload failed: " + g_err);
  h->st_base = db;
  h->st_ptr = dp;
  h->st_elem = de;
  h->st_sign = ds;
  h->n_elems = n_elems;
  return PVGLU_OK;
}

int pvglu_scatter_stamps(pvglu_numeric* h, const double* g, const double* gmin, void* stream) {
  if (!h || !g) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  if (!h->st_ptr) return fail(PVGLU_ERR_BAD_ARG, "no stamps set on this handle");
  return pvglu::run_scatter(h, h->stamps(g, gmin), nullptr, as_stream(stream));
}

int pvglu_refine(pvglu_numeric* h, const double* a_values, const double* g, const double* gmin,
                 const double* b, double* x, int flags, double tol, int max_sweeps,
                 int* sweeps_out, void* stream) {
  if (!h || !b || !x || max_sweeps <= 0 || !(tol > 0.0) || (!a_values == !g))
    return fail(PVGLU_ERR_BAD_ARG, "bad refine arguments");
  if (g && !h->st_ptr) return fail(PVGLU_ERR_BAD_ARG, "no stamps set on this handle");
  const pvglu::AValues A = a_values ? pvglu::AValues{a_values, nullptr, nullptr, nullptr,
                                                     nullptr, nullptr, nullptr, nullptr}
                                    : h->stamps(g, gmin);
  return pvglu::run_refine(h, A, b, x, (flags & PVGLU_SOLVE_TRANSPOSE) != 0, tol, max_sweeps,
                           sweeps_out, as_stream(stream));
}

int pvglu_refactor(pvglu_numeric* h, void* stream) {
  if (!h) return fail(PVGLU_ERR_BAD_ARG, "NULL handle");
  return pvglu::run_refactor(h, as_stream(stream), pvglu::SkipDone{nullptr, nullptr});
}

int pvglu_scatter_refactor(pvglu_numeric* h, const double* a_values, void* stream) {
  if (!h || !a_values) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  return pvglu::run_scatter_refactor(h, a_values, as_stream(stream));
}

int pvglu_refactor_solve(pvglu_numeric* h, void* x, int flags, void* stream) {
  if (!h || !x) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  if (flags & PVGLU_SOLVE_ORIGINAL) {
    int rc = pvglu_refactor(h, stream);
    return rc ? rc : pvglu_solve(h, x, flags, stream);
  }
  return pvglu::run_refactor_solve_perm(h, x, (flags & PVGLU_SOLVE_TRANSPOSE) != 0,
                                        pvglu::SkipDone{nullptr, nullptr}, as_stream(stream));
}

int pvglu_solve(pvglu_numeric* h, void* x, int flags, void* stream) {
  if (!h || !x) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  int dev = 0;
  PVGLU_CUDA(cudaGetDevice(&dev));
  if (dev != h->device)
    return fail(PVGLU_ERR_BAD_ARG, "the handle was created on device " +
                                       std::to_string(h->device) + ", the current device is " +
                                       std::to_string(dev));
  cudaStream_t st = as_stream(stream);
  return h->precision == PVGLU_FP64 ? solve_any<double>(h, (double*)x, flags, st)
                                    : solve_any<float>(h, (float*)x, flags, st);
}

int pvglu_numeric_check(pvglu_numeric* h, void* stream, int* code, int* column,
                        int* scenario) {
  if (!h) return fail(PVGLU_ERR_BAD_ARG, "NULL handle");
  pvglu::DevStatus hs{};
  PVGLU_CUDA(cudaMemcpyAsync(&hs, h->status, sizeof(hs), cudaMemcpyDeviceToHost,
                             as_stream(stream)));
  PVGLU_CUDA(cudaStreamSynchronize(as_stream(stream)));
  PVGLU_CUDA(cudaMemsetAsync(h->status, 0, sizeof(hs), as_stream(stream)));
  PVGLU_CUDA(cudaStreamSynchronize(as_stream(stream)));
  if (code) *code = hs.code;
  if (column) *column = hs.code ? hs.column : -1;
  if (scenario) *scenario = hs.code ? hs.scenario : -1;
  return PVGLU_OK;
}

int pvglu_refactor_host(pvglu_numeric* h, double* csc_values) {
  if (!h || !csc_values || h->precision != PVGLU_FP64 || h->S != 1)
    return fail(PVGLU_ERR_BAD_ARG, "needs a single-scenario FP64 handle");
  PVGLU_CUDA(cudaMemcpy(h->values, csc_values, (size_t)h->nnz * sizeof(double),
                        cudaMemcpyHostToDevice));
  int rc = pvglu_refactor(h, nullptr);
  if (rc) return rc;
  PVGLU_CUDA(cudaMemcpy(csc_values, h->values, (size_t)h->nnz * sizeof(double),
                        cudaMemcpyDeviceToHost));
  int code = 0, col = -1, sc = -1;
  rc = pvglu_numeric_check(h, nullptr, &code, &col, &sc);
  if (rc) return rc;
  if (code) return fail(code, "refactor failed at column " + std::to_string(col));
  return PVGLU_OK;
}

int pvglu_solve_host(pvglu_numeric* h, double* b) {
  if (!h || !b || h->precision != PVGLU_FP64 || h->S != 1)
    return fail(PVGLU_ERR_BAD_ARG, "needs a single-scenario FP64 handle");
  double* x = h->b64;
  PVGLU_CUDA(cudaMemcpy(x, b, (size_t)h->n * sizeof(double), cudaMemcpyHostToDevice));
  int rc = pvglu_solve(h, x, 0, nullptr);
  if (rc) return rc;
  PVGLU_CUDA(cudaMemcpy(b, x, (size_t)h->n * sizeof(double), cudaMemcpyDeviceToHost));
  return PVGLU_OK;
}

int pvglu_scatter_refactor_solve_host(pvglu_numeric* h, const double* a_values_host,
                                      const double* b_host, double* x_host, void* stream) {
  if (!h || !a_values_host || !b_host || !x_host || h->precision != PVGLU_FP64)
    return fail(PVGLU_ERR_BAD_ARG, "needs an FP64 handle and non-NULL buffers");
  cudaStream_t st = as_stream(stream);
  double* a = h->work64;
  double* x = h->b64;
  PVGLU_CUDA(cudaMemcpyAsync(a, a_values_host, (size_t)h->nnz_a * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  PVGLU_CUDA(cudaMemcpyAsync(x, b_host, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  int rc = pvglu_scatter_refactor(h, a, stream);
  if (!rc) rc = pvglu_solve(h, x, PVGLU_SOLVE_ORIGINAL, stream);
  if (rc) return rc;
  PVGLU_CUDA(cudaMemcpyAsync(x_host, x, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
  return PVGLU_OK;
}

int pvglu_refine_residual(pvglu_numeric* h, const double* a_values, const double* b,
                          const double* x, float* r, void* stream) {
  if (!h || !a_values || !b || !x || !r) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  if (h->precision != PVGLU_FP32) return fail(PVGLU_ERR_BAD_ARG, "needs an FP32 handle");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // Every scenario is computed: no convergence flag is set.
  PVGLU_CUDA(cudaMemsetAsync(h->ir_done, 0, (h->ld + 1) * sizeof(int), st));
  const pvglu::AValues A{a_values, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  pvglu::Refine R(h, A, b, const_cast<double*>(x), false, 1.0, 1, nullptr, nullptr);
  R.w = r;
  return R.residual(st);
}

int pvglu_refine_system_host(pvglu_numeric* h, const double* a_values_host,
                             const double* b_host, double* x_host, double tol, int max_sweeps,
                             int* sweeps_out, void* stream) {
  if (!h || !a_values_host || !b_host || !x_host || h->precision != PVGLU_FP32)
    return fail(PVGLU_ERR_BAD_ARG, "needs an FP32 handle and non-NULL buffers");
  cudaStream_t st = as_stream(stream);
  double* a = h->work64;
  PVGLU_CUDA(cudaMemcpyAsync(a, a_values_host, (size_t)h->nnz_a * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  PVGLU_CUDA(cudaMemcpyAsync(h->b64, b_host, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  int rc = pvglu_scatter_refactor(h, a, stream);
  if (!rc) rc = pvglu_solve_refined(h, a, h->b64, h->x64, tol, max_sweeps, sweeps_out, stream);
  if (rc) return rc;
  PVGLU_CUDA(cudaMemcpyAsync(x_host, h->x64, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
  return PVGLU_OK;
}

int pvglu_refine_stamps_host(pvglu_numeric* h, const double* g_host, const double* b_host,
                             double* x_host, double tol, int max_sweeps, int* sweeps_out,
                             void* stream) {
  if (!h || !g_host || !b_host || !x_host || h->precision != PVGLU_FP32)
    return fail(PVGLU_ERR_BAD_ARG, "needs an FP32 handle and non-NULL buffers");
  if (!h->st_ptr) return fail(PVGLU_ERR_BAD_ARG, "no stamps set on this handle");
  cudaStream_t st = as_stream(stream);
  const size_t g_count = (size_t)std::max(h->n_elems, 1) * h->ld;
  if (h->g64_count < g_count) {  // first call, or stamps with more elements since
    if (h->alloc(g_count, &h->g64)) return fail(PVGLU_ERR_NO_MEMORY, "conductance staging buffer");
    h->g64_count = g_count;
  }
  PVGLU_CUDA(cudaMemcpyAsync(h->g64, g_host, (size_t)h->n_elems * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  PVGLU_CUDA(cudaMemcpyAsync(h->b64, b_host, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  // A's values assembled once from the stamps (one pass), then the explicit-
  // value path: its scatter and its residual stream A with vector loads.
  double* a = h->work64;
  pvglu::k_assemble<<<pvglu::rows_grid(h->nnz_a, h->ld, 256), 256, 0, st>>>(
      h->nnz_a, h->ld, h->S, h->stamps(h->g64, nullptr), a);
  PVGLU_CUDA(cudaGetLastError());
  int rc = pvglu_scatter_refactor(h, a, stream);
  if (!rc) rc = pvglu_solve_refined(h, a, h->b64, h->x64, tol, max_sweeps, sweeps_out, stream);
  if (rc) return rc;
  PVGLU_CUDA(cudaMemcpyAsync(x_host, h->x64, (size_t)h->n * h->ld * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
  return PVGLU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free solve.  Its permuted work vector lives in this file-scope
// device array instead of the handle's work buffer.  Every GPU that loads
// the library reserves the array until the process exits.  Host code must not
// use the array's name as a device address: the address is obtained with
// cudaGetSymbolAddress, once per device and CUDA context, with that device
// current.
constexpr int64_t kNoAllocScratchElems = int64_t(1) << 20;  // 8 MiB of FP64
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchElems];

namespace {
std::mutex g_noalloc_mu;
struct NoAllocSlot {
  double* ptr = nullptr;
  unsigned long long ctx_id = 0;  // context the address belongs to
};
NoAllocSlot g_noalloc_slot[128];  // per device ordinal

// Unique id of the calling thread's current CUDA context (driver entry points
// looked up through the runtime, so the library links no driver library).  A
// device reset ends the context; the next context gets a new id, and the
// array's address is looked up again for it.
int current_context_id(unsigned long long* id) {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0{}, q1{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) ==
            cudaSuccess &&
        q0 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) ==
            cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<GetCurrent>(f0);
      get_id = reinterpret_cast<GetId>(f1);
    }
    cudaGetLastError();
    looked_up = true;
  }
  if (!get_current || !get_id) return fail(PVGLU_ERR_CUDA, "driver context entry points unavailable");
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) return fail(PVGLU_ERR_CUDA, "no current CUDA context");
  if (get_id(ctx, id) != 0) return fail(PVGLU_ERR_CUDA, "cuCtxGetId failed");
  return PVGLU_OK;
}

// Set-up of the allocation-free solve on the current device: the device
// address of g_noalloc_scratch, looked up on the first call in each context
// of each device and cached.  cudaGetSymbolAddress allocates nothing.
int noalloc_scratch(int dev, double** out) {
  if (dev < 0 || dev >= 128) return fail(PVGLU_ERR_BAD_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc) return rc;
  NoAllocSlot& slot = g_noalloc_slot[dev];
  if (!slot.ptr || slot.ctx_id != ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(PVGLU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    slot.ptr = static_cast<double*>(p);
    slot.ctx_id = ctx;
  }
  *out = slot.ptr;
  return PVGLU_OK;
}
}  // namespace

extern "C" {

int pvglu_solve_noalloc(pvglu_numeric* h, double* x, int flags, void* stream) {
  if (!h || !x) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  if (h->precision != PVGLU_FP64) return fail(PVGLU_ERR_BAD_ARG, "needs an FP64 handle");
  const int64_t need = (int64_t)h->n * h->ld;
  if (need > kNoAllocScratchElems)
    return fail(PVGLU_ERR_TOO_LARGE,
                "n * ld = " + std::to_string(need) + " exceeds the static scratch of " +
                    std::to_string(kNoAllocScratchElems) + " FP64 entries");
  int dev = 0;
  PVGLU_CUDA(cudaGetDevice(&dev));
  if (dev != h->device)
    return fail(PVGLU_ERR_BAD_ARG, "the handle was created on device " +
                                       std::to_string(h->device) + ", the current device is " +
                                       std::to_string(dev));
  double* w = nullptr;
  int rc = noalloc_scratch(dev, &w);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  const bool tr = (flags & PVGLU_SOLVE_TRANSPOSE) != 0;
  // Same sequence as the original-order pvglu_solve; every entry of w that a
  // solve reads is written by the gather first, so nothing needs clearing.
  const int* in_perm = tr ? h->d.col_orig : h->d.row_orig;
  const int* out_perm = tr ? h->d.row_orig : h->d.col_orig;
  permute<double, double>(h, in_perm, x, w, true, st);
  rc = solve_permuted<double>(h, w, tr, st);
  if (rc) return rc;
  permute<double, double>(h, out_perm, w, x, false, st);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Size-class groups: handles with different symbolic analyses refactored and
// solved together, one launch per level over the items of every class.
struct pvglu_group {
  std::vector<pvglu_numeric*> m;
  int precision = PVGLU_FP64;
  bool batch = false;
};

namespace {

template <typename T, bool B, int KIND>
int group_phase(pvglu_group* g, T* const* xs, cudaStream_t st) {
  const int ph = KIND + 1;
  int nlev = 0;
  for (auto* h : g->m) nlev = std::max(nlev, (int)h->prog_level_chain[ph].size() - 1);
  // Members whose level lv uses the same table size share a launch (a
  // launch lays out its widest table, which would cost the others occupancy).
  std::vector<int> tables;
  for (int lv = 0; lv < nlev; lv++) {
    tables.clear();
    for (size_t i = 0; i < g->m.size(); i++) {
      pvglu_numeric* h = g->m[i];
      if (lv + 1 >= (int)h->prog_level_chain[ph].size()) continue;
      if (h->prog_level_wide_len[ph][lv] > 0) {
        // A member's WIDE level: its own launch, a block per unit and group.
        const auto& lc = h->prog_level_chain[ph];
        launch_wide<T, KIND, B>(h, ph, lv, lc[lv], lc[lv + 1], xs ? xs[i] : nullptr, nullptr,
                                nullptr, st);
        continue;
      }
      if (std::find(tables.begin(), tables.end(), h->prog_level_ml[ph][lv]) == tables.end())
        tables.push_back(h->prog_level_ml[ph][lv]);
    }
    for (const int tb : tables) {
    pvglu::MultiLaunch<T> M{};
    int table = 0, items = 0;
    for (size_t i = 0; i < g->m.size(); i++) {
      pvglu_numeric* h = g->m[i];
      const auto& lc = h->prog_level_chain[ph];
      if (lv + 1 >= (int)lc.size() || h->prog_level_ml[ph][lv] != tb ||
          h->prog_level_wide_len[ph][lv] > 0)
        continue;
      auto& C = M.c[M.n++];
      C.P = h->progs.p[ph];
      C.d = h->d;
      C.v = static_cast<T*>(h->values);
      C.x = xs ? xs[i] : nullptr;
      C.ld = h->ld;
      C.S = h->S;
      C.cb = lc[lv];
      C.ce = lc[lv + 1];
      C.groups = B ? h->ld / pvglu::kGroup : 1;
      C.item_begin = items;
      C.st = h->status;
      C.pivot_tol = (T)h->pivot_tol;
      items += (C.ce - C.cb) * C.groups;
      table = std::max(table, h->prog_level_ml[ph][lv]);
    }
    if (!items) continue;
    M.items = items;
    const size_t smem = pvglu::prog_smem_bytes<T, B>(table, pvglu::kProgWarps);
    pvglu::k_prog_level_multi<T, KIND, B>
        <<<launch_blocks(items, pvglu::kProgWarps), pvglu::kProgBlock, smem, st>>>(M, table);
    }
  }
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

template <typename T, bool B>
int group_prepare() {
  const void* fns[] = {(const void*)pvglu::k_prog_level_multi<T, -1, B>,
                       (const void*)pvglu::k_prog_level_multi<T, 0, B>,
                       (const void*)pvglu::k_prog_level_multi<T, 1, B>};
  for (const void* f : fns)
    if (pvglu::allow_max_dynamic_smem(f) != cudaSuccess) return 1;
  return 0;
}

template <typename T, bool B>
int group_run(pvglu_group* g, void* const* x, int flags, cudaStream_t st) {
  std::vector<T*> xs(g->m.size(), nullptr);
  const bool orig = (flags & PVGLU_SOLVE_ORIGINAL) != 0;
  for (size_t i = 0; i < g->m.size(); i++) {
    pvglu_numeric* h = g->m[i];
    if (!x) break;
    if (orig) {
      xs[i] = static_cast<T*>(h->work);
      permute<T, T>(h, h->d.row_orig, static_cast<const T*>(x[i]), xs[i], true, st);
    } else {
      xs[i] = static_cast<T*>(x[i]);
    }
  }
  int rc = group_phase<T, B, -1>(g, nullptr, st);
  if (!rc && x) rc = group_phase<T, B, 0>(g, xs.data(), st);
  if (!rc && x) rc = group_phase<T, B, 1>(g, xs.data(), st);
  if (rc) return rc;
  if (x && orig)
    for (size_t i = 0; i < g->m.size(); i++)
      permute<T, T>(g->m[i], g->m[i]->d.col_orig, xs[i], static_cast<T*>(x[i]), false, st);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

}  // namespace

extern "C" {

int pvglu_group_create(pvglu_numeric* const* members, int count, pvglu_group** out) {
  if (!members || !out || count <= 0 || count > pvglu::kMaxClasses)
    return fail(PVGLU_ERR_BAD_ARG, "a group holds 1 to 4 handles");
  *out = nullptr;
  auto* g = new pvglu_group();
  for (int i = 0; i < count; i++) {
    pvglu_numeric* h = members[i];
    if (!h || (i > 0 && (h->precision != g->precision || h->batch != g->batch))) {
      delete g;
      return fail(PVGLU_ERR_BAD_ARG, "group members must share precision and batching");
    }
    if (i == 0) {
      g->precision = h->precision;
      g->batch = h->batch;
    }
    g->m.push_back(h);
  }
  const int prc = g->precision == PVGLU_FP64
                      ? (g->batch ? group_prepare<double, true>() : group_prepare<double, false>())
                      : (g->batch ? group_prepare<float, true>() : group_prepare<float, false>());
  if (prc) {
    delete g;
    return fail(PVGLU_ERR_CUDA, "cannot configure the group kernels");
  }
  *out = g;
  return PVGLU_OK;
}

int pvglu_group_destroy(pvglu_group* g) {
  delete g;
  return PVGLU_OK;
}

int pvglu_group_refactor_solve(pvglu_group* g, void* const* x, int flags, void* stream) {
  if (!g) return fail(PVGLU_ERR_BAD_ARG, "NULL group");
  if (flags & PVGLU_SOLVE_TRANSPOSE) return fail(PVGLU_ERR_BAD_ARG, "transposed group solve");
  if (x)
    for (size_t i = 0; i < g->m.size(); i++)
      if (!x[i] || (g->batch && (reinterpret_cast<uintptr_t>(x[i]) & 15)))
        return fail(PVGLU_ERR_BAD_ARG, "each member needs a 16-byte aligned vector");
  cudaStream_t st = as_stream(stream);
  return g->precision == PVGLU_FP64
             ? (g->batch ? group_run<double, true>(g, x, flags, st)
                         : group_run<double, false>(g, x, flags, st))
             : (g->batch ? group_run<float, true>(g, x, flags, st)
                         : group_run<float, false>(g, x, flags, st));
}

}  // extern "C"

namespace {

// Times scatter + refactor + solve of every candidate tuning on stand-in
// values and returns the fastest (autotuner core).
int autotune_over(const pvglu_symbolic* sym, int n_scenarios, int precision,
                  const std::vector<pvglu_tuning>& cands, pvglu_tuning* best_t, double* best_ms) {
  const auto& s = sym->s;
  const int ld = n_scenarios == 1 ? 1 : ((n_scenarios + 63) / 64) * 64;
  // Row-diagonally-dominant values (diagonal n + 1, every other entry -1):
  // the factorization without pivoting is stable and the timing is that of
  // any Jacobian with this pattern.
  std::vector<double> a1(s.nnz_a);
  for (int i = 0; i < s.n; i++)
    for (int p = s.a_rowptr[i]; p < s.a_rowptr[i + 1]; p++)
      a1[p] = s.a_colidx[p] == i ? (double)s.n + 1.0 : -1.0;
  std::vector<double> ah((size_t)s.nnz_a * ld);
  for (int64_t p = 0; p < s.nnz_a; p++)
    for (int k = 0; k < ld; k++) ah[(size_t)p * ld + k] = a1[p];
  double* ad = nullptr;
  if (upload(ah, &ad)) return fail(PVGLU_ERR_NO_MEMORY, "autotune buffers");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e300;
  pvglu_tuning bt{};
  const size_t xbytes = (size_t)s.n * ld * (precision == PVGLU_FP64 ? 8 : 4);
  void* xw = nullptr;
  const int rc = cudaMalloc(&xw, xbytes) == cudaSuccess ? PVGLU_OK : PVGLU_ERR_NO_MEMORY;
  for (size_t ci = 0; !rc && ci < cands.size(); ci++) {
    pvglu_numeric* h = nullptr;
    if (pvglu_numeric_create_tuned(sym, n_scenarios, precision, &cands[ci], &h)) continue;
    float total = 0.f;
    int timed = 0;
    bool ok = true;
    for (int rep = 0; rep < 4 && ok; rep++) {
      cudaMemsetAsync(xw, 0, xbytes, nullptr);
      cudaEventRecord(e0, nullptr);
      // The per-level schedule scatters and refactors in one pass; the
      // persistent schedule refactors and solves in one launch.
      ok = h->schedule == PVGLU_SCHED_LEVELS
               ? pvglu_scatter_refactor(h, ad, nullptr) == PVGLU_OK &&
                     pvglu_solve(h, xw, 0, nullptr) == PVGLU_OK
               : pvglu_scatter(h, ad, nullptr) == PVGLU_OK &&
                     pvglu_refactor_solve(h, xw, 0, nullptr) == PVGLU_OK;
      cudaEventRecord(e1, nullptr);
      if (cudaEventSynchronize(e1) != cudaSuccess) ok = false;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) {  // the first repetition warms up
        total += ms;
        timed++;
        // A candidate already twice the best so far is not timed further.
        if (ms > 2.0 * best) break;
      }
    }
    if (ok && timed > 0 && total / timed < best) {
      best = total / timed;
      bt = cands[ci];
      bt.max_locals = h->max_locals;
    }
    int code = 0, col = 0, scn = 0;
    pvglu_numeric_check(h, nullptr, &code, &col, &scn);
    pvglu_numeric_destroy(h);
  }
  cudaFree(xw);
  cudaFree(ad);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return fail(rc, "autotune allocation failed");
  if (best >= 1e300) return fail(PVGLU_ERR_CUDA, "no autotune candidate ran");
  *best_t = bt;
  if (best_ms) *best_ms = best;
  return PVGLU_OK;
}

std::vector<int> table_candidates(int ld, int precision) {
  if (ld == 1) return {0, 256, 64};
  if (precision == PVGLU_FP32) return {16, 24, 32, 48, 64};
  return {16, 24, 32, 40, 56};
}

// Programs of the refactorization and the two solves under `opt`: levels,
// chains and wide units, to tell whether an option changes anything.
std::vector<int> program_shape(const pvglu::Symbolic& s, const pvglu::ProgramOptions& opt) {
  std::vector<int> shape;
  for (int kind = -1; kind <= 1; kind++) {
    pvglu::ChainProgram pr;
    pvglu::build_chain_program(s, kind, opt, pr);
    shape.insert(shape.end(), pr.level_chain.begin(), pr.level_chain.end());
    shape.insert(shape.end(), pr.chain_unit.begin(), pr.chain_unit.end());
    shape.push_back(pr.wide_units);
  }
  return shape;
}

}  // namespace

extern "C" {

int pvglu_autotune(const pvglu_symbolic* sym, int n_scenarios, int precision,
                   int* best_max_locals, int* best_schedule, double* best_ms) {
  if (!sym || n_scenarios <= 0 || !best_max_locals || !best_schedule ||
      (precision != PVGLU_FP64 && precision != PVGLU_FP32))
    return fail(PVGLU_ERR_BAD_ARG, "bad autotune arguments");
  const int ld = n_scenarios == 1 ? 1 : ((n_scenarios + 63) / 64) * 64;
  std::vector<pvglu_tuning> cands;
  const int merge = default_merge(sym->s);
  for (const int ml : table_candidates(ld, precision))
    for (const int sc : {PVGLU_SCHED_LEVELS, PVGLU_SCHED_PERSISTENT})
      cands.push_back(pvglu_tuning{ml, 0, merge, sc});
  pvglu_tuning bt{};
  const int rc = autotune_over(sym, n_scenarios, precision, cands, &bt, best_ms);
  if (rc) return rc;
  *best_max_locals = bt.max_locals;
  *best_schedule = bt.schedule;
  return PVGLU_OK;
}

int pvglu_autotune_ex(const pvglu_symbolic* sym, int n_scenarios, int precision,
                      pvglu_tuning* best, double* best_ms) {
  if (!sym || n_scenarios <= 0 || !best || (precision != PVGLU_FP64 && precision != PVGLU_FP32))
    return fail(PVGLU_ERR_BAD_ARG, "bad autotune arguments");
  const auto& s = sym->s;
  const int ld = n_scenarios == 1 ? 1 : ((n_scenarios + 63) / 64) * 64;
  std::vector<pvglu_tuning> cands;
  for (const int ml : table_candidates(ld, precision)) {
    const int table = ml > 0 ? ml : (ld == 1 ? pvglu::kMaxLocals
                                             : (precision == PVGLU_FP32 ? 64 : 40));
    pvglu::ProgramOptions o;
    o.max_locals = table;
    // Chain merging modes that give programs of their own shape.
    std::vector<int> merges;
    std::vector<std::vector<int>> shapes;
    for (const int merge : {1, 2, 0}) {
      o.merge = merge;
      std::vector<int> sh = program_shape(s, o);
      if (std::find(shapes.begin(), shapes.end(), sh) != shapes.end()) continue;
      merges.push_back(merge);
      shapes.push_back(std::move(sh));
    }
    o.merge = 1;
    o.wide_threshold = table / 2;
    const bool wide_matters = program_shape(s, o) != shapes[0];
    for (const int merge : merges) {
      for (const int wt : {0, table / 2}) {
        if (wt > 0 && !wide_matters) continue;
        for (const int sc : {PVGLU_SCHED_LEVELS, PVGLU_SCHED_PERSISTENT})
          cands.push_back(pvglu_tuning{ml, wt, merge, sc});
      }
    }
  }
  return autotune_over(sym, n_scenarios, precision, cands, best, best_ms);
}

int pvglu_selftest_barrier_timeout(int blocks, long long max_spins, int* status_code,
                                   int* blocks_returned) {
  if (blocks <= 0 || blocks > 4096 || max_spins <= 0 || max_spins > (1LL << 24) ||
      !status_code || !blocks_returned)
    return fail(PVGLU_ERR_BAD_ARG, "bad self-test arguments");
  unsigned int* bar = nullptr;
  pvglu::DevStatus* st = nullptr;
  int* passed = nullptr;
  // Every buffer is freed on every path (cudaFree(NULL) is a no-op).
  cudaError_t e = cudaMalloc((void**)&bar, 4 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&st, sizeof(pvglu::DevStatus));
  if (e == cudaSuccess) e = cudaMalloc((void**)&passed, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(bar, 0, 4 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(st, 0, sizeof(pvglu::DevStatus));
  if (e == cudaSuccess) e = cudaMemset(passed, 0, sizeof(int));
  void* args[] = {(void*)&bar, (void*)&st, (void*)&max_spins, (void*)&passed};
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((const void*)pvglu::k_barrier_timeout_probe, dim3(blocks),
                                    dim3(64), args, 0, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  pvglu::DevStatus hs{};
  if (e == cudaSuccess) e = cudaMemcpy(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(blocks_returned, passed, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(bar);
  cudaFree(st);
  cudaFree(passed);
  if (e != cudaSuccess) return fail(PVGLU_ERR_CUDA, cudaGetErrorString(e));
  *status_code = hs.code;
  return PVGLU_OK;
}

int pvglu_solve_refined(pvglu_numeric* h, const double* a_values, const double* b,
                        double* x, double tol, int max_sweeps, int* sweeps_out,
                        void* stream) {
  if (!a_values) return fail(PVGLU_ERR_BAD_ARG, "bad solve_refined arguments");
  return pvglu_refine(h, a_values, nullptr, nullptr, b, x, 0, tol, max_sweeps, sweeps_out,
                      stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Scenario blocks: handles of one batch run side by side on their own streams.
struct pvglu_blocks {
  std::vector<pvglu_numeric*> parts;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  ~pvglu_blocks() {
    for (pvglu_numeric* h : parts)
      if (h) pvglu_numeric_destroy(h);
    for (cudaStream_t st : streams)
      if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : joins)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
  }
};

extern "C" {

int pvglu_blocks_create(const pvglu_symbolic* s, int n_scenarios, int parts, int precision,
                        const pvglu_tuning* tuning, pvglu_blocks** out) {
  if (!s || !out || parts < 1 || n_scenarios < parts || n_scenarios % parts)
    return fail(PVGLU_ERR_BAD_ARG, "blocks need n_scenarios a positive multiple of parts");
  *out = nullptr;
  auto* b = new pvglu_blocks();
  const int per = n_scenarios / parts;
  b->parts.assign(parts, nullptr);
  b->streams.assign(parts, nullptr);
  b->joins.assign(parts, nullptr);
  int rc = PVGLU_OK;
  for (int k = 0; k < parts && !rc; k++)
    rc = tuning ? pvglu_numeric_create_tuned(s, per, precision, tuning, &b->parts[k])
                : pvglu_numeric_create(s, per, precision, &b->parts[k]);
  for (int k = 0; k < parts && !rc; k++)
    if (cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming) != cudaSuccess)
      rc = fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  if (!rc && cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    rc = fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return PVGLU_OK;
}

int pvglu_blocks_destroy(pvglu_blocks* b) {
  if (!b) return fail(PVGLU_ERR_BAD_ARG, "NULL blocks");
  for (cudaStream_t st : b->streams)
    if (st) cudaStreamSynchronize(st);
  delete b;
  return PVGLU_OK;
}

int pvglu_blocks_part(pvglu_blocks* b, int k, pvglu_numeric** out) {
  if (!b || !out || k < 0 || k >= (int)b->parts.size())
    return fail(PVGLU_ERR_BAD_ARG, "bad block index");
  *out = b->parts[k];
  return PVGLU_OK;
}

int pvglu_blocks_step(pvglu_blocks* b, const double* const* a_values, const double* const* rhs,
                      double* const* x, double tol, int max_sweeps, int* const* sweeps_out,
                      int flags, void* stream) {
  if (!b || !a_values || !rhs || !x) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  const int parts = (int)b->parts.size();
  for (int k = 0; k < parts; k++)
    if (!a_values[k] || !rhs[k] || !x[k]) return fail(PVGLU_ERR_BAD_ARG, "NULL block buffer");
  if (b->parts[0]->precision == PVGLU_FP32 && (max_sweeps <= 0 || !(tol > 0.0)))
    return fail(PVGLU_ERR_BAD_ARG, "bad refinement arguments");
  cudaStream_t caller = as_stream(stream);
  PVGLU_CUDA(cudaEventRecord(b->fork, caller));
  // Every block's factorization is issued before any block's solve, so that
  // all blocks start within a few launches of each other.
  std::vector<int> rk(parts, PVGLU_OK);
  for (int k = 0; k < parts; k++) {
    pvglu_numeric* h = b->parts[k];
    cudaStream_t st = b->streams[k];
    rk[k] = cudaStreamWaitEvent(st, b->fork, 0) == cudaSuccess
                ? PVGLU_OK
                : fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    if (!rk[k]) rk[k] = pvglu_scatter_refactor(h, a_values[k], st);
  }
  int rc = PVGLU_OK;
  for (int k = 0; k < parts; k++) {
    pvglu_numeric* h = b->parts[k];
    cudaStream_t st = b->streams[k];
    if (!rk[k]) {
      if (h->precision == PVGLU_FP32) {
        rk[k] = pvglu_solve_refined(h, a_values[k], rhs[k], x[k], tol, max_sweeps,
                                    sweeps_out ? sweeps_out[k] : nullptr, st);
      } else {
        rk[k] = cudaMemcpyAsync(x[k], rhs[k], (size_t)h->n * h->ld * sizeof(double),
                                cudaMemcpyDeviceToDevice, st) == cudaSuccess
                    ? PVGLU_OK
                    : fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
        if (!rk[k]) rk[k] = pvglu_solve(h, x[k], PVGLU_SOLVE_ORIGINAL, st);
      }
    }
    // Every block joins back, also after an error, so no stream is left
    // ahead of the caller's (unless the caller joins later).
    if (!(flags & PVGLU_BLOCKS_NO_JOIN) &&
        (cudaEventRecord(b->joins[k], st) != cudaSuccess ||
         cudaStreamWaitEvent(caller, b->joins[k], 0) != cudaSuccess))
      rk[k] = rk[k] ? rk[k] : fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    rc = rc ? rc : rk[k];
  }
  return rc;
}

int pvglu_blocks_join(pvglu_blocks* b, void* stream) {
  if (!b) return fail(PVGLU_ERR_BAD_ARG, "NULL blocks");
  cudaStream_t caller = as_stream(stream);
  for (size_t k = 0; k < b->parts.size(); k++)
    if (cudaEventRecord(b->joins[k], b->streams[k]) != cudaSuccess ||
        cudaStreamWaitEvent(caller, b->joins[k], 0) != cudaSuccess)
      return fail(PVGLU_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  return PVGLU_OK;
}

}  // extern "C"

