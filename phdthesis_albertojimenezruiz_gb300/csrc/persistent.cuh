// Persistent cooperative schedule: one launch walks every level of the
// refactorization and/or the solves, separated by a software grid barrier.
//
// Replaces the reference's host loop of one launch + cudaDeviceSynchronize
// per level (factorize_electrical_system_CUDA.cu:67-115,
// triangular_substitution.cu:240-263).  All blocks are co-resident
// (cooperative launch), and every barrier wait is bounded: on expiry the
// block records PVGLU_ERR_BARRIER_TIMEOUT, raises an abort word that the other
// blocks also poll, and returns, so no launch can hang the GPU.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "chainprog.cuh"
#include "kernels.cuh"
#include "symbolic.hpp"
#include "wide.cuh"

namespace pvglu {

enum : int { PHASE_REFACTOR = 1, PHASE_SOLVE = 2, PHASE_SOLVE_T = 4 };

constexpr long long kBarrierMaxSpins = 1LL << 22;  // x ~100-1000 ns => ~0.4-4 s

// Bounded sense-by-generation grid barrier.  bar[0] = arrivals, bar[1] =
// generation, bar[2] = abort word.  Returns false when the launch must stop.
// `expected` is the number of arriving blocks (gridDim.x in every production
// launch; the timeout self-test asks for one more block than exists).
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, DevStatus* st,
                                             unsigned int expected, long long max_spins) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = bar + 1;
    volatile unsigned int* vabort = bar + 2;
    const unsigned int gen = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(bar, 1u) + 1u;
    int good = 1;
    if (arrived == expected) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*vgen == gen) {
        if (*vabort) {
          good = 0;
          break;
        }
        if (++spins > max_spins) {
          report_error(st, 6, -1, -1);
          atomicExch(bar + 2, 1u);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = good && !*vabort;
  }
  __syncthreads();
  return ok != 0;
}

// Scenario skipping for iterative refinement: done[s] != 0 skips scenario s;
// *ndone >= S (read once at entry, identical for every block) skips the
// launch.  Both NULL outside refinement.
struct SkipDone {
  const int* done;
  const int* ndone;
};

// ---------------------------------------------------------------------------
// Persistent walk over chain programs (chainprog.cuh): the levels of each
// requested phase in order, a bounded grid barrier between levels, each chain
// executed from a shared-memory table.
struct ProgSetDev {
  ProgDev p[5];  // refactor, L, U, U^T, L^T
};

template <typename T, int KIND, bool BATCH>
__device__ __forceinline__ bool prog_phase(const ProgDev& P, const DevStruct& d, T* v, T* x,
                                           int ld, int S, T* sm, WarpTma& tma,
                                           T pivot_tol, DevStatus* st, unsigned int* bar,
                                           const int* done, bool* need_sync,
                                           unsigned char* smem_raw, int smem_bytes) {
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  for (int lv = 0; lv < P.n_levels; lv++) {
    if (*need_sync) {
      if (!grid_barrier(bar, st, gridDim.x, kBarrierMaxSpins)) return false;
      // Bulk copies issued after the barrier must see what other blocks
      // wrote before it.
      if (BATCH) fence_proxy_async();
    }
    *need_sync = true;
    if (__ldg(P.level_wide + lv)) {
      // Whole blocks on the wide units; the warps' tables are their scratch.
      wide_run_level<T, KIND, BATCH>(P, d, P.level_chain[lv], P.level_chain[lv + 1], v, x, ld,
                                     S, pivot_tol, st, done, smem_raw, smem_bytes, blockIdx.x,
                                     gridDim.x);
      continue;
    }
    prog_run_level<T, KIND, BATCH>(P, d, P.level_chain[lv], P.level_chain[lv + 1], v, x, ld,
                                   S, sm, tma, pivot_tol, st, done, warp_id, n_warps);
    // A warp whose table wait ran out raises the abort word: every block
    // leaves at the next barrier.
    if (BATCH && tma.aborted && (threadIdx.x & 31) == 0) atomicExch(bar + 2, 1u);
  }
  return true;
}

template <typename T, bool BATCH>
__global__ void __launch_bounds__(kProgBlock)
k_prog_persistent(ProgSetDev PS, DevStruct d, T* __restrict__ v, T* __restrict__ x, int ld,
                  int S, T pivot_tol, DevStatus* st, unsigned int* bar, int phases,
                  SkipDone skip) {
  if (skip.ndone && __ldcg(skip.ndone) >= S) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WarpTma tma;
  T* sm = prog_setup_warp<T, BATCH>(smem_raw, PS.p[0].max_locals, tma);
  // The tables (not the mbarriers behind them) are scratch for wide levels.
  const int tables = (int)(prog_smem_bytes<T, BATCH>(PS.p[0].max_locals, kProgWarps) -
                           kProgWarps * sizeof(unsigned long long));
  bool need_sync = false;
  if (phases & PHASE_REFACTOR)
    if (!prog_phase<T, -1, BATCH>(PS.p[0], d, v, x, ld, S, sm, tma, pivot_tol, st, bar,
                                  nullptr, &need_sync, smem_raw, tables))
      return;
  if (phases & PHASE_SOLVE) {
    if (!prog_phase<T, 0, BATCH>(PS.p[1], d, v, x, ld, S, sm, tma, pivot_tol, st, bar,
                                 skip.done, &need_sync, smem_raw, tables))
      return;
    if (!prog_phase<T, 1, BATCH>(PS.p[2], d, v, x, ld, S, sm, tma, pivot_tol, st, bar,
                                 skip.done, &need_sync, smem_raw, tables))
      return;
  }
  if (phases & PHASE_SOLVE_T) {
    if (!prog_phase<T, 2, BATCH>(PS.p[3], d, v, x, ld, S, sm, tma, pivot_tol, st, bar,
                                 skip.done, &need_sync, smem_raw, tables))
      return;
    if (!prog_phase<T, 3, BATCH>(PS.p[4], d, v, x, ld, S, sm, tma, pivot_tol, st, bar,
                                 skip.done, &need_sync, smem_raw, tables))
      return;
  }
}

// Largest co-resident grid of k_prog_persistent for the given table size.
template <typename T, bool BATCH>
int prog_persistent_grid(int max_locals) {
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const size_t smem = prog_smem_bytes<T, BATCH>(max_locals, kProgWarps);
  if (allow_max_dynamic_smem((const void*)k_prog_persistent<T, BATCH>) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_prog_persistent<T, BATCH>,
                                                    kProgBlock, smem) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

template <typename T, bool BATCH>
int launch_prog_persistent(const ProgSetDev& PS, int max_chains, const DevStruct& d, T* v,
                           T* x, int ld, int S, T pivot_tol, DevStatus* st,
                           unsigned int* bar, int max_grid, int phases, cudaStream_t stream,
                           SkipDone skip) {
  if (max_grid <= 0) return 1;
  const int64_t items = (int64_t)max_chains * (BATCH ? ld / kGroup : 1);
  const int64_t want = (items + kProgWarps - 1) / kProgWarps;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, max_grid));
  if (cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned int), stream) != cudaSuccess) return 1;
  void* args[] = {(void*)&PS, (void*)&d, (void*)&v, (void*)&x, (void*)&ld, (void*)&S,
                  (void*)&pivot_tol, (void*)&st, (void*)&bar, (void*)&phases, (void*)&skip};
  const size_t smem = prog_smem_bytes<T, BATCH>(PS.p[0].max_locals, kProgWarps);
  if (cudaLaunchCooperativeKernel((const void*)k_prog_persistent<T, BATCH>, dim3(grid),
                                  dim3(kProgBlock), args, smem, stream) != cudaSuccess)
    return 1;
  return 0;
}

// Failure-path self-test: one barrier that waits for one block more than the
// launch has, so the wait can only end by its spin limit.  Every block must
// come back with PVGLU_ERR_BARRIER_TIMEOUT recorded and the abort word set.
static __global__ void k_barrier_timeout_probe(unsigned int* bar, DevStatus* st, long long max_spins,
                                        int* passed) {
  const bool ok = grid_barrier(bar, st, gridDim.x + 1u, max_spins);
  if (threadIdx.x == 0 && !ok) atomicAdd(passed, 1);
}

}  // namespace pvglu
