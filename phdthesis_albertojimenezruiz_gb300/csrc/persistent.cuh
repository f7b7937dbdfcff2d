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

#include "kernels.cuh"
#include "symbolic.hpp"

namespace pvglu {

enum : int { PHASE_REFACTOR = 1, PHASE_SOLVE = 2, PHASE_SOLVE_T = 4 };

struct PersistentPlan {
  const int* lu_sl; int lu_nl;
  const int* l_sl;  int l_nl;
  const int* u_sl;  int u_nl;
  const int* lt_sl; int lt_nl;
  int max_chains;   // widest level over all phases
};

constexpr int kPersistentBlock = 128;
constexpr long long kBarrierMaxSpins = 1LL << 22;  // x ~100-1000 ns => ~0.4-4 s

inline PersistentPlan make_plan(const Symbolic& s, std::vector<void*>& allocs, int* rc) {
  PersistentPlan p{};
  auto up = [&](const std::vector<int>& v, const int** out) {
    int* d = nullptr;
    if (cudaMalloc((void**)&d, std::max<size_t>(v.size(), 1) * sizeof(int)) != cudaSuccess) {
      *rc = 1;
      return;
    }
    allocs.push_back(d);
    if (!v.empty() &&
        cudaMemcpy(d, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
      *rc = 1;
    *out = d;
  };
  up(s.lu.start_levels, &p.lu_sl);
  up(s.l.start_levels, &p.l_sl);
  up(s.u.start_levels, &p.u_sl);
  up(s.lt.start_levels, &p.lt_sl);
  p.lu_nl = s.lu.num_levels();
  p.l_nl = s.l.num_levels();
  p.u_nl = s.u.num_levels();
  p.lt_nl = s.lt.num_levels();
  int mx = 1;
  const LevelSet* sets[4] = {&s.lu, &s.l, &s.u, &s.lt};
  for (const LevelSet* ls : sets)
    for (int lv = 0; lv < ls->num_levels(); lv++)
      mx = std::max(mx, ls->start_levels[lv + 1] - ls->start_levels[lv]);
  p.max_chains = mx;
  return p;
}

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

// One phase (a level set) of the persistent walk.  A barrier precedes every
// level except the very first one of the launch (*need_sync false).
// KIND -1 = refactorization, 0..3 = solve kinds of solve_unknown.
template <typename T, int KIND>
__device__ __forceinline__ bool run_phase(const int* sl, int nl, const int* sc, const int* cols,
                                          const DevStruct& d, T* __restrict__ v,
                                          T* __restrict__ x, int ld, int S, double pivot_tol,
                                          DevStatus* st, unsigned int* bar, const int* done,
                                          bool* need_sync) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int lv = 0; lv < nl; lv++) {
    if (*need_sync && !grid_barrier(bar, st, gridDim.x, kBarrierMaxSpins)) return false;
    *need_sync = true;
    const int cb = sl[lv], ce = sl[lv + 1];
    const int64_t items = (int64_t)(ce - cb) * ld;
    for (int64_t it = gtid; it < items; it += nthreads) {
      const int c = cb + (int)(it / ld);
      const int s = (int)(it % ld);
      if (s >= S || (done && done[s])) continue;
      for (int t = sc[c]; t < sc[c + 1]; t++) {
        if constexpr (KIND < 0) refactor_column<T>(d, cols[t], s, ld, v, pivot_tol, st);
        else solve_unknown<T, KIND>(d, cols[t], s, ld, v, x);
      }
    }
  }
  return true;
}

template <typename T>
__global__ void __launch_bounds__(kPersistentBlock)
k_persistent(PersistentPlan plan, DevStruct d, T* __restrict__ v, T* __restrict__ x,
             int ld, int S, double pivot_tol, DevStatus* st, unsigned int* bar,
             int phases, SkipDone skip) {
  if (skip.ndone && __ldcg(skip.ndone) >= S) return;
  bool need_sync = false;
  if (phases & PHASE_REFACTOR)
    if (!run_phase<T, -1>(plan.lu_sl, plan.lu_nl, d.lu_sc, d.lu_cols, d, v, x, ld, S,
                          pivot_tol, st, bar, nullptr, &need_sync))
      return;
  if (phases & PHASE_SOLVE) {
    if (!run_phase<T, 0>(plan.l_sl, plan.l_nl, d.l_sc, d.l_cols, d, v, x, ld, S, pivot_tol,
                         st, bar, skip.done, &need_sync))
      return;
    if (!run_phase<T, 1>(plan.u_sl, plan.u_nl, d.u_sc, d.u_cols, d, v, x, ld, S, pivot_tol,
                         st, bar, skip.done, &need_sync))
      return;
  }
  if (phases & PHASE_SOLVE_T) {
    if (!run_phase<T, 2>(plan.lu_sl, plan.lu_nl, d.lu_sc, d.lu_cols, d, v, x, ld, S,
                         pivot_tol, st, bar, skip.done, &need_sync))
      return;
    if (!run_phase<T, 3>(plan.lt_sl, plan.lt_nl, d.lt_sc, d.lt_cols, d, v, x, ld, S,
                         pivot_tol, st, bar, skip.done, &need_sync))
      return;
  }
}

// Largest co-resident grid for the persistent kernel (0 if cooperative
// launches are unsupported).
template <typename T>
int persistent_grid() {
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent<T>,
                                                    kPersistentBlock, 0) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

template <typename T>
int launch_persistent(const PersistentPlan& plan, const DevStruct& d, T* v, T* x, int ld,
                      int S, double pivot_tol, DevStatus* st, unsigned int* bar,
                      int max_grid, int phases, cudaStream_t stream,
                      SkipDone skip = SkipDone{nullptr, nullptr}) {
  if (max_grid <= 0) return 1;
  const int64_t want = ((int64_t)plan.max_chains * ld + kPersistentBlock - 1) / kPersistentBlock;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, max_grid));
  if (cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned int), stream) != cudaSuccess) return 1;
  void* args[] = {(void*)&plan, (void*)&d, (void*)&v, (void*)&x, (void*)&ld, (void*)&S,
                  (void*)&pivot_tol, (void*)&st, (void*)&bar, (void*)&phases, (void*)&skip};
  if (cudaLaunchCooperativeKernel((const void*)k_persistent<T>, dim3(grid),
                                  dim3(kPersistentBlock), args, 0, stream) != cudaSuccess)
    return 1;
  return 0;
}

// Failure-path self-test: one barrier that waits for one block more than the
// launch has, so the wait can only end by its spin limit.  Every block must
// come back with PVGLU_ERR_BARRIER_TIMEOUT recorded and the abort word set.
__global__ void k_barrier_timeout_probe(unsigned int* bar, DevStatus* st, long long max_spins,
                                        int* passed) {
  const bool ok = grid_barrier(bar, st, gridDim.x + 1u, max_spins);
  if (threadIdx.x == 0 && !ok) atomicAdd(passed, 1);
}

}  // namespace pvglu
