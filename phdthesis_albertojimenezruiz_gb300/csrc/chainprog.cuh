// Device executor of the chain programs (programs.hpp).
//
// Batched mode (BATCH = true): a warp runs one chain for 32 scenarios, lane
// = scenario; its local table is a [max_locals][32] tile of shared memory, so
// every table access is bank-conflict free and every global access of the
// load/store phases is one coalesced 128-byte (FP32) or 256-byte (FP64) row.
// The load phase issues kUnroll independent loads per lane before the first
// use, which keeps many requests in flight per warp.
//
// Single mode (BATCH = false): a warp runs one chain of the one scenario; the
// lanes split the loads and stores of each segment, lane 0 executes the
// operations out of shared memory.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "programs.hpp"

namespace pvglu {

struct ProgDev {
  const int* level_chain;  // [levels + 1]
  int n_levels;
  const int* chain_seg;    // [chains + 1]
  const int4* seg;         // Segment records
  const int* loads;
  const int4* ops;
  int max_locals;
};

constexpr int kLoadUnroll = 8;

// Fetch / store of one table entry.  Refactor (KIND < 0): LU slots,
// ref = slot * 2 + own.  Solves: x entries (ref = i * 2 + own) or read-only
// LU slots (ref = -(slot + 1)).
template <typename T, int KIND>
__device__ __forceinline__ T prog_fetch(int ref, const T* __restrict__ v,
                                        const T* __restrict__ x, int ld, int s) {
  if (KIND < 0) return ldv(v + (int64_t)(ref >> 1) * ld + s);
  if (ref >= 0) return ldv(x + (int64_t)(ref >> 1) * ld + s);
  return ldv(v + (int64_t)(-ref - 1) * ld + s);
}

template <typename T, int KIND>
__device__ __forceinline__ void prog_store(int ref, T val, T* __restrict__ v,
                                           T* __restrict__ x, int ld, int s) {
  if (!(ref & 1) || ref < 0) return;
  if (KIND < 0) v[(int64_t)(ref >> 1) * ld + s] = val;
  else x[(int64_t)(ref >> 1) * ld + s] = val;
}

template <typename T, int KIND, bool BATCH>
__device__ __forceinline__ void prog_exec_ops(const int4* __restrict__ ops, int n_op, T* sm,
                                              int lane, int s, int S, double pivot_tol,
                                              DevStatus* st) {
#define PVGLU_L(i) sm[BATCH ? (i) * 32 + lane : (i)]
  for (int o = 0; o < n_op; o++) {
    const int4 q = __ldg(ops + o);
    const int code = q.x & 15;
    if (code == OP_FNMA) {
      PVGLU_L(q.y) = fnms(PVGLU_L(q.y), PVGLU_L(q.z), PVGLU_L(q.w));
    } else if (code == OP_SCALE) {
      const T p = PVGLU_L(q.y);
      if (!(fabs((double)p) >= pivot_tol) && s < S) report_error(st, 3, q.w, s);
      const int cnt = q.x >> 4;
      for (int i = 0; i < cnt; i++) PVGLU_L(q.z + i) = PVGLU_L(q.z + i) / p;
    } else {
      PVGLU_L(q.y) = PVGLU_L(q.y) / PVGLU_L(q.z);
    }
  }
#undef PVGLU_L
}

// Runs every segment of `chain` for scenario s (BATCH) or the single
// scenario (s = 0).  sm: this warp's local table.
template <typename T, int KIND, bool BATCH>
__device__ __forceinline__ void prog_run_chain(const ProgDev& P, const DevStruct& d, int chain,
                                               T* __restrict__ v, T* __restrict__ x, int ld,
                                               int s, int S, T* sm, double pivot_tol,
                                               DevStatus* st) {
  const int lane = threadIdx.x & 31;
  const int g_end = __ldg(P.chain_seg + chain + 1);
  for (int g = __ldg(P.chain_seg + chain); g < g_end; g++) {
    const int4 sg = __ldg(P.seg + g);
    if (sg.y < 0) {  // DIRECT unit: straight from global memory
      if (BATCH || lane == 0) {
        if (KIND < 0) refactor_column<T>(d, sg.z, s, ld, v, pivot_tol, st);
        else solve_unknown<T, (KIND < 0 ? 0 : KIND)>(d, sg.z, s, ld, v, x);
      }
      __syncwarp();
      continue;
    }
    const int* lr = P.loads + sg.x;
    const int nl = sg.y;
    if (BATCH) {
      // kChunk refs per coalesced load, broadcast by shuffles: kChunk
      // independent value loads in flight per lane before the first use.
      constexpr int kChunk = sizeof(T) == 8 ? 16 : 32;
      for (int base = 0; base < nl; base += kChunk) {
        const int cnt = min(kChunk, nl - base);
        const int my_ref = lane < cnt ? __ldg(lr + base + lane) : 0;
        T val[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; k++) {
          const int r = __shfl_sync(0xffffffffu, my_ref, k);
          if (k < cnt) val[k] = prog_fetch<T, KIND>(r, v, x, ld, s);
        }
#pragma unroll
        for (int k = 0; k < kChunk; k++)
          if (k < cnt) sm[(base + k) * 32 + lane] = val[k];
      }
      prog_exec_ops<T, KIND, true>(P.ops + sg.z, sg.w, sm, lane, s, S, pivot_tol, st);
      for (int base = 0; base < nl; base += 32) {
        const int cnt = min(32, nl - base);
        const int my_ref = lane < cnt ? __ldg(lr + base + lane) : 0;
#pragma unroll 4
        for (int k = 0; k < cnt; k++) {
          const int r = __shfl_sync(0xffffffffu, my_ref, k);
          prog_store<T, KIND>(r, sm[(base + k) * 32 + lane], v, x, ld, s);
        }
      }
    } else {
      for (int l = lane; l < nl; l += 32) sm[l] = prog_fetch<T, KIND>(__ldg(lr + l), v, x, 1, 0);
      __syncwarp();
      if (lane == 0) prog_exec_ops<T, KIND, false>(P.ops + sg.z, sg.w, sm, 0, 0, S, pivot_tol, st);
      __syncwarp();
      for (int l = lane; l < nl; l += 32) prog_store<T, KIND>(__ldg(lr + l), sm[l], v, x, 1, 0);
      __syncwarp();
    }
  }
}

// Chains [cb, ce) of one level: work item = (chain, 32-scenario group) in
// batched mode, chain alone in single mode; one warp per item.
template <typename T, int KIND, bool BATCH>
__device__ __forceinline__ void prog_run_level(const ProgDev& P, const DevStruct& d, int cb,
                                               int ce, T* __restrict__ v, T* __restrict__ x,
                                               int ld, int S, T* sm_warp, double pivot_tol,
                                               DevStatus* st, const int* done,
                                               int64_t warp_id, int64_t n_warps) {
  const int groups = BATCH ? ld / 32 : 1;
  const int64_t items = (int64_t)(ce - cb) * groups;
  const int lane = threadIdx.x & 31;
  for (int64_t it = warp_id; it < items; it += n_warps) {
    const int c = cb + (int)(it / groups);
    const int s = BATCH ? (int)(it % groups) * 32 + lane : 0;
    if (BATCH && done && __all_sync(0xffffffffu, s >= S || done[s])) continue;
    prog_run_chain<T, KIND, BATCH>(P, d, c, v, x, ld, s, S, sm_warp, pivot_tol, st);
  }
}

template <typename T, int KIND, bool BATCH>
__global__ void k_prog_level(ProgDev P, DevStruct d, int cb, int ce, T* __restrict__ v,
                             T* __restrict__ x, int ld, int S, double pivot_tol, DevStatus* st,
                             const int* done) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw) +
          (threadIdx.x >> 5) * P.max_locals * (BATCH ? 32 : 1);
  const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  prog_run_level<T, KIND, BATCH>(P, d, cb, ce, v, x, ld, S, sm, pivot_tol, st, done, warp_id,
                                 n_warps);
}

}  // namespace pvglu
