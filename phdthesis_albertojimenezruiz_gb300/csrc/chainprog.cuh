// Device executor of the chain programs (programs.hpp).
//
// Batched mode (BATCH = true): a warp runs one chain for 32 scenarios, lane
// = scenario; its local table is a [max_locals][32] tile of shared memory, so
// every table access is bank-conflict free and every global access of the
// load/store phases is one coalesced 128-byte (FP32) or 256-byte (FP64) row.
// The load phase fetches 32 refs with one coalesced load and broadcasts them
// with shuffles, keeping kChunk independent value loads in flight per lane.
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
  const int4* seg;         // {load_begin, n_load | n_own << 16 (or -1: DIRECT), op_begin, n_op}
  const int* loads;
  const int4* ops;         // packed operations, 4 per int4
  const int* op_col;       // column of each SCALE operation
  int max_locals;
};

// Iterative-refinement accumulation fused into the U-solve store phase:
// every own entry dx_i of the correction is also added to the FP64 solution,
// x[col_orig[i]] += dx_i, and the per-scenario max|dx| / max|x| are kept.
// x64 == nullptr disables it.
struct IrFuse {
  double* x64;
  const int* col_orig;
  const int* done;
  unsigned long long* max_dx;
  unsigned long long* max_x;
};

// Per-thread running maxima of the fused accumulation, flushed with one
// atomicMax pair whenever the thread moves to another scenario.
struct IrMax {
  int s = -1;
  double dx = 0.0, x = 0.0;
  __device__ __forceinline__ void flush(const IrFuse& ir) {
    if (s >= 0 && (dx > 0.0 || x > 0.0)) {
      atomicMax(ir.max_dx + s, (unsigned long long)__double_as_longlong(dx));
      atomicMax(ir.max_x + s, (unsigned long long)__double_as_longlong(x));
    }
    dx = 0.0;
    x = 0.0;
  }
};

// Offsets are 32-bit: the handle guarantees nnz_lu * ld and n * ld < 2^31.
template <typename T, int KIND>
__device__ __forceinline__ T prog_fetch(int ref, const T* __restrict__ vs,
                                        const T* __restrict__ xs, int ld) {
  if (KIND < 0) return ldv(vs + (unsigned)ref * (unsigned)ld);
  if (ref >= 0) return ldv(xs + (unsigned)ref * (unsigned)ld);
  return ldv(vs + (unsigned)(-ref - 1) * (unsigned)ld);
}

template <typename T, int KIND>
__device__ __forceinline__ void prog_store(int ref, T val, T* __restrict__ vs,
                                           T* __restrict__ xs, int ld) {
  if (KIND < 0) vs[(unsigned)ref * (unsigned)ld] = val;
  else xs[(unsigned)ref * (unsigned)ld] = val;
}

template <typename T, bool BATCH>
__device__ __forceinline__ void prog_exec_op(uint32_t op, int op_index, const int* op_col,
                                             T* sml, int s, int S, double pivot_tol,
                                             DevStatus* st) {
  constexpr int SH = BATCH ? 5 : 0;
  const int code = op & 3;
  const int a = (op >> 2) & 1023, b = (op >> 12) & 1023, c = (op >> 22) & 1023;
  if (code == OP_FNMA) {
    sml[a << SH] = fnms(sml[a << SH], sml[b << SH], sml[c << SH]);
  } else if (code == OP_SCALE) {
    const T p = sml[a << SH];
    if (!(fabs((double)p) >= pivot_tol) && s < S) report_error(st, 3, op_col[op_index], s);
    for (int i = 0; i < c; i++) sml[(b + i) << SH] = sml[(b + i) << SH] / p;
  } else if (code == OP_DIV) {
    sml[a << SH] = sml[a << SH] / sml[b << SH];
  }
}

template <typename T, bool BATCH>
__device__ __forceinline__ void prog_exec_ops(const ProgDev& P, int op_begin, int n_op, T* sml,
                                              int s, int S, double pivot_tol, DevStatus* st) {
  const int4* o4 = P.ops + (op_begin >> 2);
  for (int k = 0; k < (n_op >> 2); k++) {
    const int4 w = __ldg(o4 + k);
    const int base = op_begin + 4 * k;
    prog_exec_op<T, BATCH>((uint32_t)w.x, base, P.op_col, sml, s, S, pivot_tol, st);
    prog_exec_op<T, BATCH>((uint32_t)w.y, base + 1, P.op_col, sml, s, S, pivot_tol, st);
    prog_exec_op<T, BATCH>((uint32_t)w.z, base + 2, P.op_col, sml, s, S, pivot_tol, st);
    prog_exec_op<T, BATCH>((uint32_t)w.w, base + 3, P.op_col, sml, s, S, pivot_tol, st);
  }
}

// Runs every segment of `chain` for scenario s (BATCH) or the single
// scenario (s = 0).  sm: this warp's local table.
template <typename T, int KIND, bool BATCH>
__device__ __forceinline__ void prog_run_chain(const ProgDev& P, const DevStruct& d, int chain,
                                               T* __restrict__ v, T* __restrict__ x, int ld,
                                               int s, int S, T* sm, double pivot_tol,
                                               DevStatus* st, const IrFuse& ir, IrMax& irm) {
  const bool fuse = KIND == 1 && ir.x64 != nullptr && s < S && !(ir.done && ir.done[s]);
  const int lane = threadIdx.x & 31;
  T* vs = v + s;
  T* xs = KIND < 0 ? nullptr : x + s;
  const int g_end = __ldg(P.chain_seg + chain + 1);
  for (int g = __ldg(P.chain_seg + chain); g < g_end; g++) {
    const int4 sg = __ldg(P.seg + g);
    if (sg.y < 0) {  // DIRECT unit: straight from global memory
      if (BATCH || lane == 0) {
        if (KIND < 0) refactor_column<T>(d, sg.z, s, ld, v, pivot_tol, st);
        else solve_unknown<T, (KIND < 0 ? 0 : KIND)>(d, sg.z, s, ld, v, x);
        if (fuse) {
          const T val = x[(unsigned)sg.z * (unsigned)ld + s];
          double* xo = ir.x64 + (unsigned)__ldg(ir.col_orig + sg.z) * (unsigned)ld + s;
          const double nx = *xo + (double)val;
          *xo = nx;
          irm.dx = fmax(irm.dx, fabs((double)val));
          irm.x = fmax(irm.x, fabs(nx));
        }
      }
      __syncwarp();
      continue;
    }
    const int* lr = P.loads + sg.x;
    const int nl = sg.y & 0xffff, n_own = sg.y >> 16;
    if (BATCH) {
      constexpr int kChunk = 16;
      T* sml = sm + lane;
      for (int base = 0; base < nl; base += kChunk) {
        const int cnt = min(kChunk, nl - base);
        const int my_ref = lane < cnt ? __ldg(lr + base + lane) : 0;
        T val[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; k++) {
          const int r = __shfl_sync(0xffffffffu, my_ref, k);
          if (k < cnt) val[k] = prog_fetch<T, KIND>(r, vs, xs, ld);
        }
#pragma unroll
        for (int k = 0; k < kChunk; k++)
          if (k < cnt) sml[(base + k) << 5] = val[k];
      }
      prog_exec_ops<T, true>(P, sg.z, sg.w, sml, s, S, pivot_tol, st);
      for (int base = 0; base < n_own; base += 32) {
        const int cnt = min(32, n_own - base);
        const int my_ref = lane < cnt ? __ldg(lr + base + lane) : 0;
        // col_orig of the rows (scenario independent), broadcast like refs
        const int my_col = (KIND == 1 && ir.x64 != nullptr && lane < cnt)
                               ? __ldg(ir.col_orig + __ldg(lr + base + lane)) : 0;
#pragma unroll 4
        for (int k = 0; k < cnt; k++) {
          const int r = __shfl_sync(0xffffffffu, my_ref, k);
          const T val = sml[(base + k) << 5];
          prog_store<T, KIND>(r, val, vs, xs, ld);
          const int co = __shfl_sync(0xffffffffu, my_col, k);
          if (fuse) {
            double* xo = ir.x64 + (unsigned)co * (unsigned)ld + s;
            const double nx = *xo + (double)val;
            *xo = nx;
            irm.dx = fmax(irm.dx, fabs((double)val));
            irm.x = fmax(irm.x, fabs(nx));
          }
        }
      }
    } else {
      for (int l = lane; l < nl; l += 32) sm[l] = prog_fetch<T, KIND>(__ldg(lr + l), v, x, 1);
      __syncwarp();
      if (lane == 0) prog_exec_ops<T, false>(P, sg.z, sg.w, sm, 0, S, pivot_tol, st);
      __syncwarp();
      for (int l = lane; l < n_own; l += 32) {
        const int r = __ldg(lr + l);
        prog_store<T, KIND>(r, sm[l], v, x, 1);
        if (fuse) {
          double* xo = ir.x64 + __ldg(ir.col_orig + r);
          const double nx = *xo + (double)sm[l];
          *xo = nx;
          irm.dx = fmax(irm.dx, fabs((double)sm[l]));
          irm.x = fmax(irm.x, fabs(nx));
        }
      }
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
                                               DevStatus* st, const int* done, int warp_id,
                                               int n_warps, const IrFuse& ir) {
  const int groups = BATCH ? ld >> 5 : 1;
  const int items = (ce - cb) * groups;
  const int lane = threadIdx.x & 31;
  IrMax irm;
  for (int it = warp_id; it < items; it += n_warps) {
    const int ci = BATCH ? it / groups : it;
    const int c = cb + ci;
    const int s = BATCH ? ((it - ci * groups) << 5) + lane : 0;
    if (BATCH && done && __all_sync(0xffffffffu, s >= S || done[s])) continue;
    if (KIND == 1 && ir.x64 && s != irm.s) {
      irm.flush(ir);
      irm.s = s;
    }
    prog_run_chain<T, KIND, BATCH>(P, d, c, v, x, ld, s, S, sm_warp, pivot_tol, st, ir, irm);
  }
  if (KIND == 1 && ir.x64) irm.flush(ir);
}

template <typename T, int KIND, bool BATCH>
__global__ void k_prog_level(ProgDev P, DevStruct d, int cb, int ce, T* __restrict__ v,
                             T* __restrict__ x, int ld, int S, double pivot_tol, DevStatus* st,
                             const int* done, IrFuse ir) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw) +
          (threadIdx.x >> 5) * P.max_locals * (BATCH ? 32 : 1);
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  prog_run_level<T, KIND, BATCH>(P, d, cb, ce, v, x, ld, S, sm, pivot_tol, st, done, warp_id,
                                 n_warps, ir);
}

}  // namespace pvglu
