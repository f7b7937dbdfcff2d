// Device executor of the chain programs (programs.hpp).
//
// Batched mode (BATCH = true): a warp runs one chain for a group of 64
// scenarios; lane l owns scenarios 2l and 2l+1 of the group, so every table
// access is one 8-byte (FP32) or 16-byte (FP64) shared-memory access for two
// scenarios.  The local table is [max_locals][64] values; one table row is
// one value of the group, which in HBM is one contiguous 256/512-byte row of
// the slot-major layout.  Rows are moved with TMA bulk copies:
// cp.async.bulk global->shared completing on a per-warp mbarrier (loads) and
// cp.async.bulk shared->global in bulk groups (stores).  A segment's loads
// are all in flight at once and need no registers.
//
// Single mode (BATCH = false): a warp runs one chain of the one scenario; the
// lanes split the loads and stores of each segment (ld.global.cg), lane 0
// executes the operations out of shared memory.
//
// Units too wide for a table are not chain-program segments: they form WIDE
// program levels of their own, executed by whole blocks (wide.cuh).
#pragma once
#include <type_traits>
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "programs.hpp"

namespace pvglu {

struct ProgDev {
  const int* level_chain;  // [levels + 1]
  const int* level_wide;   // [levels] 1: a WIDE level (wide.cuh)
  int n_levels;
  const int* chain_seg;    // [chains + 1]
  const int4* seg;         // {load_begin, n_load | n_own << 16 | n_carry << 26 |
                           //  reads_own_chain << 30 (or -1: WIDE), op_begin, n_op}
  const int4* carry;       // [segments] up to 4 moves (from << 16 | to) of table rows
  const int* loads;
  const int* load_src;     // refactorization, per load: A entry of an own row's slot
                           // (-1 at fill slots and for read-only rows); else NULL
  const int4* ops;         // packed operations, 4 per int4
  const int* op_col;       // column of each SCALE operation
  int max_locals;
  // Wide units (programs.hpp, WidePlan).
  const int* w_unit;
  const int* w_lvl;
  const int* lv_chain;
  const int* ch_tgt;
  const int4* tg_rec;      // {slot, src, n_pairs, q} per target
  const int* pr_q;
  const int* pr_p;
};

constexpr int kGroup = 64;                       // scenarios per warp item (two per lane)
constexpr int kProgBlock = 128;                  // threads per block of the executors
constexpr int kProgWarps = kProgBlock / 32;
// Resident blocks per SM the level executors are compiled for: FP32
// executors 8 (up to 64 registers; the usual tables would allow 9 blocks.
// With scenario blocks side by side, 512 scenarios of the 35k plant as 4
// blocks, 64 registers measured 0.935 against 0.949 ms per step in one A/B,
// one handle unchanged at 0.996 ms); FP64 executors up to 80 registers (6
// blocks).  Build-time settings.
#ifndef PVGLU_FP32_MIN_BLOCKS
#define PVGLU_FP32_MIN_BLOCKS 8
#endif
#ifndef PVGLU_FP64_MIN_BLOCKS
#define PVGLU_FP64_MIN_BLOCKS 6
#endif
template <typename T>
constexpr int prog_min_blocks() {
  return sizeof(T) == 4 ? PVGLU_FP32_MIN_BLOCKS : PVGLU_FP64_MIN_BLOCKS;
}
constexpr long long kMbarMaxPolls = 1LL << 20;   // bounded mbarrier waits

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + bulk (non-tensor) TMA copies.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* mbar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gsrc, unsigned bytes,
                                          unsigned long long* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(smem_dst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}
__device__ __forceinline__ void bulk_store(void* gdst, const void* smem_src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_u32(smem_src)), "r"(bytes)
               : "memory");
}
// Starts moving `bytes` (a multiple of 16) at gsrc into L2; no completion.
__device__ __forceinline__ void bulk_prefetch_l2(const void* gsrc, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(gsrc), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Source shared memory of this thread's bulk stores may be reused.
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// This thread's bulk stores are complete in global memory.
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
// Orders this thread's generic-proxy and async-proxy memory accesses.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async;" ::: "memory");
}
// The same for this CTA's shared memory only: table writes by the lanes
// before bulk stores read the table.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  using type = float2;
};
template <>
struct Vec2<double> {
  using type = double2;
};

// Lane values of the batched forms: LW scenarios per lane.  LW = 2: a warp
// item covers 64 scenarios with 16-byte accesses (the default); LW = 1: 32
// scenarios, for FP64 levels with few items, which then spread over twice
// the warps, each with half the FP64 work.
template <typename T, int LW>
using LaneV = typename std::conditional<LW == 2, typename Vec2<T>::type, T>::type;
template <typename V, typename T>
__device__ __forceinline__ V ld_lane(const T* p) {
  if constexpr (std::is_same<V, T>::value) return __ldcg(p);
  else return __ldcg(reinterpret_cast<const V*>(p));
}
template <typename T>
__device__ __forceinline__ T fnms_lane(T acc, T a, T b) { return fnms(acc, a, b); }
__device__ __forceinline__ double2 fnms_lane(double2 acc, double2 a, double2 b) {
  return {fnms(acc.x, a.x, b.x), fnms(acc.y, a.y, b.y)};
}
__device__ __forceinline__ float2 fnms_lane(float2 acc, float2 a, float2 b) {
  return {fnms(acc.x, a.x, b.x), fnms(acc.y, a.y, b.y)};
}
// Component k (< LW) of a lane value.
template <typename T>
__device__ __forceinline__ T& lane_part(T& v, int) { return v; }
__device__ __forceinline__ double& lane_part(double2& v, int k) { return k ? v.y : v.x; }
__device__ __forceinline__ float& lane_part(float2& v, int k) { return k ? v.y : v.x; }

// ---------------------------------------------------------------------------
// Single-scenario table access (ld == 1).
template <typename T, int KIND>
__device__ __forceinline__ T prog_fetch1(int ref, const T* __restrict__ v,
                                         const T* __restrict__ x) {
  if (KIND < 0) return ldv(v + ref);
  if (ref >= 0) return ldv(x + ref);
  return ldv(v + (-ref - 1));
}

template <typename T, int KIND>
__device__ __forceinline__ void prog_store1(int ref, T val, T* __restrict__ v,
                                            T* __restrict__ x) {
  if (KIND < 0) v[ref] = val;
  else x[ref] = val;
}

// Row pointer of entry `ref` for scenario group starting at s0 (batched).
template <typename T, int KIND>
__device__ __forceinline__ T* prog_row(int ref, T* v, T* x, int ld, int s0) {
  if (KIND < 0) return v + (unsigned)ref * (unsigned)ld + s0;
  if (ref >= 0) return x + (unsigned)ref * (unsigned)ld + s0;
  return v + (unsigned)(-ref - 1) * (unsigned)ld + s0;
}

__device__ __forceinline__ void decode_op(uint32_t op, int& code, int& a, int& b, int& c) {
  code = op & 3;
  a = (op >> 2) & 1023;
  b = (op >> 12) & 1023;
  c = (op >> 22) & 1023;
}

// One operation on the LW scenarios of this lane (the first is s).
template <typename T, int LW>
__device__ __forceinline__ void exec_op_lane(uint32_t op, int op_index, const int* op_col,
                                             LaneV<T, LW>* t, int s, int S, T pivot_tol,
                                             DevStatus* st) {
  using V = LaneV<T, LW>;
  int code, a, b, c;
  decode_op(op, code, a, b, c);
  if (code == OP_FNMA) {
    t[a << 5] = fnms_lane(t[a << 5], t[b << 5], t[c << 5]);
  } else if (code == OP_SCALE) {
    V p = t[a << 5];
#pragma unroll
    for (int k = 0; k < LW; k++)
      if (!(fabs(lane_part(p, k)) >= pivot_tol) && s + k < S)
        report_error(st, 3, op_col[op_index], s + k);
    if constexpr (std::is_same<T, float>::value) {
      // FP32 factors are refined afterwards: one reciprocal per pivot.
      V r;
#pragma unroll
      for (int k = 0; k < LW; k++) lane_part(r, k) = __frcp_rn(lane_part(p, k));
      for (int i = 0; i < c; i++) {
        V q = t[(b + i) << 5];
#pragma unroll
        for (int k = 0; k < LW; k++) lane_part(q, k) *= lane_part(r, k);
        t[(b + i) << 5] = q;
      }
    } else {
      // FP64 divides like the reference (GLU_CSC_CPU_levels_strings.cpp:34).
      for (int i = 0; i < c; i++) {
        V q = t[(b + i) << 5];
#pragma unroll
        for (int k = 0; k < LW; k++) lane_part(q, k) = lane_part(q, k) / lane_part(p, k);
        t[(b + i) << 5] = q;
      }
    }
  } else if (code == OP_DIV) {
    V q = t[a << 5], p = t[b << 5];
#pragma unroll
    for (int k = 0; k < LW; k++) lane_part(q, k) = lane_part(q, k) / lane_part(p, k);
    t[a << 5] = q;
  }
}

template <typename T>
__device__ __forceinline__ void exec_op1(uint32_t op, int op_index, const int* op_col, T* t,
                                         int S, T pivot_tol, DevStatus* st) {
  int code, a, b, c;
  decode_op(op, code, a, b, c);
  if (code == OP_FNMA) {
    t[a] = fnms(t[a], t[b], t[c]);
  } else if (code == OP_SCALE) {
    const T p = t[a];
    if (!(fabs(p) >= pivot_tol) && 0 < S) report_error(st, 3, op_col[op_index], 0);
    for (int i = 0; i < c; i++) t[b + i] = t[b + i] / p;
  } else if (code == OP_DIV) {
    t[a] = t[a] / t[b];
  }
}

// Per-warp state of the batched path: its table, its mbarrier and phase.
// aborted: a table wait ran out (warp-uniform); the warp then runs no more
// operations or stores and waits once more, bounded, for the loads it has in
// flight before it returns (prog_drain).
struct WarpTma {
  unsigned long long* mbar;
  unsigned phase;
  bool aborted;
};

// After an aborted table wait: a second bounded wait for the bulk loads still
// in flight into this warp's table (they must land before the block's shared
// memory can be given to another block), then for this warp's bulk stores.
__device__ __forceinline__ void prog_drain(WarpTma& tma) {
  long long polls = 0;
  while (!mbar_try_wait(tma.mbar, tma.phase) && ++polls <= kMbarMaxPolls) {
  }
  tma.phase ^= 1u;
  bulk_wait_all();
  __syncwarp();
}

// One pass from A (prog_run_chain's FROM_A): the own rows of a
// refactorization segment take A(src, s) converted to T, zero at fill slots
// (src < 0) and past S, which is what the scatter would have stored; src is
// ProgDev::load_src of the row.  Every LU slot is an own row of exactly one
// segment (its column's) and no segment reads it earlier, so these rows
// replace the scatter's write and the refactorization's first read of the
// slot.  Plain 8 * LW-byte loads by all lanes, kOwnInFlight rows at a time,
// while the table's other rows arrive by bulk copies.  FP64: four rows (35k
// plant, 512 scenarios: 2 / 4 rows 464 / 432 us); FP32: five, with the
// kernel's register budget below (from_a_min_blocks).
#ifndef PVGLU_OWN_IN_FLIGHT_F32
#define PVGLU_OWN_IN_FLIGHT_F32 5
#endif
#ifndef PVGLU_OWN_IN_FLIGHT_F64
#define PVGLU_OWN_IN_FLIGHT_F64 4
#endif
// Levels with at most one block of items per SM (the narrow levels: a few
// warps per SM, registers to spare) keep this many own rows in flight.
constexpr int kOwnInFlightNarrow = 16;

// Own rows [l_begin, l_end) of the segment whose sources start at src
// (ProgDev::load_src + load_begin).  NARROW: kOwnInFlightNarrow rows at a time.
template <typename T, int LW, bool NARROW = false>
__device__ __forceinline__ void load_own_from_a(const int* src, int l_begin, int l_end,
                                                const double* __restrict__ a, int ld, int s0,
                                                int S, LaneV<T, LW>* t) {
  using VA = LaneV<double, LW>;
  using V = LaneV<T, LW>;
  constexpr int kOwnInFlight =
      NARROW ? kOwnInFlightNarrow
             : (sizeof(T) == 4 ? PVGLU_OWN_IN_FLIGHT_F32 : PVGLU_OWN_IN_FLIGHT_F64);
  const int lane = threadIdx.x & 31;
  const int s = s0 + LW * lane;
  for (int l0 = l_begin; l0 < l_end; l0 += 32) {
    const int nb = min(32, l_end - l0);
    const int m = lane < nb ? __ldg(src + l0 + lane) : -1;
    for (int k = 0; k < nb; k += kOwnInFlight) {
      VA av[kOwnInFlight];
#pragma unroll
      for (int j = 0; j < kOwnInFlight; j++) {
        const int mj = __shfl_sync(0xffffffffu, m, (k + j) & 31);
        av[j] = VA{};
        if (k + j < nb && mj >= 0)
          av[j] = ld_lane<VA>(a + (size_t)(unsigned)mj * (unsigned)ld + s);
      }
#pragma unroll
      for (int j = 0; j < kOwnInFlight; j++) {
        if (k + j < nb) {
          V o;
#pragma unroll
          for (int p = 0; p < LW; p++)
            lane_part(o, p) = s + p < S ? convert<T>(lane_part(av[j], p)) : T(0);
          t[(l0 + k + j) << 5] = o;
        }
      }
    }
  }
}

// L2 prefetch of the A rows that load_own_from_a will read for own rows
// [0, n_a): issued a segment ahead, so that those plain loads find their rows
// in L2 instead of waiting for DRAM.  FP64 only: the FP64 levels are bound by
// the FP64 pipe and hide the prefetch's index load (486 -> 466 us at two rows
// in flight); the FP32 levels wait on it (179 -> 210 us).
template <int LW>
__device__ __forceinline__ void prefetch_own_from_a(const int* src, int n_a,
                                                    const double* __restrict__ a, int ld,
                                                    int s0) {
  for (int l = threadIdx.x & 31; l < n_a; l += 32) {
    const int m = __ldg(src + l);
    if (m >= 0)
      bulk_prefetch_l2(a + (size_t)(unsigned)m * (unsigned)ld + s0, 32 * LW * sizeof(double));
  }
}

#ifndef PVGLU_PREFETCH_OWN_F32
#define PVGLU_PREFETCH_OWN_F32 0
#endif
template <typename T>
constexpr bool kPrefetchOwn = sizeof(T) == 8 || PVGLU_PREFETCH_OWN_F32;

// Runs every segment of `chain`, batched over the 32 * LW scenarios starting
// at s0 (BATCH) or for the single scenario.  sm: this warp's table.
// FROM_A (batched refactorization only): own rows come from `a` (the
// caller's FP64 values, leading dimension ld) instead of the factor values;
// 2: a narrow level's form (load_own_from_a's NARROW).
template <typename T, int KIND, bool BATCH, int LW = 2, int FROM_A = 0>
__device__ __forceinline__ void prog_run_chain(const ProgDev& P, const DevStruct& d, int chain,
                                               T* __restrict__ v, T* __restrict__ x, int ld,
                                               int s0, int S, T* sm, WarpTma& tma,
                                               T pivot_tol, DevStatus* st,
                                               const double* __restrict__ a = nullptr) {
  static_assert(!FROM_A || (KIND < 0 && BATCH), "own rows from A: batched refactor only");
  const int lane = threadIdx.x & 31;
  const int g_begin = __ldg(P.chain_seg + chain), g_end = __ldg(P.chain_seg + chain + 1);
  // Each segment's descriptor and carry moves (read-only) are read one
  // segment ahead: a segment's copies then start without a dependent round
  // of metadata loads.
  int4 sg_next = make_int4(0, 0, 0, 0), cv_next = make_int4(-1, -1, -1, -1);
  if (g_begin < g_end) {
    sg_next = __ldg(P.seg + g_begin);
    cv_next = __ldg(P.carry + g_begin);
    if constexpr (FROM_A && kPrefetchOwn<T>)
      prefetch_own_from_a<LW>(P.load_src + sg_next.x, (sg_next.y >> 16) & 0x3ff, a, ld, s0);
  }
  for (int g = g_begin; g < g_end; g++) {
    const int4 sg = sg_next;
    const int4 cv_g = cv_next;
    if (g + 1 < g_end) {
      sg_next = __ldg(P.seg + g + 1);
      cv_next = __ldg(P.carry + g + 1);
    }
    const int* lr = P.loads + sg.x;
    const int nl = sg.y & 0xffff, n_own = (sg.y >> 16) & 0x3ff, n_carry = (sg.y >> 26) & 7;
    // Rows the previous segment of this chain left in the table: moved, not
    // loaded (to-locals kept for the load loop).
    int c_to[4] = {-1, -1, -1, -1};
    int4 cv = make_int4(-1, -1, -1, -1);
    if (n_carry) {
      cv = cv_g;
      c_to[0] = cv.x & 0xffff;
      if (n_carry > 1) c_to[1] = cv.y & 0xffff;
      if (n_carry > 2) c_to[2] = cv.z & 0xffff;
      if (n_carry > 3) c_to[3] = cv.w & 0xffff;
    }
    auto is_carried = [&](int l) {
      return l == c_to[0] || l == c_to[1] || l == c_to[2] || l == c_to[3];
    };
    if (BATCH) {
      using V2 = LaneV<T, LW>;
      constexpr int kLaneRow = 32 * LW;  // T values of a table row
      constexpr unsigned kRow = kLaneRow * sizeof(T);
      // The segment's operation words, one int4 (four operations) per lane,
      // fetched before the waits below and broadcast by shuffles: the
      // operations then wait on no memory but the table.
      const int4* o4 = P.ops + (sg.z >> 2);
      const int n_w = sg.w >> 2;
      int4 ow = make_int4(0, 0, 0, 0);
      if (lane < n_w) ow = __ldg(o4 + lane);
      // The previous segment's bulk stores must have read the table; when
      // this segment loads rows they wrote, they must also be complete.
      if ((sg.y >> 30) & 1) bulk_wait_all();
      else bulk_wait_read();
      __syncwarp();
      if (n_carry) {
        V2* t = reinterpret_cast<V2*>(sm) + lane;
        const int from[4] = {cv.x >> 16, cv.y >> 16, cv.z >> 16, cv.w >> 16};
        V2 hold[4];
        for (int c = 0; c < n_carry; c++) hold[c] = t[from[c] << 5];
        __syncwarp();
        for (int c = 0; c < n_carry; c++) t[c_to[c] << 5] = hold[c];
        __syncwarp();
      }
      // One pass from A: own rows [0, n_a) are read from A below, the rest
      // by bulk copies.
      const int n_a = FROM_A ? n_own : 0;
      int n_bulk = nl - n_a;
      for (int c = 0; c < n_carry; c++)
        if (c_to[c] >= n_a) n_bulk--;
      if (lane == 0) mbar_arrive_expect_tx(tma.mbar, (unsigned)n_bulk * kRow);
      __syncwarp();
      for (int l = n_a + lane; l < nl; l += 32)
        if (!is_carried(l))
          bulk_load(sm + l * kLaneRow, prog_row<T, KIND>(__ldg(lr + l), v, x, ld, s0), kRow,
                    tma.mbar);
      if constexpr (FROM_A) {
        if (kPrefetchOwn<T> && g + 1 < g_end)
          prefetch_own_from_a<LW>(P.load_src + sg_next.x, (sg_next.y >> 16) & 0x3ff, a, ld, s0);
        load_own_from_a<T, LW, FROM_A == 2>(P.load_src + sg.x, 0, n_a, a, ld, s0, S,
                                            reinterpret_cast<V2*>(sm) + lane);
      }
      long long polls = 0;
      bool late = false;
      while (!mbar_try_wait(tma.mbar, tma.phase)) {
        if (++polls > kMbarMaxPolls) {
          late = true;
          break;
        }
      }
      // The table is either complete for every lane or the warp stops: no
      // operation runs on a partly loaded table and nothing is stored.
      if (__any_sync(0xffffffffu, late)) {
        if (lane == 0) report_error(st, 6, -2, s0);
        tma.aborted = true;
        prog_drain(tma);
        return;
      }
      tma.phase ^= 1u;
      V2* t = reinterpret_cast<V2*>(sm) + lane;
      for (int k0 = 0; k0 < n_w; k0 += 32) {
        if (k0 > 0) ow = lane + k0 < n_w ? __ldg(o4 + k0 + lane) : make_int4(0, 0, 0, 0);
        const int kn = min(32, n_w - k0);
        for (int k = 0; k < kn; k++) {
          const uint32_t wx = (uint32_t)__shfl_sync(0xffffffffu, ow.x, k);
          const uint32_t wy = (uint32_t)__shfl_sync(0xffffffffu, ow.y, k);
          const uint32_t wz = (uint32_t)__shfl_sync(0xffffffffu, ow.z, k);
          const uint32_t ww = (uint32_t)__shfl_sync(0xffffffffu, ow.w, k);
          const int base = sg.z + 4 * (k0 + k);
          exec_op_lane<T, LW>(wx, base, P.op_col, t, s0 + LW * lane, S, pivot_tol, st);
          exec_op_lane<T, LW>(wy, base + 1, P.op_col, t, s0 + LW * lane, S, pivot_tol, st);
          exec_op_lane<T, LW>(wz, base + 2, P.op_col, t, s0 + LW * lane, S, pivot_tol, st);
          exec_op_lane<T, LW>(ww, base + 3, P.op_col, t, s0 + LW * lane, S, pivot_tol, st);
        }
      }
      // Make this lane's table writes visible to the async proxy, then let
      // lanes write back the own rows with bulk stores.
      fence_proxy_async_smem();
      __syncwarp();
      for (int l = lane; l < n_own; l += 32)
        bulk_store(prog_row<T, KIND>(__ldg(lr + l), v, x, ld, s0), sm + l * kLaneRow, kRow);
      bulk_commit();
    } else {
      if (n_carry) {
        const int from[4] = {cv.x >> 16, cv.y >> 16, cv.z >> 16, cv.w >> 16};
        T hold[4];
        for (int c = 0; c < n_carry; c++) hold[c] = sm[from[c]];
        __syncwarp();
        if (lane == 0)
          for (int c = 0; c < n_carry; c++) sm[c_to[c]] = hold[c];
      }
      for (int l = lane; l < nl; l += 32)
        if (!is_carried(l)) sm[l] = prog_fetch1<T, KIND>(__ldg(lr + l), v, x);
      __syncwarp();
      if (lane == 0) {
        const int4* o4 = P.ops + (sg.z >> 2);
        for (int k = 0; k < (sg.w >> 2); k++) {
          const int4 w = __ldg(o4 + k);
          const int base = sg.z + 4 * k;
          exec_op1<T>((uint32_t)w.x, base, P.op_col, sm, S, pivot_tol, st);
          exec_op1<T>((uint32_t)w.y, base + 1, P.op_col, sm, S, pivot_tol, st);
          exec_op1<T>((uint32_t)w.z, base + 2, P.op_col, sm, S, pivot_tol, st);
          exec_op1<T>((uint32_t)w.w, base + 3, P.op_col, sm, S, pivot_tol, st);
        }
      }
      __syncwarp();
      for (int l = lane; l < n_own; l += 32) prog_store1<T, KIND>(__ldg(lr + l), sm[l], v, x);
      __syncwarp();
    }
  }
}

// Chains [cb, ce) of one level: work item = (chain, group of 32 * LW
// scenarios) in batched mode, chain alone in single mode; one warp per item.
// In batched mode every bulk store of the warp is complete when this returns.
template <typename T, int KIND, bool BATCH, int LW = 2, int FROM_A = 0>
__device__ __forceinline__ void prog_run_level(const ProgDev& P, const DevStruct& d, int cb,
                                               int ce, T* __restrict__ v, T* __restrict__ x,
                                               int ld, int S, T* sm_warp, WarpTma& tma,
                                               T pivot_tol, DevStatus* st,
                                               const int* done, int warp_id, int n_warps,
                                               const double* __restrict__ a = nullptr) {
  constexpr int group = 32 * LW;
  const int groups = BATCH ? ld / group : 1;
  const int items = (ce - cb) * groups;
  const int lane = threadIdx.x & 31;
  for (int it = warp_id; it < items; it += n_warps) {
    if (BATCH && tma.aborted) break;
    const int ci = BATCH ? it / groups : it;
    const int c = cb + ci;
    const int s0 = BATCH ? (it - ci * groups) * group : 0;
    if (BATCH && done) {
      bool idle = true;
#pragma unroll
      for (int k = 0; k < LW; k++) {
        const int sa = s0 + LW * lane + k;
        idle = idle && (sa >= S || done[sa]);
      }
      if (__all_sync(0xffffffffu, idle)) continue;
    }
    prog_run_chain<T, KIND, BATCH, LW, FROM_A>(P, d, c, v, x, ld, s0, S, sm_warp, tma,
                                               pivot_tol, st, a);
  }
  if (BATCH) {
    bulk_wait_all();
    fence_proxy_async();
  }
}

// Host: lets `kernel` request up to the device's opt-in shared memory per
// block minus its own static shared memory.  The attribute is per kernel for
// the whole process and handles differ in table size, so it is set to the
// limit; a launch still requests only what its tables need.  Returns
// cudaSuccess or the error (cleared).
inline cudaError_t allow_max_dynamic_smem(const void* kernel) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa{};
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) cudaGetLastError();
  return e;
}

// Table layout of a block: warps_per_block tables, then one mbarrier per
// warp.  Returns this warp's table and initialises its mbarrier.
template <typename T, bool BATCH, int LW = 2>
__device__ __forceinline__ T* prog_setup_warp(unsigned char* smem_raw, int max_locals,
                                              WarpTma& tma) {
  const int w = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const size_t table = (size_t)max_locals * (BATCH ? 32 * LW : 1) * sizeof(T);
  T* sm = reinterpret_cast<T*>(smem_raw + (size_t)w * table);
  tma.mbar = reinterpret_cast<unsigned long long*>(smem_raw + (size_t)nw * table) + w;
  tma.phase = 0;
  tma.aborted = false;
  if (BATCH) {
    if ((threadIdx.x & 31) == 0) mbar_init(tma.mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
  }
  return sm;
}

template <typename T, bool BATCH, int LW = 2>
__host__ __device__ size_t prog_smem_bytes(int max_locals, int warps_per_block) {
  return (size_t)warps_per_block * max_locals * (BATCH ? 32 * LW : 1) * sizeof(T) +
         (size_t)warps_per_block * sizeof(unsigned long long);
}

// done: per-scenario skip of the solves (NULL for the refactorization);
// ndone (or NULL): the launch does nothing once every scenario is done.
// `table`: the level's table budget (its programs were built for it).
// LW: scenarios per lane of the batched form (programs do not depend on it).
template <typename T, int KIND, bool BATCH, int LW = 2>
__global__ void __launch_bounds__(kProgBlock, prog_min_blocks<T>())
k_prog_level(ProgDev P, int table, DevStruct d, int cb, int ce,
                             T* __restrict__ v, T* __restrict__ x, int ld, int S, T pivot_tol,
                             DevStatus* st, const int* done, const int* ndone) {
  if (ndone && __ldcg(ndone) >= S) return;
  // A table wait that ran out in an earlier level stops the later levels.
  if (BATCH && __ldcg(&st->code) == 6) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WarpTma tma;
  T* sm = prog_setup_warp<T, BATCH, LW>(smem_raw, table, tma);
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  prog_run_level<T, KIND, BATCH, LW>(P, d, cb, ce, v, x, ld, S, sm, tma, pivot_tol, st, done,
                                     warp_id, n_warps);
}

// One level of the batched refactorization whose own rows are read from the
// caller's FP64 values `a` (leading dimension ld): scatter and refactor in
// one pass.  Only for programs without WIDE levels, where every LU slot is an
// own row of some level's segment.  NARROW: for levels with at most one block
// of items per SM, compiled for one block per SM (more own rows in flight).
// The FP32 one pass at 8 resident blocks per SM (64 registers) keeps five
// own rows in flight without spilling (35k plant, 512 scenarios: 9 blocks
// with 4 rows 171-173 us, 8 with 5 / 6 / 7 rows 159 / 160-161 / 162 us, 7 or
// 6 blocks with 8 rows 195 / 191 us).
#ifndef PVGLU_FROM_A_MIN_BLOCKS_F32
#define PVGLU_FROM_A_MIN_BLOCKS_F32 8
#endif
template <typename T>
constexpr int from_a_min_blocks() {
  return sizeof(T) == 4 ? PVGLU_FROM_A_MIN_BLOCKS_F32 : prog_min_blocks<T>();
}
template <typename T, int LW = 2, bool NARROW = false>
__global__ void __launch_bounds__(kProgBlock, NARROW ? 1 : from_a_min_blocks<T>())
k_prog_refactor_from_a(ProgDev P, int table, DevStruct d, int cb, int ce, T* __restrict__ v,
                       const double* __restrict__ a, int ld, int S, T pivot_tol,
                       DevStatus* st) {
  if (__ldcg(&st->code) == 6) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WarpTma tma;
  T* sm = prog_setup_warp<T, true, LW>(smem_raw, table, tma);
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  prog_run_level<T, -1, true, LW, NARROW ? 2 : 1>(P, d, cb, ce, v, nullptr, ld, S, sm, tma,
                                                  pivot_tol, st, nullptr, warp_id, n_warps, a);
}

// ---------------------------------------------------------------------------
// Several size classes (numeric handles with different symbolic analyses) in
// one launch per level: the work items of level `lv` of every class are
// numbered consecutively and each warp finds its class by the item ranges.
// Classes share T, the phase and the batched layout; each keeps its own
// programs, structure, values, vector and status.
constexpr int kMaxClasses = 4;

template <typename T>
struct ClassLaunch {
  ProgDev P;
  DevStruct d;
  T* v;
  T* x;
  int ld, S, cb, ce, groups;
  int item_begin;  // first global item of this class
  DevStatus* st;
  T pivot_tol;
};

template <typename T>
struct MultiLaunch {
  ClassLaunch<T> c[kMaxClasses];
  int n;       // classes in this launch
  int items;   // total work items
};

template <typename T, int KIND, bool BATCH>
__global__ void __launch_bounds__(kProgBlock, prog_min_blocks<T>())
k_prog_level_multi(MultiLaunch<T> M, int table) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  WarpTma tma;
  T* sm = prog_setup_warp<T, BATCH>(smem_raw, table, tma);
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  // Constant class indices keep every field a direct kernel-parameter read
  // (a runtime index would copy the descriptors to local memory).
  auto run = [&](const ClassLaunch<T>& C, int it) {
    const int local = it - C.item_begin;
    const int ci = BATCH ? local / C.groups : local;
    const int s0 = BATCH ? (local - ci * C.groups) * kGroup : 0;
    prog_run_chain<T, KIND, BATCH>(C.P, C.d, C.cb + ci, C.v, C.x, C.ld, s0, C.S, sm, tma,
                                   C.pivot_tol, C.st);
  };
  for (int it = warp_id; it < M.items; it += n_warps) {
    if (BATCH && tma.aborted) break;
    if (M.n > 3 && it >= M.c[3].item_begin) run(M.c[3], it);
    else if (M.n > 2 && it >= M.c[2].item_begin) run(M.c[2], it);
    else if (M.n > 1 && it >= M.c[1].item_begin) run(M.c[1], it);
    else run(M.c[0], it);
  }
  if (BATCH) {
    bulk_wait_all();
    fence_proxy_async();
  }
}

}  // namespace pvglu
