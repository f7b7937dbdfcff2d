// Wide units: the columns (refactorization) and rows (solves) too wide for
// any chain-program table, each executed by a whole block (programs.hpp,
// WidePlan).  They are the dense trailing columns and rows of plants whose
// strings share bus nodes: eliminating a string from its bus end fills the
// bus row and column with one entry per string node.  The reference runs
// such levels with 32 threads per column once a level's longest row passes 64
// entries (factorize_electrical_system_CUDA.cu:75-77, triangular_substitution.cu:
// 153-159), walking the column's updates with atomics.
//
// FP64 stays bit-exact with the reference's sequential order: every entry
// receives its updates one at a time, in ascending j, each product and each
// subtraction rounded on its own.  The parallelism comes from elsewhere:
//   * refactorization of column k in gather form, scheduled inside the
//     column: the column's targets form chains (a target that reads only the
//     target before it, as the string nodes of a bus column do, joins that
//     target's chain), the chains of a chain level run in parallel (a thread
//     or, batched, a warp per chain), one block barrier per chain level;
//   * a target or solve row with many updates: warps of the block compute the
//     products of a chunk in parallel (each rounded as the sequential code
//     rounds it) into shared memory while one warp subtracts the previous
//     chunk's products in order (batched: a lane per scenario pair, or per
//     scenario on levels with few items; single: one lane).
// Single scenario: the column is staged in shared memory when it fits.
#pragma once
#include <cuda_runtime.h>

#include "chainprog.cuh"
#include "kernels.cuh"

namespace pvglu {

// Separately rounded product and difference (the reference's rounding).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// Products and differences of the lane values (LaneV, chainprog.cuh): a
// WIDE level with few items runs with one scenario per lane (LW = 1), on
// twice the blocks, each with half the FP64 work.
template <typename T>
__device__ __forceinline__ T mul_lane(T a, T b) { return mul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sub_lane(T a, T b) { return sub_rn(a, b); }
#define PVGLU_LANE2(V)                                                        \
  __device__ __forceinline__ V mul_lane(V a, V b) {                           \
    return {mul_rn(a.x, b.x), mul_rn(a.y, b.y)};                              \
  }                                                                           \
  __device__ __forceinline__ V sub_lane(V a, V b) {                           \
    return {sub_rn(a.x, b.x), sub_rn(a.y, b.y)};                              \
  }
PVGLU_LANE2(double2)
PVGLU_LANE2(float2)
#undef PVGLU_LANE2

// Bytes of one scratch row of the ordered sums (two scenarios per lane: the
// larger of the batched forms).
template <typename T, bool BATCH>
__host__ __device__ constexpr int wide_row_bytes() {
  return BATCH ? 32 * 2 * (int)sizeof(T) : (int)sizeof(T);
}
// Smallest scratch: one chunk row per producer thread (single) or warp
// (batched), two buffers.
template <typename T, bool BATCH>
__host__ __device__ constexpr int wide_scratch_min(int threads) {
  return 2 * (BATCH ? threads / 32 - 1 : threads - 32) * wide_row_bytes<T, BATCH>();
}
// Scratch the wide-level launches give the ordered sums: chunks of 64 rows
// (batched) or 8 products per producer thread (single), two buffers.
template <typename T, bool BATCH>
__host__ __device__ constexpr int wide_scratch_bytes(int threads) {
  return 2 * (BATCH ? 64 : 8 * (threads - 32)) * wide_row_bytes<T, BATCH>();
}

// acc - sum_e a_e * b_e in the order e = 0 .. count-1, each product and each
// difference rounded on its own.  Warps 1.. of the block form the products of
// a chunk of entries in shared memory (batched: a warp per entry, LW
// scenarios per lane; single: a thread per entry) while warp 0 subtracts the
// previous chunk's products in order (batched: every lane for its LW
// scenarios; single: lane 0), two chunk buffers in turn.  `ix(e, ia, ib)`
// gives the two operand indices of entry e and `ab(ia, ib, a, b)` the
// operands (T, or the lane's LW scenarios); a batched producer
// warp loads the indices of its entries with one lane each and broadcasts
// them, so every entry costs one round of index loads and one of operand
// loads, the entries' loads in flight together.
// Returns the result in warp 0 (single: in its lane 0).  All threads of the
// block (at least two warps) must call it.  scratch: scratch_bytes of shared
// memory, at least wide_scratch_min<T, BATCH>(blockDim.x).
template <typename T, bool BATCH, int LW, typename IX, typename AB>
__device__ __forceinline__ typename std::conditional<BATCH, LaneV<T, LW>, T>::type
ordered_sub_block(typename std::conditional<BATCH, LaneV<T, LW>, T>::type acc, int count,
                  IX ix, AB ab, unsigned char* scratch, int scratch_bytes) {
  using V = typename std::conditional<BATCH, LaneV<T, LW>, T>::type;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int producers = BATCH ? (blockDim.x >> 5) - 1 : (int)blockDim.x - 32;
  const int rb = BATCH ? 32 * LW * (int)sizeof(T) : (int)sizeof(T);
  int ch = scratch_bytes / (2 * rb);
  ch = max(producers, ch - ch % producers);  // rows per chunk, a multiple of the producers
  V* buf = reinterpret_cast<V*>(scratch);
  const int stride = BATCH ? 32 : 1;          // buffer elements per row
  const int nchunks = (count + ch - 1) / ch;
  auto produce = [&](int c) {
    V* out = buf + (size_t)(c & 1) * ch * stride;
    const int base = c * ch;
    const int me = BATCH ? warp - 1 : tid - 32;
    // Up to U entries' operands in flight, then their products (two for
    // FP64 pairs, which keeps the kernels of up to 512 threads within 128
    // registers).
    constexpr int U = (BATCH && LW * sizeof(T) == 16) ? 2 : 4;
    for (int r0 = me; r0 < ch; r0 += U * producers) {
      V a[U], b[U];
      if constexpr (BATCH) {
        int ia = 0, ib = 0;
        if (lane < U && r0 + lane * producers < ch && base + r0 + lane * producers < count)
          ix(base + r0 + lane * producers, ia, ib);
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int ja = __shfl_sync(0xffffffffu, ia, u), jb = __shfl_sync(0xffffffffu, ib, u);
          if (r0 + u * producers < ch && base + r0 + u * producers < count) ab(ja, jb, a[u], b[u]);
        }
      } else {
        int ia[U], ib[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = base + r0 + u * producers;
          if (r0 + u * producers < ch && e < count) ix(e, ia[u], ib[u]);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = base + r0 + u * producers;
          if (r0 + u * producers < ch && e < count) ab(ia[u], ib[u], a[u], b[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int r = r0 + u * producers;
        if (r < ch && base + r < count) out[r * stride + (BATCH ? lane : 0)] = mul_lane(a[u], b[u]);
      }
    }
  };
  if (warp > 0 && nchunks > 0) produce(0);
  __syncthreads();
  for (int c = 0; c < nchunks; c++) {
    if (warp == 0) {
      if (BATCH || lane == 0) {
        const V* in = buf + (size_t)(c & 1) * ch * stride;
        const int m = min(ch, count - c * ch);
        for (int i = 0; i < m; i++) acc = sub_lane(acc, in[i * stride + (BATCH ? lane : 0)]);
      }
    } else if (c + 1 < nchunks) {
      produce(c + 1);
    }
    __syncthreads();
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Refactorization of wide column k = P.w_unit[w] for the scenario group at
// s0 (batched) or the single scenario, chain level by chain level
// (programs.hpp, WidePlan): the chains of a level spread over the block's
// threads (batched: warps), each computed in order, then the level's long
// targets one at a time by the whole block.  A batched warp loads the
// records of 32 targets of its chain at a time (one per lane; the next 32
// already in flight) and broadcasts them by shuffles; the row loads of the
// next G targets (their own values, the L operand of single-pair targets)
// are then issued together.  A source written earlier in the same chain
// comes from the register that holds the previous target or, further back,
// from a plain load after the thread's own store.  smem: the block's shared
// memory (smem_bytes of it); the column is staged there in single mode when
// len * sizeof(T) + scratch fits.
template <typename T, bool BATCH, int LW = 2>
__device__ void wide_refactor(const ProgDev& P, const DevStruct& d, int w, int s0,
                              T* __restrict__ v, int ld, int S, T pivot_tol, DevStatus* st,
                              unsigned char* smem, int smem_bytes) {
  constexpr int G = sizeof(T) == 8 ? 3 : 4;  // targets whose loads are in flight together
  const int k = __ldg(P.w_unit + w);
  const int c0 = __ldg(d.colptr + k), dk = __ldg(d.diag + k), c1 = __ldg(d.colptr + k + 1);
  const int len = c1 - c0;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int l_begin = __ldg(P.w_lvl + w), l_end = __ldg(P.w_lvl + w + 1);
  auto is_long = [&](int c) {
    const int t0 = __ldg(P.ch_tgt + c);
    return __ldg(P.ch_tgt + c + 1) - t0 == 1 && __ldg(&P.tg_rec[t0].z) > kWideLong;
  };
  if constexpr (!BATCH) {
    const int scratch = min(wide_scratch_bytes<T, false>(nthr), smem_bytes);
    const bool staged = (int64_t)len * (int)sizeof(T) + scratch <= smem_bytes;
    T* col = reinterpret_cast<T*>(smem + scratch);
    unsigned char* scr = smem;
    if (staged)
      for (int i = tid; i < len; i += nthr) col[i] = ldv(v + c0 + i);
    __syncthreads();
    // Final values (earlier levels, earlier columns) and values this thread
    // wrote itself (plain accesses, ordered after its own stores).
    auto get = [&](int slot) -> T { return staged ? col[slot - c0] : ldv(v + slot); };
    auto get_own = [&](int slot) -> T { return staged ? col[slot - c0] : v[slot]; };
    auto put = [&](int slot, T val) {
      if (staged) col[slot - c0] = val;
      else v[slot] = val;
    };
    for (int l = l_begin; l < l_end; l++) {
      const int h0 = __ldg(P.lv_chain + l), h1 = __ldg(P.lv_chain + l + 1);
      for (int c = h0 + tid; c < h1; c += nthr) {
        if (is_long(c)) continue;
        const int t1 = __ldg(P.ch_tgt + c + 1);
        int prev = -1;
        T prev_v = T(0);
        for (int t = __ldg(P.ch_tgt + c); t < t1; t++) {
          const int4 r = __ldg(P.tg_rec + t);
          T acc = get(r.x);
          if (r.z == 1) {
            const T u = r.y >= 0 ? get(r.y) : (~r.y == prev ? prev_v : get_own(~r.y));
            acc = fnms(acc, ldv(v + r.w), u);
          } else {
            for (int e = r.y; e < r.y + r.z; e++) {
              const int p = __ldg(P.pr_p + e);
              const T u = p >= 0 ? get(p) : (~p == prev ? prev_v : get_own(~p));
              acc = fnms(acc, ldv(v + __ldg(P.pr_q + e)), u);
            }
          }
          put(r.x, acc);
          prev = r.x;
          prev_v = acc;
        }
      }
      __syncthreads();
      for (int c = h0; c < h1; c++) {  // long targets, one at a time by the block
        if (!is_long(c)) continue;
        const int4 r = __ldg(P.tg_rec + __ldg(P.ch_tgt + c));
        T acc = get(r.x);
        acc = ordered_sub_block<T, false, LW>(
            acc, r.z,
            [&](int e, int& ia, int& ib) {
              ia = __ldg(P.pr_q + r.y + e);
              ib = __ldg(P.pr_p + r.y + e);
            },
            [&](int ia, int ib, T& a, T& b) {
              a = ldv(v + ia);
              b = get(ib);
            },
            scr, scratch);
        if (tid == 0) put(r.x, acc);
        __syncthreads();
      }
    }
    const T piv = get(dk);
    if (tid == 0 && !(fabs(piv) >= pivot_tol) && S > 0) report_error(st, 3, k, 0);
    if constexpr (std::is_same<T, float>::value) {
      const float r = __frcp_rn(piv);
      for (int q = dk + 1 + tid; q < c1; q += nthr) put(q, get(q) * r);
    } else {
      for (int q = dk + 1 + tid; q < c1; q += nthr) put(q, get(q) / piv);
    }
    __syncthreads();
    if (staged)
      for (int i = tid; i < len; i += nthr) v[c0 + i] = col[i];
    __syncthreads();
  } else {
    using V2 = LaneV<T, LW>;
    const int lane = tid & 31, warp = tid >> 5, nw = nthr >> 5;
    const int s = s0 + LW * lane;
    auto row = [&](int slot) { return v + (int64_t)slot * ld + s; };
    auto shfl4 = [](int4 r, int src) {
      r.x = __shfl_sync(0xffffffffu, r.x, src);
      r.y = __shfl_sync(0xffffffffu, r.y, src);
      r.z = __shfl_sync(0xffffffffu, r.z, src);
      r.w = __shfl_sync(0xffffffffu, r.w, src);
      return r;
    };
    for (int l = l_begin; l < l_end; l++) {
      const int h0 = __ldg(P.lv_chain + l), h1 = __ldg(P.lv_chain + l + 1);
      for (int c = h0 + warp; c < h1; c += nw) {
        if (is_long(c)) continue;
        const int ct0 = __ldg(P.ch_tgt + c), ct1 = __ldg(P.ch_tgt + c + 1);
        int prev = -1;
        V2 prev_v{};
        // A source of this chain: the previous target's register, or a
        // plain load of a row this lane stored earlier.
        auto own = [&](int p) -> V2 {
          return p == prev ? prev_v : *reinterpret_cast<const V2*>(row(p));
        };
        int4 win = make_int4(0, 0, 0, 0);
        if (ct0 + lane < ct1) win = __ldg(P.tg_rec + ct0 + lane);
        for (int w0 = ct0; w0 < ct1; w0 += 32) {
          const int wn = min(32, ct1 - w0);
          int4 nxt = make_int4(0, 0, 0, 0);
          if (w0 + 32 + lane < ct1) nxt = __ldg(P.tg_rec + w0 + 32 + lane);
          for (int i0 = 0; i0 < wn; i0 += G) {
            int4 r[G];
            V2 cur[G], qa[G];
#pragma unroll
            for (int u = 0; u < G; u++) {
              if (i0 + u < wn) {
                r[u] = shfl4(win, i0 + u);
                cur[u] = ld_lane<V2>(row(r[u].x));
                if (r[u].z == 1) qa[u] = ld_lane<V2>(row(r[u].w));
              }
            }
#pragma unroll
            for (int u = 0; u < G; u++) {
              if (i0 + u >= wn) continue;
              V2 acc = cur[u];
              if (r[u].z == 1) {
                acc = fnms_lane(acc, qa[u], r[u].y >= 0 ? ld_lane<V2>(row(r[u].y)) : own(~r[u].y));
              } else {
                const int e1 = r[u].y + r[u].z;
                int e = r[u].y;
                // Two updates' operands in flight at a time; the
                // subtractions stay in order.
                for (; e + 2 <= e1; e += 2) {
                  V2 a[2], b[2];
                  int pp[2];
#pragma unroll
                  for (int i = 0; i < 2; i++) {
                    a[i] = ld_lane<V2>(row(__ldg(P.pr_q + e + i)));
                    pp[i] = __ldg(P.pr_p + e + i);
                    if (pp[i] >= 0) b[i] = ld_lane<V2>(row(pp[i]));
                  }
#pragma unroll
                  for (int i = 0; i < 2; i++)
                    acc = fnms_lane(acc, a[i], pp[i] >= 0 ? b[i] : own(~pp[i]));
                }
                for (; e < e1; e++) {
                  const int p = __ldg(P.pr_p + e);
                  const V2 a = ld_lane<V2>(row(__ldg(P.pr_q + e)));
                  acc = fnms_lane(acc, a, p >= 0 ? ld_lane<V2>(row(p)) : own(~p));
                }
              }
              *reinterpret_cast<V2*>(row(r[u].x)) = acc;
              prev = r[u].x;
              prev_v = acc;
            }
          }
          win = nxt;
        }
      }
      __syncthreads();
      for (int c = h0; c < h1; c++) {
        if (!is_long(c)) continue;
        const int4 r = __ldg(P.tg_rec + __ldg(P.ch_tgt + c));
        T* tp = row(r.x);
        V2 acc = ld_lane<V2>(tp);
        acc = ordered_sub_block<T, true, LW>(
            acc, r.z,
            [&](int e, int& ia, int& ib) {
              ia = __ldg(P.pr_q + r.y + e);
              ib = __ldg(P.pr_p + r.y + e);
            },
            [&](int ia, int ib, V2& a, V2& b) {
              a = ld_lane<V2>(row(ia));
              b = ld_lane<V2>(row(ib));
            },
            smem, smem_bytes);
        if (warp == 0) *reinterpret_cast<V2*>(tp) = acc;
        __syncthreads();
      }
    }
    const V2 piv = ld_lane<V2>(row(dk));
    // The L part divided by the pivot (FP32: times one reciprocal).
    auto scale = [&](T val, T pv) -> T {
      if constexpr (std::is_same<T, float>::value) return val * __frcp_rn(pv);
      else return val / pv;
    };
    if constexpr (LW == 2) {
      if (warp == 0) {
        if (!(fabs(piv.x) >= pivot_tol) && s < S) report_error(st, 3, k, s);
        if (!(fabs(piv.y) >= pivot_tol) && s + 1 < S) report_error(st, 3, k, s + 1);
      }
      for (int q = dk + 1 + warp; q < c1; q += nw) {
        V2 val = ld_lane<V2>(row(q));
        val.x = scale(val.x, piv.x);
        val.y = scale(val.y, piv.y);
        *reinterpret_cast<V2*>(row(q)) = val;
      }
    } else {
      if (warp == 0 && !(fabs(piv) >= pivot_tol) && s < S) report_error(st, 3, k, s);
      for (int q = dk + 1 + warp; q < c1; q += nw) *row(q) = scale(ld_lane<V2>(row(q)), piv);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// One wide unknown of a solve (KIND 0: L row, 1: U row, 2: U^T column, 3:
// L^T column), the same arithmetic and order as solve_unknown.
template <typename T, int KIND, bool BATCH, int LW = 2>
__device__ void wide_solve(const ProgDev& P, const DevStruct& d, int w, int s0,
                           const T* __restrict__ v, T* __restrict__ x, int ld,
                           unsigned char* smem, int smem_bytes) {
  const int i = __ldg(P.w_unit + w);
  int b0, cnt, dg = -1;
  if (KIND == 0) {
    b0 = __ldg(d.lrow_ptr + i);
    cnt = __ldg(d.lrow_ptr + i + 1) - b0;
  } else if (KIND == 1) {
    b0 = __ldg(d.urow_ptr + i);
    cnt = __ldg(d.urow_ptr + i + 1) - b0;
    dg = __ldg(d.diag + i);
  } else if (KIND == 2) {
    b0 = __ldg(d.colptr + i);
    dg = __ldg(d.diag + i);
    cnt = dg - b0;
  } else {
    b0 = __ldg(d.diag + i) + 1;
    cnt = __ldg(d.colptr + i + 1) - b0;
  }
  // Entry e (in order): value slot and solution row.
  auto entry = [&](int e, int& slot, int& col) {
    if (KIND == 0) {
      slot = __ldg(d.lrow_slot + b0 + e);
      col = __ldg(d.lrow_col + b0 + e);
    } else if (KIND == 1) {  // descending: the reference's backward sweep order
      slot = __ldg(d.urow_slot + b0 + cnt - 1 - e);
      col = __ldg(d.urow_col + b0 + cnt - 1 - e);
    } else {
      slot = b0 + e;
      col = __ldg(d.csc_row + b0 + e);
    }
  };
  if constexpr (!BATCH) {
    T acc = ldv(x + i);
    acc = ordered_sub_block<T, false, LW>(
        acc, cnt, [&](int e, int& slot, int& col) { entry(e, slot, col); },
        [&](int slot, int col, T& a, T& b) {
          a = ldv(v + slot);
          b = ldv(x + col);
        },
        smem, smem_bytes);
    if (threadIdx.x == 0) {
      if (dg >= 0) acc = acc / ldv(v + dg);
      x[i] = acc;
    }
    __syncthreads();
  } else {
    using V2 = LaneV<T, LW>;
    const int s = s0 + LW * (threadIdx.x & 31);
    V2 acc = ld_lane<V2>(x + (int64_t)i * ld + s);
    acc = ordered_sub_block<T, true, LW>(
        acc, cnt, [&](int e, int& slot, int& col) { entry(e, slot, col); },
        [&](int slot, int col, V2& a, V2& b) {
          a = ld_lane<V2>(v + (int64_t)slot * ld + s);
          b = ld_lane<V2>(x + (int64_t)col * ld + s);
        },
        smem, smem_bytes);
    if ((threadIdx.x >> 5) == 0) {
      if (dg >= 0) {
        const V2 p = ld_lane<V2>(v + (int64_t)dg * ld + s);
        if constexpr (LW == 2) {
          acc.x = acc.x / p.x;
          acc.y = acc.y / p.y;
        } else {
          acc = acc / p;
        }
      }
      *reinterpret_cast<V2*>(x + (int64_t)i * ld + s) = acc;
    }
    __syncthreads();
  }
}

// The wide units [cb, ce) of one WIDE program level: item = (unit, scenario
// group), a block per item, blocks striding over the items.  done (solves of
// a refinement): a group whose scenarios have all converged is skipped.
template <typename T, int KIND, bool BATCH, int LW = 2>
__device__ __forceinline__ void wide_run_level(const ProgDev& P, const DevStruct& d, int cb,
                                               int ce, T* __restrict__ v, T* __restrict__ x,
                                               int ld, int S, T pivot_tol, DevStatus* st,
                                               const int* done, unsigned char* smem,
                                               int smem_bytes, int block, int n_blocks) {
  constexpr int group = 32 * LW;  // scenarios of a batched item
  const int groups = BATCH ? ld / group : 1;
  const int items = (ce - cb) * groups;
  for (int it = block; it < items; it += n_blocks) {
    const int ci = BATCH ? it / groups : it;
    const int s0 = BATCH ? (it - ci * groups) * group : 0;
    if (BATCH && done) {
      __shared__ int idle;
      if (threadIdx.x == 0) {
        int all = 1;
        for (int s = s0; s < s0 + group && all; s++) all = (s >= S || done[s]);
        idle = all;
      }
      __syncthreads();
      const int skip = idle;
      __syncthreads();
      if (skip) continue;
    }
    // The chain's single WIDE segment names the wide unit.
    const int w = __ldg(&P.seg[__ldg(P.chain_seg + cb + ci)].z);
    if (KIND < 0) wide_refactor<T, BATCH, LW>(P, d, w, s0, v, ld, S, pivot_tol, st, smem, smem_bytes);
    else wide_solve<T, (KIND < 0 ? 0 : KIND), BATCH, LW>(P, d, w, s0, v, x, ld, smem, smem_bytes);
  }
}

// Launch form of a WIDE program level (the per-level schedule): kProgBlock
// threads per block, or up to kWideBlockMax when the level has few items;
// batched levels with fewer items than SMs also run with LW = 1.
constexpr int kWideBlockMax = 512;
template <typename T, int KIND, bool BATCH, int LW = 2>
__global__ void __launch_bounds__(kWideBlockMax, 1)
k_wide_level(ProgDev P, DevStruct d, int cb, int ce, T* __restrict__ v, T* __restrict__ x,
             int ld, int S, T pivot_tol, DevStatus* st, const int* done, const int* ndone,
             int smem_bytes) {
  if (ndone && __ldcg(ndone) >= S) return;
  if (__ldcg(&st->code) == 6) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  wide_run_level<T, KIND, BATCH, LW>(P, d, cb, ce, v, x, ld, S, pivot_tol, st, done, smem_raw,
                                     smem_bytes, blockIdx.x, gridDim.x);
}

}  // namespace pvglu
