// sm_103a kernels of the hot path: value scatter, left-looking GLU
// refactorization, triangular solves (forward, backward, transposed),
// permutations and the FP64 residual of iterative refinement.
//
// Layout: the value of LU slot q for scenario s lives at V[q * ld + s] (slot
// major, scenario fastest).  A warp therefore handles one slot or row for 32
// or 64 consecutive scenarios (two per lane with 8/16-byte accesses in the
// batched kernels) and every value access is a coalesced 128-512-byte
// transaction, while the structure indices it reads are warp-uniform.  With a
// single scenario (ld = 1) the same code runs one thread per chain, which is
// the reference's launch shape (factorize_electrical_system_CUDA.cu:72-98).
//
// Refactorization is LEFT-looking: processing column k reads only final
// columns j < k (its U-column dependencies, which are exactly the reference's
// GLU dependency sets, 006_get_dependencies_GLU.cpp:5-47) and writes only
// column k.  That needs no atomics (the reference's right-looking update
// uses atomicAdd, factorize_matrix_GLU_CUDA.cuh:99) and makes every result
// independent of thread scheduling.
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pvglu {

struct DevStruct {
  int n;
  int nnz;
  const int* colptr;     // [n+1] CSC column starts
  const int* csc_row;    // [nnz]
  const int* diag;       // [n] slot of M(j,j)
  const int* slot_src;   // [nnz] A-entry feeding the slot, -1 for fill
  const int* upd_ptr;    // [nnz+1] left-looking update ranges per U slot
  const int* upd_tgt;    // targets in the column being factorized
  const int* lrow_ptr;   // [n+1] strictly lower part by rows
  const int* lrow_slot;
  const int* lrow_col;
  const int* urow_ptr;   // [n+1] strictly upper part by rows
  const int* urow_slot;
  const int* urow_col;
  const int* row_orig;   // [n]
  const int* col_orig;   // [n]
  // A's own pattern (caller order) for the FP64 residual.
  const int* a_rowptr;   // [n+1]
  const int* a_colidx;   // [nnz_a]
  // Level sets: start_chains / columns on the device (start_levels host-side).
  const int* lu_sc; const int* lu_cols;
  const int* l_sc;  const int* l_cols;
  const int* u_sc;  const int* u_cols;
  const int* lt_sc; const int* lt_cols;
};

struct DevStatus {
  int code;      // 0 or first error code
  int column;
  int scenario;
  int pad;
};

__device__ __forceinline__ void report_error(DevStatus* st, int code, int col, int s) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->column = col;
    st->scenario = s;
  }
}

// Loads of values written by other blocks of the same launch bypass L1
// (persistent kernel); in per-level launches a plain load is equally safe.
template <typename T>
__device__ __forceinline__ T ldv(const T* p) { return __ldcg(p); }

// a - b * c.  FP64 rounds the product and the difference separately, as the
// reference's CPU code does (GLU_CSC_CPU_levels_strings.cpp:57,
// GLU_CSC_CPU_Triangular.cpp:10,24); with the same update order per entry the
// FP64 factors and solutions are then bit-identical to the reference's
// sequential path.  FP32 (refined afterwards in FP64) keeps the fused form.
__device__ __forceinline__ double fnms(double a, double b, double c) {
  return __dsub_rn(a, __dmul_rn(b, c));
}
__device__ __forceinline__ float fnms(float a, float b, float c) { return a - b * c; }

// ----------------------------------------------------------------------------
// float <-> double conversions on the integer pipes.  GB300 issues FP64
// instructions, conversions included, at a small fraction of its FP32 and
// INT32 rates, and the refinement kernels that convert between the FP32
// factors and the FP64 vectors would otherwise be bound by them.  Normal
// numbers convert exactly as F2F does (double -> float rounds to nearest
// even); magnitudes below the smallest normal float become signed zero,
// overflow gives infinity, NaN stays NaN.
__device__ __forceinline__ float d2f_bits(double x) {
  const unsigned lo = (unsigned)__double2loint(x), hi = (unsigned)__double2hiint(x);
  const unsigned sign = hi & 0x80000000u;
  const unsigned ahi = hi & 0x7fffffffu;
  const unsigned e = ahi >> 20;  // biased double exponent
  if (e - 897u < 254u) {         // a normal float: exponent 1..254 after rebiasing
    // The 32 bits of |x| >> 29 hold exponent and 23 mantissa bits; the
    // exponent's lost top bits cancel in the 32-bit rebias (896 << 23).
    const unsigned q = __funnelshift_l(lo, ahi, 3) - 0xC0000000u;
    // Round to nearest even on the 29 bits shifted out; a carry moves into
    // the exponent (and to infinity past the largest float), as IEEE requires.
    const unsigned up = ((lo & 0x1fffffffu) + (q & 1u) + 0x0fffffffu) >> 29;
    return __uint_as_float(sign | (q + up));
  }
  if (e == 0x7ffu) return __uint_as_float(sign | 0x7f800000u | (((ahi & 0xfffffu) | lo) ? 0x400000u : 0u));
  return __uint_as_float(e < 897u ? sign : (sign | 0x7f800000u));
}

__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned int e = (b >> 23) & 0xff;
  const unsigned long long m = (unsigned long long)(b & 0x7fffffu) << 29;
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 0xff) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | m));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) | m));
}

template <typename TO, typename TI>
__device__ __forceinline__ TO convert(TI x) { return (TO)x; }
template <>
__device__ __forceinline__ float convert<float, double>(double x) { return d2f_bits(x); }
template <>
__device__ __forceinline__ double convert<double, float>(float x) { return f2d_bits(x); }

// ----------------------------------------------------------------------------
// Row x scenario iteration without integer division: with one scenario a
// thread owns a row; with a batch a warp owns a row and its lanes stride over
// the scenarios (coalesced, ld is a multiple of 32).
template <typename F>
__device__ __forceinline__ void for_rows(int nrows, int ld, F&& f) {
  if (ld == 1) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
      f(r, 0);
  } else {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrows; r += warps)
      for (int s = lane; s < ld; s += 32) f(r, s);
  }
}

inline int rows_grid(int64_t nrows, int ld, int block) {
  const int64_t threads = ld == 1 ? nrows : nrows * 32;
  const int64_t b = (threads + block - 1) / block;
  return (int)(b < 1 ? 1 : (b > 65536 ? 65536 : b));
}

// Values of A's entries for one batch, in the caller's CSR order: either an
// explicit [nnz_a x ld] array, or a structured Jacobian whose entry e is
//   base[e] + sum over c in [ptr[e], ptr[e+1]) of sign[c] * (g[elem[c]] (+ gmin)),
// the companion stamps of the nonlinear elements on entry e over the linear
// part, added element by element in the order of
// 002b_sistema_electrico_base_matriz.cpp:183-202 (conductance G, then the
// convergence conductance gmin when it is positive).
struct AValues {
  const double* a;      // explicit values, or NULL for stamps
  const double* base;   // [nnz_a]
  const int* ptr;       // [nnz_a + 1]
  const int* elem;
  const int* sign;      // +1 / -1
  const double* g;      // [n_elems x ld] element conductances
  const double* gmin;   // [ld] per-scenario convergence conductance, or NULL
  const int* linear;    // [n_elems] elements that take no gmin (wires), or NULL
  __device__ __forceinline__ double operator()(int e, int ld, int s) const {
    if (a) return a[(int64_t)e * ld + s];
    double val = base[e];
    const double gm = gmin ? gmin[s] : 0.0;
    for (int c = ptr[e]; c < ptr[e + 1]; c++) {
      const double sg = (double)sign[c];
      val += sg * g[(int64_t)elem[c] * ld + s];
      if (gm > 0.0 && !(linear && linear[elem[c]])) val += sg * gm;
    }
    return val;
  }
};

// (a) scatter: LU(q, s) = A(slot_src[q], s), zero at fill slots.  `ndone`
// (or NULL): the launch does nothing once every scenario has converged.
template <typename T>
__global__ void k_scatter(const int* __restrict__ slot_src, int nnz, int ld, int S, AValues A,
                          T* __restrict__ v, const int* __restrict__ ndone) {
  if (ndone && __ldcg(ndone) >= S) return;
  for_rows(nnz, ld, [&](int q, int s) {
    const int src = slot_src[q];
    T val = T(0);
    if (src >= 0 && s < S) val = convert<T>(A(src, ld, s));
    v[(int64_t)q * ld + s] = val;
  });
}

// Batched row copy with conversion (ld a multiple of 64): destination row q
// takes source row map[q] (zeros for map[q] < 0, and in the padding columns
// s >= S).  One warp per row, each lane two adjacent columns per vector
// access, two column pairs in flight.  Serves the explicit-value scatter
// (map = slot_src) and the gather permutations (map = row_orig / col_orig).
template <typename TI, typename TO>
__global__ void __launch_bounds__(256)
k_rows_vec(const int* __restrict__ map, int rows, int ld, int S, const TI* __restrict__ src,
           TO* __restrict__ dst, const int* __restrict__ ndone) {
  using VI = typename std::conditional<sizeof(TI) == 8, double2, float2>::type;
  using VO = typename std::conditional<sizeof(TO) == 8, double2, float2>::type;
  if (ndone && __ldcg(ndone) >= S) return;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < rows; q += warps) {
    const int m = map[q];
    TO* drow = dst + (int64_t)q * ld;
    const TI* srow = src + (int64_t)(m < 0 ? 0 : m) * ld;
    for (int s = 2 * lane; s < ld; s += 128) {
      const bool has2 = s + 64 < ld;
      VI a = {}, b = {};
      if (m >= 0) {
        a = *reinterpret_cast<const VI*>(srow + s);
        if (has2) b = *reinterpret_cast<const VI*>(srow + s + 64);
      }
      VO oa, ob;
      oa.x = s < S ? convert<TO>(a.x) : TO(0);
      oa.y = s + 1 < S ? convert<TO>(a.y) : TO(0);
      *reinterpret_cast<VO*>(drow + s) = oa;
      if (has2) {
        ob.x = s + 64 < S ? convert<TO>(b.x) : TO(0);
        ob.y = s + 65 < S ? convert<TO>(b.y) : TO(0);
        *reinterpret_cast<VO*>(drow + s + 64) = ob;
      }
    }
  }
}

// A's entry values (caller order) from any AValues source.
static __global__ void k_assemble(int nnz_a, int ld, int S, AValues A, double* __restrict__ a) {
  for_rows(nnz_a, ld, [&](int e, int s) { a[(int64_t)e * ld + s] = s < S ? A(e, ld, s) : 0.0; });
}

// ----------------------------------------------------------------------------
// (b) left-looking GLU column k for scenario s.
//   for every U slot p of column k (rows j < k, ascending):
//     u = U(j,k); for every L slot q of column j: M(i,k) -= L(i,j) * u
//   then L(:,k) /= U(k,k).
// Same arithmetic as factorize_one_column_GLU_CSC_CPU
// (GLU_CSC_CPU_levels_strings.cpp:3-63), applied in gather order.
template <typename T>
__device__ __forceinline__ void refactor_column(const DevStruct& d, int k, int s, int ld,
                                                T* __restrict__ v, T pivot_tol,
                                                DevStatus* st) {
  const int c0 = d.colptr[k], dk = d.diag[k], c1 = d.colptr[k + 1];
  for (int p = c0; p < dk; p++) {
    const int j = d.csc_row[p];
    const T u = ldv(v + (int64_t)p * ld + s);
    const int q0 = d.diag[j] + 1, q1 = d.colptr[j + 1];
    const int* tg = d.upd_tgt + d.upd_ptr[p] - q0;
    for (int q = q0; q < q1; q++) {
      T* tp = v + (int64_t)tg[q] * ld + s;
      *tp = fnms(ldv(tp), ldv(v + (int64_t)q * ld + s), u);
    }
  }
  const T piv = ldv(v + (int64_t)dk * ld + s);
  if (!(fabs(piv) >= pivot_tol)) report_error(st, 3, k, s);
  for (int q = dk + 1; q < c1; q++) {
    T* tp = v + (int64_t)q * ld + s;
    *tp = ldv(tp) / piv;
  }
}

// One LU level: threads = chains_in_level * ld, scenario fastest.
template <typename T>
__global__ void k_refactor_level(DevStruct d, T* __restrict__ v, int ld, int S,
                                 int chain_begin, int chain_end, T pivot_tol,
                                 DevStatus* st, const int* __restrict__ ndone) {
  if (ndone && __ldcg(ndone) >= S) return;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = chain_begin + (int)(tid / ld);
  const int s = (int)(tid % ld);
  if (c >= chain_end || s >= S) return;
  for (int t = d.lu_sc[c]; t < d.lu_sc[c + 1]; t++)
    refactor_column<T>(d, d.lu_cols[t], s, ld, v, pivot_tol, st);
}

// ----------------------------------------------------------------------------
// (c) triangular solves, gather form (no atomics).
// kind 0: L y = b, rows by L levels       (Process_Column_L_CSC, GLU_CSC_CPU_Triangular.cpp:3-12)
// kind 1: U x = y, rows by U levels       (Process_Column_U_CSC, :14-25)
// kind 2: U^T z = b, columns by LU levels (adjoint, first half)
// kind 3: L^T w = z, columns by LT levels (adjoint, second half)
template <typename T, int KIND>
__device__ __forceinline__ void solve_unknown(const DevStruct& d, int i, int s, int ld,
                                              const T* __restrict__ v, T* __restrict__ x) {
  T acc = ldv(x + (int64_t)i * ld + s);
  if (KIND == 0) {  // updates arrive in ascending column order, as in the reference
    for (int e = d.lrow_ptr[i]; e < d.lrow_ptr[i + 1]; e++)
      acc = fnms(acc, ldv(v + (int64_t)d.lrow_slot[e] * ld + s),
                 ldv(x + (int64_t)d.lrow_col[e] * ld + s));
  } else if (KIND == 1) {  // descending: the reference's backward sweep order
    for (int e = d.urow_ptr[i + 1] - 1; e >= d.urow_ptr[i]; e--)
      acc = fnms(acc, ldv(v + (int64_t)d.urow_slot[e] * ld + s),
                 ldv(x + (int64_t)d.urow_col[e] * ld + s));
    acc /= ldv(v + (int64_t)d.diag[i] * ld + s);
  } else if (KIND == 2) {
    const int dg = d.diag[i];
    for (int p = d.colptr[i]; p < dg; p++)
      acc = fnms(acc, ldv(v + (int64_t)p * ld + s), ldv(x + (int64_t)d.csc_row[p] * ld + s));
    acc /= ldv(v + (int64_t)dg * ld + s);
  } else {
    for (int q = d.diag[i] + 1; q < d.colptr[i + 1]; q++)
      acc = fnms(acc, ldv(v + (int64_t)q * ld + s), ldv(x + (int64_t)d.csc_row[q] * ld + s));
  }
  x[(int64_t)i * ld + s] = acc;
}

template <typename T, int KIND>
__global__ void k_solve_level(DevStruct d, const T* __restrict__ v, T* __restrict__ x,
                              int ld, int S, int chain_begin, int chain_end,
                              const int* __restrict__ done) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = chain_begin + (int)(tid / ld);
  const int s = (int)(tid % ld);
  if (c >= chain_end || s >= S || (done && done[s])) return;
  const int* sc = KIND == 0 ? d.l_sc : KIND == 1 ? d.u_sc : KIND == 2 ? d.lu_sc : d.lt_sc;
  const int* cols = KIND == 0 ? d.l_cols : KIND == 1 ? d.u_cols : KIND == 2 ? d.lu_cols : d.lt_cols;
  for (int t = sc[c]; t < sc[c + 1]; t++) solve_unknown<T, KIND>(d, cols[t], s, ld, v, x);
}

// ----------------------------------------------------------------------------
// Permutations between the caller's order and the pivot order.
// gather:  y[r] = x[perm[r]]        scatter: y[perm[r]] = x[r]
template <typename TI, typename TO>
__global__ void k_permute(const int* __restrict__ perm, int n, int ld, int S,
                          const TI* __restrict__ x, TO* __restrict__ y, int gather) {
  for_rows(n, ld, [&](int r, int s) {
    if (s >= S) return;
    const int64_t e = (int64_t)r * ld + s;
    const int pr = perm[r];
    if (gather) y[e] = convert<TO>(x[(int64_t)pr * ld + s]);
    else y[(int64_t)pr * ld + s] = convert<TO>(x[e]);
  });
}

// ----------------------------------------------------------------------------
// Iterative refinement pieces (FP64 residual, FP32 correction).
// r = b - A x (or b - A^T x) in the caller's order; skipped for converged
// scenarios.  Rows of the product come from a CSR (ptr, idx) whose entry p
// has A-value index ent[p] (NULL: p itself, A's own rows).  Row i of the
// product is row pos[i] of the pivot-ordered system (row_pos for A,
// col_pos for A^T).
static __global__ void k_residual(const int* __restrict__ ptr, const int* __restrict__ idx,
                           const int* __restrict__ ent, int n, int ld, int S, AValues A,
                           const double* __restrict__ b, const double* __restrict__ x,
                           const int* __restrict__ done, const int* __restrict__ ndone,
                           float* __restrict__ r_perm, const int* __restrict__ pos) {
  if (__ldcg(ndone) >= S) return;
  for_rows(n, ld, [&](int i, int s) {
    if (s >= S || done[s]) return;
    double acc = b[(int64_t)i * ld + s];
    for (int p = ptr[i]; p < ptr[i + 1]; p++)
      acc -= A(ent ? ent[p] : p, ld, s) * x[(int64_t)idx[p] * ld + s];
    r_perm[(int64_t)pos[i] * ld + s] = d2f_bits(acc);
  });
}

// Batched residual with explicit values (ld a multiple of 64).  A warp item
// is one row and one chunk of 64 scenarios (two adjacent scenarios per lane
// and 16-byte load); the loads of up to three entries are issued together,
// so a row of the plant (three entries, mostly) costs one round of memory
// latency after its pattern.  A and b are read once (streaming loads); x rows
// are shared by neighbouring rows and stay cached.  Same arithmetic per
// scenario as k_residual (one FP64 FMA per entry, in the row's entry order).
static __global__ void __launch_bounds__(256, 6)
k_residual_rows(const int* __restrict__ ptr, const int* __restrict__ idx,
                const int* __restrict__ ent, int n, int ld, int S,
                const double* __restrict__ a, const double* __restrict__ b,
                const double* __restrict__ x, const int* __restrict__ done,
                const int* __restrict__ ndone, float* __restrict__ r_perm,
                const int* __restrict__ pos) {
  constexpr int kU = 3;  // entries in flight per warp
  if (__ldcg(ndone) >= S) return;
  const int lane = threadIdx.x & 31;
  const int chunks = ld >> 6;
  const int items = n * chunks;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < items; it += warps) {
    const int i = it / chunks;
    const int s = (it - i * chunks) * 64 + 2 * lane;
    const int p0 = __ldg(ptr + i), p1 = __ldg(ptr + i + 1);
    const double2 bb = __ldcs(reinterpret_cast<const double2*>(b + (int64_t)i * ld + s));
    double rx = bb.x, ry = bb.y;
    for (int p = p0; p < p1; p += kU) {
      double2 av[kU], xv[kU];
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (p + u < p1) {
          const int e = ent ? __ldg(ent + p + u) : p + u;
          const int j = __ldg(idx + p + u);
          av[u] = __ldcs(reinterpret_cast<const double2*>(a + (int64_t)e * ld + s));
          xv[u] = *reinterpret_cast<const double2*>(x + (int64_t)j * ld + s);
        }
#pragma unroll
      for (int u = 0; u < kU; u++)
        if (p + u < p1) {
          rx -= av[u].x * xv[u].x;
          ry -= av[u].y * xv[u].y;
        }
    }
    const int64_t ro = (int64_t)__ldg(pos + i) * ld;
    if (s < S && !done[s]) r_perm[ro + s] = d2f_bits(rx);
    if (s + 1 < S && !done[s + 1]) r_perm[ro + s + 1] = d2f_bits(ry);
  }
}

// x[out_perm[c]] += dx[c] (out_perm = col_orig for A, row_orig for A^T);
// per-scenario max |dx| and max |x| as the bit patterns of non-negative
// doubles, which order like the values, so atomicMax on the bits works.  The
// maxima are taken on integer bits (|dx| exactly, |x| truncated to its upper
// 32 bits, a lower bound within 2^-20): the one FP64 instruction per entry is
// the addition.
// first: x starts at 0, so x = dx without reading x (and padding columns
// s >= S are set to 0).
static __global__ void k_ir_update(const int* __restrict__ out_perm, int n, int ld, int S,
                            const float* __restrict__ dx, double* __restrict__ x,
                            const int* __restrict__ done, const int* __restrict__ ndone,
                            unsigned long long* __restrict__ max_dx,
                            unsigned long long* __restrict__ max_x, int first) {
  if (__ldcg(ndone) >= S) return;
  // block = (32 scenarios) x (8 rows); grid-stride over row tiles.
  const int s = blockIdx.y * 32 + threadIdx.x;
  __shared__ unsigned int sdx[8][33], sx[8][33];
  unsigned int mdx = 0u, mx = 0u;
  if (first && s >= S && s < ld)
    for (int c = blockIdx.x * 8 + threadIdx.y; c < n; c += gridDim.x * 8)
      x[(int64_t)out_perm[c] * ld + s] = 0.0;
  if (s < S && !done[s]) {
#pragma unroll 4
    for (int c = blockIdx.x * 8 + threadIdx.y; c < n; c += gridDim.x * 8) {
      const float df = dx[(int64_t)c * ld + s];
      double* xp = x + (int64_t)out_perm[c] * ld + s;
      const double nx = first ? f2d_bits(df) : *xp + f2d_bits(df);
      *xp = nx;
      mdx = max(mdx, __float_as_uint(df) & 0x7fffffffu);
      mx = max(mx, (unsigned int)((unsigned long long)__double_as_longlong(nx) >> 32) &
                       0x7fffffffu);
    }
  }
  sdx[threadIdx.y][threadIdx.x] = mdx;
  sx[threadIdx.y][threadIdx.x] = mx;
  __syncthreads();
  if (threadIdx.y == 0 && s < S) {
    for (int k = 1; k < 8; k++) {
      mdx = max(mdx, sdx[k][threadIdx.x]);
      mx = max(mx, sx[k][threadIdx.x]);
    }
    if (mdx) atomicMax(max_dx + s, (unsigned long long)__double_as_longlong(
                                       f2d_bits(__uint_as_float(mdx))));
    if (mx) atomicMax(max_x + s, (unsigned long long)mx << 32);
  }
}

// Refinement start for a subset: done[s] = src[s] (s < S), ndone counts them,
// x = 0 for the scenarios that will refine.  *ndone must be 0 on entry.
static __global__ void k_ir_init(int n, int ld, int S, const int* __restrict__ src,
                          int* __restrict__ done, int* __restrict__ ndone,
                          double* __restrict__ x) {
  for_rows(n, ld, [&](int i, int s) {
    const int d = s < S ? src[s] : 1;
    if (i == 0) {
      done[s] = d;
      if (d && s < S) atomicAdd(ndone, 1);
    }
    if (!d) x[(int64_t)i * ld + s] = 0.0;
  });
}

// Convergence bookkeeping after sweep `sweep` (1-based).  A scenario stops
// when its correction is small, max|dx_k| <= tol max|x|, or when the error
// left after it is: with rho = max|dx_k| / max|dx_k-1| <= 1/2 the corrections
// shrink geometrically and the remaining error is about
// max|dx_k| rho / (1 - rho) (the stopping estimate of iterative-refinement
// analyses), so the sweep that would only confirm it is skipped.
__device__ __forceinline__ bool ir_check_one(int s, int sweep, int last_sweep, double tol,
                                             int* done, int* sweeps_out,
                                             unsigned long long* max_dx,
                                             unsigned long long* max_x, double* prev_dx) {
  const double mdx = __longlong_as_double((long long)max_dx[s]);
  const double mx = __longlong_as_double((long long)max_x[s]);
  max_dx[s] = 0ull;
  max_x[s] = 0ull;
  bool ok = mdx <= tol * mx;
  if (!ok && sweep > 1) {
    const double prev = prev_dx[s];
    if (prev > 0.0 && mdx <= 0.5 * prev) {
      const double rho = mdx / prev;
      ok = mdx * rho <= tol * mx * (1.0 - rho);
    }
  }
  prev_dx[s] = mdx;
  if (ok) {
    done[s] = 1;
    if (sweeps_out) sweeps_out[s] = sweep;
  } else if (sweep == last_sweep) {
    if (sweeps_out) sweeps_out[s] = -1;
  }
  return ok;
}

static __global__ void k_ir_check(int S, int sweep, int last_sweep, double tol, int* done,
                                  int* ndone, int* sweeps_out, unsigned long long* max_dx,
                                  unsigned long long* max_x, double* prev_dx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S || done[s]) return;
  if (ir_check_one(s, sweep, last_sweep, tol, done, sweeps_out, max_dx, max_x, prev_dx))
    atomicAdd(ndone, 1);
}

// The same check in one block for the refinement replayed from a graph: the
// sweep number lives on the device (*sweeps_done, sweeps finished before this
// one), and the block sets the graph's loop condition: another sweep while a
// scenario is still refining and sweeps remain.
static __global__ void k_ir_check_loop(int S, int last_sweep, double tol, int* done, int* ndone,
                                       int* sweeps_out, unsigned long long* max_dx,
                                       unsigned long long* max_x, double* prev_dx,
                                       int* sweeps_done, cudaGraphConditionalHandle loop) {
  __shared__ int newly;
  const int sweep = *sweeps_done + 1;
  if (threadIdx.x == 0) newly = 0;
  __syncthreads();
  int mine = 0;
  for (int s = threadIdx.x; s < S; s += blockDim.x)
    if (!done[s] && ir_check_one(s, sweep, last_sweep, tol, done, sweeps_out, max_dx, max_x,
                                 prev_dx))
      mine++;
  if (mine) atomicAdd(&newly, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int total = atomicAdd(ndone, newly) + newly;
    *sweeps_done = sweep;
    cudaGraphSetConditional(loop, (total < S && sweep < last_sweep) ? 1u : 0u);
  }
}

}  // namespace pvglu
