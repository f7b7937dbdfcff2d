// Device Newton driver and adjoint (include/pvglu_newton.h) over the hot path
// of capi.cu.  Every Newton iteration is a fixed sequence of launches with no
// host decision inside, so it is captured once as a CUDA graph and replayed;
// per-scenario progress (gmin stage, iteration count, outcome) lives on the
// device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pvglu_newton.h"
#include "handle.hpp"
#include "panel_model.h"

namespace pvglu {
namespace {

constexpr int kMaxStages = 16;

struct NewtonParams {
  double gmin[kMaxStages];
  double tol;
  int n_stages;
  int max_iterations;
};

// Device view of the driver's state.
struct NtDev {
  int n, n_elems, ld, S;
  const int* hi;          // [n_elems]
  const int* lo;
  const int2* xidx;       // [n_elems] rows of hi and lo in the linear solution (-1: ground)
  const int* inc_ptr;     // [n+1] elements incident to each unknown
  const int* inc_elem;
  const int* inc_sign;    // +1: + terminal, -1: - terminal
  const double* b_lin;    // [n]
  pvglu_panel_const panel;  // constants of the element law
  const int* broken;        // [n_elems] 1: replaced by a wire (or NULL: none)
  double g_wire;            // conductance of that wire
  double* iph;            // [n_elems x ld] photocurrent
  double* v;              // voltage iterate
  double* g;              // companion conductance G
  double* ieq;            // companion current Ieq (dI/dIph in the adjoint)
  double* gmin_s;         // [ld] gmin of each scenario's current stage (0: none)
  int* stage;             // [ld]
  int* iters;             // [ld]
  int* outcome;           // [ld] PVGLU_NEWTON_*
  int* damp_fail;         // [ld]
  int* done;              // [ld + 1]: flags, then the stopped count
  int* just_done;         // [ld] stopped in the current iteration
  double* diff;           // [ld]
  double* partial;        // [n_chunks x ld] per-chunk sums of |dv|
  const NewtonParams* prm;
};

constexpr int kUpdRows = 8;            // update block: 32 scenarios x 8 element rows
constexpr int kUpdChunk = 64;          // elements per partial sum (>= 4 blocks per SM at 35k)
constexpr int kUpdPer = kUpdChunk / kUpdRows;  // elements per thread (batched)

__device__ __forceinline__ bool all_stopped(const NtDev& D) {
  return __ldcg(D.done + D.ld) >= D.S;
}

// Companion model of every element (002b_sistema_electrico_base_matriz.cpp:
// 183-197): f(V) = -I(V) is the current from the + to the - terminal,
// G = f'(V), Ieq = f(V) - G*V.  Row 0 also publishes the scenario's gmin.
__global__ void k_nt_companion(NtDev D) {
  if (all_stopped(D)) return;
  for_rows(D.n_elems, D.ld, [&](int k, int s) {
    if (s >= D.S || D.done[s]) return;
    if (k == 0) {
      const double gm = D.prm->gmin[D.stage[s]];
      D.gmin_s[s] = gm > 0.0 ? gm : 0.0;
    }
    const int64_t e = (int64_t)k * D.ld + s;
    if (D.broken && D.broken[k]) {  // linear wire: exact companion, no source
      D.g[e] = D.g_wire;
      D.ieq[e] = 0.0;
      return;
    }
    const double v = D.v[e];
    double cur, didv, didiph;
    pvglu_panel_eval(&D.panel, D.iph[e], v, &cur, &didv, &didiph);
    const double G = -didv;
    D.g[e] = G;
    D.ieq[e] = __dsub_rn(-cur, __dmul_rn(G, v));
  });
}

// b = b_lin, then per incident element in element order the current-source
// stamp of -Ieq (002b:100-110, :196): + terminal b -= Ieq, - terminal b += Ieq.
// Written at pos[i] (pivot order) or i (pos NULL).
__global__ void k_nt_rhs(NtDev D, double* __restrict__ out, const int* __restrict__ pos) {
  if (all_stopped(D)) return;
  for_rows(D.n, D.ld, [&](int i, int s) {
    if (s >= D.S || D.done[s]) return;
    double acc = D.b_lin[i];
    for (int c = D.inc_ptr[i]; c < D.inc_ptr[i + 1]; c++) {
      const double q = D.ieq[(int64_t)D.inc_elem[c] * D.ld + s];
      acc = D.inc_sign[c] > 0 ? __dsub_rn(acc, q) : __dadd_rn(acc, q);
    }
    out[(int64_t)(pos ? pos[i] : i) * D.ld + s] = acc;
  });
}

// Damped update of one element (011_calculate_new_iteration.cpp:37-90): the
// step factor m starts at 1 and halves while the candidate moves the voltage
// by more than 1 V or is NaN; below 1e-13 the element keeps its voltage and
// the scenario is flagged.
__device__ __forceinline__ bool finite_bits(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) !=
         0x7ff0000000000000ull;
}

// *change = |new - old| (|x - y| = |y - x| exactly in IEEE arithmetic).
__device__ __forceinline__ double damped_step(double old, double nv, bool* bad,
                                              double* change) {
  // m = 1: old * 0 + nv * 1 is nv itself for finite old and nonzero nv
  // (the zero case keeps the general form for the sign of zero).
  if (nv != 0.0 && finite_bits(old) && finite_bits(nv)) {
    const double d = fabs(__dsub_rn(old, nv));
    if (!(d > 1.0)) {
      *change = d;
      return nv;
    }
  }
  // Every step factor m = 2^-j with m |nv - old| >= 4 fails the 1 V test
  // whatever the rounding, so the halving starts at 2^-(e-1), e the binary
  // exponent of |nv - old|; the first factor that passes is the one the
  // full halving from m = 1 would reach.  Non-finite values take the full
  // loop.
  double m = 1.0;
  if (finite_bits(old) && finite_bits(nv)) {
    const long long db = __double_as_longlong(__dsub_rn(old, nv)) & 0x7fffffffffffffffLL;
    const int e = (int)(db >> 52) - 1023;
    if (e > 1) m = __longlong_as_double((long long)(1023 - (e - 1)) << 52);
  }
  for (;;) {
    const double t = __dadd_rn(__dmul_rn(old, __dsub_rn(1.0, m)), __dmul_rn(nv, m));
    if (m < 1e-13) {
      *bad = true;
      *change = 0.0;
      return old;
    }
    if (!isnan(old) && !isnan(t) && !(fabs(__dsub_rn(old, t)) > 1.0)) {
      *change = fabs(__dsub_rn(t, old));
      return t;
    }
    m *= 0.5;
  }
}

// New voltage drops from the solution X (rows D.xidx: pivot order for FP64
// factors, caller order after refinement), damped update, per-chunk sums of
// |change| in a fixed order (deterministic).  Block: 32 scenarios x 8
// element rows; grid: (chunks, ld / 32); a thread's elements have their
// solution rows and voltages loaded together before the updates.  With one
// scenario the 256 threads split the elements.
__global__ void __launch_bounds__(256) k_nt_update(NtDev D, const double* __restrict__ X) {
  if (all_stopped(D)) return;
  __shared__ double red[kUpdRows][33];
  const bool single = D.ld == 1;
  const int s = single ? 0 : blockIdx.y * 32 + threadIdx.x;
  const int kb = blockIdx.x * kUpdChunk;
  const int ke = min(D.n_elems, kb + kUpdChunk);
  double sum = 0.0;
  bool bad = false;
  if (s < D.S && !D.done[s]) {
    const int k0 = single ? kb + threadIdx.y * 32 + threadIdx.x : kb + threadIdx.y;
    const int dk = single ? 32 * kUpdRows : kUpdRows;
    double* __restrict__ v = D.v;
    const int ld = D.ld;
    double xh[kUpdPer], xl[kUpdPer], old[kUpdPer];
#pragma unroll
    for (int j = 0; j < kUpdPer; j++) {
      const int k = k0 + j * dk;
      if (k < ke) {
        const int2 xi = __ldg(D.xidx + k);
        xh[j] = xi.x >= 0 ? X[(int64_t)xi.x * ld + s] : 0.0;
        xl[j] = xi.y >= 0 ? X[(int64_t)xi.y * ld + s] : 0.0;
        old[j] = v[(int64_t)k * ld + s];
      }
    }
#pragma unroll
    for (int j = 0; j < kUpdPer; j++) {
      const int k = k0 + j * dk;
      if (k >= ke) continue;
      const int64_t e = (int64_t)k * ld + s;
      if (D.broken && D.broken[k]) {  // a wire is a linear element: no damping, no diff
        v[e] = __dsub_rn(xh[j], xl[j]);
        continue;
      }
      double change;
      v[e] = damped_step(old[j], __dsub_rn(xh[j], xl[j]), &bad, &change);
      sum = __dadd_rn(sum, change);
    }
  }
  if (bad) D.damp_fail[s] = 1;
  if (single) {
    // 256 partial sums of one scenario, added in thread order.
    __shared__ double all[32 * kUpdRows];
    all[threadIdx.y * 32 + threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && !D.done[0]) {
      double t = 0.0;
      for (int i = 0; i < 32 * kUpdRows; i++) t += all[i];
      D.partial[blockIdx.x] = t;
    }
    return;
  }
  red[threadIdx.y][threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.y == 0 && s < D.S && !D.done[s]) {
    double t = 0.0;
    for (int r = 0; r < kUpdRows; r++) t += red[r][threadIdx.x];
    D.partial[(int64_t)blockIdx.x * D.ld + s] = t;
  }
}

// End of an iteration for every running scenario: diff, stage advance
// (000_PVPP_simulator.cpp:172-176: a stage ends once diff < tol), outcome.
// One warp per scenario: lane l adds the chunk sums l, l + 32, ... in order,
// then the 32 lane sums are added in a fixed tree order (deterministic).
__global__ void k_nt_check(NtDev D, int n_chunks) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= D.S) return;
  if (D.done[s]) {
    if (lane == 0) D.just_done[s] = 0;
    return;
  }
  double part = 0.0;
  for (int c = lane; c < n_chunks; c += 32) part += D.partial[(int64_t)c * D.ld + s];
  for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xffffffffu, part, off);
  if (lane != 0) return;
  const double diff = part;
  D.diff[s] = diff;
  const int it = ++D.iters[s];
  int out = PVGLU_NEWTON_RUNNING;
  if (D.damp_fail[s]) {
    out = PVGLU_NEWTON_DAMPING;
  } else if (diff < D.prm->tol) {
    const int st = ++D.stage[s];
    if (st >= D.prm->n_stages) out = PVGLU_NEWTON_CONVERGED;
  }
  if (out == PVGLU_NEWTON_RUNNING && it >= D.prm->max_iterations)
    out = PVGLU_NEWTON_MAX_ITERATIONS;
  D.outcome[s] = out;
  D.just_done[s] = out != PVGLU_NEWTON_RUNNING;
  if (out != PVGLU_NEWTON_RUNNING) {
    D.done[s] = 1;
    atomicAdd(D.done + D.ld, 1);
  }
}

// FP64 handles solve in place in pivot order, and later iterations of other
// scenarios reuse that vector (a 64-scenario group solves as a whole), so a
// scenario's node solution is saved, in caller order, in the iteration where
// it stops: x[col_orig[c]] = w[c].
__global__ void k_nt_keep(NtDev D, const double* __restrict__ w, const int* __restrict__ col_pos,
                          double* __restrict__ x) {
  for_rows(D.n, D.ld, [&](int i, int s) {
    if (s < D.S && D.just_done[s]) x[(int64_t)i * D.ld + s] = w[(int64_t)col_pos[i] * D.ld + s];
  });
}

__global__ void k_nt_reset(NtDev D) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) D.done[D.ld] = 0;
  if (s >= D.ld) return;
  D.stage[s] = 0;
  D.iters[s] = 0;
  D.outcome[s] = s < D.S ? PVGLU_NEWTON_RUNNING : PVGLU_NEWTON_CONVERGED;
  D.damp_fail[s] = 0;
  D.just_done[s] = 0;
  D.done[s] = s < D.S ? 0 : 1;
  D.diff[s] = 0.0;
  D.gmin_s[s] = 0.0;
}

// Irradiance field of every scenario at time t (pvglu_shadow_irradiance),
// written as photocurrent iph = iph_per_g * G (and G itself if asked).
struct FieldDev {
  const double* x;       // [n_elems] panel positions
  const double* y;
  const double* shadow;  // [ld][max_shadows][6]
  const int* count;      // [ld]
  const double* toff;    // [ld] time offset of each scenario
  int max_shadows;
  double g_clear, iph_per_g;
};

__global__ void k_nt_field(NtDev D, FieldDev F, double t, double* __restrict__ g_out) {
  for_rows(D.n_elems, D.ld, [&](int k, int s) {
    const int64_t e = (int64_t)k * D.ld + s;
    double g = 0.0;
    if (s < D.S)
      g = pvglu_shadow_irradiance(F.x[k], F.y[k], F.shadow + (int64_t)s * F.max_shadows * 6,
                                  F.count[s], t + F.toff[s], F.g_clear);
    D.iph[e] = F.iph_per_g * g;
    if (g_out) g_out[e] = g;
  });
}

// Kirchhoff mismatch at the node solution x (caller order): element currents
// f = -I(V) with V = x[hi] - x[lo] (kept in `cur`), then per unknown
// F = A_lin x + incidence * f - b_lin and max_i |F_i| per scenario (bits of
// a non-negative double, atomicMax).
__global__ void k_nt_elem_current(NtDev D, const double* __restrict__ x,
                                  double* __restrict__ cur) {
  for_rows(D.n_elems, D.ld, [&](int k, int s) {
    if (s >= D.S) return;
    const int64_t e = (int64_t)k * D.ld + s;
    const int h = D.hi[k], l = D.lo[k];
    const double v = (h >= 0 ? x[(int64_t)h * D.ld + s] : 0.0) -
                     (l >= 0 ? x[(int64_t)l * D.ld + s] : 0.0);
    if (D.broken && D.broken[k]) {
      cur[e] = D.g_wire * v;
      return;
    }
    double c, didv, didiph;
    pvglu_panel_eval(&D.panel, D.iph[e], v, &c, &didv, &didiph);
    cur[e] = -c;
  });
}

__global__ void k_nt_mismatch(NtDev D, const int* __restrict__ a_rowptr,
                              const int* __restrict__ a_colidx, const double* __restrict__ a_lin,
                              const double* __restrict__ x, const double* __restrict__ cur,
                              unsigned long long* __restrict__ out) {
  for_rows(D.n, D.ld, [&](int i, int s) {
    if (s >= D.S) return;
    double f = -D.b_lin[i];
    for (int p = a_rowptr[i]; p < a_rowptr[i + 1]; p++)
      f += a_lin[p] * x[(int64_t)a_colidx[p] * D.ld + s];
    for (int c = D.inc_ptr[i]; c < D.inc_ptr[i + 1]; c++) {
      const double q = cur[(int64_t)D.inc_elem[c] * D.ld + s];
      f = D.inc_sign[c] > 0 ? f + q : f - q;
    }
    atomicMax(out + s, (unsigned long long)__double_as_longlong(fabs(f)));
  });
}

// Adjoint: companion conductance at the iterate without gmin, and
// dI/dIph (kept in ieq) for the sensitivity.
__global__ void k_nt_adjoint_companion(NtDev D) {
  for_rows(D.n_elems, D.ld, [&](int k, int s) {
    if (s >= D.S) return;
    const int64_t e = (int64_t)k * D.ld + s;
    if (D.broken && D.broken[k]) {
      D.g[e] = D.g_wire;
      D.ieq[e] = 0.0;  // a wire does not depend on the irradiance
      return;
    }
    double cur, didv, didiph;
    pvglu_panel_eval(&D.panel, D.iph[e], D.v[e], &cur, &didv, &didiph);
    D.g[e] = -didv;
    D.ieq[e] = didiph;
  });
}

// dP/dIph[k] = dI/dIph * (lambda[hi] - lambda[lo]); lambda in pivot order
// through lpos, or caller order when lpos is NULL.
__global__ void k_nt_adjoint_reduce(NtDev D, const double* __restrict__ lam,
                                    const int* __restrict__ lpos, double* __restrict__ out) {
  for_rows(D.n_elems, D.ld, [&](int k, int s) {
    const int64_t e = (int64_t)k * D.ld + s;
    if (s >= D.S) {
      out[e] = 0.0;
      return;
    }
    const int h = D.hi[k], l = D.lo[k];
    const double lh = h >= 0 ? lam[(int64_t)(lpos ? lpos[h] : h) * D.ld + s] : 0.0;
    const double ll = l >= 0 ? lam[(int64_t)(lpos ? lpos[l] : l) * D.ld + s] : 0.0;
    out[e] = D.ieq[e] * (lh - ll);
  });
}

}  // namespace
}  // namespace pvglu

struct pvglu_newton {
  pvglu_numeric* num = nullptr;
  int n_elems = 0, n_chunks = 1;
  std::vector<void*> allocs;
  pvglu::NtDev D{};
  pvglu::NewtonParams* prm_dev = nullptr;
  pvglu::NewtonParams prm_host{};
  double* w64 = nullptr;        // FP64 handles: right-hand side / solution, pivot order
  double* rhs64 = nullptr;      // FP32 handles: right-hand side, caller order
  double* x64 = nullptr;        // node solution, caller order (FP32: refined in place;
                                // FP64: saved when a scenario stops)
  double* lam = nullptr;        // adjoint vector
  int* pinned_ndone = nullptr;  // host-pinned copy of the stopped count
  double ir_tol = 1e-12;
  pvglu::FieldDev field{};
  bool has_field = false;
  int* broken_dev = nullptr;
  std::vector<void*> field_allocs;
  int ir_sweeps = 8;
  // Captured iteration body and what it was captured with.
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_schedule = -1, graph_sweeps = -1;
  double graph_tol = -1.0;
  bool graph_failed = false;
  int last_bodies = 0, last_graph = 0;
  ~pvglu_newton() {
    for (void* p : field_allocs) cudaFree(p);
    if (broken_dev) cudaFree(broken_dev);
    if (graph) cudaGraphExecDestroy(graph);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (pinned_ndone) cudaFreeHost(pinned_ndone);
    for (void* p : allocs) cudaFree(p);
  }
  template <typename T>
  int alloc(size_t count, T** out) {
    PVGLU_CUDA(cudaMalloc((void**)out, std::max<size_t>(count, 1) * sizeof(T)));
    allocs.push_back(*out);
    return PVGLU_OK;
  }
  template <typename T>
  int put(const std::vector<T>& h, T** out) {
    int st = upload(h, out);
    if (st) return st;
    allocs.push_back(*out);
    return PVGLU_OK;
  }
};

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// One Newton iteration for every running scenario (no host synchronization).
int newton_body(pvglu_newton* nw, cudaStream_t st) {
  pvglu_numeric* h = nw->num;
  const pvglu::NtDev& D = nw->D;
  const int* ndone = D.done + D.ld;
  const pvglu::SkipDone skip{D.done, ndone};
  const bool fp64 = h->precision == PVGLU_FP64;
  pvglu::k_nt_companion<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256, 0, st>>>(D);
  pvglu::k_nt_rhs<<<pvglu::rows_grid(D.n, D.ld, 256), 256, 0, st>>>(
      D, fp64 ? nw->w64 : nw->rhs64, fp64 ? h->row_pos : nullptr);
  const pvglu::AValues A = h->stamps(D.g, D.gmin_s, D.broken);
  int rc = pvglu::run_scatter(h, A, ndone, st);
  if (rc) return rc;
  const double* X;
  if (fp64) {  // solution in pivot order (D.xidx)
    rc = pvglu::run_refactor_solve_perm(h, nw->w64, false, skip, st);
    X = nw->w64;
  } else {  // refined solution in caller order
    rc = pvglu::run_refactor(h, st, skip);
    if (!rc)
      rc = pvglu::run_refine(h, A, nw->rhs64, nw->x64, false, nw->ir_tol, nw->ir_sweeps,
                             nullptr, st, D.done);
    X = nw->x64;
  }
  if (rc) return rc;
  const dim3 ublk(32, pvglu::kUpdRows);
  const dim3 ugrd((unsigned)nw->n_chunks, D.ld == 1 ? 1u : (unsigned)(D.ld / 32));
  pvglu::k_nt_update<<<ugrd, ublk, 0, st>>>(D, X);
  pvglu::k_nt_check<<<(D.S + 3) / 4, 128, 0, st>>>(D, nw->n_chunks);
  if (fp64)
    pvglu::k_nt_keep<<<pvglu::rows_grid(D.n, D.ld, 256), 256, 0, st>>>(D, nw->w64, h->col_pos,
                                                                         nw->x64);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

// Captures newton_body into an executable graph; on any capture failure the
// driver falls back to direct launches for good.
void capture_body(pvglu_newton* nw) {
  if (nw->graph_failed) return;
  pvglu_numeric* h = nw->num;
  if (nw->graph && nw->graph_schedule == h->schedule && nw->graph_sweeps == nw->ir_sweeps &&
      nw->graph_tol == nw->ir_tol)
    return;
  if (nw->graph) {
    cudaGraphExecDestroy(nw->graph);
    nw->graph = nullptr;
  }
  if (!nw->cap_stream &&
      cudaStreamCreateWithFlags(&nw->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    nw->graph_failed = true;
    return;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(nw->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    nw->graph_failed = true;
    return;
  }
  const int rc = newton_body(nw, nw->cap_stream);
  const cudaError_t e = cudaStreamEndCapture(nw->cap_stream, &g);
  cudaGraphExec_t ex = nullptr;
  if (rc || e != cudaSuccess || !g ||
      cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    nw->graph_failed = true;
    return;
  }
  cudaGraphDestroy(g);
  nw->graph = ex;
  nw->graph_schedule = h->schedule;
  nw->graph_sweeps = nw->ir_sweeps;
  nw->graph_tol = nw->ir_tol;
}

// Position of entry (r, c) in A's CSR (sorted rows), -1 if absent.
int find_entry(const pvglu::Symbolic& s, int r, int c) {
  const int* b = s.a_colidx.data() + s.a_rowptr[r];
  const int* e = s.a_colidx.data() + s.a_rowptr[r + 1];
  const int* p = std::lower_bound(b, e, c);
  return (p != e && *p == c) ? (int)(p - s.a_colidx.data()) : -1;
}

}  // namespace

extern "C" {

int pvglu_newton_create(pvglu_numeric* num, const pvglu_circuit* c, pvglu_newton** out) {
  if (!num || !c || !out || c->n_elems < 0 || (c->n_elems > 0 && (!c->elem_hi || !c->elem_lo)) ||
      !c->a_lin || !c->b_lin || !(c->i0 > 0) || !(c->a > 0) || !(c->rs > 0) || !(c->rsh > 0))
    return fail(PVGLU_ERR_BAD_ARG, "bad newton_create arguments");
  *out = nullptr;
  const pvglu::Symbolic& s = num->sym->s;
  const int n = s.n, ne = c->n_elems;
  for (int k = 0; k < ne; k++)
    if (c->elem_hi[k] < -1 || c->elem_hi[k] >= n || c->elem_lo[k] < -1 || c->elem_lo[k] >= n)
      return fail(PVGLU_ERR_BAD_ARG, "element terminal out of range");
  // Stamps: per A entry, the elements touching it in element order
  // (admittance stamp of 002b:5-38 at (hi,hi)+, (hi,lo)-, (lo,hi)-, (lo,lo)+).
  const int nnz_a = (int)s.nnz_a;
  std::vector<std::vector<std::pair<int, int>>> per(nnz_a);
  for (int k = 0; k < ne; k++) {
    const int hi = c->elem_hi[k], lo = c->elem_lo[k];
    const int rr[4] = {hi, hi, lo, lo}, cc[4] = {hi, lo, hi, lo}, sg[4] = {1, -1, -1, 1};
    for (int q = 0; q < 4; q++) {
      if (rr[q] < 0 || cc[q] < 0) continue;
      const int e = find_entry(s, rr[q], cc[q]);
      if (e < 0)
        return fail(PVGLU_ERR_STRUCTURAL, "element " + std::to_string(k) + " stamps (" +
                                              std::to_string(rr[q]) + "," +
                                              std::to_string(cc[q]) + ") outside the pattern");
      per[e].push_back({k, sg[q]});
    }
  }
  std::vector<int> eptr(nnz_a + 1, 0), eelem, esign;
  for (int e = 0; e < nnz_a; e++) {
    for (const auto& ks : per[e]) {
      eelem.push_back(ks.first);
      esign.push_back(ks.second);
    }
    eptr[e + 1] = (int)eelem.size();
  }
  int rc = pvglu_numeric_set_stamps(num, ne, c->a_lin, eptr.data(), eelem.data(), esign.data());
  if (rc) return rc;
  // Incidence: unknown i <- elements with a terminal there, element order.
  std::vector<std::vector<std::pair<int, int>>> inc(n);
  for (int k = 0; k < ne; k++) {
    if (c->elem_hi[k] >= 0) inc[c->elem_hi[k]].push_back({k, 1});
    if (c->elem_lo[k] >= 0) inc[c->elem_lo[k]].push_back({k, -1});
  }
  std::vector<int> iptr(n + 1, 0), ielem, isign;
  for (int i = 0; i < n; i++) {
    for (const auto& ks : inc[i]) {
      ielem.push_back(ks.first);
      isign.push_back(ks.second);
    }
    iptr[i + 1] = (int)ielem.size();
  }
  auto* nw = new pvglu_newton();
  nw->num = num;
  nw->n_elems = ne;
  nw->n_chunks = std::max(1, (ne + pvglu::kUpdChunk - 1) / pvglu::kUpdChunk);
  pvglu::NtDev& D = nw->D;
  D.n = n;
  D.n_elems = ne;
  D.ld = num->ld;
  D.S = num->S;
  const pvglu_panel_params pp{c->i0, c->a, c->rs, c->rsh};
  pvglu_panel_prepare(&pp, &D.panel);
  const size_t ev = (size_t)std::max(ne, 1) * D.ld, nv = (size_t)n * D.ld;
  std::vector<int> hi(c->elem_hi, c->elem_hi + ne), lo(c->elem_lo, c->elem_lo + ne);
  std::vector<double> bl(c->b_lin, c->b_lin + n);
  int* tmp = nullptr;
  double* dtmp = nullptr;
  rc = 0;
  rc |= nw->put(hi, &tmp);
  D.hi = tmp;
  rc |= nw->put(lo, &tmp);
  D.lo = tmp;
  {
    // Solution rows of each element's terminals: FP64 factors leave the
    // solution in pivot order (position col_pos[i] of unknown i), the
    // refinement in caller order.
    const pvglu::Symbolic& sy = num->sym->s;
    std::vector<int> pos(n);
    for (int i = 0; i < n; i++) pos[i] = i;
    if (num->precision == PVGLU_FP64)
      for (int c2 = 0; c2 < n; c2++) pos[sy.col_orig[c2]] = c2;
    std::vector<int2> xi(std::max(ne, 1), make_int2(-1, -1));
    for (int k = 0; k < ne; k++)
      xi[k] = make_int2(hi[k] >= 0 ? pos[hi[k]] : -1, lo[k] >= 0 ? pos[lo[k]] : -1);
    int2* xt = nullptr;
    rc |= nw->put(xi, &xt);
    D.xidx = xt;
  }
  rc |= nw->put(iptr, &tmp);
  D.inc_ptr = tmp;
  rc |= nw->put(ielem, &tmp);
  D.inc_elem = tmp;
  rc |= nw->put(isign, &tmp);
  D.inc_sign = tmp;
  rc |= nw->put(bl, &dtmp);
  D.b_lin = dtmp;
  rc |= nw->alloc(ev, &dtmp);
  D.iph = dtmp;
  rc |= nw->alloc(ev, &D.v);
  rc |= nw->alloc(ev, &D.g);
  rc |= nw->alloc(ev, &D.ieq);
  rc |= nw->alloc(D.ld, &D.gmin_s);
  rc |= nw->alloc(D.ld, &D.stage);
  rc |= nw->alloc(D.ld, &D.iters);
  rc |= nw->alloc(D.ld, &D.outcome);
  rc |= nw->alloc(D.ld, &D.damp_fail);
  rc |= nw->alloc(D.ld + 1, &D.done);
  rc |= nw->alloc(D.ld, &D.just_done);
  rc |= nw->alloc(D.ld, &D.diff);
  rc |= nw->alloc((size_t)nw->n_chunks * D.ld, &D.partial);
  rc |= nw->alloc(1, &nw->prm_dev);
  D.prm = nw->prm_dev;
  rc |= nw->alloc(nv, &nw->lam);
  rc |= nw->alloc(nv, &nw->x64);
  if (num->precision == PVGLU_FP64)
    rc |= nw->alloc(nv, &nw->w64);
  else
    rc |= nw->alloc(nv, &nw->rhs64);
  if (!rc && cudaMallocHost((void**)&nw->pinned_ndone, sizeof(int)) != cudaSuccess)
    rc = fail(PVGLU_ERR_NO_MEMORY, "pinned allocation failed");
  if (rc) {
    const std::string e = pvglu_last_error();
    delete nw;
    return fail(PVGLU_ERR_NO_MEMORY, "device allocation failed: " + e);
  }
  if (cudaMemset(D.iph, 0, ev * sizeof(double)) != cudaSuccess ||
      cudaMemset(D.v, 0, ev * sizeof(double)) != cudaSuccess ||
      cudaMemset(D.g, 0, ev * sizeof(double)) != cudaSuccess ||
      cudaMemset(D.ieq, 0, ev * sizeof(double)) != cudaSuccess ||
      cudaMemset(nw->lam, 0, nv * sizeof(double)) != cudaSuccess ||
      (nw->w64 && cudaMemset(nw->w64, 0, nv * sizeof(double)) != cudaSuccess) ||
      (nw->x64 && cudaMemset(nw->x64, 0, nv * sizeof(double)) != cudaSuccess) ||
      (nw->rhs64 && cudaMemset(nw->rhs64, 0, nv * sizeof(double)) != cudaSuccess)) {
    delete nw;
    return fail(PVGLU_ERR_CUDA, "cudaMemset failed");
  }
  pvglu::k_nt_reset<<<(D.ld + 127) / 128, 128>>>(D);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    delete nw;
    return fail(PVGLU_ERR_CUDA, "Newton state reset failed");
  }
  *out = nw;
  return PVGLU_OK;
}

int pvglu_newton_destroy(pvglu_newton* nw) {
  delete nw;
  return PVGLU_OK;
}

int pvglu_newton_set_iph(pvglu_newton* nw, const double* iph, void* stream) {
  if (!nw || !iph) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  PVGLU_CUDA(cudaMemcpyAsync(nw->D.iph, iph, (size_t)nw->n_elems * nw->D.ld * sizeof(double),
                             cudaMemcpyDeviceToDevice, as_stream(stream)));
  return PVGLU_OK;
}

int pvglu_newton_set_voltages(pvglu_newton* nw, const double* v, void* stream) {
  if (!nw || !v) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  PVGLU_CUDA(cudaMemcpyAsync(nw->D.v, v, (size_t)nw->n_elems * nw->D.ld * sizeof(double),
                             cudaMemcpyDeviceToDevice, as_stream(stream)));
  return PVGLU_OK;
}

int pvglu_newton_set_field(pvglu_newton* nw, const double* elem_x, const double* elem_y,
                           int max_shadows, const int* counts, const double* shadows,
                           const double* t_offset, double g_clear, double iph_per_g) {
  if (!nw || !elem_x || !elem_y || !counts || max_shadows < 0 || max_shadows > 4096 ||
      (max_shadows > 0 && !shadows))
    return fail(PVGLU_ERR_BAD_ARG, "bad set_field arguments");
  const int S = nw->D.S, ld = nw->D.ld, ne = nw->n_elems;
  for (int s = 0; s < S; s++)
    if (counts[s] < 0 || counts[s] > max_shadows)
      return fail(PVGLU_ERR_BAD_ARG, "shadow count out of range");
  std::vector<double> xs(elem_x, elem_x + ne), ys(elem_y, elem_y + ne);
  std::vector<double> sh((size_t)ld * std::max(max_shadows, 1) * 6, 0.0);
  std::copy(shadows, shadows + (size_t)S * max_shadows * 6, sh.begin());
  std::vector<int> cnt(ld, 0);
  std::copy(counts, counts + S, cnt.begin());
  std::vector<double> toff(ld, 0.0);
  if (t_offset) std::copy(t_offset, t_offset + S, toff.begin());
  for (void* p : nw->field_allocs) cudaFree(p);
  nw->field_allocs.clear();
  nw->has_field = false;
  double *dx = nullptr, *dy = nullptr, *ds = nullptr;
  int* dc = nullptr;
  int rc = 0;
  rc |= upload(xs, &dx);
  nw->field_allocs.push_back(dx);
  rc |= upload(ys, &dy);
  nw->field_allocs.push_back(dy);
  rc |= upload(sh, &ds);
  nw->field_allocs.push_back(ds);
  rc |= upload(cnt, &dc);
  nw->field_allocs.push_back(dc);
  double* dt = nullptr;
  rc |= upload(toff, &dt);
  nw->field_allocs.push_back(dt);
  if (rc) return fail(PVGLU_ERR_NO_MEMORY, "field upload failed");
  nw->field = pvglu::FieldDev{dx, dy, ds, dc, dt, max_shadows, g_clear, iph_per_g};
  nw->has_field = true;
  return PVGLU_OK;
}

int pvglu_newton_field_iph(pvglu_newton* nw, double t, double* g_out, void* stream) {
  if (!nw) return fail(PVGLU_ERR_BAD_ARG, "NULL handle");
  if (!nw->has_field) return fail(PVGLU_ERR_BAD_ARG, "no field set on this handle");
  const pvglu::NtDev& D = nw->D;
  pvglu::k_nt_field<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256, 0, as_stream(stream)>>>(
      D, nw->field, t, g_out);
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

int pvglu_newton_set_broken(pvglu_newton* nw, const int* broken, double r_wire) {
  if (!nw || (broken && !(r_wire > 0.0))) return fail(PVGLU_ERR_BAD_ARG, "bad set_broken arguments");
  if (nw->broken_dev) {
    cudaFree(nw->broken_dev);
    nw->broken_dev = nullptr;
  }
  nw->D.broken = nullptr;
  if (!broken) return PVGLU_OK;
  std::vector<int> flags(broken, broken + nw->n_elems);
  for (int& f : flags) f = f ? 1 : 0;
  int* d = nullptr;
  if (upload(flags, &d)) return fail(PVGLU_ERR_NO_MEMORY, "broken flags upload");
  nw->broken_dev = d;
  nw->D.broken = d;
  nw->D.g_wire = 1.0 / r_wire;
  // The captured body holds the old device view: capture it again.
  if (nw->graph) {
    cudaGraphExecDestroy(nw->graph);
    nw->graph = nullptr;
  }
  return PVGLU_OK;
}

int pvglu_newton_set_refinement(pvglu_newton* nw, double tol, int max_sweeps) {
  if (!nw || !(tol > 0.0) || max_sweeps <= 0 || max_sweeps > 64)
    return fail(PVGLU_ERR_BAD_ARG, "bad refinement settings");
  nw->ir_tol = tol;
  nw->ir_sweeps = max_sweeps;
  return PVGLU_OK;
}

int pvglu_newton_run(pvglu_newton* nw, const double* gmin, int n_stages, double tol,
                     int max_iterations, int check_every, void* stream) {
  if (!nw || !gmin || n_stages <= 0 || n_stages > pvglu::kMaxStages || !(tol > 0.0) ||
      max_iterations <= 0 || check_every <= 0)
    return fail(PVGLU_ERR_BAD_ARG, "bad newton_run arguments");
  cudaStream_t st = as_stream(stream);
  pvglu::NewtonParams& P = nw->prm_host;
  P = pvglu::NewtonParams{};
  for (int i = 0; i < n_stages; i++) P.gmin[i] = gmin[i];
  P.tol = tol;
  P.n_stages = n_stages;
  P.max_iterations = max_iterations;
  // The parameters live in the handle, so the copy may complete after return.
  PVGLU_CUDA(cudaMemcpyAsync(nw->prm_dev, &P, sizeof(P), cudaMemcpyHostToDevice, st));
  const pvglu::NtDev& D = nw->D;
  pvglu::k_nt_reset<<<(D.ld + 127) / 128, 128, 0, st>>>(D);
  PVGLU_CUDA(cudaGetLastError());
  PVGLU_CUDA(cudaStreamSynchronize(st));
  capture_body(nw);
  nw->last_bodies = 0;
  nw->last_graph = nw->graph ? 1 : 0;
  while (nw->last_bodies < max_iterations) {
    const int k = std::min(check_every, max_iterations - nw->last_bodies);
    for (int i = 0; i < k; i++) {
      if (nw->graph) {
        PVGLU_CUDA(cudaGraphLaunch(nw->graph, st));
      } else {
        const int rc = newton_body(nw, st);
        if (rc) return rc;
      }
    }
    nw->last_bodies += k;
    PVGLU_CUDA(cudaMemcpyAsync(nw->pinned_ndone, D.done + D.ld, sizeof(int),
                               cudaMemcpyDeviceToHost, st));
    PVGLU_CUDA(cudaStreamSynchronize(st));
    if (*nw->pinned_ndone >= D.S) break;
  }
  return PVGLU_OK;
}

int pvglu_newton_results(pvglu_newton* nw, int* iterations, int* outcome, double* diff) {
  if (!nw) return fail(PVGLU_ERR_BAD_ARG, "NULL handle");
  const int S = nw->D.S;
  PVGLU_CUDA(cudaDeviceSynchronize());
  if (iterations)
    PVGLU_CUDA(cudaMemcpy(iterations, nw->D.iters, S * sizeof(int), cudaMemcpyDeviceToHost));
  if (outcome)
    PVGLU_CUDA(cudaMemcpy(outcome, nw->D.outcome, S * sizeof(int), cudaMemcpyDeviceToHost));
  if (diff) PVGLU_CUDA(cudaMemcpy(diff, nw->D.diff, S * sizeof(double), cudaMemcpyDeviceToHost));
  return PVGLU_OK;
}

const double* pvglu_newton_voltages(const pvglu_newton* nw) { return nw ? nw->D.v : nullptr; }

int pvglu_newton_last_run(const pvglu_newton* nw, int* bodies, int* graph) {
  if (!nw) return fail(PVGLU_ERR_BAD_ARG, "NULL handle");
  if (bodies) *bodies = nw->last_bodies;
  if (graph) *graph = nw->last_graph;
  return PVGLU_OK;
}

int pvglu_newton_solution(pvglu_newton* nw, double* x, void* stream) {
  if (!nw || !x) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  pvglu_numeric* h = nw->num;
  const size_t nv = (size_t)h->n * h->ld;
  PVGLU_CUDA(cudaMemcpyAsync(x, nw->x64, nv * sizeof(double), cudaMemcpyDeviceToDevice,
                             as_stream(stream)));
  return PVGLU_OK;
}

int pvglu_newton_mismatch(pvglu_newton* nw, double* out) {
  if (!nw || !out) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  pvglu_numeric* h = nw->num;
  const pvglu::NtDev& D = nw->D;
  unsigned long long* mm = nullptr;
  PVGLU_CUDA(cudaMalloc((void**)&mm, D.ld * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(mm, 0, D.ld * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    pvglu::k_nt_elem_current<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256>>>(D, nw->x64, D.ieq);
    pvglu::k_nt_mismatch<<<pvglu::rows_grid(D.n, D.ld, 256), 256>>>(
        D, h->d.a_rowptr, h->d.a_colidx, h->st_base, nw->x64, D.ieq, mm);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> hb(D.ld);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    e = cudaMemcpy(hb.data(), mm, D.ld * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(mm);
  if (e != cudaSuccess) return fail(PVGLU_ERR_CUDA, cudaGetErrorString(e));
  for (int s = 0; s < D.S; s++) std::memcpy(&out[s], &hb[s], sizeof(double));
  return PVGLU_OK;
}

int pvglu_newton_adjoint(pvglu_newton* nw, const double* dpdx, double* dpdiph, void* stream) {
  if (!nw || !dpdx || !dpdiph) return fail(PVGLU_ERR_BAD_ARG, "NULL argument");
  pvglu_numeric* h = nw->num;
  cudaStream_t st = as_stream(stream);
  const pvglu::NtDev& D = nw->D;
  pvglu::k_nt_adjoint_companion<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256, 0, st>>>(D);
  const pvglu::AValues A = h->stamps(D.g, nullptr);
  int rc = pvglu::run_scatter(h, A, nullptr, st);
  if (rc) return rc;
  const pvglu::SkipDone none{nullptr, nullptr};
  if (h->precision == PVGLU_FP64) {
    // J^T lambda = dpdx: w = dpdx[col_orig], M^T z = w, lambda = z at row_pos.
    pvglu::k_permute<double, double><<<pvglu::rows_grid(h->n, h->ld, 256), 256, 0, st>>>(
        h->d.col_orig, h->n, h->ld, h->S, dpdx, nw->lam, 1);
    rc = pvglu::run_refactor_solve_perm(h, nw->lam, true, none, st);
    if (rc) return rc;
    pvglu::k_nt_adjoint_reduce<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256, 0, st>>>(
        D, nw->lam, h->row_pos, dpdiph);
  } else {
    rc = pvglu::run_refactor(h, st);
    if (!rc)
      rc = pvglu::run_refine(h, A, dpdx, nw->lam, true, nw->ir_tol, nw->ir_sweeps, nullptr, st);
    if (rc) return rc;
    pvglu::k_nt_adjoint_reduce<<<pvglu::rows_grid(D.n_elems, D.ld, 256), 256, 0, st>>>(
        D, nw->lam, nullptr, dpdiph);
  }
  PVGLU_CUDA(cudaGetLastError());
  return PVGLU_OK;
}

}  // extern "C"
