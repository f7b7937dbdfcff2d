/*
 * pvglu — GB300-native sparse LU hot path of the PV-plant power-flow Newton
 * iteration: Jacobian value scatter -> GLU numeric refactorization ->
 * forward/backward (and transposed) triangular solves, plus the symbolic
 * analysis that feeds them.
 *
 * C ABI: plain pointers and sizes, int status codes, no C++ or CUDA types.
 * Streams are passed as `void*` holding a cudaStream_t (NULL = legacy default
 * stream).  Device pointers are caller-owned; handles own their structure.
 * All device calls are asynchronous on the given stream unless they say
 * otherwise.  A handle is not thread-safe.
 *
 * Each entry point names the reference interface it replaces
 * (AlbertoJimenezRuiz/PhdThesis_AlbertoJimenezRuiz, PVPP_Plant_Simulator/).
 */
#ifndef PVGLU_H
#define PVGLU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference aborts on every one of these (gpu_util.h:39-47,
 * util.cpp:11-17, GLU_CSC_CPU_levels_strings.cpp:15-30); here they return. */
enum {
  PVGLU_OK = 0,
  PVGLU_ERR_BAD_ARG = 1,
  PVGLU_ERR_STRUCTURAL = 2,      /* no row exchange for a zero diagonal (004b:82) */
  PVGLU_ERR_ZERO_PIVOT = 3,      /* |U(j,j)| < pivot_tol or not finite (GLU_CSC_CPU_levels_strings.cpp:26-30) */
  PVGLU_ERR_NONFINITE = 4,
  PVGLU_ERR_CUDA = 5,
  PVGLU_ERR_BARRIER_TIMEOUT = 6, /* persistent kernel grid barrier gave up */
  PVGLU_ERR_NOT_CONVERGED = 7,
  PVGLU_ERR_NO_MEMORY = 8,
  PVGLU_ERR_TOO_LARGE = 9
};

enum { PVGLU_FP64 = 0, PVGLU_FP32 = 1 };

/* Solve flags. */
enum {
  PVGLU_SOLVE_TRANSPOSE = 1,  /* solve J^T x = b (adjoint) instead of J x = b     */
  PVGLU_SOLVE_ORIGINAL = 2    /* b and x in the caller's unknown order (the solve
                                 applies the row/column permutations); without it
                                 b and x are in the permuted order, as
                                 triangular_substitution_LU_CUDA expects */
};

/* Refactor/solve schedules.  LEVELS and PERSISTENT execute compiled chain
 * programs (each chain staged through shared memory); THREAD_CHAIN is the
 * reference's launch shape (one thread walks one chain through global memory,
 * one launch per level, factorize_electrical_system_CUDA.cu:72-115). */
enum {
  PVGLU_SCHED_LEVELS = 0,      /* one launch per level                          */
  PVGLU_SCHED_PERSISTENT = 1,  /* one cooperative launch, bounded grid barriers */
  PVGLU_SCHED_THREAD_CHAIN = 2 /* thread per chain, one launch per level        */
};

typedef struct pvglu_symbolic pvglu_symbolic;
typedef struct pvglu_numeric pvglu_numeric;
typedef struct pvglu_plant pvglu_plant;

/* Message of the last failing call on this thread ("" if none). */
const char* pvglu_last_error(void);
/* Library version string. */
const char* pvglu_version(void);

/* ---------------- symbolic analysis (host) ------------------------------- */

/* Replaces prepare_matrices (000_PVPP_simulator.cpp:10-93): ordering,
 * zero-diagonal row exchanges (004b), fill-in (005), GLU/L/U dependencies and
 * chained levels (006-009), CSR/CSC with cross maps (010).
 * rowptr/colidx: pattern of the Jacobian in the caller's unknown order (CSR,
 * n+1 / rowptr[n] entries, no duplicates).  perm: the ordering P in the
 * reference's semantics (interchanges_position_row_columns, 004a:40-42:
 * perm[k] = unknown placed at pivot k), e.g. the reference's AMD output; NULL
 * selects the built-in minimum-degree ordering. */
int pvglu_symbolic_create(int n, const int* rowptr, const int* colidx,
                          const int* perm, pvglu_symbolic** out);
int pvglu_symbolic_destroy(pvglu_symbolic* s);

/* Dump of a complete analysis to a file and back: every array of
 * pvglu_symbolic_get_array plus the execution structures, with a hash that
 * rejects a damaged file (PVGLU_ERR_BAD_ARG).  Lets a run restart without
 * re-analysis; the reference rebuilds struct_CPU_CUDA_arrays
 * (factorize_electrical_system.h:3-61) in prepare_matrices (000:10-93) at
 * every start. */
int pvglu_symbolic_save(const pvglu_symbolic* s, const char* path);
int pvglu_symbolic_load(const char* path, pvglu_symbolic** out);

typedef struct {
  int n;
  int64_t nnz_a, nnz_lu, update_count;
  int lu_levels, l_levels, u_levels, lt_levels;
  int lu_chains, l_chains, u_chains, lt_chains;
  int row_swaps;
  int perm_rows_is_involution;
  int64_t right_looking_hazards;
  double flops_refactor;
} pvglu_symbolic_info;
int pvglu_symbolic_get_info(const pvglu_symbolic* s, pvglu_symbolic_info* info);

/* Read-only views of the symbolic arrays (valid while the handle lives), by
 * name.  Reference names in brackets (struct_CPU_CUDA_arrays,
 * factorize_electrical_system.h:3-61):
 *   perm_amd [interchanges_position_row_columns], perm_rows
 *   [interchanges_position_row_columns_only_rows], row_orig, col_orig,
 *   fill_rowptr/fill_col [nonzero_values], csr_rowptr [mat_A_CSR_start_rows],
 *   csr_col, csc_colptr, csc_row, csr_to_csc
 *   [mat_A_CSR_corresponding_value_in_CSC], csc_to_csr, csr_diag_start
 *   [mat_A_CSR_start_from_diagonal], csc_diag_start, lu_sl/lu_sc/lu_cols
 *   [start_levels_unified_LU / start_chains_columns_unified_LU /
 *   chains_columns_unified_LU], l_*, u_*, lt_* (transposed-L levels),
 *   max_elements_per_column, slot_src, diag_slot. */
int pvglu_symbolic_get_array(const pvglu_symbolic* s, const char* name,
                             const int** data, int64_t* len);

/* ---------------- numeric state (device) --------------------------------- */

/* Device structure + LU value storage for n_scenarios independent Jacobians
 * sharing the symbolic analysis.  Values are stored slot-major with the
 * scenario index fastest: value(slot, s) at [slot * ld + s], ld =
 * pvglu_numeric_ld() (n_scenarios rounded up for aligned vector access).
 * Per-level schedule; chain merging as described under merge_chains of
 * pvglu_tuning.  Replaces struct_CPU_CUDA_arrays::create_CUDA
 * (factorize_electrical_system.h:63-98). */
int pvglu_numeric_create(const pvglu_symbolic* s, int n_scenarios, int precision,
                         pvglu_numeric** out);
/* As pvglu_numeric_create with the table size of the chain programs:
 * max_locals values staged in shared memory per warp and segment (0: the
 * default, 64 for batched FP32, 40 for batched FP64, 1023 for one scenario).
 * Smaller tables give more resident warps and more segments per chain.
 * PVGLU_ERR_BAD_ARG if the table does not fit in shared memory.  No
 * counterpart in the reference (its kernels read every value from global
 * memory). */
int pvglu_numeric_create_ex(const pvglu_symbolic* s, int n_scenarios, int precision,
                            int max_locals, pvglu_numeric** out);
int pvglu_numeric_max_locals(const pvglu_numeric* h);
/* How the handle executes its refactorization and solves: program levels
 * over all five phases (refactor, L, U, U^T, L^T), how many of them are WIDE
 * levels and how many wide units they hold (columns or rows too wide for
 * the table, run by a whole block each), the widest table, and the
 * operations and loads of the chain programs.  No counterpart in the
 * reference. */
typedef struct {
  int program_levels, wide_levels, wide_units, table_max;
  int64_t ops, loads;
} pvglu_numeric_info;
int pvglu_numeric_get_info(const pvglu_numeric* h, pvglu_numeric_info* info);
int pvglu_numeric_destroy(pvglu_numeric* h);
int pvglu_numeric_ld(const pvglu_numeric* h);
/* Device pointer to the LU values (double* for FP64, float* for FP32). */
void* pvglu_numeric_values(pvglu_numeric* h);
/* Refactor/solve schedule (PVGLU_SCHED_*) and the pivot threshold of the
 * zero-pivot check (default 1e-8, the reference's). */
int pvglu_numeric_set_schedule(pvglu_numeric* h, int schedule);
int pvglu_numeric_set_pivot_tol(pvglu_numeric* h, double tol);

/* (a) Scatter: LU(slot, s) = A(slot_src[slot], s), 0 at fill slots.
 * a_values: device, FP64, [nnz_a * ld], A's entries in the caller's CSR order.
 * Replaces the Newton-loop permutation + fill_values_CSC_only
 * (000_PVPP_simulator.cpp:193-210, 010_create_CSR_CSC.cpp:142-155). */
int pvglu_scatter(pvglu_numeric* h, const double* a_values, void* stream);

/* Structured Jacobian ("stamps").  A Newton Jacobian is a fixed linear part
 * plus the companion conductance of every nonlinear two-terminal element
 * stamped on up to four entries (002b_sistema_electrico_base_matriz.cpp:5-38
 * admittance stamp, :183-202 per-element G and convergence conductance).
 * Registering that structure once lets the scatter, the refinement residual
 * and the Newton driver read one FP64 conductance per element and scenario
 * instead of nnz_a FP64 values per scenario.
 * Host arrays, copied: base[nnz_a] linear values; entry e receives
 * sum over c in [entry_ptr[e], entry_ptr[e+1]) of entry_sign[c] * g[entry_elem[c]]
 * (entry_sign = +1 / -1), added after base in that order.  Replaces any
 * earlier registration on the handle. */
int pvglu_numeric_set_stamps(pvglu_numeric* h, int n_elems, const double* base,
                             const int* entry_ptr, const int* entry_elem,
                             const int* entry_sign);
/* (a) from stamps: g device FP64 [n_elems * ld] element conductances; gmin
 * device FP64 [ld] per-scenario convergence conductance added to every
 * element stamp where it is > 0, or NULL. */
int pvglu_scatter_stamps(pvglu_numeric* h, const double* g, const double* gmin, void* stream);

/* (b) GLU numeric refactorization in place, every scenario.
 * Replaces factorize_electrical_system_CUDA (factorize_electrical_system_CUDA.cu:61-152). */
int pvglu_refactor(pvglu_numeric* h, void* stream);

/* (a) + (b) in one call, with the same factors as pvglu_scatter then
 * pvglu_refactor.  Batched handles on PVGLU_SCHED_LEVELS whose
 * refactorization has no WIDE level, given 16-byte aligned a_values, run it
 * as one pass: each level reads its columns' entries straight from a_values,
 * so no scatter is launched and the factor values are written once.  Other
 * handles run pvglu_scatter, then pvglu_refactor. */
int pvglu_scatter_refactor(pvglu_numeric* h, const double* a_values, void* stream);

/* (c) Triangular solves with the stored factors, every scenario.
 * x: device, [n * ld], same precision as the factors; holds b on entry.
 * Replaces triangular_substitution_LU_CUDA (triangular_substitution.cu:232-271);
 * with PVGLU_SOLVE_TRANSPOSE it solves the adjoint system. */
int pvglu_solve(pvglu_numeric* h, void* x, int flags, void* stream);

/* (b) + (c) in one call: with the persistent schedule and a permuted-space
 * solve, a single cooperative launch walks the refactorization levels and
 * then the solve levels; otherwise pvglu_refactor then pvglu_solve. */
int pvglu_refactor_solve(pvglu_numeric* h, void* x, int flags, void* stream);

/* Error state of the last refactor (synchronizes the stream): status code,
 * first failing column and scenario (-1 if none).  Clears the state. */
int pvglu_numeric_check(pvglu_numeric* h, void* stream, int* code, int* column,
                        int* scenario);

/* Host-buffer drop-in used by the reference's C++ driver: copies the CSC
 * values (FP64, [nnz_lu], single scenario) in, refactors, copies the combined
 * LU back (factorize_electrical_system_CUDA semantics: host in, host out).
 * Synchronous. */
int pvglu_refactor_host(pvglu_numeric* h, double* csc_values);
/* Host-buffer solve (triangular_substitution_LU_CUDA semantics, permuted
 * space): b (FP64, [n]) in, x out.  Synchronous. */
int pvglu_solve_host(pvglu_numeric* h, double* b);

/* One full Newton linear step from host buffers: H2D of A's values
 * ([nnz_a * ld], FP64) and b ([n * ld], FP64, original order), scatter,
 * refactor, solve, D2H of x ([n * ld], FP64, original order).  FP64 handles
 * only.  Asynchronous on `stream` (pinned host buffers give async copies). */
int pvglu_scatter_refactor_solve_host(pvglu_numeric* h, const double* a_values_host,
                                      const double* b_host, double* x_host,
                                      void* stream);

/* ---------------- FP32 factors + FP64 iterative refinement --------------- */

/* Solves J x = b (original order) for every scenario with the FP32 factors of
 * h (pvglu_scatter + pvglu_refactor done on an FP32 handle), refining in FP64:
 * r = b - J x with J from a_values (FP64, [nnz_a * ld]), correction solved in
 * FP32, accumulated in FP64.  Stops per scenario when
 * max|dx| <= tol * max|x|, or when the error left after the sweep,
 * estimated as max|dx| rho / (1 - rho) with rho = max|dx_k| / max|dx_k-1|
 * <= 1/2, is <= tol * max|x|; after at most max_sweeps sweeps.  b, x: FP64
 * device [n * ld].  sweeps_out (device int[ld], may be NULL) receives the
 * sweeps per scenario; -1 marks a scenario that did not converge. */
int pvglu_solve_refined(pvglu_numeric* h, const double* a_values, const double* b,
                        double* x, double tol, int max_sweeps, int* sweeps_out,
                        void* stream);

/* General form of pvglu_solve_refined: A's values either explicit
 * (a_values, g NULL) or from the registered stamps (g [n_elems * ld] and
 * optional gmin [ld], a_values NULL).  flags: PVGLU_SOLVE_TRANSPOSE refines
 * J^T x = b (the adjoint system) with an FP64 residual over J's columns.
 * Launches: on a stream that is not being captured, and for the per-level
 * schedules, the sweeps run from a CUDA graph of the handle whose sweep loop
 * is a conditional while node (built on the first call with these pointers,
 * tolerance and sweep cap; replayed afterwards), so no sweep after
 * convergence is launched.  Inside a capture, with the persistent schedule,
 * or with PVGLU_REFINE_GRAPH=0 in the environment, the sweeps are launched
 * one by one, max_sweeps of them, each exiting at once after convergence.
 * The results are the same in both forms. */
int pvglu_refine(pvglu_numeric* h, const double* a_values, const double* g, const double* gmin,
                 const double* b, double* x, int flags, double tol, int max_sweeps,
                 int* sweeps_out, void* stream);

/* One residual of the refinement, for callers that run their own loop (and
 * for timing the kernel): r = b - J x with FP64 arithmetic (J from a_values,
 * [nnz_a * ld]), rounded to FP32 and stored in pivot order, the right-hand
 * side of a correction solve with pvglu_solve on this FP32 handle.  b, x:
 * FP64 device [n * ld], caller order; r: FP32 device [n * ld]; every
 * scenario s < S is computed.  No counterpart in the reference. */
int pvglu_refine_residual(pvglu_numeric* h, const double* a_values, const double* b,
                          const double* x, float* r, void* stream);

/* Host-buffer form of one refined linear step on an FP32 handle: H2D of A's
 * values ([nnz_a * ld], FP64) and b ([n * ld], FP64, original order),
 * scatter, FP32 refactor, pvglu_solve_refined, D2H of x ([n * ld], FP64).
 * sweeps_out: device int[ld] or NULL.  Asynchronous on `stream`. */
int pvglu_refine_system_host(pvglu_numeric* h, const double* a_values_host,
                             const double* b_host, double* x_host, double tol, int max_sweeps,
                             int* sweeps_out, void* stream);

/* As pvglu_refine_system_host with the Jacobian given by the stamps of
 * pvglu_numeric_set_stamps: H2D of the element conductances g ([n_elems *
 * ld], FP64) instead of A's values, A's values assembled from the stamps
 * on the device, then as pvglu_refine_system_host, D2H of x.  A Newton caller
 * computes one conductance per element (002b:183-197) before it assembles
 * A, so this moves n_elems values per scenario over the host link instead of
 * nnz_a.  No counterpart in the reference. */
int pvglu_refine_stamps_host(pvglu_numeric* h, const double* g_host, const double* b_host,
                             double* x_host, double tol, int max_sweeps, int* sweeps_out,
                             void* stream);

/* ---------------- allocation-free solve ---------------------------------- */

/* The original-order solve of pvglu_solve (flags: PVGLU_SOLVE_TRANSPOSE
 * optional, PVGLU_SOLVE_ORIGINAL implied) for FP64 handles, with its permuted
 * work vector in a static device array owned by the library instead of the
 * handle's work buffer.  It calls no cudaMalloc or cudaFree and no other
 * allocating routine.  It is meant for callers whose solve path must not
 * allocate device memory, for example an application that reserves the GPU's
 * memory up front and forbids further allocation, or a real-time loop where
 * an allocation's implicit synchronisation is not acceptable.  (The handle
 * itself is still created beforehand with pvglu_numeric_create.)
 * Limit: n * ld <= 1,048,576 FP64 entries (8 MiB, reserved on every GPU
 * that loads the library until the process exits); larger handles get
 * PVGLU_ERR_TOO_LARGE.  The handle's device must be the current device
 * (PVGLU_ERR_BAD_ARG otherwise).  Set-up: the first call on a device looks
 * the array's device address up with cudaGetSymbolAddress, with that device
 * current, and caches it; a device reset ends the context, and the first
 * call in the new context looks it up again.  Make the first call on each
 * device (and after a reset) before any stream capture.  All calls share the
 * array and it keeps the last call's contents; nothing in it needs to start
 * at zero.  Calls whose work overlaps on the GPU (other streams, other
 * threads) race on the array.
 * No counterpart in the reference. */
int pvglu_solve_noalloc(pvglu_numeric* h, double* x, int flags, void* stream);

/* ---------------- size-class groups -------------------------------------- */

/* Up to 4 numeric handles over different symbolic analyses (plants of
 * different sizes) that share precision and batching.  A group refactor +
 * solve issues one launch per level over the work items of every member
 * (level l of all members together), instead of one sequence per member.
 * Each member keeps its values (scatter them with pvglu_scatter first), its
 * status and its pivot threshold.  No counterpart in the reference (one
 * circuit per run). */
typedef struct pvglu_group pvglu_group;
int pvglu_group_create(pvglu_numeric* const* members, int count, pvglu_group** out);
int pvglu_group_destroy(pvglu_group* g);
/* Refactor every member, then solve member i's vector x[i] ([n_i * ld_i], the
 * member's precision; pivot order, or caller order with PVGLU_SOLVE_ORIGINAL).
 * x == NULL: refactor only. */
int pvglu_group_refactor_solve(pvglu_group* g, void* const* x, int flags, void* stream);

/* ---------------- autotuner ---------------------------------------------- */

/* Times scatter + refactor + solve for n_scenarios on this device over the
 * chain-program table sizes and the schedules, with diagonally dominant
 * stand-in values on s's pattern, and returns the fastest combination (for
 * pvglu_numeric_create_ex and pvglu_numeric_set_schedule) and its time per
 * call in ms.  Synchronous; allocates and frees temporary handles.  No
 * counterpart in the reference (its launch shape is fixed by the >64-entry
 * rule of 009_get_max_numbers_per_column.cpp). */
int pvglu_autotune(const pvglu_symbolic* s, int n_scenarios, int precision,
                   int* best_max_locals, int* best_schedule, double* best_ms);

/* Every execution choice of a numeric handle:
 *   max_locals      chain-program table size (0: the default), as for
 *                   pvglu_numeric_create_ex;
 *   wide_threshold  units (columns of the refactorization, unknowns of a
 *                   solve) needing more table rows than this run as wide
 *                   units, a whole block each, even where they would fit the
 *                   table (0: only those too wide for it).  The reference
 *                   switches its launch shape to 32 threads per column once a
 *                   level's longest row passes 64 entries
 *                   (009_get_max_numbers_per_column.cpp:3-31,
 *                   factorize_electrical_system_CUDA.cu:75-77);
 *   merge_chains    1: units regrouped into execution levels one unit at a
 *                   time (a unit joins the chain of its last dependency); 2:
 *                   the same, and a unit also joins a chain whose unit
 *                   before the last is its dependency (ladders of two-unit
 *                   rungs, as the string nodes of a plant ordered from the
 *                   bus end give in the U solve, become one chain); 0: the
 *                   level set's own levels and chains, merged a whole level
 *                   at a time as the reference does
 *                   (007_convert_dependencies_in_levels.cpp:89-210).
 *                   pvglu_numeric_create(_ex) chooses 2 where that halves
 *                   the execution levels of the refactorization and the L
 *                   and U solves together, 0 otherwise.  Regrouping removes
 *                   levels on deep patterns but can lengthen the chains of a
 *                   narrow level where no level is saved;
 *   schedule        PVGLU_SCHED_*. */
typedef struct {
  int max_locals;
  int wide_threshold;
  int merge_chains;
  int schedule;
} pvglu_tuning;
int pvglu_numeric_create_tuned(const pvglu_symbolic* s, int n_scenarios, int precision,
                               const pvglu_tuning* t, pvglu_numeric** out);
/* The autotuner over all of pvglu_tuning: table sizes x schedules, and, where
 * they change the handle's programs, the three chain merging modes and a
 * wide threshold at half the table.  Synchronous; allocates and frees temporary
 * handles.  best receives the fastest combination, best_ms its time per
 * scatter + refactor + solve.  No counterpart in the reference. */
int pvglu_autotune_ex(const pvglu_symbolic* s, int n_scenarios, int precision,
                      pvglu_tuning* best, double* best_ms);

/* ---------------- scenario blocks ----------------------------------------- */

/* One batch of scenarios held as `parts` numeric handles ("blocks") of
 * n_scenarios / parts scenarios each: same analysis, precision and tuning
 * (NULL: pvglu_numeric_create's defaults), each block with a CUDA stream of
 * its own.  A step runs the blocks side by side, so one block's narrow,
 * latency-bound levels and launch tails overlap the other blocks' work (512
 * scenarios of the 35k plant, FP32 + refinement, each block running its steps
 * back to back: 4 blocks of 128 take 0.948-0.972 ms per step, one handle of
 * 512 1.003-1.030 ms; 8 of 64: 0.989 ms).  Every value
 * is the same as one handle's for the same scenarios.  Buffers are per
 * block, in that block's layout (ld_k = pvglu_numeric_ld of the block).  No
 * counterpart in the reference (one circuit per run).  n_scenarios must be
 * a multiple of parts. */
typedef struct pvglu_blocks pvglu_blocks;
int pvglu_blocks_create(const pvglu_symbolic* s, int n_scenarios, int parts, int precision,
                        const pvglu_tuning* tuning, pvglu_blocks** out);
int pvglu_blocks_destroy(pvglu_blocks* b);
/* Block k's numeric handle (owned by b: do not destroy it). */
int pvglu_blocks_part(pvglu_blocks* b, int k, pvglu_numeric** out);
/* One Newton iteration's linear algebra for every block k, on the block's
 * stream: pvglu_scatter_refactor(a_values[k]), then x[k] = J^-1 b[k] in the
 * caller's order (FP32 blocks: pvglu_solve_refined with tol and max_sweeps,
 * sweeps_out[k] or NULL per block; FP64 blocks: a copy of b[k] solved with
 * PVGLU_SOLVE_ORIGINAL).  a_values[k] [nnz_a * ld_k], b[k] and x[k]
 * [n * ld_k] are FP64 device buffers.  The blocks start after the work
 * already on `stream`, and `stream` waits for all of them, also under
 * stream capture; with PVGLU_BLOCKS_NO_JOIN in flags it does not, and each
 * block's stream runs on into its next step as soon as its own step ends
 * (blocks are independent): pvglu_blocks_join then makes `stream` wait for
 * every block. */
enum { PVGLU_BLOCKS_NO_JOIN = 1 };
int pvglu_blocks_step(pvglu_blocks* b, const double* const* a_values, const double* const* rhs,
                      double* const* x, double tol, int max_sweeps, int* const* sweeps_out,
                      int flags, void* stream);
int pvglu_blocks_join(pvglu_blocks* b, void* stream);

/* ---------------- failure-path self-test --------------------------------- */

/* Runs one bounded grid barrier that waits for one block more than it
 * launches, so that it can only end by its spin limit (max_spins polls of
 * ~64 ns; at most 2^24).  Synchronous.  status_code receives the recorded
 * status (PVGLU_ERR_BARRIER_TIMEOUT expected), blocks_returned the number of
 * blocks that came back reporting the abort.  No reference counterpart: the
 * reference has no bounded waits (it aborts, gpu_util.h:39-47). */
int pvglu_selftest_barrier_timeout(int blocks, long long max_spins, int* status_code,
                                   int* blocks_returned);

#ifdef __cplusplus
}
#endif
#endif /* PVGLU_H */
