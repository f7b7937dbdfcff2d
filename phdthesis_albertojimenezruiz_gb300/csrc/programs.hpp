// Chain programs: the per-chain work of the refactorization and of the four
// triangular solves compiled, at analysis time, into segments of straight-line
// operations on a small local table.
//
// A warp runs one chain (for one group of 32 scenarios, or for the single
// scenario).  For each segment of the chain it
//   1. loads every value the segment touches into shared memory: its own
//      slots (or solution entries) and the final values it reads from earlier
//      levels -- independent coalesced loads, many in flight per warp;
//   2. executes the segment's operations out of shared memory;
//   3. writes its own values back.
// The level/chain order is the reference's (007_convert_dependencies_in_
// levels.cpp); only the way one chain is executed changes: the reference's
// kernels walk a chain column by column through global memory
// (factorize_matrix_GLU_CUDA.cuh:181-210, triangular_substitution.cu:114-144).
#pragma once
#include <cstdint>
#include <vector>

#include "symbolic.hpp"

namespace pvglu {

// Operations are packed in 32 bits: code (2) | a (10) | b (10) | c (10),
// so a local table holds at most kMaxLocals entries.
enum : int {
  OP_FNMA = 0,   // t[a] = t[a] - t[b] * t[c]
  OP_SCALE = 1,  // p = t[a]; pivot check; t[b + i] /= p for i < c
  OP_DIV = 2,    // t[a] = t[a] / t[b]
  OP_NOP = 3,    // padding to a multiple of 4 operations per segment
};
constexpr int kMaxLocals = 1023;

inline uint32_t pack_op(int code, int a, int b, int c) {
  return (uint32_t)code | ((uint32_t)a << 2) | ((uint32_t)b << 12) | ((uint32_t)c << 22);
}

// Segment header.  Loads: refactor programs reference LU slots (ref =
// slot); solve programs reference solution entries (ref = i >= 0) or
// read-only LU slots (ref = -(slot + 1)).  The first n_own loads are the
// segment's own entries, written back after the operations.
// A segment with n_load < 0 is WIDE: it is the whole chain of a wide
// program level, and op_begin indexes the program's wide units (a column or
// row too wide for any table, executed by a whole block: see WidePlan).
// Up to kMaxCarry entries a segment needs that the previous segment of the
// same chain already holds in its table are moved inside shared memory
// instead of being loaded (carry[k] = from << 16 | to, -1 unused).
constexpr int kMaxCarry = 4;

struct Segment {
  int load_begin, n_load, n_own, op_begin, n_op;
  int reads_own_chain = 0;  // loads entries written by an earlier segment of the chain
  int n_carry = 0;
  int carry[kMaxCarry] = {-1, -1, -1, -1};
};

// Execution levels.  The units (columns of the refactorization, unknowns
// of a solve) are regrouped from the reference's level set into execution
// levels of chains: walking the units in the level set's order (a
// topological order), let m be the highest execution level of a unit's
// dependencies; when all its dependencies at level m lie in one chain whose
// last unit is one of them, the unit extends that chain; otherwise it starts
// a new chain at level m + 1 (level 0 without dependencies).  Every
// dependency of a unit is then in an earlier level or earlier in its own
// chain, so any execution that runs the levels in order and each chain in
// order computes, unit for unit, the same arithmetic.  Extending a chain
// never delays a unit (it waits for that chain's last unit in any order) and
// never makes another chain wait.  Ladder merging also extends the chain
// when the dependency is the unit before its last: a unit then waits for one
// unit it does not depend on, and a ladder of two-unit rungs (each rung's
// first unit depending on the previous rung's first unit, as the string
// nodes of a plant ordered from the bus end give in the U solve) becomes one
// chain instead of one level per rung.  The reference merges chains a whole
// basic level at a time (007_convert_dependencies_in_levels.cpp:62-143): one
// unit that cannot join keeps its whole level from merging.  The level set
// itself (the symbolic arrays) is unchanged.
//
// Program levels.  Every execution level is executed as one or more program
// levels: a chain is cut around each unit too wide for the level's table
// budget, the pieces before the first wide unit form the first program
// level, the wide units of that position the next one (a WIDE level, one
// chain per wide unit), the pieces between the first and second wide unit
// the next, and so on.  Chains of one level are independent and each keeps
// its order, so the program levels in sequence compute what the level
// computes.
//
// A wide refactor unit (column k) is executed in gather form, scheduled
// inside the column: target slot t of column k receives
//     M(t) -= L(i, j) * U(j, k)   for its pairs (q = slot of L(i, j), p = slot of U(j, k))
// in ascending j (the order of the reference's right-looking loop, so FP64
// stays bit-exact).  The targets (slots with at least one pair) are grouped
// into chains and chain levels by the execution-level rule applied inside
// the column, one target at a time in slot order: a target whose sources
// that are targets lie, at their highest chain level, in one chain whose last
// target is one of them extends that chain; otherwise it starts a new chain
// one level above them.  A chain is computed in order by one thread (one warp
// batched), so a target reads a source of its own chain right after that
// thread wrote it; a block barrier separates the chain levels.  A target
// with more than kWideLong pairs is computed by the whole block (ordered
// block sum) and is a chain of its own that no target extends.  After the
// last level the L part is divided by the pivot.  A pair whose U source is
// a target of the same chain carries ~p (negative) instead of p.
//
// Each target has one record of four ints {slot, src, n_pairs, q} (one
// 16-byte load on the device): with one pair, src is its U slot (or ~slot)
// and q its L slot; otherwise src is the index of its first pair in pr_q /
// pr_p (the pairs of consecutive targets are consecutive) and q is -1.
constexpr int kWideLong = 96;
struct WidePlan {
  std::vector<int> unit;      // [W] column (refactor) or unknown (solves)
  // refactor only:
  std::vector<int> lvl;       // [W + 1] -> index into lv_chain (the unit's chain levels)
  std::vector<int> lv_chain;  // [chain levels + 1] -> index into ch_tgt
  std::vector<int> ch_tgt;    // [chains + 1] -> target index (a chain's targets, in order)
  std::vector<int> tg_rec;    // [4 T] target records
  std::vector<int> pr_q, pr_p;  // [P] L slot and U slot (~slot: same chain) of every update
  int targets() const { return (int)tg_rec.size() / 4; }
};

struct ChainProgram {
  int kind = -1;                 // -1 refactor, 0 L, 1 U, 2 U^T, 3 L^T
  int max_locals = 0;            // widest table of any level
  std::vector<int> level_max_locals;  // [levels] table size of each program level: its
                                      // widest segment, at most the level's budget
  std::vector<int> level_chain;  // [levels + 1] -> chain index
  std::vector<int> level_src;    // [levels] execution level it belongs to
  std::vector<int> level_budget; // [levels] table budget of that execution level
  std::vector<int> level_wide_at;  // [levels] units needing more rows than this are wide
  std::vector<char> level_wide;  // [levels] 1: a WIDE level
  std::vector<int> chain_seg;    // [chains + 1] -> segment index
  std::vector<int> chain_unit;   // [chains + 1] -> index into units
  std::vector<int> units;        // units of each chain, in execution order
  std::vector<Segment> seg;
  std::vector<int> loads;
  std::vector<uint32_t> ops;     // packed, each segment's run padded to 4
  std::vector<int> op_col;       // column of each SCALE operation (error reports)
  WidePlan wide;
  int longest_chain_segments = 0;
  int wide_units = 0;
  int wide_levels = 0;
};

// Table budgets: max_locals values per table; an execution level with at
// most narrow_chains chains gets max(max_locals, wide_locals) (levels with
// few chains can afford a wide table: fewer segments, and the warps they
// leave idle cost nothing).  A unit whose own table would exceed its level's
// budget is a wide unit.  merge: 0 keeps the level set's levels and chains
// as execution levels, 1 regroups them per unit, 2 with ladder merging.
struct ProgramOptions {
  int max_locals = 64;
  int wide_locals = 0;
  int narrow_chains = 0;
  int merge = 1;
  // > 0: units needing more than this many table rows run as wide units
  // even where they would fit the level's table (at most the budget).
  int wide_threshold = 0;
};

// kind -1 uses s.lu; 0 s.l; 1 s.u; 2 s.lu; 3 s.lt.
void build_chain_program(const Symbolic& s, int kind, const ProgramOptions& opt,
                         ChainProgram& out);
void build_chain_program(const Symbolic& s, int kind, int max_locals, ChainProgram& out);
// The level set a program kind walks, and the units a unit depends on.
const LevelSet& program_levels(const Symbolic& s, int kind);
// Execution levels of a program kind with chain merging `merge` (as
// ProgramOptions::merge), before any wide unit is cut out.
int execution_level_count(const Symbolic& s, int kind, int merge);
void unit_deps(const Symbolic& s, int kind, int u, std::vector<int>& deps);

}  // namespace pvglu
