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

// Operation codes (low 4 bits of Op::code).
enum : int {
  OP_FNMA = 0,   // t[a] = t[a] - t[b] * t[c]
  OP_SCALE = 1,  // p = t[a]; pivot check (column c); t[b + i] /= p, i < code >> 4
  OP_DIV = 2,    // t[a] = t[a] / t[b]
};

struct Op {
  int code, a, b, c;
};

// Segment header.  load refs: refactor programs reference LU slots
// (ref = slot * 2 + store_back); solve programs reference solution entries
// (ref = index * 2 + store_back, index >= 0) or LU slots (ref = -(slot + 1),
// read only).  A segment with n_load < 0 is DIRECT: column/row `op_begin`
// is executed straight from global memory (too wide for the local table).
struct Segment {
  int load_begin, n_load, op_begin, n_op;
};

struct ChainProgram {
  int kind = -1;                 // -1 refactor, 0 L, 1 U, 2 U^T, 3 L^T
  int max_locals = 0;            // local table budget the program was built for
  std::vector<int> level_chain;  // [levels + 1] -> chain index
  std::vector<int> chain_seg;    // [chains + 1] -> segment index
  std::vector<Segment> seg;
  std::vector<int> loads;
  std::vector<Op> ops;
  int longest_chain_segments = 0;
  int direct_segments = 0;
};

// kind -1 uses s.lu; 0 s.l; 1 s.u; 2 s.lu; 3 s.lt.
void build_chain_program(const Symbolic& s, int kind, int max_locals, ChainProgram& out);

}  // namespace pvglu
