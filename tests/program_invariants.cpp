// Test helper (host only): builds the chain programs of a CSR pattern for
// every program kind and several table budgets and checks the invariants the
// device executors rely on for memory safety and ordering.
//   usage: program_invariants <n> <rowptr.bin> <colidx.bin>
// Exit status 0 when every check passes; the first violation is printed.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "programs.hpp"
#include "symbolic.hpp"

using namespace pvglu;

namespace {

std::vector<int> read_ints(const char* path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const std::streamsize bytes = f.tellg();
  f.seekg(0);
  std::vector<int> v(bytes / (std::streamsize)sizeof(int));
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(int)));
  return v;
}

int fails = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      if (fails++ < 5) {                 \
        std::printf("FAIL %s: ", #cond); \
        std::printf(__VA_ARGS__);        \
        std::printf("\n");               \
      }                                  \
    }                                    \
  } while (0)

void check_program(const Symbolic& s, int kind, const std::vector<int>& budget) {
  ChainProgram pr;
  build_chain_program(s, kind, budget, pr);
  const LevelSet& ls = program_levels(s, kind);
  CHECK(pr.level_chain == ls.start_levels, "kind %d level_chain", kind);
  CHECK((int)pr.chain_seg.size() == ls.num_chains() + 1, "kind %d chain_seg size", kind);
  CHECK((int)pr.level_max_locals.size() == ls.num_levels(), "kind %d level tables", kind);
  for (int lv = 0; lv < ls.num_levels(); lv++) {
    const int table = pr.level_max_locals[lv];
    CHECK(table >= 1 && table <= budget[lv] && table <= pr.max_locals,
          "kind %d level %d table %d budget %d", kind, lv, table, budget[lv]);
    for (int c = ls.start_levels[lv]; c < ls.start_levels[lv + 1]; c++) {
      CHECK(pr.chain_seg[c] <= pr.chain_seg[c + 1], "kind %d chain %d segments", kind, c);
      int prev_nl = -1;  // table rows of the previous segment of the chain (-1: none)
      for (int g = pr.chain_seg[c]; g < pr.chain_seg[c + 1]; g++) {
        const Segment& sg = pr.seg[g];
        if (sg.n_load < 0) {  // DIRECT unit
          CHECK(sg.op_begin >= 0 && sg.op_begin < s.n, "kind %d DIRECT unit %d", kind,
                sg.op_begin);
          prev_nl = -1;
          continue;
        }
        CHECK(sg.n_load <= table, "kind %d level %d segment %d loads %d > table %d", kind, lv,
              g, sg.n_load, table);
        CHECK(sg.n_own >= 0 && sg.n_own <= sg.n_load, "kind %d segment %d own", kind, g);
        CHECK(sg.n_carry >= 0 && sg.n_carry <= kMaxCarry, "kind %d segment %d carries", kind, g);
        CHECK(sg.n_carry == 0 || prev_nl > 0, "kind %d segment %d carries at a chain start",
              kind, g);
        for (int k = 0; k < sg.n_carry; k++) {
          const int from = sg.carry[k] >> 16, to = sg.carry[k] & 0xffff;
          CHECK(from >= 0 && from < prev_nl, "kind %d segment %d carry from %d", kind, g, from);
          CHECK(to >= 0 && to < sg.n_load, "kind %d segment %d carry to %d", kind, g, to);
          for (int j = 0; j < k; j++)
            CHECK((sg.carry[j] & 0xffff) != to, "kind %d segment %d duplicate carry", kind, g);
        }
        for (int l = 0; l < sg.n_load; l++) {
          const int r = pr.loads[sg.load_begin + l];
          if (kind < 0) {
            CHECK(r >= 0 && r < s.nnz_lu, "kind %d load %d", kind, r);
          } else if (r >= 0) {
            CHECK(r < s.n, "kind %d solution row %d", kind, r);
          } else {
            CHECK(-r - 1 < s.nnz_lu, "kind %d value %d", kind, -r - 1);
            CHECK(l >= sg.n_own, "kind %d segment %d owns a read-only value", kind, g);
          }
        }
        CHECK(sg.n_op % 4 == 0 && sg.op_begin % 4 == 0, "kind %d segment %d op padding", kind, g);
        for (int k = 0; k < sg.n_op; k++) {
          const uint32_t op = pr.ops[sg.op_begin + k];
          const int code = op & 3, a = (op >> 2) & 1023, b = (op >> 12) & 1023,
                    cc = (op >> 22) & 1023;
          if (code == OP_FNMA) {
            CHECK(a < sg.n_load && b < sg.n_load && cc < sg.n_load, "kind %d FNMA operands",
                  kind);
          } else if (code == OP_SCALE) {
            CHECK(a < sg.n_load && (cc == 0 || b + cc <= sg.n_load), "kind %d SCALE operands",
                  kind);
          } else if (code == OP_DIV) {
            CHECK(a < sg.n_load && b < sg.n_load, "kind %d DIV operands", kind);
          }
        }
        prev_nl = sg.n_load;
      }
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::printf("usage: %s n rowptr.bin colidx.bin\n", argv[0]);
    return 2;
  }
  const int n = std::stoi(argv[1]);
  const std::vector<int> rowptr = read_ints(argv[2]), colidx = read_ints(argv[3]);
  Symbolic s;
  std::string err;
  SymbolicOptions opt;
  if (build_symbolic(n, rowptr.data(), colidx.data(), nullptr, opt, s, err)) {
    std::printf("analysis failed: %s\n", err.c_str());
    return 2;
  }
  for (int kind = -1; kind <= 3; kind++) {
    const LevelSet& ls = program_levels(s, kind);
    for (int base : {8, 16, 24, 64, 1023}) {
      std::vector<int> budget(ls.num_levels(), base);
      check_program(s, kind, budget);
      // The handle's rule: narrow levels get a wide budget.
      for (int lv = 0; lv < ls.num_levels(); lv++)
        if (ls.start_levels[lv + 1] - ls.start_levels[lv] <= 64) budget[lv] = 226;
      check_program(s, kind, budget);
    }
  }
  std::printf("%s n=%d nnz_lu=%lld\n", fails ? "FAILED" : "ok", s.n, (long long)s.nnz_lu);
  return fails ? 1 : 0;
}
