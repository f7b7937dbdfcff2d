// Test helper (host only): builds the chain programs of a CSR pattern for
// every program kind and several table budgets and checks the invariants the
// device executors rely on for memory safety and ordering.
//   usage: program_invariants <n> <rowptr.bin> <colidx.bin>
// Exit status 0 when every check passes; the first violation is printed.
#include <algorithm>
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

// Table rows a unit needs on its own (what the compiler measures).
int unit_need(const Symbolic& s, int kind, int u) {
  std::vector<int> xs, vs;
  auto x = [&](int i) { xs.push_back(i); };
  auto v = [&](int q) { vs.push_back(q); };
  if (kind == -1) {
    const int c0 = s.csc_colptr[u], dk = s.diag_slot[u], c1 = s.csc_colptr[u + 1];
    for (int q = c0; q < c1; q++) v(q);
    for (int p = c0; p < dk; p++) {
      const int j = s.csc_row[p];
      for (int q = s.diag_slot[j] + 1; q < s.csc_colptr[j + 1]; q++) v(q);
    }
  } else if (kind == 0 || kind == 1) {
    x(u);
    const auto& ptr = kind == 0 ? s.lrow_ptr : s.urow_ptr;
    const auto& slot = kind == 0 ? s.lrow_slot : s.urow_slot;
    const auto& col = kind == 0 ? s.lrow_col : s.urow_col;
    for (int e = ptr[u]; e < ptr[u + 1]; e++) {
      x(col[e]);
      v(slot[e]);
    }
    if (kind == 1) v(s.diag_slot[u]);
  } else {
    x(u);
    const int b = kind == 2 ? s.csc_colptr[u] : s.diag_slot[u] + 1;
    const int e = kind == 2 ? s.diag_slot[u] : s.csc_colptr[u + 1];
    for (int q = b; q < e; q++) {
      x(s.csc_row[q]);
      v(q);
    }
    if (kind == 2) v(s.diag_slot[u]);
  }
  std::sort(xs.begin(), xs.end());
  std::sort(vs.begin(), vs.end());
  return (int)(std::unique(xs.begin(), xs.end()) - xs.begin() +
               (std::unique(vs.begin(), vs.end()) - vs.begin()));
}

void check_program(const Symbolic& s, int kind, const ProgramOptions& opt) {
  ChainProgram pr;
  build_chain_program(s, kind, opt, pr);
  const int nlev = (int)pr.level_chain.size() - 1;
  CHECK((int)pr.level_wide_at.size() == nlev, "kind %d wide thresholds", kind);
  for (int lv = 0; lv < nlev && (int)pr.level_wide_at.size() == nlev; lv++)
    CHECK(pr.level_wide_at[lv] >= 1 && pr.level_wide_at[lv] <= pr.level_budget[lv] &&
              (opt.wide_threshold <= 0 || pr.level_wide_at[lv] <= opt.wide_threshold),
          "kind %d level %d wide threshold", kind, lv);
  CHECK((int)pr.level_src.size() == nlev && (int)pr.level_wide.size() == nlev &&
            (int)pr.level_max_locals.size() == nlev && (int)pr.level_budget.size() == nlev,
        "kind %d level arrays", kind);
  // Program levels come from the execution levels in order, and their count
  // is what execution_level_count reports (the default chain merging of a
  // handle is chosen from it).
  if (nlev > 0 && (int)pr.level_src.size() == nlev) {
    for (int lv = 1; lv < nlev; lv++)
      CHECK(pr.level_src[lv] >= pr.level_src[lv - 1], "kind %d level order", kind);
    CHECK(pr.level_src.back() + 1 == execution_level_count(s, kind, opt.merge),
          "kind %d execution levels %d vs %d", kind, pr.level_src.back() + 1,
          execution_level_count(s, kind, opt.merge));
  }
  CHECK((int)pr.chain_seg.size() == pr.level_chain.back() + 1 &&
            (int)pr.chain_unit.size() == pr.level_chain.back() + 1,
        "kind %d chain arrays", kind);
  // Every unit once; every dependency of a unit in an earlier program level
  // or earlier in the unit's own chain.
  std::vector<int> where_lv(s.n, -1), where_chain(s.n, -1), where_pos(s.n, -1);
  int pos = 0;
  for (int lv = 0; lv < nlev; lv++) {
    CHECK(lv == 0 || pr.level_src[lv] >= pr.level_src[lv - 1], "kind %d level order", kind);
    for (int c = pr.level_chain[lv]; c < pr.level_chain[lv + 1]; c++)
      for (int k = pr.chain_unit[c]; k < pr.chain_unit[c + 1]; k++) {
        const int u = pr.units[k];
        CHECK(u >= 0 && u < s.n && where_lv[u] < 0, "kind %d unit %d twice", kind, u);
        where_lv[u] = lv;
        where_chain[u] = c;
        where_pos[u] = pos++;
      }
  }
  CHECK(pos == s.n, "kind %d units %d of %d", kind, pos, s.n);
  std::vector<int> deps;
  for (int u = 0; u < s.n && pos == s.n; u++) {
    unit_deps(s, kind, u, deps);
    for (const int dd : deps)
      CHECK(where_lv[dd] < where_lv[u] ||
                (where_chain[dd] == where_chain[u] && where_pos[dd] < where_pos[u]),
            "kind %d unit %d runs before its dependency %d", kind, u, dd);
  }
  auto budget_of = [&](int lv) {
    const int b = pr.level_budget[lv];
    CHECK(b == std::min(opt.max_locals, kMaxLocals) ||
              b == std::min(std::max(opt.max_locals, opt.wide_locals), kMaxLocals),
          "kind %d level %d budget %d", kind, lv, b);
    return b;
  };
  // Refactorization: own-row count of every LU slot (a WIDE column's slots
  // count once for the column).
  std::vector<int> owned(kind < 0 ? s.nnz_lu : 0, 0);
  for (int lv = 0; lv < nlev; lv++) {
    const int table = pr.level_max_locals[lv];
    const int bud = budget_of(lv);
    CHECK(table >= 1 && table <= bud && table <= pr.max_locals,
          "kind %d level %d table %d budget %d", kind, lv, table, bud);
    for (int c = pr.level_chain[lv]; c < pr.level_chain[lv + 1]; c++) {
      CHECK(pr.chain_seg[c] <= pr.chain_seg[c + 1], "kind %d chain %d segments", kind, c);
      if (pr.level_wide[lv]) {
        CHECK(pr.chain_seg[c + 1] == pr.chain_seg[c] + 1 &&
                  pr.chain_unit[c + 1] == pr.chain_unit[c] + 1,
              "kind %d wide chain %d", kind, c);
        const Segment& sg = pr.seg[pr.chain_seg[c]];
        const int u = pr.units[pr.chain_unit[c]];
        CHECK(sg.n_load < 0 && sg.op_begin >= 0 && sg.op_begin < (int)pr.wide.unit.size() &&
                  pr.wide.unit[sg.op_begin] == u,
              "kind %d wide segment of unit %d", kind, u);
        CHECK(unit_need(s, kind, u) > pr.level_wide_at[lv], "kind %d unit %d is not wide", kind, u);
        if (kind < 0)
          for (int q = s.csc_colptr[u]; q < s.csc_colptr[u + 1]; q++) owned[q]++;
        continue;
      }
      for (int k = pr.chain_unit[c]; k < pr.chain_unit[c + 1]; k++)
        CHECK(unit_need(s, kind, pr.units[k]) <= pr.level_wide_at[lv], "kind %d unit %d too wide", kind,
              pr.units[k]);
      int prev_nl = -1;  // table rows of the previous segment of the chain (-1: none)
      for (int g = pr.chain_seg[c]; g < pr.chain_seg[c + 1]; g++) {
        const Segment& sg = pr.seg[g];
        CHECK(sg.n_load > 0, "kind %d segment %d of a program level is WIDE", kind, g);
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
          // A refactorization's own rows are the slots' first use: never
          // carried (the one-pass scatter reads them from A).
          CHECK(kind >= 0 || to >= sg.n_own, "kind %d segment %d carries an own row", kind, g);
          for (int j = 0; j < k; j++)
            CHECK((sg.carry[j] & 0xffff) != to, "kind %d segment %d duplicate carry", kind, g);
        }
        for (int l = 0; l < sg.n_load; l++) {
          const int r = pr.loads[sg.load_begin + l];
          if (kind < 0) {
            CHECK(r >= 0 && r < s.nnz_lu, "kind %d load %d", kind, r);
            if (l < sg.n_own) owned[r]++;
            else CHECK(owned[r] == 1, "kind %d slot %d read before its own segment", kind, r);
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
  for (int q = 0; q < (int)owned.size(); q++)
    CHECK(owned[q] == 1, "kind %d slot %d is an own row %d times", kind, q, owned[q]);
  // Wide refactor plans: targets inside their column, pairs in ascending j,
  // every U source of a target computed at an earlier chain level or earlier
  // in the target's own chain (and marked so), long targets alone in their
  // chain, every update of the column present once.
  if (kind == -1) {
    const WidePlan& w = pr.wide;
    CHECK(w.lvl.size() == w.unit.size() + 1, "wide lvl size");
    CHECK(w.tg_rec.size() % 4 == 0 && w.pr_q.size() == w.pr_p.size(), "wide plan sizes");
    int next_pair = 0;
    for (size_t i = 0; i < w.unit.size(); i++) {
      const int k = w.unit[i];
      const int c0 = s.csc_colptr[k], dk = s.diag_slot[k], c1 = s.csc_colptr[k + 1];
      std::vector<int> level_of(c1 - c0, 0), chain_of(c1 - c0, -1);
      int64_t updates = 0, expect = 0;
      for (int p = c0; p < dk; p++) {
        const int j = s.csc_row[p];
        expect += s.csc_colptr[j + 1] - s.diag_slot[j] - 1;
      }
      for (int l = w.lvl[i]; l < w.lvl[i + 1]; l++)
        for (int c = w.lv_chain[l]; c < w.lv_chain[l + 1]; c++)
          for (int t = w.ch_tgt[c]; t < w.ch_tgt[c + 1]; t++) {
            const int* rec = &w.tg_rec[4 * t];
            const int slot = rec[0], np = rec[2];
            CHECK(slot >= c0 && slot < c1 && level_of[slot - c0] == 0, "wide target %d", slot);
            CHECK(np > 0, "wide target %d without pairs", slot);
            CHECK(np <= kWideLong || w.ch_tgt[c + 1] - w.ch_tgt[c] == 1,
                  "long wide target %d shares its chain", slot);
            // The pairs of consecutive targets are consecutive.
            const int e0 = np == 1 ? next_pair : rec[1];
            CHECK(e0 == next_pair, "wide target %d pair index", slot);
            next_pair = e0 + np;
            if (np == 1)
              CHECK(rec[1] == w.pr_p[e0] && rec[3] == w.pr_q[e0], "wide record %d", slot);
            else
              CHECK(rec[3] == -1, "wide record %d", slot);
            int prev_p = -1;
            for (int e = e0; e < e0 + np; e++) {
              const int q = w.pr_q[e];
              const bool same = w.pr_p[e] < 0;
              const int p = same ? ~w.pr_p[e] : w.pr_p[e];
              CHECK(p >= c0 && p < dk && p > prev_p, "wide pair order %d", p);
              if (same)
                CHECK(chain_of[p - c0] == c && level_of[p - c0] == l - w.lvl[i] + 1,
                      "wide same-chain source %d", p);
              else
                CHECK(level_of[p - c0] <= l - w.lvl[i] && chain_of[p - c0] != c,
                      "wide pair level %d", p);
              const int j = s.csc_row[p];
              CHECK(q > s.diag_slot[j] && q < s.csc_colptr[j + 1] &&
                        s.csc_row[q] == s.csc_row[slot],
                    "wide pair slot %d", q);
              prev_p = p;
              updates++;
            }
            level_of[slot - c0] = l - w.lvl[i] + 1;
            chain_of[slot - c0] = c;
          }
      CHECK(updates == expect, "wide column %d updates %lld of %lld", k, (long long)updates,
            (long long)expect);
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
    for (int base : {8, 16, 24, 40, 64, 1023}) {
      for (int merge = 0; merge <= 2; merge++) {
        ProgramOptions opt;
        opt.max_locals = base;
        opt.merge = merge;
        check_program(s, kind, opt);
        // The handle's rule: narrow levels get a wide budget.
        opt.wide_locals = 226;
        opt.narrow_chains = 64;
        check_program(s, kind, opt);
        // Units over half the table run as wide units.
        opt.wide_threshold = base / 2;
        check_program(s, kind, opt);
      }
    }
  }
  std::printf("%s n=%d nnz_lu=%lld\n", fails ? "FAILED" : "ok", s.n, (long long)s.nnz_lu);
  return fails ? 1 : 0;
}
