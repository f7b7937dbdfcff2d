// Chain program compiler (see programs.hpp).
#include "programs.hpp"

#include <algorithm>

namespace pvglu {

namespace {

struct RawOp {
  int code, a, b, c, col;
};

// Local table under construction for one segment.
struct Table {
  std::vector<int> loc_of_x, loc_of_v;  // -1 when absent
  std::vector<int> used_x, used_v;      // for resetting
  std::vector<int> refs;
  std::vector<char> own;
  std::vector<RawOp> ops;
  std::vector<int> units;               // units computed in this segment
  void init(int n, int64_t nnz) {
    loc_of_x.assign(n, -1);
    loc_of_v.assign(nnz, -1);
  }
  int size() const { return (int)refs.size(); }
  void reset() {
    for (int i : used_x) loc_of_x[i] = -1;
    for (int q : used_v) loc_of_v[q] = -1;
    used_x.clear();
    used_v.clear();
    refs.clear();
    own.clear();
    ops.clear();
    units.clear();
  }
  int add(int ref, bool is_own) {
    refs.push_back(ref);
    own.push_back(is_own ? 1 : 0);
    return size() - 1;
  }
  // Refactor tables hold LU slots only (ref = slot).
  int slot_refactor(int q, bool is_own) {
    if (loc_of_v[q] < 0) {
      loc_of_v[q] = add(q, is_own);
      used_v.push_back(q);
    }
    return loc_of_v[q];
  }
  // Solve tables: x entries (ref = i) and read-only slots (ref = -(q + 1)).
  int x(int i, bool is_own) {
    if (loc_of_x[i] < 0) {
      loc_of_x[i] = add(i, is_own);
      used_x.push_back(i);
    }
    return loc_of_x[i];
  }
  int v(int q) {
    if (loc_of_v[q] < 0) {
      loc_of_v[q] = add(-(q + 1), false);
      used_v.push_back(q);
    }
    return loc_of_v[q];
  }
};

const LevelSet& level_set(const Symbolic& s, int kind) {
  switch (kind) {
    case 0: return s.l;
    case 1: return s.u;
    case 3: return s.lt;
    default: return s.lu;
  }
}

// Number of values a unit needs that are not yet in the table.
int new_locals(const Symbolic& s, int kind, int u, const Table& t) {
  int cnt = 0;
  std::vector<int> seen_x, seen_v;
  auto need_x = [&](int i) {
    if (t.loc_of_x[i] < 0 && std::find(seen_x.begin(), seen_x.end(), i) == seen_x.end()) {
      seen_x.push_back(i);
      cnt++;
    }
  };
  auto need_v = [&](int q) {
    if (t.loc_of_v[q] < 0 && std::find(seen_v.begin(), seen_v.end(), q) == seen_v.end()) {
      seen_v.push_back(q);
      cnt++;
    }
  };
  if (kind == -1) {
    const int c0 = s.csc_colptr[u], dk = s.diag_slot[u], c1 = s.csc_colptr[u + 1];
    for (int q = c0; q < c1; q++) need_v(q);
    for (int p = c0; p < dk; p++) {
      const int j = s.csc_row[p];
      for (int q = s.diag_slot[j] + 1; q < s.csc_colptr[j + 1]; q++) need_v(q);
    }
  } else if (kind == 0 || kind == 1) {
    need_x(u);
    const auto& ptr = kind == 0 ? s.lrow_ptr : s.urow_ptr;
    const auto& slot = kind == 0 ? s.lrow_slot : s.urow_slot;
    const auto& col = kind == 0 ? s.lrow_col : s.urow_col;
    for (int e = ptr[u]; e < ptr[u + 1]; e++) {
      need_x(col[e]);
      need_v(slot[e]);
    }
    if (kind == 1) need_v(s.diag_slot[u]);
  } else {
    need_x(u);
    const int b = kind == 2 ? s.csc_colptr[u] : s.diag_slot[u] + 1;
    const int e = kind == 2 ? s.diag_slot[u] : s.csc_colptr[u + 1];
    for (int q = b; q < e; q++) {
      need_x(s.csc_row[q]);
      need_v(q);
    }
    if (kind == 2) need_v(s.diag_slot[u]);
  }
  return cnt;
}

void emit_unit(const Symbolic& s, int kind, int u, Table& t) {
  if (kind == -1) {
    const int c0 = s.csc_colptr[u], dk = s.diag_slot[u], c1 = s.csc_colptr[u + 1];
    for (int q = c0; q < c1; q++) t.slot_refactor(q, true);  // own slots, CSC order
    for (int p = c0; p < dk; p++) {
      const int j = s.csc_row[p];
      const int q0 = s.diag_slot[j] + 1;
      const int up = t.loc_of_v[p];
      for (int q = q0; q < s.csc_colptr[j + 1]; q++) {
        const int tgt = s.upd_tgt[s.upd_ptr[p] + (q - q0)];
        const int lq = t.slot_refactor(q, false);
        t.ops.push_back(RawOp{OP_FNMA, t.loc_of_v[tgt], lq, up, -1});
      }
    }
    // The L slots of column u are consecutive own locals (added in CSC order).
    const int cnt = c1 - dk - 1;
    t.ops.push_back(RawOp{OP_SCALE, t.loc_of_v[dk], cnt > 0 ? t.loc_of_v[dk + 1] : 0, cnt, u});
  } else if (kind == 0 || kind == 1) {
    const int xi = t.x(u, true);
    const auto& ptr = kind == 0 ? s.lrow_ptr : s.urow_ptr;
    const auto& slot = kind == 0 ? s.lrow_slot : s.urow_slot;
    const auto& col = kind == 0 ? s.lrow_col : s.urow_col;
    // L rows take their updates in ascending column order, U rows in
    // descending order: the order in which the reference's column sweeps
    // deliver them (GLU_CSC_CPU_Triangular.cpp:27-43).
    const int n_e = ptr[u + 1] - ptr[u];
    for (int k = 0; k < n_e; k++) {
      const int e = kind == 0 ? ptr[u] + k : ptr[u + 1] - 1 - k;
      const int xj = t.x(col[e], false);
      const int vq = t.v(slot[e]);
      t.ops.push_back(RawOp{OP_FNMA, xi, vq, xj, -1});
    }
    if (kind == 1) t.ops.push_back(RawOp{OP_DIV, xi, t.v(s.diag_slot[u]), 0, -1});
  } else {
    const int xj = t.x(u, true);
    const int b = kind == 2 ? s.csc_colptr[u] : s.diag_slot[u] + 1;
    const int e = kind == 2 ? s.diag_slot[u] : s.csc_colptr[u + 1];
    for (int q = b; q < e; q++) {
      const int xi = t.x(s.csc_row[q], false);
      const int vq = t.v(q);
      t.ops.push_back(RawOp{OP_FNMA, xj, vq, xi, -1});
    }
    if (kind == 2) t.ops.push_back(RawOp{OP_DIV, xj, t.v(s.diag_slot[u]), 0, -1});
  }
  t.units.push_back(u);
}

}  // namespace

const LevelSet& program_levels(const Symbolic& s, int kind) { return level_set(s, kind); }

void unit_deps(const Symbolic& s, int kind, int u, std::vector<int>& deps) {
  deps.clear();
  if (kind == -1 || kind == 2) {  // rows of column u's U part
    for (int p = s.csc_colptr[u]; p < s.diag_slot[u]; p++) deps.push_back(s.csc_row[p]);
  } else if (kind == 0) {
    for (int e = s.lrow_ptr[u]; e < s.lrow_ptr[u + 1]; e++) deps.push_back(s.lrow_col[e]);
  } else if (kind == 1) {
    for (int e = s.urow_ptr[u]; e < s.urow_ptr[u + 1]; e++) deps.push_back(s.urow_col[e]);
  } else {  // rows of column u's L part
    for (int q = s.diag_slot[u] + 1; q < s.csc_colptr[u + 1]; q++) deps.push_back(s.csc_row[q]);
  }
}

void build_chain_program(const Symbolic& s, int kind, int max_locals, ChainProgram& out) {
  ProgramOptions opt;
  opt.max_locals = max_locals;
  build_chain_program(s, kind, opt, out);
}

namespace {

// Chain-scheduled gather plan of wide refactor unit k (WidePlan).
void plan_wide_column(const Symbolic& s, int k, WidePlan& w) {
  const int c0 = s.csc_colptr[k], dk = s.diag_slot[k], c1 = s.csc_colptr[k + 1];
  const int len = c1 - c0;
  std::vector<std::vector<std::pair<int, int>>> pairs(len);  // target -> (q, p)
  for (int p = c0; p < dk; p++) {  // ascending j
    const int j = s.csc_row[p];
    const int q0 = s.diag_slot[j] + 1, q1 = s.csc_colptr[j + 1];
    for (int q = q0; q < q1; q++) {
      const int t = s.upd_tgt[s.upd_ptr[p] + (q - q0)];
      pairs[t - c0].push_back({q, p});
    }
  }
  // Chains and chain levels (programs.hpp); a target's U sources precede it
  // in slot order, so slot order is a topological order.
  std::vector<int> clev(len, -1), chain_of(len, -1);
  std::vector<int> tail;                 // per chain: its last target
  std::vector<char> whole;               // per chain: a long target's own chain
  std::vector<std::vector<int>> members;  // per chain: its targets
  std::vector<std::vector<int>> level_chains;
  for (int t = 0; t < len; t++) {
    if (pairs[t].empty()) continue;
    const bool lng = (int)pairs[t].size() > kWideLong;
    int m = -1;
    for (const auto& qp : pairs[t]) m = std::max(m, clev[qp.second - c0]);
    int c = -1;
    bool one_chain = true, has_tail = false;
    for (const auto& qp : pairs[t]) {
      const int d = qp.second - c0;
      if (clev[d] < 0 || clev[d] != m) continue;
      if (c < 0) c = chain_of[d];
      else if (chain_of[d] != c) one_chain = false;
      if (tail[chain_of[d]] == d) has_tail = true;
    }
    if (!lng && m >= 0 && one_chain && has_tail && !whole[c]) {
      members[c].push_back(t);
      tail[c] = t;
      chain_of[t] = c;
      clev[t] = m;
      continue;
    }
    const int lv = m + 1;
    if ((int)level_chains.size() <= lv) level_chains.resize(lv + 1);
    chain_of[t] = (int)members.size();
    level_chains[lv].push_back((int)members.size());
    members.push_back({t});
    tail.push_back(t);
    whole.push_back(lng ? 1 : 0);
    clev[t] = lv;
  }
  w.lvl.push_back((int)w.lv_chain.size());
  for (auto& chains : level_chains) {
    // Longest chains first: the warps that take them start first.
    std::stable_sort(chains.begin(), chains.end(), [&](int a, int b) {
      return members[a].size() > members[b].size();
    });
    w.lv_chain.push_back((int)w.ch_tgt.size());
    for (const int c : chains) {
      w.ch_tgt.push_back(w.targets());
      for (const int t : members[c]) {
        const int e0 = (int)w.pr_q.size();
        for (const auto& qp : pairs[t]) {
          w.pr_q.push_back(qp.first);
          const int d = qp.second - c0;
          w.pr_p.push_back(clev[d] >= 0 && chain_of[d] == c ? ~qp.second : qp.second);
        }
        const int np = (int)pairs[t].size();
        w.tg_rec.insert(w.tg_rec.end(), {c0 + t, np == 1 ? w.pr_p[e0] : e0, np,
                                         np == 1 ? w.pr_q[e0] : -1});
      }
    }
  }
}

}  // namespace

namespace {

// Execution levels (see programs.hpp): every unit extends the chain that
// holds all of its dependencies of the highest level, when one of them is
// among the chain's last `1 + slack` units, and starts a new chain one level
// above them otherwise.  With slack 0 extending never delays a unit (it had
// to wait for that last unit anyway) and never makes another chain wait;
// slack 1 lets a unit also wait for one unit it does not depend on, which
// keeps two-unit rungs of a ladder (each rung's first unit depending on the
// previous rung's first unit) in one chain.
void execution_levels(const Symbolic& s, int kind, const LevelSet& ls, int slack,
                      std::vector<std::vector<std::vector<int>>>& exec) {
  std::vector<int> lvl(s.n, -1), chain_of(s.n, -1), pos(s.n, -1), deps;
  std::vector<int> len, chain_pos;  // per chain (global numbers)
  for (int k = 0; k < (int)ls.columns.size(); k++) {
    const int u = ls.columns[k];
    unit_deps(s, kind, u, deps);
    int m = -1;
    for (const int d : deps) m = std::max(m, lvl[d]);
    int c = -1;
    bool one_chain = true, near_tail = false;
    for (const int d : deps) {
      if (lvl[d] != m) continue;
      if (c < 0) c = chain_of[d];
      else if (chain_of[d] != c) one_chain = false;
      if (pos[d] >= len[chain_of[d]] - 1 - slack) near_tail = true;
    }
    if (m >= 0 && one_chain && near_tail) {
      exec[m][chain_pos[c]].push_back(u);
      chain_of[u] = c;
      pos[u] = len[c]++;
      lvl[u] = m;
      continue;
    }
    const int lv = m + 1;
    if ((int)exec.size() <= lv) exec.resize(lv + 1);
    chain_of[u] = (int)len.size();
    pos[u] = 0;
    len.push_back(1);
    chain_pos.push_back((int)exec[lv].size());
    exec[lv].push_back(std::vector<int>{u});
    lvl[u] = lv;
  }
}

}  // namespace

int execution_level_count(const Symbolic& s, int kind, int merge) {
  const LevelSet& ls = level_set(s, kind);
  if (merge <= 0) return ls.num_levels();
  std::vector<std::vector<std::vector<int>>> exec;
  execution_levels(s, kind, ls, merge - 1, exec);
  return (int)exec.size();
}

void build_chain_program(const Symbolic& s, int kind, const ProgramOptions& opt,
                         ChainProgram& out) {
  out = ChainProgram();
  out.kind = kind;
  const LevelSet& ls = level_set(s, kind);
  Table t;
  t.init(s.n, s.nnz_lu);

  // 0. Execution levels (levels -> chains -> units).
  std::vector<std::vector<std::vector<int>>> exec;
  if (opt.merge <= 0) {
    for (int lv = 0; lv < ls.num_levels(); lv++) {
      exec.emplace_back();
      for (int c = ls.start_levels[lv]; c < ls.start_levels[lv + 1]; c++)
        exec.back().emplace_back(ls.columns.begin() + ls.start_chains[c],
                                 ls.columns.begin() + ls.start_chains[c + 1]);
    }
  } else {
    execution_levels(s, kind, ls, opt.merge - 1, exec);
  }

  // 1. Program levels: each execution level cut around its wide units.
  struct PLevel {
    int src;
    bool wide;
    int budget, wide_at;
    std::vector<std::vector<int>> chains;
  };
  std::vector<PLevel> plv;
  for (int lv = 0; lv < (int)exec.size(); lv++) {
    const bool narrow = (int)exec[lv].size() <= opt.narrow_chains;
    const int budget =
        std::min(narrow ? std::max(opt.max_locals, opt.wide_locals) : opt.max_locals, kMaxLocals);
    const int wide_at = opt.wide_threshold > 0 ? std::min(budget, opt.wide_threshold) : budget;
    std::vector<std::vector<std::vector<int>>> phase;  // phase -> chains -> units
    auto put = [&](int ph, std::vector<int>&& chain) {
      if ((int)phase.size() <= ph) phase.resize(ph + 1);
      phase[ph].push_back(std::move(chain));
    };
    for (const auto& chain : exec[lv]) {
      int ph = 0;
      std::vector<int> cur;
      for (const int u : chain) {
        if (new_locals(s, kind, u, t) > wide_at) {
          if (ph % 2 == 0) {
            if (!cur.empty()) put(ph, std::move(cur));
            cur.clear();
            ph += 1;
          } else {
            ph += 2;  // a wide unit after a wide unit of the same chain
          }
          put(ph, std::vector<int>{u});
        } else {
          if (ph % 2 == 1) ph += 1;
          cur.push_back(u);
        }
      }
      if (!cur.empty()) put(ph, std::move(cur));
    }
    for (int ph = 0; ph < (int)phase.size(); ph++)
      if (!phase[ph].empty())
        plv.push_back(PLevel{lv, ph % 2 == 1, budget, wide_at, std::move(phase[ph])});
  }

  // 2. Emit the program levels.
  std::vector<int> remap;
  // Entries written by the segments of the current chain so far (by ref).
  std::vector<char> written_x(s.n, 0), written_v(s.nnz_lu, 0);
  std::vector<int> written_list;
  auto written = [&](int ref) -> char& {
    return (kind >= 0 && ref >= 0) ? written_x[ref] : written_v[kind < 0 ? ref : -ref - 1];
  };
  // Final table layout of the previous segment of the current chain
  // (ref -> local), for carries.  Empty at a chain start.
  std::vector<std::pair<int, int>> prev_layout;
  auto close = [&]() {
    if (t.units.empty()) return;
    // Own entries first (in load order), then the read-only ones.
    const int nl = t.size();
    remap.assign(nl, -1);
    Segment g;
    g.load_begin = (int)out.loads.size();
    g.n_load = nl;
    g.n_own = 0;
    g.reads_own_chain = 0;
    for (int l = 0; l < nl; l++)
      if (t.own[l]) {
        remap[l] = g.n_own++;
        out.loads.push_back(t.refs[l]);
      }
    int next = g.n_own;
    for (int l = 0; l < nl; l++)
      if (!t.own[l]) {
        remap[l] = next++;
        out.loads.push_back(t.refs[l]);
      }
    // Carries: entries the previous segment's table holds (its final values).
    std::vector<char> carried(nl, 0);
    for (int l = 0; l < nl && g.n_carry < kMaxCarry; l++)
      for (const auto& pl : prev_layout)
        if (pl.first == t.refs[l]) {
          g.carry[g.n_carry++] = (pl.second << 16) | remap[l];
          carried[l] = 1;
          break;
        }
    for (int l = 0; l < nl; l++)
      if (!t.own[l] && !carried[l] && written(t.refs[l])) g.reads_own_chain = 1;
    for (int l = 0; l < nl; l++)
      if (t.own[l] && !written(t.refs[l])) {
        written(t.refs[l]) = 1;
        written_list.push_back(t.refs[l]);
      }
    prev_layout.clear();
    for (int l = 0; l < nl; l++) prev_layout.push_back({t.refs[l], remap[l]});
    g.op_begin = (int)out.ops.size();
    for (const RawOp& o : t.ops) {
      const int a = remap[o.a];
      const int b = (o.code == OP_SCALE && o.c == 0) ? 0 : remap[o.b];
      const int c = (o.code == OP_FNMA) ? remap[o.c] : o.c;
      out.ops.push_back(pack_op(o.code, a, b, c));
      out.op_col.push_back(o.col);
    }
    while ((out.ops.size() - g.op_begin) % 4) {
      out.ops.push_back(pack_op(OP_NOP, 0, 0, 0));
      out.op_col.push_back(-1);
    }
    g.n_op = (int)out.ops.size() - g.op_begin;
    out.seg.push_back(g);
    t.reset();
  };
  for (const PLevel& L : plv) {
    out.level_chain.push_back((int)out.chain_seg.size());
    out.level_src.push_back(L.src);
    out.level_budget.push_back(L.budget);
    out.level_wide_at.push_back(L.wide_at);
    out.level_wide.push_back(L.wide ? 1 : 0);
    out.level_max_locals.push_back(L.wide ? 1 : std::min(L.budget, kMaxLocals));
    if (L.wide) out.wide_levels++;
    for (const auto& chain : L.chains) {
      out.chain_seg.push_back((int)out.seg.size());
      out.chain_unit.push_back((int)out.units.size());
      out.units.insert(out.units.end(), chain.begin(), chain.end());
      if (L.wide) {
        const int u = chain[0];
        Segment g{0, -1, 0, (int)out.wide.unit.size(), 0};
        out.seg.push_back(g);
        out.wide.unit.push_back(u);
        if (kind < 0) plan_wide_column(s, u, out.wide);
        out.wide_units++;
        continue;
      }
      for (int r : written_list) written(r) = 0;
      written_list.clear();
      prev_layout.clear();
      const int first_seg = (int)out.seg.size();
      for (const int u : chain) {
        int need = new_locals(s, kind, u, t);
        if (t.size() + need > L.budget && !t.units.empty()) close();
        emit_unit(s, kind, u, t);
      }
      close();
      out.longest_chain_segments =
          std::max(out.longest_chain_segments, (int)out.seg.size() - first_seg);
    }
  }
  out.level_chain.push_back((int)out.chain_seg.size());
  out.chain_seg.push_back((int)out.seg.size());
  out.chain_unit.push_back((int)out.units.size());
  if (kind < 0) out.wide.lvl.push_back((int)out.wide.lv_chain.size());
  out.wide.lv_chain.push_back((int)out.wide.ch_tgt.size());
  out.wide.ch_tgt.push_back(out.wide.targets());
  // A level's table is as wide as its widest segment (the budget is only an
  // upper bound): shared memory per block, and so the blocks an SM holds,
  // follow what the level uses.  The narrow levels of a plant (one segment
  // per inverter chain) need a small part of the wide budget they are given.
  out.max_locals = 1;
  for (size_t lv = 0; lv + 1 < out.level_chain.size(); lv++) {
    int used = 1;
    if (!out.level_wide[lv])
      for (int c = out.level_chain[lv]; c < out.level_chain[lv + 1]; c++)
        for (int g = out.chain_seg[c]; g < out.chain_seg[c + 1]; g++)
          used = std::max(used, out.seg[g].n_load);
    out.level_max_locals[lv] = used;
    out.max_locals = std::max(out.max_locals, used);
  }
}

}  // namespace pvglu
