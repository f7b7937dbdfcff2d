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

void build_chain_program(const Symbolic& s, int kind, int max_locals, ChainProgram& out) {
  build_chain_program(s, kind, std::vector<int>(level_set(s, kind).num_levels(), max_locals),
                      out);
}

void build_chain_program(const Symbolic& s, int kind, const std::vector<int>& level_max_locals,
                         ChainProgram& out) {
  out = ChainProgram();
  out.kind = kind;
  const LevelSet& ls = level_set(s, kind);
  out.level_chain = ls.start_levels;
  out.level_max_locals.resize(ls.num_levels());
  for (int lv = 0; lv < ls.num_levels(); lv++) {
    out.level_max_locals[lv] = std::min(level_max_locals[lv], kMaxLocals);
    out.max_locals = std::max(out.max_locals, out.level_max_locals[lv]);
  }
  int level = 0, max_locals = ls.num_levels() ? out.level_max_locals[0] : kMaxLocals;
  Table t;
  t.init(s.n, s.nnz_lu);
  std::vector<int> remap;
  // Entries written by the segments of the current chain so far (by ref).
  std::vector<char> written_x(s.n, 0), written_v(s.nnz_lu, 0);
  std::vector<int> written_list;
  auto written = [&](int ref) -> char& {
    return (kind >= 0 && ref >= 0) ? written_x[ref] : written_v[kind < 0 ? ref : -ref - 1];
  };
  // Final table layout of the previous segment of the current chain
  // (ref -> local), for carries.  Empty at a chain start and after DIRECT.
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
  for (int c = 0; c < ls.num_chains(); c++) {
    while (level + 1 < ls.num_levels() && c >= ls.start_levels[level + 1]) level++;
    max_locals = out.level_max_locals.empty() ? kMaxLocals : out.level_max_locals[level];
    for (int r : written_list) written(r) = 0;
    written_list.clear();
    prev_layout.clear();
    out.chain_seg.push_back((int)out.seg.size());
    const int first_seg = (int)out.seg.size();
    for (int k = ls.start_chains[c]; k < ls.start_chains[c + 1]; k++) {
      const int u = ls.columns[k];
      int need = new_locals(s, kind, u, t);
      if (t.size() + need > max_locals && !t.units.empty()) {
        close();
        need = new_locals(s, kind, u, t);
      }
      if (need > max_locals) {
        // Too wide for the local table: executed from global memory, after
        // the segment collected so far (chain order is execution order).
        close();
        out.seg.push_back(Segment{0, -1, 0, u, 0, 1});
        prev_layout.clear();  // the DIRECT unit updates rows in global memory
        // A DIRECT unit writes its own entries through global memory.
        const int own_ref = kind < 0 ? -1 : u;
        if (own_ref >= 0 && !written(own_ref)) {
          written(own_ref) = 1;
          written_list.push_back(own_ref);
        }
        if (kind < 0)
          for (int q = s.csc_colptr[u]; q < s.csc_colptr[u + 1]; q++)
            if (!written(q)) {
              written(q) = 1;
              written_list.push_back(q);
            }
        out.direct_segments++;
        continue;
      }
      emit_unit(s, kind, u, t);
    }
    close();
    out.longest_chain_segments =
        std::max(out.longest_chain_segments, (int)out.seg.size() - first_seg);
  }
  out.chain_seg.push_back((int)out.seg.size());
  // A level's table is as wide as its widest segment (the budget is only an
  // upper bound): shared memory per block, and so the blocks an SM holds,
  // follow what the level uses.  The narrow levels of a plant (one segment
  // per inverter chain) need a small part of the wide budget they are given.
  out.max_locals = 1;
  for (int lv = 0; lv < ls.num_levels(); lv++) {
    int used = 1;
    for (int c = ls.start_levels[lv]; c < ls.start_levels[lv + 1]; c++)
      for (int g = out.chain_seg[c]; g < out.chain_seg[c + 1]; g++)
        used = std::max(used, out.seg[g].n_load);
    out.level_max_locals[lv] = used;
    out.max_locals = std::max(out.max_locals, used);
  }
}

}  // namespace pvglu
