// Host symbolic analysis (see symbolic.hpp for the step -> reference map).
#include "symbolic.hpp"

#include <algorithm>
#include <cstring>
#include <queue>
#include <set>
#include <utility>

namespace pvglu {

namespace {

bool validate_pattern(int n, const int* rowptr, const int* colidx,
                      std::vector<int>& rp, std::vector<int>& ci,
                      std::string& err) {
  if (n <= 0 || !rowptr || !colidx) {
    err = "n must be positive and the pattern pointers non-null";
    return false;
  }
  if (rowptr[0] != 0) {
    err = "rowptr[0] must be 0";
    return false;
  }
  for (int i = 0; i < n; i++)
    if (rowptr[i + 1] < rowptr[i]) {
      err = "rowptr must be non-decreasing";
      return false;
    }
  const int64_t nnz = rowptr[n];
  rp.assign(rowptr, rowptr + n + 1);
  ci.assign(colidx, colidx + nnz);
  for (int i = 0; i < n; i++) {
    auto b = ci.begin() + rp[i], e = ci.begin() + rp[i + 1];
    std::sort(b, e);
    for (auto it = b; it != e; ++it) {
      if (*it < 0 || *it >= n) {
        err = "column index out of range in row " + std::to_string(i);
        return false;
      }
      if (it != b && *it == *(it - 1)) {
        err = "duplicate entry in row " + std::to_string(i);
        return false;
      }
    }
  }
  return true;
}

// Sorted-vector helpers for the row/column sets of 004b.
inline bool sorted_contains(const std::vector<int>& v, int x) {
  return std::binary_search(v.begin(), v.end(), x);
}

inline void sorted_replace(std::vector<int>& v, int from, int to) {
  auto it = std::lower_bound(v.begin(), v.end(), from);
  if (it == v.end() || *it != from) return;
  v.erase(it);
  v.insert(std::lower_bound(v.begin(), v.end(), to), to);
}

// 004b_remove_zeros_diagonal.cpp:12-100 with move_only_rows = true.
// rows[r] is the sorted column set of row r, cols[c] the sorted row set of
// column c.  q is the row-exchange permutation (initially the identity).
bool remove_zeros_diagonal_rows(std::vector<std::vector<int>>& rows,
                                std::vector<std::vector<int>>& cols,
                                std::vector<int>& q, int& swaps,
                                std::string& err) {
  const int n = (int)rows.size();
  swaps = 0;
  for (int r = 0; r < n; r++) {
    if (sorted_contains(rows[r], r)) continue;
    // Fill at (r, r) needs some k < r with M(r,k) != 0 and M(k,r) != 0
    // (004b:42-64; the reference's two ordered scans test exactly this).
    bool would_fill = false;
    for (int k : rows[r]) {
      if (k >= r) break;
      if (sorted_contains(cols[r], k)) {
        would_fill = true;
        break;
      }
    }
    if (would_fill) continue;
    // First row after r holding an entry in column r (004b:70-80).
    auto it = std::upper_bound(cols[r].begin(), cols[r].end(), r);
    if (it == cols[r].end()) {
      err = "structurally zero diagonal at row " + std::to_string(r) +
            " with no later row to exchange (reference 004b:82)";
      return false;
    }
    const int ri = *it;
    // Exchange rows r and ri: every column touched by either row swaps the
    // two row ids in its row set (004c:53-89, rows only).
    std::vector<int> touched;
    touched.reserve(rows[r].size() + rows[ri].size());
    std::set_union(rows[r].begin(), rows[r].end(), rows[ri].begin(),
                   rows[ri].end(), std::back_inserter(touched));
    for (int c : touched) {
      const bool has_r = sorted_contains(cols[c], r);
      const bool has_ri = sorted_contains(cols[c], ri);
      if (has_r && !has_ri) sorted_replace(cols[c], r, ri);
      else if (!has_r && has_ri) sorted_replace(cols[c], ri, r);
    }
    std::swap(rows[r], rows[ri]);
    std::swap(q[r], q[ri]);
    swaps++;
  }
  return true;
}

// Filled pattern of M: the closure "M(i,k) != 0, M(k,j) != 0, k < i, k < j
// => (i,j) filled" that the fixpoint of 005a_obtain_fillin_matrix_CUDA.cu
// (:84-203, rule at check_possible_new_nonzeros_CUDA.h:51-210) converges to.
// Computed row by row (up-looking): row i merges the strictly-upper part of
// every earlier row k it touches, in ascending k, including rows reached
// through fill created on the way.
void symbolic_fill(const std::vector<std::vector<int>>& rows,
                   std::vector<int>& fill_rowptr, std::vector<int>& fill_col) {
  const int n = (int)rows.size();
  std::vector<int> urow_ptr(n + 1, 0);  // strictly-upper part of finished rows
  std::vector<int> urow_col;
  std::vector<int> mark(n, -1);
  std::vector<int> row_buf;
  fill_rowptr.assign(n + 1, 0);
  fill_col.clear();
  std::priority_queue<int, std::vector<int>, std::greater<int>> lower;
  for (int i = 0; i < n; i++) {
    row_buf.clear();
    for (int c : rows[i]) {
      mark[c] = i;
      row_buf.push_back(c);
      if (c < i) lower.push(c);
    }
    while (!lower.empty()) {
      const int k = lower.top();
      lower.pop();
      for (int p = urow_ptr[k]; p < urow_ptr[k + 1]; p++) {
        const int j = urow_col[p];
        if (mark[j] == i) continue;
        mark[j] = i;
        row_buf.push_back(j);
        if (j < i) lower.push(j);
      }
    }
    std::sort(row_buf.begin(), row_buf.end());
    for (int c : row_buf) fill_col.push_back(c);
    fill_rowptr[i + 1] = (int)fill_col.size();
    urow_ptr[i + 1] = urow_ptr[i];
    for (int c : row_buf)
      if (c > i) {
        urow_col.push_back(c);
        urow_ptr[i + 1]++;
      }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// 007_convert_dependencies_in_levels.cpp restated.
//
// Basic levels (007:4-60): the reference sweeps the columns in ascending order
// and places a column once every dependency sits in an earlier sweep.  That
// places column i at 1 + max(level(dep)) (0 without deps), each basic level
// listing its columns in ascending order; computed here in one topological
// pass instead of repeated sweeps.
//
// Chains (007:62-210): basic level b > 0 is appended to the current custom
// level when each of its columns hooks to exactly one chain of that custom
// level (dependencies outside it ignored) and no two columns hook the same
// chain; otherwise it starts a new custom level with one chain per column.
void build_levels(const std::vector<std::vector<int>>& deps, LevelSet& out) {
  const int n = (int)deps.size();
  std::vector<int> level(n, -1);
  // Topological order (Kahn) over the dependency DAG.
  std::vector<int> indeg(n, 0), adj_ptr(n + 1, 0), adj;
  for (int i = 0; i < n; i++)
    for (int d : deps[i]) adj_ptr[d + 1]++;
  for (int i = 0; i < n; i++) adj_ptr[i + 1] += adj_ptr[i];
  adj.resize(adj_ptr[n]);
  {
    std::vector<int> fillp(adj_ptr.begin(), adj_ptr.end() - 1);
    for (int i = 0; i < n; i++)
      for (int d : deps[i]) adj[fillp[d]++] = i;
  }
  for (int i = 0; i < n; i++) indeg[i] = (int)deps[i].size();
  std::vector<int> stack;
  for (int i = 0; i < n; i++)
    if (indeg[i] == 0) {
      level[i] = 0;
      stack.push_back(i);
    }
  int num_basic = 0;
  while (!stack.empty()) {
    const int v = stack.back();
    stack.pop_back();
    num_basic = std::max(num_basic, level[v] + 1);
    for (int p = adj_ptr[v]; p < adj_ptr[v + 1]; p++) {
      const int w = adj[p];
      level[w] = std::max(level[w], level[v] + 1);
      if (--indeg[w] == 0) stack.push_back(w);
    }
  }
  std::vector<std::vector<int>> basic(num_basic);
  for (int i = 0; i < n; i++) basic[level[i]].push_back(i);  // ascending

  // Custom levels of chains.
  std::vector<std::vector<std::vector<int>>> custom;
  std::vector<int> pos(n, -1);            // chain of a column in current level
  std::vector<int> in_current;            // columns of the current custom level
  std::vector<int> hook, used_stamp;
  int stamp = 0;
  for (int b = 0; b < num_basic; b++) {
    const auto& lvl = basic[b];
    bool fuse = (b != 0);
    if (fuse) {
      hook.assign(lvl.size(), 0);
      const int nchains = (int)custom.back().size();
      if ((int)used_stamp.size() < nchains) used_stamp.resize(nchains, -1);
      stamp++;
      for (size_t idx = 0; idx < lvl.size() && fuse; idx++) {
        int found = -1;
        for (int d : deps[lvl[idx]]) {
          const int p = pos[d];
          if (p == -1 || p == found) continue;
          if (found != -1) {
            found = -2;
            break;
          }
          found = p;
        }
        if (found < 0) {
          fuse = false;
          break;
        }
        if (used_stamp[found] == stamp) {
          fuse = false;
          break;
        }
        used_stamp[found] = stamp;
        hook[idx] = found;
      }
    }
    if (fuse) {
      auto& chains = custom.back();
      for (size_t idx = 0; idx < lvl.size(); idx++) {
        chains[hook[idx]].push_back(lvl[idx]);
        pos[lvl[idx]] = hook[idx];
        in_current.push_back(lvl[idx]);
      }
    } else {
      for (int c : in_current) pos[c] = -1;
      in_current.clear();
      std::vector<std::vector<int>> chains(lvl.size());
      for (size_t idx = 0; idx < lvl.size(); idx++) {
        chains[idx].push_back(lvl[idx]);
        pos[lvl[idx]] = (int)idx;
        in_current.push_back(lvl[idx]);
      }
      custom.push_back(std::move(chains));
    }
  }

  // 008 flatten.
  out.start_levels.clear();
  out.start_chains.clear();
  out.columns.clear();
  for (const auto& lv : custom) {
    out.start_levels.push_back((int)out.start_chains.size());
    for (const auto& ch : lv) {
      out.start_chains.push_back((int)out.columns.size());
      for (int c : ch) out.columns.push_back(c);
    }
  }
  out.start_levels.push_back((int)out.start_chains.size());
  out.start_chains.push_back((int)out.columns.size());
}

// ---------------------------------------------------------------------------
// Minimum-degree ordering on the explicit elimination graph of A + A^T.
void minimum_degree_order(int n, const std::vector<int>& rowptr,
                          const std::vector<int>& colidx,
                          std::vector<int>& perm) {
  std::vector<std::vector<int>> adj(n);
  for (int i = 0; i < n; i++)
    for (int p = rowptr[i]; p < rowptr[i + 1]; p++) {
      const int j = colidx[p];
      if (j == i) continue;
      adj[i].push_back(j);
      adj[j].push_back(i);
    }
  for (auto& a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  std::set<std::pair<int, int>> pq;
  for (int i = 0; i < n; i++) pq.insert({(int)adj[i].size(), i});
  std::vector<char> done(n, 0);
  perm.clear();
  perm.reserve(n);
  std::vector<int> merged;
  while (!pq.empty()) {
    const int v = pq.begin()->second;
    pq.erase(pq.begin());
    done[v] = 1;
    perm.push_back(v);
    const std::vector<int> nb = adj[v];
    for (int w : nb) {
      pq.erase({(int)adj[w].size(), w});
      // adj[w] <- (adj[w] U nb) \ {v, w}
      merged.clear();
      std::set_union(adj[w].begin(), adj[w].end(), nb.begin(), nb.end(),
                     std::back_inserter(merged));
      adj[w].clear();
      for (int x : merged)
        if (x != v && x != w && !done[x]) adj[w].push_back(x);
      pq.insert({(int)adj[w].size(), w});
    }
    adj[v].clear();
    adj[v].shrink_to_fit();
  }
}

// ---------------------------------------------------------------------------
int build_symbolic(int n, const int* rowptr, const int* colidx, const int* perm,
                   const SymbolicOptions& opt, Symbolic& S, std::string& err) {
  S = Symbolic();
  if (!validate_pattern(n, rowptr, colidx, S.a_rowptr, S.a_colidx, err))
    return ERR_BAD_ARG;
  S.n = n;
  S.nnz_a = S.a_rowptr[n];

  // Ordering P (004a:35-42 semantics: P[k] = original index of pivot k).
  if (perm) {
    std::vector<char> seen(n, 0);
    for (int k = 0; k < n; k++) {
      if (perm[k] < 0 || perm[k] >= n || seen[perm[k]]) {
        err = "perm is not a permutation of 0..n-1";
        return ERR_BAD_ARG;
      }
      seen[perm[k]] = 1;
    }
    S.perm_amd.assign(perm, perm + n);
  } else {
    minimum_degree_order(n, S.a_rowptr, S.a_colidx, S.perm_amd);
  }
  std::vector<int> pinv(n);
  for (int k = 0; k < n; k++) pinv[S.perm_amd[k]] = k;

  // Symmetrically permuted pattern (Sparse_Matrix::interchange_row_columns,
  // sparse_matrix.h:117-134, applied with Pinv at 004a:44).
  std::vector<std::vector<int>> rows(n), cols(n);
  for (int i = 0; i < n; i++)
    for (int p = S.a_rowptr[i]; p < S.a_rowptr[i + 1]; p++) {
      const int r = pinv[i], c = pinv[S.a_colidx[p]];
      rows[r].push_back(c);
    }
  for (int r = 0; r < n; r++) {
    std::sort(rows[r].begin(), rows[r].end());
    for (int c : rows[r]) cols[c].push_back(r);
  }  // cols[] filled in ascending r -> already sorted

  S.perm_rows.resize(n);
  for (int i = 0; i < n; i++) S.perm_rows[i] = i;
  if (!remove_zeros_diagonal_rows(rows, cols, S.perm_rows, S.row_swaps, err))
    return ERR_STRUCTURAL;
  for (int i = 0; i < n; i++)
    if (S.perm_rows[S.perm_rows[i]] != i) S.perm_rows_is_involution = 0;
  S.row_orig.resize(n);
  S.col_orig.resize(n);
  for (int r = 0; r < n; r++) {
    S.row_orig[r] = S.perm_amd[S.perm_rows[r]];
    S.col_orig[r] = S.perm_amd[r];
  }

  // Fill (005).
  symbolic_fill(rows, S.fill_rowptr, S.fill_col);
  S.nnz_lu = S.fill_rowptr[n];
  for (int i = 0; i < n; i++) {
    if (!std::binary_search(S.fill_col.begin() + S.fill_rowptr[i],
                            S.fill_col.begin() + S.fill_rowptr[i + 1], i)) {
      err = "missing diagonal after fill at row " + std::to_string(i);
      return ERR_STRUCTURAL;
    }
  }

  // 010: CSR/CSC, cross maps, diagonal starts.
  const int64_t nnz = S.nnz_lu;
  if (nnz > (int64_t)0x7fffffff) {
    err = "filled pattern exceeds 2^31 entries";
    return ERR_TOO_LARGE;
  }
  S.csr_rowptr = S.fill_rowptr;
  S.csr_col = S.fill_col;
  S.csc_colptr.assign(n + 1, 0);
  for (int64_t p = 0; p < nnz; p++) S.csc_colptr[S.csr_col[p] + 1]++;
  for (int j = 0; j < n; j++) S.csc_colptr[j + 1] += S.csc_colptr[j];
  S.csc_row.resize(nnz);
  S.csc_to_csr.resize(nnz);
  S.csr_to_csc.resize(nnz);
  {
    std::vector<int> next(S.csc_colptr.begin(), S.csc_colptr.end() - 1);
    for (int i = 0; i < n; i++)
      for (int p = S.csr_rowptr[i]; p < S.csr_rowptr[i + 1]; p++) {
        const int j = S.csr_col[p];
        const int q = next[j]++;
        S.csc_row[q] = i;
        S.csc_to_csr[q] = p;
        S.csr_to_csc[p] = q;
      }
  }
  S.csr_diag_start.resize(n);
  S.csc_diag_start.resize(n);
  S.diag_slot.resize(n);
  for (int i = 0; i < n; i++) {
    int p = S.csr_rowptr[i];
    while (p < S.csr_rowptr[i + 1] && S.csr_col[p] <= i) p++;
    S.csr_diag_start[i] = p;
    int q = S.csc_colptr[i];
    while (q < S.csc_colptr[i + 1] && S.csc_row[q] <= i) q++;
    S.csc_diag_start[i] = q;
    S.diag_slot[i] = q - 1;
  }

  // 006: dependency sets, 007/008: levels.
  std::vector<std::vector<int>> deps(n);
  for (int k = 0; k < n; k++)  // GLU: {i < k : M(i,k) filled} (006:5-47)
    for (int q = S.csc_colptr[k]; q < S.csc_colptr[k + 1]; q++)
      if (S.csc_row[q] < k) deps[k].push_back(S.csc_row[q]);
  build_levels(deps, S.lu);
  for (int i = 0; i < n; i++) {  // L: {j < i : M(i,j)} (006:49-62)
    deps[i].clear();
    for (int p = S.csr_rowptr[i]; p < S.csr_rowptr[i + 1]; p++)
      if (S.csr_col[p] < i) deps[i].push_back(S.csr_col[p]);
  }
  build_levels(deps, S.l);
  for (int i = 0; i < n; i++) {  // U: {j > i : M(i,j)} (006:64-77)
    deps[i].clear();
    for (int p = S.csr_rowptr[i]; p < S.csr_rowptr[i + 1]; p++)
      if (S.csr_col[p] > i) deps[i].push_back(S.csr_col[p]);
  }
  build_levels(deps, S.u);
  if (opt.compute_transposed_levels) {
    for (int j = 0; j < n; j++) {  // L^T: {i > j : M(i,j)}
      deps[j].clear();
      for (int q = S.csc_colptr[j]; q < S.csc_colptr[j + 1]; q++)
        if (S.csc_row[q] > j) deps[j].push_back(S.csc_row[q]);
    }
    build_levels(deps, S.lt);
  }

  // 009: per LU level, the longest filled ROW among its columns.
  S.max_elements_per_column.clear();
  for (int lv = 0; lv < S.lu.num_levels(); lv++) {
    int mx = 0;
    for (int c = S.lu.start_levels[lv]; c < S.lu.start_levels[lv + 1]; c++)
      for (int t = S.lu.start_chains[c]; t < S.lu.start_chains[c + 1]; t++) {
        const int col = S.lu.columns[t];
        mx = std::max(mx, S.csr_rowptr[col + 1] - S.csr_rowptr[col]);
      }
    S.max_elements_per_column.push_back(mx);
  }

  // ---- execution structures ----
  // Value scatter map (replaces 000:193-210 + 010:142-155).
  S.slot_src.assign(nnz, -1);
  for (int j = 0; j < n; j++)
    for (int q = S.csc_colptr[j]; q < S.csc_colptr[j + 1]; q++) {
      const int ro = S.row_orig[S.csc_row[q]], co = S.col_orig[j];
      const int* b = S.a_colidx.data() + S.a_rowptr[ro];
      const int* e = S.a_colidx.data() + S.a_rowptr[ro + 1];
      const int* it = std::lower_bound(b, e, co);
      if (it != e && *it == co)
        S.slot_src[q] = (int)(it - S.a_colidx.data());
    }

  // Left-looking update targets.
  S.upd_ptr.assign(nnz + 1, 0);
  S.update_count = 0;
  S.flops_refactor = 0;
  for (int j = 0; j < n; j++) {
    const int64_t nl = S.csc_colptr[j + 1] - S.csc_diag_start[j];
    const int64_t nu = S.csr_rowptr[j + 1] - S.csr_diag_start[j];
    S.update_count += nl * nu;
    S.flops_refactor += (double)nl + 2.0 * (double)nl * (double)nu;
  }
  S.upd_tgt.resize(S.update_count);
  {
    // Slots are visited in CSC order, so upd_ptr is a prefix array: the
    // updates of slot p are upd_tgt[upd_ptr[p] .. upd_ptr[p + 1]), empty for
    // diagonal and L slots.
    std::vector<int> slot_of_row(n, -1);
    int64_t w = 0;
    for (int k = 0; k < n; k++) {
      for (int q = S.csc_colptr[k]; q < S.csc_colptr[k + 1]; q++)
        slot_of_row[S.csc_row[q]] = q;
      for (int p = S.csc_colptr[k]; p < S.csc_colptr[k + 1]; p++) {
        S.upd_ptr[p] = w;
        if (p >= S.diag_slot[k]) continue;
        const int j = S.csc_row[p];
        for (int q = S.csc_diag_start[j]; q < S.csc_colptr[j + 1]; q++) {
          const int t = slot_of_row[S.csc_row[q]];
          if (t < 0) {
            err = "filled pattern is not closed under elimination";
            return ERR_STRUCTURAL;
          }
          S.upd_tgt[w++] = t;
        }
      }
      for (int q = S.csc_colptr[k]; q < S.csc_colptr[k + 1]; q++)
        slot_of_row[S.csc_row[q]] = -1;
    }
    S.upd_ptr[nnz] = w;
  }

  // Row-gather lists.
  S.lrow_ptr.assign(n + 1, 0);
  S.urow_ptr.assign(n + 1, 0);
  S.lrow_slot.clear();
  S.lrow_col.clear();
  S.urow_slot.clear();
  S.urow_col.clear();
  for (int i = 0; i < n; i++) {
    for (int p = S.csr_rowptr[i]; p < S.csr_rowptr[i + 1]; p++) {
      const int j = S.csr_col[p];
      if (j < i) {
        S.lrow_slot.push_back(S.csr_to_csc[p]);
        S.lrow_col.push_back(j);
      } else if (j > i) {
        S.urow_slot.push_back(S.csr_to_csc[p]);
        S.urow_col.push_back(j);
      }
    }
    S.lrow_ptr[i + 1] = (int)S.lrow_slot.size();
    S.urow_ptr[i + 1] = (int)S.urow_slot.size();
  }

  // Right-looking hazard count of the reference's LU schedule.
  {
    std::vector<int> lvl(n), chain(n), posn(n);
    for (int lv = 0; lv < S.lu.num_levels(); lv++)
      for (int c = S.lu.start_levels[lv]; c < S.lu.start_levels[lv + 1]; c++)
        for (int t = S.lu.start_chains[c]; t < S.lu.start_chains[c + 1]; t++) {
          lvl[S.lu.columns[t]] = lv;
          chain[S.lu.columns[t]] = c;
          posn[S.lu.columns[t]] = t;
        }
    std::vector<int> max_u(n, -1);
    for (int i = 0; i < n; i++)
      if (S.csr_rowptr[i + 1] > S.csr_diag_start[i])
        max_u[i] = S.csr_col[S.csr_rowptr[i + 1] - 1];
    int64_t hz = 0;
    for (int j = 0; j < n; j++)
      for (int p = S.csr_rowptr[j]; p < S.csr_rowptr[j + 1]; p++) {
        const int jp = S.csr_col[p];
        if (jp >= j) break;
        if (max_u[jp] <= j) continue;
        const bool before = lvl[jp] < lvl[j] ||
                            (lvl[jp] == lvl[j] && chain[jp] == chain[j] &&
                             posn[jp] < posn[j]);
        if (!before) hz++;
      }
    S.right_looking_hazards = hz;
  }
  return OK;
}

}  // namespace pvglu
