// ORACLE — test infrastructure only.
//
// A plain CPU restatement of the reference's per-Newton-iteration sparse
// linear-algebra path (AlbertoJimenezRuiz/PhdThesis_AlbertoJimenezRuiz,
// PVPP_Plant_Simulator).  It exists to check the product library: only the
// tests, the smoke check and bench.py's CPU-baseline legs load it.  Nothing in
// the product links, calls or ships it.
//
// Every function follows the reference file:line it cites, in the same loop
// order and with the same floating-point operation order (compile with
// -ffp-contract=off so that no FMA contraction changes the rounding).  The
// AMD ordering (third-party AMD 1.1 under PVPP_Plant_Simulator/AmdLib) is not
// restated: the caller passes its permutation P.
//
// Pinned against the reference itself: oracle/ref_harness.cpp builds the
// reference's own sources into oracle/_ref/libpvref.so here, and
// tests/golden/make_golden.py records its outputs as fixtures.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <list>
#include <map>
#include <set>
#include <string>
#include <vector>

namespace {

using Row = std::map<int, double>;
using Matrix = std::vector<Row>;  // Sparse_Matrix::data, sparse_matrix.h:6-24

// Sparse_Matrix::transpose, sparse_matrix.h:100-114.
Matrix transpose(const Matrix& m) {
  Matrix t(m.size());
  for (size_t i = 0; i < m.size(); i++)
    for (const auto& e : m[i]) t[e.first].insert({(int)i, e.second});
  return t;
}

// Sparse_Matrix::interchange_row_columns, sparse_matrix.h:117-134.
Matrix interchange_row_columns(const Matrix& m, const int* new_order) {
  Matrix out(m.size());
  for (size_t i = 0; i < m.size(); i++) {
    Row r;
    for (const auto& e : m[i]) r[new_order[e.first]] = e.second;
    out[new_order[i]] = r;
  }
  return out;
}

// Sparse_Matrix::exchange_rows(int*), sparse_matrix.h:136-147.
Matrix exchange_rows(const Matrix& m, const int* new_order) {
  Matrix out(m.size());
  for (size_t i = 0; i < m.size(); i++) out[new_order[i]] = m[i];
  return out;
}

// util.cpp:70-77.
std::vector<int> invert_permutation(const std::vector<int>& p) {
  std::vector<int> r(p.size());
  for (size_t i = 0; i < p.size(); i++) r[p[i]] = (int)i;
  return r;
}

// 004c_exchange_rows_columns.cpp:7-22 and :53-89 (move_only_rows variant):
// swap keys f1 <-> f2 inside every touched row of the transpose, then swap
// the two rows of the matrix.
void exchange_map(Row& data, int f1, int f2) {
  Row nd;
  for (const auto& e : data) {
    int c = e.first;
    if (c == f1) c = f2;
    else if (c == f2) c = f1;
    nd[c] = e.second;
  }
  data = nd;
}

std::vector<int> row_keys(const Row& r) {
  std::vector<int> v;
  for (const auto& e : r) v.push_back(e.first);
  return v;
}

void interchange_only_rows(Matrix& mat, Matrix& tr, int f1, int f2) {
  std::vector<int> a = row_keys(mat[f1]), b = row_keys(mat[f2]);
  std::vector<int> c = row_keys(tr[f1]), d = row_keys(tr[f2]);
  std::set<int> all(a.begin(), a.end());
  all.insert(b.begin(), b.end());
  all.insert(c.begin(), c.end());
  all.insert(d.begin(), d.end());
  for (int r : all) exchange_map(tr[r], f1, f2);
  std::swap(mat[f1], mat[f2]);
}

// 004b_remove_zeros_diagonal.cpp:12-100, move_only_rows = true.
bool remove_zeros_diagonal(Matrix& io, std::vector<int>& perm, std::string& err) {
  Matrix h = io;
  Matrix v = transpose(h);
  const int n = (int)h.size();
  for (int cur = 0; cur < n; cur++) {
    if (h[cur].count(cur)) continue;
    bool would_fill = false;
    for (const auto& re : h[cur]) {
      if (would_fill) break;
      const int rp = re.first;
      if (rp >= cur) break;
      for (const auto& ce : v[cur]) {
        const int cp = ce.first;
        if (cp == rp) would_fill = true;
        else if (cp > rp) break;
      }
    }
    if (!would_fill) {
      int ri = -1;
      for (const auto& ce : v[cur])
        if (ce.first > cur) {
          ri = ce.first;
          break;
        }
      if (ri == -1) {
        err = "no row to exchange for zero diagonal " + std::to_string(cur);
        return false;
      }
      interchange_only_rows(h, v, cur, ri);
      std::swap(perm[cur], perm[ri]);
    }
  }
  io = h;
  return true;
}

// 005a_obtain_fillin_matrix_CUDA.cu:18-236 restated on the host: passes of
// the row-parallel search (check_possible_new_nonzeros_CUDA.h:51-210) over
// the pattern of the previous pass, merge of the new entries, and the
// row/column worklist of get_rows_and_columns_to_be_processed_CUDA.cuh:3-63
// (computed on the pattern before the merge, as the reference does), until a
// pass adds nothing.  The reference's scratch re-allocation loop only sizes
// buffers and does not change the result, so it is not restated.
std::vector<std::vector<int>> obtain_fillin(const Matrix& m) {
  const int n = (int)m.size();
  std::vector<std::vector<int>> rows(n);
  for (int i = 0; i < n; i++)
    for (const auto& e : m[i]) rows[i].push_back(e.first);
  std::vector<uint8_t> rows_process(n, 1), cols_process(n, 1);
  for (;;) {
    std::vector<std::vector<int>> holes(n);
    std::vector<uint8_t> added_rows(n, 0), added_cols(n, 0);
    bool added = false;
    for (int a = 0; a < n; a++) {
      if (!rows_process[a]) continue;
      const auto& ra = rows[a];
      for (size_t ia = 0; ia < ra.size(); ia++) {
        const int ka = ra[ia];
        if (!cols_process[ka]) continue;
        if (a <= ka) continue;
        const auto& rb = rows[ka];
        size_t ib = 0, ic = ia + 1;
        // Skip B entries left of or on the diagonal.  The reference's loop has
        // no bound here; when row ka holds nothing right of ka it walks past
        // the row end and the merge below is skipped, as it is here.
        while (ib < rb.size() && rb[ib] <= ka) ib++;
        while (ib < rb.size()) {
          const int cb = rb[ib];
          const int cc = (ic == ra.size()) ? n : ra[ic];
          if (cb < cc) {
            auto& hr = holes[a];
            auto it = std::lower_bound(hr.begin(), hr.end(), cb);
            if (it == hr.end() || *it != cb) {
              hr.insert(it, cb);
              added = true;
              added_rows[a] = 1;
              added_cols[cb] = 1;
            }
            ib++;
          } else if (cb == cc) {
            ib++;
            ic++;
          } else {
            ic++;
          }
        }
      }
    }
    // Worklist for the next pass from the pattern before the merge.
    for (int t = 0; t < n; t++) {
      uint8_t rp = 0;
      if (added_rows[t]) rp = 1;
      else
        for (int c : rows[t])
          if (added_rows[c]) rp = 1;
      rows_process[t] = rp;
      cols_process[t] = (added_cols[t] || added_rows[t]) ? 1 : 0;
    }
    for (int a = 0; a < n; a++) {
      if (holes[a].empty()) continue;
      std::vector<int> merged;
      std::merge(rows[a].begin(), rows[a].end(), holes[a].begin(), holes[a].end(),
                 std::back_inserter(merged));
      rows[a] = merged;
    }
    if (!added) break;
  }
  return rows;
}

// 006_get_dependencies_GLU.cpp:5-47, :49-62, :64-77.
std::vector<std::set<int>> deps_glu(int n, const std::vector<std::vector<int>>& f) {
  std::vector<std::vector<int>> ft(n);
  for (size_t i = 0; i < f.size(); i++)
    for (int j : f[i]) ft[j].push_back((int)i);
  std::vector<std::set<int>> d(n);
  for (int k = 0; k < n; k++) {
    for (int i : ft[k]) {
      if (i >= k) continue;
      for (int z : ft[i]) {
        if (i < z) continue;
        if (i >= n) continue;
        d[k].insert(i);
        break;
      }
    }
    for (int i : ft[k]) {
      if (i >= k) continue;
      d[k].insert(i);
    }
  }
  return d;
}
std::vector<std::set<int>> deps_l(int n, const std::vector<std::vector<int>>& f) {
  std::vector<std::set<int>> d(n);
  for (int i = 0; i < (int)f.size(); i++)
    for (int j : f[i])
      if (j < i) d[i].insert(j);
  return d;
}
std::vector<std::set<int>> deps_u(int n, const std::vector<std::vector<int>>& f) {
  std::vector<std::set<int>> d(n);
  for (int i = 0; i < (int)f.size(); i++)
    for (int j : f[i])
      if (j > i) d[i].insert(j);
  return d;
}
// Transposed-L solve dependencies (not in the reference): {i > j : M(i,j)}.
std::vector<std::set<int>> deps_lt(int n, const std::vector<std::vector<int>>& f) {
  std::vector<std::set<int>> d(n);
  for (int i = 0; i < (int)f.size(); i++)
    for (int j : f[i])
      if (i > j) d[j].insert(i);
  return d;
}

// 007_convert_dependencies_in_levels.cpp:4-60.
std::vector<std::vector<int>> get_basic_levels(const std::vector<std::set<int>>& deps) {
  std::vector<std::vector<int>> out;
  std::vector<int> where(deps.size(), -1);
  int classified = 0, cur = 0;
  while (classified != (int)deps.size()) {
    std::vector<int> lvl;
    for (int i = 0; i < (int)deps.size(); i++) {
      if (where[i] != -1) continue;
      bool ok = true;
      for (int l : deps[i])
        if (where[l] == -1 || where[l] == cur) {
          ok = false;
          break;
        }
      if (ok) {
        where[i] = cur;
        lvl.push_back(i);
        classified++;
      }
    }
    if (lvl.empty()) break;  // cyclic input; the reference would loop forever
    out.push_back(lvl);
    cur++;
  }
  return out;
}

// 007:62-87.
int chain_column_belongs_to(const std::vector<int>& pos, const std::set<int>& d) {
  int found = -1;
  for (int c : d) {
    const int p = pos[c];
    if (p == -1) continue;
    if (found == p) continue;
    if (found != -1) return -1;
    found = p;
  }
  return found;
}

// 007:89-144.
bool get_resulting_chain(int cur, const std::vector<int>& basic,
                         const std::vector<std::set<int>>& deps,
                         const std::vector<int>& pos, std::vector<int>& hooks) {
  if (cur == 0) return false;
  hooks.assign(basic.size(), 0);
  for (size_t idx = 0; idx < basic.size(); idx++) {
    const int f = chain_column_belongs_to(pos, deps[basic[idx]]);
    if (f == -1) return false;
    for (size_t j = 0; j < idx; j++)
      if (f == hooks[j]) return false;
    hooks[idx] = f;
  }
  return true;
}

// 007:146-210 then 008:4-30.
void levels_flat(const std::vector<std::set<int>>& deps, std::vector<int>& sl,
                 std::vector<int>& sc, std::vector<int>& cols,
                 std::vector<std::vector<std::list<int>>>* keep = nullptr) {
  const size_t n = deps.size();
  auto basic = get_basic_levels(deps);
  std::vector<std::vector<std::list<int>>> custom;
  std::vector<int> pos(n);
  for (int lv = 0; lv < (int)basic.size(); lv++) {
    std::vector<int> hooks;
    if (get_resulting_chain(lv, basic[lv], deps, pos, hooks)) {
      auto& prev = custom.back();
      for (size_t idx = 0; idx < hooks.size(); idx++) {
        prev[hooks[idx]].push_back(basic[lv][idx]);
        pos[basic[lv][idx]] = hooks[idx];
      }
    } else {
      std::fill(pos.begin(), pos.end(), -1);
      std::vector<std::list<int>> res(basic[lv].size());
      for (size_t s = 0; s < basic[lv].size(); s++) {
        res[s].push_back(basic[lv][s]);
        pos[basic[lv][s]] = (int)s;
      }
      custom.push_back(res);
    }
  }
  sl.clear();
  sc.clear();
  cols.clear();
  for (const auto& lv : custom) {
    sl.push_back((int)sc.size());
    for (const auto& ch : lv) {
      sc.push_back((int)cols.size());
      for (int c : ch) cols.push_back(c);
    }
  }
  sl.push_back((int)sc.size());
  sc.push_back((int)cols.size());
  if (keep) *keep = custom;
}

struct Oracle {
  int n = 0;
  std::vector<int> a_rowptr, a_colidx;
  std::vector<int> perm_amd, perm_amd_rev, perm_rows, perm_rows_rev;
  std::vector<int> fill_rowptr, fill_col;
  std::vector<int> lu_sl, lu_sc, lu_cols, l_sl, l_sc, l_cols, u_sl, u_sc, u_cols;
  std::vector<int> lt_sl, lt_sc, lt_cols;
  std::vector<int> max_elements_per_column;
  std::vector<int> csr_rowptr, csr_col, csc_colptr, csc_row, csr_to_csc,
      csc_to_csr, csr_diag_start, csc_diag_start;
  int bad_column = -1;
};

// 010_create_CSR_CSC.cpp:15-128.
void create_csr_csc(const Matrix& mat, Oracle& o) {
  const int m = (int)mat.size(), n = m;
  std::vector<std::vector<int>> csc_in_csr(n), csr_in_csc(m);
  o.csr_rowptr.clear();
  o.csr_col.clear();
  int count = 0;
  for (int i = 0; i < m; i++) {
    o.csr_rowptr.push_back(count);
    for (const auto& e : mat[i]) {
      csc_in_csr[e.first].push_back(count);
      o.csr_col.push_back(e.first);
      count++;
    }
  }
  o.csr_rowptr.push_back(count);
  const Matrix t = transpose(mat);
  o.csc_colptr.clear();
  o.csc_row.clear();
  count = 0;
  for (int j = 0; j < n; j++) {
    o.csc_colptr.push_back(count);
    for (const auto& e : t[j]) {
      csr_in_csc[e.first].push_back(count);
      o.csc_row.push_back(e.first);
      count++;
    }
  }
  o.csc_colptr.push_back((int)o.csc_row.size());
  o.csc_to_csr.clear();
  for (auto& v : csc_in_csr) o.csc_to_csr.insert(o.csc_to_csr.end(), v.begin(), v.end());
  o.csr_to_csc.clear();
  for (auto& v : csr_in_csc) o.csr_to_csc.insert(o.csr_to_csc.end(), v.begin(), v.end());
  o.csr_diag_start.clear();
  for (int i = 0; i < m; i++) {
    bool found = false;
    for (int p = o.csr_rowptr[i]; p < o.csr_rowptr[i + 1]; p++)
      if (o.csr_col[p] > i) {
        o.csr_diag_start.push_back(p);
        found = true;
        break;
      }
    if (!found) o.csr_diag_start.push_back(o.csr_rowptr[i + 1]);
  }
  o.csc_diag_start.clear();
  for (int j = 0; j < n; j++) {
    bool found = false;
    for (int p = o.csc_colptr[j]; p < o.csc_colptr[j + 1]; p++)
      if (o.csc_row[p] > j) {
        o.csc_diag_start.push_back(p);
        found = true;
        break;
      }
    if (!found) o.csc_diag_start.push_back(o.csc_colptr[j + 1]);
  }
}

// GLU_CSC_CPU_levels_strings.cpp:3-63.  Returns false on a missing diagonal
// or a pivot below 1e-8 in magnitude (the reference asserts there).
bool factorize_one_column(const Oracle& o, int j, double* v) {
  if (o.csc_colptr[j] == o.csc_diag_start[j]) return false;
  const double large = v[o.csc_diag_start[j] - 1];
  if (std::abs(large) < 1e-8) return false;
  for (int c1 = o.csc_diag_start[j]; c1 < o.csc_colptr[j + 1]; c1++) v[c1] /= large;
  for (int r2 = o.csr_diag_start[j]; r2 < o.csr_rowptr[j + 1]; r2++) {
    const int col = o.csr_col[r2];
    const double dom = v[o.csr_to_csc[r2]];
    for (int c3 = o.csc_diag_start[j]; c3 < o.csc_colptr[j + 1]; c3++) {
      const int row = o.csc_row[c3];
      const double elem = v[c3];
      for (int c1 = o.csc_colptr[col]; c1 < o.csc_colptr[col + 1]; c1++) {
        if (o.csc_row[c1] != row) continue;
        v[c1] -= elem * dom;
        break;
      }
    }
  }
  return true;
}

// GLU_CSC_CPU_Triangular.cpp:3-26.
void process_column_l(const Oracle& o, int j, const double* v, double* b) {
  for (int r = o.csc_diag_start[j]; r < o.csc_colptr[j + 1]; r++)
    b[o.csc_row[r]] -= v[r] * b[j];
}
void process_column_u(const Oracle& o, int j, const double* v, double* b) {
  const int d = o.csc_diag_start[j] - 1;
  b[j] /= v[d];
  for (int r = o.csc_colptr[j]; r < d; r++) b[o.csc_row[r]] -= v[r] * b[j];
}

}  // namespace

extern "C" {

// Symbolic analysis with a caller-supplied P (prepare_matrices,
// 000_PVPP_simulator.cpp:10-93, with the AMD call of 004a replaced by P).
void* oracle_symbolic(int n, const int* rowptr, const int* colidx, const int* perm,
                      char* err, int errlen) {
  std::string e;
  auto* o = new Oracle();
  o->n = n;
  o->a_rowptr.assign(rowptr, rowptr + n + 1);
  o->a_colidx.assign(colidx, colidx + rowptr[n]);
  Matrix a(n);
  for (int i = 0; i < n; i++)
    for (int p = rowptr[i]; p < rowptr[i + 1]; p++) a[i][colidx[p]] = 1.0;
  o->perm_amd.assign(perm, perm + n);
  std::vector<int> pinv = invert_permutation(o->perm_amd);
  Matrix m = interchange_row_columns(a, pinv.data());  // 004a:44
  o->perm_rows.resize(n);
  for (int i = 0; i < n; i++) o->perm_rows[i] = i;  // 004d:36-38
  if (!remove_zeros_diagonal(m, o->perm_rows, e)) {  // 004d:44
    if (err && errlen > 0) snprintf(err, errlen, "%s", e.c_str());
    delete o;
    return nullptr;
  }
  o->perm_amd_rev = pinv;
  o->perm_rows_rev = invert_permutation(o->perm_rows);
  auto fill = obtain_fillin(m);  // 000:33
  for (int i = 0; i < n; i++)    // 005c:4-14
    for (int c : fill[i])
      if (!m[i].count(c)) m[i][c] = 0.0;
  o->fill_rowptr.assign(1, 0);
  o->fill_col.clear();
  for (int i = 0; i < n; i++) {
    o->fill_col.insert(o->fill_col.end(), fill[i].begin(), fill[i].end());
    o->fill_rowptr.push_back((int)o->fill_col.size());
  }
  std::vector<std::vector<std::list<int>>> lu_levels;
  levels_flat(deps_glu(n, fill), o->lu_sl, o->lu_sc, o->lu_cols, &lu_levels);
  levels_flat(deps_l(n, fill), o->l_sl, o->l_sc, o->l_cols);
  levels_flat(deps_u(n, fill), o->u_sl, o->u_sc, o->u_cols);
  levels_flat(deps_lt(n, fill), o->lt_sl, o->lt_sc, o->lt_cols);
  // 009_get_max_numbers_per_column.cpp:3-31.
  o->max_elements_per_column.clear();
  for (const auto& lv : lu_levels) {
    size_t mx = 0;
    for (const auto& ch : lv)
      for (int c : ch) mx = std::max(mx, fill[c].size());
    o->max_elements_per_column.push_back((int)mx);
  }
  create_csr_csc(m, *o);  // 010:15-128
  return o;
}

void oracle_free(void* h) { delete static_cast<Oracle*>(h); }

int oracle_get(void* h, const char* name, const int** ptr, long long* len) {
  auto* o = static_cast<Oracle*>(h);
  const std::vector<int>* v = nullptr;
  const std::string s(name);
#define PVG(x) if (s == #x) v = &o->x;
  PVG(perm_amd) PVG(perm_rows) PVG(fill_rowptr) PVG(fill_col)
  PVG(lu_sl) PVG(lu_sc) PVG(lu_cols) PVG(l_sl) PVG(l_sc) PVG(l_cols)
  PVG(u_sl) PVG(u_sc) PVG(u_cols) PVG(lt_sl) PVG(lt_sc) PVG(lt_cols)
  PVG(max_elements_per_column) PVG(csr_rowptr) PVG(csr_col) PVG(csc_colptr)
  PVG(csc_row) PVG(csr_to_csc) PVG(csc_to_csr) PVG(csr_diag_start)
  PVG(csc_diag_start)
#undef PVG
  if (!v) return 1;
  *ptr = v->data();
  *len = (long long)v->size();
  return 0;
}

// Value scatter of one Newton iteration (000_PVPP_simulator.cpp:193-210):
// permute A (values in the caller's CSR order) with Pinv on both sides, then
// exchange rows with Q, then fill the CSC slots (010:142-155, 0 at fill).
int oracle_scatter(void* h, const double* a_vals, double* csc_vals) {
  auto* o = static_cast<Oracle*>(h);
  const int n = o->n;
  Matrix a(n);
  for (int i = 0; i < n; i++)
    for (int p = o->a_rowptr[i]; p < o->a_rowptr[i + 1]; p++)
      a[i][o->a_colidx[p]] = a_vals[p];
  a = interchange_row_columns(a, o->perm_amd_rev.data());
  a = exchange_rows(a, o->perm_rows.data());
  const Matrix t = transpose(a);
  for (int j = 0; j < n; j++)
    for (int p = o->csc_colptr[j]; p < o->csc_colptr[j + 1]; p++) {
      auto it = t[j].find(o->csc_row[p]);
      csc_vals[p] = (it == t[j].end()) ? 0.0 : it->second;
    }
  return 0;
}

// factorize_all_chains_of_columns_in_level_GLU_CSC_CPU
// (GLU_CSC_CPU_levels_strings.cpp:65-106) over every LU level in order.
// Returns 0, or 3 with *bad_col set on a zero/tiny pivot.
int oracle_refactor_levels(void* h, double* v, int* bad_col) {
  auto* o = static_cast<Oracle*>(h);
  for (int lv = 0; lv + 1 < (int)o->lu_sl.size(); lv++)
    for (int c = o->lu_sl[lv]; c < o->lu_sl[lv + 1]; c++)
      for (int t = o->lu_sc[c]; t < o->lu_sc[c + 1]; t++)
        if (!factorize_one_column(*o, o->lu_cols[t], v)) {
          if (bad_col) *bad_col = o->lu_cols[t];
          return 3;
        }
  return 0;
}

// GLU_CSC_CPU_sequential (GLU_CSC_CPU_levels_strings.cpp:108-132).
int oracle_refactor_sequential(void* h, double* v, int* bad_col) {
  auto* o = static_cast<Oracle*>(h);
  for (int j = 0; j < o->n; j++)
    if (!factorize_one_column(*o, j, v)) {
      if (bad_col) *bad_col = j;
      return 3;
    }
  return 0;
}

// Substitute_LU_Vector_b_CSC_CPU (GLU_CSC_CPU_Triangular.cpp:27-43), permuted
// space, b overwritten with x.
int oracle_solve(void* h, const double* v, double* b) {
  auto* o = static_cast<Oracle*>(h);
  for (int j = 0; j < o->n; j++) process_column_l(*o, j, v, b);
  for (int j = o->n - 1; j >= 0; j--) process_column_u(*o, j, v, b);
  return 0;
}

// Transposed solve M^T z = b with the same factors (M = L U): U^T w = b
// forward, then L^T z = w backward.  Not part of the reference (it has no
// adjoint); written in the same column-sweep style for the FP64 CPU adjoint.
int oracle_solve_transposed(void* h, const double* v, double* b) {
  auto* o = static_cast<Oracle*>(h);
  const int n = o->n;
  for (int j = 0; j < n; j++) {
    const int d = o->csc_diag_start[j] - 1;
    double s = b[j];
    for (int r = o->csc_colptr[j]; r < d; r++) s -= v[r] * b[o->csc_row[r]];
    b[j] = s / v[d];
  }
  for (int j = n - 1; j >= 0; j--) {
    double s = b[j];
    for (int r = o->csc_diag_start[j]; r < o->csc_colptr[j + 1]; r++)
      s -= v[r] * b[o->csc_row[r]];
    b[j] = s;
  }
  return 0;
}

// Full drop-in sequence of one Newton iteration on the CPU: scatter,
// refactor (sequential column order, GLU_CSC_CPU_sequential, when
// `sequential` is set, else the level order), permute b (000:198-201),
// solve, unpermute x (000:233).  b (length n, original order) is overwritten
// with x.
int oracle_scatter_refactor_solve(void* h, const double* a_vals, double* lu_out,
                                  double* b, int sequential) {
  auto* o = static_cast<Oracle*>(h);
  const int n = o->n;
  oracle_scatter(h, a_vals, lu_out);
  int bad = -1;
  const int st = sequential ? oracle_refactor_sequential(h, lu_out, &bad)
                            : oracle_refactor_levels(h, lu_out, &bad);
  if (st) return st;
  std::vector<double> w(b, b + n), t(n);
  for (int i = 0; i < n; i++) t[o->perm_amd_rev[i]] = w[i];  // apply_permutation(Pinv)
  for (int i = 0; i < n; i++) w[o->perm_rows[i]] = t[i];     // apply_permutation(Q)
  oracle_solve(h, lu_out, w.data());
  for (int i = 0; i < n; i++) b[o->perm_amd[i]] = w[i];      // apply_permutation(P)
  return 0;
}

}  // extern "C"
