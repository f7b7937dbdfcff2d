// Symbolic analysis dump format (pvglu_symbolic_save / pvglu_symbolic_load).
//
// The reference rebuilds its struct_CPU_CUDA_arrays (factorize_electrical_system.h:3-61)
// from the circuit at every program start (prepare_matrices,
// 000_PVPP_simulator.cpp:10-93).  Saving the analysis lets a run restart, or a
// test reuse a fixture, without the analysis.
//
// Layout (little-endian):
//   "PVGLUSYM" | u32 version | u32 0x01020304 (byte-order check)
//   i64 scalars: n, nnz_a, nnz_lu, row_swaps, perm_rows_is_involution,
//                update_count, right_looking_hazards | f64 flops_refactor
//   u32 array count, then per array: u16 name length, name bytes,
//     u8 element size (4 or 8), u64 element count, the elements
//   u64 FNV-1a hash of every byte before it
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/pvglu.h"
#include "symbolic.hpp"

namespace pvglu {
namespace {

constexpr char kMagic[8] = {'P', 'V', 'G', 'L', 'U', 'S', 'Y', 'M'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kOrder = 0x01020304u;

struct Writer {
  std::vector<unsigned char> buf;
  void bytes(const void* p, size_t n) {
    const auto* c = static_cast<const unsigned char*>(p);
    buf.insert(buf.end(), c, c + n);
  }
  template <typename T>
  void put(T v) {
    bytes(&v, sizeof v);
  }
};

struct Reader {
  const unsigned char* p;
  size_t left;
  bool ok = true;
  bool bytes(void* dst, size_t n) {
    if (!ok || n > left) return ok = false;
    std::memcpy(dst, p, n);
    p += n;
    left -= n;
    return true;
  }
  template <typename T>
  bool get(T& v) {
    return bytes(&v, sizeof v);
  }
};

uint64_t fnv1a(const unsigned char* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

// Every array of the analysis, by name (S is Symbolic or const Symbolic).
template <typename S, typename F>
void for_each_int_array(S& s, F&& f) {
  f("a_rowptr", s.a_rowptr);
  f("a_colidx", s.a_colidx);
  f("perm_amd", s.perm_amd);
  f("perm_rows", s.perm_rows);
  f("row_orig", s.row_orig);
  f("col_orig", s.col_orig);
  f("fill_rowptr", s.fill_rowptr);
  f("fill_col", s.fill_col);
  f("csr_rowptr", s.csr_rowptr);
  f("csr_col", s.csr_col);
  f("csc_colptr", s.csc_colptr);
  f("csc_row", s.csc_row);
  f("csr_to_csc", s.csr_to_csc);
  f("csc_to_csr", s.csc_to_csr);
  f("csr_diag_start", s.csr_diag_start);
  f("csc_diag_start", s.csc_diag_start);
  f("lu_sl", s.lu.start_levels);
  f("lu_sc", s.lu.start_chains);
  f("lu_cols", s.lu.columns);
  f("l_sl", s.l.start_levels);
  f("l_sc", s.l.start_chains);
  f("l_cols", s.l.columns);
  f("u_sl", s.u.start_levels);
  f("u_sc", s.u.start_chains);
  f("u_cols", s.u.columns);
  f("lt_sl", s.lt.start_levels);
  f("lt_sc", s.lt.start_chains);
  f("lt_cols", s.lt.columns);
  f("max_elements_per_column", s.max_elements_per_column);
  f("diag_slot", s.diag_slot);
  f("slot_src", s.slot_src);
  f("upd_tgt", s.upd_tgt);
  f("lrow_ptr", s.lrow_ptr);
  f("lrow_slot", s.lrow_slot);
  f("lrow_col", s.lrow_col);
  f("urow_ptr", s.urow_ptr);
  f("urow_slot", s.urow_slot);
  f("urow_col", s.urow_col);
}

// A loaded analysis is used to index device memory: every size and every
// index must be in range before it is accepted.
bool in_range(const std::vector<int>& v, int64_t lo, int64_t hi) {
  for (int x : v)
    if (x < lo || x >= hi) return false;
  return true;
}

bool monotone(const std::vector<int>& p, size_t size, int64_t last) {
  if (p.size() != size || p.empty() || p[0] != 0 || p.back() != last) return false;
  for (size_t i = 1; i < p.size(); i++)
    if (p[i] < p[i - 1]) return false;
  return true;
}

bool permutation(const std::vector<int>& p, int n) {
  if ((int)p.size() != n) return false;
  std::vector<char> seen(n, 0);
  for (int x : p) {
    if (x < 0 || x >= n || seen[x]) return false;
    seen[x] = 1;
  }
  return true;
}

bool levels_ok(const LevelSet& ls, int n, bool required) {
  if (!required && ls.start_levels.empty() && ls.start_chains.empty() && ls.columns.empty())
    return true;
  if ((int)ls.columns.size() != n || !in_range(ls.columns, 0, n)) return false;
  if (!monotone(ls.start_chains, ls.start_chains.size(), n)) return false;
  return monotone(ls.start_levels, ls.start_levels.size(), (int64_t)ls.start_chains.size() - 1);
}

bool consistent(const Symbolic& s, std::string& why) {
  const int n = s.n;
  auto need = [&](bool c, const char* what) {
    if (!c) why = what;
    return c;
  };
  if (!need(n > 0 && s.nnz_a > 0 && s.nnz_lu >= n && s.nnz_a < (1LL << 31) &&
                s.nnz_lu < (1LL << 31),
            "sizes"))
    return false;
  return need(monotone(s.a_rowptr, n + 1, s.nnz_a), "a_rowptr") &&
         need((int64_t)s.a_colidx.size() == s.nnz_a && in_range(s.a_colidx, 0, n), "a_colidx") &&
         need(permutation(s.perm_amd, n) && permutation(s.perm_rows, n) &&
                  permutation(s.row_orig, n) && permutation(s.col_orig, n),
              "orderings") &&
         need(monotone(s.fill_rowptr, n + 1, s.nnz_lu) && in_range(s.fill_col, 0, n), "fill") &&
         need(monotone(s.csr_rowptr, n + 1, s.nnz_lu) && in_range(s.csr_col, 0, n) &&
                  (int64_t)s.csr_col.size() == s.nnz_lu,
              "csr") &&
         need(monotone(s.csc_colptr, n + 1, s.nnz_lu) && in_range(s.csc_row, 0, n) &&
                  (int64_t)s.csc_row.size() == s.nnz_lu,
              "csc") &&
         need((int64_t)s.csr_to_csc.size() == s.nnz_lu && in_range(s.csr_to_csc, 0, s.nnz_lu) &&
                  (int64_t)s.csc_to_csr.size() == s.nnz_lu &&
                  in_range(s.csc_to_csr, 0, s.nnz_lu),
              "cross maps") &&
         need((int)s.csr_diag_start.size() == n && in_range(s.csr_diag_start, 0, s.nnz_lu + 1) &&
                  (int)s.csc_diag_start.size() == n &&
                  in_range(s.csc_diag_start, 0, s.nnz_lu + 1),
              "diagonal starts") &&
         need((int)s.diag_slot.size() == n && in_range(s.diag_slot, 0, s.nnz_lu) &&
                  (int64_t)s.slot_src.size() == s.nnz_lu && in_range(s.slot_src, -1, s.nnz_a),
              "slots") &&
         need(s.upd_ptr.size() == (size_t)s.nnz_lu + 1 && s.upd_ptr[0] == 0 &&
                  std::is_sorted(s.upd_ptr.begin(), s.upd_ptr.end()) &&
                  s.upd_ptr.back() == (int64_t)s.upd_tgt.size() &&
                  in_range(s.upd_tgt, 0, s.nnz_lu),
              "updates") &&
         need(monotone(s.lrow_ptr, n + 1, (int64_t)s.lrow_slot.size()) &&
                  s.lrow_col.size() == s.lrow_slot.size() && in_range(s.lrow_slot, 0, s.nnz_lu) &&
                  in_range(s.lrow_col, 0, n) &&
                  monotone(s.urow_ptr, n + 1, (int64_t)s.urow_slot.size()) &&
                  s.urow_col.size() == s.urow_slot.size() && in_range(s.urow_slot, 0, s.nnz_lu) &&
                  in_range(s.urow_col, 0, n),
              "row lists") &&
         need(levels_ok(s.lu, n, true) && levels_ok(s.l, n, true) && levels_ok(s.u, n, true) &&
                  levels_ok(s.lt, n, false),
              "level sets");
}

}  // namespace

int save_symbolic(const Symbolic& s, const char* path, std::string& err) {
  Writer w;
  w.bytes(kMagic, sizeof kMagic);
  w.put(kVersion);
  w.put(kOrder);
  w.put<int64_t>(s.n);
  w.put<int64_t>(s.nnz_a);
  w.put<int64_t>(s.nnz_lu);
  w.put<int64_t>(s.row_swaps);
  w.put<int64_t>(s.perm_rows_is_involution);
  w.put<int64_t>(s.update_count);
  w.put<int64_t>(s.right_looking_hazards);
  w.put<double>(s.flops_refactor);
  uint32_t count = 1;  // upd_ptr
  for_each_int_array(s, [&](const char*, const std::vector<int>&) { count++; });
  w.put(count);
  auto array = [&](const char* name, const void* data, uint8_t esize, uint64_t len) {
    const uint16_t nl = (uint16_t)std::strlen(name);
    w.put(nl);
    w.bytes(name, nl);
    w.put(esize);
    w.put(len);
    w.bytes(data, (size_t)esize * len);
  };
  for_each_int_array(s, [&](const char* name, const std::vector<int>& v) {
    array(name, v.data(), 4, v.size());
  });
  array("upd_ptr", s.upd_ptr.data(), 8, s.upd_ptr.size());
  const uint64_t h = fnv1a(w.buf.data(), w.buf.size());
  w.put(h);
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    err = std::string("cannot open ") + path + " for writing";
    return ERR_BAD_ARG;
  }
  const size_t wrote = std::fwrite(w.buf.data(), 1, w.buf.size(), f);
  const int closed = std::fclose(f);
  if (wrote != w.buf.size() || closed != 0) {
    err = std::string("short write to ") + path;
    return ERR_BAD_ARG;
  }
  return OK;
}

int load_symbolic(const char* path, Symbolic& s, std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open ") + path;
    return ERR_BAD_ARG;
  }
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  std::fclose(f);
  if (buf.size() < sizeof kMagic + 8 + 8 || std::memcmp(buf.data(), kMagic, sizeof kMagic)) {
    err = "not a pvglu symbolic dump";
    return ERR_BAD_ARG;
  }
  uint64_t stored;
  std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
  if (stored != fnv1a(buf.data(), buf.size() - 8)) {
    err = "symbolic dump is corrupt (hash mismatch)";
    return ERR_BAD_ARG;
  }
  Reader r{buf.data() + sizeof kMagic, buf.size() - sizeof kMagic - 8};
  uint32_t version = 0, order = 0;
  r.get(version);
  r.get(order);
  if (!r.ok || version != kVersion || order != kOrder) {
    err = "unsupported dump version or byte order";
    return ERR_BAD_ARG;
  }
  s = Symbolic();
  int64_t n, row_swaps, invol;
  r.get(n);
  r.get(s.nnz_a);
  r.get(s.nnz_lu);
  r.get(row_swaps);
  r.get(invol);
  r.get(s.update_count);
  r.get(s.right_looking_hazards);
  r.get(s.flops_refactor);
  // The counts are stored as int64 and held as int: refuse what int cannot
  // hold instead of truncating it (the hash is no defence against a crafted
  // file).
  if (!r.ok || n < 0 || n > INT_MAX || row_swaps < 0 || row_swaps > INT_MAX || invol < 0 ||
      invol > 1 || s.nnz_a < 0 || s.nnz_lu < 0 || s.update_count < 0) {
    err = "symbolic dump is malformed (counts out of range)";
    return ERR_BAD_ARG;
  }
  s.n = (int)n;
  s.row_swaps = (int)row_swaps;
  s.perm_rows_is_involution = (int)invol;
  uint32_t count = 0;
  r.get(count);
  std::map<std::string, std::vector<int>*> ints;
  for_each_int_array(s, [&](const char* name, std::vector<int>& v) { ints[name] = &v; });
  for (uint32_t a = 0; r.ok && a < count; a++) {
    uint16_t nl = 0;
    uint8_t esize = 0;
    uint64_t len = 0;
    r.get(nl);
    std::string name(nl, '\0');
    r.bytes(&name[0], nl);
    r.get(esize);
    r.get(len);
    if (!r.ok || len > r.left / (esize ? esize : 1)) break;
    if (name == "upd_ptr" && esize == 8) {
      s.upd_ptr.resize(len);
      r.bytes(s.upd_ptr.data(), 8 * len);
    } else if (ints.count(name) && esize == 4) {
      ints[name]->resize(len);
      r.bytes(ints[name]->data(), 4 * len);
    } else {
      r.ok = false;
    }
  }
  std::string why;
  if (!r.ok || r.left != 0 || !consistent(s, why)) {
    err = "symbolic dump is malformed" + (why.empty() ? std::string() : " (" + why + ")");
    s = Symbolic();
    return ERR_BAD_ARG;
  }
  return OK;
}

}  // namespace pvglu
