// Test driver of the drop-in shim's core (pvglu_shim_core.hpp): runs the
// exact call sequence of factorize_electrical_system_CUDA and
// triangular_substitution_LU_CUDA on arrays laid out as the reference's
// struct_CPU_CUDA_arrays holds them after prepare_matrices, with a stand-in
// struct that has the members the shim uses.
//
// usage: shim_driver <in.bin> <out.bin>
//   in:  int32 n, int32 nnz, int32 rowptr[n+1], int32 col[nnz],
//        f64 csc_values[nnz], f64 b_permuted[n]
//   out: f64 lu[nnz], f64 x_permuted[n], then the same two again from a
//        second factorize + solve on the same arrays (handles reused)
#include <cstdio>
#include <vector>

#include "pvglu_shim_core.hpp"

struct Arrays {  // the members of struct_CPU_CUDA_arrays the shim reads
  int n = 0;
  std::vector<int> mat_A_CSR_start_rows;
  std::vector<int> mat_A_CSR_position_columns;
  std::vector<double> mat_A_CSC_values;
};

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int n = 0, nnz = 0;
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(&nnz, 4, 1, f) != 1 || n <= 0 || nnz <= 0)
    return 4;
  Arrays a;
  a.n = n;
  a.mat_A_CSR_start_rows.resize(n + 1);
  a.mat_A_CSR_position_columns.resize(nnz);
  std::vector<double> csc(nnz), b(n);
  bool ok = std::fread(a.mat_A_CSR_start_rows.data(), 4, n + 1, f) == (size_t)n + 1 &&
            std::fread(a.mat_A_CSR_position_columns.data(), 4, nnz, f) == (size_t)nnz &&
            std::fread(csc.data(), 8, nnz, f) == (size_t)nnz &&
            std::fread(b.data(), 8, n, f) == (size_t)n;
  std::fclose(f);
  if (!ok) return 5;
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  pvglu_shim::State st;
  pvglu_numeric* first = nullptr;
  for (int round = 0; round < 2; round++) {
    a.mat_A_CSC_values = csc;
    std::vector<double> x = b;
    int rc = pvglu_shim::factorize(st, a);
    if (rc == PVGLU_OK) rc = pvglu_shim::solve(st, a, x.data());
    if (rc != PVGLU_OK) {
      std::fprintf(stderr, "round %d: status %d: %s\n", round, rc, pvglu_last_error());
      return 10 + rc;
    }
    if (round == 0) first = st.num;
    if (st.num != first) return 7;  // the second round must reuse the handles
    std::fwrite(a.mat_A_CSC_values.data(), 8, nnz, o);
    std::fwrite(x.data(), 8, n, o);
  }
  std::fclose(o);
  pvglu_shim::release(st);
  return 0;
}
