// Drop-in shim for the reference's simulator (PVPP_Plant_Simulator/): link it
// and libpvglu into the reference's binary in place of
// factorize_electrical_system_CUDA.cu and triangular_substitution.cu.  The
// two functions keep the reference's signatures
// (factorize_electrical_system.h:136-145) and host-in/host-out semantics;
// PVPP_Simulator (000_PVPP_simulator.cpp:207-231) calls them unchanged.
//
// Build (in the reference's directory, beside its other objects):
//   g++ -std=c++20 -O2 -I. -I<repo>/include -I<repo>/phdthesis_albertojimenezruiz_gb300/integration
//       -c <repo>/phdthesis_albertojimenezruiz_gb300/integration/pvglu_shim.cpp
//   link: -L<repo>/phdthesis_albertojimenezruiz_gb300 -lpvglu -Wl,-rpath,<that dir>
#include "factorize_electrical_system.h"  // struct_CPU_CUDA_arrays, Time_Measurer
#include "pvglu_shim_core.hpp"

namespace {
pvglu_shim::State g_state;

void check(int rc, const char* where) {
  if (rc != PVGLU_OK) abortmsg("%s: pvglu status %d: %s\n", where, rc, pvglu_last_error());
}
}  // namespace

// factorize_electrical_system.h:136-137
void factorize_electrical_system_CUDA(struct_CPU_CUDA_arrays& a, Time_Measurer& m) {
  m.measure("Before factorization");
  check(pvglu_shim::factorize(g_state, a), "factorize_electrical_system_CUDA");
  m.measure("After factorization");
}

// factorize_electrical_system.h:143-145.  solution_CUDA (the reference's
// device copy of the vector) is not needed: the library keeps its own.
void triangular_substitution_LU_CUDA(struct_CPU_CUDA_arrays& a, Time_Measurer& m,
                                     GPU_array_f* /*solution_CUDA*/, FLOATING_TYPE* solution) {
  m.measure("Before LU Substitution");
  check(pvglu_shim::solve(g_state, a, solution), "triangular_substitution_LU_CUDA");
  m.measure("After LU Substitution");
}
