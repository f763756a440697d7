/* adapter_shim.c -- TEST INFRASTRUCTURE ONLY: the C-ABI entry points the
 * reference-side adapter (hydro_gb300/adapter/fluid_simple_gpu.hpp) calls,
 * forwarded to the CPU oracle (liboracle.so) so that the adapter can be
 * compiled against the reference's headers and run in a container that has
 * the reference tree but no GPU.  Linked only into oracle/_ref/
 * libhydro_ref_adapter.so (oracle/Makefile); never into the library, whose
 * own entry points have no CPU path.  What it checks is the adapter: its
 * construction from the reference's solver arguments, its field and layer
 * marshalling and its step sequence through the FluidSolver /
 * AdvectionSolverMulti interfaces, against the reference's FluidSimple on
 * the same case; the GPU library behind the same entry points is checked
 * against the oracle by the GPU tests. */
#include <stddef.h>

#include "../include/hydro_gpu.h"
#include "hydro_oracle.h"

int hydro_gpu_create(const hydro_desc* d, hydro_ctx** out) {
  return oracle_create(d, (oracle_ctx**)out);
}
int hydro_gpu_destroy(hydro_ctx* x) { return oracle_destroy((oracle_ctx*)x); }
int hydro_gpu_set_field(hydro_ctx* x, int f, int l, const double* s, size_t n) {
  return oracle_set_field((oracle_ctx*)x, f, l, s, n);
}
int hydro_gpu_get_field(hydro_ctx* x, int f, int l, double* s, size_t n) {
  return oracle_get_field((oracle_ctx*)x, f, l, s, n);
}
int hydro_gpu_init_state(hydro_ctx* x) { return oracle_init_state((oracle_ctx*)x); }
int hydro_gpu_set_time_step(hydro_ctx* x, double dt, double dta) {
  return oracle_set_time_step((oracle_ctx*)x, dt, dta);
}
int hydro_gpu_start_step(hydro_ctx* x) { return oracle_start_step((oracle_ctx*)x); }
int hydro_gpu_make_iteration(hydro_ctx* x) { return oracle_make_iteration((oracle_ctx*)x); }
int hydro_gpu_finish_step(hydro_ctx* x) { return oracle_finish_step((oracle_ctx*)x); }
int hydro_gpu_get_convergence_indicator(hydro_ctx* x, double* v) {
  return oracle_get_convergence_indicator((oracle_ctx*)x, v);
}
int hydro_gpu_get_auto_time_step(hydro_ctx* x, double* v) {
  return oracle_get_auto_time_step((oracle_ctx*)x, v);
}
int hydro_gpu_advection_substep(hydro_ctx* x) { return oracle_advection_substep((oracle_ctx*)x); }
int hydro_gpu_heat_create(hydro_ctx* x, const hydro_heat_desc* h) {
  return oracle_heat_create((oracle_ctx*)x, h);
}
int hydro_gpu_heat_step(hydro_ctx* x) { return oracle_heat_step((oracle_ctx*)x); }
