// desc.cpp -- hydro_desc_default: the defaults of examples/general.hydroconf
// for the in-scope keys of hydro_desc.  Plain C++ (no device code), so that
// host-only builds that bind the C-ABI -- the reference-side adapter's
// checks -- use the same defaults as the library.
#include <string.h>

#include "../../include/hydro_gpu.h"

extern "C" {

int hydro_desc_default(hydro_desc* d) {
  if (!d) return HYDRO_ERR_ARG;
  memset(d, 0, sizeof(*d));
  d->dim = 2;
  d->n[0] = 100; d->n[1] = 100; d->n[2] = 5;
  for (int k = 0; k < 3; ++k) { d->lo[k] = 0.; d->hi[k] = 1.; }
  for (int s = 0; s < 6; ++s) d->bc_kind[s] = HYDRO_BC_WALL;
  d->dt = 0.01;
  d->cfl = 0.5;
  d->cfl_advection = 0.5;
  d->velocity_relaxation_factor = 0.8;
  d->pressure_relaxation_factor = 0.9;
  d->rhie_chow_factor = 1.;
  d->time_second_order = 1;
  d->convergence_tolerance = 1e-2;
  d->num_iterations_limit = 10;
  d->velocity_solver = HYDRO_LINEAR_JACOBI;
  d->velocity_tolerance = 1e-3;
  d->velocity_iters_limit = 1000;
  d->velocity_omega = 1.;
  d->pressure_solver = HYDRO_LINEAR_CG;
  d->pressure_tolerance = 1e-8;
  d->pressure_iters_limit = 100000;
  d->pressure_omega = 1.;
  d->precision = HYDRO_FP64;
  d->pressure_fixed_cell = -1;
  d->num_phases = 1;
  for (int i = 0; i < HYDRO_MAX_PHASES; ++i) { d->density[i] = 1.; d->viscosity[i] = 1.; }
  d->density_smooth_times = 2;
  d->viscosity_smooth_times = 2;
  d->advection_enable = 1;
  d->advection_dt_factor = 0.1;
  return HYDRO_OK;
}

}  // extern "C"
