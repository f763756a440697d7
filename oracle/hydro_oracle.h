/*
 * hydro_oracle.h -- CPU oracle for the hydro time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (divfree/hydro, source/hydro2dmpi/{fluid,conv_diff,solver,linear,
 * advection,hydro2d}.hpp).  It is the checker that tests/, the smoke test and
 * the cpu_baseline leg of bench.py compare against; the product path
 * (libhydro_gpu.so) never links or calls it.
 *
 * Parity pin: tests/test_oracle_golden.py checks this restatement against
 * golden vectors produced by the reference's own headers compiled into
 * oracle/_ref (recipe: oracle/Makefile, generator: tests/golden/make_golden.py).
 *
 * Same case description, field ids and layouts as include/hydro_gpu.h.
 */
#ifndef HYDRO_ORACLE_H_
#define HYDRO_ORACLE_H_

#include "../include/hydro_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

int oracle_create(const hydro_desc* desc, oracle_ctx** out);
int oracle_destroy(oracle_ctx* ctx);
int oracle_set_field(oracle_ctx* ctx, int field, int layer, const double* src, size_t n);
int oracle_get_field(oracle_ctx* ctx, int field, int layer, double* dst, size_t n);
int oracle_init_state(oracle_ctx* ctx);
int oracle_update_properties(oracle_ctx* ctx);
int oracle_start_step(oracle_ctx* ctx);
int oracle_make_iteration(oracle_ctx* ctx);
int oracle_finish_step(oracle_ctx* ctx);
int oracle_get_convergence_indicator(oracle_ctx* ctx, double* out);
int oracle_get_iteration_count(oracle_ctx* ctx, int* out);
int oracle_is_converged(oracle_ctx* ctx, int* out);
int oracle_get_auto_time_step(oracle_ctx* ctx, double* out);
int oracle_set_time_step(oracle_ctx* ctx, double dt, double dt_advection);
int oracle_get_time(oracle_ctx* ctx, double* fluid_time, double* advection_time);
int oracle_advection_step(oracle_ctx* ctx, int* substeps);
int oracle_advection_substep(oracle_ctx* ctx);
int oracle_step(oracle_ctx* ctx, hydro_step_stats* stats);
/* HeatSolver (heat.hpp:18-94) attached to the case; oracle_step then runs
 * one heat step after advection (hydro2d.hpp:1607-1613). */
int oracle_heat_create(oracle_ctx* ctx, const hydro_heat_desc* hd);
int oracle_heat_step(oracle_ctx* ctx);
int oracle_heat_get_temperature(oracle_ctx* ctx, double* out, size_t n);
int oracle_calc_stat(oracle_ctx* ctx, hydro_stat* out);
/* GetSmoothField (solver.hpp:636-656) on a cell array, in place. */
int oracle_smooth_field(oracle_ctx* ctx, double* field, int repeat);
/* Same contract as hydro_gpu_stencil_solve, host arrays, CG in FP64. */
int oracle_stencil_solve(int dim, int nx, int ny, int nz,
                         const double* face_coeff, double shift,
                         long pinned_cell, double pinned_value,
                         const double* rhs, double* x, int use_guess,
                         double tolerance, int iters_limit,
                         int* iterations, double* residual);
/* Threads used by the loops the reference parallelises with OpenMP. */
int oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
