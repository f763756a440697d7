/*
 * hydro_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of hydro's
 * time-step hot path: SIMPLE momentum assembly, pressure-correction solve,
 * velocity/flux correction and TVD partial-density advection on a uniform
 * Cartesian block (2D or 3D).
 *
 * Every entry point returns an int status (enum hydro_status).  Plain
 * pointers and sizes only; host arrays are in the reference's raw order:
 *   cell  (i,j,k)      -> i + Nx*(j + Ny*k)                  (mesh.hpp:552-561)
 *   faces              -> direction-blocked, x-faces first, each block
 *                         x-fastest over (N_d+1) in its own direction
 *                                                            (mesh.hpp:640-720)
 *   vector cell fields -> component-major (all x components, then y, then z).
 *                         The reference stores Vect per cell; the C++ adapter
 *                         (hydro_gb300/adapter/fluid_simple_gpu.hpp) converts.
 *
 * Reference interfaces replaced (paths inside divfree/hydro):
 *   hydro_gpu_create        FluidSimple ctor (source/hydro2dmpi/fluid.hpp:644-792)
 *                           + AdvectionSolverMultiExplicit ctor
 *                           (source/hydro2dmpi/advection.hpp:388-415)
 *   hydro_gpu_update_properties  hydro<Mesh>::UpdateFluidProperties
 *                           (source/hydro2dmpi/hydro2d.hpp:1404-1430)
 *   hydro_gpu_start_step    FluidSimple::StartStep (fluid.hpp:793-812)
 *   hydro_gpu_make_iteration FluidSimple::MakeIteration (fluid.hpp:814-1158)
 *   hydro_gpu_finish_step   FluidSimple::FinishStep (fluid.hpp:1159-1169)
 *   hydro_gpu_get_convergence_indicator
 *                           FluidSimple::GetConvergenceIndicator (fluid.hpp:1170-1172)
 *   hydro_gpu_get_iteration_count / hydro_gpu_is_converged
 *                           UnsteadyIterativeSolver (solver.hpp:710-751)
 *   hydro_gpu_get_auto_time_step FluidSimple::GetAutoTimeStep (fluid.hpp:1191-1206)
 *   hydro_gpu_set_time_step / hydro_gpu_get_time
 *                           UnsteadySolver (solver.hpp:679-708)
 *   hydro_gpu_advection_step AdvectionSolverMultiExplicit Start/MakeIteration/
 *                           Finish (advection.hpp:417-545)
 *   hydro_gpu_step          hydro<Mesh>::step (hydro2d.hpp:1531-1621)
 *   hydro_gpu_calc_stat     hydro<Mesh>::CalcStat (hydro2d.hpp:1432-1529)
 *   hydro_gpu_heat_create   hydro<Mesh>::InitHeatSolver (hydro2d.hpp:650-687)
 *   hydro_gpu_heat_step     HeatSolver StartStep/CalcStep/FinishStep
 *                           (heat.hpp:18-94, driven at hydro2d.hpp:1607-1613)
 *   hydro_gpu_get_field / hydro_gpu_set_field
 *                           FluidSolver::GetVelocity/GetPressure/GetVolumeFlux
 *                           (fluid.hpp:244-249), AdvectionSolverMulti::GetField
 *                           (advection.hpp:82), and the raw mixture-field
 *                           pointers the module hands to FluidSimple
 *                           (hydro2d.hpp:449-463)
 *   hydro_gpu_stencil_solve LinearSolver<Scal,IdxCell,Expr>::Solve
 *                           (linear.hpp:302-310) for symmetric 1+2d stencil rows
 */
#ifndef HYDRO_GPU_H_
#define HYDRO_GPU_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HYDRO_MAX_PHASES 4

enum hydro_status {
  HYDRO_OK = 0,
  HYDRO_ERR_ARG = 1,          /* invalid argument / unsupported size */
  HYDRO_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  HYDRO_ERR_NAN = 3,          /* NaN in pressure or velocity (fluid.hpp:795-797,1164-1166) */
  HYDRO_NOT_CONVERGED = 4,    /* a linear solve stopped at its iteration limit above its
                                 tolerance: the stencil solve; or a step (host-driven,
                                 graph-captured, batch) in which a pressure solve did so.
                                 Such a step is complete -- the reference goes on past a
                                 solver's limit too (linear.hpp:690-710) -- and its stats
                                 count the solves (pressure_unconverged) */
  HYDRO_ERR_UNSUPPORTED = 5,  /* option the GPU path does not implement */
  HYDRO_ERR_NOMEM = 6,        /* device allocation failed */
  HYDRO_ERR_NO_DEVICE = 7,    /* no CUDA device visible */
  HYDRO_ERR_IO = 8            /* an output file could not be written */
};

/* Sides of the block, in the reference's neighbour-face order
 * (mesh3d.hpp:297-303): xm, xp, ym, yp, zm, zp. */
enum hydro_side { HYDRO_XM = 0, HYDRO_XP, HYDRO_YM, HYDRO_YP, HYDRO_ZM, HYDRO_ZP };

/* Fluid boundary condition kinds (fluid.hpp:259-337, parsed at 392-417). */
enum hydro_bc_kind { HYDRO_BC_WALL = 0, HYDRO_BC_INLET = 1, HYDRO_BC_OUTLET = 2 };

/* Linear solvers.  The GPU has: for velocity GAUSS_SEIDEL (red-black sweeps)
 * and JACOBI; for pressure CG (Jacobi-preconditioned conjugate gradients)
 * and MGCG; for temperature JACOBI.  Any other choice is the reference's
 * CPU solver (the oracle has them all) and needs substitute_solvers. */
enum hydro_linear {
  HYDRO_LINEAR_GAUSS_SEIDEL = 0, /* linear.hpp:671-716 */
  HYDRO_LINEAR_JACOBI = 1,       /* linear.hpp:736-783 */
  HYDRO_LINEAR_CG = 2,           /* new: no Krylov solver in the reference */
  HYDRO_LINEAR_LU = 3,           /* linear.hpp:527-567 (one symmetric sweep) */
  HYDRO_LINEAR_MGCG = 4          /* new: CG preconditioned by a geometric multigrid
                                    V-cycle, in FP32, inside an FP64 iterative
                                    refinement (both precisions: the FP64 system
                                    is solved to the FP64 tolerance) */
};

/* Arithmetic of the SIMPLE iteration.  FP64: every kernel in FP64.  MIXED:
 * the assembly, the momentum sweeps and the pressure Krylov solve in FP32,
 * FP64 kept where the arithmetic cancels (BDF difference, pressure
 * gradients, face velocity, state updates) and for the refinement residual,
 * dots and norms of the pressure solve. */
enum hydro_precision { HYDRO_FP64 = 0, HYDRO_MIXED = 1 };

/* Field ids for get/set.  Vector fields have dim components (component-major). */
enum hydro_field {
  HYDRO_FIELD_VELOCITY = 0,        /* cells x dim; layers: all four */
  HYDRO_FIELD_PRESSURE = 1,        /* cells; layers: all four */
  HYDRO_FIELD_VOLUME_FLUX = 2,     /* faces; layers: all four */
  HYDRO_FIELD_PARTIAL_DENSITY = 3, /* cells x num_phases (phase-major); time_curr only */
  HYDRO_FIELD_VOLUME_FRACTION = 4, /* cells x num_phases, normalised (hydro2d.hpp:980-997) */
  HYDRO_FIELD_DENSITY = 5,         /* smoothed mixture density handed to the fluid solver */
  HYDRO_FIELD_VISCOSITY = 6,       /* smoothed mixture viscosity */
  HYDRO_FIELD_FORCE = 7,           /* cells x dim: body force rho*g + f (hydro2d.hpp:1308-1316) */
  HYDRO_FIELD_VOLUME_SOURCE = 8,   /* cells */
  HYDRO_FIELD_MASS_SOURCE = 9,     /* cells */
  HYDRO_FIELD_PRESSURE_CORRECTION = 10, /* cells: last p' solved */
  HYDRO_FIELD_DIAG_COEFF = 11,     /* cells: last momentum diagonal D_c (fluid.hpp:876-883) */
  HYDRO_FIELD_SURFACE_FORCE = 12,  /* cells x dim: surface-tension force (p_fc_stforce) */
  HYDRO_FIELD_TEMPERATURE = 13,    /* cells, layers TIME_CURR / TIME_PREV, after
                                      hydro_gpu_heat_create (HeatSolver::GetTemperature,
                                      heat.hpp:88-93) */
  HYDRO_FIELD_CONDUCTIVITY = 14,   /* cells, after hydro_gpu_heat_create: mixture
                                      conductivity (fc_conductivity, hydro2d.hpp:1428) */
  HYDRO_FIELD_PRESSURE_RHS = 15    /* cells: right-hand side f of the last pressure-
                                      correction solve, A p' = f (the pinned row
                                      included); with PRESSURE_CORRECTION and DENSITY
                                      the snapshot the learned guess trains on */
};

/* Same order as solver::Layers (solver.hpp:762). */
enum hydro_layer {
  HYDRO_TIME_CURR = 0, HYDRO_TIME_PREV = 1, HYDRO_ITER_CURR = 2, HYDRO_ITER_PREV = 3
};

/* Case description: the in-scope keys of a .hydroconf script
 * (examples/general.hydroconf), as consumed by hydro<Mesh>::Init* and the
 * FluidSimple / AdvectionSolverMultiExplicit constructors. */
typedef struct hydro_desc {
  int dim;                      /* 2 or 3 */
  int n[3];                     /* Nx, Ny, Nz (Nz ignored when dim == 2) */
  double lo[3], hi[3];          /* domain A, B */

  int bc_kind[6];               /* enum hydro_bc_kind per side (condition_left, ...) */
  double bc_velocity[6][3];     /* wall / inlet velocity per side */

  double dt;                    /* fixed time step (dt) */
  int dt_auto;                  /* dt = cfl * min V/|F| each step (hydro2d.hpp:1536-1544) */
  double cfl, cfl_advection;
  double dt_max;                /* >0: cap on dt when dt_auto (the reference has none;
                                   at rest its auto step is 1e10, fluid.hpp:1192) */

  double velocity_relaxation_factor;
  double pressure_relaxation_factor;
  double rhie_chow_factor;
  int time_second_order;
  int force_geometric_average;
  double guess_extrapolation;
  double meshvel[3];
  double convergence_tolerance; /* SIMPLE: max |u_s - u_{s-1}| */
  int num_iterations_limit;     /* SIMPLE outer iterations per step */
  int simpler;                  /* SIMPLER pressure (fluid.hpp:1059-1155); FP64 only */

  int velocity_solver;          /* enum hydro_linear: GAUSS_SEIDEL sweeps red-black
                                   Gauss-Seidel in place (mixed precision: when n[0] is
                                   even, else Jacobi); JACOBI and LU sweep Jacobi (LU is
                                   sequential).  With a tight velocity_tolerance all reach
                                   the same solution */
  double velocity_tolerance;    /* max |update| per sweep */
  int velocity_iters_limit;
  double velocity_omega;        /* relaxation of the sweep */
  int pressure_solver;          /* enum hydro_linear */
  double pressure_tolerance;    /* CG: ||r||_2 <= tol*||b||_2; GS/Jacobi: max |update| */
  int pressure_iters_limit;
  double pressure_omega;
  int precision;                /* enum hydro_precision */

  int pressure_fixed_cell;      /* -1: none (pressure_fixed_point) */
  double pressure_fixed_value;

  int num_phases;
  double density[HYDRO_MAX_PHASES];
  double viscosity[HYDRO_MAX_PHASES];
  double gravity[3], force[3];
  double sigma;                 /* surface tension coefficient */
  int density_smooth_times, viscosity_smooth_times, force_smooth_times;

  int advection_enable;
  double advection_dt_factor;
  int tvd_split;
  double sharp;

  void* stream;                 /* cudaStream_t to run on; NULL = library-owned stream */
  /* periodic directions (mesh2d.hpp / mesh3d.hpp PERX, PERZ, compile-time
   * switches in the reference, any direction here): both boundary faces of a
   * periodic direction join its last and first cells, carry no condition
   * and are solved as inner faces.  Multigrid needs an even cell count
   * along a periodic direction to coarsen it. */
  int periodic[3];
  /* rigid box (hydro2d.hpp:306-423, keys box_A / box_B): cells whose centre
   * lies in [rigid_box_lo, rigid_box_hi] (inclusive) are excluded
   * (mesh3d.hpp:183-215): identity rows in the momentum and pressure
   * systems, their state left as it is; the faces between them and the
   * fluid are no-slip walls at rest; faces between excluded cells, and
   * boundary faces of excluded cells, carry nothing.  0: no box. */
  int rigid_box;
  double rigid_box_lo[3], rigid_box_hi[3];
  /* Solvers the GPU does not have: velocity LU (the reference's one-sweep
   * sequential approximate solve, linear.hpp:527-567), pressure
   * GAUSS_SEIDEL / JACOBI / LU (stopping on the max update,
   * linear.hpp:671-783), temperature GAUSS_SEIDEL / LU.  With 0 (the
   * default) such a description gives HYDRO_ERR_UNSUPPORTED (from
   * hydro_gpu_create, hydro_gpu_heat_create, hydro_gpu_batch_create); with
   * 1 the GPU substitutes Jacobi sweeps to velocity_tolerance (velocity,
   * temperature) and CG to the relative residual pressure_tolerance
   * (pressure).  A substitute reaches the reference's numbers only with
   * tight tolerances: with the reference's loose defaults (one LU sweep,
   * SOR to a max update of 1e-3) the fields differ. */
  int substitute_solvers;
  /* Linear solves of a small case by ONE CTA each: with 0 (the default)
   * every sweep and every Krylov iteration is a grid-wide launch; with a
   * thread count (32..1024, a multiple of 32) the whole velocity Jacobi
   * loop and the whole pressure solve (FP64 refinement around the
   * multigrid CG, with CTA-wide FP64 sums in place of the grid reductions)
   * each run as one launch of one CTA of that many threads.  For batches of
   * many small cases (hydro_gpu_batch_*), where each case then holds one SM
   * per solve instead of queueing hundreds of tiny launches.  Needs
   * precision MIXED, pressure solver MGCG, no periodic direction, no
   * rigid box and fewer than 2^24 cells (HYDRO_ERR_UNSUPPORTED otherwise);
   * the pressure solve's set-up (diagonals, coarse levels, the dense
   * coarsest inverse) runs inside the same launch; a Gauss-Seidel velocity
   * solve stays grid-wide.  Results agree with the grid-wide form to the
   * solver tolerances, not bit for bit (other summation order). */
  int cta_threads;
  /* With cta_threads set: the number of CTAs (1, 2, 4 or 8; 0 means 1) of
   * the thread-block cluster that runs each of those solves -- the cluster's
   * threads share the passes, cluster barriers separate them, the coarse
   * multigrid levels run in the first CTA's shared memory.  A case's
   * coarse levels must fit that shared memory (HYDRO_ERR_UNSUPPORTED
   * otherwise). */
  int cta_cluster;
} hydro_desc;

typedef struct hydro_step_stats {
  int status;
  int outer_iterations;         /* SIMPLE iterations this step */
  double convergence_indicator; /* last max |u_s - u_{s-1}| */
  int velocity_sweeps;          /* total momentum sweeps */
  int pressure_iterations;      /* total pressure-solver iterations */
  double pressure_residual;     /* last relative residual of the pressure solve */
  int advection_substeps;
  double dt, dt_advection, time;
  int pressure_unconverged;     /* pressure solves of the step that stopped at their
                                   iteration limit above their tolerance (CG, MGCG) */
} hydro_step_stats;

typedef struct hydro_stat {
  /* hydro<Mesh>::CalcStat per phase (hydro2d.hpp:1432-1529) */
  double volume[HYDRO_MAX_PHASES];
  double mass[HYDRO_MAX_PHASES];
  double pd_min[HYDRO_MAX_PHASES], pd_max[HYDRO_MAX_PHASES];
  double center[HYDRO_MAX_PHASES][3];
  double velocity[HYDRO_MAX_PHASES][3];
  /* sum_c q_i(c) V_c in FP64: the quantity TVD advection conserves */
  double partial_mass[HYDRO_MAX_PHASES];
  /* volume flux of phase i into / out of the domain through the boundary
   * faces per unit time (hydro2d.hpp:1474-1493; the module accumulates them
   * times dt into stat_volume_in/out) */
  double volume_flux_in[HYDRO_MAX_PHASES], volume_flux_out[HYDRO_MAX_PHASES];
} hydro_stat;

typedef struct hydro_ctx hydro_ctx;

/* HeatSolver (heat.hpp:18-94) as hydro<Mesh>::InitHeatSolver sets it up
 * (hydro2d.hpp:650-687): temperature by ConvectionDiffusionScalarImplicit
 * with unit scaling, the fluid's volume fluxes and a face conductivity
 * interpolated from the mixture conductivity sum_i alpha_i k_i
 * (hydro2d.hpp:1428); boundary faces whose centre lies in [box_lo, box_hi]
 * (inclusive) hold box_temperature, the others zero derivative; one
 * iteration per step (the module creates it with limit 1). */
typedef struct hydro_heat_desc {
  double temperature_initial;
  double conductivity[HYDRO_MAX_PHASES];
  double box_lo[3], box_hi[3];
  double box_temperature;
  double relaxation_factor;     /* heat_relaxation_factor */
  int time_second_order;        /* time_second_order_heat */
  int solver;                   /* enum hydro_linear (the GPU uses Jacobi sweeps) */
  double tolerance;
  int iters_limit;
  double dt;                    /* the solver keeps the time step it is created with */
} hydro_heat_desc;

/* Fill *d with the defaults of examples/general.hydroconf for the keys above
 * (2D 100x100 unit square, walls, dt 0.01, relaxations 0.8/0.9, ...). */
int hydro_desc_default(hydro_desc* d);

int hydro_gpu_create(const hydro_desc* desc, hydro_ctx** out);
int hydro_gpu_destroy(hydro_ctx* ctx);

/* Copy a host array into / out of a field.  n = number of doubles. */
int hydro_gpu_set_field(hydro_ctx* ctx, int field, int layer, const double* src, size_t n);
int hydro_gpu_get_field(hydro_ctx* ctx, int field, int layer, double* dst, size_t n);
/* Device pointer of a field layer (no copy); NULL if the field is unknown. */
int hydro_gpu_field_ptr(hydro_ctx* ctx, int field, int layer, double** ptr);
/* The description the context was created with (d->stream: its stream). */
int hydro_gpu_get_desc(hydro_ctx* ctx, hydro_desc* d);
/* The CUDA stream (cudaStream_t) all of the context's work is ordered on;
 * work a caller enqueues on it runs after the context's pending steps. */
int hydro_gpu_get_stream(hydro_ctx* ctx, void** stream);
/* The fluid time step of the last / coming step (GetTimeStep). */
int hydro_gpu_get_time_step(hydro_ctx* ctx, double* dt);

/* Initial state: velocity (time_curr = time_prev = given), partial densities.
 * Computes the initial face fluxes (fluid.hpp:770-791) and then the mixture
 * properties.  Call once after set_field of the initial arrays. */
int hydro_gpu_init_state(hydro_ctx* ctx);

int hydro_gpu_update_properties(hydro_ctx* ctx);
int hydro_gpu_start_step(hydro_ctx* ctx);
int hydro_gpu_make_iteration(hydro_ctx* ctx);
int hydro_gpu_finish_step(hydro_ctx* ctx);
int hydro_gpu_get_convergence_indicator(hydro_ctx* ctx, double* out);
int hydro_gpu_get_iteration_count(hydro_ctx* ctx, int* out);
int hydro_gpu_is_converged(hydro_ctx* ctx, int* out);
int hydro_gpu_get_auto_time_step(hydro_ctx* ctx, double* out);
/* A value <= 0 leaves that time step unchanged. */
int hydro_gpu_set_time_step(hydro_ctx* ctx, double dt, double dt_advection);
int hydro_gpu_get_time(hydro_ctx* ctx, double* fluid_time, double* advection_time);
/* All advection substeps that bring advection time up to fluid time
 * (hydro2d.hpp:1596-1604). */
int hydro_gpu_advection_step(hydro_ctx* ctx, int* substeps);
/* Exactly one substep: AdvectionSolverMultiExplicit StartStep +
 * MakeIteration + FinishStep (advection.hpp:417-545). */
int hydro_gpu_advection_substep(hydro_ctx* ctx);

/* One full time step: dt_auto, SIMPLE loop to convergence, advection
 * substeps, property update.  stats may be NULL. */
int hydro_gpu_step(hydro_ctx* ctx, hydro_step_stats* stats);
/* The same step as one CUDA-graph launch (hydro<Mesh>::step,
 * hydro2d.hpp:1531-1621): the SIMPLE loop, momentum sweeps, refinement and
 * Krylov loops are graph WHILE nodes steered by device-side decisions, so
 * the host waits once per step.  Same results and stats as hydro_gpu_step.
 * The graph is captured on the first call and again whenever dt, the
 * advection substep count or the presence of sources changes.  Profiling
 * groups are not recorded inside it.  Afterwards the iteration layers hold
 * the final iterate in both ITER_CURR and, after an odd iteration count,
 * ITER_PREV; the time layers are as after hydro_gpu_step. */
int hydro_gpu_step_graph(hydro_ctx* ctx, hydro_step_stats* stats);
int hydro_gpu_calc_stat(hydro_ctx* ctx, hydro_stat* out);

/* ---- temperature ------------------------------------------------------
 * Attach a HeatSolver to the context: both temperature layers take
 * temperature_initial and the conductivity is computed from the current
 * volume fractions (call after hydro_gpu_init_state).  From then on every
 * step (hydro_gpu_step, hydro_gpu_step_graph, batch steps) advances the
 * temperature once after advection, with the fluid's final volume fluxes,
 * and the property update refreshes the conductivity.  A second call
 * re-initialises it with the new description.  The linear solve is Jacobi
 * sweeps for every `solver` value (tight tolerance: the same solution). */
int hydro_gpu_heat_create(hydro_ctx* ctx, const hydro_heat_desc* hd);
/* One temperature step alone (what the steps above run after advection). */
int hydro_gpu_heat_step(hydro_ctx* ctx);

/* ---- many independent cases ------------------------------------------
 * A batch of independent cases of uneven size (one hydro_desc each, e.g.
 * hundreds of small cavities), advanced together: every batch step is ONE
 * CUDA-graph launch in which each case's whole step (as in
 * hydro_gpu_step_graph) is an independent branch, so the GPU runs all cases
 * at once and the host waits once per batch step.  The reference has no
 * counterpart on its solver interface: it runs independent experiments as
 * one host thread per experiment (console.cpp:162-178, 922-965); each case
 * here behaves exactly like its own hydro_ctx stepped with hydro_gpu_step
 * (same results and stats).  Cases are reached with hydro_gpu_batch_case for
 * set_field / get_field / calc_stat; the batch owns them (do not destroy
 * them).  The batch graph is captured again when any case's dt, substep
 * count or sources change. */
typedef struct hydro_batch hydro_batch;
int hydro_gpu_batch_create(const hydro_desc* descs, int ncases, hydro_batch** out);
int hydro_gpu_batch_destroy(hydro_batch* batch);
int hydro_gpu_batch_size(hydro_batch* batch, int* ncases);
int hydro_gpu_batch_case(hydro_batch* batch, int index, hydro_ctx** out);
/* hydro_gpu_init_state of every case. */
int hydro_gpu_batch_init_state(hydro_batch* batch);
/* One step of every case; stats (may be NULL) receives ncases entries.
 * Returns the first non-OK case status. */
int hydro_gpu_batch_step(hydro_batch* batch, hydro_step_stats* stats);

/* ---- output in the reference's file formats ---------------------------
 * Fields: SessionParaviewStructured (output_paraview.hpp:34-175), one ASCII
 * .vts StructuredGrid file per frame named <basename>.<frame>.vts and the
 * collection <basename>.pvd.  `fields` lists entry names, comma or space
 * separated, of the reference's output_<name> flags (hydro2d.hpp:710-816):
 * x y z (nodes), velocity_x/y/z, pressure, density, viscosity,
 * volume_source, excluded, divergence, mass_fraction_<i>, density_<i>,
 * partial_density_<i>, volume_fraction_<i>; they are written in the
 * reference's order whatever the order of the list.  NULL or "" selects the
 * defaults of examples/general.hydroconf (x y [z] velocity_x velocity_y
 * [velocity_z] pressure volume_fraction_0 volume_fraction_1).  Names the hot
 * path does not compute (radiation, temperature, mass_source_<i>,
 * target_density_<i>) give HYDRO_ERR_UNSUPPORTED.
 * hydro_output_write copies the time_curr fields to pinned host memory on
 * a side stream ordered after the context's stream and returns; a worker
 * thread formats and writes the file while the GPU carries on (one frame in
 * flight: the next write, flush or close waits for it).  Values print as
 * the reference's ostream does (%g). */
typedef struct hydro_output hydro_output;
int hydro_output_open(hydro_ctx* ctx, const char* basename, const char* fields,
                      hydro_output** out);
int hydro_output_write(hydro_output* out, double time);
int hydro_output_flush(hydro_output* out);
/* Flushes, writes the collection footer, frees. */
int hydro_output_close(hydro_output* out);
/* One .vts frame from host arrays, synchronously: `nentries` arrays named
 * names[i], node arrays ((nx+1)(ny+1)[(nz+1)] values) where on_nodes[i],
 * else cell arrays; PointData first, then CellData, each in the given
 * order.  Needs no GPU. */
int hydro_vts_write_host(const char* path, int dim, const int* n, const double* lo,
                         const double* hi, int nentries, const char* const* names,
                         const int* on_nodes, const double* const* data);
/* Scalar series: SessionPlainScalar (output.hpp:231-261) with the entries of
 * hydro<Mesh> (hydro2d.hpp:825-905): time num_iters iter_diff_velocity,
 * per phase mass/mass_in/mass_out, volume/volume_in/volume_out,
 * pd_min/pd_max, centre and velocity components.  A row per write. */
typedef struct hydro_scalar_output hydro_scalar_output;
int hydro_scalar_output_open(hydro_ctx* ctx, const char* filename, hydro_scalar_output** out);
int hydro_scalar_output_write(hydro_scalar_output* out, double time, int num_iters);
int hydro_scalar_output_close(hydro_scalar_output* out);

/* Solve sum_j a_j x_j + c = 0 for a symmetric 7-point (3D) / 5-point (2D)
 * stencil on an nx*ny*nz block, the rows the pressure system has
 * (fluid.hpp:972-1027): coupling coefficients per face, diagonal implied as
 * the sum of the face couplings plus `shift`.
 *   face_coeff: device pointer, direction-blocked face array (same layout as
 *               volume fluxes); coupling of the two cells of an inner face is
 *               -face_coeff[f]; boundary-face entries are ignored.
 *   rhs:        device pointer, cells: the row constant c (so A x = -c).
 *   x:          device pointer, cells: output (initial guess on input when
 *               use_guess != 0).
 *   workspace:  device pointer of at least hydro_gpu_stencil_workspace_size()
 *               bytes.
 *   pinned_cell: -1, or a cell whose row is x = pinned_value with that value
 *               substituted into its neighbours' rows (the symmetric
 *               treatment of a fixed-pressure cell, fluid.hpp:996-1014).
 * Singular (shift == 0, no pinned cell) systems are solved in the subspace
 * orthogonal to the constants and return the zero-mean solution.  Returns HYDRO_NOT_CONVERGED when the limit is
 * hit; *iterations and *residual report the relative residual reached.
 * Returns HYDRO_ERR_NAN when the residual is not a number (a non-finite
 * input, or a row with neither couplings nor shift). */
size_t hydro_gpu_stencil_workspace_size(int dim, int nx, int ny, int nz);
int hydro_gpu_stencil_solve(int dim, int nx, int ny, int nz,
                            const double* face_coeff, double shift,
                            long pinned_cell, double pinned_value,
                            const double* rhs, double* x, int use_guess,
                            double tolerance, int iters_limit,
                            void* workspace, void* stream,
                            int* iterations, double* residual);

/* hydro_gpu_stencil_solve without a workspace argument, for callers that
 * cannot allocate device memory.  No counterpart in the reference (whose
 * solvers allocate host vectors on every call, linear.hpp:686).
 *
 * Who needs it: code that may not call cudaMalloc -- a plugin running
 * inside a host application that owns and budgets all device memory, or a
 * latency-critical loop where cudaMalloc's possible implicit device
 * synchronisation or out-of-memory failure is not acceptable.  The caller
 * still passes the inputs and the output (face_coeff, rhs, x: device
 * pointers); everything else the solve needs comes from one file-scope
 * device array of this library, 18,875,392 bytes (18 MiB), which every GPU
 * that loads the library holds until the process exits.
 *
 * Limits and rules:
 *  - at most HYDRO_NOALLOC_MAX_CELLS cells; larger blocks return
 *    HYDRO_ERR_ARG without touching the GPU;
 *  - every call looks up the array's device address in the calling
 *    thread's current device and context (cudaGetSymbolAddress), so the
 *    call follows cudaDeviceReset and contexts the host application makes
 *    current; the lookup allocates nothing;
 *  - like hydro_gpu_stencil_solve, the call waits for `stream` between
 *    chunks of iterations (it reads the convergence flags back to the
 *    host) and returns with the stream's work complete;
 *  - all calls share the one array, which keeps the last call's contents
 *    (each call clears what must start at zero itself); calls that overlap
 *    on the GPU -- two streams or host threads at once -- race on it, so
 *    the caller must serialise them;
 *  - it calls no cudaMalloc, cudaFree or allocating library routine.
 * Arguments, results and status codes are those of hydro_gpu_stencil_solve. */
#define HYDRO_NOALLOC_MAX_CELLS 262144
int hydro_gpu_stencil_solve_noalloc(int dim, int nx, int ny, int nz,
                                    const double* face_coeff, double shift,
                                    long pinned_cell, double pinned_value,
                                    const double* rhs, double* x, int use_guess,
                                    double tolerance, int iters_limit, void* stream,
                                    int* iterations, double* residual);

/* Measurement hooks (no counterpart in the reference; the reference's
 * MultiTimer labels fluid.0..fluid.8, fluid.hpp:603-1061, play this role
 * there).  With profiling on, every launch of the groups below is
 * bracketed by CUDA events on the context's stream; get_profile returns
 * the launches and summed device milliseconds of one group since the last
 * reset (multigrid V-cycles queued past the convergence of their Krylov
 * solve exit at once: their time is kept, their count is not).  The launch
 * count covers every kernel this library enqueued. */
enum hydro_prof_group {
  HYDRO_PROF_VEL_GRAD = 0, HYDRO_PROF_FORCE, HYDRO_PROF_MOM_ASSEMBLE, HYDRO_PROF_MOM_SWEEP,
  HYDRO_PROF_RHIE_CHOW, HYDRO_PROF_PRESSURE_RHS, HYDRO_PROF_CG_INIT, HYDRO_PROF_CG_SPMV,
  HYDRO_PROF_CG_UPDATE, HYDRO_PROF_CG_DIR, HYDRO_PROF_IR_RESIDUAL, HYDRO_PROF_CORRECT,
  HYDRO_PROF_ADV_FACES, HYDRO_PROF_ADV_UPDATE, HYDRO_PROF_PROPS, HYDRO_PROF_MG_VCYCLE,
  HYDRO_PROF_OTHER,
  HYDRO_PROF_GUESS,  /* learned initial guess of a pressure solve (hydro_net.h) */
  HYDRO_PROF_COUNT
};
int hydro_gpu_set_profiling(hydro_ctx* ctx, int on);
int hydro_gpu_reset_profile(hydro_ctx* ctx);
int hydro_gpu_get_profile(hydro_ctx* ctx, int group, long long* launches, double* ms);
int hydro_gpu_get_launch_count(long long* out);

#ifdef __cplusplus
}
#endif

#endif /* HYDRO_GPU_H_ */
