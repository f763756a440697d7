// kernels.h -- host-side launchers of the sm_103a kernels (fluid.cu,
// linear.cu, advection.cu).  All pointers are device pointers; every
// launcher enqueues on `st` and returns the launch status.
#pragma once

#include <cuda_runtime.h>

#include "../../include/hydro_gpu.h"
#include "common.cuh"

namespace hg {

#define HYDRO_MAXPH 4

// Pointer tables passed by value as kernel parameters: RT reads, WT writes.
template <class T, int N>
struct RT {
  const T* a[N];
};
template <class T, int N>
struct WT {
  T* a[N];
};
template <int N>
using CP = RT<double, N>;
template <int N>
using WP = WT<double, N>;
template <int N>
using FP = WT<float, N>;
using C3 = CP<3>;
using W3 = WP<3>;

// Per-case constants of the momentum / pressure-correction kernels, in the
// arithmetic type of the kernel that reads them.
template <class T>
struct FluidCoefT {
  T bcu[6][3];  // wall velocity per side and component
  T relax_u;    // velocity_relaxation_factor
  T relax_p;    // pressure_relaxation_factor
  T rc;         // rhie_chow_factor
  T co[3];      // BDF coefficients for (n-1, n, n+1)
  T meshvel[3];
  int geometric;  // force_geometric_average
  int sources;    // volume/mass sources present
};
using FluidCoef = FluidCoefT<double>;

// Boundary-condition kinds and given velocities per side (xm, xp, ym, yp,
// zm, zp).
struct BcSpec {
  int kind[6];
  double vel[6][3];
};

// Device scalars shared by reductions and convergence flags.
struct DevScalars {
  double red[32];        // reduced values (see enum below)
  int flag[32];          // done flags / counters
  unsigned ticket[32];   // grid-reduction tickets, one per call site
};
enum {
  RS_MOM_DIFF = 0,       // max |update| of the last momentum sweep
  RS_PCG_RZ = 1, RS_PCG_RZ_OLD = 2, RS_PCG_PAP = 3, RS_PCG_RR = 4, RS_PCG_FF = 5,
  RS_PCG_ALPHA = 6, RS_PCG_BETA = 7,
  RS_INDICATOR = 8,      // SIMPLE convergence indicator
  RS_AUTO_DT = 9,
  RS_MEAN = 10,          // mean of the right-hand side (singular systems)
  RS_PCG_TOL2 = 11,      // tol^2 * ||f||^2
  RS_IR_RR = 12,         // refinement residual norm^2
  RS_NAN = 13,
  RS_XMEAN = 14,
  RS_INNER_TOL = 15,     // tolerance of the next inner solve (device-driven refinement)
  RS_P_RES = 16,         // relative pressure residual of the last solve
  RS_IR_FF = 17,         // refinement: ||f||^2 of the first residual
  RS_OUT_FLUX = 18, RS_OUT_AREA = 19, RS_IN_FLUX = 20,  // outlet rebalancing sums
  RS_HEAT_DIFF = 21,     // max |update| of the last temperature sweep
  RS_MOM_DIFF_RED = 22,  // max |update| of the red half of a Gauss-Seidel sweep
  RS_GUESS_S0 = 23, RS_GUESS_S1 = 24,  // <x, f'>, <x, A x> of a learned initial guess
  RS_MG0_SCALE = 25,     // power-of-two scale of the FP16 finest-level couplings
  RS_PCG_RRREF = 26,     // inner multigrid CG: ||r||^2 at its last halving
  RS_KEXEC = 27          // kernels run by the conditional bodies of captured graphs (each
                         // body's closing control kernel adds its count per run; exact below 2^53)
};
enum {
  FL_MOM_DONE = 0, FL_MOM_SWEEPS = 1, FL_PCG_DONE = 2, FL_PCG_ITERS = 3, FL_NAN = 4,
  FL_PCG_LIMIT = 5,      // iteration limit of the running Krylov solve
  FL_IR_STATE = 6,       // refinement: 0 before its first residual
  FL_IR_TOTAL = 7,       // refinement: inner iterations so far
  FL_STEP_SWEEPS = 8,    // momentum sweeps of the step (graph-captured step)
  FL_STEP_PITERS = 9,    // pressure iterations of the step
  FL_ITERS = 10,         // SIMPLE iterations of the step
  FL_IR_OUTER = 11,      // refinement cycles
  FL_CONT = 12,          // last loop decision
  FL_HEAT_DONE = 13, FL_HEAT_SWEEPS = 14,  // temperature solve
  FL_STEP_PUNCONV = 15,  // pressure solves of the step that stopped above their tolerance
  FL_STEP_NAN = 16,      // a pressure solve of the step met a NaN residual
  FL_GUESS_USED = 17, FL_GUESS_DROPPED = 18,  // learned initial guesses kept / dropped
  // back-off of the learned guess: after a dropped guess the next
  // FL_GUESS_SKIP steps run without it (1, 2, 4, ... 16 steps; a kept guess
  // resets it); FL_GUESS_OFF: the current step skips it
  FL_GUESS_SKIP = 19, FL_GUESS_BACKOFF = 20, FL_GUESS_OFF = 21,
  FL_GUESS_SKIPPED = 22, // steps that skipped the guess
  FL_PCG_REFIT = 23      // inner multigrid CG: iteration of its last halving of ||r||
};
enum {
  TK_MOM = 0, TK_PCG_A = 1, TK_PCG_B = 2, TK_PCG_INIT = 3, TK_IND = 4, TK_DT = 5,
  TK_MEAN = 6, TK_MEAN2 = 7, TK_STAT = 8, TK_STAT2 = 9, TK_STAT3 = 10, TK_IR = 11,
  TK_NAN = 12, TK_PCG_INIT2 = 13, TK_F32_A = 14, TK_F32_B = 15, TK_F32_INIT = 16,
  TK_OUTLET = 17, TK_HEAT = 18, TK_MOM_RED = 19, TK_GUESS = 20, TK_MG0 = 21
};

// ---------------------------------------------------------------- fluid --
cudaError_t launch_start_step(const Mesh& m, double ge, W3 u_ic, C3 u_tc, C3 u_tp,
                              double* p_ic, const double* p_tc, const double* p_tp,
                              double* F_ic, const double* F_tc, const double* F_tp,
                              cudaStream_t st);
// bv: per-face value conditions of the velocity (boundary entries used)
cudaError_t launch_init_flux(const Mesh& m, const FluidCoef& fc, C3 u, C3 bv, double* F,
                             cudaStream_t st);
cudaError_t launch_bc_fill(const Mesh& m, const BcSpec& sp, W3 bv, FP<3> bv32, cudaStream_t st);
cudaError_t launch_qin_fill(const Mesh& m, const BcSpec& sp, int nph, CP<HYDRO_MAXPH> q,
                            WP<HYDRO_MAXPH> qin, cudaStream_t st);
// UpdateOutletBaseConditions: outlet faces from the latest iterate u, then
// the uniform normal correction (bv32, when set, mirrors bv in FP32).
cudaError_t launch_outlet_update(const Mesh& m, const BcSpec& sp, C3 u, W3 bv, FP<3> bv32,
                                 const double* Sv, double* partials, DevScalars* ds,
                                 cudaStream_t st);
// The SIMPLE-iteration kernels, templated on the arithmetic type: double
// for the FP64 path, float for the mixed path (FP32 shadows of the state).
template <class T>
cudaError_t launch_vel_grad(const Mesh& m, const FluidCoef& fc, RT<T, 3> u, RT<T, 3> bv,
                            WT<T, 9> G, cudaStream_t st);
template <class T>
cudaError_t launch_force(const Mesh& m, const FluidCoef& fc, RT<T, 3> u, RT<T, 9> G,
                         const double* p, const T* mu, const T* rho, RT<T, 3> force,
                         RT<T, 3> stforce, const T* Sv, const T* Sm, WT<T, 3> fo,
                         WT<T, 3> fres, W3 gp, cudaStream_t st);
// coef = {1/diag, 2*DIM off-diagonals}, res = DIM residuals; up64/utc64/
// utp64 are the FP64 velocity layers of the residual's time difference
template <class T>
cudaError_t launch_mom_assemble(const Mesh& m, const FluidCoef& fc, RT<T, 3> u_prev,
                                RT<T, 3> u_tc, RT<T, 3> u_tp, RT<T, 9> G, const T* F,
                                const T* rho, const T* mu, RT<T, 3> fo, C3 up64, C3 utc64,
                                C3 utp64, RT<T, 3> bv, WT<T, 7> coef, WT<T, 3> res, T* Dc,
                                int split, cudaStream_t st);
// u_prev, p, gp (cell pressure gradient from launch_force) are FP64
template <class T>
cudaError_t launch_rhie_chow(const Mesh& m, const FluidCoef& fc, C3 u_prev, RT<T, 3> du,
                             const double* p, C3 gp, RT<T, 3> force, RT<T, 3> fres,
                             const T* Dc, C3 bv, double* Fs, double* kf, float* kf32,
                             cudaStream_t st);
cudaError_t launch_d2f(long long n, const double* in, float* out, cudaStream_t st);
// Mixed path: FP32 Jacobi sweep on the o32 output of the assembly
// (o32 = {1/diag, 2*DIM off-diagonals, DIM residuals}); FP32 -> FP64 copy.
// The whole Jacobi loop of launch_mom_sweep32 (sweeps until converged or
// `limit`) by one CTA of `threads` threads (or a cluster of `cluster` such
// CTAs), for a plain block; with graph
// set it also adds its sweeps to FL_STEP_SWEEPS.
cudaError_t launch_cta_mom_jacobi32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> d0,
                                    FP<3> d1, int limit, int graph, int threads, int cluster,
                                    DevScalars* ds, cudaStream_t st);
cudaError_t launch_mom_sweep32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> din,
                               FP<3> dout, int limit, double* partials, DevScalars* ds,
                               cudaStream_t st);
cudaError_t launch_f2d3(const Mesh& m, FP<3> in, W3 out, cudaStream_t st);
// Red-black Gauss-Seidel half-sweep of the momentum corrections (the
// parallel ordering of GaussSeidel::Solve, linear.hpp:671-716), in place on
// du: the cells of `color` ((i+j+k) % 2) from the other color's current
// values, x += omega (value - x).  The red half keeps its max |value - x| in
// RS_MOM_DIFF_RED, the black half completes the sweep's max and the exit
// rules of launch_mom_sweep.  split: the coefficients and residuals are
// stored color-blocked (index color * nc/2 + c/2; nx even), the layout the
// assembly writes for this solver (FP32 always, FP64 without SIMPLER);
// launch_mom_rbgs32 is always split, and keeps du color-blocked too.
cudaError_t launch_mom_rbgs(const Mesh& m, double omega, double tol, CP<7> coef, C3 res, W3 du,
                            int color, int split, int limit, double* partials, DevScalars* ds,
                            cudaStream_t st);
// Color-blocked FP32 vectors (the momentum corrections of launch_mom_rbgs32)
// back to cell order; nx even.
cudaError_t launch_unsplit3(const Mesh& m, FP<3> in, FP<3> out, cudaStream_t st);
cudaError_t launch_mom_rbgs32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> du,
                              int color, int limit, double* partials, DevScalars* ds,
                              cudaStream_t st);
cudaError_t launch_mom_sweep(const Mesh& m, double omega, double tol, CP<7> coef, C3 res,
                             C3 din, W3 dout, int limit, double* partials, DevScalars* ds,
                             cudaStream_t st);
cudaError_t launch_pressure_rhs(const Mesh& m, const double* Fs, const double* Sv, double* f,
                                cudaStream_t st);
// du32/Dc32 non-null: FP32 velocity correction and D_c of the mixed path;
// u32, p32, F32 non-null: also write those FP32 shadows of the iterate.
cudaError_t launch_correct(const Mesh& m, const FluidCoef& fc, C3 u_prev, C3 du,
                           RT<float, 3> du32, const float* Dc32, W3 u_ic, const double* p_ip,
                           double* p_ic, const double* pc, const double* Dc, const double* Fs,
                           const double* kf, const float* kf32, double* F_ic, FP<3> u32,
                           float* p32, float* F32, double* partials, DevScalars* ds,
                           cudaStream_t st);
cudaError_t launch_auto_dt(const Mesh& m, const double* F, double* partials, DevScalars* ds,
                           cudaStream_t st);
// SIMPLER (FP64 path): right-hand side f of the delta-form pressure solve
// A x = f around the corrected pressure p; ev: dim cell arrays of scratch.
cudaError_t launch_simpler_rhs(const Mesh& m, const FluidCoef& fc, CP<7> coef, C3 res, C3 uic,
                               C3 up, C3 fres, C3 gp, C3 force, const double* Dc,
                               const double* Fic, const double* kf, const double* dg,
                               const double* p, long long pin, double pin_value, W3 ev,
                               double* f, cudaStream_t st);
cudaError_t launch_add(long long n, double* a, const double* b, cudaStream_t st);
cudaError_t launch_nan_count(long long n, const double* a, double* partials, DevScalars* ds,
                             cudaStream_t st);

// ----------------------------------------------------------- properties --
struct PhaseProps {
  double dens[HYDRO_MAXPH], idens[HYDRO_MAXPH], visc[HYDRO_MAXPH], grav[3], f0[3];
};
cudaError_t launch_props(const Mesh& m, int nph, const PhaseProps& pp,
                         CP<HYDRO_MAXPH> q, WP<HYDRO_MAXPH> alpha, double* rho_raw,
                         double* rho, double* mu, W3 force, double* Sv, double* Sm,
                         cudaStream_t st);
cudaError_t launch_smooth(const Mesh& m, const double* in, double* out, cudaStream_t st);
cudaError_t launch_stforce(const Mesh& m, double sigma, const double* alpha1, W3 G,
                           W3 out, cudaStream_t st);
// out (device): [10 sums, min, max]; partials >= 12*kMaxBlocks doubles;
// ticket[3]; F: time_curr volume fluxes
cudaError_t launch_stat(const Mesh& m, const double* q, const double* alpha, C3 u,
                        const double* F, double* partials, double* out, unsigned* ticket,
                        cudaStream_t st);

// ----------------------------------------------------------------- heat --
// Temperature boundary condition (hydro2d.hpp:660-677): a boundary face
// holds the box temperature when its centre lies in the heat box
// (Rect::IsInside, inclusive, vect.hpp:239-246), else a zero derivative.
// Face centres on a side share that side's coordinate and the transverse
// cell-centre coordinates, so the faces inside are: the sides whose plane
// meets the box (side_in) and, on them, transverse cell indices i_k in
// [a[k], b[k]).  Faces beside excluded cells (rigid box) are tested by
// their centre against [lo, hi].
struct HeatBc {
  int side_in[6];
  int a[3], b[3];
  double lo[3], hi[3];
  double value;
};
struct HeatCoef {
  double cond[HYDRO_MAXPH];  // conductivity per phase
  double co[3];              // BDF coefficients of the heat time step
  double relax;              // heat_relaxation_factor
};
// conductivity kc = sum_i k_i alpha_i (hydro2d.hpp:1428)
cudaError_t launch_heat_conductivity(const Mesh& m, int nph, const HeatCoef& hc,
                                     CP<HYDRO_MAXPH> alpha, double* kc, cudaStream_t st);
// cell gradient of T with faces carrying the temperature condition
cudaError_t launch_heat_grad(const Mesh& m, const HeatBc& bc, const double* T, W3 G,
                             cudaStream_t st);
// delta-form rows of the temperature equation around T_prev
// (ConvectionDiffusionScalarImplicit::MakeIteration, conv_diff.hpp:130-251):
// coef = [1/(aP/relax), 2*DIM off-diagonals], res = equation at T_prev
cudaError_t launch_heat_assemble(const Mesh& m, const HeatBc& bc, const HeatCoef& hc,
                                 const double* Tp, const double* Ttc, const double* Ttp,
                                 const double* F, const double* kc, C3 G, WP<7> coef,
                                 double* res, cudaStream_t st);
// Jacobi sweep of the temperature correction (omega 1), the same exit
// rules as launch_mom_sweep on FL_HEAT_DONE / FL_HEAT_SWEEPS
cudaError_t launch_heat_sweep(const Mesh& m, double tol, CP<7> coef, const double* res,
                              const double* din, double* dout, int limit, double* partials,
                              DevScalars* ds, cudaStream_t st);
// T_prev <- T_curr, T_curr <- T_curr + du, du the buffer the last sweep
// wrote (du0 after an odd number of sweeps, else du1)
cudaError_t launch_heat_finish(long long n, double* tc, double* tp, const double* du0,
                               const double* du1, const DevScalars* ds, cudaStream_t st);

// ------------------------------------------------------------ advection --
// Face fluxes q_f F_f of every phase (Superbee, solver.hpp:550-619) on the
// faces of direction `stage` (all directions when nstages == 1).
// inlet_mask: bit q set when side q is an inlet; qin: inlet values on
// those boundary faces, per phase
cudaError_t launch_adv_faces(const Mesh& m, int nph, int stage, int nstages, const double* F,
                             CP<HYDRO_MAXPH> q, int inlet_mask, CP<HYDRO_MAXPH> qin,
                             WP<HYDRO_MAXPH> qflux, cudaStream_t st);
cudaError_t launch_adv_update(const Mesh& m, int nph, int stage, int nstages, double dt,
                              CP<HYDRO_MAXPH> qflux, CP<HYDRO_MAXPH> qin,
                              WP<HYDRO_MAXPH> qout, cudaStream_t st);
// Interface sharpening (advection.hpp:481-530), in place on q (work: 1 face
// array + DIM cell arrays + 1 cell array).
cudaError_t launch_adv_sharpen(const Mesh& m, int phase, double sharp, double amax, double dt,
                               const double* F, double* q, double* qtmp, W3 G,
                               double* fwork, cudaStream_t st);

// --------------------------------------------------------------- linear --
// Pressure-correction solve on face couplings kf (coupling -kf between the
// cells of an inner face, diagonal sum kf + shift), A x = f.
// Optional timing of kernel groups with CUDA events (measurement only).
struct Profiler {
  virtual void begin(int group, cudaStream_t st) = 0;
  virtual void end(int group, cudaStream_t st) = 0;
  virtual ~Profiler() {}
};
// Kernel launches issued by this library since load (all contexts).
void count_launches(long long n);
// Kernels this library enqueued so far (every launcher counts its own).
long long launch_total();

struct PcgWork {
  double *r, *z, *p, *Ap, *dg, *idg;                     // FP64 vectors
  float *r32, *z32, *p32, *p32b, *Ap32, *dg32, *idg32, *x32, *kf32;  // FP32 inner solve
  int p32_parity;    // which of p32/p32b holds the current direction
  double* partials;  // >= 8 * kMaxBlocks doubles
  DevScalars* ds;
  long long pin;     // pinned cell or -1
  int limit;         // iteration limit of one (inner) solve
  Profiler* prof;    // may be null
};
// Diagonal and its reciprocal (plus FP32 copies of couplings when fp32).
cudaError_t pcg_prepare(const Mesh& m, const double* kf, double shift, PcgWork& w, int fp32,
                        cudaStream_t st);
// Plain FP64 PCG: init, then chunks of iterations with device-side early
// exit (ds->flag[FL_PCG_DONE], iterations in ds->flag[FL_PCG_ITERS]).
cudaError_t pcg_init(const Mesh& m, const double* kf, const double* f, double* x, int use_guess,
                     double tol, int singular, PcgWork& w, cudaStream_t st);
cudaError_t pcg_iterate(const Mesh& m, const double* kf, double* x, int chunk, PcgWork& w,
                        cudaStream_t st);
// mean(f) into ds->red[RS_MEAN]; x -= mean(x).
cudaError_t mean_sum(const Mesh& m, const double* f, PcgWork& w, cudaStream_t st);
cudaError_t sub_mean(const Mesh& m, double* x, PcgWork& w, cudaStream_t st);
// Mixed precision: FP64 residual r = f' - A x (||r||^2 in ds->red[RS_IR_RR];
// x null when the iterate is zero), FP32 PCG for A e = r to a relative
// tolerance, x += e.
cudaError_t ir_residual(const Mesh& m, const double* kf, const double* f, const double* x,
                        int singular, PcgWork& w, cudaStream_t st);
// Learned initial guess x of A x = f' (pc of the refinement): Galerkin
// scaling x *= alpha, alpha = <x, f'> / <x, A x> (x = 0 when alpha is not
// positive and finite), then -- after ir_residual(x) -- keep it only when its
// residual is below ||f'|| (ds->red[RS_IR_FF]); otherwise x = 0 and the
// residual vector and RS_IR_RR are those of the zero guess.  Counts in
// FL_GUESS_USED / FL_GUESS_DROPPED.
cudaError_t guess_scale(const Mesh& m, const double* kf, const double* f, double* x, int singular,
                        PcgWork& w, cudaStream_t st);
cudaError_t guess_accept(const Mesh& m, const double* f, double* x, int singular, PcgWork& w,
                         cudaStream_t st);
// Inner-solve start.  dev_params = 0: tolerance `tol` and limit `w.limit`
// from the host (stored on the device); 1: both already on the device
// (RS_INNER_TOL, FL_PCG_LIMIT, set by launch_ctl_refine).
cudaError_t f32_pcg_init(const Mesh& m, double tol, int dev_params, PcgWork& w, cudaStream_t st);
cudaError_t f32_pcg_iterate(const Mesh& m, int chunk, PcgWork& w, cudaStream_t st);
// One launch: p_new = z + beta p_old (z on the first iteration, read from
// the device's iteration count), Ap = A p_new, <p_new, Ap> -> alpha (FP32
// vectors, double-float dot).
cudaError_t cg32_dir_spmv(const Mesh& m, const float* kf, const float* dg, const float* z,
                          const float* pold, float* pnew, float* Ap, long long pin,
                          double* partials, DevScalars* ds, cudaStream_t st);

// ------------------------------------------------------------ multigrid --
constexpr int kMgMaxLevels = 12;
constexpr long long kMgBlockMax = 4096;    // levels this small run inside one CTA
constexpr long long kMgCoarseTarget = 64;  // coarsening stops at or below this
struct MgLevel {
  Mesh m;
  float *kf, *dg, *idg, *x, *b;
};
struct MgWork {
  int nlev;
  int top;                 // first level run inside one CTA (nlev: none)
  int smem_bytes;          // shared memory of that CTA
  int nsweep;              // (red, black) sweeps before / after the correction
  int coarse_sweeps;       // sweeps of the coarsest solve inside the CTA
  int coarse_sweeps_large; // sweeps when the coarsest level stays large
  MgLevel lev[kMgMaxLevels];
  // Finest level of a plain 3D block (no periodic direction, no excluded
  // cell, even n[0]) solved without a pinned cell: the iterate, right-hand
  // side and inverse diagonal stored colour-blocked (cell c at
  // colour * nc/2 + c/2, colour = (i+j+k) mod 2) and the face couplings in
  // FP16 scaled by a power of two, so that a half-sweep streams its own
  // colour's rows, the other colour's iterate and 2-byte couplings.  k16
  // null: not allocated (the mesh does not allow it); fast0: in use for
  // the current solve (set by mg_setup).
  unsigned short* k16[3];
  float* idg0;
  bool fast0;
  // inverse of the coarsest level's operator (rank-one completed for its
  // constant null space), dense, when that level has <= kMgCoarseTarget
  // cells and is not the top level; null otherwise
  float* cinv;
  bool cdense;
  // the solves of this context run as one CTA each (cta_pressure): no
  // colour-blocked finest level
  bool cta;
  int smem_cinv_off;  // offset (floats) of its copy in the CTA's shared memory
  // host-driven steps replay the launches of one V-cycle as a CUDA graph,
  // instantiated for these vectors (null until the first V-cycle)
  cudaGraphExec_t vc_exec;
  const float* vc_r;
  float* vc_z;
  long long vc_pin;
  DevScalars* vc_ds;
  bool vc_fast0;
  int vc_kernels;
};
Mesh mg_coarse_mesh(const Mesh& fine);
int mg_levels_for(const Mesh& m);
// Once per context: which levels run inside one CTA and that CTA's shared
// memory (set as the kernel's dynamic shared-memory limit).
cudaError_t mg_prepare(MgWork& mg);
// Coarse couplings and diagonals from level 0 (w.kf32 / dg32 / idg32).
cudaError_t mg_setup(MgWork& mg, PcgWork& w, cudaStream_t st);
// z = M^-1 r.  Inside a stream capture the launches join the capture;
// otherwise they are replayed as one graph (kernels back to back without a
// host launch between them).
cudaError_t mg_vcycle(MgWork& mg, const float* r, float* z, long long pin, DevScalars* ds,
                      cudaStream_t st);
void mg_release(MgWork& mg);
// Inner solve of the mixed path with the V-cycle as preconditioner:
// init from the FP64 residual in w.r, chunks of iterations into w.x32.
// The whole mixed pressure solve (FP64 refinement around the multigrid CG,
// x = the correction, mean-free when singular) by one CTA of `threads`
// threads, or one cluster of `cluster` such CTAs, for a plain block whose
// coarse levels fit the CTA's shared memory (mg.top < mg.nlev), after
// pcg_prepare(fp32) and mg_setup.  Leaves
// RS_P_RES, FL_PCG_ITERS (inner iterations), FL_PCG_DONE (converged) and
// with graph set adds to FL_STEP_PITERS / FL_STEP_PUNCONV / FL_STEP_NAN.
cudaError_t cta_pressure(const Mesh& m, const double* kf, const double* f, double* x,
                         int singular, double tol, double inner_min, int limit, int graph,
                         int threads, int cluster, PcgWork& w, MgWork& mg, cudaStream_t st);
cudaError_t mgcg_init(const Mesh& m, double tol, int dev_params, PcgWork& w, MgWork& mg,
                      cudaStream_t st);
cudaError_t mgcg_iterate(const Mesh& m, int chunk, PcgWork& w, MgWork& mg, cudaStream_t st);
cudaError_t f32_accumulate(const Mesh& m, double* x, PcgWork& w, cudaStream_t st);
// x += the inner multigrid CG's result (in the finest level's colour-blocked
// order when that level is in use, mg.fast0).
cudaError_t mgcg_accumulate(const Mesh& m, double* x, PcgWork& w, MgWork& mg, cudaStream_t st);
cudaError_t scale_vector(long long n, double* a, double s, cudaStream_t st);
// Right-hand side of a pinned cell (fluid.hpp:996-1014): f[pin] = value and
// the pinned value moved into the neighbours' rows.
cudaError_t pin_rhs(const Mesh& m, const double* kf, double* f, long long pin, double value,
                    cudaStream_t st);

// ------------------------------------------------------- loop control --
// One-thread kernels that take the decisions of the step's loops on the
// device.  Each writes its decision to ds->flag[FL_CONT] and, when `use`
// is set, to the graph conditional `h` of the WHILE node that repeats the
// loop (graph-captured step); the host-driven step reads the same flags.
// Momentum sweeps: continue while not converged and fewer than `limit`;
// accumulates the finished loop's sweeps into FL_STEP_SWEEPS when it stops.
cudaError_t launch_ctl_sweeps(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                              cudaStream_t st, int nk = 0);
// Krylov inner loop: continue while not done.
// The temperature sweep loop (FL_HEAT_DONE / FL_HEAT_SWEEPS).
cudaError_t launch_ctl_heat(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                            cudaStream_t st, int nk = 0);
cudaError_t launch_ctl_krylov(DevScalars* ds, cudaGraphConditionalHandle h, int use,
                              cudaStream_t st, int nk = 0);
// Refinement cycle after a residual: records ||f||^2 on the first call,
// the relative residual in RS_P_RES, adds the finished inner solve's
// iterations; continues while above `tol`, below `limit` iterations and 50
// cycles, then sets the next inner tolerance (>= inner_min) and limit.
cudaError_t launch_ctl_refine(DevScalars* ds, double tol, double inner_min, int limit,
                              cudaGraphConditionalHandle h, int use, cudaStream_t st, int nk = 0);
// End of a FP64 Krylov solve: RS_P_RES and FL_STEP_PITERS.
// Learned guess in a captured step: the IF node around it runs while the
// SIMPLE iteration count of the step is below `limit`; after the guess, the
// refinement loop's condition is decided again from the guess's residual.
cudaError_t launch_ctl_guess_gate(DevScalars* ds, int limit, cudaGraphConditionalHandle h,
                                  int use, cudaStream_t st);
cudaError_t launch_ctl_guess(DevScalars* ds, double tol, double inner_min, int limit,
                             cudaGraphConditionalHandle h, cudaStream_t st, int nk = 0);
// RS_IR_FF = RS_IR_RR (the residual of the zero guess, before a guess).
cudaError_t launch_store_ff(DevScalars* ds, cudaStream_t st);
cudaError_t launch_ctl_krylov_done(DevScalars* ds, cudaStream_t st);
// SIMPLE loop after an iteration: FL_ITERS += 1; continue while below
// `limit` and the indicator is not below `tol`.
cudaError_t launch_ctl_simple(DevScalars* ds, int limit, double tol,
                              cudaGraphConditionalHandle h, int use, cudaStream_t st, int nk = 0);
// The same for graph-captured loops with two conditionals (both set).
cudaError_t launch_ctl_simple2(DevScalars* ds, int limit, double tol,
                               cudaGraphConditionalHandle h1, cudaGraphConditionalHandle h2,
                               cudaStream_t st, int nk = 0);
// Sets a graph conditional (re-arms a loop nested in another loop's body).
cudaError_t launch_set_cond(cudaGraphConditionalHandle h, unsigned v, cudaStream_t st);
// Copies src to dst when the momentum sweep count is even (the last sweep
// wrote the second buffer), so the correction is always in the first.
cudaError_t launch_select_sweep(long long n, const double* src, double* dst, const float* src32,
                                float* dst32, const DevScalars* ds, cudaStream_t st);
// Copies src to dst when the SIMPLE iteration count is odd (the captured
// iterations alternate their layer buffers two by two).
cudaError_t launch_select_iter(long long n, const double* src, double* dst,
                               const DevScalars* ds, cudaStream_t st);

}  // namespace hg
