// control.cu -- device-side loop decisions of one time step.
//
// The reference drives its loops from the host: the SIMPLE loop of
// hydro<Mesh>::step (hydro2d.hpp:1531-1621, IsConverged at
// solver.hpp:735-741), the linear solvers' iteration loops
// (linear.hpp:685-715, 750-782).  Here each decision is a one-thread kernel
// that reads the reduced scalars the previous kernels left in DevScalars and
// writes the decision to ds->flag[FL_CONT]; in a graph-captured step it also
// sets the conditional of the WHILE node that repeats the loop, so a whole
// step runs as one graph launch without host round trips.
#include <math.h>

#include "kernels.h"

namespace hg {

namespace {

// nk: kernels of the captured body this decision closes (0 outside a
// graph), added to ds->red[RS_KEXEC] on each run of the body.
__device__ __forceinline__ void decide(DevScalars* ds, int cont, cudaGraphConditionalHandle h,
                                       int use, int nk) {
  ds->flag[FL_CONT] = cont;
  if (use) {
    cudaGraphSetConditional(h, cont ? 1u : 0u);
    ds->red[RS_KEXEC] += (double)nk;
  }
}

__global__ void k_ctl_sweeps(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                             int nk) {
  if (threadIdx.x != 0) return;
  int sweeps = ds->flag[FL_MOM_SWEEPS];
  int cont = !(ds->flag[FL_MOM_DONE] || sweeps >= limit);
  if (!cont) ds->flag[FL_STEP_SWEEPS] += sweeps;
  decide(ds, cont, h, use, nk);
}

__global__ void k_ctl_heat(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                           int nk) {
  if (threadIdx.x != 0) return;
  decide(ds, !(ds->flag[FL_HEAT_DONE] || ds->flag[FL_HEAT_SWEEPS] >= limit), h, use, nk);
}

__global__ void k_ctl_krylov(DevScalars* ds, cudaGraphConditionalHandle h, int use, int nk) {
  if (threadIdx.x != 0) return;
  decide(ds, !ds->flag[FL_PCG_DONE], h, use, nk);
}

__global__ void k_ctl_krylov_done(DevScalars* ds) {
  if (threadIdx.x != 0) return;
  double ff = ds->red[RS_PCG_FF];
  ds->red[RS_P_RES] = ff > 0. ? sqrt(ds->red[RS_PCG_RR] / ff) : 0.;
  ds->flag[FL_STEP_PITERS] += ds->flag[FL_PCG_ITERS];
  if (!(ds->red[RS_PCG_RR] <= ds->red[RS_PCG_TOL2])) ds->flag[FL_STEP_PUNCONV] += 1;
  if (isnan(ds->red[RS_PCG_RR])) ds->flag[FL_STEP_NAN] = 1;
}

// Iterative refinement (the mixed pressure solve): called after every FP64
// residual; FL_IR_STATE = 0 marks the first residual of a solve.
__global__ void k_ctl_refine(DevScalars* ds, double tol, double inner_min, int limit,
                             cudaGraphConditionalHandle h, int use, int nk) {
  if (threadIdx.x != 0) return;
  double rr = ds->red[RS_IR_RR];
  int total;
  if (ds->flag[FL_IR_STATE] == 0) {
    ds->red[RS_IR_FF] = rr;
    ds->flag[FL_IR_STATE] = 1;
    ds->flag[FL_IR_TOTAL] = 0;
    ds->flag[FL_IR_OUTER] = 0;
    total = 0;
  } else {
    total = ds->flag[FL_IR_TOTAL] + ds->flag[FL_PCG_ITERS];
    ds->flag[FL_IR_TOTAL] = total;
    ds->flag[FL_STEP_PITERS] += ds->flag[FL_PCG_ITERS];
    ds->flag[FL_IR_OUTER] += 1;
  }
  double ff = ds->red[RS_IR_FF];
  ds->red[RS_P_RES] = ff > 0. ? sqrt(rr / ff) : 0.;
  if (isnan(rr)) ds->flag[FL_STEP_NAN] = 1;  // a NaN in the system (fluid.hpp:1164-1166)
  int conv = (ff == 0. || rr <= tol * tol * ff);
  int cont = !conv && !isnan(rr) && total < limit && ds->flag[FL_IR_OUTER] < 50;
  if (cont) {
    double t = 0.5 * tol * sqrt(ff / rr);
    ds->red[RS_INNER_TOL] = t > inner_min ? t : inner_min;
    ds->flag[FL_PCG_LIMIT] = limit - total;
  } else if (!conv) {
    ds->flag[FL_STEP_PUNCONV] += 1;  // stopped at a limit (or NaN) above the tolerance
  }
  decide(ds, cont, h, use, nk);
}

// Whether this SIMPLE iteration's pressure solve starts from the learned
// guess: the first `limit` iterations of a step, unless the step is one the
// back-off skips (decided at its first iteration).
// use = 0 (host-driven step): called at the step's first iteration only,
// for the back-off bookkeeping.
__global__ void k_ctl_guess_gate(DevScalars* ds, int limit, cudaGraphConditionalHandle h,
                                 int use) {
  if (threadIdx.x != 0) return;
  const int it = use ? ds->flag[FL_ITERS] : 0;
  if (it == 0) {
    const int off = ds->flag[FL_GUESS_SKIP] > 0;
    if (off) {
      ds->flag[FL_GUESS_SKIP] -= 1;
      ds->flag[FL_GUESS_SKIPPED] += 1;
    }
    ds->flag[FL_GUESS_OFF] = off;
  }
  if (use) cudaGraphSetConditional(h, (it < limit && !ds->flag[FL_GUESS_OFF]) ? 1u : 0u);
}

// The refinement loop's first decision, again, from the residual of the
// accepted guess (no inner iterations yet: the whole limit is left).
__global__ void k_ctl_guess(DevScalars* ds, double tol, double inner_min, int limit,
                            cudaGraphConditionalHandle h, int nk) {
  if (threadIdx.x != 0) return;
  const double rr = ds->red[RS_IR_RR], ff = ds->red[RS_IR_FF];
  ds->red[RS_P_RES] = ff > 0. ? sqrt(rr / ff) : 0.;
  const int conv = (ff == 0. || rr <= tol * tol * ff);
  const int cont = !conv && !isnan(rr) && limit > 0;
  if (cont) {
    const double t = 0.5 * tol * sqrt(ff / rr);
    ds->red[RS_INNER_TOL] = t > inner_min ? t : inner_min;
    ds->flag[FL_PCG_LIMIT] = limit;
  }
  decide(ds, cont, h, 1, nk);
}

__global__ void k_store_ff(DevScalars* ds) {
  if (threadIdx.x == 0) ds->red[RS_IR_FF] = ds->red[RS_IR_RR];
}

__global__ void k_ctl_simple(DevScalars* ds, int limit, double tol,
                             cudaGraphConditionalHandle h, int use, int nk) {
  if (threadIdx.x != 0) return;
  int it = ds->flag[FL_ITERS] + 1;
  ds->flag[FL_ITERS] = it;
  double ind = ds->red[RS_INDICATOR];
  int cont = !(it >= limit || ind < tol);
  decide(ds, cont, h, use, nk);
}

// Same decision, written to two conditionals: the IF node of the second
// iteration of a loop trip and the WHILE node of the trip.
__global__ void k_ctl_simple2(DevScalars* ds, int limit, double tol, cudaGraphConditionalHandle h1,
                              cudaGraphConditionalHandle h2, int nk) {
  if (threadIdx.x != 0) return;
  int it = ds->flag[FL_ITERS] + 1;
  ds->flag[FL_ITERS] = it;
  double ind = ds->red[RS_INDICATOR];
  int cont = !(it >= limit || ind < tol);
  ds->flag[FL_CONT] = cont;
  cudaGraphSetConditional(h1, cont ? 1u : 0u);
  cudaGraphSetConditional(h2, cont ? 1u : 0u);
  ds->red[RS_KEXEC] += (double)nk;
}

// A conditional's default value is applied once per graph launch, so a
// loop nested in another loop's body is re-armed before each entry.
__global__ void k_set_cond(cudaGraphConditionalHandle h, unsigned v) {
  if (threadIdx.x == 0) cudaGraphSetConditional(h, v);
}

__global__ void k_select_sweep(long long n, const double* src, double* dst, const float* src32,
                               float* dst32, const DevScalars* ds) {
  if (ds->flag[FL_MOM_SWEEPS] % 2 != 0) return;  // the last sweep wrote dst
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (src) dst[i] = src[i];
    if (src32) dst32[i] = src32[i];
  }
}

__global__ void k_select_iter(long long n, const double* src, double* dst,
                              const DevScalars* ds) {
  if (ds->flag[FL_ITERS] % 2 == 0) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

int copy_blocks(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

cudaError_t launch_ctl_sweeps(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                              cudaStream_t st, int nk) {
  k_ctl_sweeps<<<1, 32, 0, st>>>(ds, limit, h, use, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_heat(DevScalars* ds, int limit, cudaGraphConditionalHandle h, int use,
                            cudaStream_t st, int nk) {
  k_ctl_heat<<<1, 32, 0, st>>>(ds, limit, h, use, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_krylov(DevScalars* ds, cudaGraphConditionalHandle h, int use,
                              cudaStream_t st, int nk) {
  k_ctl_krylov<<<1, 32, 0, st>>>(ds, h, use, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_refine(DevScalars* ds, double tol, double inner_min, int limit,
                              cudaGraphConditionalHandle h, int use, cudaStream_t st, int nk) {
  k_ctl_refine<<<1, 32, 0, st>>>(ds, tol, inner_min, limit, h, use, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_guess_gate(DevScalars* ds, int limit, cudaGraphConditionalHandle h,
                                  int use, cudaStream_t st) {
  k_ctl_guess_gate<<<1, 32, 0, st>>>(ds, limit, h, use);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_guess(DevScalars* ds, double tol, double inner_min, int limit,
                             cudaGraphConditionalHandle h, cudaStream_t st, int nk) {
  k_ctl_guess<<<1, 32, 0, st>>>(ds, tol, inner_min, limit, h, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_store_ff(DevScalars* ds, cudaStream_t st) {
  k_store_ff<<<1, 32, 0, st>>>(ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_krylov_done(DevScalars* ds, cudaStream_t st) {
  k_ctl_krylov_done<<<1, 32, 0, st>>>(ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_simple(DevScalars* ds, int limit, double tol,
                              cudaGraphConditionalHandle h, int use, cudaStream_t st, int nk) {
  k_ctl_simple<<<1, 32, 0, st>>>(ds, limit, tol, h, use, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_ctl_simple2(DevScalars* ds, int limit, double tol,
                               cudaGraphConditionalHandle h1, cudaGraphConditionalHandle h2,
                               cudaStream_t st, int nk) {
  k_ctl_simple2<<<1, 32, 0, st>>>(ds, limit, tol, h1, h2, nk);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_set_cond(cudaGraphConditionalHandle h, unsigned v, cudaStream_t st) {
  k_set_cond<<<1, 32, 0, st>>>(h, v);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_select_sweep(long long n, const double* src, double* dst, const float* src32,
                                float* dst32, const DevScalars* ds, cudaStream_t st) {
  k_select_sweep<<<copy_blocks(n), 256, 0, st>>>(n, src, dst, src32, dst32, ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_select_iter(long long n, const double* src, double* dst,
                               const DevScalars* ds, cudaStream_t st) {
  k_select_iter<<<copy_blocks(n), 256, 0, st>>>(n, src, dst, ds);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg
