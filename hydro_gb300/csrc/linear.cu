// linear.cu -- pressure-correction solve on sm_103a: Jacobi-preconditioned
// conjugate gradients, matrix-free on the face couplings kf of the
// flux-correction expressions (fluid.hpp:946-1014: coupling -kf between the
// two cells of an inner face, diagonal sum kf).  The reference solves these
// rows with serial Gauss-Seidel (linear.hpp:685-715); CG replaces it.
//
// Templated on the element type T: T = double is the plain FP64 path;
// T = float is the inner solve of the mixed-precision path (FP32 vectors and
// couplings, FP64 dot products / norms, FP64 iterative refinement around it).
//
// One CG iteration = three launches, each returning at once after the
// device-side `done` flag is set (so the host queues iterations in chunks
// and reads the flag once per chunk):
//   k_cg_dir    p = z + beta p
//   k_cg_spmv   Ap = A p, <p,Ap> -> alpha = rz/<p,Ap>
//   k_cg_update x += alpha p, r -= alpha Ap, z = r/diag, <r,z>, <r,r> -> beta
#include <math.h>

#include "kernels.h"
#include "loop.cuh"

namespace hg {

enum {
  PG_CG_SPMV = HYDRO_PROF_CG_SPMV,
  PG_CG_UPDATE = HYDRO_PROF_CG_UPDATE,
  PG_CG_DIR = HYDRO_PROF_CG_DIR,
  PG_IR_RESIDUAL = HYDRO_PROF_IR_RESIDUAL
};

namespace {

// Matrix-free stencil product (A p)_c = diag_c p_c - sum_f kf_f p_nb with a
// pinned cell's row the identity and its value excluded from neighbours'.
template <int DIM, bool PER, class T>
__device__ __forceinline__ T stencil_row(const Mesh& m, const Cell& X, const T* kf,
                                         const T* dg, const T* p, long long pin) {
  constexpr bool kPerT = PER;
  if (X.c == pin) return p[X.c];
  T acc = dg[X.c] * p[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    if (HAS_LO(d) && NB_LO(d, s) != pin) acc -= kf[fl] * p[NB_LO(d, s)];
    if (HAS_HI(d) && NB_HI(d, s) != pin) acc -= kf[fl + face_stride(m, d)] * p[NB_HI(d, s)];
  }
  return acc;
}

// diag = sum of the inner-face couplings + shift (1 on the pinned row and
// on excluded cells); idg = 1/diag in FP64, and with dg32 set the same in
// FP32 plus the FP32 couplings (the mixed path's copy), from one read of kf.
template <int DIM, bool PER>
__global__ void k_diag(Mesh m, const double* kf, double shift, long long pin, double* dg,
                       double* idg, float* dg32, float* idg32, float* kf32, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  double s = shift;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    const double klo = kf[fl];
    if (HAS_LO(d)) s += klo;
    if (HAS_HI(d)) s += kf[fl + face_stride(m, d)];
    if (kf32) {
      kf32[fl] = d2f(klo);
      if (X.i[d] == m.n[d] - 1) kf32[fl + face_stride(m, d)] = d2f(kf[fl + face_stride(m, d)]);
    }
  }
  if (X.c == pin || EXCLUDED()) s = 1.;  // identity rows
  dg[X.c] = s;
  if (idg) idg[X.c] = 1. / s;  // FP64 Jacobi-PCG only
  if (dg32) {
    const float s32 = d2f(s);
    dg32[X.c] = s32;
    idg32[X.c] = 1.f / s32;
  }
  CELL_LOOP_END
}

// mean of a vector over the cells that are not excluded (nfluid of them),
// for the mean projection of singular systems: the sum, divided once.
template <class T>
__global__ void __launch_bounds__(NT) k_mean(long long n, long long nfluid, const T* a,
                                             const unsigned char* ex, double* partials,
                                             double* out, unsigned* ticket) {
  double s = 0.;
  long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  for (long long i = blockIdx.x * (long long)NT + tid; i < n; i += (long long)gridDim.x * NT)
    if (!ex || !ex[i]) s += (double)a[i];
  double v[1] = {s};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, ticket, o))
    if (tid == 0) *out = o[0] / (double)nfluid;
}

// x -= mean over the cells that are not excluded
__global__ void k_sub_mean(long long n, const unsigned char* ex, double* x, const double* xmean) {
  const double mean = *xmean;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if (!ex || !ex[i]) x[i] -= mean;
}

// r = f - mean(f) - A x (x == 0 unless use_guess), z = r/diag, p = z;
// reduces <r,z>, <r,r>, <f',f'> and sets the tolerance and done flag.
template <int DIM, class T, bool PER>
__global__ void __launch_bounds__(NT) k_cg_init(Mesh m, const T* kf, const T* dg, const T* idg,
                                                const double* f, const double* fmean,
                                                const T* x, int use_guess, long long pin,
                                                T* r, T* z, T* p, double tol, int limit,
                                                int dev_params, double* partials,
                                                DevScalars* ds, int kch) {
  double s[3] = {0., 0., 0.};
  const double mean = fmean ? *fmean : 0.;
  CELL_LOOP_BEGIN(m, kch)
  double fc = EXCLUDED() ? f[X.c] : f[X.c] - mean;
  double rc = fc;
  if (use_guess) rc -= (double)stencil_row<DIM, PER>(m, X, kf, dg, x, pin);
  T rt = (T)rc;
  T zt = rt * idg[X.c];
  r[X.c] = rt;
  z[X.c] = zt;
  p[X.c] = zt;
  s[0] += (double)rt * (double)zt;
  s[1] += (double)rt * (double)rt;
  s[2] += fc * fc;
  CELL_LOOP_END
  __shared__ double o[3];
  if (grid_reduce<RED_SUM, 3>(s, partials, &ds->ticket[TK_PCG_INIT], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      if (dev_params) tol = ds->red[RS_INNER_TOL];
      else ds->flag[FL_PCG_LIMIT] = limit;
      ds->red[RS_PCG_RZ] = o[0];
      ds->red[RS_PCG_RR] = o[1];
      ds->red[RS_PCG_FF] = o[2];
      ds->red[RS_PCG_TOL2] = tol * tol * o[2];
      ds->flag[FL_PCG_ITERS] = 0;
      ds->flag[FL_PCG_DONE] =
          (o[2] == 0. || o[1] <= tol * tol * o[2] || ds->flag[FL_PCG_LIMIT] <= 0) ? 1 : 0;
    }
  }
}

template <class T>
__global__ void k_cg_dir(long long n, const T* z, T* p, const DevScalars* ds) {
  if (ds->flag[FL_PCG_DONE]) return;
  T beta = (T)ds->red[RS_PCG_BETA];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

template <int DIM, class T, bool PER>
__global__ void __launch_bounds__(NT) k_cg_spmv(Mesh m, const T* kf, const T* dg, const T* p,
                                                T* Ap, long long pin, double* partials,
                                                DevScalars* ds, int kch) {
  if (ds->flag[FL_PCG_DONE]) return;
  double s = 0.;
  CELL_LOOP_BEGIN(m, kch)
  T a = stencil_row<DIM, PER>(m, X, kf, dg, p, pin);
  Ap[X.c] = a;
  s += (double)p[X.c] * (double)a;
  CELL_LOOP_END
  double v[1] = {s};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_PCG_A], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_PCG_PAP] = o[0];
      ds->red[RS_PCG_ALPHA] = ds->red[RS_PCG_RZ] / o[0];
    }
  }
}

template <class TX, class T>
__global__ void __launch_bounds__(NT) k_cg_update(long long n, TX* x, T* r, T* z, const T* p,
                                                  const T* Ap, const T* idg, double* partials,
                                                  DevScalars* ds) {
  if (ds->flag[FL_PCG_DONE]) return;
  double alpha = ds->red[RS_PCG_ALPHA];
  T at = (T)alpha;
  double s[2] = {0., 0.};
  long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  for (long long i = blockIdx.x * (long long)NT + tid; i < n; i += (long long)gridDim.x * NT) {
    x[i] += (TX)(at * p[i]);
    T ri = r[i] - at * Ap[i];
    T zi = ri * idg[i];
    r[i] = ri;
    z[i] = zi;
    s[0] += (double)ri * (double)zi;
    s[1] += (double)ri * (double)ri;
  }
  __shared__ double o[2];
  if (grid_reduce<RED_SUM, 2>(s, partials, &ds->ticket[TK_PCG_B], o)) {
    if (tid == 0) {
      double rz_old = ds->red[RS_PCG_RZ];
      ds->red[RS_PCG_BETA] = o[0] / rz_old;
      ds->red[RS_PCG_RZ] = o[0];
      ds->red[RS_PCG_RR] = o[1];
      int it = ds->flag[FL_PCG_ITERS] + 1;
      ds->flag[FL_PCG_ITERS] = it;
      if (o[1] <= ds->red[RS_PCG_TOL2] || it >= ds->flag[FL_PCG_LIMIT] || isnan(o[1]))
        ds->flag[FL_PCG_DONE] = 1;
    }
  }
}

// FP64 residual of the refinement loop: r = f' - A x (f' = f - mean when
// singular; x null: the iterate is zero and r = f'), <r,r> reduced.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_ir_residual(Mesh m, const double* kf, const double* dg,
                                                    const double* f, const double* fmean,
                                                    const double* x, long long pin, double* r,
                                                    double* partials, DevScalars* ds, int kch) {
  double s = 0.;
  const double mean = fmean ? *fmean : 0.;
  CELL_LOOP_BEGIN(m, kch)
  double rc = EXCLUDED() ? f[X.c] : f[X.c] - mean;
  if (x) rc -= stencil_row<DIM, PER>(m, X, kf, dg, x, pin);
  r[X.c] = rc;
  s += rc * rc;
  CELL_LOOP_END
  double v[1] = {s};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_IR], o))
    if (threadIdx.x == 0 && threadIdx.y == 0) ds->red[RS_IR_RR] = o[0];
}

// <x, f'> and <x, A x> of a guess x (f' = f - mean on a singular system).
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_guess_dots(Mesh m, const double* kf, const double* dg,
                                                   const double* f, const double* fmean,
                                                   const double* x, long long pin,
                                                   double* partials, DevScalars* ds, int kch) {
  double s[2] = {0., 0.};
  const double mean = fmean ? *fmean : 0.;
  CELL_LOOP_BEGIN(m, kch)
  const double fc = EXCLUDED() ? f[X.c] : f[X.c] - mean;
  const double xc = x[X.c];
  s[0] += xc * fc;
  s[1] += xc * stencil_row<DIM, PER>(m, X, kf, dg, x, pin);
  CELL_LOOP_END
  __shared__ double o[2];
  if (grid_reduce<RED_SUM, 2>(s, partials, &ds->ticket[TK_GUESS], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_GUESS_S0] = o[0];
      ds->red[RS_GUESS_S1] = o[1];
    }
  }
}

__global__ void k_guess_scale(long long n, double* x, const DevScalars* ds) {
  double a = ds->red[RS_GUESS_S0] / ds->red[RS_GUESS_S1];
  if (!(a > 0. && a < 1e300)) a = 0.;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] *= a;
}

// After the residual of the scaled guess: keep it when its residual is
// below that of the zero guess, else restore x = 0, r = f' and RS_IR_RR.
__global__ void k_guess_accept(long long n, const unsigned char* ex, const double* f,
                               const double* fmean, double* x, double* r, DevScalars* ds) {
  const double a = ds->red[RS_GUESS_S0] / ds->red[RS_GUESS_S1];
  const bool keep = (a > 0. && a < 1e300) && ds->red[RS_IR_RR] < ds->red[RS_IR_FF];
  if (!keep) {
    const double mean = fmean ? *fmean : 0.;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
      x[i] = 0.;
      r[i] = (ex && ex[i]) ? f[i] : f[i] - mean;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (keep) {
      ds->flag[FL_GUESS_USED] += 1;
      ds->flag[FL_GUESS_BACKOFF] = 0;
    } else {
      // back off: skip the guess in the next 1, 2, 4, ... 16 steps
      ds->flag[FL_GUESS_DROPPED] += 1;
      const int b = ds->flag[FL_GUESS_BACKOFF];
      ds->flag[FL_GUESS_BACKOFF] = b ? (2 * b < 16 ? 2 * b : 16) : 1;
      ds->flag[FL_GUESS_SKIP] = ds->flag[FL_GUESS_BACKOFF];
    }
  }
}

__global__ void k_guess_rr(DevScalars* ds) {
  const double a = ds->red[RS_GUESS_S0] / ds->red[RS_GUESS_S1];
  const bool keep = (a > 0. && a < 1e300) && ds->red[RS_IR_RR] < ds->red[RS_IR_FF];
  if (threadIdx.x == 0 && !keep) ds->red[RS_IR_RR] = ds->red[RS_IR_FF];
}

int flat_blocks_l(long long n) {
  long long b = (n + NT - 1) / NT;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

}  // namespace

// ---------------------------------------------------------- drivers ------
#define LAUNCH_DIM(KERNEL, ...) CELL_LAUNCH_P(m, L, st, KERNEL, __VA_ARGS__)
#define LAUNCH_DIM_T(KERNEL, T, ...) CELL_LAUNCH_TP(m, L, st, KERNEL, T, __VA_ARGS__)

cudaError_t pcg_prepare(const Mesh& m, const double* kf, double shift, PcgWork& w, int fp32,
                        cudaStream_t st) {
  Launch L = cell_launch(m);
  CELL_LAUNCH_P(m, L, st, k_diag, m, kf, shift, w.pin, w.dg, fp32 ? nullptr : w.idg,
                fp32 ? w.dg32 : nullptr,
                fp32 ? w.idg32 : nullptr, fp32 ? w.kf32 : nullptr);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t mean_sum(const Mesh& m, const double* f, PcgWork& w, cudaStream_t st) {
  k_mean<double><<<flat_blocks_l(m.nc), dim3(BX, BY), 0, st>>>(m.nc, m.nfluid, f, m.ex,
                                                              w.partials, &w.ds->red[RS_MEAN],
                                                              &w.ds->ticket[TK_MEAN]);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t sub_mean(const Mesh& m, double* x, PcgWork& w, cudaStream_t st) {
  k_mean<double><<<flat_blocks_l(m.nc), dim3(BX, BY), 0, st>>>(m.nc, m.nfluid, x, m.ex,
                                                              w.partials, &w.ds->red[RS_XMEAN],
                                                              &w.ds->ticket[TK_MEAN2]);
  k_sub_mean<<<flat_blocks_l(m.nc), NT, 0, st>>>(m.nc, m.ex, x, &w.ds->red[RS_XMEAN]);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t pcg_init(const Mesh& m, const double* kf, const double* f, double* x, int use_guess,
                     double tol, int singular, PcgWork& w, cudaStream_t st) {
  Launch L = cell_launch(m);
  const double* msum = nullptr;
  if (singular) {
    mean_sum(m, f, w, st);
    msum = &w.ds->red[RS_MEAN];
  }
  LAUNCH_DIM_T(k_cg_init, double, m, kf, w.dg, w.idg, f, msum, x, use_guess, w.pin, w.r, w.z,
             w.p, tol, w.limit, 0, w.partials, w.ds);
  if (!use_guess) cudaMemsetAsync(x, 0, sizeof(double) * m.nc, st);
  count_launches(singular ? 2 : 1);
  return cudaGetLastError();
}

cudaError_t pcg_iterate(const Mesh& m, const double* kf, double* x, int chunk, PcgWork& w,
                        cudaStream_t st) {
  Launch L = cell_launch(m);
  int fb = flat_blocks_l(m.nc);
  for (int it = 0; it < chunk; ++it) {
    if (w.prof) w.prof->begin(PG_CG_SPMV, st);
    LAUNCH_DIM_T(k_cg_spmv, double, m, kf, w.dg, w.p, w.Ap, w.pin, w.partials, w.ds);
    if (w.prof) w.prof->end(PG_CG_SPMV, st);
    if (w.prof) w.prof->begin(PG_CG_UPDATE, st);
    k_cg_update<double, double><<<fb, dim3(BX, BY), 0, st>>>(m.nc, x, w.r, w.z, w.p, w.Ap, w.idg,
                                                             w.partials, w.ds);
    if (w.prof) w.prof->end(PG_CG_UPDATE, st);
    if (w.prof) w.prof->begin(PG_CG_DIR, st);
    k_cg_dir<double><<<fb, NT, 0, st>>>(m.nc, w.z, w.p, w.ds);
    if (w.prof) w.prof->end(PG_CG_DIR, st);
  }
  count_launches(3 * chunk);
  return cudaGetLastError();
}

// ------------------------------------------- mixed-precision (FP32) ------
cudaError_t ir_residual(const Mesh& m, const double* kf, const double* f, const double* x,
                        int singular, PcgWork& w, cudaStream_t st) {
  Launch L = cell_launch(m);
  const double* msum = singular ? &w.ds->red[RS_MEAN] : nullptr;
  if (w.prof) w.prof->begin(PG_IR_RESIDUAL, st);
  LAUNCH_DIM(k_ir_residual, m, kf, w.dg, f, msum, x, w.pin, w.r, w.partials, w.ds);
  if (w.prof) w.prof->end(PG_IR_RESIDUAL, st);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t guess_scale(const Mesh& m, const double* kf, const double* f, double* x, int singular,
                        PcgWork& w, cudaStream_t st) {
  Launch L = cell_launch(m);
  const double* msum = singular ? &w.ds->red[RS_MEAN] : nullptr;
  LAUNCH_DIM(k_guess_dots, m, kf, w.dg, f, msum, x, w.pin, w.partials, w.ds);
  k_guess_scale<<<flat_blocks_l(m.nc), NT, 0, st>>>(m.nc, x, w.ds);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t guess_accept(const Mesh& m, const double* f, double* x, int singular, PcgWork& w,
                         cudaStream_t st) {
  const double* msum = singular ? &w.ds->red[RS_MEAN] : nullptr;
  // RS_IR_RR is rewritten only by the next kernel, after every block of
  // k_guess_accept has read it
  k_guess_accept<<<flat_blocks_l(m.nc), NT, 0, st>>>(m.nc, m.ex, f, msum, x, w.r, w.ds);
  k_guess_rr<<<1, 32, 0, st>>>(w.ds);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t f32_pcg_init(const Mesh& m, double tol, int dev_params, PcgWork& w, cudaStream_t st) {
  Launch L = cell_launch(m);
  w.p32_parity = 0;
  cudaMemsetAsync(w.x32, 0, sizeof(float) * m.nc, st);
  LAUNCH_DIM_T(k_cg_init, float, m, w.kf32, w.dg32, w.idg32, w.r, (const double*)nullptr,
             w.x32, 0, w.pin, w.r32, w.z32, w.p32, tol, w.limit, dev_params, w.partials, w.ds);
  count_launches(1);
  return cudaGetLastError();
}

namespace {

// Double-float accumulation of dot products on the FP32 pipe: products are
// split exactly (p + e == a*b via fmaf), partial sums carried as an
// unevaluated pair (TwoSum), so a thread's share of a dot product is
// accurate to about 2^-44 relative before it is combined across threads in
// FP64.  GB300 runs FP64 at 1/57 of the FP32 rate, which makes per-cell
// FP64 accumulation the bottleneck of the FP32 kernels.
struct DFAcc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    float t = hi + p;
    float bp = t - hi;
    float err = (hi - (t - bp)) + (p - bp);
    hi = t;
    lo += err + e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// p_new = z + beta p_old (p_new = z on the first iteration) evaluated at the
// cell and its neighbours, A p_new, <p_new, A p_new> -> alpha.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_cg32_dir_spmv(Mesh m, const float* __restrict__ kf,
                                                      const float* __restrict__ dg,
                                                      const float* __restrict__ z,
                                                      const float* __restrict__ pold,
                                                      float* __restrict__ pnew,
                                                      float* __restrict__ Ap, long long pin,
                                                      double* partials, DevScalars* ds,
                                                      int kch) {
  pdl_wait();
  pdl_trigger();
  constexpr bool kPerT = PER;
  if (ds->flag[FL_PCG_DONE]) return;
  const bool first = ds->flag[FL_PCG_ITERS] == 0;
  const float beta = first ? 0.f : (float)ds->red[RS_PCG_BETA];
  DFAcc acc;
  CELL_LOOP_BEGIN(m, kch)
  auto P = [&](long long c) { return first ? z[c] : fmaf(beta, pold[c], z[c]); };
  float pc = P(X.c);
  pnew[X.c] = pc;
  float a;
  if (X.c == pin) {
    a = pc;
  } else {
    a = dg[X.c] * pc;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      long long s = cell_stride(m, d);
      long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
      if (HAS_LO(d) && NB_LO(d, s) != pin) a = fmaf(-kf[fl], P(NB_LO(d, s)), a);
      if (HAS_HI(d) && NB_HI(d, s) != pin)
        a = fmaf(-kf[fl + face_stride(m, d)], P(NB_HI(d, s)), a);
    }
  }
  Ap[X.c] = a;
  acc.add_prod(pc, a);
  CELL_LOOP_END
  double v[1] = {acc.value()};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_F32_A], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_PCG_PAP] = o[0];
      ds->red[RS_PCG_ALPHA] = ds->red[RS_PCG_RZ] / o[0];
    }
  }
}

// k_cg32_dir_spmv for a block without periodic directions or excluded cells
// in 32-bit index arithmetic (faces < 2^31): same loads, order of the sums
// and results.
template <int DIM>
__global__ void __launch_bounds__(NT) k_cg32_dir_spmv_i32(Mesh m, const float* __restrict__ kf,
                                                          const float* __restrict__ dg,
                                                          const float* __restrict__ z,
                                                          const float* __restrict__ pold,
                                                          float* __restrict__ pnew,
                                                          float* __restrict__ Ap, int pin,
                                                          double* partials, DevScalars* ds,
                                                          int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const bool first = ds->flag[FL_PCG_ITERS] == 0;
  const float beta = first ? 0.f : (float)ds->red[RS_PCG_BETA];
  DFAcc acc;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int n0 = m.n[0], n1 = m.n[1];
  const int nz = DIM == 3 ? m.n[2] : 1;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, nz);
  const int cs[3] = {1, n0, n0 * n1};
  const int fs[3] = {1, (int)m.fnx[1], (int)(m.fnx[2] * m.fny[2])};
  auto P = [&](int c) { return first ? z[c] : fmaf(beta, pold[c], z[c]); };
  if (i < n0 && j < n1) {
    for (int k = k0; k < k1; ++k) {
      const int id[3] = {i, j, k};
      const int c = i + n0 * (j + n1 * k);
      const float pc = P(c);
      pnew[c] = pc;
      float a;
      if (c == pin) {
        a = pc;
      } else {
        a = dg[c] * pc;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const int fl = (int)m.fofs[d] + i + (int)m.fnx[d] * (j + (int)m.fny[d] * k);
          if (id[d] > 0 && c - cs[d] != pin) a = fmaf(-kf[fl], P(c - cs[d]), a);
          if (id[d] < m.n[d] - 1 && c + cs[d] != pin) a = fmaf(-kf[fl + fs[d]], P(c + cs[d]), a);
        }
      }
      Ap[c] = a;
      acc.add_prod(pc, a);
    }
  }
  double v[1] = {acc.value()};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_F32_A], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_PCG_PAP] = o[0];
      ds->red[RS_PCG_ALPHA] = ds->red[RS_PCG_RZ] / o[0];
    }
  }
}

// x += alpha p, r -= alpha Ap, z = r/diag; <r,z>, <r,r> -> beta, stop test.
__global__ void __launch_bounds__(NT) k_cg32_update(long long n, float* x, float* r, float* z,
                                                    const float* p, const float* Ap,
                                                    const float* idg, double* partials,
                                                    DevScalars* ds) {
  if (ds->flag[FL_PCG_DONE]) return;
  const float at = (float)ds->red[RS_PCG_ALPHA];
  DFAcc rz, rr;
  long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  for (long long i = blockIdx.x * (long long)NT + tid; i < n; i += (long long)gridDim.x * NT) {
    x[i] = fmaf(at, p[i], x[i]);
    float ri = fmaf(-at, Ap[i], r[i]);
    float zi = ri * idg[i];
    r[i] = ri;
    z[i] = zi;
    rz.add_prod(ri, zi);
    rr.add_prod(ri, ri);
  }
  double s[2] = {rz.value(), rr.value()};
  __shared__ double o[2];
  if (grid_reduce<RED_SUM, 2>(s, partials, &ds->ticket[TK_F32_B], o)) {
    if (tid == 0) {
      double rz_old = ds->red[RS_PCG_RZ];
      ds->red[RS_PCG_BETA] = o[0] / rz_old;
      ds->red[RS_PCG_RZ] = o[0];
      ds->red[RS_PCG_RR] = o[1];
      int it = ds->flag[FL_PCG_ITERS] + 1;
      ds->flag[FL_PCG_ITERS] = it;
      if (o[1] <= ds->red[RS_PCG_TOL2] || it >= ds->flag[FL_PCG_LIMIT] || isnan(o[1]))
        ds->flag[FL_PCG_DONE] = 1;
    }
  }
}

}  // namespace

cudaError_t cg32_dir_spmv(const Mesh& m, const float* kf, const float* dg, const float* z,
                          const float* pold, float* pnew, float* Ap, long long pin,
                          double* partials, DevScalars* ds, cudaStream_t st) {
  if (!any_periodic(m) && m.nf < (1LL << 31)) {
    const void* k = m.dim == 3 ? (const void*)k_cg32_dir_spmv_i32<3>
                               : (const void*)k_cg32_dir_spmv_i32<2>;
    Launch L = cell_launch_waves(m, resident_ctas(k));
    if (m.dim == 3)
      PDL(k_cg32_dir_spmv_i32<3>, L.grid, L.block, 0, st, m, kf, dg, z, pold, pnew, Ap, (int)pin,
          partials, ds, L.kch);
    else
      PDL(k_cg32_dir_spmv_i32<2>, L.grid, L.block, 0, st, m, kf, dg, z, pold, pnew, Ap, (int)pin,
          partials, ds, L.kch);
    count_launches(1);
    return cudaGetLastError();
  }
  Launch L = cell_launch_waves(m, resident_ctas(CELL_KERNEL_P(m, k_cg32_dir_spmv)));
  CELL_LAUNCH_P(m, L, st, k_cg32_dir_spmv, m, kf, dg, z, pold, pnew, Ap, pin, partials, ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t f32_pcg_iterate(const Mesh& m, int chunk, PcgWork& w, cudaStream_t st) {
  Launch L = cell_launch_waves(m, resident_ctas(CELL_KERNEL_P(m, k_cg32_dir_spmv)));
  int fb = flat_blocks_l(m.nc);
  for (int it = 0; it < chunk; ++it) {
    // p lives in w.p32 / w.p32b alternately; its parity only matters while
    // iterating, and a launch after convergence returns at once
    float* pold = (w.p32_parity & 1) ? w.p32b : w.p32;
    float* pnew = (w.p32_parity & 1) ? w.p32 : w.p32b;
    if (w.prof) w.prof->begin(PG_CG_SPMV, st);
    CELL_LAUNCH_P(m, L, st, k_cg32_dir_spmv, m, w.kf32, w.dg32, w.z32, pold, pnew, w.Ap32, w.pin,
                  w.partials, w.ds);
    if (w.prof) w.prof->end(PG_CG_SPMV, st);
    if (w.prof) w.prof->begin(PG_CG_UPDATE, st);
    k_cg32_update<<<fb, dim3(BX, BY), 0, st>>>(m.nc, w.x32, w.r32, w.z32, pnew, w.Ap32, w.idg32,
                                               w.partials, w.ds);
    if (w.prof) w.prof->end(PG_CG_UPDATE, st);
    w.p32_parity ^= 1;
  }
  count_launches(2 * chunk);
  return cudaGetLastError();
}

namespace {
__global__ void k_accumulate(long long n, double* x, const float* e) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] += f2d(e[i]);
}
}  // namespace

namespace {
__global__ void k_scale(long long n, double* a, double s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] *= s;
}
}  // namespace

cudaError_t scale_vector(long long n, double* a, double s, cudaStream_t st) {
  k_scale<<<flat_blocks_l(n), NT, 0, st>>>(n, a, s);
  count_launches(1);
  return cudaGetLastError();
}

namespace {
__global__ void k_pin_rhs(Mesh m, const double* kf, double* f, long long pin, double value) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int i[3];
  i[0] = (int)(pin % m.n[0]);
  i[1] = (int)((pin / m.n[0]) % m.n[1]);
  i[2] = (int)(pin / ((long long)m.n[0] * m.n[1]));
  for (int d = 0; d < m.dim; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, i[0], i[1], i[2]);
    if (has_lo(m, d, i[d], pin, s)) f[nb_lo(m, d, i[d], pin, s)] += kf[fl] * value;
    if (has_hi(m, d, i[d], pin, s))
      f[nb_hi(m, d, i[d], pin, s)] += kf[fl + face_stride(m, d)] * value;
  }
  f[pin] = value;
}
}  // namespace

cudaError_t pin_rhs(const Mesh& m, const double* kf, double* f, long long pin, double value,
                    cudaStream_t st) {
  k_pin_rhs<<<1, 32, 0, st>>>(m, kf, f, pin, value);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t f32_accumulate(const Mesh& m, double* x, PcgWork& w, cudaStream_t st) {
  k_accumulate<<<flat_blocks_l(m.nc), NT, 0, st>>>(m.nc, x, w.x32);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg
