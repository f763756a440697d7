// heat.cu -- sm_103a kernels of the temperature equation (HeatSolver,
// heat.hpp:18-94): one ConvectionDiffusionScalarImplicit iteration per time
// step (conv_diff.hpp:130-251) with unit scaling, the mixture conductivity
// as diffusion rate, the fluid's iter_curr volume fluxes, no source, and a
// Jacobi solve of the delta-form system.  Same tiling as fluid.cu: a
// thread owns an (i, j) column of a 32x8 tile and marches the block's k
// range; geometry is implicit (uniform h).
#include "kernels.h"
#include "loop.cuh"

namespace hg {

namespace {

// Does the boundary face on side (d, side) of the cell with indices i carry
// the box temperature?  A face of the block's own boundary by the side
// table, a face beside an excluded cell by its centre.
template <int DIM>
__device__ __forceinline__ bool heat_value_face(const Mesh& m, const HeatBc& b, int d, int side,
                                                const int* i) {
  const bool domain = !m.per[d] && (side ? i[d] == m.n[d] - 1 : i[d] == 0);
  if (!domain) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      double x = k == d ? m.lo[k] + (i[k] + side) * m.h[k] : m.lo[k] + (i[k] + 0.5) * m.h[k];
      if (x < b.lo[k] || b.hi[k] < x) return false;
    }
    return true;
  }
  if (!b.side_in[2 * d + side]) return false;
#pragma unroll
  for (int k = 0; k < DIM; ++k)
    if (k != d && (i[k] < b.a[k] || i[k] >= b.b[k])) return false;
  return true;
}

template <int DIM>
__global__ void k_heat_conductivity(Mesh m, int nph, HeatCoef hc, CP<HYDRO_MAXPH> alpha,
                                    double* kc, int kch) {
  CELL_LOOP_BEGIN(m, kch)
  double s = 0.;
#pragma unroll
  for (int i = 0; i < HYDRO_MAXPH; ++i)
    if (i < nph) s += hc.cond[i] * alpha.a[i][X.c];
  kc[X.c] = s;
  CELL_LOOP_END
}

// G[d] = dT/dx_d: Green-Gauss over the two faces along d, inner faces the
// mean of their cells, boundary faces the box temperature or (zero
// derivative) the cell's own value (Gradient(Interpolate(T, cond)),
// solver.hpp:246-341, 392-470).
template <int DIM, bool PER>
__global__ void k_heat_grad(Mesh m, Geo g, HeatBc bc, const double* T, W3 G, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  const double tc = T[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    double flo = HAS_LO(d) ? avg(T[NB_LO(d, s)], tc)
                           : (heat_value_face<DIM>(m, bc, d, 0, X.i) ? bc.value : tc);
    double fhi = HAS_HI(d) ? avg(tc, T[NB_HI(d, s)])
                           : (heat_value_face<DIM>(m, bc, d, 1, X.i) ? bc.value : tc);
    G.a[d][X.c] = (fhi - flo) * g.inv_h[d];
  }
  CELL_LOOP_END
}

// Rows of the temperature equation in delta form around Tp (the
// iteration's start, equal to T_curr for the single iteration of a step):
// implicit first-order upwind convection with the deferred second-order
// correction from the upwind cell's gradient, central diffusion with face
// conductivity the mean of the cells' (zero-derivative interpolation), BDF
// time difference.  Boundary faces: the box temperature gives a convective
// constant and a half-cell diffusive coupling; a zero-derivative face
// convects the cell value and has no diffusive flux.
template <int DIM, bool PER>
__global__ void k_heat_assemble(Mesh m, Geo g, HeatBc bc, HeatCoef hc, const double* Tp,
                                const double* Ttc, const double* Ttp, const double* F,
                                const double* kc, C3 G, WP<7> coef, double* res, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  if (EXCLUDED()) {  // identity row, zero constant
    coef.a[0][X.c] = 1.;
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) coef.a[1 + q][X.c] = 0.;
    res[X.c] = 0.;
    continue;
  }
  const double kcc = kc[X.c];
  double aPc = 0.;  // convective and diffusive part of the diagonal
  double aq[2 * DIM];
  double cst = 0.;
  const double thr = 1e-10;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fs = face_stride(m, d);
    long long flo = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    const double hh = 0.5 * g.h[d];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      long long f = flo + side * fs;
      const double Ff = F[f];
      const double Fo = side ? Ff * g.invV : -(Ff * g.invV);  // outward flux / V
      bool inner = side ? HAS_HI(d) : HAS_LO(d);
      if (inner) {
        long long nb = side ? NB_HI(d, s) : NB_LO(d, s);
        double dif = avg(kcc, kc[nb]) * g.inv_h2[d];
        const bool up_m = Ff > thr, up_p = Ff < -thr;
        const bool own_up = side ? up_m : up_p;
        const bool nb_up = side ? up_p : up_m;
        const double half = 0.5 * Fo;
        double ao = own_up ? Fo : (nb_up ? 0. : half);
        double an = nb_up ? Fo : (own_up ? 0. : half);
        aPc += ao + dif;
        aq[2 * d + side] = an - dif;
        if (up_m || up_p) {
          long long cu = own_up ? X.c : nb;
          cst += G.a[d][cu] * ((up_m ? hh : -hh) * Fo);
        }
      } else if (heat_value_face<DIM>(m, bc, d, side, X.i)) {
        double dif = 2. * kcc * g.inv_h2[d];
        aPc += dif;
        aq[2 * d + side] = 0.;
        cst += bc.value * (Fo - dif);
      } else {
        aPc += Fo;
        aq[2 * d + side] = 0.;
      }
    }
  }
  const double tp = Tp[X.c];
  double r = hc.co[0] * Ttp[X.c] + hc.co[1] * Ttc[X.c] + hc.co[2] * tp + cst + aPc * tp;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    if (HAS_LO(d)) r += aq[2 * d] * Tp[NB_LO(d, s)];
    if (HAS_HI(d)) r += aq[2 * d + 1] * Tp[NB_HI(d, s)];
  }
  res[X.c] = r;
  coef.a[0][X.c] = 1. / ((hc.co[2] + aPc) / hc.relax);
#pragma unroll
  for (int q = 0; q < 2 * DIM; ++q) coef.a[1 + q][X.c] = aq[q];
  CELL_LOOP_END
}

// Jacobi::Solve (linear.hpp:750-782) with omega 1 on one component.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_heat_sweep(Mesh m, double tol, CP<7> coef,
                                                   const double* res, const double* din,
                                                   double* dout, int limit, double* partials,
                                                   DevScalars* ds, int kch) {
  constexpr bool kPerT = PER;
  if (ds->flag[FL_HEAT_DONE] || ds->flag[FL_HEAT_SWEEPS] >= limit) return;
  const bool first = ds->flag[FL_HEAT_SWEEPS] == 0;
  double dmax = 0.;
  CELL_LOOP_BEGIN(m, kch)
  double sum = 0., cur = 0.;
  if (!first) {
    cur = din[X.c];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      long long s = cell_stride(m, d);
      if (HAS_LO(d)) sum += coef.a[1 + 2 * d][X.c] * din[NB_LO(d, s)];
      if (HAS_HI(d)) sum += coef.a[2 + 2 * d][X.c] * din[NB_HI(d, s)];
    }
  }
  double value = -(res[X.c] + sum) * coef.a[0][X.c];
  dmax = fmax(dmax, fabs(value - cur));
  dout[X.c] = value;
  CELL_LOOP_END
  double v[1] = {dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[TK_HEAT], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_HEAT_DIFF] = out[0];
      ds->flag[FL_HEAT_SWEEPS] += 1;
      if (!(out[0] > tol)) ds->flag[FL_HEAT_DONE] = 1;
    }
  }
}

__global__ void k_heat_finish(long long n, double* tc, double* tp, const double* du0,
                              const double* du1, const DevScalars* ds) {
  const double* du = (ds->flag[FL_HEAT_SWEEPS] % 2 == 1) ? du0 : du1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double t = tc[i];
    tp[i] = t;
    tc[i] = t + du[i];
  }
}

}  // namespace

#define HEAT_DISPATCH(m, KERNEL, ...)                                \
  do {                                                               \
    Launch L = cell_launch(m);                                       \
    if ((m).dim == 3)                                                \
      KERNEL<3><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);     \
    else                                                             \
      KERNEL<2><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);     \
    count_launches(1);                                               \
    return cudaGetLastError();                                       \
  } while (0)
#define HEAT_DISPATCH_P(m, KERNEL, ...)                              \
  do {                                                               \
    Launch L = cell_launch(m);                                       \
    CELL_LAUNCH_P(m, L, st, KERNEL, __VA_ARGS__);                    \
    count_launches(1);                                               \
    return cudaGetLastError();                                       \
  } while (0)

cudaError_t launch_heat_conductivity(const Mesh& m, int nph, const HeatCoef& hc,
                                     CP<HYDRO_MAXPH> alpha, double* kc, cudaStream_t st) {
  HEAT_DISPATCH(m, k_heat_conductivity, m, nph, hc, alpha, kc);
}

cudaError_t launch_heat_grad(const Mesh& m, const HeatBc& bc, const double* T, W3 G,
                             cudaStream_t st) {
  HEAT_DISPATCH_P(m, k_heat_grad, m, make_geo(m), bc, T, G);
}

cudaError_t launch_heat_assemble(const Mesh& m, const HeatBc& bc, const HeatCoef& hc,
                                 const double* Tp, const double* Ttc, const double* Ttp,
                                 const double* F, const double* kc, C3 G, WP<7> coef,
                                 double* res, cudaStream_t st) {
  HEAT_DISPATCH_P(m, k_heat_assemble, m, make_geo(m), bc, hc, Tp, Ttc, Ttp, F, kc, G, coef, res);
}

cudaError_t launch_heat_sweep(const Mesh& m, double tol, CP<7> coef, const double* res,
                              const double* din, double* dout, int limit, double* partials,
                              DevScalars* ds, cudaStream_t st) {
  HEAT_DISPATCH_P(m, k_heat_sweep, m, tol, coef, res, din, dout, limit, partials, ds);
}

cudaError_t launch_heat_finish(long long n, double* tc, double* tp, const double* du0,
                               const double* du1, const DevScalars* ds, cudaStream_t st) {
  long long b = (n + NT - 1) / NT;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  k_heat_finish<<<(int)b, NT, 0, st>>>(n, tc, tp, du0, du1, ds);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg
