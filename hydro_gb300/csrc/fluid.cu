// fluid.cu -- sm_103a kernels of one SIMPLE iteration (FluidSimple::
// MakeIteration, fluid.hpp:814-1158) and of the fluid-property update
// (hydro<Mesh>::UpdateFluidProperties, hydro2d.hpp:1404-1430).
//
// One thread owns one (i, j) column of a 32x8 tile and marches the block's
// k range, so x-neighbours come from the same warp, y-neighbours from the
// same block and z-neighbours from the previous/next plane (L1/L2 hits);
// every load is coalesced along x.  Geometry is implicit (uniform h).
// Face arrays are written once per face: each cell owns its low face in
// every direction and, on the high end of the block, its high face.
#include <math.h>

#include "kernels.h"
#include "loop.cuh"

namespace hg {

namespace {

// FP64 operands of the BDF time difference (the residual's cancelling part).
struct Unsteady64 {
  double co[3];
  const double* up[3];
  const double* utc[3];
  const double* utp[3];
};

__device__ __forceinline__ double tsqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float tsqrt(float v) { return sqrtf(v); }

// Geometric average of two vectors (solver.hpp:380-390), component d.
template <int DIM, class T>
__device__ T vgeo(const T* a, const T* b, int d) {
  T av[DIM], n2 = T(0), na = T(0), nb = T(0);
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    av[k] = (a[k] + b[k]) * T(0.5);
    n2 += av[k] * av[k];
    na += a[k] * a[k];
    nb += b[k] * b[k];
  }
  T an = tsqrt(n2);
  if (an < T(1e-8)) return av[d];
  return av[d] / an * tsqrt(tsqrt(na) * tsqrt(nb));
}

// Face value (component d) of a cell vector field between cells cm and cp.
template <int DIM, class T>
__device__ T face_vec(const RT<T, 3>& f, long long cm, long long cp, int d, int geometric) {
  if (!geometric) return avg(f.a[d][cm], f.a[d][cp]);
  T a[DIM], b[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    a[k] = f.a[k][cm];
    b[k] = f.a[k][cp];
  }
  return vgeo<DIM, T>(a, b, d);
}

template <class T>
__device__ __forceinline__ T face_scal(T a, T b, int geometric) {
  return geometric ? tsqrt(a * b) : avg(a, b);
}

// ------------------------------------------------------------ StartStep --
__global__ void k_axpy_extrap(long long n, double ge, double* out, const double* tc,
                              const double* tp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = tc[i] + (tc[i] - tp[i]) * ge;
}

// FP32 copies of FP64 arrays (the shadows read by the FP32 kernels).
__global__ void k_d2f(long long n, const double* in, float* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = d2f(in[i]);
}

// ------------------------------------------------------- velocity grads --
// G[n*DIM+m] = d u_n / d x_m at cells, faces carrying the velocity value
// condition (Gradient(Interpolate(u_n, cond_n)), solver.hpp:392-470,658-677).
template <int DIM, class T, bool PER>
__global__ void k_vel_grad(Mesh m, GeoT<T> g, FluidCoefT<T> fc, RT<T, 3> u, RT<T, 3> bv,
                           WT<T, 9> G, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int n = 0; n < DIM; ++n) {
      T uc = u.a[n][X.c];
      T flo = HAS_LO(d) ? avg(u.a[n][NB_LO(d, s)], uc) : bv.a[n][fl];
      T fhi = HAS_HI(d) ? avg(uc, u.a[n][NB_HI(d, s)]) : bv.a[n][fl + face_stride(m, d)];
      G.a[n * DIM + d][X.c] = (fhi - flo) * g.inv_h[d];
    }
  }
  CELL_LOOP_END
}

// ---------------------------------------------------------------- force --
// Explicit momentum source (fluid.hpp:834-870): transposed viscous term
// sum_n d/dx_n (mu du_n/dx_m) with face gradients averaged from cells
// (zero-derivative boundaries), minus grad p (extrapolated boundary faces),
// plus the "restored" external force (fluid.hpp:612-625), surface-tension
// force and the volume-source momentum term.  Also stores the restored
// force and the FP64 cell pressure gradient for the Rhie-Chow kernel.
template <int DIM, class T, bool PER>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 6 : 1) k_force(Mesh m, GeoT<T> g, FluidCoefT<T> fc, RT<T, 3> u, RT<T, 9> G,
                        const double* p, Geo g64, const T* mu, const T* rho,
                        RT<T, 3> force, RT<T, 3> stforce, const T* Sv, const T* Sm,
                        WT<T, 3> fo, WT<T, 3> fres, W3 gp64, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  T acc[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) acc[k] = T(0);
  const T muc = mu[X.c];
#pragma unroll
  for (int n = 0; n < DIM; ++n) {
    long long s = cell_stride(m, n);
    T mlo, mhi;
    T glo[DIM], ghi[DIM];
    if (HAS_LO(n)) {
      const long long cl = NB_LO(n, s);
      mlo = face_scal(mu[cl], muc, fc.geometric);
#pragma unroll
      for (int k = 0; k < DIM; ++k)
        glo[k] = avg(G.a[n * DIM + k][cl], G.a[n * DIM + k][X.c]);
    } else {
      mlo = muc;
#pragma unroll
      for (int k = 0; k < DIM; ++k) glo[k] = G.a[n * DIM + k][X.c];
    }
    if (HAS_HI(n)) {
      const long long ch = NB_HI(n, s);
      mhi = face_scal(muc, mu[ch], fc.geometric);
#pragma unroll
      for (int k = 0; k < DIM; ++k)
        ghi[k] = avg(G.a[n * DIM + k][X.c], G.a[n * DIM + k][ch]);
    } else {
      mhi = muc;
#pragma unroll
      for (int k = 0; k < DIM; ++k) ghi[k] = G.a[n * DIM + k][X.c];
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) acc[k] += (ghi[k] * mhi - glo[k] * mlo) * g.inv_h[n];
  }
  T src = fc.sources ? rho[X.c] * Sv[X.c] - Sm[X.c] : T(0);
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    long long s = cell_stride(m, k);
    int id = X.i[k];
    // the pressure gradient stays FP64: p carries the hydrostatic level,
    // whose FP32 rounding would swamp differences across a cell
    double gpd = grad_extrap_m<PER>(m, p, X.c, k, id, s, g64.inv_h[k]);
    gp64.a[k][X.c] = gpd;
    T gp = (T)gpd;
    T fcv = force.a[k][X.c];
    T flo = HAS_LO(k) ? face_vec<DIM, T>(force, NB_LO(k, s), X.c, k, fc.geometric) : fcv;
    T fhi = HAS_HI(k) ? face_vec<DIM, T>(force, X.c, NB_HI(k, s), k, fc.geometric) : fcv;
    T fr = T(0.5) * (flo + fhi);
    fres.a[k][X.c] = fr;
    T v = -gp + fr + stforce.a[k][X.c];
    if (fc.sources) v += u.a[k][X.c] * src;
    fo.a[k][X.c] = acc[k] + v;
  }
  CELL_LOOP_END
}

// ------------------------------------------------------ momentum system --
// ConvectionDiffusionScalarImplicit::MakeIteration assembly
// (conv_diff.hpp:130-227) for all components at once: the coefficients
// depend only on F, rho, mu and are shared; the constants differ.
// Convective face value: deferred second-order upwind (solver.hpp:201-243,
// threshold 1e-10); diffusion: two-point (solver.hpp:283-341); BDF time
// term (solver.hpp:815-861).  Stores the inverse of the relaxed diagonal,
// the 2*DIM off-diagonals (face order xm,xp,ym,yp,zm,zp; 0 on boundary
// faces), the delta-form residuals r_n = row_n(u_prev) and D_c = sum of the
// relaxed row coefficients (fluid.hpp:876-883).  Per inner face the
// convective flux enters as s_f F rho/V with the upwind weights selected,
// not multiplied, and the deferred correction's factor is formed once for
// the DIM components.  The BDF time difference of the residual is formed
// in FP64 from the FP64 layers (us) whatever T is.
template <int DIM, class T, bool PER>
__global__ void k_mom_assemble(Mesh m, GeoT<T> g, FluidCoefT<T> fc, RT<T, 3> up, RT<T, 3> utc,
                               RT<T, 3> utp, RT<T, 9> G, const T* F, const T* rho, const T* mu,
                               RT<T, 3> fo, Unsteady64 us, RT<T, 3> bv, WT<T, 7> coef,
                               WT<T, 3> res, T* Dc, int split, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  // row index of the coefficients and residuals: natural, or color-blocked
  // for the red-black Gauss-Seidel sweeps
  const long long oi =
      split ? ((X.i[0] + X.i[1] + X.i[2]) & 1) * (m.nc / 2) + (X.c >> 1) : X.c;
  if (EXCLUDED()) {
    // identity row, zero constant (conv_diff.hpp:222-226); CoeffSum 1
    coef.a[0][oi] = T(1);
#pragma unroll
    for (int q = 0; q < 2 * DIM; ++q) coef.a[1 + q][oi] = T(0);
#pragma unroll
    for (int n = 0; n < DIM; ++n) res.a[n][oi] = T(0);
    Dc[X.c] = T(1);
    continue;
  }
  const T rhoc = rho[X.c], muc = mu[X.c];
  T aPc = T(0);  // convective and diffusive part of the diagonal
  T aq[2 * DIM];
  T cst[DIM];
#pragma unroll
  for (int n = 0; n < DIM; ++n) cst[n] = -fo.a[n][X.c];
  const T rv = rhoc * g.invV;
  const T thr = T(1e-10);
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fs = face_stride(m, d);
    long long flo = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    const T hh = T(0.5) * g.h[d];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      long long f = flo + side * fs;
      const T Ff = F[f];
      // outward convective flux times rho/V (s_f = -1 on the low face)
      const T Fo = side ? Ff * rv : -(Ff * rv);
      bool inner = side ? HAS_HI(d) : HAS_LO(d);
      if (inner) {
        long long nb = side ? NB_HI(d, s) : NB_LO(d, s);
        T dif = face_scal(muc, mu[nb], fc.geometric) * g.inv_h2[d];
        // the cell is the low-side cell (cm) of its high face and the
        // high-side cell (cp) of its low face
        const bool up_m = Ff > thr, up_p = Ff < -thr;
        const bool own_up = side ? up_m : up_p;
        const bool nb_up = side ? up_p : up_m;
        const T half = T(0.5) * Fo;
        T ao = own_up ? Fo : (nb_up ? T(0) : half);
        T an = nb_up ? Fo : (own_up ? T(0) : half);
        aPc += ao + dif;
        aq[2 * d + side] = an - dif;
        if (up_m || up_p) {
          long long cu = own_up ? X.c : nb;
          // -(x_up - x_f) along d times the outward flux
          T t = (up_m ? hh : -hh) * Fo;
#pragma unroll
          for (int n = 0; n < DIM; ++n) cst[n] += G.a[n * DIM + d][cu] * t;
        }
      } else {
        T dif = T(2) * muc * g.inv_h2[d];
        aPc += dif;
        aq[2 * d + side] = T(0);
        const T w = Fo - dif;
#pragma unroll
        for (int n = 0; n < DIM; ++n) cst[n] += bv.a[n][f] * w;
      }
    }
  }
  const T aP = fc.co[2] * rhoc + aPc;
  T cs = aP;
#pragma unroll
  for (int q = 0; q < 2 * DIM; ++q) cs += aq[q];
#pragma unroll
  for (int n = 0; n < DIM; ++n) {
    // BDF time difference in FP64 (its terms cancel to the small change
    // of u over the step), then scaled by rho in T
    double ut = us.co[0] * us.utp[n][X.c] + us.co[1] * us.utc[n][X.c] +
                us.co[2] * us.up[n][X.c];
    T r = (T)ut * rhoc + cst[n] + aPc * up.a[n][X.c];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      long long s = cell_stride(m, d);
      if (HAS_LO(d)) r += aq[2 * d] * up.a[n][NB_LO(d, s)];
      if (HAS_HI(d)) r += aq[2 * d + 1] * up.a[n][NB_HI(d, s)];
    }
    res.a[n][oi] = r;
  }
  T aPr = aP / fc.relax_u;
  // the sweep multiplies by the inverse diagonal
  coef.a[0][oi] = T(1) / aPr;
#pragma unroll
  for (int q = 0; q < 2 * DIM; ++q) coef.a[1 + q][oi] = aq[q];
  Dc[X.c] = cs - aP + aPr;
  CELL_LOOP_END
}

// Jacobi sweep for all components (Jacobi::Solve, linear.hpp:750-782):
// value = -(r + sum_nb a du_nb)/aP, du' = du + omega*(value - du); the max
// |value - du| is reduced into ds->red[RS_MOM_DIFF].  A launch after
// convergence or after `limit` sweeps returns at once; the first sweep
// (count 0) starts from du = 0.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_mom_sweep(Mesh m, double omega, double tol,
                                                  CP<7> coef, C3 res, C3 din, W3 dout,
                                                  int limit, double* partials, DevScalars* ds,
                                                  int kch) {
  constexpr bool kPerT = PER;
  if (ds->flag[FL_MOM_DONE] || ds->flag[FL_MOM_SWEEPS] >= limit) return;
  const bool first = ds->flag[FL_MOM_SWEEPS] == 0;
  double dmax = 0.;
  CELL_LOOP_BEGIN(m, kch)
  double iaP = coef.a[0][X.c];
  double a[2 * DIM];
#pragma unroll
  for (int q = 0; q < 2 * DIM; ++q) a[q] = coef.a[1 + q][X.c];
#pragma unroll
  for (int n = 0; n < DIM; ++n) {
    double sum = 0., cur = 0.;
    if (!first) {
      cur = din.a[n][X.c];
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        long long s = cell_stride(m, d);
        if (HAS_LO(d)) sum += a[2 * d] * din.a[n][NB_LO(d, s)];
        if (HAS_HI(d)) sum += a[2 * d + 1] * din.a[n][NB_HI(d, s)];
      }
    }
    double value = -(res.a[n][X.c] + sum) * iaP;
    double corr = value - cur;
    dmax = fmax(dmax, fabs(corr));
    dout.a[n][X.c] = cur + corr * omega;
  }
  CELL_LOOP_END
  double v[1] = {dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[TK_MOM], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_MOM_DIFF] = out[0];
      ds->flag[FL_MOM_SWEEPS] += 1;
      if (!(out[0] > tol)) ds->flag[FL_MOM_DONE] = 1;
    }
  }
}

// Red-black Gauss-Seidel half-sweep (see launch_mom_rbgs).  Thread (x, y)
// owns the color cell of the pair (2x, 2x+1) in row (j, k).  The first sweep
// starts from du = 0: its red half reads no neighbours and the own old value
// of both halves is 0.  SDU: du itself is stored color-blocked like the rows
// (a neighbour nb of the other color at (1 - color) * nc/2 + nb/2), so that a
// warp's neighbour loads are unit-stride.
template <int DIM, bool PER, class T, bool SPLIT, bool SDU>
__global__ void __launch_bounds__(NT) k_mom_rbgs(Mesh m, T omega, double tol, RT<T, 7> cf,
                                                 RT<T, 3> rs, WT<T, 3> du, int color, int limit,
                                                 double* partials, DevScalars* ds, int kch) {
  if (ds->flag[FL_MOM_DONE] || ds->flag[FL_MOM_SWEEPS] >= limit) return;
  const bool first = ds->flag[FL_MOM_SWEEPS] == 0;
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int nz = DIM == 3 ? m.n[2] : 1;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, nz);
  const long long half = m.nc / 2;
  T dmax = T(0);
  if (j < m.n[1]) {
    for (int k = k0; k < k1; ++k) {
      Cell X;
      X.i[0] = 2 * ih + ((j + k + color) & 1);
      X.i[1] = j;
      X.i[2] = k;
      if (X.i[0] >= m.n[0]) continue;
      X.c = cell_id(m, X.i[0], X.i[1], X.i[2]);
      const long long ci = SPLIT ? color * half + (X.c >> 1) : X.c;
      // every load of the cell before its first store: the three components'
      // rows and neighbours are in flight together
      const T iaP = cf.a[0][ci];
      T a[2 * DIM], r[DIM], cur[DIM], nb[DIM][2 * DIM];
#pragma unroll
      for (int q = 0; q < 2 * DIM; ++q) a[q] = cf.a[1 + q][ci];
      constexpr bool kPerT = PER;
      const bool rd = !(first && color == 0);
      const long long own = SDU ? ci : X.c;
      const long long obase = SDU ? (1 - color) * half : 0;
      auto nbi = [&](long long nb) { return SDU ? obase + (nb >> 1) : nb; };
#pragma unroll
      for (int n = 0; n < DIM; ++n) {
        r[n] = rs.a[n][ci];
        cur[n] = first ? T(0) : du.a[n][own];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          long long s = cell_stride(m, d);
          nb[n][2 * d] = rd && HAS_LO(d) ? du.a[n][nbi(NB_LO(d, s))] : T(0);
          nb[n][2 * d + 1] = rd && HAS_HI(d) ? du.a[n][nbi(NB_HI(d, s))] : T(0);
        }
      }
#pragma unroll
      for (int n = 0; n < DIM; ++n) {
        T sum = T(0);
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) sum += a[q] * nb[n][q];
        const T value = -(r[n] + sum) * iaP;
        const T corr = value - cur[n];
        dmax = fmax(dmax, fabs(corr));
        du.a[n][own] = cur[n] + corr * omega;
      }
    }
  }
  double v[1] = {(double)dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[color == 0 ? TK_MOM_RED : TK_MOM], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      if (color == 0) {
        ds->red[RS_MOM_DIFF_RED] = out[0];
      } else {
        const double mx = fmax(out[0], ds->red[RS_MOM_DIFF_RED]);
        ds->red[RS_MOM_DIFF] = mx;
        ds->flag[FL_MOM_SWEEPS] += 1;
        if (!(mx > tol)) ds->flag[FL_MOM_DONE] = 1;
      }
    }
  }
}

// k_mom_rbgs for the FP32 color-blocked rows and corrections of a block
// without periodic directions or excluded cells, in 32-bit index arithmetic
// (nc < 2^31): with n0 even, the blocked index of cell c is c/2 within its
// color's half, and its neighbours across y and z sit n0/2 and n0 n1/2
// blocked entries away.  Same loads, order of the sum and results as the
// general form.
template <int DIM>
__global__ void __launch_bounds__(NT) k_mom_rbgs_f32(Mesh m, float omega, double tol,
                                                     RT<float, 7> cf, RT<float, 3> rs, FP<3> du,
                                                     int color, int limit, double* partials,
                                                     DevScalars* ds, int kch) {
  if (ds->flag[FL_MOM_DONE] || ds->flag[FL_MOM_SWEEPS] >= limit) return;
  const bool first = ds->flag[FL_MOM_SWEEPS] == 0;
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int n0 = m.n[0], n1 = m.n[1];
  const int nz = DIM == 3 ? m.n[2] : 1;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, nz);
  const int half = (int)(m.nc / 2);
  const int hy = n0 / 2, hz = n0 / 2 * n1;
  const int ob = (1 - color) * half;
  const bool rd = !(first && color == 0);
  float dmax = 0.f;
  if (j < n1) {
    for (int k = k0; k < k1; ++k) {
      const int i = 2 * ih + ((j + k + color) & 1);
      if (i >= n0) continue;
      const int c = i + n0 * (j + n1 * k);
      const int h = c >> 1;
      const int ci = color * half + h;
      const float iaP = cf.a[0][ci];
      float a[2 * DIM], r[DIM], cur[DIM], nb[DIM][2 * DIM];
#pragma unroll
      for (int q = 0; q < 2 * DIM; ++q) a[q] = cf.a[1 + q][ci];
      bool in[2 * DIM];
      int nbi[2 * DIM];
      in[0] = rd && i > 0;
      nbi[0] = ob + ((c - 1) >> 1);
      in[1] = rd && i < n0 - 1;
      nbi[1] = ob + ((c + 1) >> 1);
      in[2] = rd && j > 0;
      nbi[2] = ob + h - hy;
      in[3] = rd && j < n1 - 1;
      nbi[3] = ob + h + hy;
      if (DIM == 3) {
        in[2 * DIM - 2] = rd && k > 0;
        nbi[2 * DIM - 2] = ob + h - hz;
        in[2 * DIM - 1] = rd && k < nz - 1;
        nbi[2 * DIM - 1] = ob + h + hz;
      }
#pragma unroll
      for (int n = 0; n < DIM; ++n) {
        r[n] = rs.a[n][ci];
        cur[n] = first ? 0.f : du.a[n][ci];
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) nb[n][q] = in[q] ? du.a[n][nbi[q]] : 0.f;
      }
#pragma unroll
      for (int n = 0; n < DIM; ++n) {
        float sum = 0.f;
#pragma unroll
        for (int q = 0; q < 2 * DIM; ++q) sum += a[q] * nb[n][q];
        const float value = -(r[n] + sum) * iaP;
        const float corr = value - cur[n];
        dmax = fmaxf(dmax, fabsf(corr));
        du.a[n][ci] = cur[n] + corr * omega;
      }
    }
  }
  double v[1] = {(double)dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[color == 0 ? TK_MOM_RED : TK_MOM], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      if (color == 0) {
        ds->red[RS_MOM_DIFF_RED] = out[0];
      } else {
        const double mx = fmax(out[0], ds->red[RS_MOM_DIFF_RED]);
        ds->red[RS_MOM_DIFF] = mx;
        ds->flag[FL_MOM_SWEEPS] += 1;
        if (!(mx > tol)) ds->flag[FL_MOM_DONE] = 1;
      }
    }
  }
}

// The same Jacobi sweep on the FP32 coefficients and residuals of the
// mixed-precision path (o32 of k_mom_assemble: inverse diagonal, 2*DIM
// off-diagonals, DIM residuals): FP32 arithmetic, FP64 only for the max.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT) k_mom_sweep32(Mesh m, float omega, double tol, FP<10> c,
                                                    FP<3> din, FP<3> dout, int limit,
                                                    double* partials, DevScalars* ds, int kch) {
  constexpr bool kPerT = PER;
  if (ds->flag[FL_MOM_DONE] || ds->flag[FL_MOM_SWEEPS] >= limit) return;
  const bool first = ds->flag[FL_MOM_SWEEPS] == 0;
  float dmax = 0.f;
  CELL_LOOP_BEGIN(m, kch)
  float iaP = c.a[0][X.c];
  float a[2 * DIM];
#pragma unroll
  for (int q = 0; q < 2 * DIM; ++q) a[q] = c.a[1 + q][X.c];
#pragma unroll
  for (int n = 0; n < DIM; ++n) {
    float sum = 0.f, cur = 0.f;
    if (!first) {
      cur = din.a[n][X.c];
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        long long s = cell_stride(m, d);
        if (HAS_LO(d)) sum = fmaf(a[2 * d], din.a[n][NB_LO(d, s)], sum);
        if (HAS_HI(d)) sum = fmaf(a[2 * d + 1], din.a[n][NB_HI(d, s)], sum);
      }
    }
    float value = -(c.a[7 + n][X.c] + sum) * iaP;
    float corr = value - cur;
    dmax = fmaxf(dmax, fabsf(corr));
    dout.a[n][X.c] = fmaf(corr, omega, cur);
  }
  CELL_LOOP_END
  double v[1] = {(double)dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[TK_MOM], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_MOM_DIFF] = out[0];
      ds->flag[FL_MOM_SWEEPS] += 1;
      if (!(out[0] > tol)) ds->flag[FL_MOM_DONE] = 1;
    }
  }
}

// The whole Jacobi loop of k_mom_sweep32 by ONE CTA (or one thread-block
// cluster, G = ClusterG) on a plain block (no periodic direction, no
// excluded cell): sweep k reads d[(k+1) % 2] and
// writes d[k % 2] as the grid launches do, with the same per-cell
// arithmetic and the same stop test on the largest correction (a maximum,
// so the result does not depend on the CTA's order), up to `limit` sweeps.
// For small cases run many at once: each takes one SM instead of queueing
// two launches per sweep.
// Group-wide largest correction, the same in every thread (red: 38 floats).
__device__ float grp_max(float v, float* red, const CtaG&) {
  const int tid = threadIdx.x, nt = blockDim.x;
  v = warp_max(v);
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    float w = tid < (nt + 31) / 32 ? red[tid] : 0.f;
    w = warp_max(w);
    if (tid == 0) red[32] = w;
  }
  __syncthreads();
  const float r = red[32];
  __syncthreads();
  return r;
}
// Cluster-wide (red: >= 38 floats): each CTA's maximum goes to red[34 +
// parity]; after one cluster barrier lane q of the first warp reads CTA q's
// and the warp's maximum reaches the CTA's threads through red[36 +
// parity] (slots alternate between calls, as for the FP64 sums of the
// pressure solve).
__device__ float grp_max(float v, float* red, const ClusterG& g) {
  const int tid = threadIdx.x, lane = tid & 31, nw = (blockDim.x + 31) >> 5;
  const int par = g.par;
  g.par ^= 1;
  v = warp_max(v);
  if (lane == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    float w = lane < nw ? red[lane] : 0.f;
    w = warp_max(w);
    if (lane == 0) red[34 + par] = w;
  }
  auto cl = cooperative_groups::this_cluster();
  cl.sync();
  if (tid < 32) {
    const int nb = (int)cl.num_blocks();
    float t = lane < nb ? *cl.map_shared_rank(&red[34 + par], lane) : 0.f;
    t = warp_max(t);
    if (lane == 0) red[36 + par] = t;
  }
  __syncthreads();
  return red[36 + par];
}

template <int DIM, class G>
__global__ void __launch_bounds__(1024) k_cta_mom_jacobi32(Mesh m, float omega, double tol,
                                                           FP<10> c, FP<3> d0, FP<3> d1,
                                                           int limit, int graph,
                                                           DevScalars* ds) {
  constexpr bool kPerT = false;
  __shared__ float red[38];
  const G g;
  const int n = (int)m.nc, tid = g.rank(), nt = g.size();
  int sweeps = 0;
  float dall = 0.f;
  bool done = false;
  for (int k = 0; k < limit; ++k) {
    const FP<3>& din = (k & 1) ? d0 : d1;
    const FP<3>& dout = (k & 1) ? d1 : d0;
    const bool first = k == 0;
    float dmax = 0.f;
    // two cells per thread per pass, every load before the stores (the
    // sweep reads din and writes dout)
    for (int q0 = tid; q0 < n; q0 += 2 * nt) {
      float out[2][DIM];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        Cell X;
        X.c = q0 + u * nt;
        if (X.c >= n) continue;
        X.i[0] = (int)(X.c % m.n[0]);
        const int r = (int)(X.c / m.n[0]);
        X.i[1] = DIM == 3 ? r % m.n[1] : r;
        X.i[2] = DIM == 3 ? r / m.n[1] : 0;
        float iaP = c.a[0][X.c];
        float a[2 * DIM];
#pragma unroll
        for (int e = 0; e < 2 * DIM; ++e) a[e] = c.a[1 + e][X.c];
#pragma unroll
        for (int v = 0; v < DIM; ++v) {
          float sum = 0.f, cur = 0.f;
          if (!first) {
            cur = din.a[v][X.c];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              long long s = cell_stride(m, d);
              if (HAS_LO(d)) sum = fmaf(a[2 * d], din.a[v][NB_LO(d, s)], sum);
              if (HAS_HI(d)) sum = fmaf(a[2 * d + 1], din.a[v][NB_HI(d, s)], sum);
            }
          }
          float value = -(c.a[7 + v][X.c] + sum) * iaP;
          float corr = value - cur;
          dmax = fmaxf(dmax, fabsf(corr));
          out[u][v] = fmaf(corr, omega, cur);
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int q = q0 + u * nt;
        if (q >= n) continue;
#pragma unroll
        for (int v = 0; v < DIM; ++v) dout.a[v][q] = out[u][v];
      }
    }
    dall = grp_max(dmax, red, g);  // also the barrier between sweeps
    sweeps = k + 1;
    if (!((double)dall > tol)) {
      done = true;
      break;
    }
  }
  if (tid == 0) {
    ds->red[RS_MOM_DIFF] = (double)dall;
    ds->flag[FL_MOM_SWEEPS] = sweeps;
    ds->flag[FL_MOM_DONE] = done ? 1 : 0;
    if (graph) ds->flag[FL_STEP_SWEEPS] += sweeps;
  }
}

__global__ void k_f2d3(long long n, int dim, FP<3> in, W3 out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    for (int k = 0; k < dim; ++k) out.a[k][i] = f2d(in.a[k][i]);
}

// ------------------------------------------------------------ Rhie-Chow --
// Face volume fluxes F* by momentum interpolation (fluid.hpp:889-942) and
// face couplings kf = A/(h D_f) of the flux-correction expressions
// (fluid.hpp:946-970); boundary faces carry u_wall.S and kf = 0.  F* and kf
// are stored in FP64 whatever the arithmetic type T, so that the pressure
// system, its FP64 residual and the flux correction see the same numbers;
// kf32 (optional) receives the FP32 couplings of the mixed-precision solve.
// The face velocity and the pressure part of the correction are FP64 (up,
// p, gp are the FP64 iterate and cell pressure gradient); D_f, the force
// terms and du are in T.
template <int DIM, class T, bool PER>
__global__ void k_rhie_chow(Mesh m, Geo g64, GeoT<T> g, FluidCoef fc64, FluidCoefT<T> fc, C3 up,
                            RT<T, 3> du, const double* p, C3 gp, RT<T, 3> force, RT<T, 3> fres,
                            const T* Dc, C3 bv, double* Fs, double* kf, float* kf32, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    int id = X.i[d], nd = m.n[d];
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    const double A = g64.A[d], hA = 0.5 * A;
    const double mv = fc64.meshvel[d] * A;
    // inner face between cm (low side) and cp (high side)
    auto inner = [&](long long cm, long long cp, long long ff) {
      // FP64: the interpolated velocity and the difference of the wide and
      // compact pressure gradients (the cell gradients come from k_force);
      // the two corrections are summed in T, the two velocities in FP64
      double vfi = ((up.a[d][cm] + up.a[d][cp]) + to_d(du.a[d][cm] + du.a[d][cp])) * hA;
      double gpf = (gp.a[d][cm] + gp.a[d][cp]) * 0.5;
      double dpw = gpf - (p[cp] - p[cm]) * g64.inv_h[d];
      T frf = face_vec<DIM, T>(fres, cm, cp, d, fc.geometric);
      T fxf = face_vec<DIM, T>(force, cm, cp, d, fc.geometric);
      T iDf = T(1) / avg(Dc[cm], Dc[cp]);
      T k = g.A[d] * g.inv_h[d] * iDf;
      T corr = fc.rc * ((to_t<T>(dpw) + (fxf - frf)) * g.A[d]) * iDf;
      Fs[ff] = mv != 0. ? vfi + to_d(corr) - mv : vfi + to_d(corr);
      kf[ff] = to_d(k);
      if (kf32) kf32[ff] = (float)k;
    };
    if (HAS_LO(d)) {
      inner(NB_LO(d, s), X.c, f);
    } else {
      Fs[f] = bv.a[d][f] * A - mv;
      kf[f] = 0.;
      if (kf32) kf32[f] = 0.f;
    }
    if (id == nd - 1) {
      long long fh = f + face_stride(m, d);
      if (PER && HAS_HI(d)) {  // across a periodic end, unless excluded
        inner(X.c, NB_HI(d, s), fh);
      } else {
        Fs[fh] = bv.a[d][fh] * A - mv;
        kf[fh] = 0.;
        if (kf32) kf32[fh] = 0.f;
      }
    }
  }
  CELL_LOOP_END
}

// Right-hand side of the pressure-correction rows (fluid.hpp:972-994):
// b_c = sum_f s_f F*_f - S_v V, written as f = -b (A p' = f).
template <int DIM>
__global__ void k_pressure_rhs(Mesh m, Geo g, const double* Fs, const double* Sv, double* f,
                               int kch) {
  CELL_LOOP_BEGIN(m, kch)
  double b = 0.;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    b += Fs[fl + face_stride(m, d)] - Fs[fl];
  }
  if (Sv) b -= Sv[X.c] * g.V;
  f[X.c] = -b;
  CELL_LOOP_END
}

// ----------------------------------------------------------- correction --
// fluid.hpp:1033-1057: p += alpha_p p'; u = u* - grad p'/D_c (p' faces
// extrapolated); F = F* + kf (p'_cm - p'_cp).  Reduces the SIMPLE
// convergence indicator max_c |u_c - u_prev,c| (CalcDiff,
// solver.hpp:804-813) into ds->red[RS_INDICATOR], the square root taken
// once on the maximum.  MIX (mixed path): the velocity and flux increments
// are formed in FP32 from the FP32 momentum correction, diagonal and
// couplings and added to the FP64 state (the p' differences stay FP64);
// the FP32 shadows of the new iterate (u32, p32, F32) are written beside it.
template <int DIM, bool MIX, bool PER>
__global__ void __launch_bounds__(NT) k_correct(Mesh m, Geo g, FluidCoef fc, C3 up, C3 du,
                                                RT<float, 3> du32, const float* Dc32, W3 uic,
                                                const double* pip, double* pic,
                                                const double* pc, const double* Dc,
                                                const double* Fs, const double* kf,
                                                const float* kf32, double* Fic, FP<3> u32,
                                                float* p32, float* F32, double* partials,
                                                DevScalars* ds, int kch) {
  constexpr bool kPerT = PER;
  double dmax = 0.;
  CELL_LOOP_BEGIN(m, kch)
  double pn = pip[X.c] + fc.relax_p * pc[X.c];
  pic[X.c] = pn;
  if (p32) p32[X.c] = d2f(pn);
  double d2 = 0.;
  if (MIX) {
    const float idc = -1.f / Dc32[X.c];
    float e2 = 0.f;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      long long s = cell_stride(m, k);
      const float gpc = d2f(grad_extrap_m<PER>(m, pc, X.c, k, X.i[k], s, g.inv_h[k]));
      const float inc = fmaf(gpc, idc, du32.a[k][X.c]);
      const double un = up.a[k][X.c] + f2d(inc);
      uic.a[k][X.c] = un;
      u32.a[k][X.c] = d2f(un);
      e2 = fmaf(inc, inc, e2);
      long long f = face_id(m, k, X.i[0], X.i[1], X.i[2]);
      const double fv =
          HAS_LO(k) ? Fs[f] + f2d(kf32[f] * d2f(pc[NB_LO(k, s)] - pc[X.c])) : Fs[f];
      Fic[f] = fv;
      F32[f] = d2f(fv);
      if (X.i[k] == m.n[k] - 1) {
        long long fh = f + face_stride(m, k);
        const double fvh =
            HAS_HI(k) ? Fs[fh] + f2d(kf32[fh] * d2f(pc[X.c] - pc[NB_HI(k, s)])) : Fs[fh];
        Fic[fh] = fvh;
        F32[fh] = d2f(fvh);
      }
    }
    d2 = e2;
  } else {
    const double idc = -1. / Dc[X.c];
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      long long s = cell_stride(m, k);
      double gpc = grad_extrap_m<PER>(m, pc, X.c, k, X.i[k], s, g.inv_h[k]);
      double u0 = up.a[k][X.c];
      double un = (u0 + du.a[k][X.c]) + gpc * idc;
      uic.a[k][X.c] = un;
      double dd = un - u0;
      d2 += dd * dd;
      long long f = face_id(m, k, X.i[0], X.i[1], X.i[2]);
      double fv = HAS_LO(k) ? Fs[f] + kf[f] * (pc[NB_LO(k, s)] - pc[X.c]) : Fs[f];
      Fic[f] = fv;
      if (X.i[k] == m.n[k] - 1) {
        // high end face: a boundary face, or across a periodic end the face
        // between this cell (cm) and the first cell (cp)
        long long fh = f + face_stride(m, k);
        double fvh = HAS_HI(k) ? Fs[fh] + kf[fh] * (pc[X.c] - pc[NB_HI(k, s)]) : Fs[fh];
        Fic[fh] = fvh;
      }
    }
  }
  dmax = fmax(dmax, d2);
  CELL_LOOP_END
  double v[1] = {dmax};
  __shared__ double out[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[TK_IND], out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) ds->red[RS_INDICATOR] = sqrt(out[0]);
  }
}

// ------------------------------------------------------------- SIMPLER --
// fluid.hpp:1059-1155, first part: the momentum equations of the iteration
// (relaxed diagonal 1/iaP, off-diagonals, delta-form constants) evaluated
// at the velocity change of the iteration, plus the restored force minus
// the iteration's cell pressure gradient.
template <int DIM, bool PER>
__global__ void k_simpler_eval(Mesh m, CP<7> coef, C3 res, C3 uic, C3 up, C3 fres, C3 gp, W3 ev,
                               int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  const double aPr = 1. / coef.a[0][X.c];
#pragma unroll
  for (int n = 0; n < DIM; ++n) {
    double r = res.a[n][X.c] + aPr * (uic.a[n][X.c] - up.a[n][X.c]);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      long long s = cell_stride(m, d);
      if (HAS_LO(d)) {
        const long long cl = NB_LO(d, s);
        r += coef.a[1 + 2 * d][X.c] * (uic.a[n][cl] - up.a[n][cl]);
      }
      if (HAS_HI(d)) {
        const long long ch = NB_HI(d, s);
        r += coef.a[2 + 2 * d][X.c] * (uic.a[n][ch] - up.a[n][ch]);
      }
    }
    ev.a[n][X.c] = r + (fres.a[n][X.c] - gp.a[n][X.c]);
  }
  CELL_LOOP_END
}

// Second part: on inner faces r_f = (ev_f - f_f).S / D_f + (F_f - u_f.S) /
// rhie_chow_factor, the constant of the pressure rows is -sum_f s_f r_f, and
// the system is solved in delta form around the corrected pressure p:
// A x = sum_f s_f r_f - A' p (A' without the pinned cell's coupling, whose
// row becomes x = value - p).
template <int DIM, bool PER>
__global__ void k_simpler_rhs(Mesh m, Geo g, FluidCoef fc, C3 ev, C3 force, const double* Dc,
                              const double* Fic, C3 uic, const double* kf, const double* dg,
                              const double* p, long long pin, double pin_value, double* f,
                              int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  if (X.c == pin) {
    f[X.c] = pin_value - p[X.c];
    continue;
  }
  double sum = 0., ap = dg[X.c] * p[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      bool inner = side ? HAS_HI(d) : HAS_LO(d);
      if (!inner) continue;
      long long nb = side ? NB_HI(d, s) : NB_LO(d, s);
      long long cm = side ? X.c : nb, cp = side ? nb : X.c;
      long long fq = side ? fl + face_stride(m, d) : fl;
      double e = avg(ev.a[d][cm], ev.a[d][cp]) - face_vec<DIM, double>(force, cm, cp, d, fc.geometric);
      double Df = avg(Dc[cm], Dc[cp]);
      double uf = avg(uic.a[d][cm], uic.a[d][cp]);
      double r = e * g.A[d] / Df + (Fic[fq] - uf * g.A[d]) / fc.rc;
      sum += side ? r : -r;
      if (nb != pin) ap -= kf[fq] * p[nb];
    }
  }
  f[X.c] = sum - ap;
  CELL_LOOP_END
}

__global__ void k_add(long long n, double* a, const double* b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    a[i] += b[i];
}

// --------------------------------------------------------- auto time step --
// FluidSimple::GetAutoTimeStep (fluid.hpp:1191-1206): min over faces with
// F != 0 of |V/F|, 1e10 when there is none.
// min over faces with F != 0 of V / |F| (at most 1e10), formed as
// V / max |F|: correctly rounded division is monotonic, so this is the same
// number, with one division instead of one per face.  The maximum runs on
// the bit patterns of |F| (ordered like the values for non-negative
// doubles; NaNs skipped), which keeps the reduction off the FP64 pipe.
__global__ void __launch_bounds__(NT) k_auto_dt(long long nf, double V, const double* F,
                                                double* partials, DevScalars* ds) {
  constexpr unsigned long long kAbs = 0x7fffffffffffffffULL, kInf = 0x7ff0000000000000ULL;
  unsigned long long bmax = 0;
  long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  for (long long f = blockIdx.x * (long long)NT + tid; f < nf; f += (long long)gridDim.x * NT) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(F[f]) & kAbs;
    if (b <= kInf && b > bmax) bmax = b;
  }
  unsigned long long v[1] = {bmax};
  __shared__ unsigned long long out[1];
  if (grid_reduce<RED_MAX, 1>(v, reinterpret_cast<unsigned long long*>(partials),
                              &ds->ticket[TK_DT], out)) {
    if (tid == 0) {
      const double fmax_abs = __longlong_as_double((long long)out[0]);
      ds->red[RS_AUTO_DT] = fmax_abs > 0. ? fmin(1e10, V / fmax_abs) : 1e10;
    }
  }
}

__global__ void __launch_bounds__(NT) k_nan_count(long long n, const double* a,
                                                  double* partials, DevScalars* ds) {
  double cnt = 0.;
  long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  for (long long i = blockIdx.x * (long long)NT + tid; i < n; i += (long long)gridDim.x * NT)
    if (isnan(a[i])) cnt += 1.;
  double v[1] = {cnt};
  __shared__ double out[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_NAN], out)) {
    if (tid == 0) ds->red[RS_NAN] = out[0];
  }
}

// ----------------------------------------------------------- properties --
// CalcPhasesVolumeFraction (hydro2d.hpp:980-997), GetVolumeAveraged of
// densities and viscosities (1221-1246), zero mass and volume sources
// (chemistry intensity 0), body force rho*g + f with the unsmoothed
// mixture density (CalcForce, hydro2d.hpp:1308-1316).
template <int DIM>
__global__ void k_props(Mesh m, int nph, PhaseProps pp, CP<HYDRO_MAXPH> q,
                        WP<HYDRO_MAXPH> alpha, double* rho_raw, double* rho, double* mu,
                        W3 force, double* Sv, double* Sm, int kch) {
  CELL_LOOP_BEGIN(m, kch)
  double a[HYDRO_MAXPH];
  double sum = 0.;
#pragma unroll
  for (int i = 0; i < HYDRO_MAXPH; ++i) {
    if (i < nph) {
      a[i] = q.a[i][X.c] * pp.idens[i];
      sum += a[i];
    }
  }
  double rr = 0., mm = 0.;
  // one FP64 division per cell (GB300's FP64 rate makes each one count)
  const double isum = 1. / sum;
#pragma unroll
  for (int i = 0; i < HYDRO_MAXPH; ++i) {
    if (i < nph) {
      a[i] *= isum;
      alpha.a[i][X.c] = a[i];
      rr += pp.dens[i] * a[i];
    }
  }
#pragma unroll
  for (int i = 0; i < HYDRO_MAXPH; ++i)
    if (i < nph) mm += pp.visc[i] * a[i];
  rho_raw[X.c] = rr;
  rho[X.c] = rr;
  mu[X.c] = mm;
  Sv[X.c] = 0.;
  Sm[X.c] = 0.;
#pragma unroll
  for (int k = 0; k < DIM; ++k) force.a[k][X.c] = pp.grav[k] * rr + pp.f0[k];
  CELL_LOOP_END
}

// One pass of GetSmoothField (solver.hpp:636-656): face averages with
// zero-derivative boundaries, then the average over the 2*DIM faces
// (solver.hpp:621-634).
template <int DIM, bool PER>
__global__ void k_smooth(Mesh m, const double* in, double* out, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  // mean over the 2 DIM faces of the face averages (the cell's own value on
  // a boundary face) = half the cell value + half the mean of the face
  // neighbours: 2 DIM + 1 FP64 operations instead of three per face
  double vc = in[X.c];
  double sum = 0.;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    sum += HAS_LO(d) ? in[NB_LO(d, s)] : vc;
    sum += HAS_HI(d) ? in[NB_HI(d, s)] : vc;
  }
  out[X.c] = fma(sum, 0.5 / (2. * DIM), 0.5 * vc);
  CELL_LOOP_END
}

// Cell gradient of a scalar with zero-derivative boundary faces.
template <int DIM, bool PER>
__global__ void k_scal_grad(Mesh m, Geo g, const double* a, W3 G, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  double vc = a[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    double flo = HAS_LO(d) ? avg(a[NB_LO(d, s)], vc) : vc;
    double fhi = HAS_HI(d) ? avg(vc, a[NB_HI(d, s)]) : vc;
    G.a[d][X.c] = (fhi - flo) * g.inv_h[d];
  }
  CELL_LOOP_END
}

// Surface-tension force (hydro2d.hpp:1318-1370): g the face gradient of the
// phase-1 volume fraction, n = g/(|g|+1e-6),
// f_c = sigma/V sum_f [ g (S.n) - S |g| ].
template <int DIM, bool PER>
__global__ void k_stforce(Mesh m, Geo g, double sigma, C3 G, W3 out, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  double f[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) f[k] = 0.;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      bool inner = side ? HAS_HI(d) : HAS_LO(d);
      long long nb = inner ? (side ? NB_HI(d, s) : NB_LO(d, s)) : X.c;
      double gv[DIM], n2 = 0.;
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        gv[k] = inner ? avg(G.a[k][side ? X.c : nb], G.a[k][side ? nb : X.c]) : G.a[k][X.c];
        n2 += gv[k] * gv[k];
      }
      double gn = sqrt(n2);
      double so = (side ? 1. : -1.) * g.A[d];
      double sn = so * (gv[d] / (gn + 1e-6));
#pragma unroll
      for (int k = 0; k < DIM; ++k) f[k] += gv[k] * sn;
      f[d] -= so * gn;
    }
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) out.a[k][X.c] = f[k] * g.invV * sigma;
  CELL_LOOP_END
}

// CalcStat (hydro2d.hpp:1432-1493) of one phase: sums of alpha V,
// x alpha V, u alpha V and q V, the boundary volume flux of the phase into
// and out of the domain (flux towards the cell times alpha); min and max
// of q.
template <int DIM>
__global__ void __launch_bounds__(NT) k_stat(Mesh m, Geo g, const double* q, const double* al,
                                             C3 u, const double* F, double* partials,
                                             double* out, unsigned* ticket, int kch) {
  double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  double qmin = 1e10, qmax = -1e10;
  CELL_LOOP_BEGIN(m, kch)
  const double alc = al[X.c];
  double a = alc * g.V;
  s[0] += a;
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    double xc = m.lo[k] + (X.i[k] + 0.5) * g.h[k];
    s[1 + k] += xc * a;
    s[4 + k] += u.a[k][X.c] * a;
  }
  double qc = q[X.c];
  s[7] += qc * g.V;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    // low boundary face: the cell is its second neighbour (flux towards
    // the cell = +F); high boundary face: its first (-F)
    for (int side = 0; side < 2; ++side) {
      bool bnd = side ? X.i[d] == m.n[d] - 1 : X.i[d] == 0;
      if (!bnd || m.per[d]) continue;
      double ftc = side ? -F[f + face_stride(m, d)] : F[f];
      if (ftc >= 0.) s[8] += ftc * alc;
      else s[9] -= ftc * alc;
    }
  }
  qmin = fmin(qmin, qc);
  qmax = fmax(qmax, qc);
  CELL_LOOP_END
  __shared__ double o10[10], o1[1], o2[1];
  if (grid_reduce<RED_SUM, 10>(s, partials, &ticket[0], o10)) {
    if (threadIdx.x == 0 && threadIdx.y == 0)
      for (int a = 0; a < 10; ++a) out[a] = o10[a];
  }
  double vmin[1] = {qmin}, vmax[1] = {qmax};
  if (grid_reduce<RED_MIN, 1>(vmin, partials + 10 * kMaxBlocks, &ticket[1], o1)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) out[10] = o1[0];
  }
  if (grid_reduce<RED_MAX, 1>(vmax, partials + 11 * kMaxBlocks, &ticket[2], o2)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) out[11] = o2[0];
  }
}

// Initial volume fluxes of the FluidSimple ctor (fluid.hpp:770-784):
// F = u_f.S - meshvel.S with the velocity value condition on boundaries.
template <int DIM, bool PER>
__global__ void k_init_flux(Mesh m, Geo g, FluidCoef fc, C3 u, C3 bv, double* F, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    double mv = fc.meshvel[d] * g.A[d];
    if (HAS_LO(d)) F[f] = avg(u.a[d][NB_LO(d, s)], u.a[d][X.c]) * g.A[d] - mv;
    else F[f] = bv.a[d][f] * g.A[d] - mv;
    if (X.i[d] == m.n[d] - 1)
      F[f + face_stride(m, d)] =
          HAS_HI(d) ? avg(u.a[d][X.c], u.a[d][NB_HI(d, s)]) * g.A[d] - mv
                   : bv.a[d][f + face_stride(m, d)] * g.A[d] - mv;
  }
  CELL_LOOP_END
}

// ------------------------------------------------- boundary conditions --
// Value conditions of the velocity on the boundary faces (fluid.hpp:695-731):
// walls and inlets their given velocity, outlets zero until the first
// rebalancing (OutletAuto, fluid.hpp:340-364).  Side kinds in `kind`.
template <int DIM>
__global__ void k_bc_fill(Mesh m, BcSpec sp, W3 bv, FP<3> bv32, int kch) {
  CELL_LOOP_BEGIN(m, kch)
  // boundary faces of an excluded cell carry no condition (velocity 0)
  const bool exc = m.ex && m.ex[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (m.per[d] || (side ? X.i[d] != m.n[d] - 1 : X.i[d] != 0)) continue;
      long long fb = side ? f + face_stride(m, d) : f;
      int q = 2 * d + side;
      for (int k = 0; k < DIM; ++k) {
        double v = (exc || sp.kind[q] == HYDRO_BC_OUTLET) ? 0. : sp.vel[q][k];
        bv.a[k][fb] = v;
        if (bv32.a[0]) bv32.a[k][fb] = (float)v;
      }
    }
  }
  CELL_LOOP_END
}

// Inlet faces carry the partial densities of their cell at the start
// (hydro2d.hpp:566-582).
template <int DIM>
__global__ void k_qin_fill(Mesh m, BcSpec sp, int nph, CP<HYDRO_MAXPH> q, WP<HYDRO_MAXPH> qin,
                           int kch) {
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (m.per[d] || (side ? X.i[d] != m.n[d] - 1 : X.i[d] != 0)) continue;
      if (sp.kind[2 * d + side] != HYDRO_BC_INLET) continue;
      long long fb = side ? f + face_stride(m, d) : f;
      for (int i = 0; i < nph; ++i) qin.a[i][fb] = q.a[i][X.c];
    }
  }
  CELL_LOOP_END
}

// UpdateOutletBaseConditions (fluid.hpp:542-600), reduction part: outlet
// faces take the velocity of their cell (the latest iterate u); sums of the
// outlet volume flux (outward), the outlet area, the inlet volume flux
// (inward) and the volume sources S_v V go to ds->red[RS_OUT_*].
template <int DIM>
__global__ void __launch_bounds__(NT) k_outlet_sums(Mesh m, Geo g, BcSpec sp, C3 u, W3 bv,
                                                    const double* Sv, double* partials,
                                                    DevScalars* ds, int kch) {
  double sm[4] = {0., 0., 0., 0.};
  CELL_LOOP_BEGIN(m, kch)
  if (Sv) sm[3] += Sv[X.c] * g.V;
  const bool exc = m.ex && m.ex[X.c];  // excluded boundary faces: no condition
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (exc) continue;
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (m.per[d] || (side ? X.i[d] != m.n[d] - 1 : X.i[d] != 0)) continue;
      long long fb = side ? f + face_stride(m, d) : f;
      int kind = sp.kind[2 * d + side];
      // the cell is the face's first neighbour on the high side
      if (kind == HYDRO_BC_OUTLET) {
        for (int k = 0; k < DIM; ++k) bv.a[k][fb] = u.a[k][X.c];
        sm[0] += bv.a[d][fb] * g.A[d] * (side ? 1. : -1.);
        sm[1] += g.A[d];
      } else if (kind == HYDRO_BC_INLET) {
        sm[2] += bv.a[d][fb] * g.A[d] * (side ? -1. : 1.);
      }
    }
  }
  CELL_LOOP_END
  __shared__ double o[4];
  if (grid_reduce<RED_SUM, 4>(sm, partials, &ds->ticket[TK_OUTLET], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      ds->red[RS_OUT_FLUX] = o[0];
      ds->red[RS_OUT_AREA] = o[1];
      ds->red[RS_IN_FLUX] = o[2] + o[3];
    }
  }
}

// Correction part: outlet velocity += normal (in - out)/area (outward).
template <int DIM>
__global__ void k_outlet_set(Mesh m, BcSpec sp, W3 bv, FP<3> bv32, const DevScalars* ds,
                             int kch) {
  const double corr = (ds->red[RS_IN_FLUX] - ds->red[RS_OUT_FLUX]) / ds->red[RS_OUT_AREA];
  CELL_LOOP_BEGIN(m, kch)
  const bool exc = m.ex && m.ex[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (exc) continue;
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (m.per[d] || (side ? X.i[d] != m.n[d] - 1 : X.i[d] != 0)) continue;
      if (sp.kind[2 * d + side] != HYDRO_BC_OUTLET) continue;
      long long fb = side ? f + face_stride(m, d) : f;
      bv.a[d][fb] = bv.a[d][fb] + corr * (side ? 1. : -1.);
      if (bv32.a[0])
        for (int k = 0; k < DIM; ++k) bv32.a[k][fb] = (float)bv.a[k][fb];
    }
  }
  CELL_LOOP_END
}

}  // namespace

// ------------------------------------------------------------ launchers --
// Cell kernels are launched in whole waves of their own occupancy
// (cell_launch_waves).
#define DISPATCH_DIM(m, KERNEL, ...)                                     \
  do {                                                                   \
    Launch L = cell_launch_waves(m, resident_ctas((m).dim == 3 ? (const void*)KERNEL<3> : (const void*)KERNEL<2>)); \
    if ((m).dim == 3)                                                    \
      KERNEL<3><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);         \
    else                                                                 \
      KERNEL<2><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);         \
    count_launches(1);                                                   \
    return cudaGetLastError();                                           \
  } while (0)
#define DISPATCH_DIM_P(m, KERNEL, ...)                                   \
  do {                                                                   \
    Launch L = cell_launch_waves(m, resident_ctas(CELL_KERNEL_P(m, KERNEL))); \
    CELL_LAUNCH_P(m, L, st, KERNEL, __VA_ARGS__);                        \
    count_launches(1);                                                   \
    return cudaGetLastError();                                           \
  } while (0)
#define DISPATCH_DIM_TP(m, KERNEL, T, ...)                               \
  do {                                                                   \
    Launch L = cell_launch_waves(m, resident_ctas(CELL_KERNEL_TP(m, KERNEL, T))); \
    CELL_LAUNCH_TP(m, L, st, KERNEL, T, __VA_ARGS__);                    \
    count_launches(1);                                                   \
    return cudaGetLastError();                                           \
  } while (0)
#define DISPATCH_DIM_T(m, KERNEL, T, ...)                                \
  do {                                                                   \
    Launch L = cell_launch_waves(m, resident_ctas((m).dim == 3 ? (const void*)KERNEL<3, T> : (const void*)KERNEL<2, T>)); \
    if ((m).dim == 3)                                                    \
      KERNEL<3, T><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);      \
    else                                                                 \
      KERNEL<2, T><<<L.grid, L.block, 0, st>>>(__VA_ARGS__, L.kch);      \
    count_launches(1);                                                   \
    return cudaGetLastError();                                           \
  } while (0)

template <class T>
FluidCoefT<T> coef_as(const FluidCoef& fc) {
  FluidCoefT<T> r;
  for (int a = 0; a < 6; ++a)
    for (int k = 0; k < 3; ++k) r.bcu[a][k] = (T)fc.bcu[a][k];
  r.relax_u = (T)fc.relax_u;
  r.relax_p = (T)fc.relax_p;
  r.rc = (T)fc.rc;
  for (int k = 0; k < 3; ++k) {
    r.co[k] = (T)fc.co[k];
    r.meshvel[k] = (T)fc.meshvel[k];
  }
  r.geometric = fc.geometric;
  r.sources = fc.sources;
  return r;
}

static int flat_blocks(long long n) {
  long long b = (n + NT - 1) / NT;
  if (b > kMaxBlocks) b = kMaxBlocks;
  if (b < 1) b = 1;
  return (int)b;
}
// grid of a grid-stride reduction: 16 blocks per SM at most, so that the
// last block folds a few thousand partials, not one per 256 elements
static int flat_blocks_red(long long n) {
  const int b = flat_blocks(n);
  return b < 152 * 16 ? b : 152 * 16;
}

cudaError_t launch_start_step(const Mesh& m, double ge, W3 u_ic, C3 u_tc, C3 u_tp,
                              double* p_ic, const double* p_tc, const double* p_tp,
                              double* F_ic, const double* F_tc, const double* F_tp,
                              cudaStream_t st) {
  int nb = flat_blocks(m.nc);
  for (int k = 0; k < m.dim; ++k)
    k_axpy_extrap<<<nb, NT, 0, st>>>(m.nc, ge, u_ic.a[k], u_tc.a[k], u_tp.a[k]);
  k_axpy_extrap<<<nb, NT, 0, st>>>(m.nc, ge, p_ic, p_tc, p_tp);
  k_axpy_extrap<<<flat_blocks(m.nf), NT, 0, st>>>(m.nf, ge, F_ic, F_tc, F_tp);
  count_launches(m.dim + 2);
  return cudaGetLastError();
}

cudaError_t launch_init_flux(const Mesh& m, const FluidCoef& fc, C3 u, C3 bv, double* F,
                             cudaStream_t st) {
  DISPATCH_DIM_P(m, k_init_flux, m, make_geo(m), fc, u, bv, F);
}

cudaError_t launch_bc_fill(const Mesh& m, const BcSpec& sp, W3 bv, FP<3> bv32, cudaStream_t st) {
  DISPATCH_DIM(m, k_bc_fill, m, sp, bv, bv32);
}

cudaError_t launch_qin_fill(const Mesh& m, const BcSpec& sp, int nph, CP<HYDRO_MAXPH> q,
                            WP<HYDRO_MAXPH> qin, cudaStream_t st) {
  DISPATCH_DIM(m, k_qin_fill, m, sp, nph, q, qin);
}

cudaError_t launch_outlet_update(const Mesh& m, const BcSpec& sp, C3 u, W3 bv, FP<3> bv32,
                                 const double* Sv, double* partials, DevScalars* ds,
                                 cudaStream_t st) {
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  if (m.dim == 3) {
    k_outlet_sums<3><<<L.grid, L.block, 0, st>>>(m, g, sp, u, bv, Sv, partials, ds, L.kch);
    k_outlet_set<3><<<L.grid, L.block, 0, st>>>(m, sp, bv, bv32, ds, L.kch);
  } else {
    k_outlet_sums<2><<<L.grid, L.block, 0, st>>>(m, g, sp, u, bv, Sv, partials, ds, L.kch);
    k_outlet_set<2><<<L.grid, L.block, 0, st>>>(m, sp, bv, bv32, ds, L.kch);
  }
  count_launches(2);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_vel_grad(const Mesh& m, const FluidCoef& fc, RT<T, 3> u, RT<T, 3> bv,
                            WT<T, 9> G, cudaStream_t st) {
  DISPATCH_DIM_TP(m, k_vel_grad, T, m, make_geo<T>(m), coef_as<T>(fc), u, bv, G);
}

template <class T>
cudaError_t launch_force(const Mesh& m, const FluidCoef& fc, RT<T, 3> u, RT<T, 9> G,
                         const double* p, const T* mu, const T* rho, RT<T, 3> force,
                         RT<T, 3> stforce, const T* Sv, const T* Sm, WT<T, 3> fo,
                         WT<T, 3> fres, W3 gp, cudaStream_t st) {
  DISPATCH_DIM_TP(m, k_force, T, m, make_geo<T>(m), coef_as<T>(fc), u, G, p, make_geo(m), mu,
                 rho, force, stforce, Sv, Sm, fo, fres, gp);
}

template <class T>
cudaError_t launch_mom_assemble(const Mesh& m, const FluidCoef& fc, RT<T, 3> u_prev,
                                RT<T, 3> u_tc, RT<T, 3> u_tp, RT<T, 9> G, const T* F,
                                const T* rho, const T* mu, RT<T, 3> fo, C3 up64, C3 utc64,
                                C3 utp64, RT<T, 3> bv, WT<T, 7> coef, WT<T, 3> res, T* Dc,
                                int split, cudaStream_t st) {
  Unsteady64 us;
  for (int k = 0; k < 3; ++k) {
    us.co[k] = fc.co[k];
    us.up[k] = up64.a[k];
    us.utc[k] = utc64.a[k];
    us.utp[k] = utp64.a[k];
  }
  DISPATCH_DIM_TP(m, k_mom_assemble, T, m, make_geo<T>(m), coef_as<T>(fc), u_prev, u_tc, u_tp,
                 G, F, rho, mu, fo, us, bv, coef, res, Dc, split);
}

template <class T>
cudaError_t launch_rhie_chow(const Mesh& m, const FluidCoef& fc, C3 u_prev, RT<T, 3> du,
                             const double* p, C3 gp, RT<T, 3> force, RT<T, 3> fres,
                             const T* Dc, C3 bv, double* Fs, double* kf, float* kf32,
                             cudaStream_t st) {
  DISPATCH_DIM_TP(m, k_rhie_chow, T, m, make_geo(m), make_geo<T>(m), fc, coef_as<T>(fc), u_prev,
                 du, p, gp, force, fres, Dc, bv, Fs, kf, kf32);
}

#define HG_INST_FLUID(T)                                                                      \
  template cudaError_t launch_vel_grad<T>(const Mesh&, const FluidCoef&, RT<T, 3>, RT<T, 3>,  \
                                          WT<T, 9>, cudaStream_t);                            \
  template cudaError_t launch_force<T>(const Mesh&, const FluidCoef&, RT<T, 3>, RT<T, 9>,     \
                                       const double*, const T*, const T*, RT<T, 3>, RT<T, 3>, \
                                       const T*, const T*, WT<T, 3>, WT<T, 3>, W3,            \
                                       cudaStream_t);                                         \
  template cudaError_t launch_mom_assemble<T>(const Mesh&, const FluidCoef&, RT<T, 3>,        \
                                              RT<T, 3>, RT<T, 3>, RT<T, 9>, const T*,         \
                                              const T*, const T*, RT<T, 3>, C3, C3, C3,       \
                                              RT<T, 3>, WT<T, 7>, WT<T, 3>, T*, int,          \
                                              cudaStream_t);                                  \
  template cudaError_t launch_rhie_chow<T>(const Mesh&, const FluidCoef&, C3, RT<T, 3>,       \
                                           const double*, C3, RT<T, 3>, RT<T, 3>, const T*,   \
                                           C3, double*, double*, float*, cudaStream_t);
HG_INST_FLUID(double)
HG_INST_FLUID(float)
#undef HG_INST_FLUID

cudaError_t launch_d2f(long long n, const double* in, float* out, cudaStream_t st) {
  k_d2f<<<flat_blocks(n), NT, 0, st>>>(n, in, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mom_sweep32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> din,
                               FP<3> dout, int limit, double* partials, DevScalars* ds,
                               cudaStream_t st) {
  DISPATCH_DIM_P(m, k_mom_sweep32, m, (float)omega, tol, c, din, dout, limit, partials, ds);
}

cudaError_t launch_cta_mom_jacobi32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> d0,
                                    FP<3> d1, int limit, int graph, int threads, int cluster,
                                    DevScalars* ds, cudaStream_t st) {
  if (any_periodic(m) || m.nc >= (1LL << 31) || threads < 32 || threads > 1024 || threads % 32 ||
      cluster < 1 || cluster > 8)
    return cudaErrorInvalidValue;
  const float om = (float)omega;
  if (cluster == 1) {
    if (m.dim == 3)
      k_cta_mom_jacobi32<3, CtaG><<<1, threads, 0, st>>>(m, om, tol, c, d0, d1, limit, graph, ds);
    else
      k_cta_mom_jacobi32<2, CtaG><<<1, threads, 0, st>>>(m, om, tol, c, d0, d1, limit, graph, ds);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(threads);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e =
        m.dim == 3
            ? cudaLaunchKernelEx(&cfg, k_cta_mom_jacobi32<3, ClusterG>, m, om, tol, c, d0, d1, limit,
                                 graph, ds)
            : cudaLaunchKernelEx(&cfg, k_cta_mom_jacobi32<2, ClusterG>, m, om, tol, c, d0, d1, limit,
                                 graph, ds);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_f2d3(const Mesh& m, FP<3> in, W3 out, cudaStream_t st) {
  k_f2d3<<<flat_blocks(m.nc), NT, 0, st>>>(m.nc, m.dim, in, out);
  count_launches(1);
  return cudaGetLastError();
}

namespace {
// Color-blocked (index color * nc/2 + c/2, nx even) to cell order: thread
// (x, y) takes the pair (2x, 2x+1) of row (j, k), whose first cell has color
// (j + k) % 2; both cells share the blocked index c/2.
template <int DIM>
__global__ void __launch_bounds__(NT) k_unsplit3(Mesh m, FP<3> in, FP<3> out, int kch) {
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int nz = DIM == 3 ? m.n[2] : 1;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, nz);
  if (2 * ih >= m.n[0] || j >= m.n[1]) return;
  const long long half = m.nc / 2;
  for (int k = k0; k < k1; ++k) {
    const long long c = cell_id(m, 2 * ih, j, k);
    const long long h = c >> 1;
    const int a = (j + k) & 1;
#pragma unroll
    for (int n = 0; n < DIM; ++n) {
      const float e = in.a[n][a * half + h], o = in.a[n][(1 - a) * half + h];
      *reinterpret_cast<float2*>(out.a[n] + c) = make_float2(e, o);
    }
  }
}
}  // namespace

cudaError_t launch_unsplit3(const Mesh& m, FP<3> in, FP<3> out, cudaStream_t st) {
  if (m.n[0] % 2) return cudaErrorInvalidValue;
  Mesh h = m;
  h.n[0] = m.n[0] / 2;
  Launch L = cell_launch(h);
  if (m.dim == 3) k_unsplit3<3><<<L.grid, L.block, 0, st>>>(m, in, out, L.kch);
  else k_unsplit3<2><<<L.grid, L.block, 0, st>>>(m, in, out, L.kch);
  count_launches(1);
  return cudaGetLastError();
}

namespace {
// Grid of a red-black half-sweep: one thread per cell pair along x, sized
// in whole waves over the half-width mesh.
Launch rb_launch(const Mesh& m, const void* kernel) {
  Mesh h = m;
  h.n[0] = (m.n[0] + 1) / 2;
  return cell_launch_waves(h, resident_ctas(kernel));
}
}  // namespace

cudaError_t launch_mom_rbgs(const Mesh& m, double omega, double tol, CP<7> coef, C3 res, W3 du,
                            int color, int split, int limit, double* partials, DevScalars* ds,
                            cudaStream_t st) {
  const bool p = any_periodic(m);
#define RBGS64(D, P, S)                                                                       \
  do {                                                                                        \
    Launch L = rb_launch(m, (const void*)k_mom_rbgs<D, P, double, S, false>);                        \
    k_mom_rbgs<D, P, double, S, false><<<L.grid, L.block, 0, st>>>(m, omega, tol, coef, res, du,     \
                                                            color, limit, partials, ds, L.kch); \
  } while (0)
  if (m.dim == 3) {
    if (split) { if (p) RBGS64(3, true, true); else RBGS64(3, false, true); }
    else { if (p) RBGS64(3, true, false); else RBGS64(3, false, false); }
  } else {
    if (split) { if (p) RBGS64(2, true, true); else RBGS64(2, false, true); }
    else { if (p) RBGS64(2, true, false); else RBGS64(2, false, false); }
  }
#undef RBGS64
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mom_rbgs32(const Mesh& m, double omega, double tol, FP<10> c, FP<3> du,
                              int color, int limit, double* partials, DevScalars* ds,
                              cudaStream_t st) {
  RT<float, 7> cf{};
  RT<float, 3> rs{};
  for (int q = 0; q < 7; ++q) cf.a[q] = c.a[q];
  for (int k = 0; k < 3; ++k) rs.a[k] = c.a[7 + k];
  const bool p = any_periodic(m);
  const float om = (float)omega;
#define RBGS32(D, P)                                                                        \
  do {                                                                                      \
    Launch L = rb_launch(m, (const void*)k_mom_rbgs<D, P, float, true, true>);              \
    k_mom_rbgs<D, P, float, true, true><<<L.grid, L.block, 0, st>>>(m, om, tol, cf, rs, du,  \
                                                                    color, limit, partials, \
                                                                    ds, L.kch);             \
  } while (0)
  if (!p && m.nc < (1LL << 31)) {
#define RBGSF(D)                                                                            \
  do {                                                                                      \
    Launch L = rb_launch(m, (const void*)k_mom_rbgs_f32<D>);                                \
    k_mom_rbgs_f32<D><<<L.grid, L.block, 0, st>>>(m, om, tol, cf, rs, du, color, limit,     \
                                                  partials, ds, L.kch);                     \
  } while (0)
    if (m.dim == 3) RBGSF(3); else RBGSF(2);
#undef RBGSF
  } else if (m.dim == 3) {
    if (p) RBGS32(3, true); else RBGS32(3, false);
  } else {
    if (p) RBGS32(2, true); else RBGS32(2, false);
  }
#undef RBGS32
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mom_sweep(const Mesh& m, double omega, double tol, CP<7> coef, C3 res,
                             C3 din, W3 dout, int limit, double* partials, DevScalars* ds,
                             cudaStream_t st) {
  DISPATCH_DIM_P(m, k_mom_sweep, m, omega, tol, coef, res, din, dout, limit, partials, ds);
}

cudaError_t launch_pressure_rhs(const Mesh& m, const double* Fs, const double* Sv, double* f,
                                cudaStream_t st) {
  DISPATCH_DIM(m, k_pressure_rhs, m, make_geo(m), Fs, Sv, f);
}

cudaError_t launch_correct(const Mesh& m, const FluidCoef& fc, C3 u_prev, C3 du,
                           RT<float, 3> du32, const float* Dc32, W3 u_ic, const double* p_ip,
                           double* p_ic, const double* pc, const double* Dc, const double* Fs,
                           const double* kf, const float* kf32, double* F_ic, FP<3> u32,
                           float* p32, float* F32, double* partials, DevScalars* ds,
                           cudaStream_t st) {
  Launch L = cell_launch_waves(m, resident_ctas(du32.a[0] ? CELL_KERNEL_TP(m, k_correct, true)
                                                          : CELL_KERNEL_TP(m, k_correct, false)));
  if (du32.a[0])
    CELL_LAUNCH_TP(m, L, st, k_correct, true, m, make_geo(m), fc, u_prev, du, du32, Dc32, u_ic,
                   p_ip, p_ic, pc, Dc, Fs, kf, kf32, F_ic, u32, p32, F32, partials, ds);
  else
    CELL_LAUNCH_TP(m, L, st, k_correct, false, m, make_geo(m), fc, u_prev, du, du32, Dc32, u_ic,
                   p_ip, p_ic, pc, Dc, Fs, kf, kf32, F_ic, u32, p32, F32, partials, ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_simpler_rhs(const Mesh& m, const FluidCoef& fc, CP<7> coef, C3 res, C3 uic,
                               C3 up, C3 fres, C3 gp, C3 force, const double* Dc,
                               const double* Fic, const double* kf, const double* dg,
                               const double* p, long long pin, double pin_value, W3 ev,
                               double* f, cudaStream_t st) {
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  C3 evc{};
  for (int k = 0; k < 3; ++k) evc.a[k] = ev.a[k];
  CELL_LAUNCH_P(m, L, st, k_simpler_eval, m, coef, res, uic, up, fres, gp, ev);
  CELL_LAUNCH_P(m, L, st, k_simpler_rhs, m, g, fc, evc, force, Dc, Fic, uic, kf, dg, p, pin,
                pin_value, f);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t launch_add(long long n, double* a, const double* b, cudaStream_t st) {
  k_add<<<flat_blocks(n), NT, 0, st>>>(n, a, b);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_auto_dt(const Mesh& m, const double* F, double* partials, DevScalars* ds,
                           cudaStream_t st) {
  k_auto_dt<<<flat_blocks_red(m.nf), dim3(BX, BY), 0, st>>>(m.nf, m.V, F, partials, ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_nan_count(long long n, const double* a, double* partials, DevScalars* ds,
                             cudaStream_t st) {
  k_nan_count<<<flat_blocks_red(n), dim3(BX, BY), 0, st>>>(n, a, partials, ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_props(const Mesh& m, int nph, const PhaseProps& pp, CP<HYDRO_MAXPH> q,
                         WP<HYDRO_MAXPH> alpha, double* rho_raw, double* rho, double* mu,
                         W3 force, double* Sv, double* Sm, cudaStream_t st) {
  DISPATCH_DIM(m, k_props, m, nph, pp, q, alpha, rho_raw, rho, mu, force, Sv, Sm);
}

cudaError_t launch_smooth(const Mesh& m, const double* in, double* out, cudaStream_t st) {
  DISPATCH_DIM_P(m, k_smooth, m, in, out);
}

cudaError_t launch_stforce(const Mesh& m, double sigma, const double* alpha1, W3 G, W3 out,
                           cudaStream_t st) {
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  C3 Gc = {{G.a[0], G.a[1], G.a[2]}};
  CELL_LAUNCH_P(m, L, st, k_scal_grad, m, g, alpha1, G);
  CELL_LAUNCH_P(m, L, st, k_stforce, m, g, sigma, Gc, out);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t launch_stat(const Mesh& m, const double* q, const double* alpha, C3 u,
                        const double* F, double* partials, double* out, unsigned* ticket,
                        cudaStream_t st) {
  DISPATCH_DIM(m, k_stat, m, make_geo(m), q, alpha, u, F, partials, out, ticket);
}

}  // namespace hg
