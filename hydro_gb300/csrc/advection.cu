// advection.cu -- explicit TVD advection of the partial densities on
// sm_103a (AdvectionSolverMultiExplicit::MakeIteration, advection.hpp:440-539).
//
// Per substep and (split) stage: k_adv_faces evaluates, for every phase,
// the Superbee face value (InterpolateSuperbee, solver.hpp:550-619) from the
// cell gradients of the two neighbours (Green-Gauss with zero-derivative
// boundary faces, hydro2d.hpp:576-590) and stores q_f F_f; k_adv_update
// applies q -= dt/V sum_f s_f q_f F_f.  Faces are computed once, the update
// is out of place (the reference evaluates all faces before updating).
#include <math.h>

#include "kernels.h"
#include "loop.cuh"

namespace hg {

namespace {

__device__ __forceinline__ double superbee(double p, double q) {
  if (p > 0. && q > 0.) return fmax(fmin(2. * p, q), fmin(p, 2. * q));
  if (p < 0. && q < 0.) return -fmax(fmin(-2. * p, -q), fmin(-p, -2. * q));
  return 0.;
}

// Superbee value on the inner face between P (low) and E (high) along an
// axis of stride s; idP is P's index along that axis.  bP / bE: values of
// P's low / E's high face when those are boundary faces (the advection
// condition: the inlet value, else the cell's own, zero derivative).
__device__ __forceinline__ double superbee_face(const double* q, long long P, long long E,
                                                long long s, int idP, int nd, double Ff,
                                                double h, double inv_h, double bP, double bE) {
  double qP = q[P], qE = q[E];
  if (Ff > 1e-8) {
    double flo = idP > 0 ? avg(q[P - s], qP) : bP;
    double gP = (avg(qP, qE) - flo) * inv_h;
    double dq = qE - qP;
    return qP + 0.5 * superbee(dq, -4. * (gP * (-0.5 * h)) - dq);
  } else if (Ff < -1e-8) {
    double fhi = idP + 1 < nd - 1 ? avg(qE, q[E + s]) : bE;
    double gE = (fhi - avg(qP, qE)) * inv_h;
    double dq = qE - qP;
    return qE - 0.5 * superbee(dq, 4. * (gE * (0.5 * h)) - dq);
  }
  return 0.5 * (qP + qE);
}

// inlet_mask: bit q set when side q (xm, xp, ym, ...) is an inlet; qin
// holds the inlet values on those boundary faces.
template <int DIM>
__global__ void k_adv_faces(Mesh m, Geo g, int nph, int stage, int nstages, const double* F,
                            CP<HYDRO_MAXPH> q, int inlet_mask, CP<HYDRO_MAXPH> qin,
                            WP<HYDRO_MAXPH> qflux, int kch) {
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (nstages > 1 && d != stage) continue;
    long long s = cell_stride(m, d);
    int id = X.i[d], nd = m.n[d];
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    long long fs = face_stride(m, d);
    const bool in_lo = (inlet_mask >> (2 * d)) & 1, in_hi = (inlet_mask >> (2 * d + 1)) & 1;
    double Ff = F[f];
    for (int i = 0; i < nph; ++i) {
      double qf;
      if (id > 0) {
        // P = X.c - s: its low face is a boundary face when id == 1; the
        // current cell E's high face when id == nd - 1
        double bP = q.a[i][X.c - s], bE = q.a[i][X.c];
        if (id == 1 && in_lo) bP = qin.a[i][f - fs];
        if (id == nd - 1 && in_hi) bE = qin.a[i][f + fs];
        qf = superbee_face(q.a[i], X.c - s, X.c, s, id - 1, nd, Ff, g.h[d], g.inv_h[d], bP, bE);
      } else {
        qf = in_lo ? qin.a[i][f] : q.a[i][X.c];
      }
      qflux.a[i][f] = qf * Ff;
    }
    if (id == nd - 1) {
      long long fh = f + fs;
      double Fh = F[fh];
      for (int i = 0; i < nph; ++i) qflux.a[i][fh] = (in_hi ? qin.a[i][fh] : q.a[i][X.c]) * Fh;
    }
  }
  CELL_LOOP_END
}

template <int DIM>
__global__ void k_adv_update(Mesh m, int nph, int stage, int nstages, double mdtv,
                             CP<HYDRO_MAXPH> qflux, CP<HYDRO_MAXPH> qin, WP<HYDRO_MAXPH> qout,
                             int kch) {
  CELL_LOOP_BEGIN(m, kch)
  for (int i = 0; i < nph; ++i) {
    double sum = 0.;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      if (nstages > 1 && d != stage) continue;
      long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
      sum += -qflux.a[i][fl];
      sum += qflux.a[i][fl + face_stride(m, d)];
    }
    qout.a[i][X.c] = qin.a[i][X.c] + mdtv * sum;
  }
  CELL_LOOP_END
}

// Interface sharpening (advection.hpp:481-530): with a the face value and gf
// the face gradient of q (zero-derivative boundaries), on faces where
// |gf| >= 1: n = gf/(|gf|+1e-6), ff = |F n_d| n_d (sharp A |gf| - a (1 -
// a/amax)); q += dt/V sum_f s_f ff.
template <int DIM>
__global__ void k_sharpen(Mesh m, Geo g, double sharp, double amax, double dtv, const double* F,
                          const double* q, C3 G, double* qout, int kch) {
  CELL_LOOP_BEGIN(m, kch)
  double sh = 0.;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      bool inner = side ? X.i[d] < m.n[d] - 1 : X.i[d] > 0;
      long long nb = side ? X.c + s : X.c - s;
      long long f = fl + side * face_stride(m, d);
      double af = inner ? avg(q[side ? X.c : nb], q[side ? nb : X.c]) : q[X.c];
      double gv[DIM], n2 = 0.;
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        gv[k] = inner ? avg(G.a[k][side ? X.c : nb], G.a[k][side ? nb : X.c]) : G.a[k][X.c];
        n2 += gv[k] * gv[k];
      }
      double gn = sqrt(n2);
      double ff = 0.;
      if (!(gn < 1.)) {
        double nf = gv[d] / (gn + 1e-6);
        double uf = F[f];
        ff = fabs(uf * nf) * nf * (sharp * g.A[d] * gn - af * (1. - af / amax));
      }
      sh += (side ? 1. : -1.) * ff;
    }
  }
  qout[X.c] = q[X.c] + dtv * sh;
  CELL_LOOP_END
}

template <int DIM>
__global__ void k_grad0(Mesh m, Geo g, const double* a, W3 G, int kch) {
  CELL_LOOP_BEGIN(m, kch)
  double vc = a[X.c];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    double flo = X.i[d] > 0 ? avg(a[X.c - s], vc) : vc;
    double fhi = X.i[d] < m.n[d] - 1 ? avg(vc, a[X.c + s]) : vc;
    G.a[d][X.c] = (fhi - flo) * g.inv_h[d];
  }
  CELL_LOOP_END
}

}  // namespace

cudaError_t launch_adv_faces(const Mesh& m, int nph, int stage, int nstages, const double* F,
                             CP<HYDRO_MAXPH> q, int inlet_mask, CP<HYDRO_MAXPH> qin,
                             WP<HYDRO_MAXPH> qflux, cudaStream_t st) {
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  if (m.dim == 3)
    k_adv_faces<3><<<L.grid, L.block, 0, st>>>(m, g, nph, stage, nstages, F, q, inlet_mask, qin,
                                               qflux, L.kch);
  else
    k_adv_faces<2><<<L.grid, L.block, 0, st>>>(m, g, nph, stage, nstages, F, q, inlet_mask, qin,
                                               qflux, L.kch);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_adv_update(const Mesh& m, int nph, int stage, int nstages, double dt,
                              CP<HYDRO_MAXPH> qflux, CP<HYDRO_MAXPH> qin, WP<HYDRO_MAXPH> qout,
                              cudaStream_t st) {
  Launch L = cell_launch(m);
  double mdtv = -dt / m.V;
  if (m.dim == 3)
    k_adv_update<3><<<L.grid, L.block, 0, st>>>(m, nph, stage, nstages, mdtv, qflux, qin, qout,
                                               L.kch);
  else
    k_adv_update<2><<<L.grid, L.block, 0, st>>>(m, nph, stage, nstages, mdtv, qflux, qin, qout,
                                               L.kch);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_adv_sharpen(const Mesh& m, int phase, double sharp, double amax, double dt,
                               const double* F, double* q, double* qtmp, W3 G, double* fwork,
                               cudaStream_t st) {
  (void)phase;
  (void)fwork;
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  C3 Gc = {{G.a[0], G.a[1], G.a[2]}};
  double dtv = dt / m.V;
  if (m.dim == 3) {
    k_grad0<3><<<L.grid, L.block, 0, st>>>(m, g, q, G, L.kch);
    k_sharpen<3><<<L.grid, L.block, 0, st>>>(m, g, sharp, amax, dtv, F, q, Gc, qtmp, L.kch);
  } else {
    k_grad0<2><<<L.grid, L.block, 0, st>>>(m, g, q, G, L.kch);
    k_sharpen<2><<<L.grid, L.block, 0, st>>>(m, g, sharp, amax, dtv, F, q, Gc, qtmp, L.kch);
  }
  cudaMemcpyAsync(q, qtmp, sizeof(double) * m.nc, cudaMemcpyDeviceToDevice, st);
  count_launches(2);
  return cudaGetLastError();
}

}  // namespace hg
