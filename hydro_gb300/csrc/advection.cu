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

// Superbee value on the inner face between P (low side) and E (high side):
// flow from P (Ff > 1e-8) with fP the value of P's other (low) face, flow
// from E (Ff < -1e-8) with fE the value of E's other (high) face, as the
// Green-Gauss cell gradients of P and E use them; the mean otherwise.  Only
// the upwind cell's other face is read.
__device__ __forceinline__ double superbee_from_p(double qP, double qE, double fP, double h,
                                                  double inv_h) {
  double gP = (avg(qP, qE) - fP) * inv_h;
  double dq = qE - qP;
  return qP + 0.5 * superbee(dq, -4. * (gP * (-0.5 * h)) - dq);
}
__device__ __forceinline__ double superbee_from_e(double qP, double qE, double fE, double h,
                                                  double inv_h) {
  double gE = (fE - avg(qP, qE)) * inv_h;
  double dq = qE - qP;
  return qE - 0.5 * superbee(dq, 4. * (gE * (0.5 * h)) - dq);
}

// inlet_mask: bit q set when side q (xm, xp, ym, ...) is an inlet; qin
// holds the inlet values on those boundary faces.  Boundary faces carry
// the advection condition (the inlet value, else zero derivative: the
// cell's own value); across a periodic end the faces are inner.
template <int DIM, bool PER>
__global__ void k_adv_faces(Mesh m, Geo g, int nph, int stage, int nstages, const double* F,
                            CP<HYDRO_MAXPH> q, int inlet_mask, CP<HYDRO_MAXPH> qin,
                            WP<HYDRO_MAXPH> qflux, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (nstages > 1 && d != stage) continue;
    long long s = cell_stride(m, d);
    int id = X.i[d], nd = m.n[d];
    long long f = face_id(m, d, X.i[0], X.i[1], X.i[2]);
    long long fs = face_stride(m, d);
    const bool in_lo = (inlet_mask >> (2 * d)) & 1, in_hi = (inlet_mask >> (2 * d + 1)) & 1;
    // the low-side face value of cell c (index ic along d) and the
    // high-side face value, for the cell gradients
    // (a boundary face inside the block is a rigid-box wall: zero derivative)
    auto lo_face = [&](const double* qa, const double* qi, long long c, int ic, long long fc) {
      if (has_lo_p<PER>(m, d, ic, c, s)) return avg(qa[nb_lo_p<PER>(m, d, ic, c, s)], qa[c]);
      return (in_lo && ic == 0) ? qi[fc] : qa[c];
    };
    auto hi_face = [&](const double* qa, const double* qi, long long c, int ic, long long fc) {
      if (has_hi_p<PER>(m, d, ic, c, s)) return avg(qa[c], qa[nb_hi_p<PER>(m, d, ic, c, s)]);
      return (in_hi && ic == nd - 1) ? qi[fc] : qa[c];
    };
    // inner face between P (index ip) and E (index ie) with face index ff
    auto inner = [&](const double* qa, const double* qi, long long P, int ip, long long E, int ie,
                     long long ff, double Ff) {
      // P's low face is ff - fs unless P wraps (then the periodic end face);
      // E's high face is ff + fs likewise
      const double qP = qa[P], qE = qa[E];
      if (Ff > 1e-8) return superbee_from_p(qP, qE, lo_face(qa, qi, P, ip, ff - fs), g.h[d],
                                            g.inv_h[d]);
      if (Ff < -1e-8) return superbee_from_e(qP, qE, hi_face(qa, qi, E, ie, ff + fs), g.h[d],
                                             g.inv_h[d]);
      return 0.5 * (qP + qE);
    };
    double Ff = F[f];
    for (int i = 0; i < nph; ++i) {
      double qf;
      if (HAS_LO(d)) {
        const int ip = id > 0 ? id - 1 : nd - 1;
        qf = inner(q.a[i], qin.a[i], NB_LO(d, s), ip, X.c, id, f, Ff);
      } else {
        qf = (in_lo && id == 0) ? qin.a[i][f] : q.a[i][X.c];
      }
      qflux.a[i][f] = qf * Ff;
    }
    if (id == nd - 1) {
      long long fh = f + fs;
      double Fh = F[fh];
      for (int i = 0; i < nph; ++i) {
        double qf;
        if (PER && HAS_HI(d)) qf = inner(q.a[i], qin.a[i], X.c, id, NB_HI(d, s), 0, fh, Fh);
        else qf = in_hi ? qin.a[i][fh] : q.a[i][X.c];
        qflux.a[i][fh] = qf * Fh;
      }
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
template <int DIM, bool PER>
__global__ void k_sharpen(Mesh m, Geo g, double sharp, double amax, double dtv, const double* F,
                          const double* q, C3 G, double* qout, int kch) {
  constexpr bool kPerT = PER;
  CELL_LOOP_BEGIN(m, kch)
  double sh = 0.;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long s = cell_stride(m, d);
    long long fl = face_id(m, d, X.i[0], X.i[1], X.i[2]);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      bool inner = side ? HAS_HI(d) : HAS_LO(d);
      long long nb = inner ? (side ? NB_HI(d, s) : NB_LO(d, s)) : X.c;
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

template <int DIM, bool PER>
__global__ void k_grad0(Mesh m, Geo g, const double* a, W3 G, int kch) {
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

}  // namespace

cudaError_t launch_adv_faces(const Mesh& m, int nph, int stage, int nstages, const double* F,
                             CP<HYDRO_MAXPH> q, int inlet_mask, CP<HYDRO_MAXPH> qin,
                             WP<HYDRO_MAXPH> qflux, cudaStream_t st) {
  Launch L = cell_launch(m);
  Geo g = make_geo(m);
  CELL_LAUNCH_P(m, L, st, k_adv_faces, m, g, nph, stage, nstages, F, q, inlet_mask, qin, qflux);
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
  CELL_LAUNCH_P(m, L, st, k_grad0, m, g, q, G);
  CELL_LAUNCH_P(m, L, st, k_sharpen, m, g, sharp, amax, dtv, F, q, Gc, qtmp);
  cudaMemcpyAsync(q, qtmp, sizeof(double) * m.nc, cudaMemcpyDeviceToDevice, st);
  count_launches(2);
  return cudaGetLastError();
}

}  // namespace hg
