// loop.cuh -- per-cell loop and stencil helpers shared by the kernel files.
#pragma once

#include "common.cuh"

namespace hg {

// Upper bound of blocks of any reduction launch; partial-sum buffers hold
// kMaxBlocks entries per reduced value.
constexpr int kMaxBlocks = 1 << 17;

__device__ __forceinline__ double avg(double a, double b) { return a * 0.5 + b * 0.5; }
__device__ __forceinline__ float avg(float a, float b) { return a * 0.5f + b * 0.5f; }

struct Cell {
  int i[3];
  long long c;
};

// Thread (x, y) of block (bx, by, bz) visits cells (i, j, k) with
// i = bx*BX + x, j = by*BY + y and k in [bz*kch, bz*kch + kch).
#define CELL_LOOP_BEGIN(m, kch)                           \
  {                                                       \
    Cell X;                                               \
    X.i[0] = blockIdx.x * BX + threadIdx.x;               \
    X.i[1] = blockIdx.y * BY + threadIdx.y;               \
    const bool act_ = X.i[0] < m.n[0] && X.i[1] < m.n[1]; \
    const int nz_ = m.dim == 3 ? m.n[2] : 1;              \
    const int k0_ = blockIdx.z * (kch);                   \
    const int k1_ = min(k0_ + (kch), nz_);                \
    for (int kk_ = k0_; kk_ < k1_; ++kk_) {               \
      X.i[2] = kk_;                                       \
      if (!act_) continue;                                \
      X.c = cell_id(m, X.i[0], X.i[1], kk_);
#define CELL_LOOP_END \
  }                   \
  }

// Cell gradient (component along the axis of stride s) of a scalar whose
// boundary faces are extrapolated (ConditionFaceExtrapolation,
// solver.hpp:446-464): Green-Gauss over the two faces, face values the
// mean of the adjacent cells, on a boundary face p_b = 2 p_c - p_f(opposite
// face) (what the reference's extrapolation reduces to on a uniform block).
// The cell value cancels, leaving one difference and one product:
// interior (p+ - p-)/(2h), low end (p+ - p_c)/h, high end (p_c - p-)/h.
// Needs nd >= 2.
template <class T>
__device__ __forceinline__ T grad_extrap(const T* p, long long c, int id, int nd, long long s,
                                         T inv_h) {
  if (id > 0 && id < nd - 1) return (p[c + s] - p[c - s]) * (T(0.5) * inv_h);
  if (id == 0) return (p[c + s] - p[c]) * inv_h;
  return (p[c] - p[c - s]) * inv_h;
}
// The same along direction d of mesh m in the general form: central
// across a periodic end; beside an excluded cell the face is a boundary
// face; a cell between two boundary faces along d gets what the
// reference's in-order extrapolation leaves there (the low face first,
// reading 0 for the not yet extrapolated high face: p_lo = 2 p_c, then
// p_hi = 2 p_c - p_lo = 0, gradient -2 p_c / h); an excluded cell 0.
template <bool P, class T>
__device__ __forceinline__ T grad_extrap_m(const Mesh& m, const T* p, long long c, int d,
                                           int id, long long s, T inv_h) {
  if (!P) return grad_extrap(p, c, id, m.n[d], s, inv_h);
  if (m.ex && m.ex[c]) return T(0);
  const bool lo = has_lo_p<P>(m, d, id, c, s), hi = has_hi_p<P>(m, d, id, c, s);
  if (lo && hi)
    return (p[nb_hi_p<P>(m, d, id, c, s)] - p[nb_lo_p<P>(m, d, id, c, s)]) * (T(0.5) * inv_h);
  if (hi) return (p[nb_hi_p<P>(m, d, id, c, s)] - p[c]) * inv_h;
  if (lo) return (p[c] - p[nb_lo_p<P>(m, d, id, c, s)]) * inv_h;
  return T(-2) * p[c] * inv_h;
}

// Shorthands inside CELL_LOOP bodies: neighbours of the cell X along d.
// kPerT is the periodic switch of the enclosing kernel: a kernel
// instantiated per periodicity declares `constexpr bool kPerT = PER;`,
// others see this default (wrap test always compiled in).
constexpr bool kPerT = true;
#define HAS_LO(d) (kPerT ? has_lo(m, (d), X.i[d], X.c, cell_stride(m, (d))) : X.i[d] > 0)
#define HAS_HI(d) (kPerT ? has_hi(m, (d), X.i[d], X.c, cell_stride(m, (d))) : X.i[d] < m.n[d] - 1)
#define EXCLUDED() (kPerT && m.ex && m.ex[X.c])
#define NB_LO(d, s) (kPerT ? nb_lo(m, (d), X.i[d], X.c, (s)) : X.c - (s))
#define NB_HI(d, s) (kPerT ? nb_hi(m, (d), X.i[d], X.c, (s)) : X.c + (s))

// Launch KERNEL<dim[, T], periodic> on the cell grid L for the mesh's
// dimension and periodicity (kernels with a trailing `bool PER` parameter).
#define CELL_LAUNCH_P(m, L, st, KERNEL, ...)                                         \
  do {                                                                               \
    const bool p_ = any_periodic(m);                                                 \
    if ((m).dim == 3) {                                                              \
      if (p_) KERNEL<3, true><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch); \
      else KERNEL<3, false><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch);   \
    } else {                                                                         \
      if (p_) KERNEL<2, true><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch); \
      else KERNEL<2, false><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch);   \
    }                                                                                \
  } while (0)
// The instantiation CELL_LAUNCH_P launches, as a pointer for occupancy
// queries.
#define CELL_KERNEL_P(m, KERNEL)                                                       \
  ((m).dim == 3 ? (any_periodic(m) ? (const void*)KERNEL<3, true>                      \
                                   : (const void*)KERNEL<3, false>)                    \
                : (any_periodic(m) ? (const void*)KERNEL<2, true>                      \
                                   : (const void*)KERNEL<2, false>))
#define CELL_KERNEL_TP(m, KERNEL, T)                                                   \
  ((m).dim == 3 ? (any_periodic(m) ? (const void*)KERNEL<3, T, true>                   \
                                   : (const void*)KERNEL<3, T, false>)                 \
                : (any_periodic(m) ? (const void*)KERNEL<2, T, true>                   \
                                   : (const void*)KERNEL<2, T, false>))
#define CELL_LAUNCH_TP(m, L, st, KERNEL, T, ...)                                        \
  do {                                                                                  \
    const bool p_ = any_periodic(m);                                                    \
    if ((m).dim == 3) {                                                                 \
      if (p_) KERNEL<3, T, true><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch); \
      else KERNEL<3, T, false><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch);   \
    } else {                                                                            \
      if (p_) KERNEL<2, T, true><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch); \
      else KERNEL<2, T, false><<<(L).grid, (L).block, 0, st>>>(__VA_ARGS__, (L).kch);   \
    }                                                                                   \
  } while (0)

template <class T>
struct GeoT {
  T inv_h[3], h[3], A[3], V, invV;
  T inv_h2[3];
};
using Geo = GeoT<double>;

// Geometry of a uniform block; the factors are formed in FP64 and rounded
// once to the kernel's arithmetic type.
template <class T = double>
inline GeoT<T> make_geo(const Mesh& m) {
  GeoT<T> g;
  for (int d = 0; d < 3; ++d) {
    g.h[d] = (T)m.h[d];
    g.inv_h[d] = (T)(1. / m.h[d]);
    g.inv_h2[d] = (T)(1. / (m.h[d] * m.h[d]));
    g.A[d] = (T)m.A[d];
  }
  g.V = (T)m.V;
  g.invV = (T)(1. / m.V);
  return g;
}

}  // namespace hg
