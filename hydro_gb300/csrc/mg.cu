// mg.cu -- geometric multigrid preconditioner for the pressure-correction
// solve of the mixed-precision path (FP32, sm_103a).
//
// The reference solves the pressure rows with Gauss-Seidel sweeps
// (linear.hpp:685-715) and has no multigrid on its main path (a dormant
// two-level experiment sits in source/test_module/test_module.hpp:311-379).
// On a uniform block the pressure operator is a 7-point (5-point) stencil of
// face couplings kf; the hierarchy here coarsens it 2:1 per direction:
//   coarse coupling  = 1/2 * sum of the 4 (2) fine couplings of the face
//                      (area x2^(dim-1), distance x2),
//   restriction      = sum of the residuals of the 2^dim children,
//   prolongation     = piecewise-constant injection,
//   smoother         = red-black Gauss-Seidel, (red, black) before and
//                      (black, red) after the coarse correction, so the
//                      V-cycle is symmetric and usable inside CG,
//   small levels     = every level of <= kMgBlockMax cells runs inside one
//                      CTA in shared memory (a complete sub-V-cycle, its
//                      coarsest level solved by symmetric red-black sweeps
//                      on the zero-mean right-hand side).
// All kernels return at once when the CG's done flag is set, so iterations
// can be queued in chunks like the other solvers.
#include <cuda_fp16.h>
#include <math.h>

#include "kernels.h"
#include "loop.cuh"

namespace hg {

namespace {

// Red-black GS half-sweep on the cells with (i+j+k) % 2 == color.  Thread
// (x, y) handles the color-matching cell of the pair (2x, 2x+1) in row
// (j, k).  With `zero` set the cell's neighbours are taken as 0 (first
// half-sweep from x = 0).  With `cx` set the neighbours are read as
// x + cx(parent): the prolongation of the coarse correction fused into the
// first post-smoothing half-sweep (the cells of the other color are
// overwritten by the next half-sweep, which never reads their old value).
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT, PER ? 6 : 8) k_mg_smooth(Mesh m, const float* kf, const float* idg, const float* b, float* x,
                            int color, int zero, long long pin, const float* cx, int cnx,
                            int cny, const DevScalars* ds, int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  const int nz = DIM == 3 ? m.n[2] : 1;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, nz);
  if (j >= m.n[1]) return;
  for (int k = k0; k < k1; ++k) {
    int i = 2 * ih + ((j + k + color) & 1);
    if (i >= m.n[0]) continue;
    long long c = cell_id(m, i, j, k);
    if (c == pin) {
      x[c] = b[c];
      continue;
    }
    float acc = b[c];
    if (!zero) {
      int id[3] = {i, j, k};
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        long long s = cell_stride(m, d);
        long long fl = face_id(m, d, i, j, k);
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          bool in = side ? has_hi_p<PER>(m, d, id[d], c, s) : has_lo_p<PER>(m, d, id[d], c, s);
          long long nb = side ? nb_hi_p<PER>(m, d, id[d], c, s) : nb_lo_p<PER>(m, d, id[d], c, s);
          if (!in || nb == pin) continue;
          float xv = x[nb];
          if (cx) {
            int q[3] = {i, j, k};
            q[d] += side ? 1 : -1;
            if (PER) {
              if (q[d] < 0) q[d] = m.n[d] - 1;
              if (q[d] >= m.n[d]) q[d] = 0;
            }
            xv += cx[(q[0] >> 1) + (long long)cnx * ((q[1] >> 1) + (long long)cny * (q[2] >> 1))];
          }
          acc = fmaf(kf[side ? fl + face_stride(m, d) : fl], xv, acc);
        }
      }
    }
    x[c] = acc * idg[c];
  }
}

// Dense inverse of the operator of a small coarsest level (n <= 64 cells),
// Dense inverse of a small level (n <= kMgDense cells) by one CTA, FP32 in
// shared memory (S: kDenseScratch floats).  A = couplings (diagonal = their
// sum); cells without couplings (inside a rigid box) decoupled as identity
// rows; the constant mode of the others completed by (d/m) e e^T, d their
// mean diagonal and m their count: A + (d/m) e e^T is SPD with the constant
// mode at eigenvalue d, inside A's own range (FP32 keeps the condition
// number of the Laplacian), and for a zero-mean right-hand side its
// solution is the zero-mean solution of A x = b.  Gauss-Jordan without
// pivoting (SPD), one barrier per pivot: the thread owning slot 64 i + j
// updates element (i, j), and the next pivot row and column are published
// through double buffers as they are written.  The result is symmetrised.
// Element ownership does not depend on the thread count, nor does the
// result.
constexpr int kMgDense = (int)kMgCoarseTarget;
static_assert(kMgDense == 64, "slot layout: 64 columns");
constexpr int kDenseScratch = kMgDense * kMgDense + 5 * kMgDense + 4;
__device__ __forceinline__ float dense_pivot_inv(float piv) {
  return fabsf(piv) > 1e-30f ? 1.f / piv : 0.f;
}
// Element (i, j) after pivot step k (ip = 1 / pivot, cik and rkj: column k
// and row k before the step).
__device__ __forceinline__ float dense_update(float a, int i, int j, int k, float ip, float cik,
                                              float rkj) {
  if (i == k) return j == k ? ip : a * ip;
  if (j == k) return -a * ip;
  return fmaf(-cik * ip, rkj, a);
}

// The pivot steps of dense_inverse with the elements in registers: the
// first 4096 / E threads take part, thread t owning slots t + s (4096 / E)
// (one column j = t & 63, rows spaced 64 / E apart); A (slot layout) holds
// the matrix before and after, rowb / colb publish row and column 0.
template <int E>
__device__ void dense_pivots_regs(float* A, float* rowb, float* colb, int n) {
  constexpr int K = kMgDense, NT = K * K / E, RS = NT / K;
  const int tid = threadIdx.x;
  const bool in = tid < NT;
  const int j = tid & (K - 1), i0 = tid >> 6;
  float a[E];
#pragma unroll
  for (int t = 0; t < E; ++t) {
    const int i = i0 + t * RS;
    a[t] = in && i < n && j < n ? A[i * K + j] : 0.f;
  }
  for (int k = 0; k < n; ++k) {
    const float* rk = rowb + (k & 1) * K;
    const float* ck = colb + (k & 1) * K;
    float* rn = rowb + ((k + 1) & 1) * K;
    float* cn = colb + ((k + 1) & 1) * K;
    if (in && j < n) {
      const float ip = dense_pivot_inv(rk[k]);
      const float rkj = rk[j];
#pragma unroll
      for (int t = 0; t < E; ++t) {
        const int i = i0 + t * RS;
        if (i >= n) continue;
        const float v = dense_update(a[t], i, j, k, ip, ck[i], rkj);
        a[t] = v;
        if (i == k + 1) rn[j] = v;
        if (j == k + 1) cn[i] = v;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int t = 0; t < E; ++t) {
    const int i = i0 + t * RS;
    if (in && i < n && j < n) A[i * K + j] = a[t];
  }
  __syncthreads();
}

template <int DIM>
__device__ void dense_inverse(const Mesh& m, const float* kf, float* P, float* S) {
  constexpr int K = kMgDense;
  float* A = S;                                       // [K][K]
  float* rowb = A + K * K;                            // [2][K]
  float* colb = rowb + 2 * K;                         // [2][K]
  int* iso = reinterpret_cast<int*>(colb + 2 * K);    // [K]
  float* alpha = reinterpret_cast<float*>(iso + K);   // [1]
  const int n = (int)m.nc, tid = threadIdx.x, nt = blockDim.x;
  const int slots = n * K;  // rows 0..n-1 of the slot grid
  for (int q = tid; q < slots; q += nt) A[q] = 0.f;
  __syncthreads();
  for (int c = tid; c < n; c += nt) {
    int id[3];
    id[0] = c % m.n[0];
    id[1] = (c / m.n[0]) % m.n[1];
    id[2] = DIM == 3 ? c / (m.n[0] * m.n[1]) : 0;
    float dg = 0.f;
    for (int d = 0; d < DIM; ++d) {
      const long long s = cell_stride(m, d);
      const long long fl = face_id(m, d, id[0], id[1], id[2]);
      if (has_lo(m, d, id[d], c, s)) {
        const float k = kf[fl];
        dg += k;
        A[c * K + (int)nb_lo(m, d, id[d], c, s)] -= k;
      }
      if (has_hi(m, d, id[d], c, s)) {
        const float k = kf[fl + face_stride(m, d)];
        dg += k;
        A[c * K + (int)nb_hi(m, d, id[d], c, s)] -= k;
      }
    }
    A[c * K + c] += dg;
    iso[c] = dg > 0.f ? 0 : 1;
  }
  __syncthreads();
  if (tid < 32) {
    float sd = 0.f;
    int cnt = 0;
    for (int c = tid; c < n; c += 32)
      if (!iso[c]) {
        sd += A[c * K + c];
        ++cnt;
      }
    sd = warp_sum(sd);
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (tid == 0) alpha[0] = cnt > 0 ? sd / (float)cnt / (float)cnt : 0.f;
  }
  __syncthreads();
  const float al = alpha[0];
  for (int q = tid; q < slots; q += nt) {
    const int i = q >> 6, j = q & (K - 1);
    if (j >= n) continue;
    float a;
    if (iso[i] || iso[j]) a = i == j ? 1.f : 0.f;
    else a = A[q] + al;
    A[q] = a;
    if (i == 0) rowb[j] = a;
    if (j == 0) colb[i] = a;
  }
  __syncthreads();
  if (nt >= 512) {
    dense_pivots_regs<8>(A, rowb, colb, n);
  } else if (nt >= 256) {
    dense_pivots_regs<16>(A, rowb, colb, n);
  } else {
    for (int k = 0; k < n; ++k) {
      const float* rk = rowb + (k & 1) * K;
      const float* ck = colb + (k & 1) * K;
      float* rn = rowb + ((k + 1) & 1) * K;
      float* cn = colb + ((k + 1) & 1) * K;
      const float ip = dense_pivot_inv(rk[k]);
      for (int q = tid; q < slots; q += nt) {
        const int i = q >> 6, j = q & (K - 1);
        if (j >= n) continue;
        const float a = dense_update(A[q], i, j, k, ip, ck[i], rk[j]);
        A[q] = a;
        if (i == k + 1) rn[j] = a;
        if (j == k + 1) cn[i] = a;
      }
      __syncthreads();
    }
  }
  for (int q = tid; q < n * n; q += nt) {
    const int i = q / n, j = q % n;
    P[q] = 0.5f * (A[i * K + j] + A[j * K + i]);
  }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_mg_coarse_inv(Mesh m, const float* kf, float* P) {
  __shared__ float S[kDenseScratch];
  dense_inverse<DIM>(m, kf, P, S);
}

// Coarse couplings of coarse cell c at I: 1/2 of the sum of the fine
// couplings of each coarse face (zero on boundary faces; across a periodic
// end the coarse face joins the last and first coarse cells like the fine
// one).
template <int DIM>
__device__ __forceinline__ void coarsen_cell(const Mesh& fm, const Mesh& cm, const float* fkf,
                                             float* ckf, const int* I, long long c) {
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long cf = face_id(cm, d, I[0], I[1], I[2]);
    int e1 = (d + 1) % DIM, e2 = (d + 2) % DIM;
    // fine faces of the coarse face at coarse index J along d: index 2J
    // along d, 2J' and 2J'+1 across
    auto fsum = [&](int J) {
      float sum = 0.f;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
#pragma unroll
        for (int bq = 0; bq < (DIM == 3 ? 2 : 1); ++bq) {
          int fi[3] = {2 * I[0], 2 * I[1], 2 * I[2]};
          fi[d] = 2 * J;
          fi[e1] += a;
          if (DIM == 3) fi[e2] += bq;
          sum += fkf[face_id(fm, d, fi[0], fi[1], DIM == 3 ? fi[2] : 0)];
        }
      }
      return sum;
    };
    ckf[cf] = has_lo(cm, d, I[d], c, cell_stride(cm, d)) ? 0.5f * fsum(I[d]) : 0.f;
    if (I[d] == cm.n[d] - 1)
      ckf[cf + face_stride(cm, d)] = cm.per[d] ? 0.5f * fsum(I[d] + 1) : 0.f;
  }
}

template <int DIM>
__global__ void k_mg_coarsen(Mesh fm, Mesh cm, const float* fkf, float* ckf, int kch) {
  pdl_wait();
  pdl_trigger();
  CELL_LOOP_BEGIN(cm, kch)
  coarsen_cell<DIM>(fm, cm, fkf, ckf, X.i, X.c);
  CELL_LOOP_END
}

// Diagonal of a coarse level's cell at I: the sum of its face couplings.
template <int DIM>
__device__ __forceinline__ float diag_cell(const Mesh& m, const float* kf, const int* I) {
  float s = 0.f;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    long long fl = face_id(m, d, I[0], I[1], I[2]);
    s += kf[fl] + kf[fl + face_stride(m, d)];
  }
  return s;
}

template <int DIM>
__global__ void k_mg_diag(Mesh m, const float* kf, float* dg, float* idg, int kch) {
  pdl_wait();
  pdl_trigger();
  CELL_LOOP_BEGIN(m, kch)
  const float s = diag_cell<DIM>(m, kf, X.i);
  dg[X.c] = s;
  idg[X.c] = s > 0.f ? 1.f / s : 0.f;
  CELL_LOOP_END
}

// Coarse right-hand side = sum over the 2^DIM children of the fine residual
// b - A x; also clears the coarse correction.  The pre-smoothing ends with
// a black half-sweep, which leaves the residual of every black cell zero
// (up to rounding), so only the red children are summed: a coarse cell's
// children (2I + ci, 2J + cj, 2K + ck) are red when ci + cj + ck is even.
// With cidg the coarse level's first half-sweep (red, from x = 0: x = b /
// diag) is done here as well; without it the coarse iterate is cleared.
template <int DIM, bool PER>
__global__ void __launch_bounds__(NT, 4) k_mg_restrict(Mesh fm, Mesh cm, const float* kf, const float* dg, const float* b,
                              const float* x, float* cb, float* cx, const float* cidg,
                              long long pin, const DevScalars* ds, int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  CELL_LOOP_BEGIN(cm, kch)
  float sum = 0.f;
#pragma unroll
  for (int ck = 0; ck < (DIM == 3 ? 2 : 1); ++ck)
#pragma unroll
    for (int cj = 0; cj < 2; ++cj)
#pragma unroll
      for (int ci = 0; ci < 2; ++ci) {
        if ((ci + cj + ck) & 1) continue;
        int id[3] = {2 * X.i[0] + ci, 2 * X.i[1] + cj, DIM == 3 ? 2 * X.i[2] + ck : 0};
        long long c = cell_id(fm, id[0], id[1], id[2]);
        float r;
        if (c == pin) {
          r = b[c] - x[c];
        } else {
          float ax = dg[c] * x[c];
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            long long s = cell_stride(fm, d);
            long long fl = face_id(fm, d, id[0], id[1], id[2]);
            const long long cl = nb_lo_p<PER>(fm, d, id[d], c, s);
            const long long ch = nb_hi_p<PER>(fm, d, id[d], c, s);
            if (has_lo_p<PER>(fm, d, id[d], c, s) && cl != pin) ax = fmaf(-kf[fl], x[cl], ax);
            if (has_hi_p<PER>(fm, d, id[d], c, s) && ch != pin)
              ax = fmaf(-kf[fl + face_stride(fm, d)], x[ch], ax);
          }
          r = b[c] - ax;
        }
        sum += r;
      }
  cb[X.c] = sum;
  cx[X.c] = cidg && ((X.i[0] + X.i[1] + X.i[2]) & 1) == 0 ? sum * cidg[X.c] : 0.f;
  CELL_LOOP_END
}

// ------------------------------------------------ levels inside one CTA --
// The levels of at most kMgBlockMax cells form a complete sub-V-cycle run
// by one CTA in shared memory: every level's couplings, inverse diagonal,
// right-hand side and iterate live in shared memory, and the smoothing,
// restriction and prolongation steps are separated by __syncthreads instead
// of kernel launches.  Same smoother and transfers as the grid levels; the
// coarsest level is solved by symmetric red-black sweeps, (red, black)^s
// then (black, red)^s, on its zero-mean right-hand side.
constexpr int kBlkThreads = 1024;

struct MgBlock {
  int nl;  // levels in the CTA, top first
  int nsweep, coarse_sweeps;
  const float* cinv;  // dense inverse of the coarsest level, or null (sweeps)
  int oc;             // its place in shared memory
  long long pin;  // pinned cell of the top level (-1: none)
  Mesh m[kMgMaxLevels];
  const float* kf[kMgMaxLevels];
  const float* idg[kMgMaxLevels];
  int ox[kMgMaxLevels], ob[kMgMaxLevels], oi[kMgMaxLevels], ok[kMgMaxLevels];
};


template <int DIM>
__device__ __forceinline__ void blk_ijk(const Mesh& m, int c, int* id) {
  id[0] = c % m.n[0];
  int r = c / m.n[0];
  id[1] = DIM == 3 ? r % m.n[1] : r;
  id[2] = DIM == 3 ? r / m.n[1] : 0;
}

// q / d (returned) and q % d (r) for 0 <= q < 2^24 and d >= 1, from rd =
// 1 / d in FP32: q rd is within 1 of q / d there, so one integer correction
// makes the quotient exact (a handful of instructions against a signed
// division's few dozen, per cell of every pass).
__device__ __forceinline__ int fdivmod(int q, int d, float rd, int& r) {
  int t = __float2int_rz((float)q * rd);
  int rem = q - t * d;
  if (rem < 0) {
    --t;
    rem += d;
  } else if (rem >= d) {
    ++t;
    rem -= d;
  }
  r = rem;
  return t;
}

// (i, j, k) of cell c of an n0 x n1 [x n2] level (r0 = 1 / n0, r1 = 1 / n1).
template <int DIM>
__device__ __forceinline__ void blk_ijk(int n0, int n1, float r0, float r1, int c, int* id) {
  const int row = fdivmod(c, n0, r0, id[0]);
  if (DIM == 3) {
    id[2] = fdivmod(row, n1, r1, id[1]);
  } else {
    id[1] = row;
    id[2] = 0;
  }
}

// Index constants of a level held in registers for a pass (the level's
// Mesh may sit in shared memory beside the arrays the pass writes, and
// would be re-read after every store otherwise): 32-bit, a level of a
// one-group solve has fewer than 2^31 faces.
template <int DIM>
struct LvIx {
  // cells, and the offsets of the y and z face blocks; the face layout is
  // fixed by the cell counts (fnx = nx + (d == 0), fny = ny + (d == 1))
  int n[3], fo1, fo2;
  __device__ __forceinline__ explicit LvIx(const Mesh& m) {
    n[0] = m.n[0];
    n[1] = m.n[1];
    n[2] = DIM == 3 ? m.n[2] : 1;
    fo1 = (int)m.fofs[1];
    fo2 = DIM == 3 ? (int)m.fofs[2] : 0;
  }
  // stride between neighbouring cells along d
  __device__ __forceinline__ int cs(int d) const {
    return d == 0 ? 1 : (d == 1 ? n[0] : n[0] * n[1]);
  }
  // stride between a cell's low and high face along d (fnx[1] = nx,
  // fnx[2] fny[2] = nx ny: the cell stride)
  __device__ __forceinline__ int fs(int d) const { return cs(d); }
  __device__ __forceinline__ int face(int d, const int* id) const {
    const int fx = n[0] + (d == 0), fy = n[1] + (d == 1);
    return (d == 0 ? 0 : d == 1 ? fo1 : fo2) + id[0] + fx * (id[1] + fy * id[2]);
  }
};

// One red-black half-sweep by the group: slot t of row (j, k) is the cell
// i = 2t + ((j + k + color) & 1); the cells of one colour are independent,
// so the order does not change the result.
template <int DIM, bool PER, class G = CtaG>
__device__ void blk_half(const Mesh& m, const float* kf, const float* idg, const float* b,
                         float* x, int color, bool zero, long long pin, const G& g = G()) {
  // U cells per thread per pass, all loads before the stores (they read
  // the other colour only), so that one thread keeps U cells' loads in
  // flight: a CTA alone on a level of tens of thousands of cells is
  // latency-bound otherwise
  constexpr int U = DIM == 3 ? 2 : 4;
  const LvIx<DIM> L(m);
  const int hx = (L.n[0] + 1) >> 1;
  const int n = hx * L.n[1] * L.n[2];
  // a thread without a cell (most of them on a small level) skips the
  // pass, leaving the issue slots to those that have one; every thread
  // meets the one barrier at the end
  if (g.rank() < n) {
    const int pn = (int)pin;
    const int step = g.size();
    const float rhx = 1.f / (float)hx, rn1 = 1.f / (float)L.n[1];
    for (int q0 = g.rank(); q0 < n; q0 += U * step) {
      float val[U];
      int cc[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u * step;
        cc[u] = -1;
        val[u] = 0.f;
        if (q >= n) continue;
        int id[3], t;
        const int row = fdivmod(q, hx, rhx, t);
        if (DIM == 3) {
          id[2] = fdivmod(row, L.n[1], rn1, id[1]);
        } else {
          id[1] = row;
          id[2] = 0;
        }
        id[0] = 2 * t + ((id[1] + id[2] + color) & 1);
        if (id[0] >= L.n[0]) continue;
        const int c = id[0] + L.n[0] * row;
        cc[u] = c;
        if (c == pn) {
          val[u] = b[c];
          continue;
        }
        float acc = b[c];
        if (!zero) {
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            const int s = L.cs(d);
            const int fl = L.face(d, id);
            if (PER) {
              const int cl = nb_lo_p<PER>(m, d, id[d], c, s);
              const int ch = nb_hi_p<PER>(m, d, id[d], c, s);
              if (has_lo_p<PER>(m, d, id[d], c, s) && cl != pn) acc = fmaf(kf[fl], x[cl], acc);
              if (has_hi_p<PER>(m, d, id[d], c, s) && ch != pn)
                acc = fmaf(kf[fl + L.fs(d)], x[ch], acc);
            } else {
              if (id[d] > 0 && c - s != pn) acc = fmaf(kf[fl], x[c - s], acc);
              if (id[d] < L.n[d] - 1 && c + s != pn) acc = fmaf(kf[fl + L.fs(d)], x[c + s], acc);
            }
          }
        }
        val[u] = acc * idg[c];
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (cc[u] >= 0) x[cc[u]] = val[u];
    }
  }
  g.sync();
}

// coarse rhs = sum over the children of the fine residual b - A x
template <int DIM, bool PER, class G = CtaG>
__device__ void blk_restrict(const Mesh& fm, const Mesh& cm, const float* kf, const float* b,
                             const float* x, float* cb, long long pin, const G& g = G()) {
  constexpr int U = DIM == 3 ? 2 : 4;  // coarse cells per thread per pass, loads first
  const int n = (int)cm.nc;
  if (g.rank() < n) {  // (threads without a coarse cell skip to the barrier)
    const LvIx<DIM> L(fm);
    const int cn0 = cm.n[0], cn1 = cm.n[1];
    const float rc0 = 1.f / (float)cn0, rc1 = 1.f / (float)cn1;
    const int pn = (int)pin;
    const int step = g.size();
    for (int C0 = g.rank(); C0 < n; C0 += U * step) {
      float sums[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int C = C0 + u * step;
        sums[u] = 0.f;
        if (C >= n) continue;
        int I[3];
        blk_ijk<DIM>(cn0, cn1, rc0, rc1, C, I);
        float sum = 0.f;
#pragma unroll
        for (int ck = 0; ck < (DIM == 3 ? 2 : 1); ++ck)
#pragma unroll
          for (int cj = 0; cj < 2; ++cj)
#pragma unroll
            for (int ci = 0; ci < 2; ++ci) {
              int id[3] = {2 * I[0] + ci, 2 * I[1] + cj, DIM == 3 ? 2 * I[2] + ck : 0};
              const int c = id[0] + L.n[0] * (id[1] + L.n[1] * id[2]);
              float r;
              if (c == pn) {
                r = b[c] - x[c];
              } else {
                float dg = 0.f, off = 0.f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                  const int s = L.cs(d);
                  const int fl = L.face(d, id);
                  float klo = kf[fl], khi = kf[fl + L.fs(d)];
                  dg += klo + khi;
                  if (PER) {
                    const int cl = nb_lo_p<PER>(fm, d, id[d], c, s);
                    const int ch = nb_hi_p<PER>(fm, d, id[d], c, s);
                    if (has_lo_p<PER>(fm, d, id[d], c, s) && cl != pn) off = fmaf(klo, x[cl], off);
                    if (has_hi_p<PER>(fm, d, id[d], c, s) && ch != pn) off = fmaf(khi, x[ch], off);
                  } else {
                    if (id[d] > 0 && c - s != pn) off = fmaf(klo, x[c - s], off);
                    if (id[d] < L.n[d] - 1 && c + s != pn) off = fmaf(khi, x[c + s], off);
                  }
                }
                r = b[c] - (dg * x[c] - off);
              }
              sum += r;
            }
        sums[u] = sum;
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (C0 + u * step < n) cb[C0 + u * step] = sums[u];
    }
  }
  g.sync();
}

// The levels of one V-cycle run by one CTA, by pointer (shared or global
// memory): b[0] is the right-hand side, x[0] receives M^-1 b.
struct CtaLevels {
  int nl;  // levels, finest first
  int nsweep, coarse_sweeps;
  const float* cinv;  // dense inverse of the coarsest level, or null (sweeps)
  long long pin;      // pinned cell of the finest level (-1: none)
  Mesh m[kMgMaxLevels];
  const float* kf[kMgMaxLevels];
  const float* idg[kMgMaxLevels];
  float* x[kMgMaxLevels];
  float* b[kMgMaxLevels];
};

// One V-cycle by the calling CTA (all its threads; red: 32 floats of shared
// scratch).  Ends with a __syncthreads.
template <int DIM, bool PER>
__device__ void cta_vcycle(const CtaLevels& B, float* red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int ns = B.nsweep;
  for (int l = 0; l + 1 < B.nl; ++l) {
    const Mesh& m = B.m[l];
    long long lp = l == 0 ? B.pin : -1;
    for (int s = 0; s < ns; ++s) {
      blk_half<DIM, PER>(m, B.kf[l], B.idg[l], B.b[l], B.x[l], 0, s == 0, lp);
      blk_half<DIM, PER>(m, B.kf[l], B.idg[l], B.b[l], B.x[l], 1, false, lp);
    }
    blk_restrict<DIM, PER>(m, B.m[l + 1], B.kf[l], B.b[l], B.x[l], B.b[l + 1], lp);
  }
  {
    const int l = B.nl - 1;
    const Mesh& m = B.m[l];
    long long lp = l == 0 ? B.pin : -1;
    const float* kf = B.kf[l];
    const float* idg = B.idg[l];
    float* b = B.b[l];
    float* x = B.x[l];
    const int n = (int)m.nc;
    if (lp < 0) {
      // singular Neumann block: project the right-hand side to zero mean
      float sv = 0.f;
      for (int c = tid; c < n; c += nt) sv += b[c];
      sv = warp_sum(sv);
      if ((tid & 31) == 0) red[tid >> 5] = sv;
      __syncthreads();
      if (tid < 32) {
        float v = tid < (nt + 31) / 32 ? red[tid] : 0.f;
        v = warp_sum(v);
        if (tid == 0) red[0] = v / (float)n;
      }
      __syncthreads();
      const float mean = red[0];
      for (int c = tid; c < n; c += nt) b[c] -= mean;
      __syncthreads();
    }
    if (B.cinv && lp < 0) {
      // exact coarsest solve: x = P b, P the symmetric inverse of the level's
      // operator completed by the constant mode (b has zero mean); one warp
      // per row of P (n <= 64)
      const float* P = B.cinv;
      const int lane = tid & 31;
      for (int c = tid >> 5; c < n; c += nt >> 5) {
        float acc = 0.f;
        for (int q = lane; q < n; q += 32) acc = fmaf(P[c * n + q], b[q], acc);
        acc = warp_sum(acc);
        if (lane == 0) x[c] = acc;
      }
      __syncthreads();
    } else {
      const int half = B.coarse_sweeps / 2 > 0 ? B.coarse_sweeps / 2 : 1;
      for (int s = 0; s < half; ++s) {
        blk_half<DIM, PER>(m, kf, idg, b, x, 0, s == 0, lp);
        blk_half<DIM, PER>(m, kf, idg, b, x, 1, false, lp);
      }
      for (int s = 0; s < half; ++s) {
        blk_half<DIM, PER>(m, kf, idg, b, x, 1, false, lp);
        blk_half<DIM, PER>(m, kf, idg, b, x, 0, false, lp);
      }
    }
  }
  for (int l = B.nl - 2; l >= 0; --l) {
    const Mesh& m = B.m[l];
    const Mesh& cm = B.m[l + 1];
    long long lp = l == 0 ? B.pin : -1;
    float* x = B.x[l];
    const float* cx = B.x[l + 1];
    const int nc = (int)m.nc, n0 = m.n[0], n1 = m.n[1], cn0 = cm.n[0], cn1 = cm.n[1];
    const float r0 = 1.f / (float)n0, r1 = 1.f / (float)n1;
    for (int c0 = tid; c0 < nc; c0 += 4 * nt) {
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = c0 + u * nt;
        v[u] = 0.f;
        if (c >= nc) continue;
        int id[3];
        blk_ijk<DIM>(n0, n1, r0, r1, c, id);
        v[u] = x[c] + cx[(id[0] >> 1) + cn0 * ((id[1] >> 1) + cn1 * (id[2] >> 1))];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (c0 + u * nt < nc) x[c0 + u * nt] = v[u];
    }
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
      blk_half<DIM, PER>(m, B.kf[l], B.idg[l], B.b[l], x, 1, false, lp);
      blk_half<DIM, PER>(m, B.kf[l], B.idg[l], B.b[l], x, 0, false, lp);
    }
  }
}

// The levels from `top` down, staged into shared memory (MgBlock offsets),
// as a CtaLevels set (built by thread 0; the caller synchronises).
// n floats from global to shared memory by the CTA, 4 loads per thread in
// flight
__device__ __forceinline__ void cta_copy(float* dst, const float* src, int n) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int q0 = tid; q0 < n; q0 += 4 * nt) {
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = q0 + u * nt < n ? src[q0 + u * nt] : 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (q0 + u * nt < n) dst[q0 + u * nt] = v[u];
  }
}

__device__ void cta_stage_levels(const MgBlock& B, float* sm, CtaLevels* V, int first = 0) {
  const int tid = threadIdx.x;
  for (int l = 0; l < B.nl; ++l) {
    cta_copy(sm + B.ok[l], B.kf[l], (int)B.m[l].nf);
    cta_copy(sm + B.oi[l], B.idg[l], (int)B.m[l].nc);
  }
  if (B.cinv) {
    const int n = (int)B.m[B.nl - 1].nc;
    cta_copy(sm + B.oc, B.cinv, n * n);
  }
  if (tid == 0) {
    V->nl = first + B.nl;
    V->nsweep = B.nsweep;
    V->coarse_sweeps = B.coarse_sweeps;
    V->cinv = B.cinv ? sm + B.oc : nullptr;
    V->pin = B.pin;
    for (int l = 0; l < B.nl; ++l) {
      V->m[first + l] = B.m[l];
      V->kf[first + l] = sm + B.ok[l];
      V->idg[first + l] = sm + B.oi[l];
      V->x[first + l] = sm + B.ox[l];
      V->b[first + l] = sm + B.ob[l];
    }
  }
}

template <int DIM, bool PER>
__global__ void __launch_bounds__(kBlkThreads)
    k_mg_block_vcycle(MgBlock B, const float* btop, float* xtop, const DevScalars* ds) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  extern __shared__ float sm[];
  __shared__ float red[32];
  __shared__ CtaLevels V;
  const int tid = threadIdx.x, nt = blockDim.x;
  cta_stage_levels(B, sm, &V);
  for (int q = tid; q < (int)B.m[0].nc; q += nt) sm[B.ob[0] + q] = btop[q];
  __syncthreads();
  cta_vcycle<DIM, PER>(V, red);
  for (int q = tid; q < (int)B.m[0].nc; q += nt) xtop[q] = sm[B.ox[0] + q];
}

struct DFAcc2 {
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

// The vector kernels of the inner solve step four cells per thread with
// 16-byte loads (every vector is 256-byte aligned, the launchers check);
// the last n % 4 cells are taken one by one by the first threads of the
// grid.

// Inner-solve start: r = FP32 copy of the FP64 refinement residual; ||r||^2
// sets the stop test.
__global__ void __launch_bounds__(NT) k_mgcg_init(long long n, const double* __restrict__ r64,
                                                  float* __restrict__ r, float* __restrict__ x,
                                                  double tol, int limit, int dev_params,
                                                  double* partials, DevScalars* ds) {
  pdl_wait();
  pdl_trigger();
  double s = 0.;
  const long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  const long long g = blockIdx.x * (long long)NT + tid, stride = (long long)gridDim.x * NT;
  const long long n4 = n >> 2;
  const double2* r2 = reinterpret_cast<const double2*>(r64);
#pragma unroll 2
  for (long long i = g; i < n4; i += stride) {
    const double2 a = r2[2 * i], b = r2[2 * i + 1];
    reinterpret_cast<float4*>(r)[i] = make_float4(d2f(a.x), d2f(a.y), d2f(b.x), d2f(b.y));
    reinterpret_cast<float4*>(x)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    s += a.x * a.x;
    s += a.y * a.y;
    s += b.x * b.x;
    s += b.y * b.y;
  }
  for (long long i = 4 * n4 + g; i < n; i += stride) {
    double v = r64[i];
    r[i] = d2f(v);
    x[i] = 0.f;
    s += v * v;
  }
  double v[1] = {s};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_F32_INIT], o)) {
    if (tid == 0) {
      if (dev_params) tol = ds->red[RS_INNER_TOL];
      else ds->flag[FL_PCG_LIMIT] = limit;
      ds->red[RS_PCG_FF] = o[0];
      ds->red[RS_PCG_RR] = o[0];
      ds->red[RS_PCG_TOL2] = tol * tol * o[0];
      ds->red[RS_PCG_RRREF] = o[0];
      ds->flag[FL_PCG_ITERS] = 0;
      ds->flag[FL_PCG_REFIT] = 0;
      ds->flag[FL_PCG_DONE] = (o[0] == 0. || ds->flag[FL_PCG_LIMIT] <= 0) ? 1 : 0;
    }
  }
}

// Iterations without a halving of ||r|| after which the inner solve stops
// and hands the FP64 refinement a fresh residual: a multigrid-preconditioned
// CG halves ||r|| every iteration or two, and in FP32 on a singular
// (all-Neumann) system the recursive residual picks up a constant component
// from rounding that the operator cannot remove, so the recursion can
// stall above the requested inner tolerance.  The restart from the
// projected FP64 residual removes it.
constexpr int kStallIters = 40;

// x += alpha p, r -= alpha Ap; ||r||^2 and the stop test.
__global__ void __launch_bounds__(NT) k_mgcg_update(long long n, float* __restrict__ x,
                                                    float* __restrict__ r,
                                                    const float* __restrict__ p,
                                                    const float* __restrict__ Ap,
                                                    double* partials, DevScalars* ds) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const float at = (float)ds->red[RS_PCG_ALPHA];
  DFAcc2 rr;
  const long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  const long long g = blockIdx.x * (long long)NT + tid, stride = (long long)gridDim.x * NT;
  const long long n4 = n >> 2;
#pragma unroll 2
  for (long long i = g; i < n4; i += stride) {
    float4 xv = reinterpret_cast<const float4*>(x)[i];
    float4 rv = reinterpret_cast<const float4*>(r)[i];
    const float4 pv = reinterpret_cast<const float4*>(p)[i];
    const float4 av = reinterpret_cast<const float4*>(Ap)[i];
    xv.x = fmaf(at, pv.x, xv.x);
    xv.y = fmaf(at, pv.y, xv.y);
    xv.z = fmaf(at, pv.z, xv.z);
    xv.w = fmaf(at, pv.w, xv.w);
    rv.x = fmaf(-at, av.x, rv.x);
    rv.y = fmaf(-at, av.y, rv.y);
    rv.z = fmaf(-at, av.z, rv.z);
    rv.w = fmaf(-at, av.w, rv.w);
    reinterpret_cast<float4*>(x)[i] = xv;
    reinterpret_cast<float4*>(r)[i] = rv;
    rr.add_prod(rv.x, rv.x);
    rr.add_prod(rv.y, rv.y);
    rr.add_prod(rv.z, rv.z);
    rr.add_prod(rv.w, rv.w);
  }
  for (long long i = 4 * n4 + g; i < n; i += stride) {
    x[i] = fmaf(at, p[i], x[i]);
    float ri = fmaf(-at, Ap[i], r[i]);
    r[i] = ri;
    rr.add_prod(ri, ri);
  }
  double s[1] = {rr.value()};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(s, partials, &ds->ticket[TK_F32_B], o)) {
    if (tid == 0) {
      ds->red[RS_PCG_RR] = o[0];
      int it = ds->flag[FL_PCG_ITERS] + 1;
      ds->flag[FL_PCG_ITERS] = it;
      if (o[0] <= 0.25 * ds->red[RS_PCG_RRREF]) {
        ds->red[RS_PCG_RRREF] = o[0];
        ds->flag[FL_PCG_REFIT] = it;
      }
      if (o[0] <= ds->red[RS_PCG_TOL2] || it >= ds->flag[FL_PCG_LIMIT] || isnan(o[0]) ||
          it - ds->flag[FL_PCG_REFIT] >= kStallIters)
        ds->flag[FL_PCG_DONE] = 1;
    }
  }
}

// <r, z> -> beta = <r,z>/<r,z>_old (first: only stores <r,z>).
__global__ void __launch_bounds__(NT) k_mgcg_dot(long long n, const float* __restrict__ r,
                                                 const float* __restrict__ z, int first,
                                                 double* partials, DevScalars* ds) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  DFAcc2 rz;
  const long long tid = threadIdx.x + blockDim.x * (long long)threadIdx.y;
  const long long g = blockIdx.x * (long long)NT + tid, stride = (long long)gridDim.x * NT;
  const long long n4 = n >> 2;
#pragma unroll 4
  for (long long i = g; i < n4; i += stride) {
    const float4 a = reinterpret_cast<const float4*>(r)[i];
    const float4 b = reinterpret_cast<const float4*>(z)[i];
    rz.add_prod(a.x, b.x);
    rz.add_prod(a.y, b.y);
    rz.add_prod(a.z, b.z);
    rz.add_prod(a.w, b.w);
  }
  for (long long i = 4 * n4 + g; i < n; i += stride) rz.add_prod(r[i], z[i]);
  double s[1] = {rz.value()};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(s, partials, &ds->ticket[TK_PCG_INIT2], o)) {
    if (tid == 0) {
      if (!first) ds->red[RS_PCG_BETA] = o[0] / ds->red[RS_PCG_RZ];
      ds->red[RS_PCG_RZ] = o[0];
    }
  }
}

bool aligned16(const void* a) { return (reinterpret_cast<uintptr_t>(a) & 15) == 0; }

// ------------------------------------------ colour-blocked finest level --
// A plain 3D block (no periodic direction, no excluded cell) with an even
// n0, solved without a pinned cell.  Cell c = i + n0 (j + n1 k) of colour
// q = (i+j+k) mod 2 sits at q * nc/2 + c/2 in the iterate, right-hand side
// and inverse diagonal: with n0 even the two cells of a pair (2h, 2h+1)
// have opposite colours, so c/2 = h + n0/2 (j + n1 k) and a warp of one
// colour reads and writes consecutive words.  The neighbours of a cell at
// blocked index p are p - 1 + (i odd) and p + (i odd) along x, p -/+ n0/2
// along y and p -/+ n0 n1/2 along z in the other colour's half.  The face
// couplings are stored in FP16 (as bit patterns) divided by 2^e, e chosen
// so that the largest coupling lies in [2^13, 2^14); the inverse diagonal
// is formed from the rounded couplings, so every row still sums to zero.
// The V-cycle stays symmetric: one face value serves both of its cells.
struct Fast0 {
  int n0, n1, n2;
  const unsigned short *kx, *ky, *kz;
};

__device__ __forceinline__ float h2f(const unsigned short* a, long long i) {
  return __half2float(__ushort_as_half(a[i]));
}

// Largest face coupling -> the power-of-two scale 2^e (RS_MG0_SCALE).
__global__ void __launch_bounds__(NT) k_mg0_scale(long long nf, const float* kf,
                                                  double* partials, DevScalars* ds) {
  double mx = 0.;
  for (long long i = blockIdx.x * (long long)NT + threadIdx.x + BX * threadIdx.y; i < nf;
       i += (long long)gridDim.x * NT)
    mx = fmax(mx, (double)kf[i]);
  double v[1] = {mx};
  __shared__ double o[1];
  if (grid_reduce<RED_MAX, 1>(v, partials, &ds->ticket[TK_MG0], o)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      int e = 0;
      frexp(o[0], &e);  // o = f 2^e, f in [0.5, 1)
      ds->red[RS_MG0_SCALE] = o[0] > 0. ? ldexp(1.0, e - 14) : 1.0;
    }
  }
}

// Face couplings of the level (direction-blocked FP32) -> three FP16 arrays.
__global__ void k_mg0_pack(Mesh m, const float* kf, const DevScalars* ds, unsigned short* kx,
                           unsigned short* ky, unsigned short* kz) {
  const float inv = (float)(1. / ds->red[RS_MG0_SCALE]);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m.nf;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned short v = __half_as_ushort(__float2half_rn(kf[i] * inv));
    if (i < m.fofs[1]) kx[i] = v;
    else if (i < m.fofs[2]) ky[i - m.fofs[1]] = v;
    else kz[i - m.fofs[2]] = v;
  }
}

// Inverse diagonal of the rounded operator, colour-blocked (one thread per
// cell pair).
__global__ void k_mg0_diag(Fast0 f, const DevScalars* ds, float* idg0) {
  const double scale = ds->red[RS_MG0_SCALE];
  const int h0 = f.n0 / 2;
  const long long half = (long long)h0 * f.n1 * f.n2;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < half;
       p += (long long)gridDim.x * blockDim.x) {
    const long long row = p / h0;
    const int ih = (int)(p - row * h0);
    const int j = (int)(row % f.n1), k = (int)(row / f.n1);
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int i = 2 * ih + e;
      const long long fx = i + (long long)(f.n0 + 1) * (j + (long long)f.n1 * k);
      const long long fy = i + (long long)f.n0 * (j + (long long)(f.n1 + 1) * k);
      const long long fz = i + (long long)f.n0 * (j + (long long)f.n1 * k);
      const float sk = h2f(f.kx, fx) + h2f(f.kx, fx + 1) + h2f(f.ky, fy) +
                       h2f(f.ky, fy + f.n0) + h2f(f.kz, fz) +
                       h2f(f.kz, fz + (long long)f.n0 * f.n1);
      const double dg = (double)sk * scale;
      const int q = (i + j + k) & 1;
      idg0[q * half + p] = dg > 0. ? (float)(1. / dg) : 0.f;
    }
  }
}

// Red-black half-sweep of one colour on the blocked arrays.  PROLONG: the
// neighbours are read as x + cx(parent) (the injected coarse correction,
// first post-smoothing half-sweep).  FROMZERO (the first black half-sweep
// of a V-cycle): the red half-sweep from x = 0 before it is folded in --
// the red neighbours are read as b / diag, and each thread also stores
// that value for the red cell of its own pair.
template <bool PROLONG, bool FROMZERO = false>
__global__ void __launch_bounds__(NT) k_mg0_smooth(Fast0 f, const float* idg0, const float* b0,
                                                   float* x0, int color, const float* cx,
                                                   const DevScalars* ds, int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const int h0 = f.n0 / 2;
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  if (ih >= h0 || j >= f.n1) return;
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, f.n2);
  const int half = h0 * f.n1 * f.n2;
  const int hz = h0 * f.n1;
  const int own = color * half, oth = (1 - color) * half;
  const float scale = (float)ds->red[RS_MG0_SCALE];
  const int cnx = f.n0 / 2, cny = f.n1 / 2;
  for (int k = k0; k < k1; ++k) {
    const int i = 2 * ih + ((j + k + color) & 1);
    const int odd = i & 1;
    const int p = ih + h0 * (j + f.n1 * k);
    const int fx = i + (f.n0 + 1) * (j + f.n1 * k);
    const int fy = i + f.n0 * (j + (f.n1 + 1) * k);
    const int fz = i + f.n0 * (j + f.n1 * k);
    float xs[6], ks[6];
    bool in[6];
    int nb[6];
    in[0] = i > 0;
    nb[0] = p - 1 + odd;
    ks[0] = h2f(f.kx, fx);
    in[1] = i < f.n0 - 1;
    nb[1] = p + odd;
    ks[1] = h2f(f.kx, fx + 1);
    in[2] = j > 0;
    nb[2] = p - h0;
    ks[2] = h2f(f.ky, fy);
    in[3] = j < f.n1 - 1;
    nb[3] = p + h0;
    ks[3] = h2f(f.ky, fy + f.n0);
    in[4] = k > 0;
    nb[4] = p - hz;
    ks[4] = h2f(f.kz, fz);
    in[5] = k < f.n2 - 1;
    nb[5] = p + hz;
    ks[5] = h2f(f.kz, fz + f.n0 * f.n1);
    if (FROMZERO) {
#pragma unroll
      for (int q = 0; q < 6; ++q)
        xs[q] = in[q] ? b0[oth + nb[q]] * idg0[oth + nb[q]] : 0.f;
      x0[oth + p] = b0[oth + p] * idg0[oth + p];  // the other cell of the pair
    } else {
#pragma unroll
      for (int q = 0; q < 6; ++q) xs[q] = in[q] ? x0[oth + nb[q]] : 0.f;
    }
    if (PROLONG) {
      const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
      const int pc = ci + cnx * (cj + cny * ck);
      // parents of the six neighbours: the own parent or the next one
      if (in[0]) xs[0] += cx[odd ? pc : pc - 1];
      if (in[1]) xs[1] += cx[odd ? pc + 1 : pc];
      if (in[2]) xs[2] += cx[(j & 1) ? pc : pc - cnx];
      if (in[3]) xs[3] += cx[(j & 1) ? pc + cnx : pc];
      if (in[4]) xs[4] += cx[(k & 1) ? pc : pc - cnx * cny];
      if (in[5]) xs[5] += cx[(k & 1) ? pc + cnx * cny : pc];
    }
    const float bb = b0[own + p], ig = idg0[own + p];
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) acc = fmaf(ks[q], xs[q], acc);
    const float xn = fmaf(scale, acc, bb) * ig;
    x0[own + p] = xn;
  }
}

// Coarse right-hand side = sum of the red children's residuals (the
// pre-smoothing ends with a black half-sweep, which leaves the black
// residuals zero up to rounding): r = b + 2^e sum_f k_f (x_nb - x_c).
// With cidg the coarse level's first half-sweep (red, from zero) as well,
// else the coarse iterate is cleared.
// Two threads per coarse cell, one per child plane ck (lanes 2t and 2t+1
// of a warp: 16 coarse cells per warp row): each sums the residuals of
// its two red children and a lane shuffle adds the pair.  Launched on the
// coarse grid with its x extent doubled (restrict0_launch).
__global__ void __launch_bounds__(NT) k_mg0_restrict(Fast0 f, Mesh cm, const float* b0,
                                                     const float* x0, float* cb, float* cx,
                                                     const float* cidg, const DevScalars* ds,
                                                     int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const int h0 = f.n0 / 2;
  const int half = h0 * f.n1 * f.n2;
  const int hz = h0 * f.n1;
  const float scale = (float)ds->red[RS_MG0_SCALE];
  const int I = blockIdx.x * (BX / 2) + (threadIdx.x >> 1);
  const int ck = threadIdx.x & 1;
  const int J = blockIdx.y * BY + threadIdx.y;
  const bool act = I < cm.n[0] && J < cm.n[1];
  const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, cm.n[2]);
  for (int K = k0; K < k1; ++K) {  // the same trip count in every lane
    float sum = 0.f;
    if (act) {
#pragma unroll
      for (int cj = 0; cj < 2; ++cj) {
        const int ci = (cj + ck) & 1;  // red children: ci + cj + ck even
        const int i = 2 * I + ci, j = 2 * J + cj, k = 2 * K + ck;
        const int odd = i & 1;
        const int p = (i >> 1) + h0 * (j + f.n1 * k);  // red: colour 0
        const int fx = i + (f.n0 + 1) * (j + f.n1 * k);
        const int fy = i + f.n0 * (j + (f.n1 + 1) * k);
        const int fz = i + f.n0 * (j + f.n1 * k);
        const float xc = x0[p];
        float acc = 0.f;
        if (i > 0) acc = fmaf(h2f(f.kx, fx), x0[half + p - 1 + odd] - xc, acc);
        if (i < f.n0 - 1) acc = fmaf(h2f(f.kx, fx + 1), x0[half + p + odd] - xc, acc);
        if (j > 0) acc = fmaf(h2f(f.ky, fy), x0[half + p - h0] - xc, acc);
        if (j < f.n1 - 1) acc = fmaf(h2f(f.ky, fy + f.n0), x0[half + p + h0] - xc, acc);
        if (k > 0) acc = fmaf(h2f(f.kz, fz), x0[half + p - hz] - xc, acc);
        if (k < f.n2 - 1)
          acc = fmaf(h2f(f.kz, fz + f.n0 * f.n1), x0[half + p + hz] - xc, acc);
        sum += fmaf(scale, acc, b0[p]);
      }
    }
    sum += __shfl_xor_sync(0xffffffffu, sum, 1);
    if (act && ck == 0) {
      const int C = I + cm.n[0] * (J + cm.n[1] * K);
      cb[C] = sum;
      cx[C] = cidg && ((I + J + K) & 1) == 0 ? sum * cidg[C] : 0.f;
    }
  }
}

// ---- inner CG in the colour-blocked order of the finest level (fast0) --
// With the colour-blocked finest level the inner CG keeps r, z, p, Ap and
// x in that order (cell c of colour q at q * nc/2 + c/2), so the V-cycle
// reads r and writes z in place: no reordering pass at either end of it.
// The FP64 side stays in cell order; these kernels convert at the borders.

// r = FP32 of the FP64 residual (cell order -> blocked), x = 0; ||r||^2.
__global__ void __launch_bounds__(NT) k_mgcg_init_blk(Fast0 f, const double* __restrict__ r64,
                                                      float* __restrict__ r,
                                                      float* __restrict__ x, double tol,
                                                      int limit, int dev_params,
                                                      double* partials, DevScalars* ds) {
  pdl_wait();
  pdl_trigger();
  const int h0 = f.n0 / 2;
  const int half = h0 * f.n1 * f.n2;  // < 2^30
  const double2* r2 = reinterpret_cast<const double2*>(r64);
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  double s = 0.;
  for (int p = blockIdx.x * NT + tid; p < half; p += gridDim.x * NT) {
    const int row = p / h0;
    const int q = (row % f.n1 + row / f.n1) & 1;  // colour of cell 2p
    const double2 v = r2[p];                              // cells 2p, 2p + 1
    r[q * half + p] = d2f(v.x);
    r[(1 - q) * half + p] = d2f(v.y);
    x[p] = 0.f;
    x[half + p] = 0.f;
    s += v.x * v.x;
    s += v.y * v.y;
  }
  double v[1] = {s};
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(v, partials, &ds->ticket[TK_F32_INIT], o)) {
    if (tid == 0) {
      if (dev_params) tol = ds->red[RS_INNER_TOL];
      else ds->flag[FL_PCG_LIMIT] = limit;
      ds->red[RS_PCG_FF] = o[0];
      ds->red[RS_PCG_RR] = o[0];
      ds->red[RS_PCG_TOL2] = tol * tol * o[0];
      ds->red[RS_PCG_RRREF] = o[0];
      ds->flag[FL_PCG_ITERS] = 0;
      ds->flag[FL_PCG_REFIT] = 0;
      ds->flag[FL_PCG_DONE] = (o[0] == 0. || ds->flag[FL_PCG_LIMIT] <= 0) ? 1 : 0;
    }
  }
}

// p = z + beta p_old (z on the first iteration), Ap = A32 p with the FP32
// operator (cell-order couplings and diagonal), <p, Ap>: one thread per
// cell pair (2h, 2h + 1) of a row on the half-width grid, so that every
// warp-wide load reads 32 consecutive words of one colour; the two cells
// share their x neighbours (each is the other's), 12 direction values per
// pair.  32-bit indices (the blocked level has < 2^30 cells).
__global__ void __launch_bounds__(NT) k_cg32_dir_spmv_blk(Fast0 f, const float* __restrict__ kf,
                                                          const float* __restrict__ dg,
                                                          const float* __restrict__ z,
                                                          const float* __restrict__ pold,
                                                          float* __restrict__ pnew,
                                                          float* __restrict__ Ap, int fofs1,
                                                          int fofs2, double* partials,
                                                          DevScalars* ds, int kch) {
  pdl_wait();
  pdl_trigger();
  if (ds->flag[FL_PCG_DONE]) return;
  const bool first = ds->flag[FL_PCG_ITERS] == 0;
  const float beta = first ? 0.f : (float)ds->red[RS_PCG_BETA];
  const int n0 = f.n0, n1 = f.n1, n2 = f.n2, h0 = n0 / 2;
  const int half = h0 * n1 * n2, hz = h0 * n1, nxy = n0 * n1;
  auto P = [&](int b) { return first ? z[b] : fmaf(beta, pold[b], z[b]); };
  DFAcc2 acc;
  const int ih = blockIdx.x * BX + threadIdx.x;
  const int j = blockIdx.y * BY + threadIdx.y;
  if (ih < h0 && j < n1) {
    const int k0 = blockIdx.z * kch, k1 = min(k0 + kch, n2);
    for (int k = k0; k < k1; ++k) {
      const int row = j + n1 * k;
      const int p = ih + h0 * row;
      const int q = (j + k) & 1;  // colour of the even cell
      const int a0 = q * half + p, a1 = (1 - q) * half + p;  // even, odd cell
      const int c0 = 2 * p;
      const int i0 = 2 * ih;
      const int fx = i0 + (n0 + 1) * row;
      const int fy = fofs1 + i0 + n0 * (j + (n1 + 1) * k);
      const int fz = fofs2 + c0;
      const float p0 = P(a0), p1 = P(a1);
      float s0 = dg[c0] * p0, s1 = dg[c0 + 1] * p1;
      // x: even cell's low neighbour is the odd cell of the pair before;
      // the odd cell's high neighbour the even cell of the pair after
      if (i0 > 0) s0 = fmaf(-kf[fx], P(a1 - 1), s0);
      s0 = fmaf(-kf[fx + 1], p1, s0);
      s1 = fmaf(-kf[fx + 1], p0, s1);
      if (i0 + 2 < n0) s1 = fmaf(-kf[fx + 2], P(a0 + 1), s1);
      if (j > 0) {
        s0 = fmaf(-kf[fy], P(a1 - h0), s0);
        s1 = fmaf(-kf[fy + 1], P(a0 - h0), s1);
      }
      if (j < n1 - 1) {
        s0 = fmaf(-kf[fy + n0], P(a1 + h0), s0);
        s1 = fmaf(-kf[fy + n0 + 1], P(a0 + h0), s1);
      }
      if (k > 0) {
        s0 = fmaf(-kf[fz], P(a1 - hz), s0);
        s1 = fmaf(-kf[fz + 1], P(a0 - hz), s1);
      }
      if (k < n2 - 1) {
        s0 = fmaf(-kf[fz + nxy], P(a1 + hz), s0);
        s1 = fmaf(-kf[fz + nxy + 1], P(a0 + hz), s1);
      }
      pnew[a0] = p0;
      pnew[a1] = p1;
      Ap[a0] = s0;
      Ap[a1] = s1;
      acc.add_prod(p0, s0);
      acc.add_prod(p1, s1);
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

// x64 (cell order) += FP64 of x32 (blocked).
__global__ void k_accumulate_blk(Fast0 f, double* __restrict__ x, const float* __restrict__ e) {
  pdl_wait();
  pdl_trigger();
  const int h0 = f.n0 / 2;
  const int half = h0 * f.n1 * f.n2;  // < 2^30
  double2* x2 = reinterpret_cast<double2*>(x);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < half; p += gridDim.x * blockDim.x) {
    const int row = p / h0;
    const int q = (row % f.n1 + row / f.n1) & 1;
    double2 v = x2[p];
    v.x += f2d(e[q * half + p]);
    v.y += f2d(e[(1 - q) * half + p]);
    x2[p] = v;
  }
}

// ------------------------------- one CTA or cluster per pressure solve --
// The whole mixed pressure solve of a small plain block (no periodic
// direction, no excluded cell) by ONE CTA or ONE thread-block cluster: FP64
// iterative refinement around the multigrid-preconditioned FP32 CG, the
// same algorithm as the grid launches (k_ir_residual / k_ctl_refine /
// k_mgcg_* / the V-cycle), with group barriers (__syncthreads, or the
// cluster barrier, which orders the CTAs' global-memory accesses) between
// the passes instead of kernel boundaries, and group-wide sums in FP64 in
// a fixed order.  Hundreds of small cases then each hold one SM (or a few)
// for their solve instead of queueing a few hundred tiny grid launches
// apiece.  The levels above `top` stay in global memory (L2 for a small
// case) and are swept by the whole group; `top` and below are staged into
// CTA 0's shared memory once per solve and run there as one sub-V-cycle
// while the other CTAs wait at the barrier (the right-hand side and the
// result of level `top` pass through its global arrays).
struct CtaPressure {
  Mesh m;
  const double *kf, *f;       // FP64 couplings, right-hand side
  double* dg;                 // FP64 diagonal (set up by the launch)
  double* x;                  // correction (out)
  float *kf32, *dg32, *idg32; // FP32 level-0 operator (set up by the launch)
  float *x32, *r32, *z32, *p, *pb, *Ap;
  long long pin;
  int singular, limit, graph;
  double tol, inner_min;
  int nl, top;  // levels; first level in shared memory (< nl)
  MgBlock blk;  // the staged levels
  Mesh mtop;    // level `top`, exchanged through global memory
  float *btop, *xtop;
  Mesh gm[kMgMaxLevels];
  const float *gkf[kMgMaxLevels], *gidg[kMgMaxLevels];
  float *gx[kMgMaxLevels], *gb[kMgMaxLevels];
  int nsweep;
  // the set-up's outputs: couplings and inverse diagonal of every level
  // (level 0: kf32, idg32) and the dense coarsest inverse (null: none)
  float *lkf[kMgMaxLevels], *lidg[kMgMaxLevels];
  float* cinv;
  DevScalars* ds;
};

// CTA-wide FP64 sum, the same value in every thread (sd: >= 34 doubles).
__device__ double cta_sum(double v, double* sd) {
  v = warp_sum(v);
  const int nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) sd[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (int)threadIdx.x < nw ? sd[threadIdx.x] : 0.;
    t = warp_sum(t);
    if (threadIdx.x == 0) sd[32] = t;
  }
  __syncthreads();
  const double r = sd[32];
  __syncthreads();
  return r;
}
__device__ double grp_sum(double v, double* sd, const CtaG&) { return cta_sum(v, sd); }
// Cluster-wide (sd: >= 38 doubles): each CTA's sum goes to sd[34 + parity];
// after one cluster barrier lane q of the first warp reads CTA q's, all in
// flight at once, lane 0 adds them in rank order and passes the total to
// the CTA's threads through sd[36 + parity].  The slots alternate between
// calls, so a slot is rewritten only after the next call's cluster (or CTA)
// barrier, which every reader of its previous value has passed; the one
// cluster barrier also orders the caller's earlier global stores.
__device__ double grp_sum(double v, double* sd, const ClusterG& g) {
  const int tid = threadIdx.x, lane = tid & 31, nw = (blockDim.x + 31) >> 5;
  const int par = g.par;
  g.par ^= 1;
  v = warp_sum(v);
  if (lane == 0) sd[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    double t = lane < nw ? sd[lane] : 0.;
    t = warp_sum(t);
    if (lane == 0) sd[34 + par] = t;
  }
  auto cl = cooperative_groups::this_cluster();
  cl.sync();
  if (tid < 32) {
    const int nb = (int)cl.num_blocks();
    const double mine = lane < nb ? *cl.map_shared_rank(&sd[34 + par], lane) : 0.;
    double t = 0.;
    for (int q = 0; q < nb; ++q) t += __shfl_sync(0xffffffffu, mine, q);
    if (lane == 0) sd[36 + par] = t;
  }
  __syncthreads();
  return sd[36 + par];
}
__device__ bool grp_lead(const CtaG&) { return true; }
__device__ bool grp_lead(const ClusterG&) {
  return cooperative_groups::this_cluster().block_rank() == 0;
}

__device__ __forceinline__ const Mesh& lvl_mesh(const CtaPressure& P, int l) {
  return l < P.top ? P.gm[l] : P.blk.m[l - P.top];
}

// The per-solve set-up that the grid form launches as separate kernels
// (k_diag, then k_mg_coarsen / k_mg_diag per level and k_mg_coarse_inv),
// with the same arithmetic: level 0's FP32 couplings and its FP64 / FP32
// diagonals (the pinned row an identity row), every coarser level's
// couplings and inverse diagonal (level l coarsened while level l - 1's
// diagonal is formed, one barrier per level), and the dense inverse of the
// coarsest level by CTA 0 with its dynamic shared memory as scratch (the
// levels are staged there afterwards).  Ends with a group barrier.
template <int DIM, class G>
__device__ void grp_setup(const CtaPressure& P, float* sm, const G& g) {
  const Mesh& m = P.m;
  const int tid = g.rank(), nt = g.size();
  const int nf = (int)m.nf, n = (int)m.nc;
  for (int f0 = tid; f0 < nf; f0 += 4 * nt) {
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = f0 + u * nt < nf ? P.kf[f0 + u * nt] : 0.;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (f0 + u * nt < nf) P.kf32[f0 + u * nt] = d2f(v[u]);
  }
  for (int c = tid; c < n; c += nt) {
    int id[3];
    blk_ijk<DIM>(m, c, id);
    double s = 0.;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const long long fl = face_id(m, d, id[0], id[1], id[2]);
      if (id[d] > 0) s += P.kf[fl];
      if (id[d] < m.n[d] - 1) s += P.kf[fl + face_stride(m, d)];
    }
    if (c == P.pin) s = 1.;
    P.dg[c] = s;
    const float s32 = d2f(s);
    P.dg32[c] = s32;
    P.idg32[c] = 1.f / s32;
  }
  g.sync();
  for (int l = 1; l <= P.nl; ++l) {
    if (l < P.nl) {
      const Mesh& fm = lvl_mesh(P, l - 1);
      const Mesh& cm = lvl_mesh(P, l);
      const int nc = (int)cm.nc;
      for (int c = tid; c < nc; c += nt) {
        int I[3];
        blk_ijk<DIM>(cm, c, I);
        coarsen_cell<DIM>(fm, cm, P.lkf[l - 1], P.lkf[l], I, c);
      }
    }
    if (l >= 2) {
      const Mesh& dm = lvl_mesh(P, l - 1);
      const int nc = (int)dm.nc;
      for (int c = tid; c < nc; c += nt) {
        int I[3];
        blk_ijk<DIM>(dm, c, I);
        const float s = diag_cell<DIM>(dm, P.lkf[l - 1], I);
        P.lidg[l - 1][c] = s > 0.f ? 1.f / s : 0.f;
      }
    }
    if (l == P.nl && P.cinv && grp_lead(g))
      dense_inverse<DIM>(lvl_mesh(P, P.nl - 1), P.lkf[P.nl - 1], P.cinv, sm);
    g.sync();
  }
}

// z = M^-1 r by the group: the global levels swept and restricted by all,
// the staged sub-V-cycle by CTA 0 (its level set V in shared memory).
template <int DIM, class G>
__device__ void grp_precondition(const CtaPressure& P, CtaLevels& V, float* sm, float* red,
                                 const G& g) {
  const int T = P.top, ns = P.nsweep;
  for (int l = 0; l < T; ++l) {
    const long long lp = l == 0 ? P.pin : -1;
    for (int s = 0; s < ns; ++s) {
      blk_half<DIM, false>(P.gm[l], P.gkf[l], P.gidg[l], P.gb[l], P.gx[l], 0, s == 0, lp, g);
      blk_half<DIM, false>(P.gm[l], P.gkf[l], P.gidg[l], P.gb[l], P.gx[l], 1, false, lp, g);
    }
    const bool last = l + 1 == T;
    blk_restrict<DIM, false>(P.gm[l], last ? P.mtop : P.gm[l + 1], P.gkf[l], P.gb[l], P.gx[l],
                             last ? P.btop : P.gb[l + 1], lp, g);
  }
  if (grp_lead(g)) {
    const int n = (int)P.mtop.nc;
    for (int q = threadIdx.x; q < n; q += blockDim.x) V.b[0][q] = P.btop[q];
    __syncthreads();
    cta_vcycle<DIM, false>(V, red);
    for (int q = threadIdx.x; q < n; q += blockDim.x) P.xtop[q] = V.x[0][q];
  }
  g.sync();
  for (int l = T - 1; l >= 0; --l) {
    const long long lp = l == 0 ? P.pin : -1;
    const bool last = l + 1 == T;
    const Mesh& m = P.gm[l];
    const Mesh& cm = last ? P.mtop : P.gm[l + 1];
    const float* cx = last ? P.xtop : P.gx[l + 1];
    float* x = P.gx[l];
    const int nc = (int)m.nc;
    const float r0 = 1.f / (float)m.n[0], r1 = 1.f / (float)m.n[1];
    for (int c = g.rank(); c < nc; c += g.size()) {
      int id[3];
      blk_ijk<DIM>(m.n[0], m.n[1], r0, r1, c, id);
      x[c] += cx[(int)cell_id(cm, id[0] >> 1, id[1] >> 1, id[2] >> 1)];
    }
    g.sync();
    for (int s = 0; s < ns; ++s) {
      blk_half<DIM, false>(m, P.gkf[l], P.gidg[l], P.gb[l], x, 1, false, lp, g);
      blk_half<DIM, false>(m, P.gkf[l], P.gidg[l], P.gb[l], x, 0, false, lp, g);
    }
  }
}

// Inner MG-CG for A e = r (FP32, e in x32) to relative tolerance t within
// `lim` iterations, stopping on a stall as k_mgcg_update does; returns the
// iterations.  The refinement's residual pass has left r in r32 (rounded
// from FP64), x32 = 0 and rr0 = <r, r> in FP64.
template <int DIM, class G>
__device__ int grp_mgcg(const CtaPressure& P, CtaLevels& V, float* sm, float* red, double* sd,
                        double rr0, double t, int lim, const G& g) {
  const Mesh& m = P.m;
  const int n = (int)m.nc, tid = g.rank(), nt = g.size();
  double s;
  if (rr0 == 0. || lim <= 0) return 0;
  const double tol2 = t * t * rr0;
  grp_precondition<DIM>(P, V, sm, red, g);
  s = 0.;
  for (int c = tid; c < n; c += nt) s += (double)P.r32[c] * (double)P.z32[c];
  double rz = grp_sum(s, sd, g);
  double rref = rr0, beta = 0.;
  int it = 0, refit = 0;
  float* pold = P.p;
  float* pnew = P.pb;
  const int cs[3] = {1, m.n[0], m.n[0] * m.n[1]};
  const int fs[3] = {1, (int)m.fnx[1], (int)(m.fnx[2] * m.fny[2])};
  const int pin = (int)P.pin;
  const float r0 = 1.f / (float)m.n[0], r1 = 1.f / (float)m.n[1];
  for (;;) {
    // p = z + beta p_old (z on the first), Ap, <p, Ap> (k_cg32_dir_spmv)
    const bool first = it == 0;
    const float bt = (float)beta;
    auto Pv = [&](int c) { return first ? P.z32[c] : fmaf(bt, pold[c], P.z32[c]); };
    // U cells per thread per pass with every load before the stores (a
    // group alone on a case is latency-bound otherwise)
    constexpr int U = 4;
    s = 0.;
    for (int c0 = tid; c0 < n; c0 += U * nt) {
      float pv[U], av[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = c0 + u * nt;
        pv[u] = av[u] = 0.f;
        if (c >= n) continue;
        int id[3];
        blk_ijk<DIM>(m.n[0], m.n[1], r0, r1, c, id);
        const float pc = Pv(c);
        float a;
        if (c == pin) {
          a = pc;
        } else {
          a = P.dg32[c] * pc;
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            const int fl = (int)m.fofs[d] + id[0] + m.fnx[d] * (id[1] + m.fny[d] * id[2]);
            if (id[d] > 0 && c - cs[d] != pin) a = fmaf(-P.kf32[fl], Pv(c - cs[d]), a);
            if (id[d] < m.n[d] - 1 && c + cs[d] != pin)
              a = fmaf(-P.kf32[fl + fs[d]], Pv(c + cs[d]), a);
          }
        }
        pv[u] = pc;
        av[u] = a;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = c0 + u * nt;
        if (c >= n) continue;
        pnew[c] = pv[u];
        P.Ap[c] = av[u];
        s += (double)pv[u] * (double)av[u];
      }
    }
    const double pAp = grp_sum(s, sd, g);
    const float at = (float)(rz / pAp);
    s = 0.;
    for (int c0 = tid; c0 < n; c0 += U * nt) {
      float xv[U], rv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = c0 + u * nt;
        xv[u] = rv[u] = 0.f;
        if (c >= n) continue;
        xv[u] = fmaf(at, pnew[c], P.x32[c]);
        rv[u] = fmaf(-at, P.Ap[c], P.r32[c]);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = c0 + u * nt;
        if (c >= n) continue;
        P.x32[c] = xv[u];
        P.r32[c] = rv[u];
        s += (double)rv[u] * (double)rv[u];
      }
    }
    const double rr = grp_sum(s, sd, g);
    ++it;
    if (rr <= 0.25 * rref) {
      rref = rr;
      refit = it;
    }
    if (rr <= tol2 || it >= lim || isnan(rr) || it - refit >= kStallIters) break;
    grp_precondition<DIM>(P, V, sm, red, g);
    s = 0.;
    for (int c = tid; c < n; c += nt) s += (double)P.r32[c] * (double)P.z32[c];
    const double rz1 = grp_sum(s, sd, g);
    beta = rz1 / rz;
    rz = rz1;
    float* tmp = pold;
    pold = pnew;
    pnew = tmp;
  }
  return it;
}

// The whole solve by the launch's group G: one CTA (CtaG) or the one
// cluster the grid is (ClusterG).
template <int DIM, class G>
__global__ void __launch_bounds__(kBlkThreads)
    k_cta_pressure(const __grid_constant__ CtaPressure P) {
  extern __shared__ float sm[];
  __shared__ float red[32];
  __shared__ double sd[38];
  __shared__ CtaLevels V;  // the staged levels (CTA 0)
  const G g;
  const Mesh& m = P.m;
  const int n = (int)m.nc, tid = g.rank(), nt = g.size();
  grp_setup<DIM>(P, sm, g);
  if (grp_lead(g)) cta_stage_levels(P.blk, sm, &V);
  double mean = 0.;
  if (P.singular) {
    double s = 0.;
    for (int c = tid; c < n; c += nt) s += P.f[c];
    mean = grp_sum(s, sd, g) / (double)n;  // also orders the staging above
  } else {
    g.sync();
    __syncthreads();
  }
  for (int c = tid; c < n; c += nt) P.x[c] = 0.;
  const int cs[3] = {1, m.n[0], m.n[0] * m.n[1]};
  const int fs[3] = {1, (int)m.fnx[1], (int)(m.fnx[2] * m.fny[2])};
  const long long pin = P.pin;
  double ff = -1., pres = 0., last = 0.;
  int total = 0, outer = 0;
  bool conv = false, nan = false;
  for (;;) {
    // FP64 residual r = f - mean - A x (x = 0 on the first pass) and its
    // FP64 <r, r>; r itself is kept only as the inner CG's FP32 start
    double s = 0.;
    for (int c0 = tid; c0 < n; c0 += 2 * nt) {
      double rv[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int c = c0 + u * nt;
        rv[u] = 0.;
        if (c >= n) continue;
        double rc = P.f[c] - mean;
        if (outer > 0) {
          double acc;
          if (c == pin) {
            acc = P.x[c];
          } else {
            int id[3];
            blk_ijk<DIM>(m, c, id);
            acc = P.dg[c] * P.x[c];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
              const int fl = (int)m.fofs[d] + id[0] + m.fnx[d] * (id[1] + m.fny[d] * id[2]);
              if (id[d] > 0 && c - cs[d] != pin) acc -= P.kf[fl] * P.x[c - cs[d]];
              if (id[d] < m.n[d] - 1 && c + cs[d] != pin)
                acc -= P.kf[fl + fs[d]] * P.x[c + cs[d]];
            }
          }
          rc -= acc;
        }
        rv[u] = rc;
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int c = c0 + u * nt;
        if (c >= n) continue;
        // the inner CG's start: r rounded to FP32, e = 0
        P.r32[c] = d2f(rv[u]);
        P.x32[c] = 0.f;
        s += rv[u] * rv[u];
      }
    }
    const double rr = grp_sum(s, sd, g);
    last = rr;
    if (isnan(rr)) {
      nan = true;
      break;
    }
    if (ff < 0.) ff = rr;
    pres = ff > 0. ? sqrt(rr / ff) : 0.;
    if (ff == 0. || rr <= P.tol * P.tol * ff) {
      conv = true;
      break;
    }
    if (total >= P.limit || outer >= 50) break;
    const double t = fmax(0.5 * P.tol * sqrt(ff / rr), P.inner_min);
    total += grp_mgcg<DIM>(P, V, sm, red, sd, rr, t, P.limit - total, g);
    for (int c0 = tid; c0 < n; c0 += 4 * nt) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = c0 + u * nt;
        v[u] = c < n ? P.x[c] + (double)P.x32[c] : 0.;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (c0 + u * nt < n) P.x[c0 + u * nt] = v[u];
    }
    ++outer;
    g.sync();
  }
  if (P.singular) {
    double s = 0.;
    for (int c = tid; c < n; c += nt) s += P.x[c];
    const double xm = grp_sum(s, sd, g) / (double)n;
    for (int c = tid; c < n; c += nt) P.x[c] -= xm;
  }
  if (tid == 0) {
    DevScalars* ds = P.ds;
    ds->red[RS_P_RES] = pres;
    ds->red[RS_IR_RR] = last;  // NaN when the system held one
    ds->flag[FL_PCG_ITERS] = total;
    ds->flag[FL_IR_OUTER] = outer;
    ds->flag[FL_PCG_DONE] = conv ? 1 : 0;
    if (P.graph) {
      ds->flag[FL_STEP_PITERS] += total;
      if (!conv) ds->flag[FL_STEP_PUNCONV] += 1;
      if (nan) ds->flag[FL_STEP_NAN] = 1;
    }
  }
}

int flat_blocks_mg(long long n) {
  long long b = (n + NT - 1) / NT;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

// Grid of a red-black half-sweep: one thread per cell pair along x, sized
// in whole waves over the half-width mesh.
Launch fast0_launch(const Mesh& m) {
  Mesh h = m;
  h.n[0] = m.n[0] / 2;
  return cell_launch_waves(h, resident_ctas((const void*)k_mg0_smooth<false>));
}

Launch half_launch(const Mesh& m) {
  const bool per = any_periodic(m);
  const void* k = m.dim == 3 ? (per ? (const void*)k_mg_smooth<3, true> : (const void*)k_mg_smooth<3, false>)
                             : (per ? (const void*)k_mg_smooth<2, true> : (const void*)k_mg_smooth<2, false>);
  Mesh h = m;
  h.n[0] = (m.n[0] + 1) / 2;
  return cell_launch_waves(h, resident_ctas(k));
}

}  // namespace

Mesh mg_coarse_mesh(const Mesh& f) {
  Mesh c = f;
  c.ex = nullptr;  // a coarse level carries the exclusion in its couplings
  for (int d = 0; d < f.dim; ++d) {
    c.n[d] = f.n[d] / 2;
    c.h[d] = f.h[d] * 2.;
  }
  c.nc = (long long)c.n[0] * c.n[1] * (f.dim == 3 ? c.n[2] : 1);
  long long off = 0;
  for (int d = 0; d < 3; ++d) {
    c.fnx[d] = c.n[0] + (d == 0);
    c.fny[d] = c.n[1] + (d == 1);
    c.fofs[d] = off;
    if (d < f.dim) off += (long long)c.fnx[d] * c.fny[d] * ((f.dim == 3 ? c.n[2] : 1) + (d == 2));
  }
  c.nf = off;
  return c;
}

int mg_levels_for(const Mesh& m) {
  int nlev = 1;
  Mesh cur = m;
  while (nlev < kMgMaxLevels && cur.nc > kMgCoarseTarget) {
    bool ok = true;
    for (int d = 0; d < cur.dim; ++d) {
      if (cur.n[d] % 2 != 0 || cur.n[d] / 2 < 2) ok = false;
      // a periodic direction keeps an even count (red-black colouring
      // across the periodic end)
      if (cur.per[d] && (cur.n[d] / 2) % 2 != 0) ok = false;
    }
    if (!ok) break;
    cur = mg_coarse_mesh(cur);
    ++nlev;
  }
  return nlev;
}

#define MG_LAUNCH(KERNEL, L, ...)                                               \
  do {                                                                          \
    if (dim == 3)                                                               \
      PDL(KERNEL<3>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);         \
    else                                                                        \
      PDL(KERNEL<2>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);         \
    count_launches(1);                                                          \
  } while (0)
// the same for kernels instantiated per periodicity (P: any periodic direction)
#define MG_LAUNCH_P(KERNEL, L, P, ...)                                          \
  do {                                                                          \
    if (dim == 3) {                                                             \
      if (P) PDL(KERNEL<3, true>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);   \
      else PDL(KERNEL<3, false>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);   \
    } else {                                                                    \
      if (P) PDL(KERNEL<2, true>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);   \
      else PDL(KERNEL<2, false>, (L).grid, (L).block, 0, st, __VA_ARGS__, (L).kch);   \
    }                                                                           \
    count_launches(1);                                                          \
  } while (0)

// First level handled inside one CTA and that CTA's shared memory (x, b,
// inverse diagonal and couplings of every level from there down, each
// array 16-byte aligned); top = nlev when the coarsest level is too large.
void mg_plan_block(MgWork& mg) {
  mg.top = mg.nlev;
  for (int l = 0; l < mg.nlev; ++l)
    if (mg.lev[l].m.nc <= kMgBlockMax) {
      mg.top = l;
      break;
    }
  long long fl = 0;
  for (int l = mg.top; l < mg.nlev; ++l) {
    const Mesh& m = mg.lev[l].m;
    fl += 3 * ((m.nc + 3) / 4 * 4) + (m.nf + 3) / 4 * 4;
  }
  mg.smem_bytes = (int)(fl * sizeof(float));
}

cudaError_t mg_setup(MgWork& mg, PcgWork& w, cudaStream_t st) {
  int dim = mg.lev[0].m.dim;
  mg.lev[0].kf = w.kf32;
  mg.lev[0].dg = w.dg32;
  mg.lev[0].idg = w.idg32;
  // the colour-blocked FP16 finest level: allocated for this mesh, no
  // pinned cell in this solve, and a grid level (not the in-CTA cycle)
  mg.fast0 = mg.k16[0] != nullptr && w.pin < 0 && mg.nlev >= 2 && mg.top >= 1 && !mg.cta;
  if (mg.fast0) {
    const Mesh& m = mg.lev[0].m;
    Fast0 f{m.n[0], m.n[1], m.n[2], mg.k16[0], mg.k16[1], mg.k16[2]};
    k_mg0_scale<<<flat_blocks_mg(m.nf), dim3(BX, BY), 0, st>>>(m.nf, w.kf32, w.partials, w.ds);
    k_mg0_pack<<<flat_blocks_mg(m.nf), NT, 0, st>>>(m, w.kf32, w.ds, mg.k16[0], mg.k16[1],
                                                    mg.k16[2]);
    k_mg0_diag<<<flat_blocks_mg(m.nc / 2), NT, 0, st>>>(f, w.ds, mg.idg0);
    count_launches(3);
  }
  for (int l = 1; l < mg.nlev; ++l) {
    MgLevel& f = mg.lev[l - 1];
    MgLevel& c = mg.lev[l];
    Launch L = cell_launch(c.m);
    MG_LAUNCH(k_mg_coarsen, L, f.m, c.m, f.kf, c.kf);
    MG_LAUNCH(k_mg_diag, L, c.m, c.kf, c.dg, c.idg);
  }
  if (mg.cdense) {
    const MgLevel& cl = mg.lev[mg.nlev - 1];
    if (dim == 3) k_mg_coarse_inv<3><<<1, 256, 0, st>>>(cl.m, cl.kf, mg.cinv);
    else k_mg_coarse_inv<2><<<1, 256, 0, st>>>(cl.m, cl.kf, mg.cinv);
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t mg_prepare(MgWork& mg) {
  mg_plan_block(mg);
  // the coarsest level is solved exactly when it is small and below the top
  // level of the in-CTA cycle (a coarse level: singular, unpinned)
  mg.cdense = mg.cinv && mg.nlev >= 2 && mg.top < mg.nlev && mg.top < mg.nlev - 1 &&
              mg.lev[mg.nlev - 1].m.nc <= kMgCoarseTarget;
  if (mg.cdense) {
    // the dense inverse joins the CTA's shared memory after the levels
    const long long n = mg.lev[mg.nlev - 1].m.nc;
    mg.smem_cinv_off = mg.smem_bytes / (int)sizeof(float);
    mg.smem_bytes += (int)(n * n * sizeof(float));
  }
  if (mg.cta && mg.cdense) {
    // the one-group solve forms the dense inverse in its dynamic shared
    // memory before staging the levels there
    const int scratch = (int)(kDenseScratch * sizeof(float));
    if (mg.smem_bytes < scratch) mg.smem_bytes = scratch;
  }
  if (mg.nlev > 0 && mg.top < mg.nlev) {
    // (the kernels' static shared memory adds a few KB)
    if (mg.smem_bytes > 220 * 1024) return cudaErrorInvalidValue;
    const bool per = any_periodic(mg.lev[0].m);
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (mg.cta && !per) {
      cudaError_t e =
          mg.lev[0].m.dim == 3
              ? cudaFuncSetAttribute(k_cta_pressure<3, CtaG>, attr, mg.smem_bytes)
              : cudaFuncSetAttribute(k_cta_pressure<2, CtaG>, attr, mg.smem_bytes);
      if (e != cudaSuccess) return e;
      e = mg.lev[0].m.dim == 3
              ? cudaFuncSetAttribute(k_cta_pressure<3, ClusterG>, attr, mg.smem_bytes)
              : cudaFuncSetAttribute(k_cta_pressure<2, ClusterG>, attr, mg.smem_bytes);
      if (e != cudaSuccess) return e;
    }
    if (mg.lev[0].m.dim == 3)
      return per ? cudaFuncSetAttribute(k_mg_block_vcycle<3, true>, attr, mg.smem_bytes)
                 : cudaFuncSetAttribute(k_mg_block_vcycle<3, false>, attr, mg.smem_bytes);
    return per ? cudaFuncSetAttribute(k_mg_block_vcycle<2, true>, attr, mg.smem_bytes)
               : cudaFuncSetAttribute(k_mg_block_vcycle<2, false>, attr, mg.smem_bytes);
  }
  return cudaSuccess;
}

namespace {
// One red-black half-sweep of a level (k_mg_smooth).
void mg_smooth(int dim, const Launch& H, bool per, const Mesh& m, const float* kf,
               const float* idg, const float* b, float* x, int color, int zero, long long pin,
               const float* cx, int cnx, int cny, const DevScalars* ds, cudaStream_t st) {
  MG_LAUNCH_P(k_mg_smooth, H, per, m, kf, idg, b, x, color, zero, pin, cx, cnx, cny, ds);
}

// z = M^-1 r: one V-cycle with `nsweep` (red, black) sweeps before and
// (black, red) sweeps after each coarse correction.  Levels above `top`
// are grid launches; `top` and below run in one CTA.
cudaError_t mg_vcycle_launch(MgWork& mg, const float* r, float* z, long long pin,
                             DevScalars* ds, cudaStream_t st) {
  int dim = mg.lev[0].m.dim;
  const bool per = any_periodic(mg.lev[0].m);
  mg.lev[0].b = const_cast<float*>(r);
  mg.lev[0].x = z;
  const int ns = mg.nsweep;
  const int top = mg.top < mg.nlev ? mg.top : mg.nlev - 1;
  const bool fast0 = mg.fast0 && top >= 1 && ns >= 1;
  const Mesh& m0 = mg.lev[0].m;
  const Fast0 f0{m0.n[0], m0.n[1], m0.n[2], mg.k16[0], mg.k16[1], mg.k16[2]};
  if (fast0) {
    // level 0 on the colour-blocked arrays, whose right-hand side and
    // iterate are the inner CG's r and z themselves (kept colour-blocked):
    // red from zero, then black, (red, black)^(ns-1), restriction of the
    // red residuals
    const Launch H = fast0_launch(m0);
    float* x0 = z;
    const float* b0 = r;
    for (int s = 0; s < ns; ++s) {
      if (s > 0) {
        PDL(k_mg0_smooth<false>, H.grid, H.block, 0, st, f0, mg.idg0, b0, x0, 0, nullptr, ds,
            H.kch);
        count_launches(1);
      }
      // the first black half-sweep carries the red one from zero
      if (s == 0)
        PDL(k_mg0_smooth<false, true>, H.grid, H.block, 0, st, f0, mg.idg0, b0, x0, 1, nullptr, ds,
            H.kch);
      else
        PDL(k_mg0_smooth<false>, H.grid, H.block, 0, st, f0, mg.idg0, b0, x0, 1, nullptr, ds,
            H.kch);
      count_launches(1);
    }
    MgLevel& c = mg.lev[1];
    Mesh c2 = c.m;  // two threads per coarse cell along x
    c2.n[0] *= 2;
    const Launch L = cell_launch_waves(c2, resident_ctas((const void*)k_mg0_restrict));
    const float* cidg = 1 < top ? c.idg : nullptr;
    PDL(k_mg0_restrict, L.grid, L.block, 0, st, f0, c.m, b0, x0, c.b, c.x, cidg, ds, L.kch);
    count_launches(1);
  }
  for (int l = fast0 ? 1 : 0; l < top; ++l) {
    MgLevel& f = mg.lev[l];
    long long lp = l == 0 ? pin : -1;
    Launch H = half_launch(f.m);
    for (int s = 0; s < ns; ++s) {
      // below the finest level the first (red, from zero) half-sweep was
      // done by the restriction
      if (s > 0 || l == 0)
        mg_smooth(dim, H, per, f.m, f.kf, f.idg, f.b, f.x, 0, s == 0, lp, nullptr, 0, 0, ds, st);
      mg_smooth(dim, H, per, f.m, f.kf, f.idg, f.b, f.x, 1, 0, lp, nullptr, 0, 0, ds, st);
    }
    MgLevel& c = mg.lev[l + 1];
    Launch L = cell_launch(c.m);
    const float* cidg = l + 1 < top && ns > 0 ? c.idg : nullptr;
    MG_LAUNCH_P(k_mg_restrict, L, per, f.m, c.m, f.kf, f.dg, f.b, f.x, c.b, c.x, cidg, lp, ds);
  }
  if (mg.top < mg.nlev) {
    MgBlock B;
    B.nl = mg.nlev - mg.top;
    B.nsweep = ns;
    B.coarse_sweeps = mg.coarse_sweeps;
    B.cinv = mg.cdense ? mg.cinv : nullptr;
    B.oc = mg.smem_cinv_off;
    B.pin = mg.top == 0 ? pin : -1;
    int off = 0;
    for (int q = 0; q < B.nl; ++q) {
      const MgLevel& lv = mg.lev[mg.top + q];
      B.m[q] = lv.m;
      B.kf[q] = lv.kf;
      B.idg[q] = lv.idg;
      const int c4 = (int)((lv.m.nc + 3) / 4 * 4), f4 = (int)((lv.m.nf + 3) / 4 * 4);
      B.ox[q] = off; off += c4;
      B.ob[q] = off; off += c4;
      B.oi[q] = off; off += c4;
      B.ok[q] = off; off += f4;
    }
    MgLevel& t = mg.lev[mg.top];
    if (dim == 3) {
      if (per) PDL(k_mg_block_vcycle<3, true>, 1, kBlkThreads, mg.smem_bytes, st, B, t.b, t.x, ds);
      else PDL(k_mg_block_vcycle<3, false>, 1, kBlkThreads, mg.smem_bytes, st, B, t.b, t.x, ds);
    } else {
      if (per) PDL(k_mg_block_vcycle<2, true>, 1, kBlkThreads, mg.smem_bytes, st, B, t.b, t.x, ds);
      else PDL(k_mg_block_vcycle<2, false>, 1, kBlkThreads, mg.smem_bytes, st, B, t.b, t.x, ds);
    }
    count_launches(1);
  } else {
    // large coarsest level (odd dimensions) or a single level: symmetric
    // smoothing only, (red, black)^s then (black, red)^s
    MgLevel& cl = mg.lev[top];
    long long lp = top == 0 ? pin : -1;
    Launch H = half_launch(cl.m);
    const int half = mg.coarse_sweeps_large / 2 > 0 ? mg.coarse_sweeps_large / 2 : 1;
    for (int s = 0; s < half; ++s) {
      mg_smooth(dim, H, per, cl.m, cl.kf, cl.idg, cl.b, cl.x, 0, s == 0, lp, nullptr, 0, 0, ds, st);
      mg_smooth(dim, H, per, cl.m, cl.kf, cl.idg, cl.b, cl.x, 1, 0, lp, nullptr, 0, 0, ds, st);
    }
    for (int s = 0; s < half; ++s) {
      mg_smooth(dim, H, per, cl.m, cl.kf, cl.idg, cl.b, cl.x, 1, 0, lp, nullptr, 0, 0, ds, st);
      mg_smooth(dim, H, per, cl.m, cl.kf, cl.idg, cl.b, cl.x, 0, 0, lp, nullptr, 0, 0, ds, st);
    }
  }
  for (int l = top - 1; l >= (fast0 ? 1 : 0); --l) {
    MgLevel& f = mg.lev[l];
    MgLevel& c = mg.lev[l + 1];
    long long lp = l == 0 ? pin : -1;
    Launch H = half_launch(f.m);
    for (int s = 0; s < ns; ++s) {
      // the first half-sweep adds the coarse correction on the fly
      const float* cx = s == 0 ? c.x : nullptr;
      mg_smooth(dim, H, per, f.m, f.kf, f.idg, f.b, f.x, 1, 0, lp, cx, c.m.n[0], c.m.n[1], ds, st);
      mg_smooth(dim, H, per, f.m, f.kf, f.idg, f.b, f.x, 0, 0, lp, nullptr, 0, 0, ds, st);
    }
  }
  if (fast0) {
    // (black + injected correction, red), (black, red)^(ns-1): z is the
    // colour-blocked iterate itself
    const Launch H = fast0_launch(m0);
    const float* cx = mg.lev[1].x;
    for (int s = 0; s < ns; ++s) {
      if (s == 0)
        PDL(k_mg0_smooth<true>, H.grid, H.block, 0, st, f0, mg.idg0, r, z, 1, cx, ds, H.kch);
      else
        PDL(k_mg0_smooth<false>, H.grid, H.block, 0, st, f0, mg.idg0, r, z, 1, nullptr, ds,
            H.kch);
      PDL(k_mg0_smooth<false>, H.grid, H.block, 0, st, f0, mg.idg0, r, z, 0, nullptr, ds, H.kch);
      count_launches(2);
    }
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t mg_vcycle(MgWork& mg, const float* r, float* z, long long pin, DevScalars* ds,
                      cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cs);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusNone) return mg_vcycle_launch(mg, r, z, pin, ds, st);
  if (!mg.vc_exec || mg.vc_r != r || mg.vc_z != z || mg.vc_pin != pin || mg.vc_ds != ds ||
      mg.vc_fast0 != mg.fast0) {
    mg_release(mg);
    cudaGraph_t g = nullptr;
    if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed)) != cudaSuccess) return e;
    cudaError_t el = mg_vcycle_launch(mg, r, z, pin, ds, st);
    e = cudaStreamEndCapture(st, &g);
    if (el != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return el != cudaSuccess ? el : e;
    }
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    e = cudaGraphInstantiate(&mg.vc_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      mg.vc_exec = nullptr;
      return e;
    }
    // the capture counted its kernels; each replay counts them
    mg.vc_kernels = (int)nodes;
    count_launches(-mg.vc_kernels);
    mg.vc_r = r;
    mg.vc_z = z;
    mg.vc_pin = pin;
    mg.vc_ds = ds;
    mg.vc_fast0 = mg.fast0;
  }
  count_launches(mg.vc_kernels);
  return cudaGraphLaunch(mg.vc_exec, st);
}

void mg_release(MgWork& mg) {
  if (mg.vc_exec) cudaGraphExecDestroy(mg.vc_exec);
  mg.vc_exec = nullptr;
}

cudaError_t cta_pressure(const Mesh& m, const double* kf, const double* f, double* x,
                         int singular, double tol, double inner_min, int limit, int graph,
                         int threads, int cluster, PcgWork& w, MgWork& mg, cudaStream_t st) {
  // (the group passes index cells through FP32 reciprocals: < 2^24 cells)
  if (any_periodic(m) || m.nc >= (1LL << 24) || mg.nlev < 1 || mg.top >= mg.nlev ||
      threads < 32 || threads > 1024 || threads % 32 || cluster < 1 || cluster > 8)
    return cudaErrorInvalidValue;
  CtaPressure P{};
  P.m = m;
  P.kf = kf;
  P.dg = w.dg;
  P.f = f;
  P.x = x;
  P.kf32 = w.kf32;
  P.dg32 = w.dg32;
  P.x32 = w.x32;
  P.r32 = w.r32;
  P.z32 = w.z32;
  P.p = w.p32;
  P.pb = w.p32b;
  P.Ap = w.Ap32;
  P.pin = w.pin;
  P.singular = singular;
  P.limit = limit;
  P.graph = graph;
  P.tol = tol;
  P.inner_min = inner_min;
  P.nl = mg.nlev;
  P.top = mg.top;
  P.nsweep = mg.nsweep;
  P.mtop = mg.lev[mg.top].m;
  P.btop = mg.top == 0 ? w.r32 : mg.lev[mg.top].b;
  P.xtop = mg.top == 0 ? w.z32 : mg.lev[mg.top].x;
  for (int l = 0; l < P.top; ++l) {
    const MgLevel& lv = mg.lev[l];
    P.gm[l] = lv.m;
    P.gkf[l] = l == 0 ? w.kf32 : lv.kf;
    P.gidg[l] = l == 0 ? w.idg32 : lv.idg;
    P.gx[l] = l == 0 ? w.z32 : lv.x;
    P.gb[l] = l == 0 ? w.r32 : lv.b;
  }
  {
    MgBlock& B = P.blk;
    B.nl = mg.nlev - mg.top;
    B.nsweep = mg.nsweep;
    B.coarse_sweeps = mg.coarse_sweeps;
    B.cinv = mg.cdense ? mg.cinv : nullptr;
    B.oc = mg.smem_cinv_off;
    B.pin = mg.top == 0 ? w.pin : -1;
    int off = 0;
    for (int q = 0; q < B.nl; ++q) {
      const MgLevel& lv = mg.lev[mg.top + q];
      B.m[q] = lv.m;
      B.kf[q] = mg.top + q == 0 ? w.kf32 : lv.kf;
      B.idg[q] = mg.top + q == 0 ? w.idg32 : lv.idg;
      const int c4 = (int)((lv.m.nc + 3) / 4 * 4), f4 = (int)((lv.m.nf + 3) / 4 * 4);
      B.ox[q] = off; off += c4;
      B.ob[q] = off; off += c4;
      B.oi[q] = off; off += c4;
      B.ok[q] = off; off += f4;
    }
  }
  for (int l = 0; l < mg.nlev; ++l) {
    P.lkf[l] = l == 0 ? w.kf32 : mg.lev[l].kf;
    P.lidg[l] = l == 0 ? w.idg32 : mg.lev[l].idg;
  }
  P.idg32 = w.idg32;
  P.cinv = mg.cdense ? mg.cinv : nullptr;
  P.ds = w.ds;
  const int smem = mg.smem_bytes;
  if (cluster == 1) {
    if (m.dim == 3) k_cta_pressure<3, CtaG><<<1, threads, smem, st>>>(P);
    else k_cta_pressure<2, CtaG><<<1, threads, smem, st>>>(P);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = m.dim == 3 ? cudaLaunchKernelEx(&cfg, k_cta_pressure<3, ClusterG>, P)
                               : cudaLaunchKernelEx(&cfg, k_cta_pressure<2, ClusterG>, P);
    if (e != cudaSuccess) return e;
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t mgcg_init(const Mesh& m, double tol, int dev_params, PcgWork& w, MgWork& mg,
                      cudaStream_t st) {
  int fb = flat_blocks_mg(m.nc);
  if (!aligned16(w.r) || !aligned16(w.r32) || !aligned16(w.x32) || !aligned16(w.z32) ||
      !aligned16(w.p32) || !aligned16(w.p32b) || !aligned16(w.Ap32))
    return cudaErrorInvalidValue;
  w.p32_parity = 0;
  if (mg.fast0) {
    const Fast0 f{m.n[0], m.n[1], m.n[2], mg.k16[0], mg.k16[1], mg.k16[2]};
    PDL(k_mgcg_init_blk, flat_blocks_mg(m.nc / 2), dim3(BX, BY), 0, st, f, w.r, w.r32, w.x32,
        tol, w.limit, dev_params, w.partials, w.ds);
  } else {
    PDL(k_mgcg_init, fb, dim3(BX, BY), 0, st, m.nc, w.r, w.r32, w.x32, tol, w.limit,
        dev_params, w.partials, w.ds);
  }
  count_launches(1);
  if (w.prof) w.prof->begin(HYDRO_PROF_MG_VCYCLE, st);
  cudaError_t e = mg_vcycle(mg, w.r32, w.z32, w.pin, w.ds, st);
  if (w.prof) w.prof->end(HYDRO_PROF_MG_VCYCLE, st);
  if (e != cudaSuccess) return e;
  PDL(k_mgcg_dot, fb, dim3(BX, BY), 0, st, m.nc, w.r32, w.z32, 1, w.partials, w.ds);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t mgcg_iterate(const Mesh& m, int chunk, PcgWork& w, MgWork& mg, cudaStream_t st) {
  int fb = flat_blocks_mg(m.nc);
  for (int it = 0; it < chunk; ++it) {
    float* pold = (w.p32_parity & 1) ? w.p32b : w.p32;
    float* pnew = (w.p32_parity & 1) ? w.p32 : w.p32b;
    if (w.prof) w.prof->begin(HYDRO_PROF_CG_SPMV, st);
    cudaError_t e;
    if (mg.fast0) {
      const Fast0 f{m.n[0], m.n[1], m.n[2], mg.k16[0], mg.k16[1], mg.k16[2]};
      Mesh hm = m;  // one thread per cell pair
      hm.n[0] = m.n[0] / 2;
      const Launch H = cell_launch_waves(hm, resident_ctas((const void*)k_cg32_dir_spmv_blk));
      PDL(k_cg32_dir_spmv_blk, H.grid, H.block, 0, st, f, w.kf32, w.dg32, w.z32, pold, pnew,
          w.Ap32, (int)m.fofs[1], (int)m.fofs[2], w.partials, w.ds, H.kch);
      count_launches(1);
      e = cudaGetLastError();
    } else {
      e = cg32_dir_spmv(m, w.kf32, w.dg32, w.z32, pold, pnew, w.Ap32, w.pin, w.partials, w.ds,
                        st);
    }
    if (w.prof) w.prof->end(HYDRO_PROF_CG_SPMV, st);
    if (e != cudaSuccess) return e;
    if (w.prof) w.prof->begin(HYDRO_PROF_CG_UPDATE, st);
    PDL(k_mgcg_update, fb, dim3(BX, BY), 0, st, m.nc, w.x32, w.r32, pnew, w.Ap32, w.partials,
        w.ds);
    if (w.prof) w.prof->end(HYDRO_PROF_CG_UPDATE, st);
    if (w.prof) w.prof->begin(HYDRO_PROF_MG_VCYCLE, st);
    e = mg_vcycle(mg, w.r32, w.z32, w.pin, w.ds, st);
    if (w.prof) w.prof->end(HYDRO_PROF_MG_VCYCLE, st);
    if (e != cudaSuccess) return e;
    PDL(k_mgcg_dot, fb, dim3(BX, BY), 0, st, m.nc, w.r32, w.z32, 0, w.partials, w.ds);
    count_launches(2);
    w.p32_parity ^= 1;
  }
  return cudaGetLastError();
}

cudaError_t mgcg_accumulate(const Mesh& m, double* x, PcgWork& w, MgWork& mg, cudaStream_t st) {
  if (!mg.fast0) return f32_accumulate(m, x, w, st);
  const Fast0 f{m.n[0], m.n[1], m.n[2], mg.k16[0], mg.k16[1], mg.k16[2]};
  PDL(k_accumulate_blk, flat_blocks_mg(m.nc / 2), NT, 0, st, f, x, w.x32);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace hg
