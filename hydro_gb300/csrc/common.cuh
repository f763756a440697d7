// common.cuh -- mesh indexing, launch geometry and deterministic reductions
// shared by the sm_103a kernels of the hydro hot path.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "fpconv.h"

namespace hg {

// Widening / narrowing between a kernel's arithmetic type and FP64 through
// the integer-pipe conversions (fpconv.h); identities for FP64 kernels.
__device__ __forceinline__ double to_d(float v) { return f2d(v); }
__device__ __forceinline__ double to_d(double v) { return v; }
template <class T>
__device__ __forceinline__ T to_t(double v);
template <>
__device__ __forceinline__ float to_t<float>(double v) { return d2f(v); }
template <>
__device__ __forceinline__ double to_t<double>(double v) { return v; }

// Uniform Cartesian block.  Cells: i + nx*(j + ny*k); faces direction-
// blocked, x-fastest over (n_d+1) in their own direction (the reference's
// raw order, mesh.hpp:552-561 and 640-720).  Geometry is implicit:
// h_d = (B_d - A_d)/N_d, V = prod h, A_d = V/h_d (InitUniformMesh,
// mesh.hpp:722-736).
struct Mesh {
  int dim;
  int n[3];
  long long nc, nf;
  long long fofs[3];  // first face of each direction block
  int fnx[3], fny[3]; // x/y extents of each direction block
  double h[3], V, A[3];
  double lo[3];
  int per[3];         // periodic directions: cells n-1 and 0 are neighbours
  // excluded cells (rigid box, mesh3d.hpp:183-215), device mask, null for
  // none: a face touching an excluded cell is not inner; nfluid = cells
  // not excluded
  const unsigned char* ex;
  long long nfluid;
};

__host__ __device__ inline long long cell_id(const Mesh& m, int i, int j, int k) {
  return i + (long long)m.n[0] * (j + (long long)m.n[1] * k);
}
__host__ __device__ inline long long face_id(const Mesh& m, int d, int i, int j, int k) {
  return m.fofs[d] + i + (long long)m.fnx[d] * (j + (long long)m.fny[d] * k);
}
// stride between neighbouring cells along d
__host__ __device__ inline long long cell_stride(const Mesh& m, int d) {
  return d == 0 ? 1 : (d == 1 ? (long long)m.n[0] : (long long)m.n[0] * m.n[1]);
}
// stride between the low and high face of a cell along d
__host__ __device__ inline long long face_stride(const Mesh& m, int d) {
  return d == 0 ? 1 : (d == 1 ? (long long)m.fnx[1] : (long long)m.fnx[2] * m.fny[2]);
}

// Neighbours along d of the cell c with index i along d (s = cell_stride).
// A neighbour exists inside the block, or across the end of a periodic
// direction (both end faces then join cells n-1 and 0, mesh3d.hpp:348-392),
// unless the cell or the neighbour is excluded.  P is a compile-time
// switch: kernels are instantiated with P = false for plain blocks (no
// periodic direction, no excluded cell), where these reduce to the bounds
// test and c -/+ s (no wrap or mask arithmetic in the hot loops).
// (I: the index type of the caller, int inside one CTA's shared memory)
template <bool P, class I>
__host__ __device__ inline I nb_lo_p(const Mesh& m, int d, int i, I c, I s) {
  return (!P || i > 0) ? c - s : c + (I)(m.n[d] - 1) * s;
}
template <bool P, class I>
__host__ __device__ inline I nb_hi_p(const Mesh& m, int d, int i, I c, I s) {
  return (!P || i < m.n[d] - 1) ? c + s : c - (I)(m.n[d] - 1) * s;
}
template <bool P, class I>
__host__ __device__ inline bool has_lo_p(const Mesh& m, int d, int i, I c, I s) {
  if (!P) return i > 0;
  if (!(i > 0 || m.per[d])) return false;
  return !m.ex || !(m.ex[c] || m.ex[nb_lo_p<P>(m, d, i, c, s)]);
}
template <bool P, class I>
__host__ __device__ inline bool has_hi_p(const Mesh& m, int d, int i, I c, I s) {
  if (!P) return i < m.n[d] - 1;
  if (!(i < m.n[d] - 1 || m.per[d])) return false;
  return !m.ex || !(m.ex[c] || m.ex[nb_hi_p<P>(m, d, i, c, s)]);
}
__host__ __device__ inline bool has_lo(const Mesh& m, int d, int i, long long c, long long s) {
  return has_lo_p<true, long long>(m, d, i, c, s);
}
__host__ __device__ inline bool has_hi(const Mesh& m, int d, int i, long long c, long long s) {
  return has_hi_p<true, long long>(m, d, i, c, s);
}
__host__ __device__ inline long long nb_lo(const Mesh& m, int d, int i, long long c, long long s) {
  return nb_lo_p<true, long long>(m, d, i, c, s);
}
__host__ __device__ inline long long nb_hi(const Mesh& m, int d, int i, long long c, long long s) {
  return nb_hi_p<true, long long>(m, d, i, c, s);
}
// is the cell excluded (general instantiations only)
template <bool P, class I>
__host__ __device__ inline bool excluded_p(const Mesh& m, I c) {
  return P && m.ex && m.ex[c];
}
// Kernels take their general instantiation for periodic directions or
// excluded cells.
inline bool any_periodic(const Mesh& m) {
  if (m.ex) return true;
  for (int d = 0; d < m.dim; ++d)
    if (m.per[d]) return true;
  return false;
}

// Programmatic dependent launch: a kernel launched with pdl() may be
// scheduled onto SMs while the kernel before it in the stream drains.  Such
// a kernel calls pdl_wait() before its first memory access -- it returns
// once the previous kernel has completed and its writes are visible, so the
// dependency is that of a plain launch -- and pdl_trigger() to let the next
// one be scheduled in turn (it takes effect once every CTA of this kernel
// has started or exited, so waiting CTAs never displace this kernel's
// own).  What overlaps is the launch latency between dependent kernels:
// a few microseconds each in the chains of small multigrid and Krylov
// kernels.  Both are no-ops for a plain launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <class... P, class... A>
inline cudaError_t pdl(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       A&&... a) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<A>(a)...);
}
// pdl() whose error, like a <<<>>> launch's, is left to cudaGetLastError
#define PDL(...) ((void)pdl(__VA_ARGS__))


// Thread groups of the in-CTA helpers: one CTA (__syncthreads) or one
// thread-block cluster (its CTAs' threads numbered CTA-major; the cluster
// barrier also orders the CTAs' global-memory accesses).
struct CtaG {
  __device__ int rank() const { return threadIdx.x; }
  __device__ int size() const { return blockDim.x; }
  __device__ void sync() const { __syncthreads(); }
};
struct ClusterG {
  int r, n;
  // parity of the cluster-wide reductions so far (their shared-memory
  // slots are double-buffered); every thread runs the same sequence
  mutable int par = 0;
  __device__ ClusterG()
      : r((int)(cooperative_groups::this_cluster().block_rank() * blockDim.x + threadIdx.x)),
        n((int)(cooperative_groups::this_cluster().num_blocks() * blockDim.x)) {}
  __device__ int rank() const { return r; }
  __device__ int size() const { return n; }
  __device__ void sync() const { cooperative_groups::this_cluster().sync(); }
};

// Launch geometry: blocks of 32x8 threads over (i, j); each block marches
// KCH planes in k so that the grid stays a few waves deep on 152 SMs.
constexpr int BX = 32, BY = 8, NT = BX * BY;

struct Launch {
  dim3 grid, block;
  int kch;
  int nblocks() const { return grid.x * grid.y * grid.z; }
};

inline Launch cell_launch(const Mesh& m, int target_blocks = 152 * 16) {
  Launch L;
  L.block = dim3(BX, BY, 1);
  int gx = (m.n[0] + BX - 1) / BX, gy = (m.n[1] + BY - 1) / BY;
  int nz = m.dim == 3 ? m.n[2] : 1;
  int per = gx * gy;
  int gz = (target_blocks + per - 1) / per;
  if (gz > nz) gz = nz;
  if (gz < 1) gz = 1;
  L.kch = (nz + gz - 1) / gz;
  gz = (nz + L.kch - 1) / L.kch;
  L.grid = dim3(gx, gy, gz);
  return L;
}

// CTAs of `kernel` (NT threads, no dynamic shared memory) resident on the
// whole GPU at once; queried once per kernel.
int resident_ctas(const void* kernel);

// Cell launch sized in whole waves: a CTA marches kch planes, and a grid of
// C CTAs with R resident takes ceil(C / R) rounds of kch planes plus a
// fixed cost per CTA (start, block reduction: about two planes); among the
// grids that fill the GPU at least once, the cheapest (ties: fewer CTAs),
// so that no nearly empty last wave holds the whole GPU for a full march.
inline Launch cell_launch_waves(const Mesh& m, int resident) {
  Launch L = cell_launch(m);
  if (resident <= 0) return L;
  const int nz = m.dim == 3 ? m.n[2] : 1;
  const long long per = (long long)L.grid.x * L.grid.y;
  if (per * nz < resident) return L;
  long long best = -1;
  for (int gz = 1; gz <= nz; ++gz) {
    const int kch = (nz + gz - 1) / gz;
    if ((nz + kch - 1) / kch != gz) continue;  // same march as a smaller grid
    if (per * gz < resident) continue;
    if (per * gz > (1 << 17)) break;
    const long long cost = (per * gz + resident - 1) / resident * (kch + 2);
    if (best < 0 || cost < best) {
      best = cost;
      L.kch = kch;
      L.grid.z = (unsigned)gz;
    }
  }
  return L;
}

// ------------------------------------------------------------ reductions --
// Deterministic grid reduction: every block writes its partial, the last
// block to arrive (atomic ticket) combines the partials in index order and
// runs the finaliser.  The ticket is reset for the next launch.

template <class T>
__device__ inline T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
template <class T>
__device__ inline T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
template <class T>
__device__ inline T warp_min(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

enum RedOp { RED_SUM = 0, RED_MAX = 1, RED_MIN = 2 };

template <int OP, class T>
__device__ inline T red_combine(T a, T b) {
  if (OP == RED_SUM) return a + b;
  if (OP == RED_MAX) return a > b ? a : b;
  return a < b ? a : b;
}
template <int OP, class T>
__device__ inline T warp_red(T v) {
  if (OP == RED_SUM) return warp_sum(v);
  if (OP == RED_MAX) return warp_max(v);
  return warp_min(v);
}

// Block reduction of NV values; result valid in thread 0.
template <int OP, int NV, class T>
__device__ inline void block_reduce(T (&v)[NV], T* sh /* [NV][32] */) {
  int tid = threadIdx.x + blockDim.x * threadIdx.y;
  int lane = tid & 31, wid = tid >> 5;
  int nw = (blockDim.x * blockDim.y + 31) >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) v[a] = warp_red<OP>(v[a]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) sh[a * 32 + wid] = v[a];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      T x = lane < nw ? sh[a * 32 + lane] : (OP == RED_SUM ? T(0) : sh[a * 32]);
      v[a] = warp_red<OP>(x);
    }
  }
}

// Writes this block's NV partials; returns true in the (single) last block,
// whose thread 0..NT-1 then see `out` = the reduced values in shared memory.
// partials layout: [NV][nblocks].
template <int OP, int NV, class T>
__device__ inline bool grid_reduce(T (&v)[NV], T* partials, unsigned* ticket, T* out_sh) {
  __shared__ T sh[NV * 32];
  __shared__ bool last;
  block_reduce<OP, NV>(v, sh);
  int tid = threadIdx.x + blockDim.x * threadIdx.y;
  int nthr = blockDim.x * blockDim.y;
  unsigned nb = gridDim.x * gridDim.y * gridDim.z;
  unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  if (tid == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) partials[(size_t)a * nb + bid] = v[a];
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    last = (t == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // fixed-order combine: thread t folds partials t, t+nthr, ... in order,
  // then a fixed tree over threads.  The partials are read from L2 (ld.cg:
  // written by other blocks, made visible by their fences), eight in flight
  // per thread before they are folded.
  T acc[NV];
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    const T* pa = partials + (size_t)a * nb;
    T x = (OP == RED_SUM) ? T(0) : __ldcg(pa);
    unsigned b = tid;
    for (; b + 7u * nthr < nb; b += 8u * nthr) {
      T y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = __ldcg(pa + b + u * nthr);
#pragma unroll
      for (int u = 0; u < 8; ++u) x = red_combine<OP>(x, y[u]);
    }
    for (; b < nb; b += nthr) x = red_combine<OP>(x, __ldcg(pa + b));
    acc[a] = x;
  }
  block_reduce<OP, NV>(acc, sh);
  if (tid == 0) {
#pragma unroll
    for (int a = 0; a < NV; ++a) out_sh[a] = acc[a];
    *ticket = 0u;
  }
  __syncthreads();
  return true;
}

}  // namespace hg
