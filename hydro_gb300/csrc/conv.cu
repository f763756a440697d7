// conv.cu -- 3x3x3 convolutions of the learned pressure guess on the 5th-
// generation tensor cores: BF16 operands, FP32 accumulation in tensor memory.
//
// Activations are BF16, channels-last: [batch][z][y][x][C], C in {16, 32, 64}
// (the network's two input channels are padded to 16).  A convolution is an
// implicit GEMM over a tile of 8 x 16 x 4 output positions (x, y, z): four
// M = 128 row blocks (one per z-plane) that share one halo tile of the input.
//
//  * forward / backward-data (k_conv): the halo tile (10 x 18 x 6 positions,
//    every 8-channel chunk in its own region of 16-byte rows) is loaded by TMA
//    (cp.async.bulk.tensor, zero fill outside the grid); the 27 taps are 27
//    views into it -- the A operand of tap (dx, dy, dz) starts dx + 10 dy +
//    180 dz rows into the tile, with its 8-row core matrices 10 rows (160 B)
//    apart -- so the input crosses HBM once per tile, not 27 times.  The
//    weights of one tap ([ci/8][co][8] BF16, K-major) are bulk copies: all
//    27 resident for the 16/32-channel layers, else a ring of 9 (or 3).  One thread issues tcgen05.mma
//    (M = 128, N = Cout, K = 16) into four accumulators of Cout columns in
//    TMEM; the four warps read them back with tcgen05.ld and apply the
//    epilogue (bias, addend, ReLU, mask) before a 16-byte-vector store.
//    Backward-data is the same kernel with the taps mirrored and the
//    weight's channel roles swapped.
//  * weight gradient (k_conv_wgrad): dW[tap][co][ci] = sum_p g[p][co]
//    x[p + off(tap)][ci] is a GEMM with K = positions: A = g^T (M = co, K = p)
//    and B = the shifted halo view (N = ci, K = p), both MN-major.  g is
//    staged by the threads in the MN-major core-matrix layout; rows of A past
//    Cout read other staged rows (their accumulator rows are never read).  A
//    persistent CTA accumulates its tiles in TMEM and adds its partial
//    gradient to the global FP32 gradient once.
//
// Every wait on an mbarrier is bounded; a wait that runs out sets *err,
// waits (bounded) for the copies this CTA has in flight, frees its tensor
// memory and returns.  No multicast, no clusters: one GPU's own memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "conv.h"

namespace hg {
namespace nn {

namespace {

// Weight stages of the forward kernel: all 27 taps resident in shared
// memory when they take at most 28 KB (the 16- and 32-channel layers of the
// finest levels: no wait on the tensor pipe between taps), else a ring of 9
// (a bulk copy's latency is hidden behind the MMAs of 8 taps) where the
// shared memory allows, else 3.
constexpr int stages_for(int cin, int cout) {
  return 27 * cin * cout * 2 <= 28 * 1024                          ? 27
         : (cin / 8) * kRegion + 9 * cin * cout * 2 <= 212 * 1024 ? 9
                                                                   : 3;
}
constexpr long kWaitPolls = 1L << 24;      // bounded mbarrier waits (~1 s)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase `parity` of an mbarrier; false (and *err set)
// when it did not complete within the bound.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (long i = 0; i < kWaitPolls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 32) __nanosleep(64);
  }
  if (err) atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4),
      "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor, no swizzle: start address, the byte
// distance between core matrices along K (lbo) and along M/N (sbo).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the sm_100 family
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 accumulator.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
         ((b_mn ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr uint32_t tmem_cols(int n) {
  uint32_t c = 32;
  while (c < (uint32_t)n) c <<= 1;
  return c;
}

__device__ __forceinline__ unsigned char* align1024(unsigned char* p) {
  return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 1023) &
                                          ~uintptr_t(1023));
}

__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }

}  // namespace

// ------------------------------------------------------------ forward --
// out[p][co] = epi(sum_tap sum_ci x[p + off(tap)][ci] w[tap][co][ci]).
// w: [27][CIN/8][COUT][8] BF16 (K-major core matrices per tap).
template <int CIN, int COUT, int kNStage>
__global__ void __launch_bounds__(128) k_conv(const __grid_constant__ CUtensorMap xin,
                                              ConvDims dm, const __nv_bfloat16* __restrict__ w,
                                              Epilogue ep, __nv_bfloat16* __restrict__ out,
                                              int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = align1024(smem_raw);
  constexpr int NCH = CIN / 8;
  constexpr uint32_t WB = CIN * COUT * 2;
  constexpr uint32_t NCOLS = tmem_cols(kTZ * COUT);
  unsigned char* halo = sm;
  unsigned char* wring = halo + NCH * kRegion;
  uint64_t* bars = reinterpret_cast<uint64_t*>(wring + kNStage * WB);
  uint64_t* bar_halo = bars;
  uint64_t* bar_full = bars + 1;
  uint64_t* bar_empty = bars + 1 + kNStage;
  uint64_t* bar_done = bars + 1 + 2 * kNStage;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 + 2 * kNStage);
  float* sbias = reinterpret_cast<float*>(tslot + 4);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int tiles_z = (dm.nz + kTZ - 1) / kTZ;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int b = blockIdx.z / tiles_z, z0 = (blockIdx.z % tiles_z) * kTZ;

  if (tid < COUT) sbias[tid] = ep.bias ? ep.bias[tid] : 0.f;
  if (tid == 0) {
    mbar_init(bar_halo, 1);
    for (int s = 0; s < kNStage; ++s) {
      mbar_init(&bar_full[s], 1);
      mbar_init(&bar_empty[s], 1);
    }
    mbar_init(bar_done, 1);
    fence_barrier_init();
  }
  __syncwarp();
  if (warp == 0) tmem_alloc(tslot, NCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (tid == 0) {
    bool ok = true;
    int loaded = 0;  // weight taps whose copy was issued
    mbar_expect_tx(bar_halo, (uint32_t)NCH * kHRows * 16);
    for (int c = 0; c < NCH; ++c)
      tma_load_5d(halo + c * kRegion, &xin, bar_halo, c * 8, x0 - 1, y0 - 1, z0 - 1, b);
    for (int s = 0; s < kNStage; ++s) {
      mbar_expect_tx(&bar_full[s], WB);
      bulk_load(wring + s * WB, w + (size_t)s * (WB / 2), WB, &bar_full[s]);
      ++loaded;
    }
    ok = mbar_wait(bar_halo, 0, err);
    constexpr uint32_t idesc = idesc_bf16(128, COUT, false, false);
    const uint32_t hbase = smem_u32(halo), wbase = smem_u32(wring);
    int done_taps = 0;  // taps whose MMAs were issued and committed
    for (int t = 0; t < 27 && ok; ++t) {
      const int s = t % kNStage;
      if (!(ok = mbar_wait(&bar_full[s], (t / kNStage) & 1, err))) break;
      tc_fence_after();
      const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
#pragma unroll
      for (int mz = 0; mz < kTZ; ++mz) {
        const uint32_t row0 = dx + kHX * dy + kHX * kHY * (mz + dz);
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc) {
          const uint64_t a = sdesc(hbase + (2 * kc) * kRegion + row0 * 16, kRegion, kHX * 16);
          const uint64_t bd = sdesc(wbase + s * WB + (2 * kc) * COUT * 16, COUT * 16, 128);
          mma_bf16(tmem + mz * COUT, a, bd, idesc, (t | kc) ? 1u : 0u);
        }
      }
      mma_commit(&bar_empty[s]);
      ++done_taps;
      if (t >= 1 && t - 1 + kNStage < 27) {
        // tap t is queued behind tap t-1: once t-1 has read its stage,
        // refill that stage with tap t-1+kNStage
        const int sp = (t - 1) % kNStage;
        if (!(ok = mbar_wait(&bar_empty[sp], ((t - 1) / kNStage) & 1, err))) break;
        mbar_expect_tx(&bar_full[sp], WB);
        bulk_load(wring + sp * WB, w + (size_t)(t - 1 + kNStage) * (WB / 2), WB, &bar_full[sp]);
        ++loaded;
      }
    }
    mma_commit(bar_done);
    if (!ok) {
      // drain: every weight copy issued must land before the CTA exits
      for (int t = done_taps; t < loaded; ++t)
        mbar_wait(&bar_full[t % kNStage], (t / kNStage) & 1, nullptr);
      mbar_wait(bar_halo, 0, nullptr);
    }
  }
  __syncwarp();
  const bool okd = mbar_wait(bar_done, 0, err);
  __syncwarp();
  tc_fence_after();
  // epilogue: warp w reads TMEM lanes 32w..32w+31 = rows of the M block
  const int r = tid;
  const int xx = x0 + (r % kTX), yy = y0 + (r / kTX);
#pragma unroll 1
  for (int mz = 0; mz < kTZ; ++mz) {
    const int zz = z0 + mz;
    const bool in = okd && xx < dm.nx && yy < dm.ny && zz < dm.nz;
    const size_t pos = (((size_t)b * dm.nz + zz) * dm.ny + yy) * dm.nx + xx;
#pragma unroll
    for (int j = 0; j < COUT / 16; ++j) {
      float v[16];
      __syncwarp();
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + mz * COUT + 16 * j, v);
      if (!in) continue;
      const size_t base = pos * COUT + 16 * j;
      if (ep.addend) {
        const uint4* ap = reinterpret_cast<const uint4*>(ep.addend + base);
        uint4 q[2] = {ap[0], ap[1]};
        const __nv_bfloat16* a16 = reinterpret_cast<const __nv_bfloat16*>(q);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += bf(a16[i]);
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        v[i] += sbias[16 * j + i];
        if (ep.relu) v[i] = fmaxf(v[i], 0.f);
      }
      if (ep.mask) {
        const uint4* mp = reinterpret_cast<const uint4*>(ep.mask + base);
        uint4 q[2] = {mp[0], mp[1]};
        const __nv_bfloat16* m16 = reinterpret_cast<const __nv_bfloat16*>(q);
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (!(bf(m16[i]) > 0.f)) v[i] = 0.f;
      }
      uint4 o[2];
      __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(o);
#pragma unroll
      for (int i = 0; i < 8; ++i) o2[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
      uint4* op = reinterpret_cast<uint4*>(out + base);
      op[0] = o[0];
      op[1] = o[1];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, NCOLS);
}

// ----------------------------------------------------- weight gradient --
// dw[tap][co][ci] += sum_p g[p][co] x[p + off(tap)][ci] over the tiles this
// persistent CTA takes (blockIdx.x, stride gridDim.x) for the taps
// [blockIdx.y * TPP, ...) of its pass.  dw: FP32 [27][COUT][CIN].
template <int CIN, int COUT, int TPP>
__global__ void __launch_bounds__(128) k_conv_wgrad(const __grid_constant__ CUtensorMap xin,
                                                    ConvDims dm,
                                                    const __nv_bfloat16* __restrict__ g,
                                                    float* __restrict__ dw, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = align1024(smem_raw);
  constexpr int NCH = CIN / 8;
  constexpr int GCH = COUT / 8;
  constexpr uint32_t NCOLS = tmem_cols(TPP * CIN);
  constexpr int GBYTES = kTZ * kTY * GCH * 128 + 2048;  // + rows past COUT read by M = 128
  unsigned char* halo = sm;
  unsigned char* gbuf = halo + NCH * kRegion;
  uint64_t* bars = reinterpret_cast<uint64_t*>(gbuf + GBYTES);
  uint64_t* bar_halo = bars;
  uint64_t* bar_mma = bars + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int tap0 = blockIdx.y * TPP;
  const int ntap = min(TPP, 27 - tap0);
  const int tx = (dm.nx + kTX - 1) / kTX, ty = (dm.ny + kTY - 1) / kTY;
  const int tz = (dm.nz + kTZ - 1) / kTZ;
  const int ntiles = tx * ty * tz * dm.nb;

  if (tid == 0) {
    mbar_init(bar_halo, 1);
    mbar_init(bar_mma, 1);
    fence_barrier_init();
  }
  // the tail of the staging buffer (read by the accumulator rows past COUT)
  for (int i = tid; i < 2048 / 16; i += 128)
    reinterpret_cast<uint4*>(gbuf + GBYTES - 2048)[i] = make_uint4(0, 0, 0, 0);
  __syncwarp();
  if (warp == 0) tmem_alloc(tslot, NCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  constexpr uint32_t idesc = idesc_bf16(128, CIN, true, true);
  __shared__ int s_ok;
  bool ok = true;
  int ncommit = 0;  // commits of bar_mma (one per tile that was started)
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int rem = tile;
    const int bx = rem % tx;
    rem /= tx;
    const int by = rem % ty;
    rem /= ty;
    const int bz = rem % tz;
    const int b = rem / tz;
    const int x0 = bx * kTX, y0 = by * kTY, z0 = bz * kTZ;
    if (ncommit > 0) {
      // the previous tile's MMAs read both buffers: wait before refilling
      const bool w = mbar_wait(bar_mma, (ncommit - 1) & 1, err);
      tc_fence_after();
      if (!__syncthreads_and(w)) {
        ok = false;
        break;
      }
    }
    if (tid == 0) {
      mbar_expect_tx(bar_halo, (uint32_t)NCH * kHRows * 16);
      for (int c = 0; c < NCH; ++c)
        tma_load_5d(halo + c * kRegion, &xin, bar_halo, c * 8, x0 - 1, y0 - 1, z0 - 1, b);
    }
    // stage g: A[m = co][k = p], 8 positions x 8 channels per core matrix,
    // core matrices of one K group (8 positions) 128 B apart along co
    for (int q = tid; q < kTZ * kTY * kTX * GCH; q += 128) {
      const int cc = q % GCH;
      const int pp = q / GCH;
      const int xl = pp % kTX, yl = (pp / kTX) % kTY, zl = pp / (kTX * kTY);
      const int xx = x0 + xl, yy = y0 + yl, zz = z0 + zl;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (xx < dm.nx && yy < dm.ny && zz < dm.nz)
        v = *reinterpret_cast<const uint4*>(
            g + ((((size_t)b * dm.nz + zz) * dm.ny + yy) * dm.nx + xx) * COUT + cc * 8);
      *reinterpret_cast<uint4*>(gbuf + ((zl * kTY + yl) * GCH + cc) * 128 + xl * 16) = v;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      bool okh = mbar_wait(bar_halo, ncommit & 1, err);
      tc_fence_after();
      if (okh) {
        const uint32_t hbase = smem_u32(halo), gbase = smem_u32(gbuf);
        for (int mz = 0; mz < kTZ; ++mz)
          for (int ky = 0; ky < kTY / 2; ++ky) {
            const uint64_t a =
                sdesc(gbase + ((mz * kTY + 2 * ky) * GCH) * 128, GCH * 128, 128);
            const uint32_t acc = (ncommit > 0 || mz > 0 || ky > 0) ? 1u : 0u;
            for (int tt = 0; tt < ntap; ++tt) {
              const int t = tap0 + tt;
              const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
              const uint32_t row0 = dx + kHX * (2 * ky + dy) + kHX * kHY * (mz + dz);
              const uint64_t bd = sdesc(hbase + row0 * 16, kHX * 16, kRegion);
              mma_bf16(tmem + tt * CIN, a, bd, idesc, acc);
            }
          }
      } else {
        mbar_wait(bar_halo, ncommit & 1, nullptr);  // drain the copy before leaving
      }
      mma_commit(bar_mma);
      s_ok = okh ? 1 : 0;
    }
    ++ncommit;
    __syncthreads();
    if (!s_ok) {
      ok = false;
      break;
    }
  }
  // the last commit covers every MMA: then the accumulators are complete
  if (ncommit > 0) {
    const bool okd = mbar_wait(bar_mma, (ncommit - 1) & 1, err);
    __syncwarp();
    tc_fence_after();
    if (ok && okd && warp * 32 < COUT) {
      const int co = warp * 32 + (tid & 31);
      for (int tt = 0; tt < ntap; ++tt)
#pragma unroll
        for (int j = 0; j < CIN / 16; ++j) {
          float v[16];
          __syncwarp();
          tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + tt * CIN + 16 * j, v);
          if (co < COUT) {
            float* dst = dw + ((size_t)(tap0 + tt) * COUT + co) * CIN + 16 * j;
#pragma unroll
            for (int i = 0; i < 16; ++i) atomicAdd(dst + i, v[i]);
          }
        }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, NCOLS);
}

// ------------------------------------------------------------- host ------
namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

int fwd_smem(int cin, int cout) {
  const int ns = stages_for(cin, cout);
  return 1024 + (cin / 8) * kRegion + ns * cin * cout * 2 + 8 * (3 + 2 * ns) + 16 + 4 * 64;
}

int wgrad_smem(int cin, int cout) {
  return 1024 + (cin / 8) * kRegion + kTZ * kTY * (cout / 8) * 128 + 2048 + 64;
}

template <int CIN, int COUT>
cudaError_t run_conv(const CUtensorMap& map, ConvDims dm, const __nv_bfloat16* w, Epilogue ep,
                     __nv_bfloat16* out, int* err, cudaStream_t st) {
  constexpr int NS = stages_for(CIN, COUT);
  const int smem = fwd_smem(CIN, COUT);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv<CIN, COUT, NS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid((dm.nx + kTX - 1) / kTX, (dm.ny + kTY - 1) / kTY,
            ((dm.nz + kTZ - 1) / kTZ) * dm.nb);
  k_conv<CIN, COUT, NS><<<grid, 128, smem, st>>>(map, dm, w, ep, out, err);
  return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t run_wgrad(const CUtensorMap& map, ConvDims dm, const __nv_bfloat16* g, float* dw,
                      int* err, int sms, cudaStream_t st) {
  constexpr int TPP = (27 * CIN <= 512) ? 27 : 512 / CIN;
  constexpr int NPASS = (27 + TPP - 1) / TPP;
  const int smem = wgrad_smem(CIN, COUT);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad<CIN, COUT, TPP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long ntiles = (long)((dm.nx + kTX - 1) / kTX) * ((dm.ny + kTY - 1) / kTY) *
                      ((dm.nz + kTZ - 1) / kTZ) * dm.nb;
  // one CTA per SM holds a full TMEM: spread the passes and tiles over the SMs
  long per_pass = sms / NPASS;
  if (per_pass < 1) per_pass = 1;
  if (per_pass > ntiles) per_pass = ntiles;
  dim3 grid((unsigned)per_pass, NPASS);
  k_conv_wgrad<CIN, COUT, TPP><<<grid, 128, smem, st>>>(map, dm, g, dw, err);
  return cudaGetLastError();
}

}  // namespace

int make_act_map(CUtensorMap* map, const void* base, ConvDims dm, int c) {
  EncodeTiled enc = encoder();
  if (!enc) return 1;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || c % 8) return 2;
  cuuint64_t dims[5] = {(cuuint64_t)c, (cuuint64_t)dm.nx, (cuuint64_t)dm.ny, (cuuint64_t)dm.nz,
                        (cuuint64_t)dm.nb};
  cuuint64_t strides[4] = {(cuuint64_t)c * 2, (cuuint64_t)c * 2 * dm.nx,
                           (cuuint64_t)c * 2 * dm.nx * dm.ny,
                           (cuuint64_t)c * 2 * dm.nx * dm.ny * dm.nz};
  cuuint32_t box[5] = {8, kHX, kHY, kHZ, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims,
                   strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : 3;
}

cudaError_t conv3d(const CUtensorMap& xmap, ConvDims dm, int cin, int cout,
                   const __nv_bfloat16* w, Epilogue ep, __nv_bfloat16* out, int* err,
                   cudaStream_t st) {
#define HG_CONV(A, B) \
  if (cin == A && cout == B) return run_conv<A, B>(xmap, dm, w, ep, out, err, st);
  HG_CONV(16, 16) HG_CONV(16, 32) HG_CONV(32, 16) HG_CONV(32, 32) HG_CONV(32, 64)
  HG_CONV(64, 32) HG_CONV(64, 64) HG_CONV(64, 16) HG_CONV(16, 64)
#undef HG_CONV
  return cudaErrorInvalidValue;
}

cudaError_t conv3d_wgrad(const CUtensorMap& xmap, ConvDims dm, int cin, int cout,
                         const __nv_bfloat16* g, float* dw, int* err, int sms, cudaStream_t st) {
#define HG_WG(A, B) \
  if (cin == A && cout == B) return run_wgrad<A, B>(xmap, dm, g, dw, err, sms, st);
  HG_WG(16, 16) HG_WG(16, 32) HG_WG(32, 16) HG_WG(32, 32) HG_WG(32, 64) HG_WG(64, 32)
  HG_WG(64, 64) HG_WG(64, 16) HG_WG(16, 64)
#undef HG_WG
  return cudaErrorInvalidValue;
}

}  // namespace nn
}  // namespace hg
