// net.cu -- the learned pressure guess: network object, forward / backward /
// Adam training step, single-layer C-ABI for gradient checks.
//
// Activations and their gradients are BF16 channels-last tensors; weights are
// kept in FP32 (with Adam moments) and re-arranged into the BF16 K-major tap
// blocks the tensor-core convolutions read after every update.  All the
// convolution work -- forward, backward-data and weight gradient -- runs on
// the tcgen05 kernels of conv.cu; pooling, upsampling, the loss, the bias
// gradients and Adam are streaming kernels here.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <new>
#include <vector>

#include "../../include/hydro_net.h"
#include "conv.h"
#include "kernels.h"

using hg::nn::ConvDims;
using hg::nn::Epilogue;

namespace hg {
namespace nn {
namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 1024;  // blocks of the deterministic reductions

int blocks_for(long long n, int per = kThreads) {
  long long b = (n + per - 1) / per;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

__device__ __forceinline__ float bf(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 tobf(float v) { return __float2bfloat16_rn(v); }

// Deterministic sums of NV FP64 quantities over a grid (fixed-order fold of
// the block partials in the last block).
template <int NV>
struct Red {
  double* partials;  // [NV][kRedBlocks]
  unsigned* ticket;
  double* out;       // NV results
};

// ------------------------------------------------ weight arrangement ------
// w [cout][cin][27] FP32 -> wf [27][cin/8][cout][8] (forward: K = ci) and
// wb [27][cout/8][cin][8] (backward-data: K = co, taps mirrored).
__global__ void k_arrange(const float* __restrict__ w, int cin, int cout,
                          __nv_bfloat16* __restrict__ wf, __nv_bfloat16* __restrict__ wb) {
  const int n = 27 * cin * cout;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int t = i % 27, ci = (i / 27) % cin, co = i / (27 * cin);
    const __nv_bfloat16 v = tobf(w[i]);
    wf[(((size_t)t * (cin / 8) + ci / 8) * cout + co) * 8 + ci % 8] = v;
    const int tb = 26 - t;
    if (wb) wb[(((size_t)tb * (cout / 8) + co / 8) * cin + ci) * 8 + co % 8] = v;
  }
}

// dwi [27][cout][cin] -> dw [cout][cin][27]
__global__ void k_dw_reorder(const float* __restrict__ dwi, int cin, int cout,
                             float* __restrict__ dw) {
  const int n = 27 * cin * cout;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int t = i % 27, ci = (i / 27) % cin, co = i / (27 * cin);
    dw[i] = dwi[((size_t)t * cout + co) * cin + ci];
  }
}

// ---------------------------------------------- pooling / upsampling -----
// Tensors [nb][z][y][x][c]; (nx, ny, nz): the fine grid.  One thread per
// coarse position and 8-channel chunk.
__global__ void k_pool(const __nv_bfloat16* __restrict__ in, ConvDims fine, int c,
                       __nv_bfloat16* __restrict__ out) {
  const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
  const long long n = (long long)cx * cy * cz * fine.nb * (c / 8);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % (c / 8));
    long long r = i / (c / 8);
    const int x = (int)(r % cx);
    r /= cx;
    const int y = (int)(r % cy);
    r /= cy;
    const int z = (int)(r % cz);
    const int b = (int)(r / cz);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; ++d) {
      const int xx = 2 * x + (d & 1), yy = 2 * y + ((d >> 1) & 1), zz = 2 * z + (d >> 2);
      const size_t p = (((size_t)b * fine.nz + zz) * fine.ny + yy) * fine.nx + xx;
      const uint4 q = *reinterpret_cast<const uint4*>(in + p * c + ch * 8);
      const __nv_bfloat16* v = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
      for (int e = 0; e < 8; ++e) acc[e] += bf(v[e]);
    }
    uint4 o;
    __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) o2[e] = __floats2bfloat162_rn(acc[2 * e] * 0.125f, acc[2 * e + 1] * 0.125f);
    const size_t pc = (((size_t)b * cz + z) * cy + y) * cx + x;
    *reinterpret_cast<uint4*>(out + pc * c + ch * 8) = o;
  }
}

// out (fine) = in (coarse) at the parent, nearest neighbour.
__global__ void k_up(const __nv_bfloat16* __restrict__ in, ConvDims fine, int c,
                     __nv_bfloat16* __restrict__ out) {
  const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
  const long long n = (long long)fine.nx * fine.ny * fine.nz * fine.nb * (c / 8);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % (c / 8));
    const long long p = i / (c / 8);
    long long r = p;
    const int x = (int)(r % fine.nx);
    r /= fine.nx;
    const int y = (int)(r % fine.ny);
    r /= fine.ny;
    const int z = (int)(r % fine.nz);
    const int b = (int)(r / fine.nz);
    const size_t pc = (((size_t)b * cz + z / 2) * cy + y / 2) * cx + x / 2;
    *reinterpret_cast<uint4*>(out + p * c + ch * 8) =
        *reinterpret_cast<const uint4*>(in + pc * c + ch * 8);
  }
}

// Backward of the upsampling followed by the ReLU mask of the coarse
// activation y: g (coarse) = (sum over the 8 children of gu) * (y > 0).
__global__ void k_upsum_mask(const __nv_bfloat16* __restrict__ gu, ConvDims fine, int c,
                             const __nv_bfloat16* __restrict__ y, __nv_bfloat16* __restrict__ g) {
  const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
  const long long n = (long long)cx * cy * cz * fine.nb * (c / 8);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % (c / 8));
    long long r = i / (c / 8);
    const long long pc = r;
    const int x = (int)(r % cx);
    r /= cx;
    const int yy0 = (int)(r % cy);
    r /= cy;
    const int z = (int)(r % cz);
    const int b = (int)(r / cz);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; ++d) {
      const int xx = 2 * x + (d & 1), yy = 2 * yy0 + ((d >> 1) & 1), zz = 2 * z + (d >> 2);
      const size_t p = (((size_t)b * fine.nz + zz) * fine.ny + yy) * fine.nx + xx;
      const uint4 q = *reinterpret_cast<const uint4*>(gu + p * c + ch * 8);
      const __nv_bfloat16* v = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
      for (int e = 0; e < 8; ++e) acc[e] += bf(v[e]);
    }
    const uint4 mq = *reinterpret_cast<const uint4*>(y + pc * c + ch * 8);
    const __nv_bfloat16* mv = reinterpret_cast<const __nv_bfloat16*>(&mq);
    uint4 o;
    __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e)
      o2[e] = __floats2bfloat162_rn(bf(mv[2 * e]) > 0.f ? acc[2 * e] : 0.f,
                                    bf(mv[2 * e + 1]) > 0.f ? acc[2 * e + 1] : 0.f);
    *reinterpret_cast<uint4*>(g + pc * c + ch * 8) = o;
  }
}

// Backward of the average pooling, plus the gradient of a skip branch, then
// the ReLU mask of the fine activation y:
// g (fine) = (gp[parent] / 8 + skip) * (y > 0); skip may be null.
__global__ void k_poolback_mask(const __nv_bfloat16* __restrict__ gp, ConvDims fine, int c,
                                const __nv_bfloat16* __restrict__ skip,
                                const __nv_bfloat16* __restrict__ y,
                                __nv_bfloat16* __restrict__ g) {
  const int cx = fine.nx / 2, cy = fine.ny / 2, cz = fine.nz / 2;
  const long long n = (long long)fine.nx * fine.ny * fine.nz * fine.nb * (c / 8);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % (c / 8));
    const long long p = i / (c / 8);
    long long r = p;
    const int x = (int)(r % fine.nx);
    r /= fine.nx;
    const int yy = (int)(r % fine.ny);
    r /= fine.ny;
    const int z = (int)(r % fine.nz);
    const int b = (int)(r / fine.nz);
    const size_t pc = (((size_t)b * cz + z / 2) * cy + yy / 2) * cx + x / 2;
    const uint4 gq = *reinterpret_cast<const uint4*>(gp + pc * c + ch * 8);
    const uint4 mq = *reinterpret_cast<const uint4*>(y + p * c + ch * 8);
    uint4 sq = make_uint4(0, 0, 0, 0);
    if (skip) sq = *reinterpret_cast<const uint4*>(skip + p * c + ch * 8);
    const __nv_bfloat16* gv = reinterpret_cast<const __nv_bfloat16*>(&gq);
    const __nv_bfloat16* mv = reinterpret_cast<const __nv_bfloat16*>(&mq);
    const __nv_bfloat16* sv = reinterpret_cast<const __nv_bfloat16*>(&sq);
    uint4 o;
    __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float a = bf(gv[2 * e]) * 0.125f + bf(sv[2 * e]);
      float b2 = bf(gv[2 * e + 1]) * 0.125f + bf(sv[2 * e + 1]);
      o2[e] = __floats2bfloat162_rn(bf(mv[2 * e]) > 0.f ? a : 0.f,
                                    bf(mv[2 * e + 1]) > 0.f ? b2 : 0.f);
    }
    *reinterpret_cast<uint4*>(g + p * c + ch * 8) = o;
  }
}

// db[c] = sum_p g[p][c] (FP32 partials per block, then atomics).
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ g, long long np, int c,
                            float* __restrict__ db) {
  __shared__ float acc[64];
  for (int i = threadIdx.x; i < c; i += blockDim.x) acc[i] = 0.f;
  __syncthreads();
  float loc = 0.f;
  // thread t sums channel t % c of the positions it strides over (c divides 256)
  const int ch = threadIdx.x % c;
  const int lanes = blockDim.x / c;
  for (long long p = blockIdx.x * (long long)lanes + threadIdx.x / c; p < np;
       p += (long long)gridDim.x * lanes)
    loc += bf(g[p * c + ch]);
  atomicAdd(&acc[ch], loc);
  __syncthreads();
  for (int i = threadIdx.x; i < c; i += blockDim.x) atomicAdd(&db[i], acc[i]);
}

// Adam on a flat block of parameters; grad index remapped for a weight
// block ([cout][cin][27] from the [27][cout][cin] gradient) when cin > 0.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, int n, int cin, int cout,
                       float lr, float b1, float b2, float c1, float c2, float eps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float gi;
    if (cin > 0) {
      const int t = i % 27, ci = (i / 27) % cin, co = i / (27 * cin);
      gi = grad[((size_t)t * cout + co) * cin + ci];
    } else {
      gi = grad[i];
    }
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

// ------------------------------------------------------ reductions -------
// out[0] = sum a, out[1] = sum a^2 (a: n doubles; NULL entries skipped by
// passing n = 0).
__global__ void k_sum_sumsq(const double* __restrict__ a, long long n, Red<2> r) {
  double s[2] = {0., 0.};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = a[i];
    s[0] += v;
    s[1] += v * v;
  }
  __shared__ double o[2];
  if (grid_reduce<RED_SUM, 2>(s, r.partials, r.ticket, o)) {
    if (threadIdx.x == 0) {
      r.out[0] = o[0];
      r.out[1] = o[1];
    }
  }
}

// ------------------------------------------ inputs, samples, outputs -----
// st[0..1]: sum, sum of squares of f over n cells -> mean, rms.
__device__ __forceinline__ void mean_rms(const double* st, long long n, double* mean,
                                         double* inv) {
  const double mu = st[0] / (double)n;
  const double var = st[1] / (double)n - mu * mu;
  *mean = mu;
  *inv = var > 0. ? 1. / sqrt(var) : 0.;
}

// X0[p] = {(f - mean) / rms, rho * rho_scale, 0, ...} (16 channels).
__global__ void k_input(const double* __restrict__ f, const double* __restrict__ rho,
                        const double* __restrict__ fst, double rho_scale, long long n,
                        __nv_bfloat16* __restrict__ x0) {
  double mu, inv;
  mean_rms(fst, n, &mu, &inv);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint4 o[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(o);
    o2[0] = __floats2bfloat162_rn((float)((f[i] - mu) * inv), (float)(rho[i] * rho_scale));
    uint4* dst = reinterpret_cast<uint4*>(x0 + i * 16);
    dst[0] = o[0];
    dst[1] = o[1];
  }
}

// Packed sample: per cell {(f - mean_f) / rms_f, rho * rho_scale,
// (p - mean_p) / rms_p} as BF16.
__global__ void k_pack(const double* __restrict__ f, const double* __restrict__ rho,
                       const double* __restrict__ pc, const double* __restrict__ fst,
                       const double* __restrict__ pst, double rho_scale, long long n,
                       __nv_bfloat16* __restrict__ dst) {
  double mf, inf, mp, inp;
  mean_rms(fst, n, &mf, &inf);
  mean_rms(pst, n, &mp, &inp);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    dst[3 * i] = tobf((float)((f[i] - mf) * inf));
    dst[3 * i + 1] = tobf((float)(rho[i] * rho_scale));
    dst[3 * i + 2] = tobf((float)((pc[i] - mp) * inp));
  }
}

// Sample slot b of the batch: inputs into X0, target into tgt (FP32).
__global__ void k_unpack(const __nv_bfloat16* __restrict__ s, long long n,
                         __nv_bfloat16* __restrict__ x0, float* __restrict__ tgt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint4 o[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    __nv_bfloat16* ov = reinterpret_cast<__nv_bfloat16*>(o);
    ov[0] = s[3 * i];
    ov[1] = s[3 * i + 1];
    uint4* dst = reinterpret_cast<uint4*>(x0 + i * 16);
    dst[0] = o[0];
    dst[1] = o[1];
    tgt[i] = bf(s[3 * i + 2]);
  }
}

// Loss 0.5 * mean (out_0 - t)^2 over n positions (all samples); g_out: its
// gradient (channel 0; channels 1..15 zero).
__global__ void k_loss(const __nv_bfloat16* __restrict__ out, const float* __restrict__ tgt,
                       long long n, int want_grad, __nv_bfloat16* __restrict__ g, Red<1> r) {
  double s[1] = {0.};
  const float inv_n = 1.f / (float)n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float d = bf(out[i * 16]) - tgt[i];
    s[0] += (double)d * (double)d;
    if (want_grad) {
      uint4 o[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
      reinterpret_cast<__nv_bfloat16*>(o)[0] = tobf(d * inv_n);
      uint4* dst = reinterpret_cast<uint4*>(g + i * 16);
      dst[0] = o[0];
      dst[1] = o[1];
    }
  }
  __shared__ double o[1];
  if (grid_reduce<RED_SUM, 1>(s, r.partials, r.ticket, o))
    if (threadIdx.x == 0) r.out[0] = 0.5 * o[0] / (double)n;
}

__global__ void k_output(const __nv_bfloat16* __restrict__ out, long long n,
                         double* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = (double)bf(out[i * 16]);
}

// ------------------------------------------------------------ layers -----
struct Tensor {
  __nv_bfloat16* p = nullptr;
  ConvDims dm{};  // full batch
  int c = 0;
  CUtensorMap map;
  bool has_map = false;
  size_t elems() const { return (size_t)dm.nx * dm.ny * dm.nz * dm.nb * c; }
};

struct Layer {
  int cin, cout;
  size_t woff, boff;     // offsets in the flat FP32 parameter array
  __nv_bfloat16* wf;     // forward tap blocks
  __nv_bfloat16* wb;     // backward-data tap blocks
  float* dwi;            // weight gradient [27][cout][cin]
};

}  // namespace
}  // namespace nn
}  // namespace hg

using namespace hg;
using namespace hg::nn;

struct hydro_net {
  int n[3] = {0, 0, 0};
  int batch = 0;
  int sms = 152;
  std::vector<void*> allocs;
  // parameters
  size_t nparam = 0;
  float* param = nullptr;
  float* grad = nullptr;  // bias gradients (weights' live in Layer::dwi)
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  long long adam_t = 0;
  Layer L[11];
  // activations (index = layer output), pooled / upsampled tensors, grads
  Tensor X0, A[11], P1, P2, U2, U1;
  Tensor G[11];   // G[l]: gradient of layer l's pre-activation (G[10]: of the output)
  Tensor GU1, GU2, GP1, GP2;
  float* tgt = nullptr;
  // reductions
  double* red_partials = nullptr;
  unsigned* red_ticket = nullptr;
  double* red_out = nullptr;  // [8]
  int* err = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.;
  int last_launches = 0;
  bool timed = false;
};

namespace {

int dev_alloc(hydro_net* net, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return HYDRO_ERR_NOMEM;
  }
  net->allocs.push_back(*p);
  return HYDRO_OK;
}

int make_tensor(hydro_net* net, Tensor& t, int nx, int ny, int nz, int c, bool map) {
  t.dm = {nx, ny, nz, net->batch};
  t.c = c;
  int rc = dev_alloc(net, (void**)&t.p, t.elems() * 2);
  if (rc) return rc;
  cudaMemset(t.p, 0, t.elems() * 2);
  if (map) {
    if (make_act_map(&t.map, t.p, t.dm, c)) return HYDRO_ERR_CUDA;
    t.has_map = true;
  }
  return HYDRO_OK;
}

// Layer table: (cin, cout) of e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b out.
const int kLayerC[11][2] = {{16, 16}, {16, 16}, {16, 32}, {32, 32}, {32, 64}, {64, 64},
                            {64, 32}, {32, 32}, {32, 16}, {16, 16}, {16, 16}};

// Simple seeded generator for the He-normal initialisation.
struct Rng {
  unsigned long long s;
  double uniform() {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return ((s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  }
  double normal() {
    double u1 = uniform(), u2 = uniform();
    return sqrt(-2. * log(u1)) * cos(6.283185307179586 * u2);
  }
};

cudaError_t arrange_all(hydro_net* net, cudaStream_t st) {
  for (auto& l : net->L) {
    k_arrange<<<blocks_for(27 * l.cin * l.cout), kThreads, 0, st>>>(net->param + l.woff, l.cin,
                                                                   l.cout, l.wf, l.wb);
  }
  count_launches(11);
  return cudaGetLastError();
}

Red<2> red2(hydro_net* net, int slot) {
  return {net->red_partials, net->red_ticket + slot, net->red_out + 2 * slot};
}
Red<1> red1(hydro_net* net, int slot) {
  return {net->red_partials, net->red_ticket + slot, net->red_out + 2 * slot};
}

cudaError_t conv(hydro_net* net, const Tensor& x, int layer, int nb, const __nv_bfloat16* addend,
                 int relu, Tensor& y, cudaStream_t st) {
  const Layer& l = net->L[layer];
  Epilogue ep{net->param + l.boff, addend, nullptr, relu};
  ConvDims dm = x.dm;
  dm.nb = nb;
  count_launches(1);
  return conv3d(x.map, dm, l.cin, l.cout, l.wf, ep, y.p, net->err, st);
}

// gx = conv^T(gy) (+ addend) * (mask > 0)
cudaError_t conv_bwd(hydro_net* net, const Tensor& gy, int layer, int nb,
                     const __nv_bfloat16* addend, const __nv_bfloat16* mask, Tensor& gx,
                     cudaStream_t st) {
  const Layer& l = net->L[layer];
  Epilogue ep{nullptr, addend, mask, 0};
  ConvDims dm = gy.dm;
  dm.nb = nb;
  count_launches(1);
  return conv3d(gy.map, dm, l.cout, l.cin, l.wb, ep, gx.p, net->err, st);
}

cudaError_t wgrad(hydro_net* net, const Tensor& x, const Tensor& gy, int layer, int nb,
                  cudaStream_t st) {
  const Layer& l = net->L[layer];
  ConvDims dm = x.dm;
  dm.nb = nb;
  cudaError_t e = conv3d_wgrad(x.map, dm, l.cin, l.cout, gy.p, l.dwi, net->err, net->sms, st);
  if (e != cudaSuccess) return e;
  const long long np = (long long)gy.dm.nx * gy.dm.ny * gy.dm.nz * nb;
  k_bias_grad<<<blocks_for(np, 256), 256, 0, st>>>(gy.p, np, l.cout, net->grad + l.boff);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t pool(const Tensor& in, int nb, Tensor& out, cudaStream_t st) {
  ConvDims f = in.dm;
  f.nb = nb;
  k_pool<<<blocks_for((long long)out.dm.nx * out.dm.ny * out.dm.nz * nb * in.c / 8), kThreads, 0,
           st>>>(in.p, f, in.c, out.p);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t up(const Tensor& in, int nb, Tensor& out, cudaStream_t st) {
  ConvDims f = out.dm;
  f.nb = nb;
  k_up<<<blocks_for((long long)f.nx * f.ny * f.nz * nb * in.c / 8), kThreads, 0, st>>>(
      in.p, f, in.c, out.p);
  count_launches(1);
  return cudaGetLastError();
}

#define CKC(x)                                  \
  do {                                          \
    cudaError_t e_ = (x);                       \
    if (e_ != cudaSuccess) return e_;           \
  } while (0)

cudaError_t forward(hydro_net* net, int nb, cudaStream_t st) {
  Tensor* A = net->A;
  CKC(conv(net, net->X0, 0, nb, nullptr, 1, A[0], st));
  CKC(conv(net, A[0], 1, nb, nullptr, 1, A[1], st));
  CKC(pool(A[1], nb, net->P1, st));
  CKC(conv(net, net->P1, 2, nb, nullptr, 1, A[2], st));
  CKC(conv(net, A[2], 3, nb, nullptr, 1, A[3], st));
  CKC(pool(A[3], nb, net->P2, st));
  CKC(conv(net, net->P2, 4, nb, nullptr, 1, A[4], st));
  CKC(conv(net, A[4], 5, nb, nullptr, 1, A[5], st));
  CKC(up(A[5], nb, net->U2, st));
  CKC(conv(net, net->U2, 6, nb, A[3].p, 1, A[6], st));
  CKC(conv(net, A[6], 7, nb, nullptr, 1, A[7], st));
  CKC(up(A[7], nb, net->U1, st));
  CKC(conv(net, net->U1, 8, nb, A[1].p, 1, A[8], st));
  CKC(conv(net, A[8], 9, nb, nullptr, 1, A[9], st));
  CKC(conv(net, A[9], 10, nb, nullptr, 0, A[10], st));
  return cudaSuccess;
}

// Gradients of every layer from G[10] (the output's gradient).
cudaError_t backward(hydro_net* net, int nb, cudaStream_t st) {
  Tensor *A = net->A, *G = net->G;
  for (auto& l : net->L)
    CKC(cudaMemsetAsync(l.dwi, 0, sizeof(float) * 27 * l.cin * l.cout, st));
  CKC(cudaMemsetAsync(net->grad, 0, sizeof(float) * net->nparam, st));
  // out = conv(A9)
  CKC(wgrad(net, A[9], G[10], 10, nb, st));
  CKC(conv_bwd(net, G[10], 10, nb, nullptr, A[9].p, G[9], st));
  // A9 = relu(conv(A8))
  CKC(wgrad(net, A[8], G[9], 9, nb, st));
  CKC(conv_bwd(net, G[9], 9, nb, nullptr, A[8].p, G[8], st));
  // A8 = relu(conv(U1) + A1)
  CKC(wgrad(net, net->U1, G[8], 8, nb, st));
  CKC(conv_bwd(net, G[8], 8, nb, nullptr, nullptr, net->GU1, st));
  {
    ConvDims f = net->U1.dm;
    f.nb = nb;
    k_upsum_mask<<<blocks_for((long long)A[7].dm.nx * A[7].dm.ny * A[7].dm.nz * nb * 32 / 8),
                   kThreads, 0, st>>>(net->GU1.p, f, 32, A[7].p, G[7].p);
    count_launches(1);
  }
  // A7 = relu(conv(A6))
  CKC(wgrad(net, A[6], G[7], 7, nb, st));
  CKC(conv_bwd(net, G[7], 7, nb, nullptr, A[6].p, G[6], st));
  // A6 = relu(conv(U2) + A3)
  CKC(wgrad(net, net->U2, G[6], 6, nb, st));
  CKC(conv_bwd(net, G[6], 6, nb, nullptr, nullptr, net->GU2, st));
  {
    ConvDims f = net->U2.dm;
    f.nb = nb;
    k_upsum_mask<<<blocks_for((long long)A[5].dm.nx * A[5].dm.ny * A[5].dm.nz * nb * 64 / 8),
                   kThreads, 0, st>>>(net->GU2.p, f, 64, A[5].p, G[5].p);
    count_launches(1);
  }
  // A5 = relu(conv(A4)), A4 = relu(conv(P2))
  CKC(wgrad(net, A[4], G[5], 5, nb, st));
  CKC(conv_bwd(net, G[5], 5, nb, nullptr, A[4].p, G[4], st));
  CKC(wgrad(net, net->P2, G[4], 4, nb, st));
  CKC(conv_bwd(net, G[4], 4, nb, nullptr, nullptr, net->GP2, st));
  {
    // A3 feeds the pool and the skip of layer 6
    ConvDims f = A[3].dm;
    f.nb = nb;
    k_poolback_mask<<<blocks_for((long long)f.nx * f.ny * f.nz * nb * 32 / 8), kThreads, 0,
                      st>>>(net->GP2.p, f, 32, G[6].p, A[3].p, G[3].p);
    count_launches(1);
  }
  CKC(wgrad(net, A[2], G[3], 3, nb, st));
  CKC(conv_bwd(net, G[3], 3, nb, nullptr, A[2].p, G[2], st));
  CKC(wgrad(net, net->P1, G[2], 2, nb, st));
  CKC(conv_bwd(net, G[2], 2, nb, nullptr, nullptr, net->GP1, st));
  {
    // A1 feeds the pool and the skip of layer 8
    ConvDims f = A[1].dm;
    f.nb = nb;
    k_poolback_mask<<<blocks_for((long long)f.nx * f.ny * f.nz * nb * 16 / 8), kThreads, 0,
                      st>>>(net->GP1.p, f, 16, G[8].p, A[1].p, G[1].p);
    count_launches(1);
  }
  CKC(wgrad(net, A[0], G[1], 1, nb, st));
  CKC(conv_bwd(net, G[1], 1, nb, nullptr, A[0].p, G[0], st));
  CKC(wgrad(net, net->X0, G[0], 0, nb, st));
  return cudaSuccess;
}

cudaError_t adam(hydro_net* net, double lr, cudaStream_t st) {
  net->adam_t += 1;
  const double b1 = 0.9, b2 = 0.999;
  const float c1 = (float)(1. / (1. - pow(b1, (double)net->adam_t)));
  const float c2 = (float)(1. / (1. - pow(b2, (double)net->adam_t)));
  for (auto& l : net->L) {
    const int nw = 27 * l.cin * l.cout;
    k_adam<<<blocks_for(nw), kThreads, 0, st>>>(net->param + l.woff, l.dwi,
                                                net->adam_m + l.woff, net->adam_v + l.woff, nw,
                                                l.cin, l.cout, (float)lr, (float)b1, (float)b2,
                                                c1, c2, 1e-8f);
    k_adam<<<1, 64, 0, st>>>(net->param + l.boff, net->grad + l.boff, net->adam_m + l.boff,
                             net->adam_v + l.boff, l.cout, 0, 0, (float)lr, (float)b1,
                             (float)b2, c1, c2, 1e-8f);
  }
  count_launches(22);
  return arrange_all(net, st);
}

long long cells(const hydro_net* net) { return (long long)net->n[0] * net->n[1] * net->n[2]; }

int finish(hydro_net* net, cudaError_t e) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    return HYDRO_ERR_CUDA;
  }
  return HYDRO_OK;
}

int load_batch(hydro_net* net, const void* const* samples, int count, cudaStream_t st) {
  const long long n = cells(net);
  for (int b = 0; b < count; ++b) {
    if (!samples[b]) return HYDRO_ERR_ARG;
    k_unpack<<<blocks_for(n), kThreads, 0, st>>>(
        static_cast<const __nv_bfloat16*>(samples[b]), n, net->X0.p + (size_t)b * n * 16,
        net->tgt + (size_t)b * n);
  }
  count_launches(count);
  return HYDRO_OK;
}

int read_err(hydro_net* net, cudaStream_t st) {
  int h = 0;
  if (cudaMemcpyAsync(&h, net->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return HYDRO_ERR_CUDA;
  }
  return h ? HYDRO_ERR_CUDA : HYDRO_OK;
}

}  // namespace

// ------------------------------------------------------------- C-ABI -----
extern "C" {

int hydro_net_create(int nx, int ny, int nz, int batch, unsigned long long seed,
                     hydro_net** out) {
  if (!out || nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4 || batch < 1)
    return HYDRO_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return HYDRO_ERR_NO_DEVICE;
  }
  hydro_net* net = new (std::nothrow) hydro_net();
  if (!net) return HYDRO_ERR_NOMEM;
  net->n[0] = nx;
  net->n[1] = ny;
  net->n[2] = nz;
  net->batch = batch;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&net->sms, cudaDevAttrMultiProcessorCount, dev);
  int rc = HYDRO_OK;
  size_t off = 0;
  for (int l = 0; l < 11; ++l) {
    net->L[l].cin = kLayerC[l][0];
    net->L[l].cout = kLayerC[l][1];
    net->L[l].woff = off;
    off += (size_t)27 * kLayerC[l][0] * kLayerC[l][1];
    net->L[l].boff = off;
    off += kLayerC[l][1];
  }
  net->nparam = off;
  auto fail = [&](int r) {
    hydro_net_destroy(net);
    return r;
  };
  if ((rc = dev_alloc(net, (void**)&net->param, off * 4)) ||
      (rc = dev_alloc(net, (void**)&net->grad, off * 4)) ||
      (rc = dev_alloc(net, (void**)&net->adam_m, off * 4)) ||
      (rc = dev_alloc(net, (void**)&net->adam_v, off * 4)))
    return fail(rc);
  cudaMemset(net->adam_m, 0, off * 4);
  cudaMemset(net->adam_v, 0, off * 4);
  for (auto& l : net->L) {
    if ((rc = dev_alloc(net, (void**)&l.wf, (size_t)27 * l.cin * l.cout * 2)) ||
        (rc = dev_alloc(net, (void**)&l.wb, (size_t)27 * l.cin * l.cout * 2)) ||
        (rc = dev_alloc(net, (void**)&l.dwi, (size_t)27 * l.cin * l.cout * 4)))
      return fail(rc);
  }
  // He-normal weights (fan-in 27 cin; the first layer's two used channels),
  // zero biases; padded channels zero: e1a's inputs 2..15, out's outputs 1..15
  {
    std::vector<float> h(off, 0.f);
    Rng g{seed * 0x9E3779B97F4A7C15ULL + 12345ULL};
    for (int li = 0; li < 11; ++li) {
      const Layer& l = net->L[li];
      const int cin_used = li == 0 ? 2 : l.cin;
      const int cout_used = li == 10 ? 1 : l.cout;
      const double sd = sqrt(2. / (27. * cin_used)) * (li == 10 ? 0.5 : 1.);
      for (int co = 0; co < l.cout; ++co)
        for (int ci = 0; ci < l.cin; ++ci)
          for (int t = 0; t < 27; ++t) {
            const double v = g.normal() * sd;
            if (co < cout_used && ci < cin_used)
              h[l.woff + ((size_t)co * l.cin + ci) * 27 + t] = (float)v;
          }
    }
    if (cudaMemcpy(net->param, h.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(HYDRO_ERR_CUDA);
  }
  const int n2x = nx / 2, n2y = ny / 2, n2z = nz / 2, n4x = nx / 4, n4y = ny / 4, n4z = nz / 4;
  Tensor* A = net->A;
  Tensor* G = net->G;
  if ((rc = make_tensor(net, net->X0, nx, ny, nz, 16, true)) ||
      (rc = make_tensor(net, A[0], nx, ny, nz, 16, true)) ||
      (rc = make_tensor(net, A[1], nx, ny, nz, 16, false)) ||
      (rc = make_tensor(net, net->P1, n2x, n2y, n2z, 16, true)) ||
      (rc = make_tensor(net, A[2], n2x, n2y, n2z, 32, true)) ||
      (rc = make_tensor(net, A[3], n2x, n2y, n2z, 32, false)) ||
      (rc = make_tensor(net, net->P2, n4x, n4y, n4z, 32, true)) ||
      (rc = make_tensor(net, A[4], n4x, n4y, n4z, 64, true)) ||
      (rc = make_tensor(net, A[5], n4x, n4y, n4z, 64, false)) ||
      (rc = make_tensor(net, net->U2, n2x, n2y, n2z, 64, true)) ||
      (rc = make_tensor(net, A[6], n2x, n2y, n2z, 32, true)) ||
      (rc = make_tensor(net, A[7], n2x, n2y, n2z, 32, false)) ||
      (rc = make_tensor(net, net->U1, nx, ny, nz, 32, true)) ||
      (rc = make_tensor(net, A[8], nx, ny, nz, 16, true)) ||
      (rc = make_tensor(net, A[9], nx, ny, nz, 16, true)) ||
      (rc = make_tensor(net, A[10], nx, ny, nz, 16, false)))
    return fail(rc);
  // gradients of the pre-activations (inputs of the backward-data convs)
  const int gdims[11][4] = {{nx, ny, nz, 16},    {nx, ny, nz, 16},    {n2x, n2y, n2z, 32},
                            {n2x, n2y, n2z, 32}, {n4x, n4y, n4z, 64}, {n4x, n4y, n4z, 64},
                            {n2x, n2y, n2z, 32}, {n2x, n2y, n2z, 32}, {nx, ny, nz, 16},
                            {nx, ny, nz, 16},    {nx, ny, nz, 16}};
  for (int l = 0; l < 11; ++l)
    if ((rc = make_tensor(net, G[l], gdims[l][0], gdims[l][1], gdims[l][2], gdims[l][3],
                          l > 0)))
      return fail(rc);
  if ((rc = make_tensor(net, net->GU1, nx, ny, nz, 32, false)) ||
      (rc = make_tensor(net, net->GU2, n2x, n2y, n2z, 64, false)) ||
      (rc = make_tensor(net, net->GP1, n2x, n2y, n2z, 16, false)) ||
      (rc = make_tensor(net, net->GP2, n4x, n4y, n4z, 32, false)))
    return fail(rc);
  if ((rc = dev_alloc(net, (void**)&net->tgt, sizeof(float) * (size_t)batch * nx * ny * nz)) ||
      (rc = dev_alloc(net, (void**)&net->red_partials, sizeof(double) * 2 * kRedBlocks)) ||
      (rc = dev_alloc(net, (void**)&net->red_ticket, sizeof(unsigned) * 8)) ||
      (rc = dev_alloc(net, (void**)&net->red_out, sizeof(double) * 16)) ||
      (rc = dev_alloc(net, (void**)&net->err, sizeof(int))))
    return fail(rc);
  cudaMemset(net->red_ticket, 0, sizeof(unsigned) * 8);
  cudaMemset(net->err, 0, sizeof(int));
  if (cudaEventCreate(&net->ev0) != cudaSuccess || cudaEventCreate(&net->ev1) != cudaSuccess)
    return fail(HYDRO_ERR_CUDA);
  if (arrange_all(net, 0) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    cudaGetLastError();
    return fail(HYDRO_ERR_CUDA);
  }
  *out = net;
  return HYDRO_OK;
}

int hydro_net_destroy(hydro_net* net) {
  if (!net) return HYDRO_OK;
  cudaDeviceSynchronize();
  for (void* p : net->allocs) cudaFree(p);
  if (net->ev0) cudaEventDestroy(net->ev0);
  if (net->ev1) cudaEventDestroy(net->ev1);
  delete net;
  return HYDRO_OK;
}

int hydro_net_num_params(hydro_net* net, size_t* n) {
  if (!net || !n) return HYDRO_ERR_ARG;
  *n = net->nparam;
  return HYDRO_OK;
}

int hydro_net_get_params(hydro_net* net, float* host, size_t n) {
  if (!net || !host || n != net->nparam) return HYDRO_ERR_ARG;
  if (cudaMemcpy(host, net->param, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return finish(net, cudaErrorUnknown);
  return HYDRO_OK;
}

int hydro_net_set_params(hydro_net* net, const float* host, size_t n) {
  if (!net || !host || n != net->nparam) return HYDRO_ERR_ARG;
  if (cudaMemcpy(net->param, host, n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return finish(net, cudaErrorUnknown);
  cudaMemset(net->adam_m, 0, n * 4);
  cudaMemset(net->adam_v, 0, n * 4);
  net->adam_t = 0;
  if (arrange_all(net, 0) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
    return finish(net, cudaErrorUnknown);
  return HYDRO_OK;
}

size_t hydro_net_sample_bytes(hydro_net* net) {
  return net ? (size_t)cells(net) * 3 * 2 : 0;
}

int hydro_net_pack_sample(hydro_net* net, const double* rhs, const double* rho,
                          const double* pcorr, double rho_scale, void* dst, void* stream) {
  if (!net || !rhs || !rho || !pcorr || !dst) return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = cells(net);
  k_sum_sumsq<<<kRedBlocks, kThreads, 0, st>>>(rhs, n, red2(net, 0));
  k_sum_sumsq<<<kRedBlocks, kThreads, 0, st>>>(pcorr, n, red2(net, 1));
  k_pack<<<blocks_for(n), kThreads, 0, st>>>(rhs, rho, pcorr, net->red_out, net->red_out + 2,
                                            rho_scale, n, static_cast<__nv_bfloat16*>(dst));
  count_launches(3);
  return finish(net, cudaGetLastError());
}

static int train_or_eval(hydro_net* net, const void* const* samples, int count, double lr,
                         double* loss, void* stream, bool train) {
  if (!net || !samples || count < 1 || count > net->batch) return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = load_batch(net, samples, count, st);
  if (rc) return rc;
  cudaError_t e = forward(net, count, st);
  if (e != cudaSuccess) return finish(net, e);
  const long long n = cells(net) * count;
  k_loss<<<kRedBlocks, kThreads, 0, st>>>(net->A[10].p, net->tgt, n, train ? 1 : 0,
                                          net->G[10].p, red1(net, 2));
  count_launches(1);
  if (train) {
    if ((e = backward(net, count, st)) != cudaSuccess) return finish(net, e);
    if ((e = adam(net, lr, st)) != cudaSuccess) return finish(net, e);
  }
  if ((rc = read_err(net, st))) return rc;
  if (loss) {
    if (cudaMemcpy(loss, net->red_out + 4, sizeof(double), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
      return finish(net, cudaErrorUnknown);
  }
  return HYDRO_OK;
}

int hydro_net_train_step(hydro_net* net, const void* const* samples, int count, double lr,
                         double* loss, void* stream) {
  return train_or_eval(net, samples, count, lr, loss, stream, true);
}

int hydro_net_eval_loss(hydro_net* net, const void* const* samples, int count, double* loss,
                        void* stream) {
  return train_or_eval(net, samples, count, 0., loss, stream, false);
}

int hydro_net_gradient(hydro_net* net, const void* const* samples, int count, float* grad,
                       size_t n, double* loss, void* stream) {
  if (!net || !samples || !grad || n != net->nparam || count < 1 || count > net->batch)
    return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = load_batch(net, samples, count, st);
  if (rc) return rc;
  cudaError_t e = forward(net, count, st);
  if (e != cudaSuccess) return finish(net, e);
  const long long np = cells(net) * count;
  k_loss<<<kRedBlocks, kThreads, 0, st>>>(net->A[10].p, net->tgt, np, 1, net->G[10].p,
                                          red1(net, 2));
  count_launches(1);
  if ((e = backward(net, count, st)) != cudaSuccess) return finish(net, e);
  // weights: [27][cout][cin] -> the parameter layout [cout][cin][27]
  for (auto& l : net->L) {
    k_dw_reorder<<<blocks_for(27LL * l.cin * l.cout), kThreads, 0, st>>>(l.dwi, l.cin, l.cout,
                                                                        net->grad + l.woff);
    count_launches(1);
  }
  if ((rc = read_err(net, st))) return rc;
  if (cudaMemcpy(grad, net->grad, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      (loss && cudaMemcpy(loss, net->red_out + 4, sizeof(double), cudaMemcpyDeviceToHost) !=
                   cudaSuccess))
    return finish(net, cudaErrorUnknown);
  return HYDRO_OK;
}

int hydro_net_last_predict(hydro_net* net, double* ms, int* launches) {
  if (!net) return HYDRO_ERR_ARG;
  if (ms) {
    float f = 0.f;
    if (net->timed && cudaEventElapsedTime(&f, net->ev0, net->ev1) == cudaSuccess)
      *ms = f;
    else
      *ms = -1.;
    cudaGetLastError();
  }
  if (launches) *launches = net->last_launches;
  return HYDRO_OK;
}

}  // extern "C"

// Forward pass on one sample of FP64 fields into out (FP64); enqueued on st
// without host synchronisation (usable inside a stream capture).
int net_predict_async(hydro_net* net, const double* rhs, const double* rho, double rho_scale,
                      double* out, cudaStream_t st) {
  const long long n = cells(net);
  long long l0 = launch_total();
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  net->timed = cs == cudaStreamCaptureStatusNone;
  if (net->timed) cudaEventRecord(net->ev0, st);
  k_sum_sumsq<<<kRedBlocks, kThreads, 0, st>>>(rhs, n, red2(net, 3));
  k_input<<<blocks_for(n), kThreads, 0, st>>>(rhs, rho, net->red_out + 6, rho_scale, n,
                                             net->X0.p);
  count_launches(2);
  cudaError_t e = forward(net, 1, st);
  if (e != cudaSuccess) return finish(net, e);
  k_output<<<blocks_for(n), kThreads, 0, st>>>(net->A[10].p, n, out);
  count_launches(1);
  if (net->timed) cudaEventRecord(net->ev1, st);
  net->last_launches = (int)(launch_total() - l0);
  return finish(net, cudaGetLastError());
}

int net_check_grid(const hydro_net* net, int dim, const int* n) {
  return net && dim == 3 && n[0] == net->n[0] && n[1] == net->n[1] && n[2] == net->n[2];
}

int net_error(hydro_net* net, cudaStream_t st) { return read_err(net, st); }

extern "C" int hydro_net_predict(hydro_net* net, const double* rhs, const double* rho,
                                 double rho_scale, double* out, void* stream) {
  if (!net || !rhs || !rho || !out) return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = net_predict_async(net, rhs, rho, rho_scale, out, st);
  if (rc) return rc;
  return read_err(net, st);
}

// --------------------------------------------------- single layers -------
namespace {

struct Scratch {
  __nv_bfloat16 *wf = nullptr, *wb = nullptr;
  float* dwi = nullptr;
  int* err = nullptr;
  ~Scratch() {
    if (wf) cudaFree(wf);
    if (wb) cudaFree(wb);
    if (dwi) cudaFree(dwi);
    if (err) cudaFree(err);
  }
};

bool valid_c(int c) { return c == 16 || c == 32 || c == 64; }

int layer_prep(int cin, int cout, const float* w, Scratch& s, cudaStream_t st, bool need_dwi) {
  const size_t nw = (size_t)27 * cin * cout;
  if (cudaMalloc(&s.wf, nw * 2) != cudaSuccess || cudaMalloc(&s.wb, nw * 2) != cudaSuccess ||
      cudaMalloc(&s.err, sizeof(int)) != cudaSuccess ||
      (need_dwi && cudaMalloc(&s.dwi, nw * 4) != cudaSuccess)) {
    cudaGetLastError();
    return HYDRO_ERR_NOMEM;
  }
  cudaMemsetAsync(s.err, 0, sizeof(int), st);
  if (w) {
    k_arrange<<<blocks_for((long long)nw), kThreads, 0, st>>>(w, cin, cout, s.wf, s.wb);
    count_launches(1);
  }
  return HYDRO_OK;
}

int layer_done(Scratch& s, cudaStream_t st) {
  int h = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&h, s.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return HYDRO_ERR_CUDA;
  }
  return h ? HYDRO_ERR_CUDA : HYDRO_OK;
}

}  // namespace

extern "C" {

int hydro_conv3d_forward(int nx, int ny, int nz, int nb, int cin, int cout, const void* x,
                         const float* w, const float* bias, const void* addend, int relu,
                         void* y, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || nb < 1 || !valid_c(cin) || !valid_c(cout) || !x || !w ||
      !y)
    return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  Scratch s;
  int rc = layer_prep(cin, cout, w, s, st, false);
  if (rc) return rc;
  ConvDims dm{nx, ny, nz, nb};
  CUtensorMap map;
  if (make_act_map(&map, x, dm, cin)) return HYDRO_ERR_CUDA;
  Epilogue ep{bias, static_cast<const __nv_bfloat16*>(addend), nullptr, relu};
  count_launches(1);
  if (conv3d(map, dm, cin, cout, s.wf, ep, static_cast<__nv_bfloat16*>(y), s.err, st) !=
      cudaSuccess)
    return finish(nullptr, cudaErrorUnknown);
  return layer_done(s, st);
}

int hydro_conv3d_backward_data(int nx, int ny, int nz, int nb, int cin, int cout,
                               const void* gy, const float* w, const void* addend,
                               const void* mask, void* gx, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || nb < 1 || !valid_c(cin) || !valid_c(cout) || !gy || !w ||
      !gx)
    return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  Scratch s;
  int rc = layer_prep(cin, cout, w, s, st, false);
  if (rc) return rc;
  ConvDims dm{nx, ny, nz, nb};
  CUtensorMap map;
  if (make_act_map(&map, gy, dm, cout)) return HYDRO_ERR_CUDA;
  Epilogue ep{nullptr, static_cast<const __nv_bfloat16*>(addend),
              static_cast<const __nv_bfloat16*>(mask), 0};
  count_launches(1);
  if (conv3d(map, dm, cout, cin, s.wb, ep, static_cast<__nv_bfloat16*>(gx), s.err, st) !=
      cudaSuccess)
    return finish(nullptr, cudaErrorUnknown);
  return layer_done(s, st);
}

int hydro_conv3d_backward_weight(int nx, int ny, int nz, int nb, int cin, int cout,
                                 const void* x, const void* gy, float* dw, float* db,
                                 void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || nb < 1 || !valid_c(cin) || !valid_c(cout) || !x || !gy ||
      !dw)
    return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  Scratch s;
  int rc = layer_prep(cin, cout, nullptr, s, st, true);
  if (rc) return rc;
  ConvDims dm{nx, ny, nz, nb};
  CUtensorMap map;
  if (make_act_map(&map, x, dm, cin)) return HYDRO_ERR_CUDA;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaMemsetAsync(s.dwi, 0, sizeof(float) * 27 * cin * cout, st);
  count_launches(1);
  if (conv3d_wgrad(map, dm, cin, cout, static_cast<const __nv_bfloat16*>(gy), s.dwi, s.err, sms,
                   st) != cudaSuccess)
    return finish(nullptr, cudaErrorUnknown);
  k_dw_reorder<<<blocks_for(27LL * cin * cout), kThreads, 0, st>>>(s.dwi, cin, cout, dw);
  count_launches(1);
  if (db) {
    const long long np = (long long)nx * ny * nz * nb;
    cudaMemsetAsync(db, 0, sizeof(float) * cout, st);
    k_bias_grad<<<blocks_for(np, 256), 256, 0, st>>>(static_cast<const __nv_bfloat16*>(gy), np,
                                                     cout, db);
    count_launches(1);
  }
  return layer_done(s, st);
}

}  // extern "C"
