// conv.h -- tensor-core 3x3x3 convolutions of the learned pressure guess
// (conv.cu) and the tile geometry they share with the network code (net.cu).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace hg {
namespace nn {

// Output tile of one CTA: 8 x 16 x 4 positions = four M = 128 row blocks;
// the input halo tile is one position wider on every side.
constexpr int kTX = 8, kTY = 16, kTZ = 4;
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kHRows = kHX * kHY * kHZ;  // 1080 rows of 16 B per 8-channel chunk
constexpr int kRegion = kHRows * 16;     // bytes of one 8-channel chunk of the halo tile

// Grid of one activation tensor: [nb][nz][ny][nx][C] BF16.
struct ConvDims {
  int nx, ny, nz, nb;
};

// Epilogue of a convolution, applied per output value v (FP32 accumulator):
// v += bias[co] (bias may be null); v += addend[p][co] (may be null);
// relu: v = max(v, 0); mask: v = 0 where mask[p][co] <= 0 (may be null).
struct Epilogue {
  const float* bias;
  const __nv_bfloat16* addend;
  const __nv_bfloat16* mask;
  int relu;
};

// TMA descriptor of an activation tensor with c channels (c % 8 == 0):
// boxes of 8 channels x the halo tile.  0 on success.
int make_act_map(CUtensorMap* map, const void* base, ConvDims dm, int c);

// out = epi(conv(x, w)); w: [27][cin/8][cout][8] BF16.  The (cin, cout)
// pairs built: 16, 32 and 64 in every combination.
cudaError_t conv3d(const CUtensorMap& xmap, ConvDims dm, int cin, int cout,
                   const __nv_bfloat16* w, Epilogue ep, __nv_bfloat16* out, int* err,
                   cudaStream_t st);

// dw[27][cout][cin] (FP32) += sum_p g[p][co] x[p + off(tap)][ci]; sms: the
// number of SMs to spread the persistent CTAs over.
cudaError_t conv3d_wgrad(const CUtensorMap& xmap, ConvDims dm, int cin, int cout,
                         const __nv_bfloat16* g, float* dw, int* err, int sms,
                         cudaStream_t st);

}  // namespace nn
}  // namespace hg
