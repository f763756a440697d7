// noalloc.cu -- hydro_gpu_stencil_solve_noalloc: the stencil solve of
// hydro_gpu_stencil_solve for callers that cannot allocate device memory.
//
// Its scratch (the CG vectors, reduction partials and device scalars the
// workspace of hydro_gpu_stencil_solve holds) lives in g_noalloc_scratch,
// a file-scope device array of this library: every GPU that loads the
// library holds it until the process exits.  Host code cannot pass the
// array's name to a kernel (on the host that name is only a stand-in, not a
// device address), so every call looks the address up with
// cudaGetSymbolAddress, with the calling device and context current.  The
// address belongs to a CUDA context, not to a device number: a lookup per
// call stays right after cudaDeviceReset or when the host application
// makes its own context current, where a cached address would point into
// a context that no longer exists.  The lookup is a host-side table query
// and allocates nothing.
#include <cuda_runtime.h>

#include "../../include/hydro_gpu.h"
#include "kernels.h"
#include "loop.cuh"

namespace {

// Size of the workspace hydro_gpu_stencil_solve carves for
// HYDRO_NOALLOC_MAX_CELLS cells: 7 vectors of doubles, 4 x kMaxBlocks
// reduction partials, the device scalars, 256-byte alignment of each piece.
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kScratchBytes =
    7 * align_up(sizeof(double) * (size_t)HYDRO_NOALLOC_MAX_CELLS) +
    align_up(sizeof(double) * 4 * (size_t)hg::kMaxBlocks) + align_up(sizeof(hg::DevScalars)) +
    2 * kAlign;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch in the current context.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return HYDRO_ERR_NO_DEVICE;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return HYDRO_ERR_CUDA;
  }
  *out = p;
  return HYDRO_OK;
}

}  // namespace

static_assert(kScratchBytes == 18875392, "header states the scratch size");

extern "C" int hydro_gpu_stencil_solve_noalloc(int dim, int nx, int ny, int nz,
                                               const double* face_coeff, double shift,
                                               long pinned_cell, double pinned_value,
                                               const double* rhs, double* x, int use_guess,
                                               double tolerance, int iters_limit, void* stream,
                                               int* iterations, double* residual) {
  if (dim != 2 && dim != 3) return HYDRO_ERR_ARG;
  if (nx < 2 || ny < 2 || (dim == 3 && nz < 2)) return HYDRO_ERR_ARG;
  long long cells = (long long)nx * ny * (dim == 3 ? nz : 1);
  if (cells > HYDRO_NOALLOC_MAX_CELLS) return HYDRO_ERR_ARG;
  size_t need = hydro_gpu_stencil_workspace_size(dim, nx, ny, dim == 3 ? nz : 1);
  if (need == 0 || need > kScratchBytes) return HYDRO_ERR_ARG;
  void* ws = nullptr;
  int rc = scratch_address(&ws);
  if (rc != HYDRO_OK) return rc;
  // hydro_gpu_stencil_solve clears the device scalars it needs at zero
  // (reduction tickets, flags) at the start of every call; the vectors are
  // fully written before they are read.
  return hydro_gpu_stencil_solve(dim, nx, ny, nz, face_coeff, shift, pinned_cell, pinned_value,
                                 rhs, x, use_guess, tolerance, iters_limit, ws, stream,
                                 iterations, residual);
}
