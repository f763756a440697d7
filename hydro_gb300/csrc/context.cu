// context.cu -- the C-ABI of include/hydro_gpu.h and the host-side
// orchestration (C++) of the hot path on one GPU:
//   FluidSimple::StartStep / MakeIteration / FinishStep (fluid.hpp:793-1169)
//   AdvectionSolverMultiExplicit substeps (advection.hpp:417-545,
//     hydro2d.hpp:1596-1604)
//   hydro<Mesh>::UpdateFluidProperties / CalcStat / step (hydro2d.hpp:1404-1621)
//
// All fields live in one device arena owned by the context; host arrays are
// copied only by set_field/get_field.  Inner loops (momentum sweeps, CG
// iterations) are queued in chunks; kernels stop themselves once the
// device-side convergence flag is set and the host reads the flags once per
// chunk, so the GPU never waits on the host between iterations of a chunk.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <new>
#include <unordered_map>
#include <utility>
#include <array>
#include <vector>

#include "../../include/hydro_gpu.h"
#include "../../include/hydro_net.h"
#include "kernels.h"

// the network of the learned pressure guess (net.cu)
int net_predict_async(hydro_net* net, const double* rhs, const double* rho, double rho_scale,
                      double* out, cudaStream_t st);
int net_check_grid(const hydro_net* net, int dim, const int* n);
int net_error(hydro_net* net, cudaStream_t st);
#include "loop.cuh"

using namespace hg;

namespace hg {
static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_total() { return g_launches.load(); }

int resident_ctas(const void* kernel) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(kernel);
  if (it != cache.end()) return it->second;
  int dev = 0, sms = 0, per_sm = 0;
  int r = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, 0) == cudaSuccess)
    r = per_sm * sms;
  cache[kernel] = r;
  return r;
}
}  // namespace hg

namespace {

// CUDA-event timing of kernel groups (hydro_gpu_set_profiling).
struct EventProfiler : Profiler {
  bool on = false;
  cudaEvent_t open = nullptr;
  struct Pair {
    int g;
    cudaEvent_t a, b;
  };
  std::vector<Pair> pending;
  std::vector<cudaEvent_t> pool;
  long long launches[HYDRO_PROF_COUNT] = {};
  double ms[HYDRO_PROF_COUNT] = {};
  cudaEvent_t get() {
    if (pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  void begin(int, cudaStream_t st) override {
    if (!on) return;
    if (open) pool.push_back(open);  // an inner group replaces an open outer one
    open = get();
    cudaEventRecord(open, st);
  }
  void end(int g, cudaStream_t st) override {
    if (!on || !open) return;
    cudaEvent_t e = get();
    cudaEventRecord(e, st);
    pending.push_back({g, open, e});
    open = nullptr;
  }
  // after a stream synchronisation: fold finished pairs into the totals
  void collect() {
    for (auto& p : pending) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
        launches[p.g] += 1;
        ms[p.g] += t;
      }
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
  }
  void reset() {
    for (int g = 0; g < HYDRO_PROF_COUNT; ++g) {
      launches[g] = 0;
      ms[g] = 0.;
    }
  }
  // bracketed launches that found the solve converged and exited at once
  // (queued past convergence by the chunked host loop): kept in the time,
  // taken out of the count
  void uncount(int g, long long n) {
    if (on && n > 0) launches[g] -= n;
  }
  ~EventProfiler() {
    for (auto& p : pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
    if (open) cudaEventDestroy(open);
  }
};

constexpr int kSweepChunk = 8;
constexpr int kCgChunk = 32;
constexpr int kMgChunk = 4;

struct Arena {
  char* base = nullptr;
  size_t used = 0, cap = 0;
  template <class T>
  T* take(size_t n) {
    size_t bytes = ((n * sizeof(T)) + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

}  // namespace

struct hydro_ctx {
  hydro_desc d;
  Mesh m;
  int dim = 2, nph = 1;
  int device = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  Arena arena;
  // fluid layers (solver::Layers order); vector fields component-major
  double* u[4] = {};
  double* p[4] = {};
  double* F[4] = {};
  // mixture fields (hydro2d.hpp:449-463)
  double *rho = nullptr, *mu = nullptr, *rho_raw = nullptr, *smtmp = nullptr;
  double *force = nullptr, *stforce = nullptr, *Sv = nullptr, *Sm = nullptr;
  // phases
  double *q = nullptr, *qtmp = nullptr, *alpha = nullptr, *qflux = nullptr;
  // iteration work
  double *G = nullptr, *fo = nullptr, *fres = nullptr, *coef = nullptr, *res = nullptr;
  double* du[2] = {};
  // mixed path: FP32 momentum coefficients/residuals and Jacobi iterates
  float* o32 = nullptr;
  float* du32[2] = {};
  FP<10> o32p() {
    FP<10> r{};
    if (!o32) return r;
    int w = 2 * dim + 1;
    for (int q = 0; q < w; ++q) r.a[q] = o32 + (size_t)q * m.nc;
    for (int k = 0; k < dim; ++k) r.a[7 + k] = o32 + (size_t)(w + k) * m.nc;
    return r;
  }
  double *Dc = nullptr, *Fs = nullptr, *kf = nullptr, *pc = nullptr, *prhs = nullptr;
  double* gp = nullptr;  // FP64 cell pressure gradient of the iteration
  // boundary conditions: per-face velocity of the value condition (dim face
  // arrays; walls and inlets fixed, outlets refreshed every iteration), its
  // FP32 mirror for the mixed path, inlet partial densities per phase
  BcSpec bc{};
  double* bcu = nullptr;
  float* bcu32 = nullptr;
  unsigned char* exmask = nullptr;  // excluded cells (rigid box), device
  double* qin = nullptr;
  int inlet_mask = 0, has_outlet = 0;
  // mixed path: FP32 shadows of the state and mixture fields read by the
  // FP32 SIMPLE-iteration kernels (refreshed at StartStep, the iterate by
  // the correction kernel) and their FP32 work arrays
  struct Shadow32 {
    float* u[4] = {};  // per layer, component-major
    float* F[4] = {};  // iteration layers only
    float *rho = nullptr, *mu = nullptr, *force = nullptr, *stforce = nullptr;
    float *Sv = nullptr, *Sm = nullptr;
    float *G = nullptr, *fo = nullptr, *fres = nullptr, *Dc = nullptr;
  } s32;
  bool mixed = false;
  // momentum solver: red-black Gauss-Seidel (velocity_solver GAUSS_SEIDEL;
  // the FP32 path then stores its rows color-blocked, which needs an even
  // Nx) or Jacobi
  bool mom_gs = false;
  bool mom_split64 = false;
  // graph-captured step (hydro_gpu_step_graph): capture state and the
  // instantiated step with the values it was captured for
  bool graph_mode = false;
  cudaGraph_t cap_graph = nullptr;
  cudaStream_t cap_streams[4] = {};
  int cap_depth = 0;
  // kernel counts of a capture: per nesting level (0: the graph itself)
  // the launch counter at its start and the kernels of the bodies nested
  // in it; kernels a graph launch runs outside any body; the device body
  // counter (RS_KEXEC) as last read
  long long cap_start[5] = {}, cap_nested[5] = {};
  long long graph_top = 0;
  double kexec_seen = 0.;
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    double dt = -1., adv_dt = -1.;
    int substeps = -1, sources = -1, heat_gen = -1;
    // the time and iteration layers the graph was captured on: a
    // host-driven step rotates them, after which the graph is captured
    // again
    std::array<const void*, 30> layers{};
  } sg;
  // temperature (HeatSolver, heat.hpp:18-94; hydro_gpu_heat_create): its
  // two time layers and the mixture conductivity; the step's gradient,
  // rows and Jacobi iterates use the momentum work arrays G, coef, res and
  // du, free once the fluid step has finished
  struct HeatState {
    bool on = false;
    int gen = 0;  // bumped by every hydro_gpu_heat_create
    hydro_heat_desc hd{};
    HeatBc bc{};
    HeatCoef hc{};
    double* mem = nullptr;
    double *tc = nullptr, *tp = nullptr, *kc = nullptr;
  } heat;
  PcgWork pw{};
  double* stat_out = nullptr;
  unsigned* stat_ticket = nullptr;
  DevScalars* hds = nullptr;  // pinned host mirror
  // scalars
  double time = 0., dt = 0., adv_time = 0., adv_dt = 0.;
  int iter_count = 0, cd_iter_count = 0;
  int vel_sweeps = 0, p_iters = 0;
  int p_unconv = 0;  // pressure solves of the step that stopped above their tolerance
  // learned initial guess of the first net_iters pressure solves of a step
  hydro_net* net = nullptr;
  int net_iters = 0;
  double net_rho_scale = 1.;
  bool guess_off = false;  // host-driven step: this step skips the guess (back-off)
  double p_res = 0., indicator = 1.;
  int du_cur = 0;
  int status = HYDRO_OK;
  FluidCoef fc{};
  PhaseProps pp{};
  EventProfiler prof;
  MgWork mg{};

  double* ucomp(int layer, int k) { return u[layer] + (size_t)k * m.nc; }
  C3 uc3(int layer) {
    C3 r{};
    for (int k = 0; k < 3; ++k) r.a[k] = k < dim ? ucomp(layer, k) : nullptr;
    return r;
  }
  W3 uw3(int layer) {
    W3 r{};
    for (int k = 0; k < 3; ++k) r.a[k] = k < dim ? ucomp(layer, k) : nullptr;
    return r;
  }
  template <class P>
  P vec(double* base, int n, long long stride) {
    P r{};
    for (int k = 0; k < n; ++k) r.a[k] = base + (size_t)k * stride;
    return r;
  }
  // FP32 component table over arrays of stride `stride`
  FP<3> vf3f(float* base, long long stride) {
    FP<3> r{};
    for (int k = 0; k < dim; ++k) r.a[k] = base + (size_t)k * stride;
    return r;
  }
  // FP32 component tables over nc-strided arrays
  template <class P>
  P vf(float* base, int n) {
    P r{};
    for (int k = 0; k < n && base; ++k) r.a[k] = base + (size_t)k * m.nc;
    return r;
  }
};

namespace {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return HYDRO_OK;
  if (e == cudaErrorMemoryAllocation) return HYDRO_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return HYDRO_ERR_NO_DEVICE;
  return HYDRO_ERR_CUDA;
}

#define CK(expr)                              \
  do {                                        \
    cudaError_t e_ = (expr);                  \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

// CK with the launch bracketed by the profiler's events for `group`.
#define PK(x, group, expr)                         \
  do {                                             \
    (x)->prof.begin(group, (x)->st);               \
    cudaError_t e_ = (expr);                       \
    (x)->prof.end(group, (x)->st);                 \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

int init_mesh(Mesh& m, int dim, const int* n, const double* lo, const double* hi) {
  memset(&m, 0, sizeof(m));
  if (dim != 2 && dim != 3) return HYDRO_ERR_ARG;
  m.dim = dim;
  for (int d = 0; d < 3; ++d) {
    m.n[d] = d < dim ? n[d] : 1;
    if (d < dim && m.n[d] < 2) return HYDRO_ERR_ARG;
    m.lo[d] = d < dim ? lo[d] : 0.;
    m.h[d] = d < dim ? (hi[d] - lo[d]) / (double)n[d] : 1.;
    if (d < dim && !(m.h[d] > 0.)) return HYDRO_ERR_ARG;
  }
  m.nc = (long long)m.n[0] * m.n[1] * m.n[2];
  long long off = 0;
  for (int d = 0; d < 3; ++d) {
    m.fnx[d] = m.n[0] + (d == 0);
    m.fny[d] = m.n[1] + (d == 1);
    m.fofs[d] = off;
    if (d < dim) off += (long long)m.fnx[d] * m.fny[d] * (m.n[2] + (d == 2));
  }
  m.nf = off;
  m.nfluid = m.nc;
  m.V = 1.;
  for (int d = 0; d < dim; ++d) m.V *= m.h[d];
  for (int d = 0; d < 3; ++d) m.A[d] = d < dim ? m.V / m.h[d] : 0.;
  return HYDRO_OK;
}

// GetDerivativeApproxCoeffs(0, {-2dt, -dt, 0}, skip) (solver.hpp:815-861).
void bdf_coeffs(double dt, int second, double* co) {
  double args[3] = {-2. * dt, -dt, 0.};
  int skip = second ? 0 : 1;
  int sz = 3 - skip;
  co[0] = co[1] = co[2] = 0.;
  for (int i = 0; i < sz; ++i) {
    double denom = 1., numer = 0.;
    for (int j = 0; j < sz; ++j) {
      if (j == i) continue;
      denom *= args[skip + i] - args[skip + j];
      double term = 1.;
      for (int k = 0; k < sz; ++k)
        if (k != i && k != j) term *= 0. - args[skip + k];
      numer += term;
    }
    co[skip + i] = numer / denom;
  }
}

int sync_scalars(hydro_ctx* x) {
  CK(cudaMemcpyAsync(x->hds, x->pw.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, x->st));
  CK(cudaStreamSynchronize(x->st));
  x->prof.collect();
  return HYDRO_OK;
}

int reset_flags(hydro_ctx* x, int first, int count) {
  CK(cudaMemsetAsync(&x->pw.ds->flag[first], 0, sizeof(int) * count, x->st));
  return HYDRO_OK;
}

// ------------------------------------------------- graph-captured loops --
// Conditional handles belong to the top-level graph being captured.
int new_handle(hydro_ctx* x, unsigned def, cudaGraphConditionalHandle* h) {
  CK(cudaGraphConditionalHandleCreate(h, x->cap_graph, def, cudaGraphCondAssignDefault));
  return HYDRO_OK;
}

// Kernels of the body being captured up to and including the next launch
// (its closing control kernel), bodies nested in it excluded.
int body_kernels(const hydro_ctx* x) {
  return (int)(launch_total() + 1 - x->cap_start[x->cap_depth] - x->cap_nested[x->cap_depth]);
}

// Adds a WHILE (or IF) node after the work captured so far on x->st and
// captures `body` into it on the next capture stream.
template <class Body>
int add_conditional(hydro_ctx* x, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    Body body) {
  if (x->cap_depth >= 4) return HYDRO_ERR_UNSUPPORTED;
  cudaStream_t outer = x->st;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(outer, &cs, nullptr, &g, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive) return HYDRO_ERR_CUDA;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  CK(cudaStreamUpdateCaptureDependencies(outer, &node, nullptr, 1,
                                         cudaStreamSetCaptureDependencies));
  cudaGraph_t bg = p.conditional.phGraph_out[0];
  cudaStream_t inner = x->cap_streams[x->cap_depth++];
  x->cap_start[x->cap_depth] = launch_total();
  x->cap_nested[x->cap_depth] = 0;
  CK(cudaStreamBeginCaptureToGraph(inner, bg, nullptr, nullptr, 0,
                                   cudaStreamCaptureModeRelaxed));
  x->st = inner;
  int rc = body();
  x->st = outer;
  cudaGraph_t done = nullptr;
  cudaError_t e = cudaStreamEndCapture(inner, &done);
  const long long inner_kernels = launch_total() - x->cap_start[x->cap_depth];
  x->cap_depth--;
  x->cap_nested[x->cap_depth] += inner_kernels;
  if (rc) return rc;
  CK(e);
  return HYDRO_OK;
}
template <class Body>
int add_while(hydro_ctx* x, cudaGraphConditionalHandle h, Body body) {
  return add_conditional(x, h, cudaGraphCondTypeWhile, body);
}
// A WHILE loop entered with its condition set (a handle's default value is
// applied only once per launch, not on each entry into an enclosing body).
template <class Body>
int add_loop(hydro_ctx* x, cudaGraphConditionalHandle h, Body body) {
  CK(launch_set_cond(h, 1u, x->st));
  return add_conditional(x, h, cudaGraphCondTypeWhile, body);
}
template <class Body>
int add_if(hydro_ctx* x, cudaGraphConditionalHandle h, Body body) {
  return add_conditional(x, h, cudaGraphCondTypeIf, body);
}

// ------------------------------------------------------------- momentum --
// Jacobi sweeps until the device flags convergence or `limit` sweeps
// (do { } while (iter++ < limit)); sweep k reads du[(k+1)%2], writes du[k%2].
int solve_momentum(hydro_ctx* x) {
  const hydro_desc& d = x->d;
  int dim = x->dim;
  CP<7> cc = x->vec<CP<7>>(x->coef, 2 * dim + 1, x->m.nc);
  C3 resc = x->vec<C3>(x->res, dim, x->m.nc);
  int rc = reset_flags(x, FL_MOM_DONE, 2);
  if (rc) return rc;
  const int limit = d.velocity_iters_limit + 1;
  const bool f32 = x->o32 != nullptr;
  auto fp3 = [&](float* base) {
    FP<3> r{};
    for (int k = 0; k < dim; ++k) r.a[k] = base + (size_t)k * x->m.nc;
    return r;
  };
  if (x->mom_gs) {
    // red-black Gauss-Seidel, in place on du[0] / du32[0]
    auto gs_sweep = [&]() -> int {
      for (int color = 0; color < 2; ++color) {
        if (f32)
          PK(x, HYDRO_PROF_MOM_SWEEP,
             launch_mom_rbgs32(x->m, d.velocity_omega, d.velocity_tolerance, x->o32p(),
                               fp3(x->du32[0]), color, limit, x->pw.partials, x->pw.ds, x->st));
        else
          PK(x, HYDRO_PROF_MOM_SWEEP,
             launch_mom_rbgs(x->m, d.velocity_omega, d.velocity_tolerance, cc, resc,
                             x->vec<W3>(x->du[0], dim, x->m.nc), color, x->mom_split64 ? 1 : 0,
                             limit, x->pw.partials, x->pw.ds, x->st));
      }
      return HYDRO_OK;
    };
    x->du_cur = 0;
    if (x->graph_mode) {
      cudaGraphConditionalHandle h;
      if ((rc = new_handle(x, 1, &h))) return rc;
      rc = add_loop(x, h, [&]() -> int {
        int r;
        if ((r = gs_sweep()) || (r = gs_sweep())) return r;
        CK(launch_ctl_sweeps(x->pw.ds, limit, h, 1, x->st, body_kernels(x)));
        return HYDRO_OK;
      });
      if (rc) return rc;
    } else {
      int queued = 0;
      for (;;) {
        int n = std::min(kSweepChunk, limit - queued);
        for (int s = 0; s < n; ++s)
          if ((rc = gs_sweep())) return rc;
        queued += n;
        rc = sync_scalars(x);
        if (rc) return rc;
        if (x->hds->flag[FL_MOM_DONE] || queued >= limit) break;
      }
      x->vel_sweeps += x->hds->flag[FL_MOM_SWEEPS];
    }
    if (f32) {
      // the FP32 corrections are color-blocked: cell order in du32[1] for the
      // Rhie-Chow and correction kernels
      CK(launch_unsplit3(x->m, fp3(x->du32[0]), fp3(x->du32[1]), x->st));
      x->du_cur = 1;
    }
    return HYDRO_OK;
  }
  if (f32 && d.cta_threads > 0) {
    // the whole Jacobi loop by one CTA
    CK(launch_cta_mom_jacobi32(x->m, d.velocity_omega, d.velocity_tolerance, x->o32p(),
                               fp3(x->du32[0]), fp3(x->du32[1]), limit, x->graph_mode ? 1 : 0,
                               d.cta_threads, d.cta_cluster > 1 ? d.cta_cluster : 1, x->pw.ds,
                               x->st));
    if (x->graph_mode) {
      const long long n = x->m.nc * dim;
      CK(launch_select_sweep(n, nullptr, x->du[0], x->du32[1], x->du32[0], x->pw.ds, x->st));
      x->du_cur = 0;
      return HYDRO_OK;
    }
    rc = sync_scalars(x);
    if (rc) return rc;
    const int sweeps = x->hds->flag[FL_MOM_SWEEPS];
    x->vel_sweeps += sweeps;
    x->du_cur = sweeps > 0 ? (sweeps - 1) % 2 : 0;
    return HYDRO_OK;
  }
  auto sweep = [&](int k) -> int {
    if (f32) {
      PK(x, HYDRO_PROF_MOM_SWEEP,
         launch_mom_sweep32(x->m, d.velocity_omega, d.velocity_tolerance, x->o32p(),
                            fp3(x->du32[(k + 1) % 2]), fp3(x->du32[k % 2]), limit,
                            x->pw.partials, x->pw.ds, x->st));
    } else {
      C3 din = x->vec<C3>(x->du[(k + 1) % 2], dim, x->m.nc);
      W3 dout = x->vec<W3>(x->du[k % 2], dim, x->m.nc);
      PK(x, HYDRO_PROF_MOM_SWEEP,
         launch_mom_sweep(x->m, d.velocity_omega, d.velocity_tolerance, cc, resc, din, dout,
                          limit, x->pw.partials, x->pw.ds, x->st));
    }
    return HYDRO_OK;
  };
  if (x->graph_mode) {
    cudaGraphConditionalHandle h;
    if ((rc = new_handle(x, 1, &h))) return rc;
    rc = add_loop(x, h, [&]() -> int {
      int r;
      if ((r = sweep(0)) || (r = sweep(1))) return r;
      CK(launch_ctl_sweeps(x->pw.ds, limit, h, 1, x->st, body_kernels(x)));
      return HYDRO_OK;
    });
    if (rc) return rc;
    // the correction always ends in du[0] / du32[0]
    const long long n = x->m.nc * dim;
    CK(launch_select_sweep(n, f32 ? nullptr : x->du[1], x->du[0], f32 ? x->du32[1] : nullptr,
                           x->du32[0], x->pw.ds, x->st));
    x->du_cur = 0;
    return HYDRO_OK;
  }
  int queued = 0;
  for (;;) {
    int n = std::min(kSweepChunk, limit - queued);
    for (int s = 0; s < n; ++s)
      if ((rc = sweep(queued + s))) return rc;
    queued += n;
    rc = sync_scalars(x);
    if (rc) return rc;
    if (x->hds->flag[FL_MOM_DONE] || queued >= limit) break;
  }
  int sweeps = x->hds->flag[FL_MOM_SWEEPS];
  x->vel_sweeps += sweeps;
  x->du_cur = (sweeps - 1) % 2;
  // mixed path: the Rhie-Chow and correction kernels read du32 directly
  return HYDRO_OK;
}

// ----------------------------------------------------------------- heat --
// One HeatSolver step (StartStep, one MakeIteration, FinishStep): rows of
// the temperature equation around T_curr, Jacobi sweeps to the heat
// tolerance (a WHILE node in a captured step, chunks between host checks
// otherwise), then T_prev <- T_curr <- T_curr + correction.
int heat_step(hydro_ctx* x) {
  const Mesh& m = x->m;
  auto& h = x->heat;
  const int dim = x->dim;
  int rc = reset_flags(x, FL_HEAT_DONE, 2);
  if (rc) return rc;
  CK(launch_heat_grad(m, h.bc, h.tc, x->vec<W3>(x->G, dim, m.nc), x->st));
  CK(launch_heat_assemble(m, h.bc, h.hc, h.tc, h.tc, h.tp, x->F[HYDRO_ITER_CURR], h.kc,
                          x->vec<C3>(x->G, dim, m.nc), x->vec<WP<7>>(x->coef, 2 * dim + 1, m.nc),
                          x->res, x->st));
  CP<7> cc = x->vec<CP<7>>(x->coef, 2 * dim + 1, m.nc);
  const int limit = h.hd.iters_limit + 1;
  auto sweep = [&](int k) -> int {
    CK(launch_heat_sweep(m, h.hd.tolerance, cc, x->res, x->du[(k + 1) % 2], x->du[k % 2], limit,
                         x->pw.partials, x->pw.ds, x->st));
    return HYDRO_OK;
  };
  if (x->graph_mode) {
    cudaGraphConditionalHandle hc;
    if ((rc = new_handle(x, 1, &hc))) return rc;
    rc = add_loop(x, hc, [&]() -> int {
      int r;
      if ((r = sweep(0)) || (r = sweep(1))) return r;
      CK(launch_ctl_heat(x->pw.ds, limit, hc, 1, x->st, body_kernels(x)));
      return HYDRO_OK;
    });
    if (rc) return rc;
  } else {
    int queued = 0;
    for (;;) {
      int n = std::min(kSweepChunk, limit - queued);
      for (int s = 0; s < n; ++s)
        if ((rc = sweep(queued + s))) return rc;
      queued += n;
      if ((rc = sync_scalars(x))) return rc;
      if (x->hds->flag[FL_HEAT_DONE] || queued >= limit) break;
    }
  }
  CK(launch_heat_finish(m.nc, h.tc, h.tp, x->du[0], x->du[1], x->pw.ds, x->st));
  return HYDRO_OK;
}

// ------------------------------------------------------------- pressure --
// The network's initial guess of the refinement iterate x->pc, after the
// residual of the zero guess (RS_IR_RR = ||f'||^2) has been reduced:
// predict, project (singular), Galerkin-scale, its residual, keep or drop.
int apply_guess(hydro_ctx* x, int singular) {
  const Mesh& m = x->m;
  PcgWork& w = x->pw;
  CK(launch_store_ff(w.ds, x->st));
  int rc = net_predict_async(x->net, x->prhs, x->rho, x->net_rho_scale, x->pc, x->st);
  if (rc) return rc;
  if (singular) CK(sub_mean(m, x->pc, w, x->st));
  CK(guess_scale(m, x->kf, x->prhs, x->pc, singular, w, x->st));
  CK(ir_residual(m, x->kf, x->prhs, x->pc, singular, w, x->st));
  CK(guess_accept(m, x->prhs, x->pc, singular, w, x->st));
  return HYDRO_OK;
}

// Graph-captured form of the pressure solve: the refinement and Krylov loops
// become WHILE nodes steered by the control kernels.
int solve_pressure_graph(hydro_ctx* x, int singular, int mixed, bool apply_pin_guess) {
  const hydro_desc& d = x->d;
  const Mesh& m = x->m;
  PcgWork& w = x->pw;
  int rc;
  if (!mixed) {
    w.limit = d.pressure_iters_limit;
    CK(pcg_init(m, x->kf, x->prhs, x->pc, 0, d.pressure_tolerance, singular, w, x->st));
    cudaGraphConditionalHandle h;
    if ((rc = new_handle(x, 1, &h))) return rc;
    rc = add_loop(x, h, [&]() -> int {
      CK(pcg_iterate(m, x->kf, x->pc, 4, w, x->st));
      CK(launch_ctl_krylov(w.ds, h, 1, x->st, body_kernels(x)));
      return HYDRO_OK;
    });
    if (rc) return rc;
    CK(launch_ctl_krylov_done(w.ds, x->st));
  } else {
    const bool mgcg = d.pressure_solver == HYDRO_LINEAR_MGCG;
    const double inner_min = mgcg ? 1e-5 : 1e-4;
    if (mgcg) CK(mg_setup(x->mg, w, x->st));
    if (singular) CK(mean_sum(m, x->prhs, w, x->st));
    CK(cudaMemsetAsync(x->pc, 0, sizeof(double) * m.nc, x->st));
    if ((rc = reset_flags(x, FL_IR_STATE, 1))) return rc;
    cudaGraphConditionalHandle hr, hk;
    if ((rc = new_handle(x, 0, &hr))) return rc;
    if ((rc = new_handle(x, 1, &hk))) return rc;
    CK(ir_residual(m, x->kf, x->prhs, nullptr, singular, w, x->st));
    CK(launch_ctl_refine(w.ds, d.pressure_tolerance, inner_min, d.pressure_iters_limit, hr, 1,
                         x->st));
    if (x->net && x->net_iters > 0 && apply_pin_guess) {
      // the learned guess, for the first net_iters SIMPLE iterations
      cudaGraphConditionalHandle hg2;
      if ((rc = new_handle(x, 0, &hg2))) return rc;
      CK(launch_ctl_guess_gate(w.ds, x->net_iters, hg2, 1, x->st));
      rc = add_if(x, hg2, [&]() -> int {
        int r;
        if ((r = apply_guess(x, singular))) return r;
        CK(launch_ctl_guess(w.ds, d.pressure_tolerance, inner_min, d.pressure_iters_limit, hr,
                            x->st, body_kernels(x)));
        return HYDRO_OK;
      });
      if (rc) return rc;
    }
    rc = add_while(x, hr, [&]() -> int {
      int r;
      if (mgcg) CK(mgcg_init(m, 0., 1, w, x->mg, x->st));
      else CK(f32_pcg_init(m, 0., 1, w, x->st));
      r = add_loop(x, hk, [&]() -> int {
        if (mgcg) CK(mgcg_iterate(m, 2, w, x->mg, x->st));
        else CK(f32_pcg_iterate(m, 4, w, x->st));
        CK(launch_ctl_krylov(w.ds, hk, 1, x->st, body_kernels(x)));
        return HYDRO_OK;
      });
      if (r) return r;
      if (mgcg) CK(mgcg_accumulate(m, x->pc, w, x->mg, x->st));
      else CK(f32_accumulate(m, x->pc, w, x->st));
      CK(ir_residual(m, x->kf, x->prhs, x->pc, singular, w, x->st));
      CK(launch_ctl_refine(w.ds, d.pressure_tolerance, inner_min, d.pressure_iters_limit, hr, 1,
                           x->st, body_kernels(x)));
      return HYDRO_OK;
    });
    if (rc) return rc;
  }
  if (singular) CK(sub_mean(m, x->pc, w, x->st));
  return HYDRO_OK;
}

// apply_pin = false: x->prhs is already the complete right-hand side (its
// pinned row included), as for the SIMPLER solve.
int solve_pressure(hydro_ctx* x, bool apply_pin = true) {
  const hydro_desc& d = x->d;
  const Mesh& m = x->m;
  int singular = (d.pressure_fixed_cell < 0);
  PcgWork& w = x->pw;
  w.pin = d.pressure_fixed_cell;
  if (w.pin >= 0 && apply_pin)
    CK(pin_rhs(m, x->kf, x->prhs, w.pin, d.pressure_fixed_value, x->st));
  // FP64 iterative refinement around an FP32 inner solve: the mixed path,
  // and the FP64 path with the multigrid preconditioner (the FP64 system is
  // still solved to the FP64 tolerance; only the inner corrections are FP32)
  int mixed = (d.precision == HYDRO_MIXED) || d.pressure_solver == HYDRO_LINEAR_MGCG;
  if (d.cta_threads > 0) {
    // the whole solve, its set-up (diagonals, coarse levels) included, by
    // one CTA or cluster
    CK(cta_pressure(m, x->kf, x->prhs, x->pc, singular, d.pressure_tolerance, 1e-5,
                    d.pressure_iters_limit, x->graph_mode ? 1 : 0, d.cta_threads,
                    d.cta_cluster > 1 ? d.cta_cluster : 1, w, x->mg, x->st));
    if (x->graph_mode) return HYDRO_OK;
    int rc = sync_scalars(x);
    if (rc) return rc;
    x->p_iters += x->hds->flag[FL_PCG_ITERS];
    x->p_res = x->hds->red[RS_P_RES];
    if (!x->hds->flag[FL_PCG_DONE]) {
      if (std::isnan(x->hds->red[RS_IR_RR])) return HYDRO_ERR_NAN;
      x->p_unconv++;
    }
    return HYDRO_OK;
  }
  CK(pcg_prepare(m, x->kf, 0., w, mixed, x->st));
  if (x->graph_mode) return solve_pressure_graph(x, singular, mixed, apply_pin);
  int rc;
  if (!mixed) {
    w.limit = d.pressure_iters_limit;
    PK(x, HYDRO_PROF_CG_INIT,
       pcg_init(m, x->kf, x->prhs, x->pc, 0, d.pressure_tolerance, singular, w, x->st));
    int queued = 0;
    for (;;) {
      int n = std::min(kCgChunk, std::max(1, d.pressure_iters_limit - queued));
      CK(pcg_iterate(m, x->kf, x->pc, n, w, x->st));
      queued += n;
      rc = sync_scalars(x);
      if (rc) return rc;
      if (x->hds->flag[FL_PCG_DONE] || queued >= d.pressure_iters_limit) break;
    }
    int it = x->hds->flag[FL_PCG_ITERS];
    x->p_iters += it;
    double ff = x->hds->red[RS_PCG_FF];
    x->p_res = ff > 0. ? sqrt(x->hds->red[RS_PCG_RR] / ff) : 0.;
    if (std::isnan(x->hds->red[RS_PCG_RR])) return HYDRO_ERR_NAN;
    if (!(x->hds->red[RS_PCG_RR] <= x->hds->red[RS_PCG_TOL2])) x->p_unconv++;
  } else {
    // FP64 iterative refinement around an FP32 PCG (Jacobi or multigrid
    // preconditioned)
    const bool mgcg = d.pressure_solver == HYDRO_LINEAR_MGCG;
    if (mgcg) CK(mg_setup(x->mg, w, x->st));
    if (singular) CK(mean_sum(m, x->prhs, w, x->st));
    CK(cudaMemsetAsync(x->pc, 0, sizeof(double) * m.nc, x->st));
    double ff = -1.;
    int total = 0;
    bool conv = false;
    const double inner_tol = mgcg ? 1e-5 : 1e-4;
    for (int outer = 0; outer < 50; ++outer) {
      CK(ir_residual(m, x->kf, x->prhs, outer ? x->pc : nullptr, singular, w, x->st));
      rc = sync_scalars(x);
      if (rc) return rc;
      double rr = x->hds->red[RS_IR_RR];
      if (std::isnan(rr)) return HYDRO_ERR_NAN;  // a NaN in the system (fluid.hpp:1164-1166)
      if (ff < 0.) ff = rr;
      bool guess = outer == 0 && apply_pin && x->net && x->iter_count < x->net_iters;
      if (guess) {
        // the back-off (the device flags as of the last read-back, which
        // follows the last guess): the same decision the gate kernel
        // applies on the device
        if (x->iter_count == 0) {
          x->guess_off = x->hds->flag[FL_GUESS_SKIP] > 0;
          CK(launch_ctl_guess_gate(w.ds, x->net_iters, cudaGraphConditionalHandle{}, 0, x->st));
        }
        guess = !x->guess_off && ff > 0.;
      }
      if (guess) {
        // start from the network's guess when it beats the zero guess
        x->prof.begin(HYDRO_PROF_GUESS, x->st);
        rc = apply_guess(x, singular);
        x->prof.end(HYDRO_PROF_GUESS, x->st);
        if (rc) return rc;
        if ((rc = sync_scalars(x))) return rc;
        rr = x->hds->red[RS_IR_RR];
      }
      x->p_res = ff > 0. ? sqrt(rr / ff) : 0.;
      if (ff == 0. || rr <= d.pressure_tolerance * d.pressure_tolerance * ff) {
        conv = true;
        break;
      }
      if (total >= d.pressure_iters_limit) break;
      w.limit = d.pressure_iters_limit - total;
      double tol = std::max(inner_tol, 0.5 * d.pressure_tolerance * sqrt(ff / rr));
      if (mgcg)
        PK(x, HYDRO_PROF_CG_INIT, mgcg_init(m, tol, 0, w, x->mg, x->st));
      else
        PK(x, HYDRO_PROF_CG_INIT, f32_pcg_init(m, tol, 0, w, x->st));
      int queued = 0;
      const int chunk = mgcg ? kMgChunk : kCgChunk;
      for (;;) {
        if (mgcg)
          CK(mgcg_iterate(m, chunk, w, x->mg, x->st));
        else
          CK(f32_pcg_iterate(m, chunk, w, x->st));
        queued += chunk;
        rc = sync_scalars(x);
        if (rc) return rc;
        if (x->hds->flag[FL_PCG_DONE] || queued >= w.limit) break;
      }
      if (mgcg) {
        // brackets: the start and `queued` iterations; V-cycles that ran: the
        // start and every iteration but a converging last one
        const int it = x->hds->flag[FL_PCG_ITERS];
        x->prof.uncount(HYDRO_PROF_MG_VCYCLE,
                        1 + queued - (x->hds->flag[FL_PCG_DONE] && it > 0 ? it : it + 1));
      }
      total += x->hds->flag[FL_PCG_ITERS];
      if (mgcg) CK(mgcg_accumulate(m, x->pc, w, x->mg, x->st));
      else CK(f32_accumulate(m, x->pc, w, x->st));
    }
    x->p_iters += total;
    if (!conv) x->p_unconv++;
  }
  if (singular) CK(sub_mean(m, x->pc, w, x->st));
  return HYDRO_OK;
}

int nan_check(hydro_ctx* x, const double* a, long long n) {
  CK(launch_nan_count(n, a, x->pw.partials, x->pw.ds, x->st));
  int rc = sync_scalars(x);
  if (rc) return rc;
  return x->hds->red[RS_NAN] > 0. ? HYDRO_ERR_NAN : HYDRO_OK;
}

int fluid_field(hydro_ctx* x, int field, int layer, double** ptr, long long* n) {
  const Mesh& m = x->m;
  if (layer < 0 || layer > 3) return HYDRO_ERR_ARG;
  *n = m.nc;
  switch (field) {
    case HYDRO_FIELD_VELOCITY: *ptr = x->u[layer]; *n = m.nc * x->dim; return HYDRO_OK;
    case HYDRO_FIELD_PRESSURE: *ptr = x->p[layer]; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_FLUX: *ptr = x->F[layer]; *n = m.nf; return HYDRO_OK;
    case HYDRO_FIELD_PARTIAL_DENSITY: *ptr = x->q; *n = m.nc * x->nph; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_FRACTION: *ptr = x->alpha; *n = m.nc * x->nph; return HYDRO_OK;
    case HYDRO_FIELD_DENSITY: *ptr = x->rho; return HYDRO_OK;
    case HYDRO_FIELD_VISCOSITY: *ptr = x->mu; return HYDRO_OK;
    case HYDRO_FIELD_FORCE: *ptr = x->force; *n = m.nc * x->dim; return HYDRO_OK;
    case HYDRO_FIELD_VOLUME_SOURCE: *ptr = x->Sv; return HYDRO_OK;
    case HYDRO_FIELD_MASS_SOURCE: *ptr = x->Sm; return HYDRO_OK;
    case HYDRO_FIELD_PRESSURE_CORRECTION: *ptr = x->pc; return HYDRO_OK;
    case HYDRO_FIELD_PRESSURE_RHS: *ptr = x->prhs; return HYDRO_OK;
    case HYDRO_FIELD_DIAG_COEFF: *ptr = x->Dc; return HYDRO_OK;
    case HYDRO_FIELD_SURFACE_FORCE: *ptr = x->stforce; *n = m.nc * x->dim; return HYDRO_OK;
    case HYDRO_FIELD_TEMPERATURE:
      if (!x->heat.on) return HYDRO_ERR_ARG;
      if (layer == HYDRO_TIME_CURR) { *ptr = x->heat.tc; return HYDRO_OK; }
      if (layer == HYDRO_TIME_PREV) { *ptr = x->heat.tp; return HYDRO_OK; }
      return HYDRO_ERR_ARG;
    case HYDRO_FIELD_CONDUCTIVITY:
      if (!x->heat.on) return HYDRO_ERR_ARG;
      *ptr = x->heat.kc;
      return HYDRO_OK;
  }
  return HYDRO_ERR_ARG;
}

}  // namespace

// ================================================================ C-ABI ==
extern "C" {

int hydro_gpu_create(const hydro_desc* desc, hydro_ctx** out) {
  if (!desc || !out) return HYDRO_ERR_ARG;
  *out = nullptr;
  // SIMPLER is built on the FP64 path (its equations are the FP64 rows)
  if (desc->simpler && desc->precision != HYDRO_FP64) return HYDRO_ERR_UNSUPPORTED;
  if (desc->simpler && desc->rhie_chow_factor == 0.) return HYDRO_ERR_ARG;
  if (desc->num_phases < 1 || desc->num_phases > HYDRO_MAX_PHASES) return HYDRO_ERR_ARG;
  for (int s = 0; s < 2 * desc->dim && s < 6; ++s)
    if (desc->bc_kind[s] < HYDRO_BC_WALL || desc->bc_kind[s] > HYDRO_BC_OUTLET)
      return HYDRO_ERR_ARG;
  if (desc->velocity_omega <= 0. || desc->velocity_relaxation_factor <= 0.)
    return HYDRO_ERR_ARG;
  // solvers the GPU does not have are substituted only on request
  {
    const int vs = desc->velocity_solver, ps = desc->pressure_solver;
    const bool v_ok = vs == HYDRO_LINEAR_GAUSS_SEIDEL || vs == HYDRO_LINEAR_JACOBI;
    const bool p_ok = ps == HYDRO_LINEAR_CG || ps == HYDRO_LINEAR_MGCG;
    const bool v_known = v_ok || vs == HYDRO_LINEAR_LU;
    const bool p_known = p_ok || ps == HYDRO_LINEAR_GAUSS_SEIDEL || ps == HYDRO_LINEAR_JACOBI ||
                         ps == HYDRO_LINEAR_LU;
    if (!v_known || !p_known) return HYDRO_ERR_ARG;
    if ((!v_ok || !p_ok) && !desc->substitute_solvers) return HYDRO_ERR_UNSUPPORTED;
  }
  if (desc->cta_cluster != 0 && desc->cta_cluster != 1 && desc->cta_cluster != 2 &&
      desc->cta_cluster != 4 && desc->cta_cluster != 8)
    return HYDRO_ERR_ARG;
  if (desc->cta_cluster > 1 && desc->cta_threads == 0) return HYDRO_ERR_ARG;
  if (desc->cta_threads != 0) {
    const int t = desc->cta_threads;
    if (t < 32 || t > 1024 || t % 32) return HYDRO_ERR_ARG;
    if (desc->precision != HYDRO_MIXED || desc->pressure_solver != HYDRO_LINEAR_MGCG ||
        desc->rigid_box)
      return HYDRO_ERR_UNSUPPORTED;
    for (int d = 0; d < desc->dim && d < 3; ++d)
      if (desc->periodic[d]) return HYDRO_ERR_UNSUPPORTED;
    long long cells = 1;
    for (int d = 0; d < desc->dim && d < 3; ++d) cells *= desc->n[d];
    if (cells >= (1LL << 24)) return HYDRO_ERR_UNSUPPORTED;  // one group's solve
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return HYDRO_ERR_NO_DEVICE;
  hydro_ctx* x = new (std::nothrow) hydro_ctx();
  if (!x) return HYDRO_ERR_NOMEM;
  x->d = *desc;
  int rc = init_mesh(x->m, desc->dim, desc->n, desc->lo, desc->hi);
  if (rc) { delete x; return rc; }
  for (int d = 0; d < desc->dim; ++d) {
    x->m.per[d] = desc->periodic[d] != 0;
    // red-black multigrid colouring needs an even count across a periodic end
    if (x->m.per[d] && desc->pressure_solver == HYDRO_LINEAR_MGCG && x->m.n[d] % 2) {
      delete x;
      return HYDRO_ERR_UNSUPPORTED;
    }
  }
  if (desc->pressure_fixed_cell >= x->m.nc) { delete x; return HYDRO_ERR_ARG; }
  // rigid box: cells whose centre lies in it (Rect::IsInside, inclusive)
  std::vector<unsigned char> exmask;
  if (desc->rigid_box) {
    if (desc->simpler) { delete x; return HYDRO_ERR_UNSUPPORTED; }
    exmask.assign((size_t)x->m.nc, 0);
    long long nex = 0;
    for (long long c = 0; c < x->m.nc; ++c) {
      long long r = c;
      int in = 1;
      for (int d = 0; d < 3; ++d) {
        long long i = r % x->m.n[d];
        r /= x->m.n[d];
        if (d >= desc->dim) continue;
        double xc = x->m.lo[d] + (i + 0.5) * x->m.h[d];
        if (xc < desc->rigid_box_lo[d] || desc->rigid_box_hi[d] < xc) in = 0;
      }
      exmask[(size_t)c] = (unsigned char)in;
      nex += in;
    }
    if (nex == x->m.nc ||
        (desc->pressure_fixed_cell >= 0 && exmask[(size_t)desc->pressure_fixed_cell])) {
      delete x;
      return HYDRO_ERR_ARG;
    }
    if (nex == 0) exmask.clear();
    x->m.nfluid = x->m.nc - nex;
  }
  const Mesh& m = x->m;
  x->dim = desc->dim;
  x->nph = desc->num_phases;
  x->mixed = desc->precision == HYDRO_MIXED;
  x->mom_gs = desc->velocity_solver == HYDRO_LINEAR_GAUSS_SEIDEL &&
              (!x->mixed || x->m.n[0] % 2 == 0);
  // FP64 rows color-blocked too, unless SIMPLER reads them in cell order
  x->mom_split64 = x->mom_gs && !x->mixed && !desc->simpler && x->m.n[0] % 2 == 0;
  cudaGetDevice(&x->device);
  if (desc->stream) {
    x->st = (cudaStream_t)desc->stream;
  } else {
    if (cudaStreamCreateWithFlags(&x->st, cudaStreamNonBlocking) != cudaSuccess) {
      delete x;
      return HYDRO_ERR_CUDA;
    }
    x->own_stream = true;
  }
  // arena layout
  long long nc = m.nc, nf = m.nf;
  int dim = x->dim, nph = x->nph;
  auto plan = [&](Arena& a) {
    for (int l = 0; l < 4; ++l) x->u[l] = a.take<double>(nc * dim);
    for (int l = 0; l < 4; ++l) x->p[l] = a.take<double>(nc);
    for (int l = 0; l < 4; ++l) x->F[l] = a.take<double>(nf);
    x->rho = a.take<double>(nc);
    x->mu = a.take<double>(nc);
    x->rho_raw = a.take<double>(nc);
    x->smtmp = a.take<double>(nc);
    x->force = a.take<double>(nc * dim);
    x->stforce = a.take<double>(nc * dim);
    x->Sv = a.take<double>(nc);
    x->Sm = a.take<double>(nc);
    x->q = a.take<double>(nc * nph);
    x->qtmp = a.take<double>(nc * nph);
    x->alpha = a.take<double>(nc * nph);
    x->qflux = a.take<double>(nf * nph);
    x->G = a.take<double>(nc * dim * dim);
    x->fo = a.take<double>(nc * dim);
    x->fres = a.take<double>(nc * dim);
    x->coef = a.take<double>(nc * (2 * dim + 1));
    x->res = a.take<double>(nc * dim);
    x->du[0] = a.take<double>(nc * dim);
    x->du[1] = a.take<double>(nc * dim);
    if (desc->precision == HYDRO_MIXED) {
      x->o32 = a.take<float>(nc * (2 * dim + 1 + dim));
      x->du32[0] = a.take<float>(nc * dim);
      x->du32[1] = a.take<float>(nc * dim);
      auto& s3 = x->s32;
      for (int l = 0; l < 4; ++l) s3.u[l] = a.take<float>(nc * dim);
      for (int l : {HYDRO_ITER_CURR, HYDRO_ITER_PREV}) s3.F[l] = a.take<float>(nf);
      s3.rho = a.take<float>(nc);
      s3.mu = a.take<float>(nc);
      s3.force = a.take<float>(nc * dim);
      s3.stforce = a.take<float>(nc * dim);
      s3.Sv = a.take<float>(nc);
      s3.Sm = a.take<float>(nc);
      s3.G = a.take<float>(nc * dim * dim);
      s3.fo = a.take<float>(nc * dim);
      s3.fres = a.take<float>(nc * dim);
      s3.Dc = a.take<float>(nc);
    }
    x->gp = a.take<double>(nc * dim);
    x->bcu = a.take<double>(nf * dim);
    x->exmask = exmask.empty() ? nullptr : a.take<unsigned char>(nc);
    if (desc->precision == HYDRO_MIXED) x->bcu32 = a.take<float>(nf * dim);
    x->qin = a.take<double>(nf * nph);
    x->Dc = a.take<double>(nc);
    x->Fs = a.take<double>(nf);
    x->kf = a.take<double>(nf);
    x->pc = a.take<double>(nc);
    x->prhs = a.take<double>(nc);
    PcgWork& w = x->pw;
    w.r = a.take<double>(nc);
    w.z = a.take<double>(nc);
    w.p = a.take<double>(nc);
    w.Ap = a.take<double>(nc);
    w.dg = a.take<double>(nc);
    w.idg = a.take<double>(nc);
    w.r32 = a.take<float>(nc);
    w.z32 = a.take<float>(nc);
    w.p32 = a.take<float>(nc);
    w.p32b = a.take<float>(nc);
    w.Ap32 = a.take<float>(nc);
    w.dg32 = a.take<float>(nc);
    w.idg32 = a.take<float>(nc);
    w.x32 = a.take<float>(nc);
    w.kf32 = a.take<float>(nf);
    w.partials = a.take<double>((size_t)12 * kMaxBlocks);
    // multigrid hierarchy (level 0 shares the FP32 CG arrays)
    MgWork& mg = x->mg;
    mg.nlev = desc->pressure_solver == HYDRO_LINEAR_MGCG ? mg_levels_for(m) : 0;
    mg.nsweep = 2;
    mg.coarse_sweeps = 8;
    mg.coarse_sweeps_large = 16;
    if (mg.nlev > 0) mg.lev[0].m = m;
    for (int l = 1; l < mg.nlev; ++l) {
      MgLevel& lv = mg.lev[l];
      lv.m = mg_coarse_mesh(mg.lev[l - 1].m);
      lv.kf = a.take<float>(lv.m.nf);
      lv.dg = a.take<float>(lv.m.nc);
      lv.idg = a.take<float>(lv.m.nc);
      lv.x = a.take<float>(lv.m.nc);
      lv.b = a.take<float>(lv.m.nc);
    }
    mg.cinv = mg.nlev >= 2 ? a.take<float>(kMgCoarseTarget * kMgCoarseTarget) : nullptr;
    // colour-blocked FP16 finest level (plain 3D block, even n[0])
    const bool plain = !m.per[0] && !m.per[1] && !m.per[2] && exmask.empty();
    if (mg.nlev >= 2 && m.dim == 3 && plain && m.n[0] % 2 == 0 && m.nc < (1LL << 30) &&
        !desc->cta_threads) {
      const long long n0 = m.n[0], n1 = m.n[1], n2 = m.n[2];
      mg.k16[0] = a.take<unsigned short>((n0 + 1) * n1 * n2);
      mg.k16[1] = a.take<unsigned short>(n0 * (n1 + 1) * n2);
      mg.k16[2] = a.take<unsigned short>(n0 * n1 * (n2 + 1));
      mg.idg0 = a.take<float>(nc);
    } else {
      mg.k16[0] = mg.k16[1] = mg.k16[2] = nullptr;
    }
    w.ds = a.take<DevScalars>(1);
    x->stat_out = a.take<double>(16);
    x->stat_ticket = a.take<unsigned>(4);
  };
  Arena probe;
  plan(probe);
  size_t bytes = probe.used;
  if (cudaMalloc(&x->arena.base, bytes) != cudaSuccess) {
    cudaGetLastError();
    if (x->own_stream) cudaStreamDestroy(x->st);
    delete x;
    return HYDRO_ERR_NOMEM;
  }
  x->arena.cap = bytes;
  plan(x->arena);
  if (cudaMallocHost(&x->hds, sizeof(DevScalars)) != cudaSuccess) {
    cudaFree(x->arena.base);
    if (x->own_stream) cudaStreamDestroy(x->st);
    delete x;
    return HYDRO_ERR_NOMEM;
  }
  if (cudaMemsetAsync(x->arena.base, 0, bytes, x->st) != cudaSuccess ||
      cudaStreamSynchronize(x->st) != cudaSuccess) {
    hydro_gpu_destroy(x);
    return HYDRO_ERR_CUDA;
  }
  if (x->exmask) {
    // the mask of the context's mesh; multigrid levels keep none (their
    // couplings carry the exclusion)
    if (cudaMemcpyAsync(x->exmask, exmask.data(), exmask.size(), cudaMemcpyHostToDevice,
                        x->st) != cudaSuccess ||
        cudaStreamSynchronize(x->st) != cudaSuccess) {
      hydro_gpu_destroy(x);
      return HYDRO_ERR_CUDA;
    }
    x->m.ex = x->exmask;
  }
  x->pw.pin = desc->pressure_fixed_cell;
  x->pw.prof = &x->prof;
  x->mg.cta = desc->cta_threads > 0;
  if (mg_prepare(x->mg) != cudaSuccess) {
    hydro_gpu_destroy(x);
    return HYDRO_ERR_CUDA;
  }
  if (x->mg.cta && x->mg.top >= x->mg.nlev) {
    // the one-CTA solve runs its coarse levels in shared memory
    hydro_gpu_destroy(x);
    return HYDRO_ERR_UNSUPPORTED;
  }
  for (int q = 0; q < 6; ++q) {
    // the sides of a periodic direction carry no condition
    const int kind =
        (q < 2 * dim && !x->m.per[q / 2]) ? desc->bc_kind[q] : HYDRO_BC_WALL;
    x->bc.kind[q] = kind;
    for (int k = 0; k < 3; ++k) x->bc.vel[q][k] = k < dim ? desc->bc_velocity[q][k] : 0.;
    if (kind == HYDRO_BC_INLET) x->inlet_mask |= 1 << q;
    if (kind == HYDRO_BC_OUTLET) x->has_outlet = 1;
  }
  if (launch_bc_fill(m, x->bc, x->vec<W3>(x->bcu, dim, m.nf),
                     x->bcu32 ? x->vf3f(x->bcu32, m.nf) : FP<3>{}, x->st) != cudaSuccess ||
      cudaStreamSynchronize(x->st) != cudaSuccess) {
    hydro_gpu_destroy(x);
    return HYDRO_ERR_CUDA;
  }
  // constants
  for (int s = 0; s < 6; ++s)
    for (int k = 0; k < 3; ++k) x->fc.bcu[s][k] = (k < dim) ? desc->bc_velocity[s][k] : 0.;
  x->fc.relax_u = desc->velocity_relaxation_factor;
  x->fc.relax_p = desc->pressure_relaxation_factor;
  x->fc.rc = desc->rhie_chow_factor;
  for (int k = 0; k < 3; ++k) x->fc.meshvel[k] = k < dim ? desc->meshvel[k] : 0.;
  x->fc.geometric = desc->force_geometric_average;
  x->fc.sources = 0;
  for (int i = 0; i < HYDRO_MAXPH; ++i) {
    x->pp.dens[i] = desc->density[i];
    x->pp.idens[i] = 1. / desc->density[i];
    x->pp.visc[i] = desc->viscosity[i];
  }
  for (int k = 0; k < 3; ++k) {
    x->pp.grav[k] = k < dim ? desc->gravity[k] : 0.;
    x->pp.f0[k] = k < dim ? desc->force[k] : 0.;
  }
  x->dt = desc->dt;
  x->adv_dt = desc->dt * desc->advection_dt_factor;
  *out = x;
  return HYDRO_OK;
}

int hydro_gpu_destroy(hydro_ctx* x) {
  if (!x) return HYDRO_OK;
  if (x->st) cudaStreamSynchronize(x->st);
  if (x->sg.exec) cudaGraphExecDestroy(x->sg.exec);
  mg_release(x->mg);
  for (auto& cs : x->cap_streams)
    if (cs) cudaStreamDestroy(cs);
  if (x->arena.base) cudaFree(x->arena.base);
  if (x->heat.mem) cudaFree(x->heat.mem);
  if (x->hds) cudaFreeHost(x->hds);
  if (x->own_stream && x->st) cudaStreamDestroy(x->st);
  delete x;
  return HYDRO_OK;
}

int hydro_gpu_get_desc(hydro_ctx* x, hydro_desc* d) {
  if (!x || !d) return HYDRO_ERR_ARG;
  *d = x->d;
  d->stream = (void*)x->st;
  return HYDRO_OK;
}

int hydro_gpu_get_stream(hydro_ctx* x, void** st) {
  if (!x || !st) return HYDRO_ERR_ARG;
  *st = (void*)x->st;
  return HYDRO_OK;
}

int hydro_gpu_get_time_step(hydro_ctx* x, double* dt) {
  if (!x || !dt) return HYDRO_ERR_ARG;
  *dt = x->dt;
  return HYDRO_OK;
}

int hydro_gpu_field_ptr(hydro_ctx* x, int field, int layer, double** ptr) {
  if (!x || !ptr) return HYDRO_ERR_ARG;
  long long n;
  return fluid_field(x, field, layer, ptr, &n);
}

int hydro_gpu_set_field(hydro_ctx* x, int field, int layer, const double* src, size_t n) {
  if (!x || !src) return HYDRO_ERR_ARG;
  double* p;
  long long len;
  int rc = fluid_field(x, field, layer, &p, &len);
  if (rc) return rc;
  if ((long long)n != len) return HYDRO_ERR_ARG;
  CK(cudaMemcpyAsync(p, src, sizeof(double) * n, cudaMemcpyHostToDevice, x->st));
  CK(cudaStreamSynchronize(x->st));
  // caller-supplied sources enter the force sum and the pressure rows
  // (fluid.hpp:861-869, 985-988)
  if (field == HYDRO_FIELD_VOLUME_SOURCE || field == HYDRO_FIELD_MASS_SOURCE) {
    for (size_t i = 0; i < n; ++i)
      if (src[i] != 0.) {
        x->fc.sources = 1;
        break;
      }
  }
  return HYDRO_OK;
}

int hydro_gpu_get_field(hydro_ctx* x, int field, int layer, double* dst, size_t n) {
  if (!x || !dst) return HYDRO_ERR_ARG;
  double* p;
  long long len;
  int rc = fluid_field(x, field, layer, &p, &len);
  if (rc) return rc;
  if ((long long)n != len) return HYDRO_ERR_ARG;
  CK(cudaMemcpyAsync(dst, p, sizeof(double) * n, cudaMemcpyDeviceToHost, x->st));
  CK(cudaStreamSynchronize(x->st));
  return HYDRO_OK;
}

int hydro_gpu_update_properties(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  const hydro_desc& d = x->d;
  int dim = x->dim;
  PK(x, HYDRO_PROF_PROPS, launch_props(m, x->nph, x->pp, x->vec<CP<HYDRO_MAXPH>>(x->q, x->nph, m.nc),
                  x->vec<WP<HYDRO_MAXPH>>(x->alpha, x->nph, m.nc), x->rho_raw, x->rho, x->mu,
                  x->vec<W3>(x->force, dim, m.nc), x->Sv, x->Sm, x->st));
  auto smooth = [&](double* a, int times) -> int {
    double* in = a;
    double* tmp = x->smtmp;
    for (int r = 0; r < times; ++r) {
      PK(x, HYDRO_PROF_PROPS, launch_smooth(m, in, tmp, x->st));
      std::swap(in, tmp);
    }
    if (in != a) CK(cudaMemcpyAsync(a, in, sizeof(double) * m.nc, cudaMemcpyDeviceToDevice, x->st));
    return HYDRO_OK;
  };
  int rc = smooth(x->rho, d.density_smooth_times);
  if (rc) return rc;
  rc = smooth(x->mu, d.viscosity_smooth_times);
  if (rc) return rc;
  if (x->nph >= 2 && d.sigma != 0.) {
    CK(launch_stforce(m, d.sigma, x->alpha + m.nc, x->vec<W3>(x->G, dim, m.nc),
                      x->vec<W3>(x->stforce, dim, m.nc), x->st));
  }
  for (int k = 0; k < dim; ++k) {
    rc = smooth(x->force + (size_t)k * m.nc, d.force_smooth_times);
    if (rc) return rc;
  }
  if (x->heat.on)
    CK(launch_heat_conductivity(m, x->nph, x->heat.hc,
                                x->vec<CP<HYDRO_MAXPH>>(x->alpha, x->nph, m.nc), x->heat.kc,
                                x->st));
  CK(cudaGetLastError());
  return HYDRO_OK;
}

int hydro_gpu_init_state(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  CK(cudaMemcpyAsync(x->u[HYDRO_TIME_PREV], x->u[HYDRO_TIME_CURR],
                     sizeof(double) * m.nc * x->dim, cudaMemcpyDeviceToDevice, x->st));
  CK(cudaMemsetAsync(x->p[HYDRO_TIME_CURR], 0, sizeof(double) * m.nc, x->st));
  CK(cudaMemsetAsync(x->p[HYDRO_TIME_PREV], 0, sizeof(double) * m.nc, x->st));
  CK(launch_qin_fill(m, x->bc, x->nph, x->vec<CP<HYDRO_MAXPH>>(x->q, x->nph, m.nc),
                     x->vec<WP<HYDRO_MAXPH>>(x->qin, x->nph, m.nf), x->st));
  CK(launch_init_flux(m, x->fc, x->uc3(HYDRO_TIME_CURR), x->vec<C3>(x->bcu, x->dim, m.nf),
                      x->F[HYDRO_TIME_CURR], x->st));
  CK(cudaMemcpyAsync(x->F[HYDRO_TIME_PREV], x->F[HYDRO_TIME_CURR], sizeof(double) * m.nf,
                     cudaMemcpyDeviceToDevice, x->st));
  x->time = 0.;
  x->adv_time = 0.;
  return hydro_gpu_update_properties(x);
}

int hydro_gpu_start_step(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  x->iter_count = 0;
  x->cd_iter_count = 0;
  x->vel_sweeps = 0;
  x->p_iters = 0;
  x->p_unconv = 0;
  x->p_res = 0.;
  x->indicator = 1.;
  bdf_coeffs(x->dt, x->d.time_second_order, x->fc.co);
  CK(launch_start_step(m, x->d.guess_extrapolation, x->uw3(HYDRO_ITER_CURR),
                       x->uc3(HYDRO_TIME_CURR), x->uc3(HYDRO_TIME_PREV), x->p[HYDRO_ITER_CURR],
                       x->p[HYDRO_TIME_CURR], x->p[HYDRO_TIME_PREV], x->F[HYDRO_ITER_CURR],
                       x->F[HYDRO_TIME_CURR], x->F[HYDRO_TIME_PREV], x->st));
  if (x->mixed) {
    // FP32 shadows of everything the FP32 iteration kernels read; the
    // iteration layers are kept current by the correction kernel
    auto& s3 = x->s32;
    const long long nu = m.nc * x->dim;
    CK(launch_d2f(nu, x->u[HYDRO_ITER_CURR], s3.u[HYDRO_ITER_CURR], x->st));
    CK(launch_d2f(nu, x->u[HYDRO_TIME_CURR], s3.u[HYDRO_TIME_CURR], x->st));
    CK(launch_d2f(nu, x->u[HYDRO_TIME_PREV], s3.u[HYDRO_TIME_PREV], x->st));
    CK(launch_d2f(m.nf, x->F[HYDRO_ITER_CURR], s3.F[HYDRO_ITER_CURR], x->st));
    CK(launch_d2f(m.nc, x->rho, s3.rho, x->st));
    CK(launch_d2f(m.nc, x->mu, s3.mu, x->st));
    CK(launch_d2f(nu, x->force, s3.force, x->st));
    CK(launch_d2f(nu, x->stforce, s3.stforce, x->st));
    if (x->fc.sources) {
      CK(launch_d2f(m.nc, x->Sv, s3.Sv, x->st));
      CK(launch_d2f(m.nc, x->Sm, s3.Sm, x->st));
    }
  }
  return HYDRO_OK;
}

int hydro_gpu_make_iteration(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  const hydro_desc& d = x->d;
  int dim = x->dim;
  // layer shift: iter_prev <- iter_curr (fluid.hpp:815-818, conv_diff.hpp:133)
  std::swap(x->p[HYDRO_ITER_CURR], x->p[HYDRO_ITER_PREV]);
  std::swap(x->F[HYDRO_ITER_CURR], x->F[HYDRO_ITER_PREV]);
  std::swap(x->u[HYDRO_ITER_CURR], x->u[HYDRO_ITER_PREV]);
  C3 up = x->uc3(HYDRO_ITER_PREV);
  const double* pip = x->p[HYDRO_ITER_PREV];
  const double* Fip = x->F[HYDRO_ITER_PREV];
  auto& s3 = x->s32;
  int rc;
  // UpdateOutletBaseConditions (fluid.hpp:542-600) from the latest iterate
  if (x->has_outlet)
    CK(launch_outlet_update(m, x->bc, up, x->vec<W3>(x->bcu, dim, m.nf),
                            x->bcu32 ? x->vf3f(x->bcu32, m.nf) : FP<3>{},
                            x->fc.sources ? x->Sv : nullptr, x->pw.partials, x->pw.ds, x->st));
  C3 bv64 = x->vec<C3>(x->bcu, dim, m.nf);
  if (x->mixed) {
    // FP32 assembly on the shadows
    std::swap(s3.F[HYDRO_ITER_CURR], s3.F[HYDRO_ITER_PREV]);
    std::swap(s3.u[HYDRO_ITER_CURR], s3.u[HYDRO_ITER_PREV]);
    using R3 = RT<float, 3>;
    using V3 = WT<float, 3>;
    R3 up32 = x->vf<R3>(s3.u[HYDRO_ITER_PREV], dim);
    R3 bv32{};
    for (int k = 0; k < dim; ++k) bv32.a[k] = x->bcu32 + (size_t)k * m.nf;
    R3 force32 = x->vf<R3>(s3.force, dim), fres32 = x->vf<R3>(s3.fres, dim);
    PK(x, HYDRO_PROF_VEL_GRAD,
       launch_vel_grad<float>(m, x->fc, up32, bv32, x->vf<WT<float, 9>>(s3.G, dim * dim),
                              x->st));
    PK(x, HYDRO_PROF_FORCE,
       launch_force<float>(m, x->fc, up32, x->vf<RT<float, 9>>(s3.G, dim * dim), pip, s3.mu,
                           s3.rho, force32, x->vf<R3>(s3.stforce, dim), s3.Sv, s3.Sm,
                           x->vf<V3>(s3.fo, dim), x->vf<V3>(s3.fres, dim),
                           x->vec<W3>(x->gp, dim, m.nc), x->st));
    FP<10> o = x->o32p();
    WT<float, 7> coef32{};
    V3 res32{};
    for (int q = 0; q < 2 * dim + 1; ++q) coef32.a[q] = o.a[q];
    for (int k = 0; k < dim; ++k) res32.a[k] = o.a[7 + k];
    PK(x, HYDRO_PROF_MOM_ASSEMBLE,
       launch_mom_assemble<float>(m, x->fc, up32, x->vf<R3>(s3.u[HYDRO_TIME_CURR], dim),
                                  x->vf<R3>(s3.u[HYDRO_TIME_PREV], dim),
                                  x->vf<RT<float, 9>>(s3.G, dim * dim), s3.F[HYDRO_ITER_PREV],
                                  s3.rho, s3.mu, x->vf<R3>(s3.fo, dim), up,
                                  x->uc3(HYDRO_TIME_CURR), x->uc3(HYDRO_TIME_PREV), bv32,
                                  coef32, res32, s3.Dc, x->mom_gs ? 1 : 0, x->st));
    rc = solve_momentum(x);
    if (rc) return rc;
    x->cd_iter_count++;
    PK(x, HYDRO_PROF_RHIE_CHOW,
       launch_rhie_chow<float>(m, x->fc, up, x->vf<R3>(x->du32[x->du_cur], dim), pip,
                               x->vec<C3>(x->gp, dim, m.nc), force32, fres32, s3.Dc, bv64,
                               x->Fs, x->kf, nullptr, x->st));
  } else {
    C3 force = x->vec<C3>(x->force, dim, m.nc);
    C3 fres = x->vec<C3>(x->fres, dim, m.nc);
    PK(x, HYDRO_PROF_VEL_GRAD,
       launch_vel_grad<double>(m, x->fc, up, bv64, x->vec<WP<9>>(x->G, dim * dim, m.nc),
                               x->st));
    PK(x, HYDRO_PROF_FORCE,
       launch_force<double>(m, x->fc, up, x->vec<CP<9>>(x->G, dim * dim, m.nc), pip, x->mu,
                            x->rho, force, x->vec<C3>(x->stforce, dim, m.nc), x->Sv, x->Sm,
                            x->vec<W3>(x->fo, dim, m.nc), x->vec<W3>(x->fres, dim, m.nc),
                            x->vec<W3>(x->gp, dim, m.nc), x->st));
    PK(x, HYDRO_PROF_MOM_ASSEMBLE,
       launch_mom_assemble<double>(m, x->fc, up, x->uc3(HYDRO_TIME_CURR),
                                   x->uc3(HYDRO_TIME_PREV),
                                   x->vec<CP<9>>(x->G, dim * dim, m.nc), Fip, x->rho, x->mu,
                                   x->vec<C3>(x->fo, dim, m.nc), up, x->uc3(HYDRO_TIME_CURR),
                                   x->uc3(HYDRO_TIME_PREV), bv64,
                                   x->vec<WP<7>>(x->coef, 2 * dim + 1, m.nc),
                                   x->vec<W3>(x->res, dim, m.nc), x->Dc,
                                   x->mom_split64 ? 1 : 0, x->st));
    rc = solve_momentum(x);
    if (rc) return rc;
    C3 du = x->vec<C3>(x->du[x->du_cur], dim, m.nc);
    x->cd_iter_count++;
    PK(x, HYDRO_PROF_RHIE_CHOW,
       launch_rhie_chow<double>(m, x->fc, up, du, pip, x->vec<C3>(x->gp, dim, m.nc), force, fres,
                                x->Dc, bv64, x->Fs, x->kf, nullptr, x->st));
  }
  PK(x, HYDRO_PROF_PRESSURE_RHS, launch_pressure_rhs(m, x->Fs, x->fc.sources ? x->Sv : nullptr, x->prhs, x->st));
  rc = solve_pressure(x);
  if (rc) return rc;
  C3 du = x->vec<C3>(x->du[x->du_cur], dim, m.nc);
  if (x->mixed)
    PK(x, HYDRO_PROF_CORRECT,
       launch_correct(m, x->fc, up, du, x->vf<RT<float, 3>>(x->du32[x->du_cur], dim), s3.Dc,
                      x->uw3(HYDRO_ITER_CURR), pip, x->p[HYDRO_ITER_CURR], x->pc, x->Dc, x->Fs,
                      x->kf, x->pw.kf32, x->F[HYDRO_ITER_CURR],
                      x->vf<FP<3>>(s3.u[HYDRO_ITER_CURR], dim), nullptr, s3.F[HYDRO_ITER_CURR],
                      x->pw.partials, x->pw.ds, x->st));
  else
    PK(x, HYDRO_PROF_CORRECT,
       launch_correct(m, x->fc, up, du, RT<float, 3>{}, nullptr, x->uw3(HYDRO_ITER_CURR), pip,
                      x->p[HYDRO_ITER_CURR], x->pc, x->Dc, x->Fs, x->kf, nullptr,
                      x->F[HYDRO_ITER_CURR], FP<3>{}, nullptr, nullptr, x->pw.partials, x->pw.ds,
                      x->st));
  if (d.simpler) {
    // SIMPLER pressure (fluid.hpp:1059-1155): a second solve with the same
    // matrix, in delta form around the corrected pressure
    const long long pin = d.pressure_fixed_cell;
    CK(launch_simpler_rhs(m, x->fc, x->vec<CP<7>>(x->coef, 2 * dim + 1, m.nc),
                          x->vec<C3>(x->res, dim, m.nc), x->uc3(HYDRO_ITER_CURR), up,
                          x->vec<C3>(x->fres, dim, m.nc), x->vec<C3>(x->gp, dim, m.nc),
                          x->vec<C3>(x->force, dim, m.nc), x->Dc, x->F[HYDRO_ITER_CURR], x->kf,
                          x->pw.dg, x->p[HYDRO_ITER_CURR], pin, d.pressure_fixed_value,
                          x->vec<W3>(x->fo, dim, m.nc), x->prhs, x->st));
    rc = solve_pressure(x, false);
    if (rc) return rc;
    CK(launch_add(m.nc, x->p[HYDRO_ITER_CURR], x->pc, x->st));
  }
  if (x->graph_mode) {
    // the SIMPLE loop's control kernel reads the indicator on the device
    x->iter_count++;
    return HYDRO_OK;
  }
  rc = sync_scalars(x);
  if (rc) return rc;
  x->indicator = x->hds->red[RS_INDICATOR];
  x->iter_count++;
  if (isnan(x->indicator)) return HYDRO_ERR_NAN;
  return HYDRO_OK;
}

int hydro_gpu_get_convergence_indicator(hydro_ctx* x, double* out) {
  if (!x || !out) return HYDRO_ERR_ARG;
  *out = x->cd_iter_count == 0 ? 1. : x->indicator;
  return HYDRO_OK;
}

int hydro_gpu_get_iteration_count(hydro_ctx* x, int* out) {
  if (!x || !out) return HYDRO_ERR_ARG;
  *out = x->iter_count;
  return HYDRO_OK;
}

int hydro_gpu_is_converged(hydro_ctx* x, int* out) {
  if (!x || !out) return HYDRO_ERR_ARG;
  double ind = x->cd_iter_count == 0 ? 1. : x->indicator;
  *out = (x->iter_count >= x->d.num_iterations_limit) || (ind < x->d.convergence_tolerance);
  return HYDRO_OK;
}

int hydro_gpu_finish_step(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  // time_prev <- time_curr (pointer rotation), time_curr <- iter_curr (copy)
  std::swap(x->p[HYDRO_TIME_PREV], x->p[HYDRO_TIME_CURR]);
  std::swap(x->F[HYDRO_TIME_PREV], x->F[HYDRO_TIME_CURR]);
  std::swap(x->u[HYDRO_TIME_PREV], x->u[HYDRO_TIME_CURR]);
  CK(cudaMemcpyAsync(x->p[HYDRO_TIME_CURR], x->p[HYDRO_ITER_CURR], sizeof(double) * m.nc,
                     cudaMemcpyDeviceToDevice, x->st));
  CK(cudaMemcpyAsync(x->F[HYDRO_TIME_CURR], x->F[HYDRO_ITER_CURR], sizeof(double) * m.nf,
                     cudaMemcpyDeviceToDevice, x->st));
  CK(cudaMemcpyAsync(x->u[HYDRO_TIME_CURR], x->u[HYDRO_ITER_CURR],
                     sizeof(double) * m.nc * x->dim, cudaMemcpyDeviceToDevice, x->st));
  x->time += x->dt;
  return nan_check(x, x->p[HYDRO_TIME_CURR], m.nc);
}

int hydro_gpu_get_auto_time_step(hydro_ctx* x, double* out) {
  if (!x || !out) return HYDRO_ERR_ARG;
  CK(launch_auto_dt(x->m, x->F[HYDRO_TIME_CURR], x->pw.partials, x->pw.ds, x->st));
  int rc = sync_scalars(x);
  if (rc) return rc;
  *out = x->hds->red[RS_AUTO_DT];
  return HYDRO_OK;
}

int hydro_gpu_set_time_step(hydro_ctx* x, double dt, double dta) {
  if (!x || isnan(dt) || isnan(dta)) return HYDRO_ERR_ARG;
  if (dt > 0.) x->dt = dt;
  if (dta > 0.) x->adv_dt = dta;
  return HYDRO_OK;
}

int hydro_gpu_get_time(hydro_ctx* x, double* ft, double* at) {
  if (!x) return HYDRO_ERR_ARG;
  if (ft) *ft = x->time;
  if (at) *at = x->adv_time;
  return HYDRO_OK;
}

int hydro_gpu_advection_substep(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  const hydro_desc& d = x->d;
  int nst = d.tvd_split ? x->dim : 1;
  const double* F = x->F[HYDRO_TIME_CURR];
  for (int stage = 0; stage < nst; ++stage) {
    PK(x, HYDRO_PROF_ADV_FACES,
       launch_adv_faces(m, x->nph, stage, nst, F, x->vec<CP<HYDRO_MAXPH>>(x->q, x->nph, m.nc),
                        x->inlet_mask, x->vec<CP<HYDRO_MAXPH>>(x->qin, x->nph, m.nf),
                        x->vec<WP<HYDRO_MAXPH>>(x->qflux, x->nph, m.nf), x->st));
    PK(x, HYDRO_PROF_ADV_UPDATE,
       launch_adv_update(m, x->nph, stage, nst, x->adv_dt,
                         x->vec<CP<HYDRO_MAXPH>>(x->qflux, x->nph, m.nf),
                         x->vec<CP<HYDRO_MAXPH>>(x->q, x->nph, m.nc),
                         x->vec<WP<HYDRO_MAXPH>>(x->qtmp, x->nph, m.nc), x->st));
    std::swap(x->q, x->qtmp);
  }
  if (fabs(d.sharp) > 1e-10) {
    for (int i = 0; i < x->nph; ++i)
      CK(launch_adv_sharpen(m, i, d.sharp, d.density[i], x->adv_dt, F, x->q + (size_t)i * m.nc,
                            x->smtmp, x->vec<W3>(x->G, x->dim, m.nc), x->Fs, x->st));
  }
  x->adv_time += x->adv_dt;
  CK(cudaGetLastError());
  return HYDRO_OK;
}

int hydro_gpu_advection_step(hydro_ctx* x, int* substeps) {
  if (!x) return HYDRO_ERR_ARG;
  int ns = 0;
  while (x->adv_time < x->time - 0.5 * x->adv_dt) {
    int rc = hydro_gpu_advection_substep(x);
    if (rc) return rc;
    ++ns;
  }
  if (substeps) *substeps = ns;
  return HYDRO_OK;
}

int hydro_gpu_step(hydro_ctx* x, hydro_step_stats* stats) {
  if (!x) return HYDRO_ERR_ARG;
  const hydro_desc& d = x->d;
  hydro_step_stats s;
  memset(&s, 0, sizeof(s));
  int rc;
  if (d.dt_auto) {
    double dtm;
    rc = hydro_gpu_get_auto_time_step(x, &dtm);
    if (rc) return rc;
    double dt = dtm * d.cfl, dta = dtm * d.cfl_advection;
    if (d.dt_max > 0. && dt > d.dt_max) {
      dta = dta * (d.dt_max / dt);
      dt = d.dt_max;
    }
    x->dt = dt;
    x->adv_dt = dta;
  }
  rc = hydro_gpu_start_step(x);
  if (rc) return rc;
  for (;;) {
    int conv;
    hydro_gpu_is_converged(x, &conv);
    if (conv) break;
    rc = hydro_gpu_make_iteration(x);
    if (rc) {
      if (stats) { s.status = rc; *stats = s; }
      return rc;
    }
  }
  hydro_gpu_get_convergence_indicator(x, &s.convergence_indicator);
  s.outer_iterations = x->iter_count;
  s.velocity_sweeps = x->vel_sweeps;
  s.pressure_iterations = x->p_iters;
  s.pressure_residual = x->p_res;
  rc = hydro_gpu_finish_step(x);
  if (rc) {
    if (stats) { s.status = rc; *stats = s; }
    return rc;
  }
  if (d.advection_enable) {
    rc = hydro_gpu_advection_step(x, &s.advection_substeps);
    if (rc) return rc;
  }
  // heat after advection (hydro2d.hpp:1607-1613)
  if (x->heat.on && (rc = heat_step(x))) return rc;
  rc = hydro_gpu_update_properties(x);
  if (rc) return rc;
  s.dt = x->dt;
  s.dt_advection = x->adv_dt;
  s.time = x->time;
  // a pressure solve that stopped at its limit does not stop the step (the
  // reference goes on past a solver's limit, linear.hpp:690-710); the
  // status reports it once the step is complete
  s.pressure_unconverged = x->p_unconv;
  s.status = x->p_unconv ? HYDRO_NOT_CONVERGED : HYDRO_OK;
  if (stats) *stats = s;
  return s.status;
}

// ------------------------------------------------------ graph-captured step --
namespace {

// Number of advection substeps the host loop of hydro_gpu_advection_step
// would take after the fluid time advanced by dt; *t_out is the advection
// time it ends at.
int advection_substeps(const hydro_ctx* x, double dt, double* t_out) {
  double t = x->adv_time, tf = x->time + dt;
  int n = 0;
  if (x->d.advection_enable)
    while (t < tf - 0.5 * x->adv_dt && n < 1000000) {
      t += x->adv_dt;
      ++n;
    }
  *t_out = t;
  return n;
}

// Host-side scalars a capture changes (it enqueues work of a step that has
// not run); restored once the capture is complete.
struct HostSnapshot {
  double time, adv_time, p_res, indicator;
  int iter_count, cd_iter_count, vel_sweeps, p_iters, p_unconv;
  bool prof;
};

int begin_capture_of(hydro_ctx* x, HostSnapshot* s) {
  for (int i = 0; i < 4; ++i)
    if (!x->cap_streams[i]) CK(cudaStreamCreateWithFlags(&x->cap_streams[i], cudaStreamNonBlocking));
  *s = {x->time, x->adv_time, x->p_res, x->indicator, x->iter_count, x->cd_iter_count,
        x->vel_sweeps, x->p_iters, x->p_unconv, x->prof.on};
  x->cap_depth = 0;
  x->cap_start[0] = launch_total();
  x->cap_nested[0] = 0;
  x->prof.on = false;
  x->graph_mode = true;
  return HYDRO_OK;
}

void end_capture_of(hydro_ctx* x, const HostSnapshot& s) {
  x->graph_mode = false;
  x->cap_graph = nullptr;
  x->prof.on = s.prof;
  x->time = s.time;
  x->adv_time = s.adv_time;
  x->p_res = s.p_res;
  x->indicator = s.indicator;
  x->iter_count = s.iter_count;
  x->cd_iter_count = s.cd_iter_count;
  x->vel_sweeps = s.vel_sweeps;
  x->p_iters = s.p_iters;
  x->p_unconv = s.p_unconv;
}

// Enqueues one whole step (StartStep, SIMPLE loop, FinishStep, advection
// substeps, property update, next auto time step) on x->st, which is
// capturing into x->cap_graph.  Loops whose length the device decides are
// WHILE nodes; two SIMPLE iterations are captured per loop trip (the second
// under an IF node) so that the iteration layers alternate their buffers as
// the pointer swaps of the host-driven step do; select copies leave every
// result where the host pointers expect it.
int enqueue_step_body(hydro_ctx* x, int substeps) {
  const Mesh& m = x->m;
  const hydro_desc& d = x->d;
  double* q0 = x->q;
    int r;
    if ((r = reset_flags(x, FL_STEP_SWEEPS, 3))) return r;  // sweeps, p iterations, SIMPLE
    if ((r = reset_flags(x, FL_STEP_PUNCONV, 2))) return r;  // unconverged solves, NaN
    if ((r = hydro_gpu_start_step(x))) return r;
    const int limit = d.num_iterations_limit;
    const double tol = d.convergence_tolerance;
    const int cont0 = !(0 >= limit || 1. < tol);
    cudaGraphConditionalHandle hw, hi;
    if ((r = new_handle(x, cont0, &hw)) || (r = new_handle(x, 0, &hi))) return r;
    r = add_while(x, hw, [&]() -> int {
      int q;
      if ((q = hydro_gpu_make_iteration(x))) return q;
      CK(launch_ctl_simple2(x->pw.ds, limit, tol, hi, hw, x->st, body_kernels(x)));
      return add_if(x, hi, [&]() -> int {
        int z;
        if ((z = hydro_gpu_make_iteration(x))) return z;
        CK(launch_ctl_simple(x->pw.ds, limit, tol, hw, 1, x->st, body_kernels(x)));
        return HYDRO_OK;
      });
    });
    if (r) return r;
    // an odd iteration count leaves the iterate in the other buffer
    CK(launch_select_iter(m.nc * x->dim, x->u[HYDRO_ITER_PREV], x->u[HYDRO_ITER_CURR],
                          x->pw.ds, x->st));
    CK(launch_select_iter(m.nc, x->p[HYDRO_ITER_PREV], x->p[HYDRO_ITER_CURR], x->pw.ds,
                          x->st));
    CK(launch_select_iter(m.nf, x->F[HYDRO_ITER_PREV], x->F[HYDRO_ITER_CURR], x->pw.ds,
                          x->st));
    // FinishStep with copies instead of the pointer rotation
    CK(cudaMemcpyAsync(x->p[HYDRO_TIME_PREV], x->p[HYDRO_TIME_CURR], sizeof(double) * m.nc,
                       cudaMemcpyDeviceToDevice, x->st));
    CK(cudaMemcpyAsync(x->F[HYDRO_TIME_PREV], x->F[HYDRO_TIME_CURR], sizeof(double) * m.nf,
                       cudaMemcpyDeviceToDevice, x->st));
    CK(cudaMemcpyAsync(x->u[HYDRO_TIME_PREV], x->u[HYDRO_TIME_CURR],
                       sizeof(double) * m.nc * x->dim, cudaMemcpyDeviceToDevice, x->st));
    CK(cudaMemcpyAsync(x->p[HYDRO_TIME_CURR], x->p[HYDRO_ITER_CURR], sizeof(double) * m.nc,
                       cudaMemcpyDeviceToDevice, x->st));
    CK(cudaMemcpyAsync(x->F[HYDRO_TIME_CURR], x->F[HYDRO_ITER_CURR], sizeof(double) * m.nf,
                       cudaMemcpyDeviceToDevice, x->st));
    CK(cudaMemcpyAsync(x->u[HYDRO_TIME_CURR], x->u[HYDRO_ITER_CURR],
                       sizeof(double) * m.nc * x->dim, cudaMemcpyDeviceToDevice, x->st));
    CK(launch_nan_count(m.nc, x->p[HYDRO_TIME_CURR], x->pw.partials, x->pw.ds, x->st));
    x->time += x->dt;
    for (int i = 0; i < substeps; ++i)
      if ((r = hydro_gpu_advection_substep(x))) return r;
    if (x->q != q0) {
      // odd number of stage swaps: bring the fractions back to the buffer
      // the next launch reads
      CK(cudaMemcpyAsync(q0, x->q, sizeof(double) * m.nc * x->nph, cudaMemcpyDeviceToDevice,
                         x->st));
      std::swap(x->q, x->qtmp);
    }
    if (x->heat.on && (r = heat_step(x))) return r;
    if ((r = hydro_gpu_update_properties(x))) return r;
    CK(launch_auto_dt(m, x->F[HYDRO_TIME_CURR], x->pw.partials, x->pw.ds, x->st));
    return HYDRO_OK;
}

// After a context's step was captured: what a launch runs outside the
// bodies, and the captured launches taken off the launch counter (kernels
// are counted when a graph launch runs them, finish_graph_step).
void end_capture_count(hydro_ctx* x) {
  x->graph_top = launch_total() - x->cap_start[0] - x->cap_nested[0];
  count_launches(-(launch_total() - x->cap_start[0]));
}

// Captures one step of one context into x->sg.exec.
int capture_step(hydro_ctx* x, int substeps) {
  if (x->sg.exec) {
    cudaGraphExecDestroy(x->sg.exec);
    x->sg.exec = nullptr;
  }
  HostSnapshot snap;
  int rc = begin_capture_of(x, &snap);
  if (rc) return rc;
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) {
    end_capture_of(x, snap);
    return HYDRO_ERR_CUDA;
  }
  x->cap_graph = g;
  if (cudaStreamBeginCaptureToGraph(x->st, g, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed) == cudaSuccess) {
    rc = enqueue_step_body(x, substeps);
    end_capture_count(x);
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(x->st, &out);
    if (!rc && e2 != cudaSuccess) rc = HYDRO_ERR_CUDA;
    if (!rc && cudaGraphInstantiate(&x->sg.exec, g, 0) != cudaSuccess) {
      x->sg.exec = nullptr;
      rc = HYDRO_ERR_CUDA;
    }
  } else {
    rc = HYDRO_ERR_CUDA;
  }
  cudaGraphDestroy(g);
  end_capture_of(x, snap);
  cudaGetLastError();
  return rc;
}

// dt of the coming step (hydro<Mesh>::step, hydro2d.hpp:1541-1553).
int next_dt(hydro_ctx* x) {
  const hydro_desc& d = x->d;
  if (!d.dt_auto) return HYDRO_OK;
  double dtm;
  int rc = hydro_gpu_get_auto_time_step(x, &dtm);
  if (rc) return rc;
  double dt = dtm * d.cfl, dta = dtm * d.cfl_advection;
  if (d.dt_max > 0. && dt > d.dt_max) {
    dta = dta * (d.dt_max / dt);
    dt = d.dt_max;
  }
  x->dt = dt;
  x->adv_dt = dta;
  return HYDRO_OK;
}

std::array<const void*, 30> layer_key(const hydro_ctx* x) {
  std::array<const void*, 30> k{};
  int n = 0;
  for (int l = 0; l < 4; ++l) {
    k[n++] = x->u[l];
    k[n++] = x->p[l];
    k[n++] = x->F[l];
    k[n++] = x->s32.u[l];
    k[n++] = x->s32.F[l];
  }
  k[n++] = x->q;
  k[n++] = x->qtmp;
  k[n++] = x->heat.tc;
  k[n++] = x->heat.tp;
  return k;
}

bool graph_stale(const hydro_ctx* x, int substeps) {
  return x->sg.dt != x->dt || x->sg.adv_dt != x->adv_dt || x->sg.substeps != substeps ||
         x->sg.sources != x->fc.sources || x->sg.heat_gen != x->heat.gen ||
         x->sg.layers != layer_key(x);
}

void graph_key(hydro_ctx* x, int substeps) {
  x->sg.layers = layer_key(x);
  x->sg.dt = x->dt;
  x->sg.adv_dt = x->adv_dt;
  x->sg.substeps = substeps;
  x->sg.sources = x->fc.sources;
  x->sg.heat_gen = x->heat.gen;
}

// After a graph launch completed and x->hds holds the device scalars.
int finish_graph_step(hydro_ctx* x, int substeps, double adv_end, hydro_step_stats* stats) {
  hydro_step_stats s;
  memset(&s, 0, sizeof(s));
  const DevScalars& h = *x->hds;
  // the kernels this launch ran: those outside the bodies once, those of
  // every body run as counted on the device
  count_launches(x->graph_top + (long long)(h.red[RS_KEXEC] - x->kexec_seen));
  x->kexec_seen = h.red[RS_KEXEC];
  x->iter_count = h.flag[FL_ITERS];
  x->cd_iter_count = h.flag[FL_ITERS];
  x->indicator = h.red[RS_INDICATOR];
  x->p_res = h.red[RS_P_RES];
  x->vel_sweeps = h.flag[FL_STEP_SWEEPS];
  x->p_iters = h.flag[FL_STEP_PITERS];
  x->du_cur = 0;
  x->time += x->dt;
  x->adv_time = adv_end;
  s.outer_iterations = x->iter_count;
  s.convergence_indicator = x->cd_iter_count == 0 ? 1. : x->indicator;
  s.velocity_sweeps = x->vel_sweeps;
  s.pressure_iterations = x->p_iters;
  s.pressure_residual = x->p_res;
  s.advection_substeps = substeps;
  s.dt = x->dt;
  s.dt_advection = x->adv_dt;
  s.time = x->time;
  x->p_unconv = h.flag[FL_STEP_PUNCONV];
  s.pressure_unconverged = x->p_unconv;
  s.status = (h.red[RS_NAN] > 0. || isnan(x->indicator) || h.flag[FL_STEP_NAN]) ? HYDRO_ERR_NAN
             : x->p_unconv                                 ? HYDRO_NOT_CONVERGED
                                                           : HYDRO_OK;
  if (stats) *stats = s;
  return s.status;
}

}  // namespace

int hydro_gpu_step_graph(hydro_ctx* x, hydro_step_stats* stats) {
  if (!x) return HYDRO_ERR_ARG;
  int rc = next_dt(x);
  if (rc) return rc;
  double adv_end;
  const int substeps = advection_substeps(x, x->dt, &adv_end);
  if (!x->sg.exec || graph_stale(x, substeps)) {
    rc = capture_step(x, substeps);
    if (rc) return rc;
    graph_key(x, substeps);
  }
  CK(cudaGraphLaunch(x->sg.exec, x->st));
  rc = sync_scalars(x);
  if (rc) return rc;
  return finish_graph_step(x, substeps, adv_end, stats);
}

// ----------------------------------------------------------------- batch --
// Many independent cases (hydro_gpu_batch_*): one context per case, and one
// CUDA graph per batch step in which every case's step is an independent
// branch (fork from the launching stream, join back), so a single launch
// runs all cases concurrently with their loops steered on the device.
struct hydro_batch {
  std::vector<hydro_ctx*> cases;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec = nullptr;
  std::vector<int> substeps;
  std::vector<double> adv_end;
};

int hydro_gpu_batch_destroy(hydro_batch* b) {
  if (!b) return HYDRO_OK;
  if (b->st) cudaStreamSynchronize(b->st);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto* x : b->cases) hydro_gpu_destroy(x);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return HYDRO_OK;
}

int hydro_gpu_batch_create(const hydro_desc* descs, int ncases, hydro_batch** out) {
  if (!descs || !out || ncases < 1) return HYDRO_ERR_ARG;
  *out = nullptr;
  hydro_batch* b = new (std::nothrow) hydro_batch();
  if (!b) return HYDRO_ERR_NOMEM;
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    hydro_gpu_batch_destroy(b);
    return HYDRO_ERR_CUDA;
  }
  for (int i = 0; i < ncases; ++i) {
    hydro_desc d = descs[i];
    d.stream = nullptr;  // every case owns its stream (its graph branch)
    hydro_ctx* x = nullptr;
    int rc = hydro_gpu_create(&d, &x);
    if (rc) {
      hydro_gpu_batch_destroy(b);
      return rc;
    }
    b->cases.push_back(x);
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      hydro_gpu_batch_destroy(b);
      return HYDRO_ERR_CUDA;
    }
    b->join.push_back(e);
  }
  b->substeps.assign(ncases, -1);
  b->adv_end.assign(ncases, 0.);
  *out = b;
  return HYDRO_OK;
}

int hydro_gpu_batch_size(hydro_batch* b, int* n) {
  if (!b || !n) return HYDRO_ERR_ARG;
  *n = (int)b->cases.size();
  return HYDRO_OK;
}

int hydro_gpu_batch_case(hydro_batch* b, int i, hydro_ctx** out) {
  if (!b || !out || i < 0 || i >= (int)b->cases.size()) return HYDRO_ERR_ARG;
  *out = b->cases[i];
  return HYDRO_OK;
}

int hydro_gpu_batch_init_state(hydro_batch* b) {
  if (!b) return HYDRO_ERR_ARG;
  for (auto* x : b->cases) {
    int rc = hydro_gpu_init_state(x);
    if (rc) return rc;
  }
  return HYDRO_OK;
}

namespace {

int capture_batch(hydro_batch* b) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  int rc = HYDRO_OK;
  const int n = (int)b->cases.size();
  std::vector<HostSnapshot> snaps(n);
  std::vector<int> begun(n, 0);
  if (cudaStreamBeginCaptureToGraph(b->st, g, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGraphDestroy(g);
    return HYDRO_ERR_CUDA;
  }
  if (cudaEventRecord(b->fork, b->st) != cudaSuccess) rc = HYDRO_ERR_CUDA;
  for (int i = 0; i < n && !rc; ++i) {
    hydro_ctx* x = b->cases[i];
    if ((rc = begin_capture_of(x, &snaps[i]))) break;
    begun[i] = 1;
    x->cap_graph = g;
    if (cudaStreamWaitEvent(x->st, b->fork, 0) != cudaSuccess) {
      rc = HYDRO_ERR_CUDA;
      break;
    }
    rc = enqueue_step_body(x, b->substeps[i]);
    end_capture_count(x);
    if (!rc && (cudaEventRecord(b->join[i], x->st) != cudaSuccess ||
                cudaStreamWaitEvent(b->st, b->join[i], 0) != cudaSuccess))
      rc = HYDRO_ERR_CUDA;
  }
  cudaGraph_t outg = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b->st, &outg);
  if (!rc && e2 != cudaSuccess) rc = HYDRO_ERR_CUDA;
  if (!rc && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
    b->exec = nullptr;
    rc = HYDRO_ERR_CUDA;
  }
  cudaGraphDestroy(g);
  for (int i = 0; i < n; ++i)
    if (begun[i]) end_capture_of(b->cases[i], snaps[i]);
  cudaGetLastError();
  return rc;
}

}  // namespace

int hydro_gpu_batch_step(hydro_batch* b, hydro_step_stats* stats) {
  if (!b) return HYDRO_ERR_ARG;
  const int n = (int)b->cases.size();
  bool stale = !b->exec;
  for (int i = 0; i < n; ++i) {
    hydro_ctx* x = b->cases[i];
    int rc = next_dt(x);
    if (rc) return rc;
    int ns = advection_substeps(x, x->dt, &b->adv_end[i]);
    if (ns != b->substeps[i] || graph_stale(x, ns)) stale = true;
    b->substeps[i] = ns;
  }
  if (stale) {
    int rc = capture_batch(b);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) graph_key(b->cases[i], b->substeps[i]);
  }
  CK(cudaGraphLaunch(b->exec, b->st));
  for (auto* x : b->cases)
    CK(cudaMemcpyAsync(x->hds, x->pw.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, b->st));
  CK(cudaStreamSynchronize(b->st));
  int status = HYDRO_OK;
  for (int i = 0; i < n; ++i) {
    int rc = finish_graph_step(b->cases[i], b->substeps[i], b->adv_end[i],
                               stats ? &stats[i] : nullptr);
    if (rc && !status) status = rc;
  }
  return status;
}

// --------------------------------------------------------------- heat --
int hydro_gpu_heat_create(hydro_ctx* x, const hydro_heat_desc* hd) {
  if (!x || !hd) return HYDRO_ERR_ARG;
  if (!(hd->dt > 0.) || !(hd->relaxation_factor > 0.) || hd->iters_limit < 0 ||
      !(hd->tolerance >= 0.) || !std::isfinite(hd->box_temperature) ||
      !std::isfinite(hd->temperature_initial))
    return HYDRO_ERR_ARG;
  if (hd->solver != HYDRO_LINEAR_JACOBI && hd->solver != HYDRO_LINEAR_GAUSS_SEIDEL &&
      hd->solver != HYDRO_LINEAR_LU)
    return HYDRO_ERR_ARG;
  // the temperature rows are swept by Jacobi; another solver is substituted
  // only on request
  if (hd->solver != HYDRO_LINEAR_JACOBI && !x->d.substitute_solvers)
    return HYDRO_ERR_UNSUPPORTED;
  const Mesh& m = x->m;
  auto& h = x->heat;
  if (!h.mem) {
    if (cudaMalloc(&h.mem, sizeof(double) * 3 * m.nc) != cudaSuccess) {
      cudaGetLastError();
      h.mem = nullptr;
      return HYDRO_ERR_NOMEM;
    }
    h.tc = h.mem;
    h.tp = h.mem + m.nc;
    h.kc = h.mem + 2 * m.nc;
  }
  h.hd = *hd;
  // boundary faces in the box: centre coordinates as the mesh forms them
  // (node lo + i h along the face normal, cell centre lo + (i + 1/2) h
  // across), compared inclusively with the box
  HeatBc bc{};
  auto inside = [&](int k, double v) { return hd->box_lo[k] <= v && v <= hd->box_hi[k]; };
  for (int k = 0; k < 3; ++k) {
    bc.a[k] = 0;
    bc.b[k] = 0;
    if (k >= x->dim) continue;
    int first = -1, last = -2;
    for (int i = 0; i < m.n[k]; ++i)
      if (inside(k, m.lo[k] + (i + 0.5) * m.h[k])) {
        if (first < 0) first = i;
        last = i;
      }
    if (first >= 0) {
      bc.a[k] = first;
      bc.b[k] = last + 1;
    }
    bc.side_in[2 * k] = inside(k, m.lo[k]);
    bc.side_in[2 * k + 1] = inside(k, m.lo[k] + m.n[k] * m.h[k]);
  }
  for (int k = 0; k < 3; ++k) {
    bc.lo[k] = hd->box_lo[k];
    bc.hi[k] = hd->box_hi[k];
  }
  bc.value = hd->box_temperature;
  h.bc = bc;
  for (int i = 0; i < HYDRO_MAXPH; ++i) h.hc.cond[i] = i < x->nph ? hd->conductivity[i] : 0.;
  bdf_coeffs(hd->dt, hd->time_second_order, h.hc.co);
  h.hc.relax = hd->relaxation_factor;
  std::vector<double> t0((size_t)m.nc, hd->temperature_initial);
  CK(cudaMemcpyAsync(h.tc, t0.data(), sizeof(double) * m.nc, cudaMemcpyHostToDevice, x->st));
  CK(cudaMemcpyAsync(h.tp, t0.data(), sizeof(double) * m.nc, cudaMemcpyHostToDevice, x->st));
  CK(launch_heat_conductivity(m, x->nph, h.hc, x->vec<CP<HYDRO_MAXPH>>(x->alpha, x->nph, m.nc),
                              h.kc, x->st));
  CK(cudaStreamSynchronize(x->st));
  h.on = true;
  h.gen += 1;  // a captured step holds the old constants
  return HYDRO_OK;
}

int hydro_gpu_heat_step(hydro_ctx* x) {
  if (!x || !x->heat.on) return HYDRO_ERR_ARG;
  return heat_step(x);
}

int hydro_gpu_calc_stat(hydro_ctx* x, hydro_stat* out) {
  if (!x || !out) return HYDRO_ERR_ARG;
  const Mesh& m = x->m;
  memset(out, 0, sizeof(*out));
  double h[16];
  for (int i = 0; i < x->nph; ++i) {
    CK(cudaMemsetAsync(x->stat_ticket, 0, sizeof(unsigned) * 4, x->st));
    CK(launch_stat(m, x->q + (size_t)i * m.nc, x->alpha + (size_t)i * m.nc,
                   x->uc3(HYDRO_TIME_CURR), x->F[HYDRO_TIME_CURR], x->pw.partials, x->stat_out,
                   x->stat_ticket, x->st));
    CK(cudaMemcpyAsync(h, x->stat_out, sizeof(double) * 12, cudaMemcpyDeviceToHost, x->st));
    CK(cudaStreamSynchronize(x->st));
    out->volume[i] = h[0];
    out->mass[i] = h[0] * x->d.density[i];
    for (int k = 0; k < x->dim; ++k) {
      out->center[i][k] = h[1 + k] / h[0];
      out->velocity[i][k] = h[4 + k] / h[0];
    }
    out->partial_mass[i] = h[7];
    out->volume_flux_in[i] = h[8];
    out->volume_flux_out[i] = h[9];
    out->pd_min[i] = h[10];
    out->pd_max[i] = h[11];
  }
  return HYDRO_OK;
}

int hydro_gpu_set_profiling(hydro_ctx* x, int on) {
  if (!x) return HYDRO_ERR_ARG;
  CK(cudaStreamSynchronize(x->st));
  x->prof.collect();
  x->prof.on = on != 0;
  return HYDRO_OK;
}

int hydro_gpu_reset_profile(hydro_ctx* x) {
  if (!x) return HYDRO_ERR_ARG;
  CK(cudaStreamSynchronize(x->st));
  x->prof.collect();
  x->prof.reset();
  return HYDRO_OK;
}

int hydro_gpu_get_profile(hydro_ctx* x, int group, long long* launches, double* ms) {
  if (!x || group < 0 || group >= HYDRO_PROF_COUNT) return HYDRO_ERR_ARG;
  CK(cudaStreamSynchronize(x->st));
  x->prof.collect();
  if (launches) *launches = x->prof.launches[group];
  if (ms) *ms = x->prof.ms[group];
  return HYDRO_OK;
}

int hydro_gpu_get_launch_count(long long* out) {
  if (!out) return HYDRO_ERR_ARG;
  *out = hg::g_launches.load();
  return HYDRO_OK;
}

// ------------------------------------------------- stencil solve (C-ABI) --
size_t hydro_gpu_stencil_workspace_size(int dim, int nx, int ny, int nz) {
  Mesh m;
  int n[3] = {nx, ny, nz};
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  if (init_mesh(m, dim, n, lo, hi)) return 0;
  Arena a;
  for (int i = 0; i < 7; ++i) a.take<double>(m.nc);
  a.take<double>((size_t)4 * kMaxBlocks);
  a.take<DevScalars>(1);
  return a.used + 256;
}

int hydro_gpu_stencil_solve(int dim, int nx, int ny, int nz, const double* face_coeff,
                            double shift, long pinned_cell, double pinned_value,
                            const double* rhs, double* xsol, int use_guess, double tolerance,
                            int iters_limit, void* workspace, void* stream, int* iterations,
                            double* residual) {
  Mesh m;
  int n[3] = {nx, ny, nz};
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  if (init_mesh(m, dim, n, lo, hi)) return HYDRO_ERR_ARG;
  if (!face_coeff || !rhs || !xsol || !workspace) return HYDRO_ERR_ARG;
  if (pinned_cell >= m.nc || iters_limit < 1 || !(tolerance >= 0.)) return HYDRO_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  Arena a;
  a.base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
  PcgWork w{};
  w.r = a.take<double>(m.nc);
  w.z = a.take<double>(m.nc);
  w.p = a.take<double>(m.nc);
  w.Ap = a.take<double>(m.nc);
  w.dg = a.take<double>(m.nc);
  w.idg = a.take<double>(m.nc);
  double* f = a.take<double>(m.nc);
  w.partials = a.take<double>((size_t)4 * kMaxBlocks);
  w.ds = a.take<DevScalars>(1);
  w.pin = pinned_cell;
  w.limit = iters_limit;
  CK(cudaMemsetAsync(w.ds, 0, sizeof(DevScalars), st));
  // f = -c
  CK(cudaMemcpyAsync(f, rhs, sizeof(double) * m.nc, cudaMemcpyDeviceToDevice, st));
  CK(scale_vector(m.nc, f, -1., st));
  if (pinned_cell >= 0) CK(pin_rhs(m, face_coeff, f, pinned_cell, pinned_value, st));
  int singular = (shift == 0. && pinned_cell < 0);
  CK(pcg_prepare(m, face_coeff, shift, w, 0, st));
  CK(pcg_init(m, face_coeff, f, xsol, use_guess, tolerance, singular, w, st));
  DevScalars h;
  int queued = 0;
  for (;;) {
    int nchunk = std::min(kCgChunk, iters_limit - queued);
    if (nchunk < 1) nchunk = 1;
    CK(pcg_iterate(m, face_coeff, xsol, nchunk, w, st));
    queued += nchunk;
    CK(cudaMemcpyAsync(&h, w.ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h.flag[FL_PCG_DONE] || queued >= iters_limit) break;
  }
  if (singular) {
    PcgWork& ww = w;
    CK(sub_mean(m, xsol, ww, st));
  }
  CK(cudaStreamSynchronize(st));
  double ff = h.red[RS_PCG_FF], rr = h.red[RS_PCG_RR];
  double res = ff > 0. ? sqrt(rr / ff) : 0.;
  if (iterations) *iterations = h.flag[FL_PCG_ITERS];
  if (residual) *residual = res;
  // a zero row (no couplings, no shift) or a non-finite input ends the
  // iteration with a NaN residual: reported, never taken as converged
  if (std::isnan(rr) || std::isnan(ff)) return HYDRO_ERR_NAN;
  return (ff > 0. && rr > tolerance * tolerance * ff) ? HYDRO_NOT_CONVERGED : HYDRO_OK;
}

// ------------------------------------------------- learned guess ------
int hydro_gpu_set_pressure_guess(hydro_ctx* x, hydro_net* net, int iterations,
                                 double rho_scale) {
  if (!x || iterations < 0 || !(rho_scale > 0.)) return HYDRO_ERR_ARG;
  if (!net || iterations == 0) {
    x->net = nullptr;
    x->net_iters = 0;
    return HYDRO_OK;
  }
  const bool refine = x->d.precision == HYDRO_MIXED || x->d.pressure_solver == HYDRO_LINEAR_MGCG;
  if (!refine || x->d.cta_threads > 0 || !net_check_grid(net, x->dim, x->m.n))
    return HYDRO_ERR_UNSUPPORTED;
  // one forward pass outside any capture: kernel attributes and module
  // loading happen here, not inside a captured step
  int rc = net_predict_async(net, x->prhs, x->rho, rho_scale, x->pc, x->st);
  if (rc) return rc;
  if ((rc = net_error(net, x->st))) return rc;
  x->net = net;
  x->net_iters = iterations;
  x->net_rho_scale = rho_scale;
  x->guess_off = false;
  if ((rc = reset_flags(x, FL_GUESS_USED, 2)) || (rc = reset_flags(x, FL_GUESS_SKIP, 4)))
    return rc;
  if ((rc = sync_scalars(x))) return rc;
  if (x->sg.exec) {  // a captured step without (or with another) guess
    cudaGraphExecDestroy(x->sg.exec);
    x->sg.exec = nullptr;
  }
  return HYDRO_OK;
}

int hydro_gpu_get_guess_stats(hydro_ctx* x, long long* used, long long* dropped,
                              long long* skipped) {
  if (!x) return HYDRO_ERR_ARG;
  int rc = sync_scalars(x);
  if (rc) return rc;
  if (used) *used = x->hds->flag[FL_GUESS_USED];
  if (dropped) *dropped = x->hds->flag[FL_GUESS_DROPPED];
  if (skipped) *skipped = x->hds->flag[FL_GUESS_SKIPPED];
  if ((rc = reset_flags(x, FL_GUESS_USED, 2))) return rc;
  return reset_flags(x, FL_GUESS_SKIPPED, 1);
}

}  // extern "C"
