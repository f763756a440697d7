// output.cu -- field and scalar output of the hot path's state in the
// reference's on-disk formats, written asynchronously.
//
//   .vts/.pvd  SessionParaviewStructured (output_paraview.hpp:34-175): one
//              ASCII StructuredGrid file per frame, node entries as
//              PointData, cell entries as CellData, the node coordinates as
//              Points, every value printed as the reference's ostream does
//              (%g, 6 significant digits); a .pvd collection with one DataSet
//              line per frame and the footer written on close.
//   .dat       SessionPlainScalar (output.hpp:231-261) with the entries of
//              hydro<Mesh> (hydro2d.hpp:825-905) from CalcStat
//              (hydro2d.hpp:1432-1529).
//
// Entries carry the reference's names and order (content_pool,
// hydro2d.hpp:710-816); a frame copies the needed device arrays into
// pinned host memory on a side stream ordered after the context's stream,
// and a worker thread formats and writes the file while the GPU carries on.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hydro_gpu.h"

namespace {

enum Src {
  S_NODE_X, S_NODE_Y, S_NODE_Z, S_VEL, S_PRESSURE, S_DENSITY, S_VISCOSITY, S_VOLUME_SOURCE,
  S_EXCLUDED, S_DIVERGENCE, S_MASS_FRACTION, S_TRUE_DENSITY, S_PARTIAL_DENSITY,
  S_VOLUME_FRACTION, S_TEMPERATURE
};

struct Entry {
  std::string name;
  Src src;
  int comp;  // velocity component or phase
  bool node() const { return src <= S_NODE_Z; }
};

void put_g(std::string& out, double v) {
  char b[40];
  int k = snprintf(b, sizeof(b), "%g ", v);
  out.append(b, k);
}

struct Grid {
  int dim = 2;
  int n[3] = {1, 1, 1};
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  long long cells() const { return (long long)n[0] * n[1] * n[2]; }
  long long nodes() const {
    return (long long)(n[0] + 1) * (n[1] + 1) * (dim == 3 ? n[2] + 1 : 1);
  }
  // InitUniformMesh (mesh.hpp:723-736): lb + (i/n) * (hb - lb)
  double node(int d, int i) const {
    return lo[d] + ((double)i / (double)n[d]) * (hi[d] - lo[d]);
  }
};

// One frame in the reference's text layout.
std::string format_vts(const Grid& g, const std::vector<Entry>& ents,
                       const std::vector<const double*>& data) {
  std::string o;
  const int nz = g.dim == 3 ? g.n[2] : 0;
  o += "<?xml version=\"1.0\"?>\n";
  o += "<VTKFile type=\"StructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  char b[160];
  snprintf(b, sizeof(b), "  <StructuredGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n", g.n[0], g.n[1], nz);
  o += b;
  snprintf(b, sizeof(b), "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", g.n[0], g.n[1], nz);
  o += b;
  auto header = [&](const std::string& name, int ncomp) {
    o += "        <DataArray Name=\"" + name + "\" NumberOfComponents=\"" + std::to_string(ncomp) +
         "\" type=\"Float32\" format=\"ascii\">\n";
  };
  auto footer = [&]() { o += "        </DataArray>\n"; };
  for (int pass = 0; pass < 2; ++pass) {
    o += pass == 0 ? "      <PointData>\n" : "      <CellData>\n";
    for (size_t e = 0; e < ents.size(); ++e) {
      if (ents[e].node() != (pass == 0)) continue;
      header(ents[e].name, 1);
      const long long cnt = pass == 0 ? g.nodes() : g.cells();
      for (long long i = 0; i < cnt; ++i) put_g(o, data[e][i]);
      o += "\n";
      footer();
    }
    o += pass == 0 ? "      </PointData>\n" : "      </CellData>\n";
  }
  o += "      <Points>\n";
  header("mesh", 3);
  const int kz = g.dim == 3 ? g.n[2] + 1 : 1;
  for (int k = 0; k < kz; ++k)
    for (int j = 0; j <= g.n[1]; ++j)
      for (int i = 0; i <= g.n[0]; ++i) {
        put_g(o, g.node(0, i));
        put_g(o, g.node(1, j));
        put_g(o, g.dim == 3 ? g.node(2, k) : 0.);
      }
  footer();
  o += "      </Points>\n";
  o += "    </Piece>\n";
  o += "  </StructuredGrid>\n";
  o += "</VTKFile>\n";
  return o;
}

int write_file(const std::string& path, const std::string& text) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return HYDRO_ERR_IO;
  size_t w = fwrite(text.data(), 1, text.size(), f);
  int rc = (w == text.size()) ? HYDRO_OK : HYDRO_ERR_IO;
  if (fclose(f) != 0) rc = HYDRO_ERR_IO;
  return rc;
}

// Reference entry order (content_pool, hydro2d.hpp:710-816); phases are
// expanded per group.  "temperature" needs hydro_gpu_heat_create.  Names
// outside the hot path (radiation, mass_source_i, target_density_i) are not
// produced here.
std::vector<Entry> all_entries(int nph) {
  std::vector<Entry> v = {
      {"x", S_NODE_X, 0},          {"y", S_NODE_Y, 1},
      {"z", S_NODE_Z, 2},          {"velocity_x", S_VEL, 0},
      {"velocity_y", S_VEL, 1},    {"velocity_z", S_VEL, 2},
      {"pressure", S_PRESSURE, 0}, {"density", S_DENSITY, 0},
      {"viscosity", S_VISCOSITY, 0}, {"volume_source", S_VOLUME_SOURCE, 0},
      {"temperature", S_TEMPERATURE, 0},
      {"excluded", S_EXCLUDED, 0}, {"divergence", S_DIVERGENCE, 0}};
  const char* groups[4] = {"mass_fraction_", "density_", "partial_density_", "volume_fraction_"};
  const Src gs[4] = {S_MASS_FRACTION, S_TRUE_DENSITY, S_PARTIAL_DENSITY, S_VOLUME_FRACTION};
  for (int gi = 0; gi < 4; ++gi)
    for (int i = 0; i < nph; ++i) v.push_back({groups[gi] + std::to_string(i), gs[gi], i});
  return v;
}

// Selection from a comma/space separated list (or the defaults of
// examples/general.hydroconf:156-180 when null or empty).
int select_entries(const char* list, int dim, int nph, std::vector<Entry>* out) {
  std::vector<Entry> all = all_entries(nph);
  std::vector<std::string> want;
  if (!list || !*list) {
    want = {"x", "y", "velocity_x", "velocity_y", "pressure"};
    if (dim == 3) {
      want.push_back("z");
      want.push_back("velocity_z");
    }
    for (int i = 0; i < nph && i < 2; ++i) want.push_back("volume_fraction_" + std::to_string(i));
  } else {
    std::string cur;
    for (const char* p = list;; ++p) {
      if (*p == ',' || *p == ' ' || *p == 0) {
        if (!cur.empty()) want.push_back(cur);
        cur.clear();
        if (!*p) break;
      } else {
        cur += *p;
      }
    }
  }
  for (auto& w : want) {
    bool found = false;
    for (auto& e : all) found |= (e.name == w);
    if (!found) return HYDRO_ERR_UNSUPPORTED;
  }
  out->clear();
  for (auto& e : all)
    for (auto& w : want)
      if (e.name == w) {
        out->push_back(e);
        break;
      }
  return HYDRO_OK;
}

}  // namespace

// ------------------------------------------------------------------ API --
extern "C" int hydro_vts_write_host(const char* path, int dim, const int* n, const double* lo,
                                    const double* hi, int nentries, const char* const* names,
                                    const int* on_nodes, const double* const* data) {
  if (!path || !n || !lo || !hi || nentries < 0 || (nentries && (!names || !on_nodes || !data)) ||
      (dim != 2 && dim != 3))
    return HYDRO_ERR_ARG;
  Grid g;
  g.dim = dim;
  for (int d = 0; d < dim; ++d) {
    if (n[d] < 1) return HYDRO_ERR_ARG;
    g.n[d] = n[d];
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
  }
  std::vector<Entry> ents;
  std::vector<const double*> ptrs;
  for (int i = 0; i < nentries; ++i) {
    ents.push_back({names[i], on_nodes[i] ? S_NODE_X : S_PRESSURE, 0});
    ptrs.push_back(data[i]);
  }
  return write_file(path, format_vts(g, ents, ptrs));
}

struct hydro_output {
  hydro_ctx* ctx = nullptr;
  hydro_desc d;
  Grid g;
  std::string base;
  std::vector<Entry> ents;
  FILE* pvd = nullptr;
  int frame = 0;
  // staging: pinned host copies of the device arrays a frame needs
  double *h_u = nullptr, *h_p = nullptr, *h_rho = nullptr, *h_mu = nullptr, *h_sv = nullptr;
  double* h_T = nullptr;
  double *h_F = nullptr, *h_q = nullptr, *h_a = nullptr;
  std::vector<double> nodes[3];
  cudaStream_t st = nullptr;
  cudaEvent_t ready = nullptr, done = nullptr;
  // worker
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  bool busy = false, quit = false;
  double job_time = 0.;
  int job_frame = 0;
  int status = HYDRO_OK;
  bool need(Src s) const {
    for (auto& e : ents)
      if (e.src == s) return true;
    return false;
  }
  void run();
};

void hydro_output::run() {
  for (;;) {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return busy || quit; });
    if (!busy && quit) return;
    double t = job_time;
    int fr = job_frame;
    lk.unlock();
    int rc = cudaEventSynchronize(done) == cudaSuccess ? HYDRO_OK : HYDRO_ERR_CUDA;
    if (!rc) {
      const long long nc = g.cells();
      std::vector<std::vector<double>> tmp;
      std::vector<const double*> ptrs;
      for (auto& e : ents) {
        const double* p = nullptr;
        switch (e.src) {
          case S_NODE_X: case S_NODE_Y: case S_NODE_Z: p = nodes[e.comp].data(); break;
          case S_VEL: {
            if (e.comp < g.dim) {
              p = h_u + (size_t)e.comp * nc;
            } else {
              tmp.emplace_back(nc, 0.);
              p = tmp.back().data();
            }
            break;
          }
          case S_PRESSURE: p = h_p; break;
          case S_DENSITY: p = h_rho; break;
          case S_VISCOSITY: p = h_mu; break;
          case S_VOLUME_SOURCE: p = h_sv; break;
          case S_TEMPERATURE: p = h_T; break;
          case S_EXCLUDED: tmp.emplace_back(nc, 0.); p = tmp.back().data(); break;
          case S_PARTIAL_DENSITY: p = h_q + (size_t)e.comp * nc; break;
          case S_VOLUME_FRACTION: p = h_a + (size_t)e.comp * nc; break;
          case S_TRUE_DENSITY: tmp.emplace_back(nc, d.density[e.comp]); p = tmp.back().data(); break;
          case S_MASS_FRACTION: {
            tmp.emplace_back(nc);
            for (long long c = 0; c < nc; ++c)
              tmp.back()[c] = h_q[(size_t)e.comp * nc + c] / h_rho[c];
            p = tmp.back().data();
            break;
          }
          case S_DIVERGENCE: {
            // sum of outward volume fluxes / V (hydro2d.hpp:752-760)
            tmp.emplace_back(nc);
            double V = 1.;
            for (int k = 0; k < g.dim; ++k) V *= (g.hi[k] - g.lo[k]) / g.n[k];
            long long fofs = 0;
            std::vector<long long> base(3, 0);
            for (int k = 0; k < g.dim; ++k) {
              base[k] = fofs;
              fofs += (long long)(g.n[0] + (k == 0)) * (g.n[1] + (k == 1)) *
                      (g.dim == 3 ? g.n[2] + (k == 2) : 1);
            }
            for (int kk = 0; kk < (g.dim == 3 ? g.n[2] : 1); ++kk)
              for (int j = 0; j < g.n[1]; ++j)
                for (int i = 0; i < g.n[0]; ++i) {
                  double s = 0.;
                  for (int k = 0; k < g.dim; ++k) {
                    long long fx = g.n[0] + (k == 0), fy = g.n[1] + (k == 1);
                    long long f = base[k] + i + fx * (j + fy * (long long)kk);
                    long long st = k == 0 ? 1 : (k == 1 ? fx : fx * fy);
                    s += h_F[f + st] - h_F[f];
                  }
                  tmp.back()[i + (long long)g.n[0] * (j + (long long)g.n[1] * kk)] = s / V;
                }
            p = tmp.back().data();
            break;
          }
        }
        ptrs.push_back(p);
      }
      std::string name = base + "." + std::to_string(fr) + ".vts";
      rc = write_file(name, format_vts(g, ents, ptrs));
      if (!rc && pvd) {
        char line[64];
        snprintf(line, sizeof(line), "%g", t);
        fprintf(pvd, "    <DataSet timestep=\"%s\" group=\"\" part=\"0\" file=\"%s\"/>\n", line,
                name.c_str());
        fflush(pvd);
      }
    }
    lk.lock();
    if (rc && !status) status = rc;
    busy = false;
    cv.notify_all();
  }
}

namespace {

void free_output(hydro_output* o) {
  if (o->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(o->mu);
      o->quit = true;
    }
    o->cv.notify_all();
    o->worker.join();
  }
  double* hs[] = {o->h_u, o->h_p, o->h_rho, o->h_mu, o->h_sv, o->h_F, o->h_q, o->h_a, o->h_T};
  for (double* h : hs)
    if (h) cudaFreeHost(h);
  if (o->ready) cudaEventDestroy(o->ready);
  if (o->done) cudaEventDestroy(o->done);
  if (o->st) cudaStreamDestroy(o->st);
  if (o->pvd) fclose(o->pvd);
  delete o;
}

}  // namespace

extern "C" int hydro_output_open(hydro_ctx* ctx, const char* basename, const char* fields,
                                 hydro_output** out) {
  if (!ctx || !basename || !out) return HYDRO_ERR_ARG;
  *out = nullptr;
  hydro_output* o = new (std::nothrow) hydro_output();
  if (!o) return HYDRO_ERR_NOMEM;
  o->ctx = ctx;
  int rc = hydro_gpu_get_desc(ctx, &o->d);
  if (!rc) rc = select_entries(fields, o->d.dim, o->d.num_phases, &o->ents);
  if (!rc && o->need(S_TEMPERATURE)) {
    double* t = nullptr;  // the temperature exists once heat is attached
    rc = hydro_gpu_field_ptr(ctx, HYDRO_FIELD_TEMPERATURE, HYDRO_TIME_CURR, &t);
  }
  if (rc) {
    delete o;
    return rc;
  }
  o->base = basename;
  o->g.dim = o->d.dim;
  for (int k = 0; k < o->d.dim; ++k) {
    o->g.n[k] = o->d.n[k];
    o->g.lo[k] = o->d.lo[k];
    o->g.hi[k] = o->d.hi[k];
  }
  const long long nc = o->g.cells();
  const long long nf = [&] {
    long long s = 0;
    for (int k = 0; k < o->g.dim; ++k)
      s += (long long)(o->g.n[0] + (k == 0)) * (o->g.n[1] + (k == 1)) *
           (o->g.dim == 3 ? o->g.n[2] + (k == 2) : 1);
    return s;
  }();
  // node coordinate entries, once
  for (int k = 0; k < 3; ++k) {
    o->nodes[k].resize(o->g.nodes());
    long long idx = 0;
    const int kz = o->g.dim == 3 ? o->g.n[2] + 1 : 1;
    for (int c = 0; c < kz; ++c)
      for (int j = 0; j <= o->g.n[1]; ++j)
        for (int i = 0; i <= o->g.n[0]; ++i) {
          int q[3] = {i, j, c};
          o->nodes[k][idx++] = k < o->g.dim ? o->g.node(k, q[k]) : 0.;
        }
  }
  const int nph = o->d.num_phases;
  bool ok = cudaStreamCreateWithFlags(&o->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&o->ready, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&o->done, cudaEventDisableTiming) == cudaSuccess;
  auto pin = [&](double** h, long long n) {
    if (ok && cudaMallocHost(h, sizeof(double) * n) != cudaSuccess) ok = false;
  };
  if (o->need(S_VEL)) pin(&o->h_u, nc * o->g.dim);
  if (o->need(S_PRESSURE)) pin(&o->h_p, nc);
  if (o->need(S_DENSITY) || o->need(S_MASS_FRACTION)) pin(&o->h_rho, nc);
  if (o->need(S_VISCOSITY)) pin(&o->h_mu, nc);
  if (o->need(S_VOLUME_SOURCE)) pin(&o->h_sv, nc);
  if (o->need(S_TEMPERATURE)) pin(&o->h_T, nc);
  if (o->need(S_DIVERGENCE)) pin(&o->h_F, nf);
  if (o->need(S_PARTIAL_DENSITY) || o->need(S_MASS_FRACTION)) pin(&o->h_q, nc * nph);
  if (o->need(S_VOLUME_FRACTION)) pin(&o->h_a, nc * nph);
  if (ok) o->pvd = fopen((o->base + ".pvd").c_str(), "wb");
  if (!ok || !o->pvd) {
    cudaGetLastError();
    free_output(o);
    return ok ? HYDRO_ERR_IO : HYDRO_ERR_NOMEM;
  }
  fprintf(o->pvd,
          "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\" "
          "byte_order=\"LittleEndian\">\n  <Collection>\n");
  fflush(o->pvd);
  o->worker = std::thread([o] { o->run(); });
  *out = o;
  return HYDRO_OK;
}

extern "C" int hydro_output_flush(hydro_output* o) {
  if (!o) return HYDRO_ERR_ARG;
  std::unique_lock<std::mutex> lk(o->mu);
  o->cv.wait(lk, [&] { return !o->busy; });
  return o->status;
}

extern "C" int hydro_output_write(hydro_output* o, double time) {
  if (!o) return HYDRO_ERR_ARG;
  int rc = hydro_output_flush(o);  // one frame in flight at a time
  if (rc) return rc;
  void* cst = nullptr;
  if ((rc = hydro_gpu_get_stream(o->ctx, &cst))) return rc;
  const long long nc = o->g.cells();
  const int nph = o->d.num_phases;
  auto copy = [&](double* h, int field, int layer, long long n) -> int {
    if (!h) return HYDRO_OK;
    double* dptr = nullptr;
    int r = hydro_gpu_field_ptr(o->ctx, field, layer, &dptr);
    if (r) return r;
    if (cudaMemcpyAsync(h, dptr, sizeof(double) * n, cudaMemcpyDeviceToHost, o->st) != cudaSuccess)
      return HYDRO_ERR_CUDA;
    return HYDRO_OK;
  };
  if (cudaEventRecord(o->ready, (cudaStream_t)cst) != cudaSuccess ||
      cudaStreamWaitEvent(o->st, o->ready, 0) != cudaSuccess)
    return HYDRO_ERR_CUDA;
  long long nf = 0;
  for (int k = 0; k < o->g.dim; ++k)
    nf += (long long)(o->g.n[0] + (k == 0)) * (o->g.n[1] + (k == 1)) *
          (o->g.dim == 3 ? o->g.n[2] + (k == 2) : 1);
  if ((rc = copy(o->h_u, HYDRO_FIELD_VELOCITY, HYDRO_TIME_CURR, nc * o->g.dim)) ||
      (rc = copy(o->h_p, HYDRO_FIELD_PRESSURE, HYDRO_TIME_CURR, nc)) ||
      (rc = copy(o->h_rho, HYDRO_FIELD_DENSITY, HYDRO_TIME_CURR, nc)) ||
      (rc = copy(o->h_mu, HYDRO_FIELD_VISCOSITY, HYDRO_TIME_CURR, nc)) ||
      (rc = copy(o->h_sv, HYDRO_FIELD_VOLUME_SOURCE, HYDRO_TIME_CURR, nc)) ||
      (rc = copy(o->h_T, HYDRO_FIELD_TEMPERATURE, HYDRO_TIME_CURR, nc)) ||
      (rc = copy(o->h_F, HYDRO_FIELD_VOLUME_FLUX, HYDRO_TIME_CURR, nf)) ||
      (rc = copy(o->h_q, HYDRO_FIELD_PARTIAL_DENSITY, HYDRO_TIME_CURR, nc * nph)) ||
      (rc = copy(o->h_a, HYDRO_FIELD_VOLUME_FRACTION, HYDRO_TIME_CURR, nc * nph)))
    return rc;
  if (cudaEventRecord(o->done, o->st) != cudaSuccess) return HYDRO_ERR_CUDA;
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->job_time = time;
    o->job_frame = o->frame++;
    o->busy = true;
  }
  o->cv.notify_all();
  return HYDRO_OK;
}

extern "C" int hydro_output_close(hydro_output* o) {
  if (!o) return HYDRO_OK;
  int rc = hydro_output_flush(o);
  if (o->pvd) {
    fprintf(o->pvd, "  </Collection>\n</VTKFile>\n");
    if (fclose(o->pvd) != 0 && !rc) rc = HYDRO_ERR_IO;
    o->pvd = nullptr;
  }
  free_output(o);
  return rc;
}

// ------------------------------------------------------- scalar series --
struct hydro_scalar_output {
  hydro_ctx* ctx = nullptr;
  hydro_desc d;
  FILE* f = nullptr;
  double vin[HYDRO_MAX_PHASES] = {}, vout[HYDRO_MAX_PHASES] = {};
};

extern "C" int hydro_scalar_output_open(hydro_ctx* ctx, const char* filename,
                                        hydro_scalar_output** out) {
  if (!ctx || !filename || !out) return HYDRO_ERR_ARG;
  *out = nullptr;
  hydro_scalar_output* s = new (std::nothrow) hydro_scalar_output();
  if (!s) return HYDRO_ERR_NOMEM;
  s->ctx = ctx;
  int rc = hydro_gpu_get_desc(ctx, &s->d);
  if (rc) {
    delete s;
    return rc;
  }
  s->f = fopen(filename, "wb");
  if (!s->f) {
    delete s;
    return HYDRO_ERR_IO;
  }
  const int nph = s->d.num_phases, dim = s->d.dim;
  std::string h = "time num_iters iter_diff_velocity ";
  for (int i = 0; i < nph; ++i)
    h += "mass_" + std::to_string(i) + " mass_in_" + std::to_string(i) + " mass_out_" +
         std::to_string(i) + " ";
  for (int i = 0; i < nph; ++i)
    h += "volume_" + std::to_string(i) + " volume_in_" + std::to_string(i) + " volume_out_" +
         std::to_string(i) + " ";
  for (int i = 0; i < nph; ++i)
    h += "pd_min_" + std::to_string(i) + " pd_max_" + std::to_string(i) + " ";
  const char* cn[3] = {"cx_", "cy_", "cz_"};
  const char* vn[3] = {"vx_", "vy_", "vz_"};
  for (int i = 0; i < nph; ++i) {
    for (int k = 0; k < dim; ++k) h += cn[k] + std::to_string(i) + " ";
    for (int k = 0; k < dim; ++k) h += vn[k] + std::to_string(i) + " ";
  }
  fprintf(s->f, "%s\n", h.c_str());
  fflush(s->f);
  *out = s;
  return HYDRO_OK;
}

// One row: time and the SIMPLE iteration count are the caller's (the
// module's "t" and "s"), the rest comes from the context.  The boundary
// in/out volumes accumulate the current step's boundary fluxes times dt
// (hydro2d.hpp:1474-1509).
extern "C" int hydro_scalar_output_write(hydro_scalar_output* s, double time, int num_iters) {
  if (!s) return HYDRO_ERR_ARG;
  hydro_stat st;
  int rc = hydro_gpu_calc_stat(s->ctx, &st);
  if (rc) return rc;
  double ind = 0.;
  if ((rc = hydro_gpu_get_convergence_indicator(s->ctx, &ind))) return rc;
  double dt = 0.;
  if ((rc = hydro_gpu_get_time_step(s->ctx, &dt))) return rc;
  const int nph = s->d.num_phases, dim = s->d.dim;
  for (int i = 0; i < nph; ++i) {
    s->vin[i] += st.volume_flux_in[i] * dt;
    s->vout[i] += st.volume_flux_out[i] * dt;
  }
  std::string r;
  put_g(r, time);
  put_g(r, (double)num_iters);
  put_g(r, ind);
  for (int i = 0; i < nph; ++i) {
    put_g(r, st.mass[i]);
    put_g(r, s->vin[i] * s->d.density[i]);
    put_g(r, s->vout[i] * s->d.density[i]);
  }
  for (int i = 0; i < nph; ++i) {
    put_g(r, st.volume[i]);
    put_g(r, s->vin[i]);
    put_g(r, s->vout[i]);
  }
  for (int i = 0; i < nph; ++i) {
    put_g(r, st.pd_min[i]);
    put_g(r, st.pd_max[i]);
  }
  for (int i = 0; i < nph; ++i) {
    for (int k = 0; k < dim; ++k) put_g(r, st.center[i][k]);
    for (int k = 0; k < dim; ++k) put_g(r, st.velocity[i][k]);
  }
  fprintf(s->f, "%s\n", r.c_str());
  fflush(s->f);
  return HYDRO_OK;
}

extern "C" int hydro_scalar_output_close(hydro_scalar_output* s) {
  if (!s) return HYDRO_OK;
  int rc = HYDRO_OK;
  if (s->f && fclose(s->f) != 0) rc = HYDRO_ERR_IO;
  delete s;
  return rc;
}
