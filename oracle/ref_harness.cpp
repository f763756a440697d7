// ref_harness.cpp -- drives the reference's own solver classes (divfree/hydro,
// source/hydro2dmpi/*.hpp, included unchanged from the reference tree) so
// that golden vectors can be produced for the parity tests.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ in
// the container that holds the reference; never part of the product and
// never run on the GPU machine.  The orchestration below restates
// hydro<Mesh>::step (hydro2d.hpp:1531-1621) and UpdateFluidProperties
// (hydro2d.hpp:1404-1430) because the module class needs the console
// runtime; the solver arithmetic is entirely the reference's:
// FluidSimple (fluid.hpp:421-1207), AdvectionSolverMultiExplicit
// (advection.hpp:368-555), GetSmoothField/Interpolate/Gradient
// (solver.hpp), and the linear solvers of linear.hpp.
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "mesh2d.hpp"
#include "mesh3d.hpp"
#include "fluid.hpp"
#include "advection.hpp"
#include "heat.hpp"

// The ParaView session names its files with an integer-to-text helper from
// the reference's common library (not part of these headers); the harness
// supplies one (decimal, as an ostream prints it).
#include <sstream>
#include <string>
static std::string IntToStr(size_t a) {
  std::ostringstream s;
  s << a;
  return s.str();
}
#include "output_paraview.hpp"

#include "../include/hydro_gpu.h"

// HYDRO_ADAPTER: the same harness with the reference-side adapter classes
// (FluidSimpleGpu, AdvectionSolverMultiGpu) in place of FluidSimple and
// AdvectionSolverMultiExplicit, constructed with the same arguments and
// stepped through the same FluidSolver / AdvectionSolverMulti calls; linked
// with adapter_shim.c, which forwards the C-ABI to the CPU oracle.
#ifdef HYDRO_ADAPTER
#include "../hydro_gb300/adapter/fluid_simple_gpu.hpp"
#endif

namespace {

template <class Mesh>
struct Case {
  static constexpr size_t dim = Mesh::dim;
  using Scal = double;
  using Vect = typename Mesh::Vect;
  using MIdx = typename Mesh::MIdx;
  template <class T> using FieldCell = geom::FieldCell<T>;
  template <class T> using FieldFace = geom::FieldFace<T>;
  using IdxCell = geom::IdxCell;
  using IdxFace = geom::IdxFace;

  hydro_desc d;
  Mesh mesh;
  size_t nph;
  FieldCell<Scal> fc_density, fc_density_smooth, fc_viscosity_smooth;
  FieldCell<Scal> fc_volume_source, fc_mass_source;
  std::vector<FieldCell<Scal>> v_fc_mass_source, v_fc_volume_fraction;
  std::vector<FieldFace<Scal>> v_ff_volume_flux_slip;
  std::vector<const FieldFace<Scal>*> v_p_ff_volume_flux_slip;
  std::vector<const FieldCell<Scal>*> v_p_fc_mass_source;
  FieldCell<Vect> fc_force, fc_stforce;
  FieldFace<Vect> ff_stforce;
  std::vector<geom::MapFace<std::shared_ptr<solver::ConditionFace>>> v_cond;
  MultiTimer<std::string> timer;
#ifdef HYDRO_ADAPTER
  using Fluid = solver::FluidSimpleGpu<Mesh>;
  using Adv = solver::AdvectionSolverMultiGpu<Mesh>;
#else
  using Fluid = solver::FluidSimple<Mesh>;
  using Adv = solver::AdvectionSolverMultiExplicit<Mesh, FieldFace<Scal>>;
#endif
  std::shared_ptr<Fluid> fluid;
  std::shared_ptr<Adv> adv;
  // heat (hydro2d.hpp:650-687), when hd is given
  const hydro_heat_desc* hd = nullptr;
  FieldCell<Scal> fc_conductivity, fc_temperature_source;
  std::shared_ptr<solver::HeatSolver<Mesh>> heat;
  std::shared_ptr<const solver::LinearSolverFactory> fheat;

  static std::shared_ptr<const solver::LinearSolverFactory> Factory(
      int kind, double tol, int limit, double omega) {
    using namespace solver;
    switch (kind) {
      case HYDRO_LINEAR_LU:
        return std::make_shared<const LinearSolverFactory>(
            std::make_shared<const LuDecompositionFactory>());
      case HYDRO_LINEAR_JACOBI:
        return std::make_shared<const LinearSolverFactory>(
            std::make_shared<const JacobiFactory>(tol, limit, omega));
      default:
        return std::make_shared<const LinearSolverFactory>(
            std::make_shared<const GaussSeidelFactory>(tol, limit, omega));
    }
  }

  Vect V3(const double* a) const {
    Vect v;
    for (size_t i = 0; i < dim; ++i) v[i] = a[i];
    return v;
  }

  // side of a boundary face (mesh-block index at the low/high end)
  int Side(IdxFace f) const {
    auto dir = mesh.GetDirection(f);
    auto mi = mesh.GetBlockFaces().GetMIdx(f);
    if (mi[dir] == 0) return 2 * int(dir);
    return 2 * int(dir) + 1;
  }

  Case(const hydro_desc& desc, const double* u0, const double* q0,
       const hydro_heat_desc* heat_desc = nullptr)
      : d(desc), hd(heat_desc) {
    MIdx size;
    Vect lo, hi;
    for (size_t i = 0; i < dim; ++i) {
      size[i] = d.n[i];
      lo[i] = d.lo[i];
      hi[i] = d.hi[i];
    }
    geom::InitUniformMesh(mesh, geom::Rect<Vect>(lo, hi), size);
    nph = d.num_phases;
    size_t nc = mesh.GetNumCells();

    // fluid conditions: one per boundary face (hydro2d.hpp:357-383); with a
    // rigid box, "wall 0 0 0" on the faces between box and fluid cells,
    // then the box cells are excluded and the conditions of excluded faces
    // erased (hydro2d.hpp:306-423)
    geom::MapFace<std::shared_ptr<solver::ConditionFaceFluid>> fluid_cond;
    geom::Rect<Vect> rigid_box(V3(d.rigid_box_lo), V3(d.rigid_box_hi));
    auto in_box = [&](IdxCell c) {
      return d.rigid_box && !c.IsNone() && rigid_box.IsInside(mesh.GetCenter(c));
    };
    for (auto f : mesh.Faces()) {
      if (!mesh.IsInner(f)) {
        int s = Side(f);
        Vect vel = V3(d.bc_velocity[s]);
        if (d.bc_kind[s] == HYDRO_BC_INLET) {
          fluid_cond[f] = std::make_shared<solver::fluid_condition::InletFixed<Mesh>>(
              vel, mesh.GetValidNeighbourCellId(f));
        } else if (d.bc_kind[s] == HYDRO_BC_OUTLET) {
          fluid_cond[f] = std::make_shared<solver::fluid_condition::OutletAuto<Mesh>>(
              mesh.GetValidNeighbourCellId(f));
        } else {
          fluid_cond[f] =
              std::make_shared<solver::fluid_condition::NoSlipWallFixed<Mesh>>(vel);
        }
      } else if (in_box(mesh.GetNeighbourCell(f, 0)) != in_box(mesh.GetNeighbourCell(f, 1))) {
        fluid_cond[f] =
            std::make_shared<solver::fluid_condition::NoSlipWallFixed<Mesh>>(Vect(0));
      }
    }
    if (d.rigid_box) {
      std::vector<IdxCell> excluded;
      for (auto c : mesh.Cells())
        if (in_box(c)) excluded.push_back(c);
      mesh.ExcludeCells(excluded);
      for (auto f : mesh.Faces())
        if (mesh.IsExcluded(f)) fluid_cond.erase(f);
    }
    geom::MapCell<std::shared_ptr<solver::ConditionCellFluid>> mc_cond;
    if (d.pressure_fixed_cell >= 0) {
      mc_cond[IdxCell(d.pressure_fixed_cell)] = std::make_shared<
          solver::fluid_condition::GivenPressureFixed<Mesh>>(d.pressure_fixed_value);
    }
    FieldCell<Vect> fc_vel0(mesh);
    for (size_t c = 0; c < nc; ++c)
      for (size_t k = 0; k < dim; ++k) fc_vel0[IdxCell(c)][k] = u0[k * nc + c];

    fc_density.Reinit(mesh, 0.);
    fc_density_smooth.Reinit(mesh, 0.);
    fc_viscosity_smooth.Reinit(mesh, 0.);
    fc_volume_source.Reinit(mesh, 0.);
    fc_mass_source.Reinit(mesh, 0.);
    fc_force.Reinit(mesh, Vect(0));
    fc_stforce.Reinit(mesh, Vect(0));
    ff_stforce.Reinit(mesh, Vect(0));

    auto fv = Factory(d.velocity_solver, d.velocity_tolerance,
                      d.velocity_iters_limit, d.velocity_omega);
    auto fp = Factory(d.pressure_solver, d.pressure_tolerance,
                      d.pressure_iters_limit, d.pressure_omega);
    fluid = std::make_shared<Fluid>(
        mesh, fc_vel0, fluid_cond, mc_cond, d.velocity_relaxation_factor,
        d.pressure_relaxation_factor, d.rhie_chow_factor, &fc_density_smooth,
        &fc_viscosity_smooth, &fc_force, &fc_stforce, &ff_stforce,
        &fc_volume_source, &fc_mass_source, 0., d.dt, *fv, *fp,
        d.convergence_tolerance, d.num_iterations_limit, &timer,
        d.time_second_order != 0, d.simpler != 0, d.force_geometric_average != 0,
        d.guess_extrapolation, V3(d.meshvel));
#ifdef HYDRO_ADAPTER
    fluid->SetLinearTolerances(d.velocity_tolerance, d.velocity_iters_limit,
                               d.pressure_tolerance, d.pressure_iters_limit);
#endif

    // advection (hydro2d.hpp:483-600): zero-derivative walls, value inlets
    v_fc_mass_source.resize(nph);
    v_ff_volume_flux_slip.resize(nph);
    v_fc_volume_fraction.resize(nph);
    v_p_ff_volume_flux_slip.resize(nph);
    v_p_fc_mass_source.resize(nph);
    std::vector<FieldCell<Scal>> q_init(nph);
    v_cond.resize(nph);
    for (size_t i = 0; i < nph; ++i) {
      v_fc_mass_source[i].Reinit(mesh, 0.);
      v_ff_volume_flux_slip[i].Reinit(mesh, 0.);
      v_fc_volume_fraction[i].Reinit(mesh, 0.);
      v_p_ff_volume_flux_slip[i] = &v_ff_volume_flux_slip[i];
      v_p_fc_mass_source[i] = &v_fc_mass_source[i];
      q_init[i].Reinit(mesh);
      for (size_t c = 0; c < nc; ++c) q_init[i][IdxCell(c)] = q0[i * nc + c];
      // one per fluid condition (hydro2d.hpp:563-583): inlets hold the
      // initial value of their cell, the others zero derivative
      for (auto it = fluid_cond.cbegin(); it != fluid_cond.cend(); ++it) {
        IdxFace f = it->GetIdx();
        if (dynamic_cast<solver::fluid_condition::Inlet<Mesh>*>(it->GetValue().get())) {
          IdxCell cc = mesh.GetNeighbourCell(f, mesh.GetValidNeighbourCellId(f));
          v_cond[i][f] = std::make_shared<solver::ConditionFaceValueFixed<Scal>>(q_init[i][cc]);
        } else {
          v_cond[i][f] = std::make_shared<solver::ConditionFaceDerivativeFixed<Scal>>(0.);
        }
      }
    }
    std::vector<Scal> rho(d.density, d.density + nph);
#ifdef HYDRO_ADAPTER
    // the adapters share one context: the fluxes stay on its side
    adv = std::make_shared<Adv>(*fluid, mesh, q_init, v_cond, nullptr, v_p_ff_volume_flux_slip,
                                v_p_fc_mass_source, 0., d.dt * d.advection_dt_factor,
                                d.tvd_split != 0, d.sharp, rho);
#else
    adv = std::make_shared<Adv>(
        mesh, q_init, v_cond, &fluid->GetVolumeFlux(solver::Layers::iter_curr),
        v_p_ff_volume_flux_slip, v_p_fc_mass_source, 0.,
        d.dt * d.advection_dt_factor, d.tvd_split != 0, d.sharp, rho);
#endif
    UpdateProperties();
#ifdef HYDRO_ADAPTER
    if (hd) throw std::runtime_error("the adapter variant runs no temperature");
#endif
    if (hd) {
      geom::MapFace<std::shared_ptr<solver::ConditionFace>> tcond;
      geom::Rect<Vect> box(V3(hd->box_lo), V3(hd->box_hi));
      for (auto f : mesh.Faces()) {
        if (mesh.IsInner(f)) continue;
        if (box.IsInside(mesh.GetCenter(f)))
          tcond[f] = std::make_shared<solver::ConditionFaceValueFixed<Scal>>(hd->box_temperature);
        else
          tcond[f] = std::make_shared<solver::ConditionFaceDerivativeFixed<Scal>>(0.);
      }
      fc_temperature_source.Reinit(mesh, 0.);
      fheat = Factory(hd->solver, hd->tolerance, hd->iters_limit, 1.);
      heat = std::make_shared<solver::HeatSolver<Mesh>>(
          mesh, FieldCell<Scal>(mesh, hd->temperature_initial), tcond, hd->relaxation_factor,
          &fc_conductivity, &fc_temperature_source,
          &fluid->GetVolumeFlux(solver::Layers::iter_curr), 0., hd->dt, *fheat, 0.5, 1,
          hd->time_second_order != 0);
    }
  }

  // UpdateFluidProperties (hydro2d.hpp:1404-1430), mass sources zero.
  void UpdateProperties() {
    size_t nc = mesh.GetNumCells();
    for (size_t c = 0; c < nc; ++c) {
      IdxCell ic(c);
      Scal sum = 0.;
      for (size_t i = 0; i < nph; ++i) {
        v_fc_volume_fraction[i][ic] = adv->GetField(i)[ic] / d.density[i];
        sum += v_fc_volume_fraction[i][ic];
      }
      for (size_t i = 0; i < nph; ++i) v_fc_volume_fraction[i][ic] /= sum;
    }
    FieldCell<Scal> mu(mesh, 0.);
    fc_density.Reinit(mesh, 0.);
    for (size_t i = 0; i < nph; ++i)
      for (size_t c = 0; c < nc; ++c)
        fc_density[IdxCell(c)] += d.density[i] * v_fc_volume_fraction[i][IdxCell(c)];
    for (size_t i = 0; i < nph; ++i)
      for (size_t c = 0; c < nc; ++c)
        mu[IdxCell(c)] += d.viscosity[i] * v_fc_volume_fraction[i][IdxCell(c)];
    fc_density_smooth = solver::GetSmoothField(fc_density, mesh, d.density_smooth_times);
    fc_viscosity_smooth = solver::GetSmoothField(mu, mesh, d.viscosity_smooth_times);
    fc_mass_source.Reinit(mesh, 0.);
    fc_volume_source.Reinit(mesh, 0.);
    Vect g = V3(d.gravity), f0 = V3(d.force);
    fc_force.Reinit(mesh);
    for (size_t c = 0; c < nc; ++c)
      fc_force[IdxCell(c)] = g * fc_density[IdxCell(c)] + f0;
    fc_stforce.Reinit(mesh, Vect(0));
    ff_stforce.Reinit(mesh, Vect(0));
    if (nph >= 2) {
      // surface tension from the reference operators (hydro2d.hpp:1318-1370)
      auto& a = v_fc_volume_fraction[1];
      auto af = solver::Interpolate(a, v_cond[0], mesh);
      auto gc = solver::Gradient(af, mesh);
      geom::MapFace<std::shared_ptr<solver::ConditionFace>> mfvz;
      for (auto f : mesh.Faces())
        if (!mesh.IsExcluded(f) && !mesh.IsInner(f))
          mfvz[f] = std::make_shared<solver::ConditionFaceDerivativeFixed<Vect>>(Vect(0));
      auto gf = solver::Interpolate(gc, mfvz, mesh);
      for (auto c : mesh.Cells()) {
        Vect f(0);
        for (size_t i = 0; i < mesh.GetNumNeighbourFaces(c); ++i) {
          IdxFace fi = mesh.GetNeighbourFace(c, i);
          Vect gv = gf[fi];
          Vect nv = gf[fi];
          nv /= (nv.norm() + 1e-6);
          Vect s = mesh.GetOutwardSurface(c, i);
          f += gv * s.dot(nv);
          f -= s * gv.norm();
        }
        f /= mesh.GetVolume(c);
        fc_stforce[c] = f * d.sigma;
      }
    }
    fc_force = solver::GetSmoothField(fc_force, mesh, d.force_smooth_times);
    if (hd) {
      fc_conductivity.Reinit(mesh, 0.);
      for (size_t i = 0; i < nph; ++i)
        for (size_t c = 0; c < nc; ++c)
          fc_conductivity[IdxCell(c)] += hd->conductivity[i] * v_fc_volume_fraction[i][IdxCell(c)];
    }
  }

  // hydro<Mesh>::step (hydro2d.hpp:1531-1621)
  void Step(hydro_step_stats* st) {
    if (d.dt_auto) {
      double dtm = fluid->GetAutoTimeStep();
      double dt = dtm * d.cfl, dta = dtm * d.cfl_advection;
      if (d.dt_max > 0. && dt > d.dt_max) {
        dta = dta * (d.dt_max / dt);
        dt = d.dt_max;
      }
      fluid->SetTimeStep(dt);
      adv->SetTimeStep(dta);
    }
    fluid->StartStep();
    while (!fluid->IsConverged()) fluid->MakeIteration();
    st->outer_iterations = (int)fluid->GetIterationCount();
    st->convergence_indicator = fluid->GetConvergenceIndicator();
    fluid->FinishStep();
    int ns = 0;
    if (d.advection_enable) {
      while (adv->GetTime() < fluid->GetTime() - 0.5 * adv->GetTimeStep()) {
        adv->StartStep();
        adv->CalcStep();
        adv->FinishStep();
        ++ns;
      }
    }
    st->advection_substeps = ns;
    if (heat) {
      heat->StartStep();
      heat->CalcStep();
      heat->FinishStep();
    }
    st->dt = fluid->GetTimeStep();
    st->dt_advection = adv->GetTimeStep();
    st->time = fluid->GetTime();
    UpdateProperties();
  }

  void Dump(double* u, double* p, double* F, double* q) {
    size_t nc = mesh.GetNumCells(), nf = mesh.GetNumFaces();
    const auto& vel = fluid->GetVelocity();
    const auto& pr = fluid->GetPressure();
    const auto& fl = fluid->GetVolumeFlux();
    for (size_t c = 0; c < nc; ++c) {
      for (size_t k = 0; k < dim; ++k) u[k * nc + c] = vel[IdxCell(c)][k];
      p[c] = pr[IdxCell(c)];
    }
    for (size_t f = 0; f < nf; ++f) F[f] = fl[IdxFace(f)];
    for (size_t i = 0; i < nph; ++i)
      for (size_t c = 0; c < nc; ++c) q[i * nc + c] = adv->GetField(i)[IdxCell(c)];
  }
};

template <class Mesh>
int Run(const hydro_desc* d, const double* u0, const double* q0, int nsteps,
        double* u, double* p, double* F, double* q, hydro_step_stats* stats,
        const hydro_heat_desc* hd = nullptr, double* T = nullptr) {
  // The reference's linear solvers print one line per solve
  // (linear.hpp:647,712,779); keep it off the test output.
  std::streambuf* saved = std::cout.rdbuf(nullptr);
  int rc = HYDRO_OK;
  try {
    Case<Mesh> cs(*d, u0, q0, hd);
    for (int s = 0; s < nsteps; ++s) cs.Step(&stats[s]);
    cs.Dump(u, p, F, q);
    if (hd && T) {
      const auto& t = cs.heat->GetTemperature();
      for (size_t c = 0; c < cs.mesh.GetNumCells(); ++c) T[c] = t[geom::IdxCell(c)];
    }
  } catch (const std::string& e) {
    rc = HYDRO_ERR_NAN;
  } catch (...) {
    rc = HYDRO_ERR_ARG;
  }
  std::cout.rdbuf(saved);
  std::cout.clear();
  return rc;
}

}  // namespace

extern "C" int ref_run(const hydro_desc* d, const double* u0, const double* q0,
                       int nsteps, double* u, double* p, double* F, double* q,
                       hydro_step_stats* stats) {
  if (d->dim == 2)
    return Run<geom::geom2d::MeshStructured<double>>(d, u0, q0, nsteps, u, p, F, q, stats);
  if (d->dim == 3)
    return Run<geom::geom3d::MeshStructured<double>>(d, u0, q0, nsteps, u, p, F, q, stats);
  return HYDRO_ERR_ARG;
}

// GetSmoothField (solver.hpp:636-656) of a cell field, for pinning the
// initialisation helpers.
extern "C" int ref_run_heat(const hydro_desc* d, const hydro_heat_desc* hd, const double* u0,
                            const double* q0, int nsteps, double* u, double* p, double* F,
                            double* q, double* T, hydro_step_stats* stats) {
  if (d->dim == 2)
    return Run<geom::geom2d::MeshStructured<double>>(d, u0, q0, nsteps, u, p, F, q, stats, hd,
                                                     T);
  return Run<geom::geom3d::MeshStructured<double>>(d, u0, q0, nsteps, u, p, F, q, stats, hd, T);
}

extern "C" int ref_smooth(int dim, const int* n, double* field, int repeat) {
  if (dim == 2) {
    using Mesh = geom::geom2d::MeshStructured<double>;
    Mesh m;
    geom::InitUniformMesh(m, geom::Rect<Mesh::Vect>(Mesh::Vect(0., 0.), Mesh::Vect(1., 1.)),
                          Mesh::MIdx(n[0], n[1]));
    geom::FieldCell<double> fc(m);
    for (size_t c = 0; c < m.GetNumCells(); ++c) fc[geom::IdxCell(c)] = field[c];
    fc = solver::GetSmoothField(fc, m, repeat);
    for (size_t c = 0; c < m.GetNumCells(); ++c) field[c] = fc[geom::IdxCell(c)];
    return HYDRO_OK;
  }
  using Mesh = geom::geom3d::MeshStructured<double>;
  Mesh m;
  geom::InitUniformMesh(m, geom::Rect<Mesh::Vect>(Mesh::Vect(0., 0., 0.), Mesh::Vect(1., 1., 1.)),
                        Mesh::MIdx(n[0], n[1], n[2]));
  geom::FieldCell<double> fc(m);
  for (size_t c = 0; c < m.GetNumCells(); ++c) fc[geom::IdxCell(c)] = field[c];
  fc = solver::GetSmoothField(fc, m, repeat);
  for (size_t c = 0; c < m.GetNumCells(); ++c) field[c] = fc[geom::IdxCell(c)];
  return HYDRO_OK;
}

// Writes one frame with the reference's ParaView session
// (output_paraview.hpp:34-175) for given node and cell arrays on a uniform
// block (InitUniformMesh, mesh.hpp:723-736); the collection footer is
// written when the session ends.  Golden output for the GPU library's
// .vts/.pvd writer.
namespace {
template <class Mesh>
int write_vts(const int* n, const double* lo, const double* hi, int nnode, const char** nnames,
              const double** ndata, int ncell, const char** cnames, const double** cdata,
              const char* base, int nframes, const double* times) {
  using MIdx = typename Mesh::MIdx;
  using Vect = typename Mesh::Vect;
  using IdxNode = geom::IdxNode;
  using IdxCell = geom::IdxCell;
  Mesh mesh;
  MIdx size;
  Vect a, b;
  for (size_t k = 0; k < Mesh::dim; ++k) {
    size[k] = n[k];
    a[k] = lo[k];
    b[k] = hi[k];
  }
  geom::InitUniformMesh(mesh, geom::Rect<Vect>(a, b), size);
  output::Content content;
  for (int i = 0; i < nnode; ++i) {
    const double* f = ndata[i];
    content.push_back(std::make_shared<output::EntryFunction<double, IdxNode, Mesh>>(
        nnames[i], mesh, [f](IdxNode idx) { return f[idx.GetRaw()]; }));
  }
  for (int i = 0; i < ncell; ++i) {
    const double* f = cdata[i];
    content.push_back(std::make_shared<output::EntryFunction<double, IdxCell, Mesh>>(
        cnames[i], mesh, [f](IdxCell idx) { return f[idx.GetRaw()]; }));
  }
  {
    output::SessionParaviewStructured<Mesh> session(content, "title", base, mesh);
    for (int f = 0; f < nframes; ++f) session.Write(times[f], "");
  }
  return 0;
}
}  // namespace

extern "C" int ref_write_vts(int dim, const int* n, const double* lo, const double* hi,
                             int nnode, const char** nnames, const double** ndata, int ncell,
                             const char** cnames, const double** cdata, const char* base,
                             int nframes, const double* times) {
  if (dim == 2)
    return write_vts<geom::geom2d::MeshStructured<double>>(n, lo, hi, nnode, nnames, ndata, ncell,
                                                           cnames, cdata, base, nframes, times);
  return write_vts<geom::geom3d::MeshStructured<double>>(n, lo, hi, nnode, nnames, ndata, ncell,
                                                         cnames, cdata, base, nframes, times);
}
