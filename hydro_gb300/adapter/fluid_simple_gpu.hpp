// fluid_simple_gpu.hpp -- reference-side binding of libhydro_gpu.so.
//
// Drop-in classes for divfree/hydro's module (source/hydro2dmpi/hydro2d.hpp):
//   solver::FluidSimpleGpu<Mesh>            : solver::FluidSolver<Mesh>
//       constructed with FluidSimple's argument list (fluid.hpp:644-670)
//   solver::AdvectionSolverMultiGpu<Mesh>   : solver::AdvectionSolverMulti<Mesh, FieldFace>
//       constructed with AdvectionSolverMultiExplicit's list (advection.hpp:388-398)
//   solver::HeatSolverGpu<Mesh>             : solver::UnsteadyIterativeSolver
//       constructed with HeatSolver's list (heat.hpp:33-47)
// All share one GPU context (GpuHotPath).  Fields the module owns (density,
// viscosity, force, surface-tension force, sources) are read through the
// same raw pointers FluidSimple keeps and uploaded at StartStep; layers the
// solver owns are downloaded on Get*(layer).  Errors follow the reference:
// NaN -> throw std::string (fluid.hpp:795-797, 1164-1166), configuration ->
// std::runtime_error (fluid.hpp:415, 720).
//
// Include after the reference headers (mesh*.hpp, fluid.hpp, advection.hpp)
// and link with -lhydro_gpu.
#pragma once

#include <algorithm>
#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hydro_gpu.h"

namespace solver {

template <class Mesh>
class GpuHotPath {
 public:
  using Scal = typename Mesh::Scal;
  using Vect = typename Mesh::Vect;
  static constexpr size_t dim = Mesh::dim;

  explicit GpuHotPath(const Mesh& mesh) : mesh_(mesh) {
    hydro_desc_default(&desc_);
    desc_.dim = (int)dim;
    auto n = mesh.GetBlockCells().GetDimensions();
    auto nodes = mesh.GetBlockNodes();
    Vect lo = mesh.GetNode(nodes.GetIdx(nodes.GetBegin()));
    auto last = nodes.GetEnd();
    for (size_t d = 0; d < dim; ++d) last[d] -= 1;
    Vect hi = mesh.GetNode(nodes.GetIdx(last));
    for (size_t d = 0; d < dim; ++d) {
      desc_.n[d] = (int)n[d];
      desc_.lo[d] = lo[d];
      desc_.hi[d] = hi[d];
    }
    // the reference's compile-time periodicity (mesh2d.hpp:288,
    // mesh3d.hpp:306-317)
#ifdef PERX
    desc_.periodic[0] = 1;
#endif
#ifdef PERZ
    if (dim == 3) desc_.periodic[2] = 1;
#endif
  }
  ~GpuHotPath() {
    if (ctx_) hydro_gpu_destroy(ctx_);
  }
  hydro_desc& desc() { return desc_; }
  const Mesh& mesh() const { return mesh_; }
  size_t nc() const { return mesh_.GetNumCells(); }
  size_t nf() const { return mesh_.GetNumFaces(); }

  static void Check(int st, const char* where) {
    // a solve stopped at its iteration limit is not an error: the reference
    // goes on past a solver's limit (linear.hpp:690-710)
    if (st == HYDRO_OK || st == HYDRO_NOT_CONVERGED) return;
    if (st == HYDRO_ERR_NAN) throw std::string("NaN pressure");
    throw std::runtime_error(std::string(where) + ": hydro_gpu status " + std::to_string(st));
  }

  // The context is created at first use, once both adapters are built.
  hydro_ctx* ctx() {
    if (!ctx_) {
      Check(hydro_gpu_create(&desc_, &ctx_), "hydro_gpu_create");
      Check(hydro_gpu_set_field(ctx_, HYDRO_FIELD_VELOCITY, HYDRO_TIME_CURR, u0_.data(),
                                u0_.size()),
            "set velocity");
      if (q0_.empty()) q0_.assign(nc() * desc_.num_phases, desc_.density[0]);
      Check(hydro_gpu_set_field(ctx_, HYDRO_FIELD_PARTIAL_DENSITY, HYDRO_TIME_CURR, q0_.data(),
                                q0_.size()),
            "set partial densities");
      Check(hydro_gpu_init_state(ctx_), "init_state");
    }
    return ctx_;
  }
  bool created() const { return ctx_ != nullptr; }
  std::vector<double>& u0() { return u0_; }
  std::vector<double>& q0() { return q0_; }

  // host FieldCell<Vect> <-> component-major doubles
  void Upload(int field, const geom::FieldCell<Vect>& fc) {
    std::vector<double> buf(nc() * dim);
    for (size_t c = 0; c < nc(); ++c)
      for (size_t k = 0; k < dim; ++k) buf[k * nc() + c] = fc[geom::IdxCell(c)][k];
    Check(hydro_gpu_set_field(ctx(), field, HYDRO_TIME_CURR, buf.data(), buf.size()), "set");
  }
  void Upload(int field, const geom::FieldCell<Scal>& fc) {
    Check(hydro_gpu_set_field(ctx(), field, HYDRO_TIME_CURR, fc.data(), fc.size()), "set");
  }
  void Download(int field, int layer, geom::FieldCell<Vect>& fc) {
    std::vector<double> buf(nc() * dim);
    Check(hydro_gpu_get_field(ctx(), field, layer, buf.data(), buf.size()), "get");
    fc.Reinit(mesh_);
    for (size_t c = 0; c < nc(); ++c)
      for (size_t k = 0; k < dim; ++k) fc[geom::IdxCell(c)][k] = buf[k * nc() + c];
  }
  template <class Field>
  void Download(int field, int layer, Field& f, size_t n) {
    f.resize(n);
    Check(hydro_gpu_get_field(ctx(), field, layer, f.data(), n), "get");
  }

 private:
  const Mesh& mesh_;
  hydro_desc desc_;
  hydro_ctx* ctx_ = nullptr;
  std::vector<double> u0_, q0_;
};

template <class Mesh>
class FluidSimpleGpu : public FluidSolver<Mesh> {
  using Scal = typename Mesh::Scal;
  using Vect = typename Mesh::Vect;
  static constexpr size_t dim = Mesh::dim;
  template <class T>
  using FieldCell = geom::FieldCell<T>;
  template <class T>
  using FieldFace = geom::FieldFace<T>;
  using IdxCell = geom::IdxCell;
  using IdxFace = geom::IdxFace;

 public:
  FluidSimpleGpu(const Mesh& mesh, const FieldCell<Vect>& fc_velocity_initial,
                 const geom::MapFace<std::shared_ptr<ConditionFaceFluid>>& mf_cond,
                 const geom::MapCell<std::shared_ptr<ConditionCellFluid>>& mc_cond,
                 Scal velocity_relaxation_factor, Scal pressure_relaxation_factor,
                 Scal rhie_chow_factor, FieldCell<Scal>* p_fc_density,
                 FieldCell<Scal>* p_fc_viscosity, FieldCell<Vect>* p_fc_force,
                 FieldCell<Vect>* p_fc_stforce, FieldFace<Vect>* p_ff_stforce,
                 FieldCell<Scal>* p_fc_volume_source, FieldCell<Scal>* p_fc_mass_source,
                 double time, double time_step, const LinearSolverFactory& /*velocity*/,
                 const LinearSolverFactory& /*pressure*/, double convergence_tolerance,
                 size_t num_iterations_limit, MultiTimer<std::string>* /*timer*/,
                 bool time_second_order, bool simpler, bool force_geometric_average,
                 Scal guess_extrapolation = 0., Vect meshvel = Vect(0))
      : FluidSolver<Mesh>(time, time_step, p_fc_density, p_fc_viscosity, p_fc_force,
                          p_fc_stforce, p_ff_stforce, p_fc_volume_source, p_fc_mass_source,
                          convergence_tolerance, num_iterations_limit, meshvel),
        path_(std::make_shared<GpuHotPath<Mesh>>(mesh)),
        mesh_(mesh) {
    using namespace fluid_condition;
    hydro_desc& d = path_->desc();
    d.simpler = simpler;
    // per-side kind and velocity from the face conditions (fluid.hpp:695-731):
    // walls and inlets carry their velocity, outlets are rebalanced on the
    // device (fluid.hpp:542-600); one kind and one velocity per side
    std::array<bool, 6> seen{};
    for (auto it = mf_cond.cbegin(); it != mf_cond.cend(); ++it) {
      IdxFace f = it->GetIdx();
      auto* c = it->GetValue().get();
      int kind;
      Vect v(0);
      if (auto* wall = dynamic_cast<NoSlipWall<Mesh>*>(c)) {
        kind = HYDRO_BC_WALL;
        v = wall->GetVelocity();
      } else if (auto* in = dynamic_cast<Inlet<Mesh>*>(c)) {
        kind = HYDRO_BC_INLET;
        v = in->GetVelocity();
      } else if (dynamic_cast<Outlet<Mesh>*>(c)) {
        kind = HYDRO_BC_OUTLET;
      } else {
        throw std::runtime_error("FluidSimpleGpu: unknown face condition");
      }
      size_t dir = mesh.GetDirection(f);
      auto mi = mesh.GetBlockFaces().GetMIdx(f);
      if (mi[dir] != 0 && mi[dir] != mesh.GetBlockCells().GetDimensions()[dir]) {
        // a face inside the block: the rigid box's wall at rest
        if (kind != HYDRO_BC_WALL || !(v == Vect(0)))
          throw std::runtime_error("FluidSimpleGpu: inner faces must be walls at rest");
        continue;
      }
      int side = 2 * (int)dir + (mi[dir] == 0 ? 0 : 1);
      if (seen[side] && d.bc_kind[side] != kind)
        throw std::runtime_error("FluidSimpleGpu: one condition kind per side");
      for (size_t k = 0; k < dim; ++k) {
        if (seen[side] && d.bc_velocity[side][k] != v[k])
          throw std::runtime_error("FluidSimpleGpu: condition velocity must be uniform per side");
        d.bc_velocity[side][k] = v[k];
      }
      d.bc_kind[side] = kind;
      seen[side] = true;
    }
    // excluded cells (mesh.ExcludeCells, the rigid box of hydro2d.hpp:306-423):
    // the box is the bounding box of their centres, checked to select
    // exactly them
    {
      bool any = false;
      Vect lo(0), hi(0);
      for (auto c : mesh.Cells()) {
        if (!mesh.IsExcluded(c)) continue;
        Vect x = mesh.GetCenter(c);
        for (size_t k = 0; k < dim; ++k) {
          lo[k] = any ? std::min(lo[k], x[k]) : x[k];
          hi[k] = any ? std::max(hi[k], x[k]) : x[k];
        }
        any = true;
      }
      if (any) {
        // widen by a quarter cell: the library recomputes the centres with
        // its own formula, which may differ from the mesh's in the last bit
        for (size_t k = 0; k < dim; ++k) {
          const double h = (d.hi[k] - d.lo[k]) / d.n[k];
          lo[k] -= 0.25 * h;
          hi[k] += 0.25 * h;
        }
        for (auto c : mesh.Cells()) {
          Vect x = mesh.GetCenter(c);
          bool in = true;
          for (size_t k = 0; k < dim; ++k) in = in && lo[k] <= x[k] && x[k] <= hi[k];
          if (in != mesh.IsExcluded(c))
            throw std::runtime_error("FluidSimpleGpu: excluded cells must form a box");
        }
        d.rigid_box = 1;
        for (size_t k = 0; k < dim; ++k) {
          d.rigid_box_lo[k] = lo[k];
          d.rigid_box_hi[k] = hi[k];
        }
      }
    }
    for (auto it = mc_cond.cbegin(); it != mc_cond.cend(); ++it) {
      auto* gp = dynamic_cast<GivenPressure<Mesh>*>(it->GetValue().get());
      if (!gp) throw std::runtime_error("FluidSimpleGpu: only given-pressure cells are built");
      d.pressure_fixed_cell = (int)it->GetIdx().GetRaw();
      d.pressure_fixed_value = gp->GetPressure();
    }
    d.velocity_relaxation_factor = velocity_relaxation_factor;
    d.pressure_relaxation_factor = pressure_relaxation_factor;
    d.rhie_chow_factor = rhie_chow_factor;
    d.time_second_order = time_second_order;
    d.force_geometric_average = force_geometric_average;
    d.guess_extrapolation = guess_extrapolation;
    for (size_t k = 0; k < dim; ++k) d.meshvel[k] = meshvel[k];
    d.dt = time_step;
    d.convergence_tolerance = convergence_tolerance;
    d.num_iterations_limit = (int)num_iterations_limit;
    d.advection_enable = 0;
    auto& u0 = path_->u0();
    u0.assign(mesh.GetNumCells() * dim, 0.);
    for (size_t c = 0; c < mesh.GetNumCells(); ++c)
      for (size_t k = 0; k < dim; ++k)
        u0[k * mesh.GetNumCells() + c] = fc_velocity_initial[IdxCell(c)][k];
  }

  // Tolerances of the GPU solves (the reference's factories are opaque).
  void SetLinearTolerances(double velocity_tol, int velocity_limit, double pressure_tol,
                           int pressure_limit, bool mixed_precision = false) {
    hydro_desc& d = path_->desc();
    d.velocity_tolerance = velocity_tol;
    d.velocity_iters_limit = velocity_limit;
    d.pressure_tolerance = pressure_tol;
    d.pressure_iters_limit = pressure_limit;
    d.precision = mixed_precision ? HYDRO_MIXED : HYDRO_FP64;
  }
  std::shared_ptr<GpuHotPath<Mesh>> path() { return path_; }

  void StartStep() override {
    this->ClearIterationCount();
    // mixture fields owned by the module (hydro2d.hpp:453-458)
    path_->Upload(HYDRO_FIELD_DENSITY, *this->p_fc_density_);
    path_->Upload(HYDRO_FIELD_VISCOSITY, *this->p_fc_viscosity_);
    path_->Upload(HYDRO_FIELD_FORCE, *this->p_fc_force_);
    path_->Upload(HYDRO_FIELD_SURFACE_FORCE, *this->p_fc_stforce_);
    path_->Upload(HYDRO_FIELD_VOLUME_SOURCE, *this->p_fc_volume_source_);
    path_->Upload(HYDRO_FIELD_MASS_SOURCE, *this->p_fc_mass_source_);
    GpuHotPath<Mesh>::Check(hydro_gpu_set_time_step(path_->ctx(), this->GetTimeStep(), 0.),
                            "set_time_step");
    GpuHotPath<Mesh>::Check(hydro_gpu_start_step(path_->ctx()), "start_step");
  }
  void MakeIteration() override {
    GpuHotPath<Mesh>::Check(hydro_gpu_make_iteration(path_->ctx()), "make_iteration");
    this->IncIterationCount();
  }
  void FinishStep() override {
    GpuHotPath<Mesh>::Check(hydro_gpu_finish_step(path_->ctx()), "finish_step");
    this->IncTime();
  }
  double GetConvergenceIndicator() const override {
    double v = 1.;
    if (path_->created())
      hydro_gpu_get_convergence_indicator(const_cast<GpuHotPath<Mesh>&>(*path_).ctx(), &v);
    return v;
  }
  const FieldCell<Vect>& GetVelocity() override { return GetVelocity(Layers::time_curr); }
  const FieldCell<Vect>& GetVelocity(Layers layer) override {
    auto& f = vel_.Get(layer);
    path_->Download(HYDRO_FIELD_VELOCITY, (int)layer, f);
    return f;
  }
  const FieldCell<Scal>& GetPressure() override { return GetPressure(Layers::time_curr); }
  const FieldCell<Scal>& GetPressure(Layers layer) override {
    auto& f = pres_.Get(layer);
    path_->Download(HYDRO_FIELD_PRESSURE, (int)layer, f, mesh_.GetNumCells());
    return f;
  }
  const FieldFace<Scal>& GetVolumeFlux() override { return GetVolumeFlux(Layers::time_curr); }
  const FieldFace<Scal>& GetVolumeFlux(Layers layer) override {
    auto& f = flux_.Get(layer);
    path_->Download(HYDRO_FIELD_VOLUME_FLUX, (int)layer, f, mesh_.GetNumFaces());
    return f;
  }
  double GetAutoTimeStep() override {
    double v;
    GpuHotPath<Mesh>::Check(hydro_gpu_get_auto_time_step(path_->ctx(), &v), "auto_time_step");
    return v;
  }

 private:
  std::shared_ptr<GpuHotPath<Mesh>> path_;
  const Mesh& mesh_;
  LayersData<FieldCell<Vect>> vel_;
  LayersData<FieldCell<Scal>> pres_;
  LayersData<FieldFace<Scal>> flux_;
};

template <class Mesh>
class AdvectionSolverMultiGpu
    : public AdvectionSolverMulti<Mesh, geom::FieldFace<typename Mesh::Scal>> {
  using Scal = typename Mesh::Scal;
  using Base = AdvectionSolverMulti<Mesh, geom::FieldFace<Scal>>;

 public:
  // Same arguments as AdvectionSolverMultiExplicit (advection.hpp:388-398)
  // plus the fluid adapter whose context it shares.  Boundary conditions:
  // zero derivative on walls (hydro2d.hpp:576-590); slip fluxes and mass
  // sources must be zero.
  AdvectionSolverMultiGpu(
      FluidSimpleGpu<Mesh>& fluid, const Mesh& mesh,
      const std::vector<geom::FieldCell<Scal>>& v_fc_u_initial,
      const std::vector<geom::MapFace<std::shared_ptr<ConditionFace>>>& /*v_mf_u_cond*/,
      const geom::FieldFace<Scal>* p_ff_volume_flux,
      const std::vector<const geom::FieldFace<Scal>*>& /*v_p_ff_volume_flux_slip*/,
      const std::vector<const geom::FieldCell<Scal>*>& v_p_fc_source, double time,
      double time_step, bool spatial_split, Scal sharp, std::vector<Scal> sharp_max)
      : Base(time, time_step, p_ff_volume_flux, v_p_fc_source),
        path_(fluid.path()),
        mesh_(mesh),
        cache_(v_fc_u_initial.size()) {
    hydro_desc& d = path_->desc();
    if (path_->created()) throw std::runtime_error("AdvectionSolverMultiGpu: construct first");
    if (v_fc_u_initial.size() > HYDRO_MAX_PHASES)
      throw std::runtime_error("AdvectionSolverMultiGpu: too many phases");
    d.num_phases = (int)v_fc_u_initial.size();
    for (size_t i = 0; i < sharp_max.size() && i < HYDRO_MAX_PHASES; ++i)
      d.density[i] = sharp_max[i];  // the module passes the true densities
    d.tvd_split = spatial_split;
    d.sharp = sharp;
    d.advection_enable = 1;
    d.advection_dt_factor = time_step / d.dt;
    auto& q0 = path_->q0();
    size_t nc = mesh.GetNumCells();
    q0.assign(nc * v_fc_u_initial.size(), 0.);
    for (size_t i = 0; i < v_fc_u_initial.size(); ++i)
      for (size_t c = 0; c < nc; ++c) q0[i * nc + c] = v_fc_u_initial[i][geom::IdxCell(c)];
  }
  void StartStep() override { this->ClearIterationCount(); }
  void MakeIteration() override {
    GpuHotPath<Mesh>::Check(
        hydro_gpu_set_time_step(path_->ctx(), 0., this->GetTimeStep()),
        "set_time_step");
    GpuHotPath<Mesh>::Check(hydro_gpu_advection_substep(path_->ctx()), "advection_substep");
    this->IncIterationCount();
  }
  void FinishStep() override { this->IncTime(); }
  double GetConvergenceIndicator() const override {
    return this->GetIterationCount() == 0 ? 1. : 0.;
  }
  const geom::FieldCell<Scal>& GetField(size_t i) override {
    size_t nc = mesh_.GetNumCells();
    std::vector<double> all(nc * path_->desc().num_phases);
    GpuHotPath<Mesh>::Check(hydro_gpu_get_field(path_->ctx(), HYDRO_FIELD_PARTIAL_DENSITY,
                                                HYDRO_TIME_CURR, all.data(), all.size()),
                            "get partial density");
    cache_[i].Reinit(mesh_);
    for (size_t c = 0; c < nc; ++c) cache_[i][geom::IdxCell(c)] = all[i * nc + c];
    return cache_[i];
  }

 private:
  std::shared_ptr<GpuHotPath<Mesh>> path_;
  const Mesh& mesh_;
  std::vector<geom::FieldCell<Scal>> cache_;
};

// Drop-in for HeatSolver<Mesh> (heat.hpp:18-94) with its argument list,
// plus the fluid adapter whose context and volume fluxes it shares.  The
// temperature conditions must be the ones hydro<Mesh>::InitHeatSolver
// builds (hydro2d.hpp:660-677): one fixed value on the boundary faces whose
// centre lies in a box, zero derivative on the others.  The box is
// recovered as the bounding box of the value faces' centres and checked
// against the map.  The module's conductivity (p_fc_conductivity) is
// uploaded at every StartStep; the source must be zero; the linear solve is
// Jacobi sweeps (SetLinearTolerance; the factory is opaque).
template <class Mesh>
class HeatSolverGpu : public UnsteadyIterativeSolver {
  using Scal = typename Mesh::Scal;
  using Vect = typename Mesh::Vect;
  static constexpr size_t dim = Mesh::dim;

 public:
  HeatSolverGpu(FluidSimpleGpu<Mesh>& fluid, const Mesh& mesh,
                const geom::FieldCell<Scal>& fc_temperature_initial,
                const geom::MapFace<std::shared_ptr<ConditionFace>>& mf_temperature_cond,
                Scal relaxation_factor, const geom::FieldCell<Scal>* p_fc_conductivity,
                const geom::FieldCell<Scal>* /*p_fc_source*/,
                const geom::FieldFace<Scal>* /*p_ff_vol_flux*/, double time, double time_step,
                const LinearSolverFactory& /*linear_factory*/, double convergence_tolerance,
                size_t num_iterations_limit, bool time_second_order = true)
      : UnsteadyIterativeSolver(time, time_step, convergence_tolerance, num_iterations_limit),
        path_(fluid.path()),
        mesh_(mesh),
        p_fc_conductivity_(p_fc_conductivity),
        t0_(fc_temperature_initial) {
    hd_ = hydro_heat_desc();
    hd_.relaxation_factor = relaxation_factor;
    hd_.time_second_order = time_second_order;
    hd_.solver = HYDRO_LINEAR_JACOBI;
    hd_.tolerance = 1e-12;
    hd_.iters_limit = 10000;
    hd_.dt = time_step;
    hd_.temperature_initial = fc_temperature_initial[geom::IdxCell(0)];
    bool any = false;
    Vect lo(0), hi(0);
    for (auto it = mf_temperature_cond.cbegin(); it != mf_temperature_cond.cend(); ++it) {
      auto* c = it->GetValue().get();
      if (auto* v = dynamic_cast<ConditionFaceValueFixed<Scal>*>(c)) {
        Vect x = mesh.GetCenter(it->GetIdx());
        if (any && v->GetValue() != hd_.box_temperature)
          throw std::runtime_error("HeatSolverGpu: one fixed temperature");
        hd_.box_temperature = v->GetValue();
        for (size_t k = 0; k < dim; ++k) {
          lo[k] = any ? std::min(lo[k], x[k]) : x[k];
          hi[k] = any ? std::max(hi[k], x[k]) : x[k];
        }
        any = true;
      } else if (!dynamic_cast<ConditionFaceDerivativeFixed<Scal>*>(c)) {
        throw std::runtime_error("HeatSolverGpu: value or zero-derivative conditions only");
      }
    }
    for (size_t k = 0; k < 3; ++k) {
      hd_.box_lo[k] = k < dim ? lo[k] : 0.;
      hd_.box_hi[k] = k < dim ? hi[k] : 0.;
    }
    if (!any) {  // no value face: an empty box below the domain
      for (size_t k = 0; k < 3; ++k) {
        hd_.box_lo[k] = 1.;
        hd_.box_hi[k] = -1.;
      }
    }
    for (auto it = mf_temperature_cond.cbegin(); it != mf_temperature_cond.cend(); ++it) {
      Vect x = mesh.GetCenter(it->GetIdx());
      bool in = any;
      for (size_t k = 0; k < dim; ++k) in = in && lo[k] <= x[k] && x[k] <= hi[k];
      bool value = dynamic_cast<ConditionFaceValueFixed<Scal>*>(it->GetValue().get()) != nullptr;
      if (in != value) throw std::runtime_error("HeatSolverGpu: value faces must form a box");
    }
  }
  void SetLinearTolerance(double tol, int limit) {
    hd_.tolerance = tol;
    hd_.iters_limit = limit;
  }
  void StartStep() override {
    this->ClearIterationCount();
    if (!created_) {
      GpuHotPath<Mesh>::Check(hydro_gpu_heat_create(path_->ctx(), &hd_), "heat_create");
      path_->Upload(HYDRO_FIELD_TEMPERATURE, t0_);
      GpuHotPath<Mesh>::Check(hydro_gpu_set_field(path_->ctx(), HYDRO_FIELD_TEMPERATURE,
                                                  HYDRO_TIME_PREV, t0_.data(), t0_.size()),
                              "set temperature");
      created_ = true;
    }
    path_->Upload(HYDRO_FIELD_CONDUCTIVITY, *p_fc_conductivity_);
  }
  void MakeIteration() override {
    GpuHotPath<Mesh>::Check(hydro_gpu_heat_step(path_->ctx()), "heat_step");
    this->IncIterationCount();
  }
  void FinishStep() override { this->IncTime(); }
  double GetConvergenceIndicator() const override { return 0.; }
  const geom::FieldCell<Scal>& GetTemperature() { return GetTemperature(Layers::time_curr); }
  const geom::FieldCell<Scal>& GetTemperature(Layers layer) {
    if (!created_) return t0_;
    auto& f = cache_.Get(layer);
    path_->Download(HYDRO_FIELD_TEMPERATURE, (int)layer, f, mesh_.GetNumCells());
    return f;
  }

 private:
  std::shared_ptr<GpuHotPath<Mesh>> path_;
  const Mesh& mesh_;
  const geom::FieldCell<Scal>* p_fc_conductivity_;
  geom::FieldCell<Scal> t0_;
  hydro_heat_desc hd_;
  bool created_ = false;
  LayersData<geom::FieldCell<Scal>> cache_;
};

}  // namespace solver
