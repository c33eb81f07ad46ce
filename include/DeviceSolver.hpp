/*
 * DeviceSolver.hpp -- PanNDE::Model implementations that run the RSG
 * leapfrog on a GB300 through the C ABI of pannde_gb300.h.
 *
 * Drop-in for the reference solver classes:
 *   DeviceSolver::DeviceRSGTDUT  <->  HostSolver::HostRSGTDUT
 *        (modules/HostSolver/include/HostRSGTDUT.hpp:87-520)
 *   DeviceSolver::DeviceUTModel  <->  HostSolver::HostUTModel
 *        (modules/HostSolver/include/HostUTModel.hpp:84-528)
 * with the same constructors, makeShared, solve(nsteps), getStates(),
 * applyTransducer and both applyMomentExcitation overloads.  The header needs
 * the PanNDE interface headers (modules/PanNDE/include) on the include path
 * and links against libpannde_gb300.so.
 *
 * Semantics kept from the reference:
 * - the model aliases the caller's initial_condition bundle as its solution
 *   (HostRSGTDUT.hpp:235-239): getStates() downloads the device state into
 *   that bundle's fields and returns the bundle;
 * - time advances by dt per step in FP64 on the host, and every source is
 *   evaluated at the pre-step time through the caller's own
 *   MultiVariate::evalAt (HostRSGTDUT.hpp:387-402, HostUTModel.hpp:296-311);
 * - errors raise the reference's exception types: std::logic_error("DX" /
 *   "DY" / "DZ") for a degenerate spacing (RightHex.hpp:305-307),
 *   std::out_of_range for a bad node id, std::runtime_error otherwise.
 *
 * Sources: a source's window is its MultiVariate::checkAt at every cell
 * centre (forces) or node (moments), and its signal at a step is its
 * evalAt at one in-window point.  This equals the reference for every
 * source of the form evalAt(p,t) = checkAt(p) * signal(t), which is how
 * Stubs::HostNormalXDZ (HostNormalXDZ.hpp:117-145), the source the
 * reference's runners build (applications/include/Boss.hpp:502-627), is
 * defined.
 *
 * Differences: solve() only enqueues device work; the host bundle is brought
 * up to date by getStates().  Host edits of the solution bundle reach the
 * device through pushStates().  One partition: a communicator, when given, is
 * only told about the solution bundle (setupDataLinks, as the reference does);
 * no halo exchange runs between device steps.
 */
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Communicator.hpp"
#include "Field.hpp"
#include "Mesh.hpp"
#include "Model.hpp"
#include "MultiVariate.hpp"
#include "StandardNames.hpp"
#include "pannde_gb300.h"

/* Precision of models built without an explicit precision argument -- the
   runners name HostSolver::HostRSGTDUT / HostUTModel and never pass one.
   Define PN_DEFAULT_PRECISION (e.g. -DPN_DEFAULT_PRECISION=PN_PREC_F64_EXACT
   for results bit-identical to HostSolver) to choose another form. */
#ifndef PN_DEFAULT_PRECISION
#define PN_DEFAULT_PRECISION PN_PREC_F64
#endif

namespace DeviceSolver {

/* Rethrow a C-ABI status as the exception type the reference raises. */
inline void check(int code) {
  if (code == PN_OK) return;
  const std::string msg = pn_last_error();
  switch (code) {
    case PN_ERR_SPACING: throw std::logic_error(msg);
    case PN_ERR_RANGE: throw std::out_of_range(msg);
    case PN_ERR_INVALID: throw std::invalid_argument(msg);
    default: throw std::runtime_error(msg);
  }
}

class DeviceModel : public PanNDE::Model {
 public:
  // PanNDE::Model declares no virtual destructor; shared_ptrs made by
  // makeShared keep the concrete deleter
  virtual ~DeviceModel() {
    if (handle_) pn_solver_destroy(handle_);
  }
  DeviceModel(const DeviceModel &) = delete;
  DeviceModel &operator=(const DeviceModel &) = delete;
  DeviceModel(DeviceModel &&o) noexcept { *this = std::move(o); }
  DeviceModel &operator=(DeviceModel &&o) noexcept {
    std::swap(handle_, o.handle_);
    domain_ = o.domain_;
    solution_ = o.solution_;
    mesh_ = o.mesh_;
    comm_ = o.comm_;
    dt_ = o.dt_;
    time_ = o.time_;
    sources_ = std::move(o.sources_);
    stale_ = o.stale_;
    force_groups_ = o.force_groups_;
    moment_groups_ = o.moment_groups_;
    return *this;
  }

  /* Model::solve: nsteps leapfrog steps; returns the new time. */
  double solve(int nsteps = 1) override {
    if (nsteps <= 0) return time_;
    const size_t ns = sources_.size();
    std::vector<double> values((size_t)nsteps * (ns ? ns : 1), 0.0);
    double t = time_;
    for (int k = 0; k < nsteps; k++) {
      for (size_t i = 0; i < ns; i++) {
        Source &s = sources_[i];
        if (!s.has_probe) continue;  // empty window: the source adds nothing
        double args[4] = {s.probe[0], s.probe[1], s.probe[2], t};
        values[(size_t)k * ns + i] = s.mv->evalAt(args);
      }
      t += dt_;
    }
    check(pn_solver_solve_signals(handle_, nsteps, ns ? values.data() : nullptr, &time_));
    stale_ = true;
    return time_;
  }

  /* Model::getStates: the solution bundle, brought up to date from the device. */
  std::shared_ptr<PanNDE::FieldBundle> getStates() override {
    if (stale_) {
      double *V[3], *S[6];
      for (int k = 0; k < 3; k++) V[k] = solution_->field(names_.V[k])->data();
      for (int k = 0; k < 6; k++) S[k] = solution_->field(names_.SI[k])->data();
      check(pn_solver_get_state(handle_, V, S));
      stale_ = false;
    }
    return solution_;
  }

  /* Upload host edits of the solution bundle (no counterpart: the reference
     solves on the host bundle itself). */
  void pushStates() {
    const double *V[3], *S[6];
    for (int k = 0; k < 3; k++) V[k] = solution_->field(names_.V[k])->data();
    for (int k = 0; k < 6; k++) S[k] = solution_->field(names_.SI[k])->data();
    check(pn_solver_set_state(handle_, V, S));
    stale_ = false;
  }

  /* The C-ABI handle, for device-side access (pn_solver_device_state, ...). */
  pn_solver *handle() const { return handle_; }

 protected:
  DeviceModel(double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
              std::shared_ptr<PanNDE::FieldBundle> initial_condition,
              std::shared_ptr<PanNDE::Communicator> comm, int32_t precision) {
    dt_ = dt;
    domain_ = domain;
    mesh_ = domain->mesh();
    solution_ = initial_condition;
    comm_ = comm;
    if (comm_) comm_->setupDataLinks(solution_);
    createSolver(precision);
    pushStates();
  }

  /* Adds source slot (kind, group, component) backed by a MultiVariate. */
  void addSource(int32_t kind, int32_t group, int32_t component,
                 std::shared_ptr<PanNDE::MultiVariate> mv) {
    if (nullptr == mv) return;  // a null slot adds 0 (HostRSGTDUT.hpp:398)
    const bool force = kind == PN_SOURCE_FORCE;
    const int32_t n = force ? mesh_->cellCount() : mesh_->nodeCount();
    std::vector<uint8_t> inside((size_t)n, 0);
    Source s;
    s.mv = mv;
    s.has_probe = false;
    for (int32_t e = 0; e < n; e++) {
      double p[4] = {0., 0., 0., 0.};
      if (force) cellCenter(e, p);
      else mesh_->nodeCoordinate(e, p);
      inside[e] = mv->checkAt(p) ? 1 : 0;
      if (inside[e] && !s.has_probe) {
        s.probe = {p[0], p[1], p[2]};
        s.has_probe = true;
      }
    }
    pn_window_mask m;
    m.kind = kind;
    m.group = group;
    m.component = component;
    m.inside = inside.data();
    check(pn_solver_add_window_masks(handle_, &m, 1));
    sources_.push_back(s);
  }

  int32_t nextGroup(int32_t kind) {
    int32_t &g = kind == PN_SOURCE_FORCE ? force_groups_ : moment_groups_;
    return g++;
  }

 private:
  struct Source {
    std::shared_ptr<PanNDE::MultiVariate> mv;
    std::array<double, 3> probe;
    bool has_probe;
  };

  // HostRSGTDUT::cellcenter (HostRSGTDUT.hpp:419-428)
  void cellCenter(int32_t c, double cc[3]) {
    int32_t box[8];
    double pt[3];
    cc[0] = cc[1] = cc[2] = 0.;
    mesh_->cell(c, box);
    for (int kb = 0; kb < 8; kb++) {
      mesh_->nodeCoordinate(box[kb], pt);
      for (int kd = 0; kd < 3; kd++) cc[kd] += 0.125 * pt[kd];
    }
  }

  void createSolver(int32_t precision) {
    const int32_t nn = mesh_->nodeCount(), nc = mesh_->cellCount();
    std::vector<double> x(nn), y(nn), z(nn);
    std::vector<int32_t> hexes((size_t)nc * 8), owner(nn);
    for (int32_t k = 0; k < nn; k++) {
      double p[3];
      mesh_->nodeCoordinate(k, p);
      x[k] = p[0];
      y[k] = p[1];
      z[k] = p[2];
      owner[k] = mesh_->nodeHomePartition(k);
    }
    for (int32_t c = 0; c < nc; c++) mesh_->cell(c, &hexes[(size_t)c * 8]);
    pn_mesh m;
    m.n_nodes = nn;
    m.n_cells = nc;
    m.x = x.data();
    m.y = y.data();
    m.z = z.data();
    m.hexes = hexes.data();
    m.node_owner = owner.data();
    m.partition_id = mesh_->partitionId();
    pn_material mat;
    mat.density = fieldOf(names_p_.density);
    int idx = 0;
    for (int i = 0; i < 6; i++)
      for (int j = i; j < 6; j++) mat.cij[idx++] = fieldOf(names_p_.CIJ[i][j]);
    check(pn_solver_create(&m, &mat, dt_, precision, &handle_));
  }

  pn_field fieldOf(const std::string &name) {
    auto f = domain_->field(name);
    pn_field r;
    r.type = (int32_t)f->type();
    r.data = f->data();
    return r;
  }

  pn_solver *handle_ = nullptr;
  std::shared_ptr<PanNDE::FieldBundle> domain_, solution_;
  std::shared_ptr<PanNDE::Mesh> mesh_;
  std::shared_ptr<PanNDE::Communicator> comm_;
  double dt_ = 0., time_ = 0.;
  std::vector<Source> sources_;
  bool stale_ = false;
  int32_t force_groups_ = 0, moment_groups_ = 0;
  PanNDE::ElasticStateNames names_;
  PanNDE::ElasticMaterialNames names_p_;
};

/* HostSolver::HostRSGTDUT on the device (transducer forces in the velocity
   update). */
class DeviceRSGTDUT : public DeviceModel {
 public:
  static std::shared_ptr<DeviceRSGTDUT> makeShared(
      double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
      std::shared_ptr<PanNDE::FieldBundle> initial_condition,
      std::shared_ptr<PanNDE::MultiVariate> transducers[][3], int Nxducers = 0,
      std::shared_ptr<PanNDE::Communicator> comm = nullptr, int32_t precision = PN_DEFAULT_PRECISION) {
    return std::make_shared<DeviceRSGTDUT>(dt, domain, initial_condition, transducers, Nxducers, comm,
                                           precision);
  }

  DeviceRSGTDUT(double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
                std::shared_ptr<PanNDE::FieldBundle> initial_condition,
                std::shared_ptr<PanNDE::MultiVariate> transducer[3],
                std::shared_ptr<PanNDE::Communicator> comm = nullptr,
                int32_t precision = PN_DEFAULT_PRECISION)
      : DeviceModel(dt, domain, initial_condition, comm, precision) {
    addTransducer(transducer);
  }

  DeviceRSGTDUT(double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
                std::shared_ptr<PanNDE::FieldBundle> initial_condition,
                std::shared_ptr<PanNDE::MultiVariate> transducers[][3], int Nxducers = 0,
                std::shared_ptr<PanNDE::Communicator> comm = nullptr,
                int32_t precision = PN_DEFAULT_PRECISION)
      : DeviceModel(dt, domain, initial_condition, comm, precision) {
    for (int k = 0; k < Nxducers; k++) addTransducer(transducers[k]);
  }

 private:
  void addTransducer(std::shared_ptr<PanNDE::MultiVariate> xd[3]) {
    const int32_t g = nextGroup(PN_SOURCE_FORCE);
    for (int d = 0; d < 3; d++) addSource(PN_SOURCE_FORCE, g, d, xd[d]);
  }
};

/* HostSolver::HostUTModel on the device (transducer forces and moment-tensor
   excitations). */
class DeviceUTModel : public DeviceModel {
 public:
  static std::shared_ptr<DeviceUTModel> makeShared(
      double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
      std::shared_ptr<PanNDE::FieldBundle> initial_condition,
      std::shared_ptr<PanNDE::Communicator> comm = nullptr, int32_t precision = PN_DEFAULT_PRECISION) {
    return std::make_shared<DeviceUTModel>(dt, domain, initial_condition, comm, precision);
  }

  DeviceUTModel(double dt, std::shared_ptr<PanNDE::FieldBundle> domain,
                std::shared_ptr<PanNDE::FieldBundle> initial_condition,
                std::shared_ptr<PanNDE::Communicator> comm = nullptr,
                int32_t precision = PN_DEFAULT_PRECISION)
      : DeviceModel(dt, domain, initial_condition, comm, precision) {}

  /* HostUTModel::applyTransducer (HostUTModel.hpp:138-141) */
  void applyTransducer(std::shared_ptr<PanNDE::MultiVariate> xducer[3]) {
    const int32_t g = nextGroup(PN_SOURCE_FORCE);
    for (int d = 0; d < 3; d++) addSource(PN_SOURCE_FORCE, g, d, xducer[d]);
  }

  /* HostUTModel::applyMomentExcitation, Voigt order xx,yy,zz,yz,xz,xy
     (HostUTModel.hpp:152-156) */
  void applyMomentExcitation(std::shared_ptr<PanNDE::MultiVariate> moment_tensor[6]) {
    const int32_t g = nextGroup(PN_SOURCE_MOMENT);
    for (int k = 0; k < 6; k++) addSource(PN_SOURCE_MOMENT, g, k, moment_tensor[k]);
  }

  /* HostUTModel::applyMomentExcitation from a 3x3 tensor (HostUTModel.hpp:165-170) */
  void applyMomentExcitation(std::shared_ptr<PanNDE::MultiVariate> moment_tensor[3][3]) {
    std::shared_ptr<PanNDE::MultiVariate> v[6] = {moment_tensor[0][0], moment_tensor[1][1],
                                                  moment_tensor[2][2], moment_tensor[1][2],
                                                  moment_tensor[0][2], moment_tensor[0][1]};
    applyMomentExcitation(v);
  }
};

}  // namespace DeviceSolver
