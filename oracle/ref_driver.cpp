/*
 * ref_driver.cpp -- runs the reference PanNDE HostSolver through its own
 * public API (PanNDE::Model) on inputs given as plain C arrays.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
 * reference's own headers where they lie (HostData, HostSolver, Stubs,
 * PanNDE), into oracle/_ref/libpannde_ref.so.  Used to produce the golden
 * fixtures under tests/golden and to pin the C oracle (pn_oracle.c) to the
 * reference bit for bit.  Nothing here is part of the product.
 *
 * The only project-written pieces are the glue below: a single-rank
 * PanNDE::Communicator whose halo calls do nothing (one partition; the
 * reference's MPICommunicator needs MPI, which is absent), and the
 * conversion of C arrays into HexMesh / HostField / HostUnivariate /
 * HostNormalXDZ objects, as applications/include/Boss.hpp does from a .vtu.
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Communicator.hpp"
#include "HexMesh.hpp"
#include "HostArray.hpp"
#include "HostField.hpp"
#include "HostNormalXDZ.hpp"
#include "HostRSGTDUT.hpp"
#include "HostUTModel.hpp"
#include "HostUnivariate.hpp"
#include "StandardNames.hpp"

#include "../include/pannde_gb300.h"

namespace {

/* One process, one partition: every exchange is a no-op. */
class SingleRankComm : public PanNDE::Communicator {
 public:
  void Init(int &, char **&) override {}
  void Init(int &, char **&, std::shared_ptr<PanNDE::Mesh>) override {}
  int getProcessId() override { return 0; }
  int getGlobalId() override { return 0; }
  int getNumberOfProcesses() override { return 1; }
  int getNumberOfAllProcesses() override { return 1; }
  void Finalize() override {}
  void determineExchangePattern(std::shared_ptr<PanNDE::Mesh>) override {}
  void setupDataLinks(std::string, std::shared_ptr<PanNDE::Field>) override {}
  void setupDataLinks(std::shared_ptr<PanNDE::FieldBundle>) override {}
  void startHaloExchange(std::string) override {}
  void waitUntilDone(std::string) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<double>>, int) override {}
  void sendArray(double *, int, int) override {}
  std::shared_ptr<PanNDE::Array<double>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<double>>,
                                                   int) override { return nullptr; }
  void broadcastArray(std::shared_ptr<PanNDE::Array<double>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int32_t>>, int) override {}
  void sendArray(int32_t *, int, int) override {}
  std::shared_ptr<PanNDE::Array<int32_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int32_t>>,
                                                    int) override { return nullptr; }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int32_t>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int64_t>>, int) override {}
  void sendArray(int64_t *, int, int) override {}
  std::shared_ptr<PanNDE::Array<int64_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int64_t>>,
                                                    int) override { return nullptr; }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int64_t>> &, int) override {}
  void sendValue(double, int) override {}
  void recvValue(double *, int) override {}
  void broadcastValue(double *, int) override {}
  std::shared_ptr<PanNDE::Array<double>> allGatherValue(
      double, std::shared_ptr<PanNDE::ArrayFactory<double>>) override { return nullptr; }
  void sendValue(int32_t, int) override {}
  void recvValue(int32_t *, int) override {}
  void broadcastValue(int32_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int32_t>> allGatherValue(
      int32_t, std::shared_ptr<PanNDE::ArrayFactory<int32_t>>) override { return nullptr; }
  void sendValue(int64_t, int) override {}
  void recvValue(int64_t *, int) override {}
  void broadcastValue(int64_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int64_t>> allGatherValue(
      int64_t, std::shared_ptr<PanNDE::ArrayFactory<int64_t>>) override { return nullptr; }
  void waitall() override {}
  void barrier() override {}
};

thread_local std::string g_msg;

std::shared_ptr<PanNDE::Mesh> make_mesh(const pn_mesh *m) {
  HostData::HexMeshFactory mf;
  std::vector<PanNDE::Mesh::Node> nodes;
  std::vector<PanNDE::Mesh::Cell> cells;
  nodes.reserve(m->n_nodes);
  cells.reserve(m->n_cells);
  for (int32_t n = 0; n < m->n_nodes; n++) {
    double p[3] = {m->x[n], m->y[n], m->z[n]};
    nodes.push_back(mf.makeNode(p, n, m->node_owner ? m->node_owner[n] : m->partition_id));
  }
  for (int32_t c = 0; c < m->n_cells; c++) {
    int32_t box[8];
    for (int k = 0; k < 8; k++) box[k] = m->hexes[(int64_t)c * 8 + k];
    cells.push_back(mf.makeCell(box, 8, c));
  }
  return mf.makeManagedMesh(nodes.data(), nodes.size(), cells.data(), cells.size(),
                            m->partition_id);
}

std::shared_ptr<PanNDE::Field> make_field(std::shared_ptr<PanNDE::Mesh> mesh, const pn_field &f) {
  auto type = (PanNDE::Field::FieldType)f.type;
  auto field = std::make_shared<HostData::HostField>(HostData::HostField(mesh, type));
  for (int32_t k = 0; k < field->size(); k++) field->data()[k] = f.data[k];
  return field;
}

std::shared_ptr<PanNDE::MultiVariate> make_source(const pn_window_source &s) {
  auto times = HostData::HostArray<double>::makeShared();
  auto vals = HostData::HostArray<double>::makeShared();
  times->resize(s.signal.n);
  vals->resize(s.signal.n);
  for (int32_t k = 0; k < s.signal.n; k++) {
    times->at(k) = s.signal.t[k];
    vals->at(k) = s.signal.v[k];
  }
  auto sig = HostData::HostUnivariate::makeShared(times, vals);
  double c[3] = {s.center[0], s.center[1], s.center[2]};
  return Stubs::HostNormalXDZ::makeShared(c, s.radius, s.ds, sig);
}

}  // namespace

extern "C" {

const char *pnref_last_error(void) { return g_msg.c_str(); }

/* model_kind 0: HostSolver::HostRSGTDUT (force sources only);
   model_kind 1: HostSolver::HostUTModel (applyTransducer + applyMomentExcitation).
   Same arguments as pn_oracle_run. */
int pnref_run(int32_t model_kind, const pn_mesh *m, const pn_material *mat, double dt,
              const double *const *V0, const double *const *S0, const pn_window_source *src,
              int32_t nsrc, int32_t nsteps, const int32_t *sensors, int32_t nsens, double *traces,
              double *const *Vout, double *const *Sout, double *time_out) {
  g_msg.clear();
  try {
    auto mesh = make_mesh(m);
    PanNDE::ElasticMaterialNames pn;
    PanNDE::ElasticStateNames sn;
    auto domain = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
    domain->emplaceField(pn.density, make_field(mesh, mat->density));
    int idx = 0;
    for (int i = 0; i < 6; i++)
      for (int j = i; j < 6; j++) domain->emplaceField(pn.CIJ[i][j], make_field(mesh, mat->cij[idx++]));
    auto sol = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
    for (int k = 0; k < 3; k++) {
      sol->emplaceField(sn.V[k], PanNDE::Field::NODE);
      auto f = sol->field(sn.V[k]);
      for (int32_t n = 0; n < m->n_nodes; n++) f->at(n) = (V0 && V0[k]) ? V0[k][n] : 0.;
    }
    for (int k = 0; k < 6; k++) {
      sol->emplaceField(sn.SI[k], PanNDE::Field::CELL);
      auto f = sol->field(sn.SI[k]);
      for (int32_t c = 0; c < m->n_cells; c++) f->at(c) = (S0 && S0[k]) ? S0[k][c] : 0.;
    }
    std::shared_ptr<PanNDE::Communicator> comm = std::make_shared<SingleRankComm>();

    int ngf = 0, ngm = 0;
    for (int32_t i = 0; i < nsrc; i++) {
      if (src[i].kind == PN_SOURCE_FORCE) ngf = std::max(ngf, src[i].group + 1);
      else ngm = std::max(ngm, src[i].group + 1);
    }
    std::vector<std::shared_ptr<PanNDE::MultiVariate>> xds(3 * ngf, nullptr);
    std::vector<std::shared_ptr<PanNDE::MultiVariate>> moms(6 * ngm, nullptr);
    for (int32_t i = 0; i < nsrc; i++) {
      if (src[i].kind == PN_SOURCE_FORCE) xds[3 * src[i].group + src[i].component] = make_source(src[i]);
      else moms[6 * src[i].group + src[i].component] = make_source(src[i]);
    }

    std::shared_ptr<PanNDE::Model> model;
    if (model_kind == 0) {
      if (ngm > 0) throw std::invalid_argument("HostRSGTDUT has no moment sources");
      auto arr = (std::shared_ptr<PanNDE::MultiVariate>(*)[3])xds.data();
      model = std::make_shared<HostSolver::HostRSGTDUT>(
          HostSolver::HostRSGTDUT(dt, domain, sol, arr, ngf, comm));
    } else {
      auto ut = std::make_shared<HostSolver::HostUTModel>(
          HostSolver::HostUTModel(dt, domain, sol, comm));
      for (int g = 0; g < ngf; g++) ut->applyTransducer(&xds[3 * g]);
      for (int g = 0; g < ngm; g++) ut->applyMomentExcitation(&moms[6 * g]);
      model = ut;
    }
    double t = 0.;
    for (int32_t step = 0; step < nsteps; step++) {
      t = model->solve(1);
      auto st = model->getStates();
      for (int32_t i = 0; i < nsens; i++)
        for (int d = 0; d < 3; d++)
          traces[((int64_t)step * nsens + i) * 3 + d] = st->field(sn.V[d])->at(sensors[i]);
    }
    auto st = model->getStates();
    for (int k = 0; k < 3; k++) std::memcpy(Vout[k], st->field(sn.V[k])->data(), sizeof(double) * m->n_nodes);
    for (int k = 0; k < 6; k++) std::memcpy(Sout[k], st->field(sn.SI[k])->data(), sizeof(double) * m->n_cells);
    if (time_out) *time_out = t;
    return PN_OK;
  } catch (const std::out_of_range &e) {
    g_msg = e.what();
    return PN_ERR_RANGE;
  } catch (const std::invalid_argument &e) {
    g_msg = e.what();
    return PN_ERR_INVALID;
  } catch (const std::logic_error &e) {
    g_msg = e.what();
    return PN_ERR_SPACING;
  } catch (const std::runtime_error &e) {
    g_msg = e.what();
    return PN_ERR_RUNTIME;
  } catch (const std::exception &e) {
    g_msg = e.what();
    return PN_ERR_INVALID;
  }
}

/* RightHex operators on a mesh (RightHexTests known answers). */
int pnref_dd(const pn_mesh *m, const double *field, int32_t on_nodes, int32_t idx, int32_t axis,
             double *out, double *spacing_out) {
  g_msg.clear();
  try {
    auto mesh = make_mesh(m);
    HostSolver::RightHex rh(mesh);
    HostData::HostFieldFactory ff;
    auto f = ff.makeManagedField(mesh, on_nodes ? PanNDE::Field::NODE : PanNDE::Field::CELL);
    for (int32_t k = 0; k < f->size(); k++) f->at(k) = field[k];
    if (on_nodes) {
      *out = axis == 0 ? rh.DDx_cc(idx, f) : axis == 1 ? rh.DDy_cc(idx, f) : rh.DDz_cc(idx, f);
    } else {
      *out = axis == 0 ? rh.DDx_nc(idx, f) : axis == 1 ? rh.DDy_nc(idx, f) : rh.DDz_nc(idx, f);
      if (spacing_out)
        *spacing_out = axis == 0 ? rh.getNodeDx(idx) : axis == 1 ? rh.getNodeDy(idx) : rh.getNodeDz(idx);
    }
    return PN_OK;
  } catch (const std::logic_error &e) {
    g_msg = e.what();
    return PN_ERR_SPACING;
  } catch (const std::exception &e) {
    g_msg = e.what();
    return PN_ERR_INVALID;
  }
}

}  // extern "C"
