// standin_check.cpp -- the reference runners' model-building statements,
// unchanged, compiled with include/standin ahead of the HostSolver headers:
//   TransducerModel.cpp:99-105   make_shared<HostSolver::HostRSGTDUT>(HostRSGTDUT(dt,domain,
//                                solution,xds,xducers.size()/3,comm))
//   WaterColumnModel.cpp:127-135 make_shared<HostSolver::HostUTModel>(HostUTModel(dt,domain,
//                                solution,comm)); applyMomentExcitation(moment_excitation.at(k).data())
//   TransducerModel.cpp:66-73    while(time<write_times[k]) time=model->solve();
// and the write-time read of getStates() (TransducerModel.cpp:143-149).
// Prints "no-device <what>" when device creation fails, else "ran <steps> <Vz>".
#include <array>
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <vector>

#include "Communicator.hpp"
#include "HexMesh.hpp"
#include "HostArray.hpp"
#include "HostField.hpp"
#include "HostNormalXDZ.hpp"
#include "HostRSGTDUT.hpp"  // resolves to include/standin/HostRSGTDUT.hpp
#include "HostUTModel.hpp"  // resolves to include/standin/HostUTModel.hpp
#include "HostUnivariate.hpp"
#include "PlateBuilder.hpp"
#include "StandardNames.hpp"

static_assert(std::is_same<HostSolver::HostRSGTDUT, DeviceSolver::DeviceRSGTDUT>::value,
              "stand-in header not picked up");

int main() {
  auto mf = std::make_shared<HostData::HexMeshFactory>(HostData::HexMeshFactory());
  Stubs::PlateBuilder pb;
  auto mesh = pb.makeMesh(mf, 1.2e-3, 1.2e-3, 0.3e-3, 12, 3, false);
  PanNDE::ElasticMaterialNames pn;
  PanNDE::ElasticStateNames sn;
  auto domain = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
  domain->emplaceField(pn.density, PanNDE::Field::CONSTANT);
  domain->field(pn.density)->at(0) = 2700.;
  for (int i = 0; i < 6; i++)
    for (int j = i; j < 6; j++) {
      domain->emplaceField(pn.CIJ[i][j], PanNDE::Field::CONSTANT);
      domain->field(pn.CIJ[i][j])->at(0) = (i < 3 && j < 3) ? (i == j ? 104e9 : 51e9) : (i == j ? 26e9 : 0.);
    }
  auto solution = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
  for (int k = 0; k < 3; k++) solution->emplaceField(sn.V[k], PanNDE::Field::NODE);
  for (int k = 0; k < 6; k++) solution->emplaceField(sn.SI[k], PanNDE::Field::CELL);
  auto wc = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
  for (int k = 0; k < 3; k++) wc->emplaceField(sn.V[k], PanNDE::Field::NODE);
  for (int k = 0; k < 6; k++) wc->emplaceField(sn.SI[k], PanNDE::Field::CELL);

  const double dt = 8e-9;
  auto t = HostData::HostArray<double>::makeShared(), v = HostData::HostArray<double>::makeShared();
  t->resize(50);
  v->resize(50);
  for (int k = 0; k < 50; k++) {
    t->at(k) = k * dt;
    v->at(k) = std::sin(0.3 * k);
  }
  double c[3] = {0.6e-3, 0.6e-3, 0.3e-3};
  auto sig = HostData::HostUnivariate::makeShared(t, v);
  std::vector<std::shared_ptr<PanNDE::MultiVariate>> xducers = {
      nullptr, nullptr, Stubs::HostNormalXDZ::makeShared(c, 0.35e-3, 1e-4, sig)};
  std::vector<std::array<std::shared_ptr<PanNDE::MultiVariate>, 6>> moment_excitation;
  moment_excitation.push_back({xducers[2], xducers[2], xducers[2], nullptr, nullptr, nullptr});
  std::shared_ptr<PanNDE::Communicator> comm = nullptr;
  std::shared_ptr<PanNDE::Model> model;
  try {
    auto xds = (std::shared_ptr<PanNDE::MultiVariate>(*)[3])xducers.data();
    model = std::make_shared<HostSolver::HostRSGTDUT>(
        HostSolver::HostRSGTDUT(dt, domain, solution, xds, xducers.size() / 3, comm));
    auto utmodel = std::make_shared<HostSolver::HostUTModel>(HostSolver::HostUTModel(dt, domain, wc, comm));
    for (size_t k = 0; k < moment_excitation.size(); k++)
      utmodel->applyMomentExcitation(moment_excitation.at(k).data());
    double time = 0;
    const double write_time = 30 * dt;
    int steps = 0;
    while (time < write_time) {
      time = model->solve();
      utmodel->solve();
      steps++;
    }
    int expected = 0;  // the same FP64 accumulation as the reference's time += dt
    for (double tt = 0; tt < write_time; tt += dt) expected++;
    const double vz = model->getStates()->field(sn.V[2])->at(mesh->nodeCount() / 2);
    const double sxx = utmodel->getStates()->field(sn.SI[0])->at(mesh->cellCount() / 2);
    std::printf("ran %d %d %.6e %.6e\n", steps, expected, vz, sxx);
  } catch (const std::runtime_error &e) {
    std::printf("no-device %s\n", e.what());
  }
  return 0;
}
