// adapter_check.cpp -- builds the reference's own objects (HexMesh via
// PlateBuilder, HostField bundles, HostUnivariate + HostNormalXDZ transducer,
// as TransducerModel / Boss.hpp do) and runs DeviceSolver::DeviceRSGTDUT and
// DeviceUTModel beside HostSolver::HostRSGTDUT / HostUTModel.
//
// Test program (tests/test_adapter_cpu.py compiles it against the reference
// headers).  Output lines:
//   no-device <what>            device creation failed with std::runtime_error
//   max-rel <form> <value>      largest relative difference over all fields
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Communicator.hpp"
#include "DeviceSolver.hpp"
#include "HexMesh.hpp"
#include "HostArray.hpp"
#include "HostField.hpp"
#include "HostNormalXDZ.hpp"
#include "HostRSGTDUT.hpp"
#include "HostUTModel.hpp"
#include "HostUnivariate.hpp"
#include "PlateBuilder.hpp"
#include "StandardNames.hpp"

namespace {

class OneRank : public PanNDE::Communicator {
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
  std::shared_ptr<PanNDE::Array<double>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<double>>, int) override {
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<double>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int32_t>>, int) override {}
  void sendArray(int32_t *, int, int) override {}
  std::shared_ptr<PanNDE::Array<int32_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int32_t>>, int) override {
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int32_t>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int64_t>>, int) override {}
  void sendArray(int64_t *, int, int) override {}
  std::shared_ptr<PanNDE::Array<int64_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int64_t>>, int) override {
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int64_t>> &, int) override {}
  void sendValue(double, int) override {}
  void recvValue(double *, int) override {}
  void broadcastValue(double *, int) override {}
  std::shared_ptr<PanNDE::Array<double>> allGatherValue(double, std::shared_ptr<PanNDE::ArrayFactory<double>>) override {
    return nullptr;
  }
  void sendValue(int32_t, int) override {}
  void recvValue(int32_t *, int) override {}
  void broadcastValue(int32_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int32_t>> allGatherValue(int32_t, std::shared_ptr<PanNDE::ArrayFactory<int32_t>>) override {
    return nullptr;
  }
  void sendValue(int64_t, int) override {}
  void recvValue(int64_t *, int) override {}
  void broadcastValue(int64_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int64_t>> allGatherValue(int64_t, std::shared_ptr<PanNDE::ArrayFactory<int64_t>>) override {
    return nullptr;
  }
  void waitall() override {}
  void barrier() override {}
};

PanNDE::ElasticMaterialNames pnames;
PanNDE::ElasticStateNames snames;

std::shared_ptr<PanNDE::FieldBundle> solution_bundle(std::shared_ptr<PanNDE::Mesh> mesh) {
  auto b = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
  for (int k = 0; k < 3; k++) b->emplaceField(snames.V[k], PanNDE::Field::NODE);
  for (int k = 0; k < 6; k++) b->emplaceField(snames.SI[k], PanNDE::Field::CELL);
  return b;
}

double max_rel(std::shared_ptr<PanNDE::FieldBundle> a, std::shared_ptr<PanNDE::FieldBundle> b) {
  double worst = 0.;
  const std::string names[9] = {"Vx", "Vy", "Vz", "Sxx", "Syy", "Szz", "Syz", "Sxz", "Sxy"};
  for (auto &n : names) {
    auto fa = a->field(n), fb = b->field(n);
    double num = 0., den = 0.;
    for (int32_t k = 0; k < fa->size(); k++) {
      const double d = fa->at(k) - fb->at(k);
      num += d * d;
      den += fb->at(k) * fb->at(k);
    }
    if (den > 0) worst = std::max(worst, std::sqrt(num / den));
  }
  return worst;
}

}  // namespace

int main() {
  auto mf = std::make_shared<HostData::HexMeshFactory>(HostData::HexMeshFactory());
  Stubs::PlateBuilder pb;
  auto mesh = pb.makeMesh(mf, 1.6e-3, 1.6e-3, 0.4e-3, 16, 4, false);
  auto domain = std::make_shared<HostData::HostFieldBundle>(HostData::HostFieldBundle(mesh));
  const double lam = 51.08e9, mu = 26.32e9, rho = 2700.;
  domain->emplaceField(pnames.density, PanNDE::Field::CELL);
  for (int32_t c = 0; c < mesh->cellCount(); c++) domain->field(pnames.density)->at(c) = rho;
  for (int i = 0; i < 6; i++)
    for (int j = i; j < 6; j++) {
      domain->emplaceField(pnames.CIJ[i][j], PanNDE::Field::CELL);
      double v = 0.;
      if (i < 3 && j < 3) v = (i == j) ? lam + 2 * mu : lam;
      else if (i == j) v = mu;
      for (int32_t c = 0; c < mesh->cellCount(); c++) domain->field(pnames.CIJ[i][j])->at(c) = v;
    }
  const double dt = 0.5 * 1e-4 / (std::sqrt((lam + 2 * mu) / rho) * std::sqrt(3.));
  auto times = HostData::HostArray<double>::makeShared();
  auto vals = HostData::HostArray<double>::makeShared();
  times->resize(200);
  vals->resize(200);
  for (int k = 0; k < 200; k++) {
    times->at(k) = k * dt;
    vals->at(k) = std::sin(2 * M_PI * 2e6 * k * dt) * std::sin(M_PI * k / 199.);
  }
  auto sig = HostData::HostUnivariate::makeShared(times, vals);
  double center[3] = {0.8e-3, 0.8e-3, 0.4e-3};
  std::shared_ptr<PanNDE::MultiVariate> xd = Stubs::HostNormalXDZ::makeShared(center, 0.45e-3, 1e-4, sig);
  std::shared_ptr<PanNDE::MultiVariate> xds[1][3] = {{nullptr, nullptr, xd}};
  std::shared_ptr<PanNDE::Communicator> comm = std::make_shared<OneRank>();
  double wc[3] = {0.5e-3, 0.6e-3, 0.3e-3};
  std::shared_ptr<PanNDE::MultiVariate> mom = Stubs::HostNormalXDZ::makeShared(wc, 0.3e-3, 1e-4, sig);
  std::shared_ptr<PanNDE::MultiVariate> mt[6] = {mom, mom, mom, nullptr, nullptr, nullptr};

  const int32_t forms[3] = {PN_PREC_F64_EXACT, PN_PREC_F64, PN_PREC_DF64};
  const char *names[3] = {"f64_exact", "f64", "df64"};
  for (int f = 0; f < 3; f++) {
    auto sh = solution_bundle(mesh), sd = solution_bundle(mesh);
    auto uh = solution_bundle(mesh), ud = solution_bundle(mesh);
    HostSolver::HostRSGTDUT host(dt, domain, sh, xds, 1, comm);
    HostSolver::HostUTModel uhost(dt, domain, uh, comm);
    uhost.applyTransducer(xds[0]);
    uhost.applyMomentExcitation(mt);
    try {
      auto dev = DeviceSolver::DeviceRSGTDUT::makeShared(dt, domain, sd, xds, 1, comm, forms[f]);
      DeviceSolver::DeviceUTModel udev(dt, domain, ud, comm, forms[f]);
      udev.applyTransducer(xds[0]);
      udev.applyMomentExcitation(mt);
      double th = 0., td = 0.;
      for (int k = 0; k < 40; k++) {
        th = host.solve();
        td = dev->solve();
        uhost.solve();
        udev.solve(1);
      }
      if (th != td) {
        std::printf("time-mismatch %.17g %.17g\n", th, td);
        return 1;
      }
      std::printf("max-rel %s %.3e\n", names[f], max_rel(dev->getStates(), host.getStates()));
      std::printf("max-rel-ut %s %.3e\n", names[f], max_rel(udev.getStates(), uhost.getStates()));
    } catch (const std::runtime_error &e) {
      std::printf("no-device %s\n", e.what());
      return 0;
    }
  }
  return 0;
}
