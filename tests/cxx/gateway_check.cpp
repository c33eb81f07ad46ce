// The stand-in VTKIO::VTKGateway against the reference's HostData factories:
// open a job, read the mesh, a CELL and a NODE field, a value and an array,
// then write the bundle back as a solution (<base>_<index>.vtu) and a table
// (<base>_<index>.vtt).  Prints what it read for the Python side to check.
#include <cstdio>
#include <string>

#include "HexMesh.hpp"
#include "HostArray.hpp"
#include "HostField.hpp"
#include "VTKGateway.hpp"

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  auto meshes = std::make_shared<HostData::HexMeshFactory>();
  auto fields = std::make_shared<HostData::HostFieldFactory>();
  auto arrays = std::make_shared<HostData::HostArrayFactory<double>>();
  auto gw = VTKIO::VTKGateway::makeShared(nullptr);
  gw->open(argv[1]);
  auto mesh = gw->getMesh(meshes);
  auto rho = gw->getField("density", fields);
  auto vx = gw->getField("Vx", fields);
  const double dt = gw->getValue("dt");
  auto wt = gw->getArray("write_times", arrays);
  double rsum = 0, vsum = 0;
  for (int k = 0; k < rho->size(); k++) rsum += rho->at(k);
  for (int k = 0; k < vx->size(); k++) vsum += vx->at(k);
  std::printf("%d %d %d %d %.17g %.17g %.17g %lld\n", mesh->nodeCount(), mesh->cellCount(), (int)rho->type(),
              (int)vx->type(), rsum, vsum, dt, (long long)wt->size());
  try {
    gw->getValue("no such key");
    std::printf("missing key accepted\n");
    return 1;
  } catch (const std::runtime_error &) {
  }
  auto bundle = fields->makeEmptyManagedFieldBundle();
  bundle->mesh() = mesh;
  bundle->emplaceField("density", rho);
  bundle->emplaceField("Vx", vx);
  auto meta = arrays->makeManagedDataBundle();
  meta->emplaceScalar("time", 1.5e-6);
  gw->writeSolution(std::string(argv[2]), bundle, meta, 3);
  auto tab = arrays->makeManagedDataBundle();
  tab->emplaceArray("write_times", wt);
  gw->writeTable(std::string(argv[2]) + "_table", tab, 3);
  return 0;
}
