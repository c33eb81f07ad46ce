// VTKGateway.hpp (stand-in) -- VTKIO::VTKGateway without the VTK library.
//
// The reference's gateway (modules/VTKIO/include/VTKGateway.hpp) reads the
// job's .vtu and writes solutions and tables through VTK.  This class keeps
// its name, constructor and Controller::Gateway behaviour on top of the
// project's own VTK-XML reader / writer (pn_vtu.hpp):
//   open          loads a .vtu (ascii, binary, appended raw/base64; zlib
//                 blocks when <zlib.h> is present)
//   getMesh       points -> nodes (owner 0), hexahedra -> cells, in file order
//                 (VTKRead.hpp:205-231)
//   getField      PointData -> NODE field, CellData -> CELL field, first
//                 component (VTKRead.hpp:148-160, 264-297)
//   getValue      first entry of the FieldData array of that name
//   getArray      the FieldData array of that name
//   writeSolution <base>_<index>.vtu (<base>.vtu without an index): the
//                 bundle's mesh, NODE fields as PointData, the others as
//                 CellData, meta scalars and arrays as FieldData
//                 (VTKWrite.hpp:216-231 naming, one process)
//   writeTable    <base>_<index>.vtt (<base>.vtt): data arrays as columns,
//                 data scalars and meta as FieldData
// Missing names throw std::runtime_error("no data by this name present"), as
// the reference does.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Array.hpp"
#include "Communicator.hpp"
#include "Field.hpp"
#include "Gateway.hpp"
#include "Mesh.hpp"
#include "pn_vtu.hpp"

namespace VTKIO {

class VTKGateway : public Controller::Gateway {
 public:
  VTKGateway(std::shared_ptr<PanNDE::Communicator> communicator = nullptr) : comm_(communicator) {}

  static inline std::shared_ptr<VTKIO::VTKGateway> makeShared(
      std::shared_ptr<PanNDE::Communicator> communicator = nullptr) {
    return std::make_shared<VTKIO::VTKGateway>(communicator);
  }

  void open(std::string filename) override {
    grid_ = std::make_shared<pnvtu::Grid>(pnvtu::read_vtu(filename));
    file_ = filename;
    mesh_ = nullptr;
  }

  void close() override {
    grid_ = nullptr;
    mesh_ = nullptr;
  }

  std::shared_ptr<PanNDE::Array<double>> getArray(std::string keyname,
                                                  std::shared_ptr<PanNDE::ArrayFactory<double>> maker) override {
    const pnvtu::DataArray &a = field_array(keyname);
    auto out = maker->makeManagedArray();
    out->resize((int64_t)a.values.size());
    for (int64_t k = 0; k < out->size(); k++) out->at(k) = a.values[(size_t)k];
    return out;
  }

  double getValue(std::string keyname) override {
    const pnvtu::DataArray &a = field_array(keyname);
    if (a.values.empty()) throw std::runtime_error("no data by this name present");
    return a.values[0];
  }

  std::shared_ptr<PanNDE::Mesh> getMesh(std::shared_ptr<PanNDE::MeshFactory> maker, int host_id = 0) override {
    if (comm_ && comm_->getProcessId() != host_id) return nullptr;
    need_file();
    if (mesh_) return mesh_;
    const pnvtu::Grid &g = *grid_;
    std::vector<PanNDE::Mesh::Node> nodes;
    std::vector<PanNDE::Mesh::Cell> cells;
    nodes.reserve((size_t)g.n_points());
    cells.reserve((size_t)g.n_cells());
    for (int64_t p = 0; p < g.n_points(); p++) {
      double pt[3] = {g.points[(size_t)(3 * p)], g.points[(size_t)(3 * p + 1)], g.points[(size_t)(3 * p + 2)]};
      nodes.push_back(maker->makeNode(pt, p, 0));
    }
    int64_t begin = 0;
    for (int64_t c = 0; c < g.n_cells(); c++) {
      const int64_t end = (int64_t)g.offsets[(size_t)c];
      if (end - begin != 8) throw std::runtime_error("vtu: only 8-node hexahedral cells are supported");
      int32_t box[8];
      for (int k = 0; k < 8; k++) box[k] = (int32_t)g.connectivity[(size_t)(begin + k)];
      cells.push_back(maker->makeCell(box, 8, c, 0));
      begin = end;
    }
    mesh_ = maker->makeManagedMesh(nodes.data(), (int64_t)nodes.size(), cells.data(), (int64_t)cells.size());
    return mesh_;
  }

  std::shared_ptr<PanNDE::Field> getField(std::string keyname, std::shared_ptr<PanNDE::FieldFactory> maker,
                                          int host_id = 0) override {
    if (comm_ && comm_->getProcessId() != host_id) return nullptr;
    need_file();
    if (!mesh_) throw std::runtime_error("no mesh loaded");
    const pnvtu::Grid &g = *grid_;
    const pnvtu::DataArray *a = pnvtu::Grid::find(g.point_data, keyname);
    PanNDE::Field::FieldType type = PanNDE::Field::NODE;
    if (!a) {
      a = pnvtu::Grid::find(g.cell_data, keyname);
      type = PanNDE::Field::CELL;
    }
    if (!a) throw std::runtime_error("no data by this name present");
    auto f = maker->makeManagedField(mesh_, type);
    const int nc = a->components > 0 ? a->components : 1;
    for (int32_t k = 0; k < f->size(); k++) f->at(k) = a->values[(size_t)k * nc];
    return f;
  }

  void writeSolution(std::string base, std::shared_ptr<PanNDE::FieldBundle> solution, int write_index) override {
    write_grid(base + "_" + std::to_string(write_index), solution, nullptr);
  }
  void writeSolution(std::string base, std::shared_ptr<PanNDE::FieldBundle> solution,
                     std::shared_ptr<PanNDE::DataBundle<double>> meta, int write_index) override {
    write_grid(base + "_" + std::to_string(write_index), solution, meta);
  }
  void writeSolution(std::string base, std::shared_ptr<PanNDE::FieldBundle> solution,
                     std::shared_ptr<PanNDE::DataBundle<double>> meta) override {
    write_grid(base, solution, meta);
  }
  void writeSolution(std::string base, std::shared_ptr<PanNDE::FieldBundle> solution) override {
    write_grid(base, solution, nullptr);
  }

  void writeTable(std::string base, std::shared_ptr<PanNDE::DataBundle<double>> data,
                  std::shared_ptr<PanNDE::DataBundle<double>> meta, int write_index) override {
    write_table(base + "_" + std::to_string(write_index), data, meta);
  }
  void writeTable(std::string base, std::shared_ptr<PanNDE::DataBundle<double>> data,
                  std::shared_ptr<PanNDE::DataBundle<double>> meta) override {
    write_table(base, data, meta);
  }
  void writeTable(std::string base, std::shared_ptr<PanNDE::DataBundle<double>> data, int write_index) override {
    write_table(base + "_" + std::to_string(write_index), data, nullptr);
  }
  void writeTable(std::string base, std::shared_ptr<PanNDE::DataBundle<double>> data) override {
    write_table(base, data, nullptr);
  }

  std::string currentlyActiveFile() { return file_; }

 private:
  void need_file() const {
    if (!grid_) throw std::runtime_error("no file provided");
  }
  const pnvtu::DataArray &field_array(const std::string &name) const {
    need_file();
    const pnvtu::DataArray *a = pnvtu::Grid::find(grid_->field_data, name);
    if (!a) throw std::runtime_error("no data by this name present");
    return *a;
  }

  static void add_bundle(std::vector<pnvtu::DataArray> &out, std::shared_ptr<PanNDE::DataBundle<double>> b) {
    if (!b) return;
    for (int k = 0; k < b->scalarCount(); k++) {
      const std::string n = b->scalarName(k);
      out.push_back(pnvtu::DataArray{n, "Float64", 1, {b->scalar(n)}});
    }
    for (int k = 0; k < b->arrayCount(); k++) {
      const std::string n = b->arrayName(k);
      auto a = b->array(n);
      pnvtu::DataArray d{n, "Float64", 1, {}};
      d.values.assign(a->data(), a->data() + a->size());
      out.push_back(std::move(d));
    }
  }

  static void write_grid(const std::string &name, std::shared_ptr<PanNDE::FieldBundle> sol,
                         std::shared_ptr<PanNDE::DataBundle<double>> meta) {
    auto mesh = sol->mesh();
    pnvtu::Grid g;
    const int32_t nn = mesh->nodeCount(), nc = mesh->cellCount();
    g.points.resize((size_t)nn * 3);
    for (int32_t n = 0; n < nn; n++) mesh->nodeCoordinate(n, &g.points[(size_t)n * 3]);
    g.connectivity.resize((size_t)nc * 8);
    g.offsets.resize((size_t)nc);
    g.types.assign((size_t)nc, 12.0);  // VTK_HEXAHEDRON
    for (int32_t c = 0; c < nc; c++) {
      int32_t box[8];
      mesh->cell(c, box);
      for (int k = 0; k < 8; k++) g.connectivity[(size_t)c * 8 + k] = box[k];
      g.offsets[(size_t)c] = 8.0 * (c + 1);
    }
    for (int k = 0; k < sol->fieldCount(); k++) {
      const std::string n = sol->fieldName(k);
      auto f = sol->field(n);
      pnvtu::DataArray d{n, "Float64", 1, {}};
      d.values.assign(f->data(), f->data() + f->size());
      if (f->type() == PanNDE::Field::NODE) g.point_data.push_back(std::move(d));
      else if (f->size() == nc) g.cell_data.push_back(std::move(d));
      else g.field_data.push_back(std::move(d));  // CONSTANT: one value
    }
    add_bundle(g.field_data, meta);
    pnvtu::write_vtu(name + ".vtu", g);
  }

  static void write_table(const std::string &name, std::shared_ptr<PanNDE::DataBundle<double>> data,
                          std::shared_ptr<PanNDE::DataBundle<double>> meta) {
    pnvtu::Table t;
    for (int k = 0; k < data->arrayCount(); k++) {
      const std::string n = data->arrayName(k);
      auto a = data->array(n);
      pnvtu::DataArray d{n, "Float64", 1, {}};
      d.values.assign(a->data(), a->data() + a->size());
      t.columns.push_back(std::move(d));
    }
    for (int k = 0; k < data->scalarCount(); k++) {
      const std::string n = data->scalarName(k);
      t.field_data.push_back(pnvtu::DataArray{n, "Float64", 1, {data->scalar(n)}});
    }
    add_bundle(t.field_data, meta);
    pnvtu::write_vtt(name + ".vtt", t);
  }

  std::shared_ptr<PanNDE::Communicator> comm_;
  std::shared_ptr<pnvtu::Grid> grid_;
  std::shared_ptr<PanNDE::Mesh> mesh_;
  std::string file_;
};

}  // namespace VTKIO
