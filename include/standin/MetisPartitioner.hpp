// MetisPartitioner.hpp (stand-in) -- NetMPI::MetisPartitioner for one
// partition.
//
// The reference partitions the global mesh with METIS for its MPI ranks
// (modules/NetMPI/include/MetisPartitioner.hpp); the GB300 build runs a
// single partition per GPU, and the runners' Boss::METISManager already
// returns the global mesh and fields untouched when there is one process
// (Boss.hpp:344-360).  This class keeps the constructor the runners call and
// hands back the whole mesh / field as partition 0; asking for more than one
// partition throws std::runtime_error.
#pragma once
#include <memory>
#include <stdexcept>

#include "Array.hpp"
#include "Communicator.hpp"
#include "Field.hpp"
#include "Mesh.hpp"
#include "Partitioner.hpp"

namespace NetMPI {

class MetisPartitioner : public Controller::Partitioner {
 public:
  MetisPartitioner(std::shared_ptr<PanNDE::ArrayFactory<int32_t>> i32,
                   std::shared_ptr<PanNDE::ArrayFactory<int64_t>> i64,
                   std::shared_ptr<PanNDE::ArrayFactory<double>> f64,
                   std::shared_ptr<PanNDE::Communicator> comm)
      : i32_(i32), i64_(i64), f64_(f64), comm_(comm) {}

  void partitionMesh(int Nparts, std::shared_ptr<PanNDE::Mesh> global_mesh) override {
    if (Nparts != 1) throw std::runtime_error("single-partition build: cannot split a mesh into parts");
    mesh_ = global_mesh;
  }

  std::shared_ptr<PanNDE::Array<std::shared_ptr<PanNDE::Mesh>>> distributeMeshPartitions(
      std::shared_ptr<PanNDE::Array<int>> partitionIds, std::shared_ptr<PanNDE::MeshFactory> maker,
      int = 0) override {
    check_ids(partitionIds);
    auto out = maker->makeManagedMeshArray();
    out->resize(1);
    out->at(0) = mesh_;
    return out;
  }

  std::shared_ptr<PanNDE::Array<std::shared_ptr<PanNDE::Field>>> distributeFieldPartitions(
      std::shared_ptr<PanNDE::Array<int>> partitionIds, std::shared_ptr<PanNDE::FieldFactory> maker,
      std::shared_ptr<PanNDE::Field> global_field = nullptr, int = 0) override {
    check_ids(partitionIds);
    auto out = maker->makeManagedFieldArray();
    out->resize(1);
    out->at(0) = global_field;
    return out;
  }

 private:
  static void check_ids(std::shared_ptr<PanNDE::Array<int>> ids) {
    if (ids && (ids->size() != 1 || ids->at(0) != 0))
      throw std::runtime_error("single-partition build: only partition 0 exists");
  }
  std::shared_ptr<PanNDE::ArrayFactory<int32_t>> i32_;
  std::shared_ptr<PanNDE::ArrayFactory<int64_t>> i64_;
  std::shared_ptr<PanNDE::ArrayFactory<double>> f64_;
  std::shared_ptr<PanNDE::Communicator> comm_;
  std::shared_ptr<PanNDE::Mesh> mesh_;
};

}  // namespace NetMPI
