// MPICommunicator.hpp (stand-in) -- NetMPI::MPICommunicator for one process.
//
// The GB300 build runs one partition on one GPU, so the reference runners'
// communicator (modules/NetMPI/include/MPICommunicator.hpp) collapses to a
// single rank: this header, placed ahead of the NetMPI headers on the include
// path, gives the runners the same class name without MPI.  Rank 0 of 1;
// barriers and broadcasts are no-ops, gathers return the caller's own value,
// halo exchanges have nothing to exchange; a receive from another rank has
// no sender and throws std::runtime_error.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>

#include "Array.hpp"
#include "Communicator.hpp"
#include "Field.hpp"
#include "Mesh.hpp"

namespace NetMPI {

class MPICommunicator : public PanNDE::Communicator {
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

  void sendArray(std::shared_ptr<PanNDE::Array<double>>, int r) override { no_peer(r); }
  void sendArray(double *, int, int r) override { no_peer(r); }
  std::shared_ptr<PanNDE::Array<double>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<double>>,
                                                   int s) override {
    no_peer(s);
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<double>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int32_t>>, int r) override { no_peer(r); }
  void sendArray(int32_t *, int, int r) override { no_peer(r); }
  std::shared_ptr<PanNDE::Array<int32_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int32_t>>,
                                                    int s) override {
    no_peer(s);
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int32_t>> &, int) override {}
  void sendArray(std::shared_ptr<PanNDE::Array<int64_t>>, int r) override { no_peer(r); }
  void sendArray(int64_t *, int, int r) override { no_peer(r); }
  std::shared_ptr<PanNDE::Array<int64_t>> recvArray(std::shared_ptr<PanNDE::ArrayFactory<int64_t>>,
                                                    int s) override {
    no_peer(s);
    return nullptr;
  }
  void broadcastArray(std::shared_ptr<PanNDE::Array<int64_t>> &, int) override {}

  void sendValue(double, int r) override { no_peer(r); }
  void recvValue(double *, int s) override { no_peer(s); }
  void broadcastValue(double *, int) override {}
  std::shared_ptr<PanNDE::Array<double>> allGatherValue(double v,
                                                        std::shared_ptr<PanNDE::ArrayFactory<double>> m) override {
    return gather_one(v, m);
  }
  void sendValue(int32_t, int r) override { no_peer(r); }
  void recvValue(int32_t *, int s) override { no_peer(s); }
  void broadcastValue(int32_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int32_t>> allGatherValue(int32_t v,
                                                         std::shared_ptr<PanNDE::ArrayFactory<int32_t>> m) override {
    return gather_one(v, m);
  }
  void sendValue(int64_t, int r) override { no_peer(r); }
  void recvValue(int64_t *, int s) override { no_peer(s); }
  void broadcastValue(int64_t *, int) override {}
  std::shared_ptr<PanNDE::Array<int64_t>> allGatherValue(int64_t v,
                                                         std::shared_ptr<PanNDE::ArrayFactory<int64_t>> m) override {
    return gather_one(v, m);
  }
  void waitall() override {}
  void barrier() override {}

 private:
  // a message to or from rank 0 itself is the only one a single rank could
  // send; there is no transport for it, nor for any other rank
  static void no_peer(int rank) {
    throw std::runtime_error("single-process communicator: no rank " + std::to_string(rank) + " to exchange with");
  }
  template <typename T>
  static std::shared_ptr<PanNDE::Array<T>> gather_one(T v, std::shared_ptr<PanNDE::ArrayFactory<T>> m) {
    auto a = m->makeManagedArray();
    a->resize(1);
    a->at(0) = v;
    return a;
  }
};

}  // namespace NetMPI
