// iqs_gb300/mpi_env.hpp -- iqs::mpi::Environment and the barrier / print helpers of
// intel/intel-qs (include/mpi_env.hpp:40-175) for callers written against them. Here a process
// drives one GPU and holds one whole state: a pool of one state on one rank (rank 0, sizes 1),
// the layout the reference has without MPI. Barriers return at once; prints follow the
// reference's non-MPI formats (src/mpi_env.cpp:66-87).
#pragma once

#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>

namespace iqs {
namespace mpi {

class Environment {
 public:
  Environment(int& /*argc*/, char**& /*argv*/, bool /*is_verbose*/ = true) {}
  Environment() = default;
  Environment(Environment const&) = delete;
  Environment& operator=(Environment const&) = delete;

  static void UpdateStateComm(int num_states) {
    if (num_states != 1) throw std::invalid_argument("UpdateStateComm: one process holds one state here");
    std::printf("MPI not enabled.\n");
  }
  static bool IsUsefulRank() { return true; }
  static int GetPoolRank() { return 0; }
  static int GetStateRank() { return 0; }
  static int GetRank() { return 0; }
  static int GetPoolSize() { return 1; }
  static int GetStateSize() { return 1; }
  static int GetSize() { return 1; }
  template <class Type>
  static Type IncoherentSumOverAllStatesOfPool(Type local_value) {
    return local_value;
  }
  static int GetNumRanksPerNode() { return 1; }
  static int GetNumNodes() { return 1; }
  static int GetNodeId() { return 0; }
  static int GetStateId() { return 0; }
  static int GetNumStates() { return 1; }
  static void RemapStateRank(int /*newme*/) {}

  static void Init() {
    if (shared_instance_) throw std::runtime_error("MPI Environment is already initialized!");
    shared_instance_ = new Environment;
  }
  static void Init(int& argc, char**& argv) {
    if (shared_instance_) throw std::runtime_error("MPI Environment is already initialized!");
    shared_instance_ = new Environment(argc, argv);
  }
  static void Finalize() {
    delete shared_instance_;
    shared_instance_ = nullptr;
  }
  static Environment* GetSharedInstance() { return shared_instance_; }

 private:
  static inline Environment* shared_instance_ = nullptr;
};

inline void PoolBarrier() {}
inline void StateBarrier() {}
inline void Barrier() {}

inline void StatePrint(std::string s, bool all = false) {
  if (all) {
    std::printf("[|%d>:%3d] %s\n", Environment::GetStateId(), Environment::GetStateRank(), s.c_str());
    std::fflush(stdout);
  } else {
    std::cout << s << std::endl;
  }
}
inline void PoolPrint(std::string s, bool all = false) { StatePrint(s, all); }
inline void Print(std::string s, bool all = false) { StatePrint(s, all); }

}  // namespace mpi
}  // namespace iqs
