// latticeflow_gpu_interface.hpp -- drop-in LatticeFlowInterface over the GPU engine.
//
// Header-only adapter for the reference's abstract solver interface
// (solver/interface.hpp:15-145).  Compile it with the reference's solver/
// directory on the include path; it needs nothing else from the reference.
// getGPULatticeFlowInterface mirrors getLatticeFlowInterface
// (solver/interface.hpp:170-184) and throws BadSolverOrKernelName
// (solver/interface.hpp:152-168) for unknown names, as the generated factory
// does (install/templates/factory/file.cpp:83-95).  Other failures of the C ABI
// become std::runtime_error / std::out_of_range with the library's message.
#ifndef LATTICEFLOW_GPU_INTERFACE_HPP
#define LATTICEFLOW_GPU_INTERFACE_HPP

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "interface.hpp"
#include "latticeflow_gpu.h"

namespace latticeQBP {

class GPULatticeFlowInterface : public LatticeFlowInterface {
 public:
  GPULatticeFlowInterface(const std::string& solver, const std::string& kernel, size_t* dims) {
    const int nd = lf_kernel_dimension(kernel.c_str());
    if (nd < 0 || !lf_is_valid_solver(solver.c_str()))
      throw BadSolverOrKernelName(solver + ", " + kernel);
    check(lf_create(solver.c_str(), kernel.c_str(), nd, dims, &h_));
    const int ne = lf_n_filling_edges(h_);
    std::vector<int> deltas(size_t(ne) * nd);
    check(lf_edge_deltas(h_, deltas.data()));
    init(size_t(nd), size_t(ne), std::vector<size_t>(dims, dims + nd), deltas);
  }

  ~GPULatticeFlowInterface() { lf_destroy(h_); }

  GPULatticeFlowInterface(const GPULatticeFlowInterface&) = delete;
  GPULatticeFlowInterface& operator=(const GPULatticeFlowInterface&) = delete;

  void addEnergyPotentials(long* unary, long* binary) override {
    static_assert(sizeof(long) == sizeof(int64_t), "long must be 64-bit");
    check(lf_add_energy_potentials(h_, reinterpret_cast<const int64_t*>(unary),
                                   reinterpret_cast<const int64_t*>(binary)));
  }

  void run() override { check(lf_run(h_)); }

  double runTime() override { return lf_run_time(h_); }

  // Minimal on-set for the binary cut (see latticeflow_gpu.h), 1 = on.
  vector<int> getCut() const override {
    vector<int> cut(nNodes());
    check(lf_get_cut(h_, cut.data()));
    return cut;
  }

  lf_lattice* handle() const { return h_; }

 private:
  static void check(int rc) {
    if (rc == LF_OK) return;
    if (rc == LF_ERR_BAD_NAME) throw BadSolverOrKernelName(lf_last_error());
    if (rc == LF_ERR_RANGE) throw std::out_of_range(lf_last_error());
    throw std::runtime_error(lf_last_error());
  }

  lf_lattice* h_ = nullptr;
};

// getLatticeFlowInterface(solver, kernel, dims) for the GPU engine.
inline solver_ptr getGPULatticeFlowInterface(const string& solver, const string& kernel,
                                             size_t* dims) {
  return solver_ptr(new GPULatticeFlowInterface(solver, kernel, dims));
}

}  // namespace latticeQBP

#endif  // LATTICEFLOW_GPU_INTERFACE_HPP
