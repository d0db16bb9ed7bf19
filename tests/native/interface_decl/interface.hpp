// Test-only declaration of latticeQBP::LatticeFlowInterface with the members of
// the reference's abstract solver interface (solver/interface.hpp:15-145,
// 152-168): the virtual calls addEnergyPotentials / run / runTime / getCut,
// the metadata accessors, the protected init(), BadSolverOrKernelName and
// solver_ptr.  It lets the drop-in adapter (include/latticeflow_gpu_interface.hpp)
// be compiled and run where the reference's sources are absent (the GPU
// host); where they are present, tests/test_adapter.py compiles the adapter
// against the reference's own header.
#ifndef LATTICEFLOW_TEST_INTERFACE_DECL_HPP
#define LATTICEFLOW_TEST_INTERFACE_DECL_HPP

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace latticeQBP {

using std::string;
using std::vector;

class LatticeFlowInterface {
 public:
  virtual ~LatticeFlowInterface() {}
  size_t nDimensions() const { return n_dimensions_; }
  const vector<size_t>& shape() const { return shape_; }
  size_t nNodes() const { return n_nodes_; }
  size_t nFillingEdges() const { return n_filling_edges_; }
  const vector<int>& edgeDeltas() const { return edge_deltas_; }
  virtual void addEnergyPotentials(long* unary_energy_array, long* binary_energy_array) = 0;
  virtual void run() = 0;
  virtual double runTime() = 0;
  virtual vector<int> getCut() const = 0;

 protected:
  LatticeFlowInterface() {}
  void init(size_t n_dimensions, size_t n_filling_edges, vector<size_t> shape,
            vector<int> edge_deltas) {
    n_dimensions_ = n_dimensions;
    n_filling_edges_ = n_filling_edges;
    n_nodes_ = 1;
    for (size_t v : shape) n_nodes_ *= v;
    shape_ = shape;
    edge_deltas_ = edge_deltas;
  }

 private:
  size_t n_dimensions_ = 0, n_filling_edges_ = 0, n_nodes_ = 0;
  vector<size_t> shape_;
  vector<int> edge_deltas_;
};

typedef std::shared_ptr<LatticeFlowInterface> solver_ptr;

class BadSolverOrKernelName : public std::runtime_error {
 public:
  explicit BadSolverOrKernelName(const string& s) : std::runtime_error(s) {}
};

}  // namespace latticeQBP

#endif
