// Runs the drop-in adapter (include/latticeflow_gpu_interface.hpp) through
// the abstract interface's virtual calls: factory, metadata, fill, run,
// getCut.  Usage: adapter_run kernel n0 n1 unary.bin binary.bin cut.out
// (int64 energies in the interface's layout; the cut written as int32).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "latticeflow_gpu_interface.hpp"

using namespace latticeQBP;

template <class T>
std::vector<T> load(const char* path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  const std::streamsize n = f.tellg();
  f.seekg(0);
  std::vector<T> v(size_t(n) / sizeof(T));
  f.read(reinterpret_cast<char*>(v.data()), n);
  return v;
}

int main(int argc, char** argv) {
  if (argc != 7) return 2;
  size_t dims[2] = {size_t(std::stoul(argv[2])), size_t(std::stoul(argv[3]))};
  try {
    getGPULatticeFlowInterface("NoSuchSolver", argv[1], dims);
    std::cerr << "bad solver name accepted\n";
    return 3;
  } catch (const BadSolverOrKernelName&) {
  }
  solver_ptr s = getGPULatticeFlowInterface("LatticeEnergyMinimizer", argv[1], dims);
  LatticeFlowInterface& L = *s;  // the calls below go through the base's vtable
  std::vector<long> u = load<long>(argv[4]), b = load<long>(argv[5]);
  if (L.nDimensions() != 2 || L.nNodes() != dims[0] * dims[1] ||
      u.size() != 2 * L.nNodes() || b.size() != 4 * L.nNodes() * L.nFillingEdges() ||
      L.edgeDeltas().size() != 2 * L.nFillingEdges()) {
    std::cerr << "metadata mismatch\n";
    return 4;
  }
  L.addEnergyPotentials(u.data(), b.data());
  L.run();
  const std::vector<int> cut = L.getCut();
  std::ofstream o(argv[6], std::ios::binary);
  o.write(reinterpret_cast<const char*>(cut.data()), cut.size() * sizeof(int));
  std::printf("ok %zu nodes, %zu filling edges, %.6f s\n", L.nNodes(), L.nFillingEdges(), L.runTime());
  return 0;
}
