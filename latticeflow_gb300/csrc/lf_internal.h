// Internal declarations shared by the engine translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace lfg {

constexpr int kMaxK = 48;       // largest generated kernel (Full2d_48)
constexpr int kMaxDims = 3;

// One named neighbourhood kernel, in lattice order: offsets [0, K/2) are the
// positive half in ascending linear-jump order and offset i + K/2 is the
// reverse of offset i (lattices/kernellattice.hpp:61-96).
struct KernelDef {
  std::string name;
  std::string alias_of;          // empty unless a duplicate offset set
  int nd = 0;
  int K = 0;
  bool geocut = false;
  std::vector<int> delta;        // K * nd
  std::vector<double> weight;    // K geocut weights (1.0 when not applicable)
};

const std::vector<KernelDef>& kernel_registry();
const KernelDef* find_kernel(const std::string& name);
const std::vector<std::string>& solver_names();

void set_error(const std::string& msg);

}  // namespace lfg
