// C-ABI driver around the UNMODIFIED reference solvers (test infrastructure).
//
// Compiled by oracle/Makefile against the reference headers where they lie,
// with the shims in oracle/shim and the kernel header written by
// oracle/gen_ref_kernels.py.  Output goes to oracle/_ref/ only.  The entry
// points run the reference's own public paths:
//   * LatticeFlowDirectInterface<Solver<nd, Kernel>>  (interfacing/direct_interface.hpp:11-108)
//     for Solver in {LatticeEnergyMinimizer (energy.hpp:39-49),
//                    BKGCEnergyMinimizer (energy.hpp:54-66),
//                    LatticeLevelReductions (parametricflow/pf_policies.hpp:31-46)}
//   * calculate2dTV<Kernel, long> single-lambda and path (tv/tv_solver.hpp:650-681)
#include <chrono>
#include <cstring>
#include <string>
#include <vector>
#include <memory>

#include "solvers.hpp"
#include "interfacing/direct_interface.hpp"

using namespace latticeQBP;

namespace {

template <class Solver, int nd>
int run_direct(const size_t* dims, long* unary, long* binary, int* cut_out,
               double* wall_s, double* cpu_s, int* filling_deltas) {
  Array<size_t, nd> d;
  for (int i = 0; i < nd; ++i) d[i] = dims[i];
  LatticeFlowDirectInterface<Solver> iface(d);
  if (filling_deltas) {
    const auto& ed = iface.edgeDeltas();
    for (size_t i = 0; i < ed.size(); ++i) filling_deltas[i] = ed[i];
  }
  if (!unary) return int(iface.nFillingEdges());
  iface.addEnergyPotentials(unary, binary);
  auto t0 = std::chrono::steady_clock::now();
  iface.run();
  auto t1 = std::chrono::steady_clock::now();
  if (wall_s) *wall_s = std::chrono::duration<double>(t1 - t0).count();
  if (cpu_s) *cpu_s = iface.runTime();
  std::vector<int> cut = iface.getCut();
  std::memcpy(cut_out, cut.data(), cut.size() * sizeof(int));
  return int(iface.nFillingEdges());
}

template <template <int, typename, typename> class S, int nd, class K>
int run_solver(const size_t* dims, long* u, long* b, int* c, double* w, double* cp, int* fd) {
  return run_direct<S<nd, K, long>, nd>(dims, u, b, c, w, cp, fd);
}

}  // namespace

// The kernel instantiations are split over four translation units, compiled
// in parallel from this file with -DLF_REF_PART=1..4; part 0 holds the C
// entry points and the TV functions.  Solver ids: 0 LatticeEnergyMinimizer,
// 1 BKGCEnergyMinimizer, 2 LatticeLevelReductions.
#define LF_KERNELS_1(X) X(2, Full2d_4) X(2, Full2d_8) X(2, Full2d_12) X(2, Star2d_16) \
                        X(1, Full1d_2) X(1, Full1d_4)
#define LF_KERNELS_2(X) X(2, Full2d_20) X(2, Full2d_24) X(2, Star2d_24) X(2, Full2d_28) \
                        X(1, Full1d_6) X(1, Full1d_8)
#define LF_KERNELS_3(X) X(2, Star2d_32) X(2, Full2d_36) X(2, Full2d_48) X(1, Full1d_10) \
                        X(1, Full1d_12)
#define LF_KERNELS_4(X) X(3, Full3d_6) X(3, Full3d_18) X(3, Star3d_26) X(3, Full3d_32) \
                        X(1, Full1d_14) X(4, Full4d_8)

#define LF_PART_DECL(N)                                                                   \
  int lf_ref_part_##N(int solver, const std::string& k, const size_t* dims, long* u, long* b, \
                      int* c, double* w, double* cp, int* fd)
LF_PART_DECL(1);
LF_PART_DECL(2);
LF_PART_DECL(3);
LF_PART_DECL(4);

#if defined(LF_REF_PART) && LF_REF_PART >= 1
#if LF_REF_PART == 1
#define LF_KERNELS LF_KERNELS_1
#elif LF_REF_PART == 2
#define LF_KERNELS LF_KERNELS_2
#elif LF_REF_PART == 3
#define LF_KERNELS LF_KERNELS_3
#else
#define LF_KERNELS LF_KERNELS_4
#endif

namespace {
template <template <int, typename, typename> class S>
int dispatch(const std::string& k, const size_t* dims, long* u, long* b, int* c, double* w,
             double* cp, int* fd) {
#define X(ND, KN) if (k == #KN) return run_solver<S, ND, KN>(dims, u, b, c, w, cp, fd);
  LF_KERNELS(X)
#undef X
  return -1;
}
}  // namespace

#define LF_PART_DEF(N)                                                                 \
  LF_PART_DECL(N) {                                                                     \
    if (solver == 0) return dispatch<LatticeEnergyMinimizer>(k, dims, u, b, c, w, cp, fd); \
    if (solver == 1) return dispatch<BKGCEnergyMinimizer>(k, dims, u, b, c, w, cp, fd);    \
    if (solver == 2) return dispatch<LatticeLevelReductions>(k, dims, u, b, c, w, cp, fd); \
    return -1;                                                                          \
  }
#if LF_REF_PART == 1
LF_PART_DEF(1)
#elif LF_REF_PART == 2
LF_PART_DEF(2)
#elif LF_REF_PART == 3
LF_PART_DEF(3)
#else
LF_PART_DEF(4)
#endif

#else  // part 0: the C entry points

extern "C" {

// Solve one lattice problem with a reference solver.  unary: 2*N longs (E0,E1),
// binary: N*(K/2)*4 longs (E00,E01,E10,E11), both as interface.hpp:49-60.
// Passing unary == NULL only reports the filling deltas.  Returns K/2 or -1.
int ref_solve(const char* solver, const char* kernel, const size_t* dims,
              long* unary, long* binary, int* cut_out, double* wall_s,
              double* cpu_s, int* filling_deltas) {
  std::string s(solver);
  const int id = s == "LatticeEnergyMinimizer" ? 0 : s == "BKGCEnergyMinimizer" ? 1
               : s == "LatticeLevelReductions" ? 2 : -1;
  if (id < 0) return -1;
  std::string k(kernel);
  if (k == "Full3d_26") k = "Star3d_26";
  if (k == "Star2d_4") k = "Full2d_4";
  if (k == "Star2d_8") k = "Full2d_8";
  if (k == "Star3d_6") k = "Full3d_6";
  if (k == "Star3d_18") k = "Full3d_18";
  if (k == "Star4d_8") k = "Full4d_8";
  for (auto part : {lf_ref_part_1, lf_ref_part_2, lf_ref_part_3, lf_ref_part_4}) {
    const int r = part(id, k, dims, unary, binary, cut_out, wall_s, cpu_s, filling_deltas);
    if (r >= 0) return r;
  }
  return -1;
}

// calculate2dTV<Kernel, long>(nx, ny, f, lambda)  (tv/tv_solver.hpp:650-655)
int ref_tv_single(const char* kernel, size_t nx, size_t ny, double* f, double lam,
                  double* out, double* wall_s) {
  std::string k(kernel);
  FuncMapPtr R;
  auto t0 = std::chrono::steady_clock::now();
  if (k == "Full2d_4" || k == "Star2d_4") R = calculate2dTV<Full2d_4, long>(nx, ny, f, lam);
  else if (k == "Full2d_8" || k == "Star2d_8") R = calculate2dTV<Full2d_8, long>(nx, ny, f, lam);
  else if (k == "Star2d_16") R = calculate2dTV<Star2d_16, long>(nx, ny, f, lam);
  else return -1;
  auto t1 = std::chrono::steady_clock::now();
  if (wall_s) *wall_s = std::chrono::duration<double>(t1 - t0).count();
  for (size_t x = 0; x < nx; ++x)
    for (size_t y = 0; y < ny; ++y) out[x * ny + y] = R->at(x, y);
  return 0;
}

// calculate2dTV<Kernel, long>(nx, ny, f, lambdas)  (tv/tv_solver.hpp:659-681)
int ref_tv_path(const char* kernel, size_t nx, size_t ny, double* f, int nl,
                const double* lams, double* out, double* wall_s) {
  std::string k(kernel);
  std::vector<double> lv(lams, lams + nl);
  RegPathPtr R;
  auto t0 = std::chrono::steady_clock::now();
  if (k == "Full2d_4" || k == "Star2d_4") R = calculate2dTV<Full2d_4, long>(nx, ny, f, lv);
  else if (k == "Full2d_8" || k == "Star2d_8") R = calculate2dTV<Full2d_8, long>(nx, ny, f, lv);
  else if (k == "Star2d_16") R = calculate2dTV<Star2d_16, long>(nx, ny, f, lv);
  else return -1;
  auto t1 = std::chrono::steady_clock::now();
  if (wall_s) *wall_s = std::chrono::duration<double>(t1 - t0).count();
  for (int i = 0; i < nl; ++i)
    for (size_t x = 0; x < nx; ++x)
      for (size_t y = 0; y < ny; ++y) out[(size_t(i) * nx + x) * ny + y] = R->at(size_t(i), x, y);
  return 0;
}

}  // extern "C"

#endif  // LF_REF_PART
