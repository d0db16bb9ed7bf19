// Host-side engine: one lattice, one CUDA stream, all device state.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lf_device.cuh"
#include "lf_internal.h"

namespace lfg {

// launchers (lf_kernels.cu)
template <typename T> cudaError_t launch_pr_tile(const PRParams<T>& p, cudaStream_t s);
cudaError_t launch_bfs_tile(const BFSParams& p, cudaStream_t s);
cudaError_t launch_reach_tile(const ReachParams& p, cudaStream_t s);
template <typename T>
cudaError_t launch_mask(const Geo& g, int K, const T* res, const uint64_t* kmask, uint64_t* mask,
                        cudaStream_t s);
cudaError_t launch_fill_energy(const Geo& g, const Stencil& st, int nd, long long N,
                               const int64_t* u, const int64_t* b, long long* exc, long long* cap,
                               long long* c0, int* err, cudaStream_t s);
cudaError_t launch_fill_energy_pf(const Geo& g, const Stencil& st, int nd, long long N,
                                  const int64_t* u, const int64_t* b, long long* exc,
                                  long long* cap, int* err, cudaStream_t s);
cudaError_t launch_fill_caps(const Geo& g, const Stencil& st, int nd, long long N,
                             const int32_t* src, const int32_t* snk, const int32_t* edge,
                             long long* exc, long long* cap, long long* c0, int* err,
                             int pf2x, cudaStream_t s);
cudaError_t launch_range_bound(const Geo& g, const Stencil& st, const long long* exc,
                               const long long* cap, unsigned long long* out, cudaStream_t s);
template <typename T>
cudaError_t launch_convert(long long n, const long long* src, T* dst, cudaStream_t s);
template <typename T>
cudaError_t launch_sum_pos(long long n, const T* x, long long* out, cudaStream_t s);
template <typename T>
cudaError_t launch_init_heights(const Geo& g, const T* exc, const uint64_t* kmask, int* h,
                                cudaStream_t s);
template <typename T>
cudaError_t launch_active(const Geo& g, const T* exc, const int* h, int* act,
                          unsigned long long* count, cudaStream_t s);
template <typename T>
cudaError_t launch_init_marks(long long n, const T* exc, int* mark, cudaStream_t s);
cudaError_t launch_extract_cuts(const Geo& g, int nd, long long N, const int* mark, const int* h,
                                int* cmin, int* cmax, cudaStream_t s);
size_t pr_smem_bytes_for(const Geo& g, const Stencil& st, int elem_bytes);

struct LfError {
  int code;
  std::string msg;
};

struct Tuning {
  int tile_rows = 0;             // TB (2-d) / TB with TA = 4 (3-d); 0 = auto
  int sweeps = 0;                // local push/relabel rounds per tile launch
  int launches_per_relabel = 0;  // tile launches between global relabels
  int height_slack = 0;          // heights above (BFS depth + slack) park until the next relabel
  int pass_chunk = 0;            // BFS / closure passes launched between host checks
};

struct SolveStats {
  long long epochs = 0, pr_launches = 0, bfs_passes = 0, reach_passes = 0;
  unsigned long long tiles_processed = 0;
};

class Engine {
 public:
  Engine(const std::string& solver, const KernelDef* kd, int nd, const size_t* dims);
  ~Engine();

  // metadata
  std::string solver_name, kernel_name;
  const KernelDef* kd;
  bool parametric = false;
  int nd;
  std::vector<size_t> dims;
  long long N = 0;
  Geo g{};
  Stencil st{};
  cudaStream_t stream = nullptr;
  Tuning tune;
  SolveStats stats;

  void add_energy(const int64_t* unary, const int64_t* binary, bool device_ptrs);
  void clear();
  void add_caps(const int32_t* src, const int32_t* snk, const int32_t* edge);
  void run();
  void get_cut(int* out, bool maximal) const;
  void get_levels(int64_t* out) const;

  bool solved = false;
  long long flow = 0, energy = 0;
  double run_time = 0;
  int elem_bytes = 0;  // 4 or 8: working capacity type of the last solve

  // --- internals (public for the parametric / TV driver)
  long long *d_exc64 = nullptr, *d_cap64 = nullptr, *d_c0 = nullptr;
  int* d_err = nullptr;
  void *d_res = nullptr, *d_exc = nullptr;
  int* d_h = nullptr;
  uint64_t* d_mask = nullptr;
  uint64_t* d_kmask = nullptr;
  int* d_mark = nullptr;
  int *d_act[2] = {nullptr, nullptr}, *d_dirty[2] = {nullptr, nullptr};
  int* d_flag = nullptr;
  unsigned long long* d_u64 = nullptr;  // [0] active count, [1] range bound, [2..3] counters
  long long* d_sum = nullptr;           // [0] stuck excess, [1] initial supply
  int* h_pinned = nullptr;              // small pinned scratch
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // profiling: event pairs around launches, summed per category after run()
  bool profiling = false;
  std::vector<cudaEvent_t> pev;
  std::vector<int> pcat;
  size_t pev_used = 0;
  double prof_ms[4] = {0, 0, 0, 0};
  long long prof_cnt[6] = {0, 0, 0, 0, 0, 0};
  long long launches = 0;  // kernel launches since creation
  cudaError_t counted(cudaError_t e) { ++launches; return e; }
  void prof_mark(int cat, bool end);
  void prof_collect();
  std::vector<int> cut_min_host, cut_max_host;
  std::vector<int64_t> levels_host;

  void choose_geometry(int elem);
  void alloc_accumulators();
  void prepare_working(int elem);
  template <typename T> void maxflow(bool compute_sets);
  template <typename T> void global_relabel();
  template <typename T> void reach();
  void sync_read(void* host, const void* dev, size_t bytes);
  void check(cudaError_t e, const char* what) const;
  void free_working();
  void fetch_cuts();
};

void engine_run_parametric(Engine& E);  // lf_param.cu
int tv_2d(const KernelDef* kd, size_t nx, size_t ny, const double* f, double lambda, double* out,
          int64_t* levels_out);

}  // namespace lfg
