// Host-side engine: one lattice, one CUDA stream, all device state.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lf_device.cuh"
#include "lf_internal.h"
#include "lf_pool_runner.h"

namespace lfg {

// Stream-ordered temporary device buffer (no device-wide synchronisation,
// so concurrent solves on other streams keep running), freed in stream order
// when it goes out of scope, on error paths too.
template <class T>
struct DevBuf {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  void alloc(size_t count, cudaStream_t st) {
    s = st;
    cudaError_t e = cudaMallocAsync(&p, count * sizeof(T), st);
    if (e != cudaSuccess) {
      p = nullptr;
      throw LfError{e == cudaErrorMemoryAllocation ? 5 : 6,
                    std::string("cudaMallocAsync: ") + cudaGetErrorString(e)};
    }
  }
  ~DevBuf() { if (p) cudaFreeAsync(p, s); }
};

// per-lattice element kernels (lf_kernels.cu)
cudaError_t launch_fill_energy(const Geo& g, const Stencil& st, int nd, long long N,
                               const int64_t* u, const int64_t* b, long long* exc, long long* cap,
                               long long* c0, int* err, int form, cudaStream_t s);
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
cudaError_t launch_convert_bounded(long long NP, int K, const long long* exc64,
                                  const long long* cap64, int* exc, int* res,
                                  unsigned long long* mx, cudaStream_t s);
template <typename T>
cudaError_t launch_sum_pos(long long n, const T* x, long long* out, cudaStream_t s);
cudaError_t launch_extract_cuts(const Geo& g, int nd, long long N, const int* mark, const int* h,
                                int* cmin, int* cmax, cudaStream_t s);
size_t pr_smem_bytes_for(const Geo& g, const Stencil& st, int elem_bytes);

// Geometry of one lattice: padding fixed by the largest tile, tile extents
// chosen per working element size so that the push/relabel tile fits.
void lattice_geometry(int nd, const size_t* dims, const Stencil& st, int elem, int tile_rows,
                      Geo& g);
Stencil make_stencil(const KernelDef* kd);
// the device address of a pinned (page-locked) host array, which kernels can
// read in place (over NVLink-C2C on GB300), or null for other memory
const void* mapped_host_ptr(const void* p);

class Engine : public ProfHooks {
 public:
  Engine(const std::string& solver, const KernelDef* kd, int nd, const size_t* dims);
  ~Engine();

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
  void get_cut(int* out, bool maximal);
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
  void* d_stage = nullptr;  // host_stage: device copy of pinned energies (kept)
  size_t stage_bytes = 0;
  unsigned long long* d_u64 = nullptr;  // [1] range bound
  long long* d_sum = nullptr;           // [0] stuck excess, [1] initial supply
  int* h_pinned = nullptr;              // small pinned scratch
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  PoolRunner runner;
  bool runner_ready = false;
  // > 1: the lattice holds sub_count independent lattices of sub_real_rows
  // rows each, stacked every sub_rows (a multiple of 32) rows; each is its
  // own pool instance in the solve
  int sub_count = 1, sub_rows = 0, sub_real_rows = 0;
  // profiling: event pairs around launches, summed per category after run()
  std::vector<cudaEvent_t> pev;
  std::vector<int> pcat;
  size_t pev_used = 0;
  double prof_ms[4] = {0, 0, 0, 0};
  long long prof_cnt[6] = {0, 0, 0, 0, 0, 0};
  void mark(int cat, bool end) override;
  void prof_collect();
  cudaError_t counted(cudaError_t e) { ++launches; return e; }
  int* d_cuts = nullptr;  // [2N] minimal / maximal on-set, filled by extract_cuts
  std::vector<int64_t> levels_host;
  // parametric solver: level set of every node (row-major), numbered in the
  // order the reference returns its level sets (pf_solver.hpp:180-203)
  std::vector<int> level_sets_host;

  void choose_geometry(int elem);
  void alloc_accumulators();
  void prepare_working(int elem, bool convert = true);
  template <typename T> void maxflow(bool compute_sets);
  void sync_read(void* host, const void* dev, size_t bytes);
  void check(cudaError_t e, const char* what) const;
  void free_working();
  void extract_cuts();
};

void engine_run_parametric(Engine& E);  // lf_param.cu
// engine of `count` stacked nx x ny TV problems (count 1: a plain lattice)
Engine* new_tv_stack_engine(const KernelDef* kd, size_t nx, size_t ny, size_t count);
int cut_2d_noalloc(const char* kernel, size_t nx, size_t ny, const int32_t* src,
                   const int32_t* snk, const int32_t* edge, int32_t* cut, int64_t* flow_energy,
                   cudaStream_t s);  // lf_noalloc.cu
int tv_2d(const KernelDef* kd, size_t nx, size_t ny, const double* f, double lambda, double* out,
          int64_t* levels_out, int32_t* sets_out = nullptr);
void tv_fill_single(Engine& E, const double* f, double lambda, double* mean, double* scale,
                    std::vector<int64_t>* base_fv, std::vector<long long>* pwf2_out);
// the reference's regularisation path (lf_tvpath.cu); stats (may be null,
// else 10 entries): [0] path segments, [1] region probes, [2] events, [3]
// initial level sets, [4] probes on the lattice-wide solver, [5]-[7]
// microseconds in those probes, in fused probes, in segment set-ups,
// [8] [9] epochs and BFS levels of the fused probes
int tv_2d_path(const KernelDef* kd, size_t nx, size_t ny, const double* f, size_t n_lambda,
               const double* lambdas, double* out, int64_t* stats);
int tv_2d_on(Engine& E, const double* f, double lambda, double* out, int64_t* levels_out);
int tv_2d_stack_on(Engine& E, size_t nx, size_t ny, size_t count, const double* f,
                   size_t f_stride, const double* lambdas, double* out, int64_t* levels_out);
size_t tv_stack_size(size_t nx, size_t ny, size_t count, size_t max_nodes);
constexpr size_t kTVStackNodes = size_t(1) << 18;  // default bound of one TV stack
int tv_2d_batch(const KernelDef* kd, size_t nx, size_t ny, size_t count, const double* f,
                size_t f_stride, const double* lambdas, double* out, int64_t* levels_out,
                size_t max_nodes, int workers = 0);

}  // namespace lfg
