// Batch of lattices solved in one instance pool (see lf_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "lf_engine.h"

namespace lfg {

struct Member {
  const KernelDef* kd = nullptr;
  int nd = 0;
  std::vector<size_t> dims;
  long long N = 0;
  Stencil st{};
  Geo g{};
  long long node_base = 0, res_base = 0;
  int tile_base = 0;
  long long flow = 0, energy = 0;
  long long cut_off = 0;
};

class Batch {
 public:
  Batch();
  ~Batch();
  int add(const KernelDef* kd, int nd, const size_t* dims);
  void add_caps(int i, const int32_t* src, const int32_t* snk, const int32_t* edge);
  void add_energy(int i, const int64_t* unary, const int64_t* binary);
  void add_caps_packed(const int32_t* src, const int32_t* snk, const int32_t* edge);
  void get_cuts_packed(int* out, bool maximal);
  void clear();
  void run();
  void get_cut(int i, int* out, bool maximal);
  Member& member(int i);
  void relayout() { runner_ready = false; }

  std::vector<Member> members;
  Tuning tune;
  SolveStats stats;
  bool solved = false;
  bool defer_checks = false;  // validate fills once, at run()
  double run_time = 0;
  int elem_bytes = 0;
  cudaStream_t stream = nullptr;

 private:
  void check(cudaError_t e, const char* what) const;
  void check_err(const char* msg);
  void release();
  void layout(int elem);
  void alloc_accumulators();
  void fetch_cuts();
  void upload_table();

  bool laid_out = false, runner_ready = false, cuts_fetched = false;
  long long NP = 0, RES = 0, cut_total = 0;
  int tiles = 0;
  long long *d_exc64 = nullptr, *d_cap64 = nullptr, *d_c0 = nullptr;
  int* d_err = nullptr;
  unsigned long long* d_u64 = nullptr;
  void *d_res = nullptr, *d_exc = nullptr;
  int* d_h = nullptr;
  uint64_t* d_mask = nullptr;
  int* d_mark = nullptr;
  void* d_table = nullptr;       // lattice table of the batch-wide kernels
  long long* d_begins = nullptr;  // first node / packed node / packed edge per lattice
  bool table_ok = false;
  void* d_stage = nullptr;  // kept staging buffer of the packed fill
  size_t stage_bytes = 0;
  int h_err = 0;
  unsigned long long h_bound = 0;
  std::vector<int> host_cuts;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  PoolRunner runner;
};

}  // namespace lfg
