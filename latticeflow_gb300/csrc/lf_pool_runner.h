// Host runner of the instance pool (see lf_pool.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lf_pool.cuh"

namespace lfg {

struct LfError {
  int code;
  std::string msg;
};

struct Tuning {
  int tile_rows = 0;             // TB (2-d) / TB with TA = 4 (3-d); 0 = auto
  int sweeps = 0;                // local push/relabel rounds per tile visit
  int launches_per_relabel = 0;  // push/relabel passes between global relabels
  int height_slack = 0;          // heights above (BFS depth + slack) park until the next relabel
  int pass_chunk = 0;            // BFS / closure passes launched between host checks
  int tail_active = 0;           // active nodes at most for the tail step; 0 = 64, < 0 = off
  int max_epochs = 0;            // global relabels per solve at most; 0 = 1,000,000
  int tail_tree_nodes = 0;       // nodes of one tail-step tree at most; 0 = 65,536
  int pr_kernel = 0;             // push/relabel pass of a plain 2-d cut: 0 = TMA-staged
                                 // (40 registers), 1 = generic tile kernel, 2 = TMA-staged
                                 // with 32 registers, 3 = TMA-staged, one warp per tile
                                 // (one launch per pass)
  int bfs_kernel = 0;            // BFS pass of a single 2-d lattice: 0 = TMA-staged,
                                 // 1 = generic tile kernel
  int device_loops = 0;          // TMA-staged passes: 1 = device-side pass loops (CUDA
                                 // graphs with conditional nodes), 0 = one launch per
                                 // pass from the host
  int fill_kernel = 0;           // energy fill of device-resident arrays: 0 = gathered, one
                                 // lane per filling edge where K / 2 divides a warp (else
                                 // per node), 1 = gathered per node, 2 = scattered with
                                 // atomics (pinned host arrays read in place: always 2)
  int host_stage = 0;            // pinned host energies: 0 = read in place by the fill
                                 // kernel over the host link, 1 = copied into HBM by the
                                 // copy engine first (the SMs stay free for other solves
                                 // during the transfer)
};

struct SolveStats {
  long long epochs = 0, pr_launches = 0, bfs_passes = 0, reach_passes = 0, tail_steps = 0;
  unsigned long long tiles_processed = 0, bfs_tiles = 0;
};

// Profiling hooks of the owner (events around launches, launch counting).
struct ProfHooks {
  bool profiling = false;
  long long launches = 0;
  virtual void mark(int cat, bool end) = 0;
  virtual ~ProfHooks() {}
};

size_t pool_smem_head_bytes();

// Device scratch of the tail step (lf_pool_tail.cu): a BFS tree of at most
// `cap` nodes and `lvl_cap` levels per active node, at most max_active
// active nodes per step.
struct TailScratch {
  int* vis = nullptr;            // [NP] tree stamp per node
  long long* node = nullptr;     // [cap] tree nodes in BFS order
  int* par = nullptr;            // [cap] position of the parent
  unsigned char* dir = nullptr;  // [cap] direction parent -> node
  long long* dem = nullptr;      // [cap] demand / contribution
  long long* rem = nullptr;      // [cap] flow still to pass on
  int* lvl = nullptr;            // [lvl_cap + 2] first position of each level
  long long* list = nullptr;     // [max_active] active nodes
  unsigned* count = nullptr;     // active nodes found
  int cap = 0, lvl_cap = 0, max_active = 0;
};

template <typename T>
cudaError_t launch_pool_tail(const InstDesc* insts, const long long* nbase, int n, long long NP,
                             T* res, T* exc, const int* h, const uint64_t* kmask,
                             const TailScratch& s, int stamp0, unsigned long long* moved,
                             cudaStream_t st);

template <typename T>
size_t pool_pr_smem(int K, int NT, int HV) {
  return pool_smem_head_bytes() + size_t(K + 1) * NT * sizeof(T) + size_t(HV) * sizeof(int);
}

template <typename T>
cudaError_t launch_pool_pr(const PoolPR<T>& p, int KA, int KB, int threads, size_t smem,
                           bool single, int grid, cudaStream_t s);

// The TMA-staged 2-d passes (lf_pool_pr2d.cu): the kernel size they take a
// lattice with (4 or 8), or 0 when it does not fit them (not a pool of one,
// not a 2-d 3x3 neighbourhood in registry order; the push/relabel pass also
// takes no section mask).
int lattice2d_kernel_size(const InstDesc& I, bool single);
int pr2d_kernel_size(const PoolPR<int>& p, bool single);
// variant: 0 = at most 40 registers per thread, 1 = at most 32
cudaError_t launch_pool_pr2d(const PoolPR<int>& p, int K, int variant, unsigned long long* fault,
                             int tiles, cudaStream_t s);
cudaError_t launch_pool_bfs2d(const PoolBFS& p, int K, unsigned long long* fault, int tiles,
                              cudaStream_t s);

// The TMA-staged 3-d push/relabel pass (lf_pool_pr3d.cu): the kernel size it
// takes a lattice with (6, 18 or 26: a pool of one 3-d lattice, radius-1
// neighbourhood, 4-plane tiles of 2, 4 or 8 rows whose two stage buffers fit
// shared memory, no section mask), else 0.
int pr3d_kernel_size(const PoolPR<int>& p, bool single);
cudaError_t launch_pool_pr3d(const PoolPR<int>& p, int K, unsigned long long* fault, int tiles,
                             cudaStream_t s);
// The TMA-staged 3-d BFS pass: the kernel size it takes a lattice with (a
// pool of one 3-d lattice, radius-1 neighbourhood, 4-plane tiles of 2, 4 or
// 8 rows; any capacity type), else 0.
int lattice3d_kernel_size(const InstDesc& I, bool single);
cudaError_t launch_pool_bfs3d(const PoolBFS& p, int K, unsigned long long* fault, int tiles,
                              cudaStream_t s);

// Device-side loops of those passes (one CUDA graph launch runs passes until
// the next tile list is empty or `cap` passes ran; ctl: two device words the
// loop keeps its list index and pass count in; passes: incremented per pass;
// overflow: set when the cap ends a loop that still had tiles queued).  A
// PassLoop caches the instantiated graph for the arrays it was built for.
struct PassLoop;
PassLoop* pass_loop_new();
void pass_loop_free(PassLoop* L);
cudaError_t loop_pool_pr2d(PassLoop* L, const PoolPR<int>& p, int K, int variant,
                           unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                           unsigned long long* passes, cudaStream_t s);
cudaError_t loop_pool_bfs2d(PassLoop* L, const PoolBFS& p, int K, unsigned long long* fault,
                            int tiles, int* ctl, unsigned cap, unsigned long long* passes,
                            unsigned long long* overflow, cudaStream_t s);

// The push/relabel pass for 64-bit capacities with section masks (parametric
// and TV section solves) on one 2-d lattice: pr2d64_kernel_size gives the
// kernel size it takes (0 when the pass does not fit it); pr2d64 runs one
// launch (L null) or a device-side loop of passes.
int pr2d64_kernel_size(const PoolPR<long long>& p, bool single);
cudaError_t pr2d64(PassLoop* L, const PoolPR<long long>& p, int K, unsigned long long* fault,
                   int tiles, int* ctl, unsigned cap, unsigned long long* passes, cudaStream_t s);

// The same passes over a pool of many 2-d lattices (Full2d_4 / Full2d_8 mixed,
// one tile height): pool2d_tile_rows gives that tile height, or 0 when the
// pool does not fit them.  The tensor maps of every lattice live in device
// memory (PoolMaps, rebuilt when the arrays move).  L: null for one launch
// (p.cur), else a device-side loop of passes as above.
struct PoolMaps;
PoolMaps* pool_maps_new();
void pool_maps_free(PoolMaps* m);
int pool2d_tile_rows(const std::vector<InstDesc>& insts);
const void* pool_maps_pr(PoolMaps* M, const std::vector<InstDesc>& insts, int* res, int* exc,
                         int* h, cudaStream_t s);
const void* pool_maps_bfs(PoolMaps* M, const std::vector<InstDesc>& insts, int* h,
                          const uint64_t* mask, cudaStream_t s);
cudaError_t pool_pr2d(PassLoop* L, const void* maps, const PoolPR<int>& p, int TB, int variant,
                      unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                      unsigned long long* passes, cudaStream_t s);
cudaError_t pool_bfs2d(PassLoop* L, const void* maps, const PoolBFS& p, int TB,
                       unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                       unsigned long long* passes, unsigned long long* overflow, cudaStream_t s);

cudaError_t launch_pool_bfs(const PoolBFS& p, int KA, int KB, bool single, int grid, int threads,
                            size_t smem, cudaStream_t s);
cudaError_t launch_pool_reach(const PoolReach& p, int KA, int KB, bool single, int grid,
                              int threads, size_t smem, cudaStream_t s);

template <typename T>
cudaError_t pool_init_heights(const InstDesc* insts, const long long* nbase, int n, long long NP,
                              const T* exc, const uint64_t* kmask, int* h, cudaStream_t s);
template <typename T>
cudaError_t pool_mask(const InstDesc* insts, const long long* nbase, int n, long long NP,
                      const T* res, const uint64_t* kmask, uint64_t* mask, cudaStream_t s);
cudaError_t pool_queue_all(const InstDesc* insts, const int* tile_inst, int tiles, TileQueue q,
                           cudaStream_t s);
template <typename T>
cudaError_t pool_active(const InstDesc* insts, const long long* nbase, int n, long long NP,
                        const T* exc, const int* h, TileQueue q, unsigned long long* cnt,
                        unsigned* hmx, cudaStream_t s);
cudaError_t pool_update(InstDesc* insts, int n, const unsigned long long* cnt, const unsigned* hmx,
                        long long cap, int slack, unsigned long long* total, cudaStream_t s);
cudaError_t pool_reset(InstDesc* insts, int n, cudaStream_t s);
template <typename T>
cudaError_t pool_init_marks(const InstDesc* insts, const long long* nbase, int n, long long NP,
                            const T* exc, int* mark, cudaStream_t s);
cudaError_t pool_queue_active(const InstDesc* insts, const int* tile_inst, int tiles, TileQueue q,
                              cudaStream_t s);
template <typename T>
cudaError_t pool_sum_pos(const InstDesc* insts, const long long* nbase, int n, long long NP,
                         const T* exc, long long* sums, cudaStream_t s);

class PoolRunner {
 public:
  ~PoolRunner();
  void setup(const std::vector<InstDesc>& insts, cudaStream_t s);
  void set_active(const std::vector<int>& act);
  template <typename T>
  void maxflow(T* res, T* exc, int* h, uint64_t* mask, const uint64_t* kmask, int* mark,
               SolveStats& stats, bool sets);
  template <typename T> void stuck_excess(const T* exc, long long* out_host);

  Tuning tune;
  ProfHooks* hooks = nullptr;
  std::vector<InstDesc> host;
  int n = 0, tiles = 0;
  long long NP = 0;
  InstDesc* d_inst = nullptr;

 private:
  template <typename T>
  void maxflow_epochs(T* res, T* exc, int* h, uint64_t* mask, const uint64_t* kmask, int* mark,
                      SolveStats& stats, bool sets);
  template <typename T>
  void global_relabel(const T* res, const T* exc, int* h, uint64_t* mask, const uint64_t* kmask,
                      SolveStats& stats);
  template <typename T> unsigned long long activate(const T* exc, const int* h);
  template <typename T> void reach(const T* exc, const uint64_t* mask, int* mark, SolveStats& stats);
  void prep_pass(int cur);
  void drain_queue();
  void sync_read(void* dst, const void* src, size_t bytes);
  void mark(int cat, bool end);
  void count_launch();
  void check(cudaError_t e, const char* what);
  void release();

  cudaStream_t stream = nullptr;
  long long* d_nbase = nullptr;
  int* d_tile_inst = nullptr;
  TileQueue q{{nullptr, nullptr}, {nullptr, nullptr}, nullptr};
  unsigned long long* d_cnt = nullptr;
  unsigned* d_hmx = nullptr;
  long long* d_sum = nullptr;
  int* d_flag = nullptr;
  unsigned long long* d_counters = nullptr;  // [0] pr tiles, [1] bfs tiles, [2] tail moved,
                                             // [3] active total, [4] staging fault, [5] bfs
                                             // passes and [6] pr passes of device-side loops,
                                             // [7] a device-side BFS loop hit its cap
  int* d_ctl = nullptr;                      // control words of the device-side loops
  PassLoop* loop_pr = nullptr;
  PassLoop* loop_bfs = nullptr;
  PoolMaps* pool_maps = nullptr;  // tensor maps of the pool passes (batches)
  void* h_pin = nullptr;
  int threads = 1, hv_max = 0;
  int ka = 0, kb = 0;  // kernel sizes present in the pool
  TailScratch tail;
  int tail_stamp = 1;
  void alloc_tail();
  void free_tail();
  int grid_bfs = 0, grid_reach = 0;
};

}  // namespace lfg
