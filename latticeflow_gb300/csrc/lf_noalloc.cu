// Binary cut of one small 2-d lattice without allocating any memory.
//
// Who needs it: callers that may not allocate device memory at all while they
// run — code executing inside another framework's memory budget or pool,
// real-time or embedded hosts that forbid allocation after start-up, and
// plugins whose host process owns every allocation.  They pass device
// buffers for the capacities and the results; every intermediate array of the
// solve (accumulators, residual planes, heights, masks, marks, tile queues,
// counters) lives in one file-scope device array, sized for at most
// kNoAllocMaxNodes padded nodes.
//
// The array is shared by every call in the process and keeps the last call's
// contents: each call clears what must start at zero.  Two calls whose GPU
// work overlapped would race on it; this entry point holds a process-wide lock
// for the whole call and synchronises the caller's stream before it returns,
// so calls from one process never overlap.
//
// Host code cannot use the array's name as a device address, so every call
// looks the address up (cudaGetSymbolAddress) with the caller's device
// current.  The first call on a device also loads the array's module there:
// make that first call before any stream capture.  Looking the address up on
// every call, instead of caching it, keeps it right after a cudaDeviceReset
// or any other change of the device's primary context.
#include <climits>
#include <cstring>
#include <mutex>

#include "../../include/latticeflow_gpu.h"
#include "lf_engine.h"
#include "lf_pool_runner.h"

namespace lfg {

// 65,536 padded nodes (e.g. 256 x 256; padding rounds both sides up to 32),
// Full2d_4 or Full2d_8 (K <= 8): 8.5 MiB of device memory per GPU.
constexpr long long kNoAllocMaxNodes = 65536;
constexpr int kNoAllocMaxK = 8;
constexpr size_t kNoAllocScratchBytes = size_t(8) * 1024 * 1024 + 512 * 1024;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_noalloc_lock;

__global__ void k_noalloc_finish(const long long* supply, const long long* stuck,
                                 const long long* c0, int64_t* out) {
  out[0] = supply[0] - stuck[0];
  out[1] = c0[0] - stuck[0];
}

struct Carve {
  unsigned char* p;
  size_t used, cap;
  template <class T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
    if (used + bytes > cap) throw LfError{LF_ERR_RANGE, "no-allocation scratch exhausted"};
    T* r = reinterpret_cast<T*>(p + used);
    used += bytes;
    return r;
  }
};

void ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw LfError{LF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

template <class T>
void read_back(T* host, const T* dev, cudaStream_t s) {
  ok(cudaMemcpyAsync(host, dev, sizeof(T), cudaMemcpyDeviceToHost, s), "memcpy");
  ok(cudaStreamSynchronize(s), "stream sync");
}

}  // namespace

namespace {

void cut_2d_noalloc_locked(const KernelDef* kd, size_t nx, size_t ny, const int32_t* src,
                           const int32_t* snk, const int32_t* edge, int32_t* cut,
                           int64_t* flow_energy, cudaStream_t s);

}  // namespace

int cut_2d_noalloc(const char* kernel, size_t nx, size_t ny, const int32_t* src,
                   const int32_t* snk, const int32_t* edge, int32_t* cut, int64_t* flow_energy,
                   cudaStream_t s) {
  const KernelDef* kd = kernel ? find_kernel(kernel) : nullptr;
  if (!kd) throw LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                              (kernel ? kernel : "(null)")};
  if (kd->nd != 2 || kd->K > kNoAllocMaxK)
    throw LfError{LF_ERR_SHAPE, "the no-allocation cut takes 2-d kernels of at most 8 neighbours"};
  if (!src || !snk || !edge || !cut || !flow_energy)
    throw LfError{LF_ERR_INVALID, "null argument"};
  if (nx == 0 || ny == 0) throw LfError{LF_ERR_SHAPE, "empty lattice"};
  if (nx > (size_t)INT_MAX / 2 || ny > (size_t)INT_MAX / 2)
    throw LfError{LF_ERR_RANGE, "lattice extent too large"};
  std::lock_guard<std::mutex> guard(g_noalloc_lock);
  try {
    cut_2d_noalloc_locked(kd, nx, ny, src, snk, edge, cut, flow_energy, s);
  } catch (...) {
    // work of this call that is still queued on `s` uses the shared array:
    // let it finish before the lock lets the next call in
    cudaStreamSynchronize(s);
    throw;
  }
  return LF_OK;
}

namespace {

void cut_2d_noalloc_locked(const KernelDef* kd, size_t nx, size_t ny, const int32_t* src,
                           const int32_t* snk, const int32_t* edge, int32_t* cut,
                           int64_t* flow_energy, cudaStream_t s) {
  const Stencil st = make_stencil(kd);
  Geo g{};
  const size_t dims[2] = {nx, ny};
  lattice_geometry(2, dims, st, 4, 0, g);
  if (g.NP > kNoAllocMaxNodes)
    throw LfError{LF_ERR_RANGE, "lattice too large for the no-allocation cut: " +
                                    std::to_string(g.NP) + " padded nodes (sides rounded up to 32), "
                                    "at most " + std::to_string(kNoAllocMaxNodes)};
  const long long N = (long long)nx * (long long)ny;
  const int K = st.K;

  void* base = nullptr;  // the array's address on the current device
  {
    cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
    if (e != cudaSuccess || !base)
      throw LfError{LF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
  }
  Carve c{static_cast<unsigned char*>(base), 0, kNoAllocScratchBytes};
  long long* exc64 = c.take<long long>(g.NP);
  long long* cap64 = c.take<long long>((size_t)K * g.NP);
  int* res = c.take<int>((size_t)K * g.NP);
  int* exc = c.take<int>(g.NP);
  int* h = c.take<int>(g.NP);
  uint64_t* mask = c.take<uint64_t>(g.NP);
  int* mark = c.take<int>(g.NP);
  InstDesc* d_inst = c.take<InstDesc>(1);
  long long* nbase = c.take<long long>(2);
  int* tile_inst = c.take<int>(g.ntiles);
  TileQueue q;
  q.flag[0] = c.take<int>(g.ntiles);
  q.flag[1] = c.take<int>(g.ntiles);
  q.list[0] = c.take<int>(g.ntiles);
  q.list[1] = c.take<int>(g.ntiles);
  q.ctr = c.take<unsigned>(4);
  // small counters, one slot each: 0 c0, 1 err, 2 bound, 3 active count,
  // 4 hmax, 5 total active, 6 changed flag, 7 supply, 8 stuck, 9..12 tile counters
  long long* small = c.take<long long>(16);
  long long* c0 = small + 0;
  int* err = reinterpret_cast<int*>(small + 1);
  unsigned long long* bound = reinterpret_cast<unsigned long long*>(small + 2);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(small + 3);
  unsigned* hmx = reinterpret_cast<unsigned*>(small + 4);
  unsigned long long* total = reinterpret_cast<unsigned long long*>(small + 5);
  int* changed = reinterpret_cast<int*>(small + 6);
  long long* supply = small + 7;
  long long* stuck = small + 8;
  unsigned long long* counters = reinterpret_cast<unsigned long long*>(small + 9);

  // everything that must start at zero
  ok(cudaMemsetAsync(exc64, 0, g.NP * sizeof(long long), s), "memset");
  ok(cudaMemsetAsync(cap64, 0, (size_t)K * g.NP * sizeof(long long), s), "memset");
  ok(cudaMemsetAsync(tile_inst, 0, g.ntiles * sizeof(int), s), "memset");
  ok(cudaMemsetAsync(q.flag[0], 0, g.ntiles * sizeof(int), s), "memset");
  ok(cudaMemsetAsync(q.flag[1], 0, g.ntiles * sizeof(int), s), "memset");
  ok(cudaMemsetAsync(small, 0, 16 * sizeof(long long), s), "memset");
  InstDesc I{};
  I.g = g;
  I.st = st;
  I.plane = g.NP;
  I.hmax = kHInf - 2;
  I.active = 1;
  const long long nb[2] = {0, g.NP};
  ok(cudaMemcpyAsync(d_inst, &I, sizeof(InstDesc), cudaMemcpyHostToDevice, s), "memcpy");
  ok(cudaMemcpyAsync(nbase, nb, sizeof(nb), cudaMemcpyHostToDevice, s), "memcpy");

  // fill (capacity form) and the 32-bit range check
  ok(launch_fill_caps(g, st, 2, N, src, snk, edge, exc64, cap64, c0, err, 0, s), "fill");
  ok(launch_range_bound(g, st, exc64, cap64, bound, s), "range bound");
  int h_err = 0;
  unsigned long long h_bound = 0;
  read_back(&h_err, err, s);
  read_back(&h_bound, bound, s);
  if (h_err) throw LfError{LF_ERR_RANGE, "capacities must be non-negative"};
  if (h_bound >= (unsigned long long)INT_MAX)
    throw LfError{LF_ERR_RANGE, "capacities too large for the 32-bit no-allocation cut"};
  ok(launch_convert<int>((long long)K * g.NP, cap64, res, s), "convert");
  ok(launch_convert<int>(g.NP, exc64, exc, s), "convert");
  ok(pool_sum_pos<int>(d_inst, nbase, 1, g.NP, exc, supply, s), "sum");

  // the solve: the pool runner's epoch loop for a pool of one
  const int threads = g.TA * g.TB * g.TC;
  const int HV = (g.TA + 2 * st.HA) * (g.TB + 2 * st.HB) * (g.TC + 2 * st.HC);
  const size_t smem_graph = pool_smem_head_bytes() + size_t(HV) * sizeof(int);
  const size_t smem_reach = pool_smem_head_bytes() + size_t(threads) * sizeof(int);
  const size_t smem_pr = pool_pr_smem<int>(K, threads, HV);
  const int grid = g.ntiles;
  const int M = 4, R = 4, slack = 16, chunk = 4;
  const long long pass_cap = 4LL * g.ntiles + 64;
  ok(pool_reset(d_inst, 1, s), "reset");
  for (int epoch = 0;; ++epoch) {
    if (epoch > 20000) throw LfError{LF_ERR_NO_CONVERGENCE, "push-relabel did not converge"};
    // global relabel
    ok(pool_init_heights<int>(d_inst, nbase, 1, g.NP, exc, nullptr, h, s), "heights");
    ok(pool_mask<int>(d_inst, nbase, 1, g.NP, res, nullptr, mask, s), "mask");
    ok(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), s), "memset");
    ok(pool_queue_all(d_inst, tile_inst, g.ntiles, q, s), "queue");
    int cur = 0;
    for (long long pass = 0;;) {
      if (pass > pass_cap) throw LfError{LF_ERR_NO_CONVERGENCE, "global relabel did not converge"};
      for (int k = 0; k < chunk; ++k, ++pass) {
        ok(cudaMemsetAsync(q.ctr + (cur ? 0 : 2), 0, 2 * sizeof(unsigned), s), "memset");
        ok(cudaMemsetAsync(changed, 0, sizeof(int), s), "memset");
        PoolBFS p{I, d_inst, tile_inst, h, mask, q, cur, 64, changed, counters};
        ok(launch_pool_bfs(p, K, K, true, grid, threads, smem_graph, s), "bfs");
        cur ^= 1;
      }
      int h_changed = 0;
      read_back(&h_changed, changed, s);
      if (!h_changed) break;
    }
    // active nodes and the epoch height cap
    ok(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), s), "memset");
    ok(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s), "memset");
    ok(cudaMemsetAsync(hmx, 0, sizeof(unsigned), s), "memset");
    ok(cudaMemsetAsync(total, 0, sizeof(unsigned long long), s), "memset");
    ok(pool_active<int>(d_inst, nbase, 1, g.NP, exc, h, q, cnt, hmx, s), "active");
    ok(pool_update(d_inst, 1, cnt, hmx, (long long)kHInf - 2, slack, total, s), "update");
    unsigned long long h_total = 0;
    read_back(&h_total, total, s);
    if (h_total == 0) break;
    read_back(&I, d_inst, s);
    cur = 0;
    for (int l = 0; l < M; ++l) {
      ok(cudaMemsetAsync(q.ctr + (cur ? 0 : 2), 0, 2 * sizeof(unsigned), s), "memset");
      PoolPR<int> p{I, d_inst, tile_inst, res, exc, h, nullptr, q, cur, R, counters};
      ok(launch_pool_pr<int>(p, K, K, threads, smem_pr, true, grid, s), "push-relabel");
      cur ^= 1;
    }
    ok(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), s), "memset");
    ok(cudaMemsetAsync(q.flag[0], 0, g.ntiles * sizeof(int), s), "memset");
    ok(cudaMemsetAsync(q.flag[1], 0, g.ntiles * sizeof(int), s), "memset");
    I.done = 0;
  }
  // minimal on-set: forward closure of the excess nodes
  ok(pool_init_marks<int>(d_inst, nbase, 1, g.NP, exc, mark, s), "marks");
  ok(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), s), "memset");
  ok(pool_queue_active(d_inst, tile_inst, g.ntiles, q, s), "queue");
  int cur = 0;
  for (long long pass = 0;;) {
    if (pass > pass_cap) throw LfError{LF_ERR_NO_CONVERGENCE, "cut-set closure did not converge"};
    for (int k = 0; k < chunk; ++k, ++pass) {
      ok(cudaMemsetAsync(q.ctr + (cur ? 0 : 2), 0, 2 * sizeof(unsigned), s), "memset");
      ok(cudaMemsetAsync(changed, 0, sizeof(int), s), "memset");
      PoolReach p{I, d_inst, tile_inst, mark, mask, q, cur, 256, changed};
      ok(launch_pool_reach(p, K, K, true, grid, threads, smem_reach, s), "closure");
      cur ^= 1;
    }
    int h_changed = 0;
    read_back(&h_changed, changed, s);
    if (!h_changed) break;
  }
  ok(pool_sum_pos<int>(d_inst, nbase, 1, g.NP, exc, stuck, s), "sum");
  k_noalloc_finish<<<1, 1, 0, s>>>(supply, stuck, c0, flow_energy);
  ok(cudaGetLastError(), "finish");
  ok(launch_extract_cuts(g, 2, N, mark, h, cut, nullptr, s), "extract cut");
  ok(cudaStreamSynchronize(s), "stream sync");
}

}  // namespace

}  // namespace lfg
