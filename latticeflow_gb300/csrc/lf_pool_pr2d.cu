// Launchers of the TMA-staged 2-d passes (push/relabel, lf_pool_pr2d.cuh; BFS
// relabel, lf_pool_bfs2d.cuh): tensor maps of the lattice's arrays, launch
// shapes, and the test of whether a pass can take these kernels.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "lf_pool_bfs2d.cuh"
#include "lf_pool_pr2d.cuh"
#include "lf_pool_launch.cuh"
#include "lf_pool_runner.h"
#include "lf_tensor_map.h"

namespace lfg {

namespace {

template <int K>
bool stencil_is(const Stencil& st) {
  if (st.K != K) return false;
  for (int k = 0; k < K; ++k)
    if (st.da[k] != 0 || st.db[k] != s2_db<K>(k) || st.dc[k] != s2_dc<K>(k)) return false;
  return true;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() { return tensor_map_encoder(); }

bool encode(CUtensorMap* m, void* base, int rank, const cuuint64_t* dims,
            const cuuint64_t* strides, const cuuint32_t* box,
            CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_INT32) {
  return encode_tensor_map(m, base, rank, dims, strides, box, type);
}

// Tensor maps of the last lattice this host thread launched for (a solve
// launches its passes on the same arrays).
struct MapCache {
  const void *res = nullptr, *exc = nullptr, *h = nullptr;
  int Cp = 0, Bp = 0, K = 0, TB = 0;
  long long NP = 0;
  PR2dMaps maps;
};

bool maps_for(const PoolPR<int>& p, int K, int TB, PR2dMaps& out) {
  thread_local MapCache c;
  const Geo& g = p.inst0.g;
  if (c.res == p.res && c.exc == p.exc && c.h == p.h && c.Cp == g.Cp && c.Bp == g.Bp &&
      c.NP == g.NP && c.K == K && c.TB == TB) {
    out = c.maps;
    return true;
  }
  PR2dMaps m;
  const cuuint64_t d3[3] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)K};
  const cuuint64_t s3[2] = {(cuuint64_t)g.Cp * 4, (cuuint64_t)g.NP * 4};
  const cuuint32_t b3[3] = {32, (cuuint32_t)TB, (cuuint32_t)K};
  const cuuint64_t d2[2] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp};
  const cuuint64_t s2[1] = {(cuuint64_t)g.Cp * 4};
  const cuuint32_t be[2] = {32, (cuuint32_t)TB};
  const cuuint32_t bh[2] = {(cuuint32_t)kPr2dHaloW, (cuuint32_t)(TB + 2)};
  if (!encode(&m.res, p.res, 3, d3, s3, b3) || !encode(&m.exc, p.exc, 2, d2, s2, be) ||
      !encode(&m.h, p.h, 2, d2, s2, bh))
    return false;
  c.res = p.res; c.exc = p.exc; c.h = p.h;
  c.Cp = g.Cp; c.Bp = g.Bp; c.NP = g.NP; c.K = K; c.TB = TB;
  c.maps = m;
  out = m;
  return true;
}

template <int K, int TB, int REGS>
void* kt_setup(int& grid) {
  using Ly = PR2dLayout<K, TB>;
  auto kern = k_pool_pr2d<K, TB, REGS>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

template <int K, int TB, int REGS>
cudaError_t launch_kt(const PR2dMaps& maps, const PoolPR<int>& p, unsigned long long* fault,
                      int tiles, cudaStream_t s) {
  using Ly = PR2dLayout<K, TB>;
  int grid = 0;
  kt_setup<K, TB, REGS>(grid);
  k_pool_pr2d<K, TB, REGS><<<std::max(1, std::min(grid, tiles)), Ly::NT, Ly::smem_bytes, s>>>(
      maps, p, fault, nullptr);
  return cudaGetLastError();
}

// The warp-per-tile variant: 4 warps per block, each with its own stage
// buffers.
constexpr int kPr2dWarps = 4;

template <int K, int TB>
size_t kt_warp_smem() {
  return size_t(kPr2dWarps) * PR2dWarpLayout<K, TB>::per_warp + 128;
}

template <int K, int TB>
void* kt_warp_setup(int& grid) {
  auto kern = k_pool_pr2d_warp<K, TB, kPr2dWarps>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(kt_warp_smem<K, TB>()));
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, kPr2dWarps * 32, kt_warp_smem<K, TB>());
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

template <int K, int TB>
cudaError_t launch_kt_warp(const PR2dMaps& maps, const PoolPR<int>& p, unsigned long long* fault,
                           int tiles, cudaStream_t s) {
  int grid = 0;
  kt_warp_setup<K, TB>(grid);
  const int need = (tiles + kPr2dWarps - 1) / kPr2dWarps;
  k_pool_pr2d_warp<K, TB, kPr2dWarps><<<std::max(1, std::min(grid, need)), kPr2dWarps * 32,
                                        kt_warp_smem<K, TB>(), s>>>(maps, p, fault);
  return cudaGetLastError();
}

// Tensor maps of the 64-bit pass with section masks, cached per host thread.
struct MapCache64 {
  const void *res = nullptr, *exc = nullptr, *h = nullptr, *km = nullptr;
  int Cp = 0, Bp = 0, K = 0, TB = 0;
  long long NP = 0;
  PR2dMaps64 maps;
};

bool maps64_for(const PoolPR<long long>& p, int K, int TB, PR2dMaps64& out) {
  thread_local MapCache64 c;
  const Geo& g = p.inst0.g;
  if (c.res == p.res && c.exc == p.exc && c.h == p.h && c.km == p.kmask && c.Cp == g.Cp &&
      c.Bp == g.Bp && c.NP == g.NP && c.K == K && c.TB == TB) {
    out = c.maps;
    return true;
  }
  PR2dMaps64 m;
  const cuuint64_t d3[3] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)K};
  const cuuint64_t s3[2] = {(cuuint64_t)g.Cp * 8, (cuuint64_t)g.NP * 8};
  const cuuint32_t b3[3] = {32, (cuuint32_t)TB, (cuuint32_t)K};
  const cuuint64_t d2[2] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp};
  const cuuint64_t s8[1] = {(cuuint64_t)g.Cp * 8};
  const cuuint64_t s4[1] = {(cuuint64_t)g.Cp * 4};
  const cuuint32_t be[2] = {32, (cuuint32_t)TB};
  const cuuint32_t bh[2] = {(cuuint32_t)kPr2dHaloW, (cuuint32_t)(TB + 2)};
  if (!encode(&m.res, p.res, 3, d3, s3, b3, CU_TENSOR_MAP_DATA_TYPE_INT64) ||
      !encode(&m.exc, p.exc, 2, d2, s8, be, CU_TENSOR_MAP_DATA_TYPE_INT64) ||
      !encode(&m.h, p.h, 2, d2, s4, bh) ||
      !encode(&m.km, const_cast<uint64_t*>(p.kmask), 2, d2, s8, be, CU_TENSOR_MAP_DATA_TYPE_UINT64))
    return false;
  c.res = p.res; c.exc = p.exc; c.h = p.h; c.km = p.kmask;
  c.Cp = g.Cp; c.Bp = g.Bp; c.NP = g.NP; c.K = K; c.TB = TB;
  c.maps = m;
  out = m;
  return true;
}

template <int K, int TB>
void* kt64_setup(int& grid) {
  using Ly = PR2dLayout64<K, TB>;
  auto kern = k_pool_pr2d64<K, TB>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

// Tensor maps of the BFS pass (heights with halo, masks), cached like the
// push/relabel ones.
struct BfsMapCache {
  const void *h = nullptr, *mask = nullptr;
  int Cp = 0, Bp = 0, TB = 0;
  BFS2dMaps maps;
};

bool bfs_maps_for(const PoolBFS& p, int TB, BFS2dMaps& out) {
  thread_local BfsMapCache c;
  const Geo& g = p.inst0.g;
  if (c.h == p.h && c.mask == p.mask && c.Cp == g.Cp && c.Bp == g.Bp && c.TB == TB) {
    out = c.maps;
    return true;
  }
  BFS2dMaps m;
  const cuuint64_t d2[2] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp};
  const cuuint64_t s4[1] = {(cuuint64_t)g.Cp * 4};
  const cuuint64_t s8[1] = {(cuuint64_t)g.Cp * 8};
  const cuuint32_t bh[2] = {(cuuint32_t)kPr2dHaloW, (cuuint32_t)(TB + 2)};
  const cuuint32_t bm[2] = {32, (cuuint32_t)TB};
  if (!encode(&m.h, p.h, 2, d2, s4, bh) ||
      !encode(&m.mask, const_cast<uint64_t*>(p.mask), 2, d2, s8, bm, CU_TENSOR_MAP_DATA_TYPE_UINT64))
    return false;
  c.h = p.h; c.mask = p.mask; c.Cp = g.Cp; c.Bp = g.Bp; c.TB = TB;
  c.maps = m;
  out = m;
  return true;
}

template <int K, int TB>
void* bfs_kt_setup(int& grid) {
  using Ly = BFS2dLayout<TB>;
  auto kern = k_pool_bfs2d<K, TB>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

template <int K, int TB>
cudaError_t launch_bfs_kt(const BFS2dMaps& maps, const PoolBFS& p, unsigned long long* fault,
                          int tiles, cudaStream_t s) {
  using Ly = BFS2dLayout<TB>;
  int grid = 0;
  bfs_kt_setup<K, TB>(grid);
  k_pool_bfs2d<K, TB><<<std::max(1, std::min(grid, tiles)), Ly::NT, Ly::smem_bytes, s>>>(
      maps, p, fault, nullptr);
  return cudaGetLastError();
}

// ------------------------------------------------------ device-side pass loop
//
// A CUDA graph: a memset node zeroes the loop's control words, then a while
// node runs [pass kernel, k_pass_ctl] until k_pass_ctl finds the list of the
// next pass empty or the pass cap reached.  k_pass_ctl does between two
// passes what the host does between two launches (zero the count of the list
// just consumed, swap the lists) and counts the passes.

// ctl[0]: list the next pass consumes, ctl[1]: passes run in this loop
__global__ void k_pass_ctl(TileQueue q, int* ctl, unsigned cap, unsigned long long* passes,
                           unsigned long long* overflow, cudaGraphConditionalHandle h) {
  const int c = ctl[0], nx = c ^ 1;
  q.ctr[q_count_idx(c)] = 0;  // consumed; the next pass fills it
  q.ctr[q_head_idx(nx)] = 0;
  const unsigned n = q.ctr[q_count_idx(nx)];
  const unsigned run = (unsigned)ctl[1] + 1;
  ctl[1] = (int)run;
  ctl[0] = nx;
  *passes += 1;
  if (n > 0 && run >= cap && overflow) *overflow = 1;
  cudaGraphSetConditional(h, (n > 0 && run < cap) ? 1u : 0u);
}

template <int TB, int REGS>
void* kt_pool_setup(int& grid) {
  using Ly = PR2dPoolLayout<TB>;
  auto kern = k_pool_pr2d_pool<TB, REGS>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

template <int TB>
void* bfs_kt_pool_setup(int& grid) {
  using Ly = BFS2dLayout<TB>;
  auto kern = k_pool_bfs2d_pool<TB>;
  static std::mutex mu;
  static int cap = 0;
  std::lock_guard<std::mutex> lk(mu);
  if (!cap) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
  }
  grid = cap;
  return reinterpret_cast<void*>(kern);
}

}  // namespace

// Tensor maps of every lattice of a pool, in device memory: three per
// lattice for the push/relabel pass (residual planes, excess, heights; int32
// arrays) and two for the BFS pass (heights, masks).  Rebuilt when the
// arrays move.
struct PoolMaps {
  void* d_pr = nullptr;
  void* d_bfs = nullptr;
  size_t pr_n = 0, bfs_n = 0;
  const void* pr_key[3] = {nullptr, nullptr, nullptr};
  const void* bfs_key[2] = {nullptr, nullptr};
  ~PoolMaps() {
    cudaFree(d_pr);
    cudaFree(d_bfs);
  }
};

PoolMaps* pool_maps_new() { return new PoolMaps(); }
void pool_maps_free(PoolMaps* m) { delete m; }

int pool2d_tile_rows(const std::vector<InstDesc>& insts) {
  if (insts.size() < 2 || !encode_fn()) return 0;
  const int TB = insts[0].g.TB;
  if (TB != 4 && TB != 8 && TB != 16 && TB != 32) return 0;
  for (const InstDesc& I : insts) {
    if (I.g.TB != TB || I.g.TA != 1 || I.g.A != 1 || I.g.Ap != 1 || I.g.TC != 32) return 0;
    if (I.g.Cp % 32 || I.g.Bp % TB) return 0;
    if (!stencil_is<4>(I.st) && !stencil_is<8>(I.st)) return 0;
    // 16-byte aligned bases and plane strides for the tensor maps
    if (I.node_base % 4 || I.res_base % 4 || I.plane % 4) return 0;
  }
  return TB;
}

const void* pool_maps_pr(PoolMaps* M, const std::vector<InstDesc>& insts, int* res, int* exc,
                         int* h, cudaStream_t s) {
  if (M->d_pr && M->pr_key[0] == res && M->pr_key[1] == exc && M->pr_key[2] == h &&
      M->pr_n == insts.size())
    return M->d_pr;
  std::vector<CUtensorMap> maps(3 * insts.size());
  for (size_t i = 0; i < insts.size(); ++i) {
    const InstDesc& I = insts[i];
    const Geo& g = I.g;
    const int TB = g.TB;
    const cuuint64_t d3[3] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)I.st.K};
    const cuuint64_t s3[2] = {(cuuint64_t)g.Cp * 4, (cuuint64_t)I.plane * 4};
    const cuuint32_t b3[3] = {32, (cuuint32_t)TB, (cuuint32_t)I.st.K};
    const cuuint64_t d2[2] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp};
    const cuuint64_t s2[1] = {(cuuint64_t)g.Cp * 4};
    const cuuint32_t be[2] = {32, (cuuint32_t)TB};
    const cuuint32_t bh[2] = {(cuuint32_t)kPr2dHaloW, (cuuint32_t)(TB + 2)};
    if (!encode(&maps[3 * i], res + I.res_base, 3, d3, s3, b3) ||
        !encode(&maps[3 * i + 1], exc + I.node_base, 2, d2, s2, be) ||
        !encode(&maps[3 * i + 2], h + I.node_base, 2, d2, s2, bh))
      return nullptr;
  }
  cudaFree(M->d_pr);
  M->d_pr = nullptr;
  const size_t bytes = maps.size() * sizeof(CUtensorMap);
  if (cudaMalloc(&M->d_pr, bytes) != cudaSuccess) return nullptr;
  if (cudaMemcpyAsync(M->d_pr, maps.data(), bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return nullptr;
  M->pr_key[0] = res; M->pr_key[1] = exc; M->pr_key[2] = h;
  M->pr_n = insts.size();
  return M->d_pr;
}

const void* pool_maps_bfs(PoolMaps* M, const std::vector<InstDesc>& insts, int* h,
                          const uint64_t* mask, cudaStream_t s) {
  if (M->d_bfs && M->bfs_key[0] == h && M->bfs_key[1] == mask && M->bfs_n == insts.size())
    return M->d_bfs;
  std::vector<CUtensorMap> maps(2 * insts.size());
  for (size_t i = 0; i < insts.size(); ++i) {
    const InstDesc& I = insts[i];
    const Geo& g = I.g;
    const int TB = g.TB;
    const cuuint64_t d2[2] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp};
    const cuuint64_t s4[1] = {(cuuint64_t)g.Cp * 4};
    const cuuint64_t s8[1] = {(cuuint64_t)g.Cp * 8};
    const cuuint32_t bh[2] = {(cuuint32_t)kPr2dHaloW, (cuuint32_t)(TB + 2)};
    const cuuint32_t bm[2] = {32, (cuuint32_t)TB};
    if (!encode(&maps[2 * i], h + I.node_base, 2, d2, s4, bh) ||
        !encode(&maps[2 * i + 1], const_cast<uint64_t*>(mask) + I.node_base, 2, d2, s8, bm,
                CU_TENSOR_MAP_DATA_TYPE_UINT64))
      return nullptr;
  }
  cudaFree(M->d_bfs);
  M->d_bfs = nullptr;
  const size_t bytes = maps.size() * sizeof(CUtensorMap);
  if (cudaMalloc(&M->d_bfs, bytes) != cudaSuccess) return nullptr;
  if (cudaMemcpyAsync(M->d_bfs, maps.data(), bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return nullptr;
  M->bfs_key[0] = h; M->bfs_key[1] = mask;
  M->bfs_n = insts.size();
  return M->d_bfs;
}

// What a pass loop was built for: it is rebuilt when any of these changes.
struct PassLoopKey {
  long long v[32];
};

struct PassLoop {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  PassLoopKey key{};
  ~PassLoop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

PassLoop* pass_loop_new() { return new PassLoop(); }
void pass_loop_free(PassLoop* L) { delete L; }

namespace {

cudaError_t run_loop(PassLoop* L, const PassLoopKey& key, void* kern, int grid, int threads,
                     size_t smem, void** kargs, const TileQueue& q, int* ctl, unsigned cap,
                     unsigned long long* passes, unsigned long long* overflow, cudaStream_t s) {
  if (!(L->exec && std::memcmp(&L->key, &key, sizeof(key)) == 0)) {
    if (L->exec) cudaGraphExecDestroy(L->exec);
    if (L->graph) cudaGraphDestroy(L->graph);
    L->exec = nullptr;
    L->graph = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return e;
    L->graph = g;
    cudaMemsetParams mp{};
    mp.dst = ctl;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = 2;
    mp.height = 1;
    cudaGraphNode_t mnode;
    if ((e = cudaGraphAddMemsetNode(&mnode, g, nullptr, 0, &mp)) != cudaSuccess) return e;
    cudaGraphConditionalHandle h;
    if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
      return e;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    if ((e = cudaGraphAddNode(&wnode, g, &mnode, nullptr, 1, &cp)) != cudaSuccess) return e;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaKernelNodeParams kp{};
    kp.func = kern;
    kp.gridDim = dim3(grid);
    kp.blockDim = dim3(threads);
    kp.sharedMemBytes = (unsigned)smem;
    kp.kernelParams = kargs;
    cudaGraphNode_t knode;
    if ((e = cudaGraphAddKernelNode(&knode, body, nullptr, 0, &kp)) != cudaSuccess) return e;
    TileQueue qq = q;
    int* c = ctl;
    unsigned capv = cap;
    unsigned long long* pp = passes;
    unsigned long long* ov = overflow;
    void* cargs[] = {&qq, &c, &capv, &pp, &ov, &h};
    cudaKernelNodeParams cpk{};
    cpk.func = reinterpret_cast<void*>(k_pass_ctl);
    cpk.gridDim = dim3(1);
    cpk.blockDim = dim3(1);
    cpk.kernelParams = cargs;
    cudaGraphNode_t cnode;
    if ((e = cudaGraphAddKernelNode(&cnode, body, &knode, 1, &cpk)) != cudaSuccess) return e;
    cudaGraphExec_t x = nullptr;
    if ((e = cudaGraphInstantiate(&x, g, 0)) != cudaSuccess) return e;
    L->exec = x;
    L->key = key;
  }
  return cudaGraphLaunch(L->exec, s);
}

void key_common(PassLoopKey& k, int& i, const TileQueue& q, const Geo& g, const InstDesc* inst,
                const unsigned long long* counters, const unsigned long long* fault,
                const int* ctl, unsigned cap, int K, int TB, int grid) {
  auto put = [&](long long v) { k.v[i++] = v; };
  put((long long)(uintptr_t)q.flag[0]); put((long long)(uintptr_t)q.flag[1]);
  put((long long)(uintptr_t)q.list[0]); put((long long)(uintptr_t)q.list[1]);
  put((long long)(uintptr_t)q.ctr); put((long long)(uintptr_t)inst);
  put((long long)(uintptr_t)counters); put((long long)(uintptr_t)fault);
  put((long long)(uintptr_t)ctl); put(cap); put(K); put(TB); put(grid);
  put(g.Cp); put(g.Bp); put(g.NP); put(g.ntb); put(g.ntc);
}

}  // namespace

int lattice2d_kernel_size(const InstDesc& I, bool single) {
  if (!single || !encode_fn()) return 0;
  if (I.g.TA != 1 || I.g.A != 1 || I.g.Ap != 1 || I.g.TC != 32) return 0;
  if (I.node_base != 0 || I.res_base != 0 || I.tile_base != 0 || I.plane != I.g.NP) return 0;
  if (I.g.TB != 4 && I.g.TB != 8 && I.g.TB != 16 && I.g.TB != 32) return 0;
  if (I.g.Cp % 32 || I.g.Bp % I.g.TB) return 0;
  if (stencil_is<4>(I.st)) return 4;
  if (stencil_is<8>(I.st)) return 8;
  return 0;
}

int pr2d_kernel_size(const PoolPR<int>& p, bool single) {
  return p.kmask ? 0 : lattice2d_kernel_size(p.inst0, single);
}

cudaError_t launch_pool_pr2d(const PoolPR<int>& p, int K, int variant, unsigned long long* fault,
                             int tiles, cudaStream_t s) {
  PR2dMaps maps;
  if (!maps_for(p, K, p.inst0.g.TB, maps)) return cudaErrorInvalidValue;
  const int TB = p.inst0.g.TB;
#define LF_PR2D(KK, BB)                                                                \
  if (K == KK && TB == BB) {                                                             \
    if (variant == 1) return launch_kt<KK, BB, 32>(maps, p, fault, tiles, s);            \
    if (variant == 2 && BB <= 8) return launch_kt_warp<KK, (BB <= 8 ? BB : 8)>(maps, p, fault, tiles, s); \
    return launch_kt<KK, BB, 40>(maps, p, fault, tiles, s);                              \
  }
  LF_PR2D(4, 4) LF_PR2D(4, 8) LF_PR2D(4, 16) LF_PR2D(4, 32) LF_PR2D(8, 4) LF_PR2D(8, 8)
  LF_PR2D(8, 16) LF_PR2D(8, 32)
#undef LF_PR2D
  return cudaErrorInvalidValue;
}

template <int K, int TB, int REGS>
cudaError_t loop_kt(PassLoop* L, const PR2dMaps& maps, const PoolPR<int>& p,
                    unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                    unsigned long long* passes, cudaStream_t s) {
  using Ly = PR2dLayout<K, TB>;
  int grid = 0;
  void* kern = kt_setup<K, TB, REGS>(grid);
  grid = std::max(1, std::min(grid, tiles));
  PassLoopKey key{};
  int i = 0;
  key.v[i++] = 1;  // push/relabel
  key_common(key, i, p.q, p.inst0.g, p.inst, p.counters, fault, ctl, cap, K, TB, grid);
  key.v[i++] = REGS;
  key.v[i++] = p.sweeps;
  key.v[i++] = (long long)(uintptr_t)p.res;
  key.v[i++] = (long long)(uintptr_t)p.exc;
  key.v[i++] = (long long)(uintptr_t)p.h;
  const int* cp = ctl;
  void* kargs[] = {const_cast<PR2dMaps*>(&maps), const_cast<PoolPR<int>*>(&p), &fault, &cp};
  return run_loop(L, key, kern, grid, Ly::NT, Ly::smem_bytes, kargs, p.q, ctl, cap, passes,
                  nullptr, s);
}

template <int K, int TB>
cudaError_t bfs_loop_kt(PassLoop* L, const BFS2dMaps& maps, const PoolBFS& p,
                        unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                        unsigned long long* passes, unsigned long long* overflow,
                        cudaStream_t s) {
  using Ly = BFS2dLayout<TB>;
  int grid = 0;
  void* kern = bfs_kt_setup<K, TB>(grid);
  grid = std::max(1, std::min(grid, tiles));
  PassLoopKey key{};
  int i = 0;
  key.v[i++] = 2;  // BFS
  key_common(key, i, p.q, p.inst0.g, p.inst, p.counters, fault, ctl, cap, K, TB, grid);
  key.v[i++] = p.max_local;
  key.v[i++] = (long long)(uintptr_t)p.h;
  key.v[i++] = (long long)(uintptr_t)p.mask;
  key.v[i++] = (long long)(uintptr_t)p.any_changed;
  key.v[i++] = (long long)(uintptr_t)overflow;
  const int* cp = ctl;
  void* kargs[] = {const_cast<BFS2dMaps*>(&maps), const_cast<PoolBFS*>(&p), &fault, &cp};
  return run_loop(L, key, kern, grid, Ly::NT, Ly::smem_bytes, kargs, p.q, ctl, cap, passes,
                  overflow, s);
}

cudaError_t loop_pool_pr2d(PassLoop* L, const PoolPR<int>& p, int K, int variant,
                           unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                           unsigned long long* passes, cudaStream_t s) {
  PR2dMaps maps;
  if (!maps_for(p, K, p.inst0.g.TB, maps)) return cudaErrorInvalidValue;
  const int TB = p.inst0.g.TB;
#define LF_PR2D(KK, BB)                                                                      \
  if (K == KK && TB == BB) {                                                                   \
    if (variant == 1) return loop_kt<KK, BB, 32>(L, maps, p, fault, tiles, ctl, cap, passes, s); \
    return loop_kt<KK, BB, 40>(L, maps, p, fault, tiles, ctl, cap, passes, s);                  \
  }
  LF_PR2D(4, 4) LF_PR2D(4, 8) LF_PR2D(4, 16) LF_PR2D(4, 32) LF_PR2D(8, 4) LF_PR2D(8, 8)
  LF_PR2D(8, 16) LF_PR2D(8, 32)
#undef LF_PR2D
  return cudaErrorInvalidValue;
}

cudaError_t loop_pool_bfs2d(PassLoop* L, const PoolBFS& p, int K, unsigned long long* fault,
                            int tiles, int* ctl, unsigned cap, unsigned long long* passes,
                            unsigned long long* overflow, cudaStream_t s) {
  BFS2dMaps maps;
  const int TB = p.inst0.g.TB;
  if (!bfs_maps_for(p, TB, maps)) return cudaErrorInvalidValue;
#define LF_BFS2D(KK, BB)                                                                      \
  if (K == KK && TB == BB)                                                                      \
    return bfs_loop_kt<KK, BB>(L, maps, p, fault, tiles, ctl, cap, passes, overflow, s);
  LF_BFS2D(4, 4) LF_BFS2D(4, 8) LF_BFS2D(4, 16) LF_BFS2D(4, 32) LF_BFS2D(8, 4) LF_BFS2D(8, 8)
  LF_BFS2D(8, 16) LF_BFS2D(8, 32)
#undef LF_BFS2D
  return cudaErrorInvalidValue;
}

int pr2d64_kernel_size(const PoolPR<long long>& p, bool single) {
  return p.kmask ? lattice2d_kernel_size(p.inst0, single) : 0;
}

// the 64-bit pass with section masks: one launch (L null, p.cur) or a
// device-side loop of passes
cudaError_t pr2d64(PassLoop* L, const PoolPR<long long>& p, int K, unsigned long long* fault,
                   int tiles, int* ctl, unsigned cap, unsigned long long* passes, cudaStream_t s) {
  PR2dMaps64 maps;
  const int TB = p.inst0.g.TB;
  if (!maps64_for(p, K, TB, maps)) return cudaErrorInvalidValue;
  int grid = 0, threads = TB * 32;
  void* kern = nullptr;
  size_t smem = 0;
#define LF_P64(KK, BB)                                  \
  if (K == KK && TB == BB) {                            \
    kern = kt64_setup<KK, BB>(grid);                    \
    smem = PR2dLayout64<KK, BB>::smem_bytes;            \
  }
  LF_P64(4, 4) LF_P64(4, 8) LF_P64(4, 16) LF_P64(4, 32) LF_P64(8, 4) LF_P64(8, 8)
  LF_P64(8, 16) LF_P64(8, 32)
#undef LF_P64
  if (!kern) return cudaErrorInvalidValue;
  grid = std::max(1, std::min(grid, tiles));
  if (!L) {
    const int* no_ctl = nullptr;
    void* kargs[] = {&maps, const_cast<PoolPR<long long>*>(&p), &fault, &no_ctl};
    return cudaLaunchKernel(kern, dim3(grid), dim3(threads), kargs, smem, s);
  }
  PassLoopKey key{};
  int i = 0;
  key.v[i++] = 5;  // 64-bit push/relabel with section masks
  key_common(key, i, p.q, p.inst0.g, p.inst, p.counters, fault, ctl, cap, K, TB, grid);
  key.v[i++] = p.sweeps;
  key.v[i++] = (long long)(uintptr_t)p.res;
  key.v[i++] = (long long)(uintptr_t)p.exc;
  key.v[i++] = (long long)(uintptr_t)p.h;
  key.v[i++] = (long long)(uintptr_t)p.kmask;
  const int* cp = ctl;
  void* kargs[] = {&maps, const_cast<PoolPR<long long>*>(&p), &fault, &cp};
  return run_loop(L, key, kern, grid, threads, smem, kargs, p.q, ctl, cap, passes, nullptr, s);
}

cudaError_t pool_pr2d(PassLoop* L, const void* maps, const PoolPR<int>& p, int TB, int variant,
                      unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                      unsigned long long* passes, cudaStream_t s) {
  int grid = 0, threads = TB * 32;
  void* kern = nullptr;
  size_t smem = 0;
#define LF_PP(BB)                                                                    \
  if (TB == BB) {                                                                    \
    kern = variant == 1 ? kt_pool_setup<BB, 32>(grid) : kt_pool_setup<BB, 40>(grid); \
    smem = PR2dPoolLayout<BB>::smem_bytes;                                           \
  }
  LF_PP(4) LF_PP(8) LF_PP(16) LF_PP(32)
#undef LF_PP
  if (!kern) return cudaErrorInvalidValue;
  grid = std::max(1, std::min(grid, tiles));
  const CUtensorMap* m = static_cast<const CUtensorMap*>(maps);
  if (!L) {
    const int* no_ctl = nullptr;
    void* kargs[] = {&m, const_cast<PoolPR<int>*>(&p), &fault, &no_ctl};
    return cudaLaunchKernel(kern, dim3(grid), dim3(threads), kargs, smem, s);
  }
  PassLoopKey key{};
  int i = 0;
  key.v[i++] = 3;  // push/relabel over a pool
  key_common(key, i, p.q, p.inst0.g, p.inst, p.counters, fault, ctl, cap, 0, TB, grid);
  key.v[i++] = variant;
  key.v[i++] = p.sweeps;
  key.v[i++] = (long long)(uintptr_t)m;
  key.v[i++] = (long long)(uintptr_t)p.res;
  key.v[i++] = (long long)(uintptr_t)p.exc;
  key.v[i++] = (long long)(uintptr_t)p.h;
  key.v[i++] = (long long)(uintptr_t)p.tile_inst;
  const int* cp = ctl;
  void* kargs[] = {&m, const_cast<PoolPR<int>*>(&p), &fault, &cp};
  return run_loop(L, key, kern, grid, threads, smem, kargs, p.q, ctl, cap, passes, nullptr, s);
}

cudaError_t pool_bfs2d(PassLoop* L, const void* maps, const PoolBFS& p, int TB,
                       unsigned long long* fault, int tiles, int* ctl, unsigned cap,
                       unsigned long long* passes, unsigned long long* overflow, cudaStream_t s) {
  int grid = 0, threads = TB * 32;
  void* kern = nullptr;
  size_t smem = 0;
#define LF_PB(BB)                              \
  if (TB == BB) {                              \
    kern = bfs_kt_pool_setup<BB>(grid);        \
    smem = BFS2dLayout<BB>::smem_bytes;        \
  }
  LF_PB(4) LF_PB(8) LF_PB(16) LF_PB(32)
#undef LF_PB
  if (!kern) return cudaErrorInvalidValue;
  grid = std::max(1, std::min(grid, tiles));
  const CUtensorMap* m = static_cast<const CUtensorMap*>(maps);
  if (!L) {
    const int* no_ctl = nullptr;
    void* kargs[] = {&m, const_cast<PoolBFS*>(&p), &fault, &no_ctl};
    return cudaLaunchKernel(kern, dim3(grid), dim3(threads), kargs, smem, s);
  }
  PassLoopKey key{};
  int i = 0;
  key.v[i++] = 4;  // BFS over a pool
  key_common(key, i, p.q, p.inst0.g, p.inst, p.counters, fault, ctl, cap, 0, TB, grid);
  key.v[i++] = p.max_local;
  key.v[i++] = (long long)(uintptr_t)m;
  key.v[i++] = (long long)(uintptr_t)p.h;
  key.v[i++] = (long long)(uintptr_t)p.mask;
  key.v[i++] = (long long)(uintptr_t)p.any_changed;
  key.v[i++] = (long long)(uintptr_t)p.tile_inst;
  key.v[i++] = (long long)(uintptr_t)overflow;
  const int* cp = ctl;
  void* kargs[] = {&m, const_cast<PoolBFS*>(&p), &fault, &cp};
  return run_loop(L, key, kern, grid, threads, smem, kargs, p.q, ctl, cap, passes, overflow, s);
}

cudaError_t launch_pool_bfs2d(const PoolBFS& p, int K, unsigned long long* fault, int tiles,
                              cudaStream_t s) {
  BFS2dMaps maps;
  const int TB = p.inst0.g.TB;
  if (!bfs_maps_for(p, TB, maps)) return cudaErrorInvalidValue;
#define LF_BFS2D(KK, BB) \
  if (K == KK && TB == BB) return launch_bfs_kt<KK, BB>(maps, p, fault, tiles, s);
  LF_BFS2D(4, 4) LF_BFS2D(4, 8) LF_BFS2D(4, 16) LF_BFS2D(4, 32) LF_BFS2D(8, 4) LF_BFS2D(8, 8)
  LF_BFS2D(8, 16) LF_BFS2D(8, 32)
#undef LF_BFS2D
  return cudaErrorInvalidValue;
}

}  // namespace lfg
