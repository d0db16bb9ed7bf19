// Launchers of the TMA-staged 2-d passes (push/relabel, lf_pool_pr2d.cuh; BFS
// relabel, lf_pool_bfs2d.cuh): tensor maps of the lattice's arrays, launch
// shapes, and the test of whether a pass can take these kernels.
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "lf_pool_bfs2d.cuh"
#include "lf_pool_pr2d.cuh"
#include "lf_pool_launch.cuh"
#include "lf_pool_runner.h"

namespace lfg {

namespace {

template <int K>
bool stencil_is(const Stencil& st) {
  if (st.K != K) return false;
  for (int k = 0; k < K; ++k)
    if (st.da[k] != 0 || st.db[k] != s2_db<K>(k) || st.dc[k] != s2_dc<K>(k)) return false;
  return true;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool encode(CUtensorMap* m, void* base, int rank, const cuuint64_t* dims,
            const cuuint64_t* strides, const cuuint32_t* box,
            CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_INT32) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, type, rank, base, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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
cudaError_t launch_kt(const PR2dMaps& maps, const PoolPR<int>& p, unsigned long long* fault,
                      int tiles, cudaStream_t s) {
  using Ly = PR2dLayout<K, TB>;
  auto kern = k_pool_pr2d<K, TB, REGS>;
  static std::mutex mu;
  static int cap = 0;
  int grid;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!cap) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
    }
    grid = cap;
  }
  kern<<<std::max(1, std::min(grid, tiles)), Ly::NT, Ly::smem_bytes, s>>>(
      maps, p, fault);
  return cudaGetLastError();
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
cudaError_t launch_bfs_kt(const BFS2dMaps& maps, const PoolBFS& p, unsigned long long* fault,
                          int tiles, cudaStream_t s) {
  using Ly = BFS2dLayout<TB>;
  auto kern = k_pool_bfs2d<K, TB>;
  static std::mutex mu;
  static int cap = 0;
  int grid;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!cap) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
    }
    grid = cap;
  }
  kern<<<std::max(1, std::min(grid, tiles)), Ly::NT, Ly::smem_bytes, s>>>(maps, p, fault);
  return cudaGetLastError();
}

}  // namespace

int lattice2d_kernel_size(const InstDesc& I, bool single) {
  if (!single || !encode_fn()) return 0;
  if (I.g.TA != 1 || I.g.A != 1 || I.g.Ap != 1 || I.g.TC != 32) return 0;
  if (I.node_base != 0 || I.res_base != 0 || I.tile_base != 0 || I.plane != I.g.NP) return 0;
  if (I.g.TB != 8 && I.g.TB != 16 && I.g.TB != 32) return 0;
  if (I.g.Cp % 32 || I.g.Bp % I.g.TB) return 0;
  if (stencil_is<4>(I.st)) return 4;
  if (stencil_is<8>(I.st)) return 8;
  return 0;
}

int pr2d_kernel_size(const PoolPR<int>& p, bool single) {
  return p.kmask ? 0 : lattice2d_kernel_size(p.inst0, single);
}

cudaError_t launch_pool_pr2d(const PoolPR<int>& p, int K, int regs, unsigned long long* fault,
                             int tiles, cudaStream_t s) {
  PR2dMaps maps;
  if (!maps_for(p, K, p.inst0.g.TB, maps)) return cudaErrorInvalidValue;
  const int TB = p.inst0.g.TB;
#define LF_PR2D(KK, BB)                                                              \
  if (K == KK && TB == BB)                                                             \
    return regs == 32 ? launch_kt<KK, BB, 32>(maps, p, fault, tiles, s)                \
                      : launch_kt<KK, BB, 40>(maps, p, fault, tiles, s);
  LF_PR2D(4, 8) LF_PR2D(4, 16) LF_PR2D(4, 32) LF_PR2D(8, 8) LF_PR2D(8, 16) LF_PR2D(8, 32)
#undef LF_PR2D
  return cudaErrorInvalidValue;
}

cudaError_t launch_pool_bfs2d(const PoolBFS& p, int K, unsigned long long* fault, int tiles,
                              cudaStream_t s) {
  BFS2dMaps maps;
  const int TB = p.inst0.g.TB;
  if (!bfs_maps_for(p, TB, maps)) return cudaErrorInvalidValue;
#define LF_BFS2D(KK, BB) \
  if (K == KK && TB == BB) return launch_bfs_kt<KK, BB>(maps, p, fault, tiles, s);
  LF_BFS2D(4, 8) LF_BFS2D(4, 16) LF_BFS2D(4, 32) LF_BFS2D(8, 8) LF_BFS2D(8, 16) LF_BFS2D(8, 32)
#undef LF_BFS2D
  return cudaErrorInvalidValue;
}

}  // namespace lfg
