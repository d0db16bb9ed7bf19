// Launchers of the TMA-staged 3-d passes (push/relabel and BFS,
// lf_pool_pr3d.cuh): their tensor maps, launch shapes, and the test of
// whether a pass can take them.
#include <algorithm>
#include <mutex>

#include "lf_pool_launch.cuh"
#include "lf_pool_pr3d.cuh"
#include "lf_pool_runner.h"
#include "lf_tensor_map.h"

namespace lfg {

namespace {

// the lattice's stencil is the compile-time table of that size
template <int K>
bool stencil3_is(const Stencil& st) {
  if (st.K != K) return false;
  for (int k = 0; k < K; ++k)
    if (st.da[k] != s3_da<K>(k) || st.db[k] != s3_db<K>(k) || st.dc[k] != s3_dc<K>(k) ||
        st.rev[k] != (k < K / 2 ? k + K / 2 : k - K / 2))
      return false;
  return true;
}

bool radius1_3d(const InstDesc& I) {
  return stencil3_is<6>(I.st) || stencil3_is<18>(I.st) || stencil3_is<26>(I.st);
}

template <int K, int TA, int TB>
constexpr bool pr3d_fits() {
  return PR3dLayout<K, TA, TB>::smem_bytes <= 227 * 1024;
}

// Tensor maps of the last lattice this host thread launched for.
struct Map3Cache {
  const void *res = nullptr, *exc = nullptr, *h = nullptr;
  int Cp = 0, Bp = 0, Ap = 0, K = 0, TA = 0, TB = 0;
  PR3dMaps maps;
};

bool maps3_for(const PoolPR<int>& p, int K, int TA, int TB, PR3dMaps& out) {
  thread_local Map3Cache c;
  const Geo& g = p.inst0.g;
  if (c.res == p.res && c.exc == p.exc && c.h == p.h && c.Cp == g.Cp && c.Bp == g.Bp &&
      c.Ap == g.Ap && c.K == K && c.TA == TA && c.TB == TB) {
    out = c.maps;
    return true;
  }
  PR3dMaps m;
  const cuuint64_t row = (cuuint64_t)g.Cp * 4, pl = row * (cuuint64_t)g.Bp;
  const cuuint64_t d4[4] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)g.Ap, (cuuint64_t)K};
  const cuuint64_t s4[3] = {row, pl, (cuuint64_t)g.NP * 4};
  const cuuint32_t b4[4] = {32, (cuuint32_t)TB, (cuuint32_t)TA, (cuuint32_t)K};
  const cuuint64_t d3[3] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)g.Ap};
  const cuuint64_t s3[2] = {row, pl};
  const cuuint32_t be[3] = {32, (cuuint32_t)TB, (cuuint32_t)TA};
  const cuuint32_t bh[3] = {(cuuint32_t)kPr3dHaloW, (cuuint32_t)(TB + 2), (cuuint32_t)(TA + 2)};
  if (!encode_tensor_map(&m.res, p.res, 4, d4, s4, b4) ||
      !encode_tensor_map(&m.exc, p.exc, 3, d3, s3, be) ||
      !encode_tensor_map(&m.h, p.h, 3, d3, s3, bh))
    return false;
  c.res = p.res; c.exc = p.exc; c.h = p.h;
  c.Cp = g.Cp; c.Bp = g.Bp; c.Ap = g.Ap; c.K = K; c.TA = TA; c.TB = TB;
  c.maps = m;
  out = m;
  return true;
}

template <int K, int TA, int TB>
cudaError_t launch_k3(const PR3dMaps& maps, const PoolPR<int>& p, unsigned long long* fault,
                      int tiles, cudaStream_t s) {
  if constexpr (!pr3d_fits<K, TA, TB>()) {
    return cudaErrorInvalidValue;
  } else {
    using Ly = PR3dLayout<K, TA, TB>;
    auto kern = k_pool_pr3d<K, TA, TB>;
    static std::mutex mu;
    static int cap = 0;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!cap) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
      }
    }
    kern<<<std::max(1, std::min(cap, tiles)), Ly::NT, Ly::smem_bytes, s>>>(maps, p, fault);
    return cudaGetLastError();
  }
}

struct Bfs3MapCache {
  const void *h = nullptr, *mask = nullptr;
  int Cp = 0, Bp = 0, Ap = 0, TA = 0, TB = 0;
  BFS3dMaps maps;
};

bool bfs3_maps_for(const PoolBFS& p, int TA, int TB, BFS3dMaps& out) {
  thread_local Bfs3MapCache c;
  const Geo& g = p.inst0.g;
  if (c.h == p.h && c.mask == p.mask && c.Cp == g.Cp && c.Bp == g.Bp && c.Ap == g.Ap &&
      c.TA == TA && c.TB == TB) {
    out = c.maps;
    return true;
  }
  BFS3dMaps m;
  const cuuint64_t d3[3] = {(cuuint64_t)g.Cp, (cuuint64_t)g.Bp, (cuuint64_t)g.Ap};
  const cuuint64_t s4[2] = {(cuuint64_t)g.Cp * 4, (cuuint64_t)g.Cp * 4 * g.Bp};
  const cuuint64_t s8[2] = {(cuuint64_t)g.Cp * 8, (cuuint64_t)g.Cp * 8 * g.Bp};
  const cuuint32_t bh[3] = {(cuuint32_t)kPr3dHaloW, (cuuint32_t)(TB + 2), (cuuint32_t)(TA + 2)};
  const cuuint32_t bm[3] = {32, (cuuint32_t)TB, (cuuint32_t)TA};
  if (!encode_tensor_map(&m.h, p.h, 3, d3, s4, bh) ||
      !encode_tensor_map(&m.mask, const_cast<uint64_t*>(p.mask), 3, d3, s8, bm,
                         CU_TENSOR_MAP_DATA_TYPE_UINT64))
    return false;
  c.h = p.h; c.mask = p.mask; c.Cp = g.Cp; c.Bp = g.Bp; c.Ap = g.Ap; c.TA = TA; c.TB = TB;
  c.maps = m;
  out = m;
  return true;
}

template <int K, int TA, int TB>
cudaError_t launch_b3(const BFS3dMaps& maps, const PoolBFS& p, unsigned long long* fault,
                      int tiles, cudaStream_t s) {
  using Ly = BFS3dLayout<TA, TB>;
  auto kern = k_pool_bfs3d<K, TA, TB>;
  static std::mutex mu;
  static int cap = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!cap) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Ly::smem_bytes);
      cap = occupancy_grid(kern, Ly::NT, Ly::smem_bytes);
    }
  }
  kern<<<std::max(1, std::min(cap, tiles)), Ly::NT, Ly::smem_bytes, s>>>(maps, p, fault);
  return cudaGetLastError();
}

}  // namespace

int lattice3d_kernel_size(const InstDesc& I, bool single) {
  if (!single || !tensor_map_encoder()) return 0;
  if (I.g.TC != 32 || I.g.TA != 4 || (I.g.TB != 2 && I.g.TB != 4 && I.g.TB != 8)) return 0;
  if (I.node_base != 0 || I.res_base != 0 || I.tile_base != 0 || I.plane != I.g.NP) return 0;
  if (I.g.Cp % 32 || I.g.Bp % I.g.TB || I.g.Ap % I.g.TA) return 0;
  return radius1_3d(I) ? I.st.K : 0;
}

cudaError_t launch_pool_bfs3d(const PoolBFS& p, int K, unsigned long long* fault, int tiles,
                              cudaStream_t s) {
  const int TA = p.inst0.g.TA, TB = p.inst0.g.TB;
  BFS3dMaps maps;
  if (!bfs3_maps_for(p, TA, TB, maps)) return cudaErrorInvalidValue;
#define LF_BFS3D(KK, BB) \
  if (K == KK && TA == 4 && TB == BB) return launch_b3<KK, 4, BB>(maps, p, fault, tiles, s);
  LF_BFS3D(6, 2) LF_BFS3D(6, 4) LF_BFS3D(6, 8) LF_BFS3D(18, 2) LF_BFS3D(18, 4) LF_BFS3D(18, 8)
  LF_BFS3D(26, 2) LF_BFS3D(26, 4) LF_BFS3D(26, 8)
#undef LF_BFS3D
  return cudaErrorInvalidValue;
}

int pr3d_kernel_size(const PoolPR<int>& p, bool single) {
  const InstDesc& I = p.inst0;
  if (p.kmask || !lattice3d_kernel_size(I, single)) return 0;
  const int K = I.st.K, TB = I.g.TB;
  const bool fits = (K == 6) || (K == 18 && TB <= 4) || (K == 26 && TB <= 4);
  return fits ? K : 0;
}

cudaError_t launch_pool_pr3d(const PoolPR<int>& p, int K, unsigned long long* fault, int tiles,
                             cudaStream_t s) {
  const int TA = p.inst0.g.TA, TB = p.inst0.g.TB;
  PR3dMaps maps;
  if (!maps3_for(p, K, TA, TB, maps)) return cudaErrorInvalidValue;
#define LF_PR3D(KK, BB) \
  if (K == KK && TA == 4 && TB == BB) return launch_k3<KK, 4, BB>(maps, p, fault, tiles, s);
  LF_PR3D(6, 2) LF_PR3D(6, 4) LF_PR3D(6, 8) LF_PR3D(18, 2) LF_PR3D(18, 4) LF_PR3D(26, 2)
  LF_PR3D(26, 4)
#undef LF_PR3D
  return cudaErrorInvalidValue;
}

}  // namespace lfg
