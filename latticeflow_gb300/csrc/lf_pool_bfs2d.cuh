// Global-relabel BFS pass specialised for one 2-d lattice with a 3x3
// neighbourhood (Full2d_4, Full2d_8), tiles staged into shared memory by TMA.
//
// Same relaxation as bfs_tile (lf_pool_graph.cuh): exact distance to the
// nearest deficit node along residual edges, iterated inside the tile until
// stable, rows relaxed whole by segmented warp min-scans.  It reads only the
// residual mask and the heights, so it serves 32- and 64-bit capacities
// alike.  Differences:
//   * compile-time stencil (immediate shared-memory offsets);
//   * one elected thread stages a visit with two bulk tensor copies: the
//     heights with their halo ({40 x (TB + 2)} from column c0 - 4, as the
//     push/relabel pass) and the masks ({32 x TB}, 64-bit); two stage
//     buffers, the next tile's copies in flight during the current visit;
//   * a changed node on the tile edge queues only the tiles that hold its
//     neighbours across that edge (an edge row / column queues the tile
//     beside it, a corner node also the diagonal tile), not all eight.
// Heights only decrease during a relabel, so a stale staged halo is an upper
// bound like any other and the fixed point is the same exact distance.
#pragma once

#include "lf_pool_graph.cuh"
#include "lf_pool_pr2d.cuh"

namespace lfg {

struct BFS2dMaps {
  CUtensorMap h;
  CUtensorMap mask;
};

template <int TB>
struct BFS2dLayout {
  static constexpr int NT = TB * 32;
  static constexpr int h_bytes = (TB + 2) * kPr2dHaloW * 4;
  static constexpr int mask_off = (h_bytes + 127) / 128 * 128;
  static constexpr int mask_bytes = NT * 8;
  static constexpr int stage_bytes = (mask_off + mask_bytes + 127) / 128 * 128;
  static constexpr int tx_bytes = h_bytes + mask_bytes;
  // two stage buffers, two mbarriers, an edge-flag word per buffer, alignment slack
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
};

template <int TB>
__device__ __forceinline__ void bfs2d_issue(const BFS2dMaps& maps, const Geo& g, int tile,
                                            unsigned stage, unsigned bar) {
  using Ly = BFS2dLayout<TB>;
  if (!tile_ok(tile, g.ntiles)) {
    mbar_expect_tx(bar, 0);
    return;
  }
  const int tc = tile % g.ntc, tb = tile / g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_2d(stage, &maps.h, c0 - 4, b0 - 1, bar);
  tma_load_2d(stage + Ly::mask_off, &maps.mask, c0, b0, bar);
}

// Edge flags of a changed node: bit 0 up, 1 down, 2 left, 3 right (the tile
// beside that edge), 4..7 the diagonal tiles up-left, up-right, down-left,
// down-right (8-connected only, corner nodes).
template <int K, int TB>
__device__ __forceinline__ unsigned bfs2d_edge_bits(int ib, int ic) {
  const bool up = ib == 0, dn = ib == TB - 1, lf = ic == 0, rt = ic == 31;
  unsigned b = (up ? 1u : 0u) | (dn ? 2u : 0u) | (lf ? 4u : 0u) | (rt ? 8u : 0u);
  if (K == 8)
    b |= (up && lf ? 16u : 0u) | (up && rt ? 32u : 0u) | (dn && lf ? 64u : 0u) |
         (dn && rt ? 128u : 0u);
  return b;
}

// LAT as for pr2d_tile.
template <int K, int TB, class LAT>
__device__ __forceinline__ void bfs2d_tile(const PoolBFS& p, const LAT& L, int cur,
                                           unsigned char* stage, unsigned* s_flags, int tile,
                                           int my_h, const uint64_t m) {
  constexpr int HW = kPr2dHaloW;
  int* s_h = reinterpret_cast<int*>(stage);
  const int t = threadIdx.x;
  const int ic = t & 31, ib = t >> 5;
  const int tc = tile % lat_ntc(L), tb = tile / lat_ntc(L);
  const long long gi = (long long)(tb * TB + ib) * lat_Cp(L) + (tc * 32 + ic) + lat_node_base(L);
  const int tile_g = lat_tile_base(L) + tile;
  const int hidx = (ib + 1) * HW + (ic + 4);
  const int nxt = cur ^ 1;
  // the row directions of both stencils: (0, 1) is entry 0, (0, -1) entry K/2
  constexpr int kr = 0, kl = K / 2;
  const bool can_l = (m >> kl) & 1, can_r = (m >> kr) & 1;
  bool changed = false;
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int best = my_h;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((m >> k) & 1) {
        const int hn = s_h[hidx + s2_db<K>(k) * HW + s2_dc<K>(k)] + 1;
        best = hn < best ? hn : best;
      }
    }
    // after the first iteration the row is consistent along its row edges
    // (each node at most one above a neighbour it can push to), and stays so
    // while no node of the row improves: the scans change nothing then
    if (it == 0 || __any_sync(0xffffffffu, best < my_h)) {
      best = row_scan_from_left(best, can_l, ic);
      best = row_scan_from_right(best, can_r, ic);
    }
    const int c = best < my_h;
    if (c) {
      my_h = best;
      s_h[hidx] = best;
      changed = true;
    }
    if (!__syncthreads_or(c)) { converged = 1; break; }
  }
  if (changed) p.h[gi] = my_h;
  // tiles beside the edges whose nodes changed
  unsigned bits = changed ? bfs2d_edge_bits<K, TB>(ib, ic) : 0u;
  bits = __reduce_or_sync(0xffffffffu, bits);
  if (ic == 0 && bits) atomicOr(s_flags, bits);
  // the buffer's next contents come from the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const unsigned f = *s_flags;
  if (t < 8 && ((f >> t) & 1u)) {
    const int dtb = (t == 0 || t == 4 || t == 5) ? -1 : (t == 1 || t == 6 || t == 7) ? 1 : 0;
    const int dtc = (t == 2 || t == 4 || t == 6) ? -1 : (t == 3 || t == 5 || t == 7) ? 1 : 0;
    const int a = tb + dtb, c = tc + dtc;
    if (a >= 0 && a < lat_ntb(L) && c >= 0 && c < lat_ntc(L))
      enqueue_tile(p.q, nxt, lat_tile_base(L) + a * lat_ntc(L) + c);
  }
  if (t == 0) {
    if (f) *p.any_changed = 1;
    if (!converged) { enqueue_tile(p.q, nxt, tile_g); *p.any_changed = 1; }
  }
}

// One lattice (the pool of one).  `fault` records a copy that did not land
// in time; ctl as for k_pool_pr2d.
template <int K, int TB>
__global__ void __launch_bounds__(TB * 32, 2048 / (TB * 32))
    k_pool_bfs2d(const __grid_constant__ BFS2dMaps maps, PoolBFS p, unsigned long long* fault,
                 const int* ctl) {
  using Ly = BFS2dLayout<TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);  // two mbarriers, 8 bytes apart
  // edge flags of the visit on each buffer: a word is cleared two visits
  // after its last readers, who have passed two barriers since
  unsigned* s_flags = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const Geo& g = p.inst0.g;
  const int cur = ctl ? *ctl : p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = (ctl ? p.inst[0].done : p.inst0.done) != 0;
  if (threadIdx.x == 0 && !done) bfs2d_issue<TB>(maps, g, list[blockIdx.x], stage0, bar0);
  unsigned phases = 0;
  unsigned buf = 0;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x, buf ^= 1) {
    const int gt = list[i];
    if (threadIdx.x == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[1], 1ull);
      s_flags[buf] = 0;
    }
    if (done) continue;
    const unsigned nx = i + gridDim.x;
    if (threadIdx.x == 0 && nx < n)
      bfs2d_issue<TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes, bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    unsigned char* st = smem + buf * Ly::stage_bytes;
    const int h0 = reinterpret_cast<const int*>(st)[((threadIdx.x >> 5) + 1) * kPr2dHaloW +
                                                     (threadIdx.x & 31) + 4];
    const uint64_t m = reinterpret_cast<const uint64_t*>(st + Ly::mask_off)[threadIdx.x];
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicExch(fault, 1ull);
      mbar_wait_bounded(bar, par, kPr2dWaitLimit);
      if (nx < n) mbar_wait_bounded(bar0 + (buf ^ 1) * 8, (phases >> (buf ^ 1)) & 1u, kPr2dWaitLimit);
      return;
    }
    if (!tile_ok(gt, g.ntiles)) {
      if (threadIdx.x == 0) atomicExch(fault, 2ull);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      continue;
    }
    bfs2d_tile<K, TB>(p, g, cur, st, s_flags + buf, gt, h0, m);
  }
}

// A lattice's two tensor maps (heights, masks) in the pool's map array.
template <int TB>
__device__ __forceinline__ void bfs2d_pool_issue(const PoolBFS& p, const CUtensorMap* maps, int gt,
                                                 unsigned stage, unsigned bar) {
  using Ly = BFS2dLayout<TB>;
  const int ii = p.tile_inst[gt];
  const InstDesc& I = p.inst[ii];
  const int tile = gt - I.tile_base;
  const int tc = tile % I.g.ntc, tb = tile / I.g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_2d(stage, &maps[2 * ii], c0 - 4, b0 - 1, bar);
  tma_load_2d(stage + Ly::mask_off, &maps[2 * ii + 1], c0, b0, bar);
}

// Many 2-d lattices (Full2d_4 / Full2d_8, one tile height) in one pool, any
// capacity type: the same pass as k_pool_bfs2d with each tile's own
// lattice, stencil and tensor maps.
template <int TB>
__global__ void __launch_bounds__(TB * 32, 2048 / (TB * 32))
    k_pool_bfs2d_pool(const CUtensorMap* maps, PoolBFS p, unsigned long long* fault,
                      const int* ctl) {
  using Ly = BFS2dLayout<TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);
  unsigned* s_flags = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const int cur = ctl ? *ctl : p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) bfs2d_pool_issue<TB>(p, maps, list[blockIdx.x], stage0, bar0);
  unsigned phases = 0;
  unsigned buf = 0;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x, buf ^= 1) {
    const int gt = list[i];
    if (threadIdx.x == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[1], 1ull);
      s_flags[buf] = 0;
    }
    const unsigned nx = i + gridDim.x;
    if (threadIdx.x == 0 && nx < n)
      bfs2d_pool_issue<TB>(p, maps, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                           bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    unsigned char* st = smem + buf * Ly::stage_bytes;
    const int h0 = reinterpret_cast<const int*>(st)[((threadIdx.x >> 5) + 1) * kPr2dHaloW +
                                                     (threadIdx.x & 31) + 4];
    const uint64_t m = reinterpret_cast<const uint64_t*>(st + Ly::mask_off)[threadIdx.x];
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicExch(fault, 1ull);
      mbar_wait_bounded(bar, par, kPr2dWaitLimit);
      if (nx < n) mbar_wait_bounded(bar0 + (buf ^ 1) * 8, (phases >> (buf ^ 1)) & 1u, kPr2dWaitLimit);
      return;
    }
    const InstDesc& I = p.inst[p.tile_inst[gt]];
    if (I.done) {  // the whole block reads the same flag
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      continue;
    }
    const Lat2d L = lat2d_of(I);
    const int tile = gt - L.tile_base;
    if (I.st.K == 8)
      bfs2d_tile<8, TB>(p, L, cur, st, s_flags + buf, tile, h0, m);
    else
      bfs2d_tile<4, TB>(p, L, cur, st, s_flags + buf, tile, h0, m);
  }
}

}  // namespace lfg
