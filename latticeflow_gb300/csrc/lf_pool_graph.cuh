// Residual-graph passes of the pool: global-relabel BFS and forward closure.
//
// BFS relabel (the reference's hotStart BFS, push_relabel.hpp:306-415):
// exact distance to the nearest deficit node along residual edges, iterated
// inside the tile until stable; a changed edge node queues the neighbour
// tiles.  Nodes left at kHInf cannot reach a deficit node; the reference
// flips exactly those (push_relabel.hpp:394-402, gap flip :692-711).
// Forward closure: marks spread along residual edges from the excess nodes,
// the unique minimal on-set.
// The kernel size is a template argument so that the per-direction halo
// offsets live in registers across the tile iterations.
#pragma once

#include "lf_pool_launch.cuh"

namespace lfg {

// Distances along one tile row (the 32 lanes of a warp hold its 32 nodes):
// a node that can push to its left neighbour (can = residual in that
// direction) is at most that neighbour's distance + 1.  Segmented min-scan
// of (h - lane) from the left; a lane that cannot push left starts a
// segment.  Lane 0's left neighbour lies in the halo and is relaxed by the
// ordinary stencil step.  Values at or above kHInf stay there (min with h).
__device__ __forceinline__ int row_scan_from_left(int h, bool can, int lane) {
  int v = h - lane;
  bool head = !can || lane == 0;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int vu = __shfl_up_sync(0xffffffffu, v, off);
    const int hu = __shfl_up_sync(0xffffffffu, (int)head, off);
    if (lane >= off && !head) {
      v = vu < v ? vu : v;
      head = hu;
    }
  }
  const int r = v + lane;
  return r < h ? r : h;
}

// The same from the right (pushes to the right neighbour).
__device__ __forceinline__ int row_scan_from_right(int h, bool can, int lane) {
  int v = h + lane;
  bool head = !can || lane == 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int vd = __shfl_down_sync(0xffffffffu, v, off);
    const int hd = __shfl_down_sync(0xffffffffu, (int)head, off);
    if (lane + off < 32 && !head) {
      v = vd < v ? vd : v;
      head = hd;
    }
  }
  const int r = v - lane;
  return r < h ? r : h;
}

template <int K>
__device__ __forceinline__ void bfs_tile(const PoolBFS& p, const InstDesc& I, PoolSmemHead* hd,
                                         int* s_h, int gtile) {
  const Geo& g = I.g;
  const Stencil& st = I.st;
  const int tile = gtile - I.tile_base;
  const TileCtx x = tile_ctx(g, st, tile);
  const int t = threadIdx.x;
  const bool live = t < x.NT;
  const int nxt = p.cur ^ 1;
  int* h = p.h + I.node_base;
  load_halo_heights(g, st, x, h, s_h);
  int hoff[K];
  uint64_t m = 0;
  bool boundary = false;
  int kl = -1, kr = -1;  // the directions along the row, if the stencil has them
#pragma unroll
  for (int k = 0; k < K; ++k) {
    hoff[k] = (st.da[k] * x.HBB + st.db[k]) * x.HCC + st.dc[k];
    if (outside_tile(g, x, st.da[k], st.db[k], st.dc[k])) boundary = true;
    if (st.da[k] == 0 && st.db[k] == 0) {
      if (st.dc[k] == -1) kl = k;
      if (st.dc[k] == 1) kr = k;
    }
  }
  if (live) m = p.mask[I.node_base + x.gi];
  const bool can_l = kl >= 0 && ((m >> kl) & 1);
  const bool can_r = kr >= 0 && ((m >> kr) & 1);
  const int lane = x.ic;  // tiles are 32 nodes wide: one warp per row
  __syncthreads();
  int my_h = live ? s_h[x.hidx] : kHInf;
  bool changed = false;
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int best = my_h;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((m >> k) & 1) {
        const int hn = s_h[x.hidx + hoff[k]] + 1;
        best = hn < best ? hn : best;
      }
    }
    // whole rows at once: every lane of the warp takes part (after the first
    // iteration a row is consistent along its row edges and stays so while
    // none of its nodes improves: the scans change nothing then)
    if (it == 0 || __any_sync(0xffffffffu, best < my_h)) {
      if (kl >= 0) best = row_scan_from_left(best, can_l, lane);
      if (kr >= 0) best = row_scan_from_right(best, can_r, lane);
    }
    const int c = best < my_h;
    if (c) {
      my_h = best;
      s_h[x.hidx] = best;
      changed = true;
    }
    if (!__syncthreads_or(c)) { converged = 1; break; }
  }
  if (changed) h[x.gi] = my_h;
  const int any_b = __syncthreads_or(changed && boundary && live);
  // neighbour tiles are queued by 26 threads at once (one atomic pair each)
  if (any_b && t < 27 && t != 13) {
    const int da = t / 9 - 1, db = (t / 3) % 3 - 1, dc = t % 3 - 1;
    const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
    const int a = ta + da, b = tb + db, c = tc + dc;
    if (a >= 0 && a < g.nta && b >= 0 && b < g.ntb && c >= 0 && c < g.ntc)
      enqueue_tile(p.q, nxt, I.tile_base + (a * g.ntb + b) * g.ntc + c);
  }
  if (t == 0) {
    if (any_b) *p.any_changed = 1;
    if (!converged) { enqueue_tile(p.q, nxt, gtile); *p.any_changed = 1; }
  }
}

template <int KA, int KB, bool SINGLE>
__global__ void __launch_bounds__(1024, 2) k_pool_bfs(PoolBFS p) {
  extern __shared__ __align__(16) unsigned char smem[];
  PoolSmemHead* hd = reinterpret_cast<PoolSmemHead*>(smem);
  int* s_h = reinterpret_cast<int*>(smem + sizeof(PoolSmemHead));
  const unsigned n = queued_count(p.q, p.cur);
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x) {
    const int gt = p.q.list[p.cur][i];
    __syncthreads();
    if (!SINGLE) {
      load_inst(&p.inst[p.tile_inst[gt]], &hd->inst);
      __syncthreads();
    }
    const InstDesc& I = SINGLE ? p.inst0 : hd->inst;
    if (threadIdx.x == 0) {
      p.q.flag[p.cur][gt] = 0;
      atomicAdd(&p.counters[1], 1ull);
    }
    if (I.done) continue;
    if (I.st.K == KA) bfs_tile<KA>(p, I, hd, s_h, gt);
    else if (KB != KA && I.st.K == KB) bfs_tile<KB>(p, I, hd, s_h, gt);
  }
}

template <int K>
__device__ __forceinline__ void reach_tile(const PoolReach& p, const InstDesc& I, int* s_mark,
                                           int gtile) {
  const Geo& g = I.g;
  const Stencil& st = I.st;
  const int tile = gtile - I.tile_base;
  const TileCtx x = tile_ctx(g, st, tile);
  const int t = threadIdx.x;
  const bool live = t < x.NT;
  const int nxt = p.cur ^ 1;
  int* mark = p.mark + I.node_base;
  int toff[K];
  uint64_t outm = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    toff[k] = (st.da[k] * g.TB + st.db[k]) * g.TC + st.dc[k];
    if (outside_tile(g, x, st.da[k], st.db[k], st.dc[k])) outm |= 1ull << k;
  }
  int m0 = 0;
  uint64_t m = 0;
  if (live) {
    m0 = mark[x.gi];
    s_mark[t] = m0;
    m = p.mask[I.node_base + x.gi];
  }
  __syncthreads();
  const uint64_t in = m & ~outm;
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int c = 0;
    if (live && s_mark[t]) {
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if ((in >> k) & 1) {
          const int tn = t + toff[k];
          if (!s_mark[tn]) { s_mark[tn] = 1; c = 1; }
        }
      }
    }
    if (!__syncthreads_or(c)) { converged = 1; break; }
  }
  int sent = 0;
  if (live && s_mark[t]) {
    if (!m0) mark[x.gi] = 1;
    const uint64_t out = m & outm;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((out >> k) & 1) {
        const int A_ = x.a0 + x.ia + st.da[k], B_ = x.b0 + x.ib + st.db[k],
                  C_ = x.c0 + x.ic + st.dc[k];
        const long long gn = ((long long)A_ * g.Bp + B_) * g.Cp + C_;
        if (!mark[gn]) {
          mark[gn] = 1;
          enqueue_tile(p.q, nxt, I.tile_base + tile_of(g, A_, B_, C_));
          sent = 1;
        }
      }
    }
  }
  const int any_sent = __syncthreads_or(sent);
  if (t == 0) {
    if (any_sent) *p.any_changed = 1;
    if (!converged) { enqueue_tile(p.q, nxt, gtile); *p.any_changed = 1; }
  }
}

template <int KA, int KB, bool SINGLE>
__global__ void __launch_bounds__(1024, 2) k_pool_reach(PoolReach p) {
  extern __shared__ __align__(16) unsigned char smem[];
  PoolSmemHead* hd = reinterpret_cast<PoolSmemHead*>(smem);
  int* s_mark = reinterpret_cast<int*>(smem + sizeof(PoolSmemHead));
  const unsigned n = queued_count(p.q, p.cur);
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x) {
    const int gt = p.q.list[p.cur][i];
    __syncthreads();
    if (!SINGLE) {
      load_inst(&p.inst[p.tile_inst[gt]], &hd->inst);
      __syncthreads();
    }
    const InstDesc& I = SINGLE ? p.inst0 : hd->inst;
    if (threadIdx.x == 0) p.q.flag[p.cur][gt] = 0;
    if (I.st.K == KA) reach_tile<KA>(p, I, s_mark, gt);
    else if (KB != KA && I.st.K == KB) reach_tile<KB>(p, I, s_mark, gt);
  }
}

}  // namespace lfg
