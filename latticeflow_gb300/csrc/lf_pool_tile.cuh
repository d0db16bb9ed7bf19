// Tile work of the pool kernels: push/relabel, BFS relabel, forward closure.
//
// Each persistent CTA pops one queued tile at a time, copies the tile's
// lattice descriptor into shared memory and works on the tile:
//
// push/relabel (one CTA stages all residual planes, the excess and the
// heights with a halo in shared memory, then runs up to `sweeps` rounds of)
//   push:    every node with excess sends flow to lower neighbours with
//            residual capacity, lowest direction index first; heights are
//            frozen during the phase, so an edge carries flow one way only and
//            the only shared update is the atomic excess add;
//   relabel: a node that still has excess and no lower residual neighbour
//            moves to one above its lowest residual neighbour, capped at the
//            lattice's epoch limit;
// until no node of the tile is active.  Flow pushed across the tile edge is
// delivered at once with global atomics (the edge's residual, the reverse
// edge's residual and the neighbour's excess) and queues the neighbour tile;
// edge nodes write back their excess as a delta for the same reason.  Stale halo heights can leave
// labels invalid; the next global relabel recomputes them exactly, and the
// final answer depends only on the residual graph, never on labels.
//
// BFS relabel: exact distance to the nearest deficit node along residual
// edges, iterated inside the tile until stable; a changed edge node queues
// the neighbour tiles.  Forward closure: marks spread along residual edges.
#pragma once

#include "lf_pool.cuh"
#include "lf_tile_common.cuh"

namespace lfg {

struct alignas(16) PoolSmemHead {
  InstDesc inst;
  int slot;
  unsigned nbr;  // neighbour tiles reached by pushes of the current visit
  int hoff[kMaxKDev];
  int toff[kMaxKDev];
};

__device__ __forceinline__ void load_inst(const InstDesc* src, InstDesc* dst) {
  const int n = int(sizeof(InstDesc) / sizeof(int));
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
}

__device__ __forceinline__ bool outside_tile(const Geo& g, const TileCtx& x, int da, int db,
                                             int dc) {
  int na = x.ia + da, nb = x.ib + db, nc = x.ic + dc;
  return na < 0 || na >= g.TA || nb < 0 || nb >= g.TB || nc < 0 || nc >= g.TC;
}

// ------------------------------------------------------------ push/relabel

template <typename T, int K>
__device__ void pr_tile(const PoolPR<T>& p, const InstDesc& I, PoolSmemHead* hd, unsigned char* sbuf,
                        int gtile) {
  const Geo& g = I.g;
  const Stencil& st = I.st;
  const int tile = gtile - I.tile_base;
  const TileCtx x = tile_ctx(g, st, tile);
  const int NT = x.NT;
  const int t = threadIdx.x;
  const bool live = t < NT;
  const int nxt = p.cur ^ 1;
  T* res = p.res + I.res_base;
  T* exc = p.exc + I.node_base;
  int* h = p.h + I.node_base;
  T* s_res = reinterpret_cast<T*>(sbuf);
  T* s_exc = s_res + (size_t)K * NT;
  int* s_h = reinterpret_cast<int*>(s_exc + NT);
  if (t < K) {
    hd->hoff[t] = (st.da[t] * x.HBB + st.db[t]) * x.HCC + st.dc[t];
    hd->toff[t] = (st.da[t] * g.TB + st.db[t]) * g.TC + st.dc[t];
  }
  // neighbour tiles reached by this visit's pushes: bit (da+1)*9 + (db+1)*3 +
  // (dc+1) of the tile offset (every stencil's halo fits in one tile); its
  // readers of the last visit have passed the loop's barrier
  if (t == 0) hd->nbr = 0;
  load_halo_heights(g, st, x, h, s_h);
  uint64_t outm = 0;
  T e0 = 0;
  uint64_t km = 0;
  if (live) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      s_res[k * NT + t] = res[(long long)k * I.plane + x.gi];
      if (outside_tile(g, x, st.da[k], st.db[k], st.dc[k])) outm |= 1ull << k;
    }
    e0 = exc[x.gi];
    s_exc[t] = e0;
    km = p.kmask ? p.kmask[I.node_base + x.gi] : ~0ull;
  }
  __syncthreads();
  const int hmax = I.hmax;
  int my_h = live ? s_h[x.hidx] : kHInf;
  for (int it = 0; it < p.sweeps; ++it) {
    T e = live ? s_exc[t] : (T)0;
    // a node parked at the epoch cap no longer relabels but still pushes
    // downhill (a lower neighbour may be a deficit)
    if (e > 0) {
      T sent = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (!((km >> k) & 1)) continue;
        const T rem = e - sent;
        if (rem <= 0) break;
        const T r = s_res[k * NT + t];
        if (r <= 0) continue;
        if (s_h[x.hidx + hd->hoff[k]] >= my_h) continue;
        const T d = rem < r ? rem : r;
        s_res[k * NT + t] = r - d;
        sent += d;
        if (!((outm >> k) & 1)) {
          const int tn = t + hd->toff[k];
          atom_add(&s_exc[tn], d);
          s_res[st.rev[k] * NT + tn] += d;
        } else {
          // across the tile edge: delivered at once with global atomics (the
          // neighbour's tile applies only deltas to these entries too)
          atom_add(&res[(long long)k * I.plane + x.gi], (T)-d);
          const int A_ = x.a0 + x.ia + st.da[k], B_ = x.b0 + x.ib + st.db[k],
                    C_ = x.c0 + x.ic + st.dc[k];
          const long long gn = ((long long)A_ * g.Bp + B_) * g.Cp + C_;
          atom_add(&res[(long long)st.rev[k] * I.plane + gn], d);
          atom_add(&exc[gn], d);
          const int dta = A_ < x.a0 ? -1 : A_ >= x.a0 + g.TA ? 1 : 0;
          const int dtb = B_ < x.b0 ? -1 : B_ >= x.b0 + g.TB ? 1 : 0;
          const int dtc = C_ < x.c0 ? -1 : C_ >= x.c0 + g.TC ? 1 : 0;
          atomicOr(&hd->nbr, 1u << ((dta + 1) * 9 + (dtb + 1) * 3 + (dtc + 1)));
        }
      }
      if (sent) atom_add(&s_exc[t], (T)-sent);
    }
    __syncthreads();
    e = live ? s_exc[t] : (T)0;
    int act = 0;
    if (e > 0 && my_h < hmax) {
      int hmin = kHInf;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (((km >> k) & 1) && s_res[k * NT + t] > 0) {
          const int hn = s_h[x.hidx + hd->hoff[k]];
          hmin = hn < hmin ? hn : hmin;
        }
      }
      if (hmin >= my_h) {
        my_h = (hmin >= hmax - 1) ? hmax : hmin + 1;
        s_h[x.hidx] = my_h;
      }
      act = my_h < hmax;
    }
    // after the last sweep no vote and no barrier: the write-back below
    // reads only this node's own excess and residuals, final since the
    // barrier after the push phase (the relabel phase writes heights only)
    if (it + 1 == p.sweeps) break;
    if (!__syncthreads_or(act)) break;
  }
  int still = 0;
  if (live) {
    const T ef = s_exc[t];
    if (outm) atom_add(&exc[x.gi], (T)(ef - e0));
    else exc[x.gi] = ef;
#pragma unroll
    for (int k = 0; k < K; ++k)  // edges across the tile edge were updated by their pushes
      if (!((outm >> k) & 1)) res[(long long)k * I.plane + x.gi] = s_res[k * NT + t];
    h[x.gi] = my_h;
    still = ef > 0 && my_h < hmax;
  }
  const bool again = __syncthreads_or(still);
  // each neighbour tile reached is queued once (27 threads, bit 13 = this tile)
  if (t < 27 && t != 13 && ((hd->nbr >> t) & 1u)) {
    const int da = t / 9 - 1, db = (t / 3) % 3 - 1, dc = t % 3 - 1;
    const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
    enqueue_tile(p.q, nxt, I.tile_base + ((ta + da) * g.ntb + (tb + db)) * g.ntc + (tc + dc));
  }
  if (again && t == 0) enqueue_tile(p.q, nxt, gtile);
}

// SINGLE: the pool holds one lattice, whose descriptor is a kernel parameter
// (constant bank); otherwise the tile's descriptor is copied to shared memory.
template <typename T, int KA, int KB, bool SINGLE>
__device__ __forceinline__ void pool_pr_body(const PoolPR<T>& p) {
  extern __shared__ __align__(16) unsigned char smem[];
  PoolSmemHead* hd = reinterpret_cast<PoolSmemHead*>(smem);
  unsigned char* sbuf = smem + sizeof(PoolSmemHead);
  const unsigned n = queued_count(p.q, p.cur);
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x) {
    const int gt = p.q.list[p.cur][i];
    __syncthreads();  // the previous tile is done with shared memory
    if (!SINGLE) {
      load_inst(&p.inst[p.tile_inst[gt]], &hd->inst);
      __syncthreads();
    }
    const InstDesc& I = SINGLE ? p.inst0 : hd->inst;
    if (threadIdx.x == 0) {
      p.q.flag[p.cur][gt] = 0;
      atomicAdd(&p.counters[0], 1ull);
    }
    if (I.done) continue;
    if (I.st.K == KA) pr_tile<T, KA>(p, I, hd, sbuf, gt);
    else if (KB != KA && I.st.K == KB) pr_tile<T, KB>(p, I, hd, sbuf, gt);
  }
}

// 32-bit capacities, at most 8 directions: at most 40 registers, so three
// 512-thread tiles share an SM (measured: push/relabel passes 11% faster
// than at 60 registers).
template <int KA, int KB, bool SINGLE>
__global__ void __maxnreg__(40) k_pool_pr(PoolPR<int> p) {
  pool_pr_body<int, KA, KB, SINGLE>(p);
}

// 64-bit capacities or larger kernels: no register cap (the cap spills to
// local memory there).
template <typename T, int KA, int KB, bool SINGLE>
__global__ void __launch_bounds__(1024) k_pool_pr_wide(PoolPR<T> p) {
  pool_pr_body<T, KA, KB, SINGLE>(p);
}

}  // namespace lfg
