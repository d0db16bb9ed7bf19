// Push/relabel and global-relabel BFS tile passes for one 3-d lattice with
// a radius-1 neighbourhood (Full3d_6, Full3d_18, Full3d_26), tiles staged
// into shared memory by TMA (push/relabel: 32-bit capacities; BFS: any).
//
// The algorithm and the hazards are those of the 2-d staged pass
// (lf_pool_pr2d.cuh): up to `sweeps` rounds of a push phase with frozen
// heights and a relabel phase per tile visit, pushes across the tile edge
// delivered at once with global atomics, edge nodes' excess written back as
// a delta, two stage buffers so that the next tile's copies fly while the
// current one is worked on.  What differs is the box: a tile is TA x TB x 32
// nodes (a-planes x b-rows x c-columns), and one elected thread stages it
// with three bulk tensor copies:
//   * every residual plane as one 4-d box {32 x TB x TA x K};
//   * the excess as a 3-d box {32 x TB x TA};
//   * the heights with their one-node halo as a 3-d box
//     {40 x (TB + 2) x (TA + 2)} starting at (c0 - 4, b0 - 1, a0 - 1): the
//     innermost coordinate stays a multiple of 16 bytes, and the copy's zero
//     fill stands in for nodes outside the lattice, whose heights are never
//     read because no residual leads there.
// The stencil is a compile-time table in the registry's lattice order (the
// launcher checks the lattice's own stencil against it).
#pragma once

#include <cuda.h>

#include "lf_pool.cuh"
#include "lf_pool_graph.cuh"
#include "lf_pool_pr2d.cuh"
#include "lf_tile_common.cuh"

namespace lfg {

constexpr int kPr3dHaloW = 40;  // staged height row: columns c0-4 .. c0+35

// Compile-time 3-d stencils, lattice order of the kernel registry (the
// positive half first, entry k + K/2 the reverse of entry k).  Each a / b /
// c offset (-1, 0, 1) is stored as offset + 1 in two bits.
template <int K> struct Stencil3d;
template <> struct Stencil3d<6> {
  static constexpr unsigned long long kDA = 0x165ull, kDB = 0x459ull, kDC = 0x516ull;
};
template <> struct Stencil3d<18> {
  static constexpr unsigned long long kDA = 0x156aa55ull, kDB = 0x1580654a9ull,
                                      kDC = 0x464619192ull;
};
template <> struct Stencil3d<26> {
  static constexpr unsigned long long kDA = 0x156aaaa55ull, kDB = 0x15a806a540a9ull,
                                      kDC = 0x1861862492492ull;
};
template <int K> __host__ __device__ constexpr int s3_da(int k) {
  return int((Stencil3d<K>::kDA >> (2 * k)) & 3ull) - 1;
}
template <int K> __host__ __device__ constexpr int s3_db(int k) {
  return int((Stencil3d<K>::kDB >> (2 * k)) & 3ull) - 1;
}
template <int K> __host__ __device__ constexpr int s3_dc(int k) {
  return int((Stencil3d<K>::kDC >> (2 * k)) & 3ull) - 1;
}

struct PR3dMaps {
  CUtensorMap res;  // 4-d {Cp, Bp, Ap, K}
  CUtensorMap exc;  // 3-d {Cp, Bp, Ap}
  CUtensorMap h;    // 3-d {Cp, Bp, Ap}
};

template <int K, int TA, int TB>
struct PR3dLayout {
  static constexpr int NT = TA * TB * 32;
  static constexpr int HB = TB + 2;
  static constexpr int HA = TA + 2;
  static constexpr int res_bytes = K * NT * 4;
  static constexpr int exc_bytes = NT * 4;
  static constexpr int h_bytes = HA * HB * kPr3dHaloW * 4;
  static constexpr int stage_bytes = (res_bytes + exc_bytes + h_bytes + 127) / 128 * 128;
  static constexpr int tx_bytes = res_bytes + exc_bytes + h_bytes;
  // two stage buffers, two mbarriers, a neighbour-tile flag word per buffer,
  // alignment slack
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
  // blocks per SM the register budget aims at: what shared memory holds,
  // but no fewer than 48 registers a thread
  static constexpr int by_smem = (228 * 1024) / smem_bytes;
  static constexpr int by_regs = 65536 / (NT * 48);
  static constexpr int min_blocks =
      (by_smem < by_regs ? by_smem : by_regs) < 1 ? 1 : (by_smem < by_regs ? by_smem : by_regs);
};

__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap* map, int x, int y,
                                            int z, int w, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}

template <int K, int TA, int TB>
__device__ __forceinline__ void pr3d_issue(const PR3dMaps& maps, const Geo& g, int tile,
                                           unsigned stage, unsigned bar) {
  using Ly = PR3dLayout<K, TA, TB>;
  if (!tile_ok(tile, g.ntiles)) {
    mbar_expect_tx(bar, 0);
    return;
  }
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  const int a0 = ta * TA, b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_4d(stage, &maps.res, c0, b0, a0, 0, bar);
  tma_load_3d(stage + Ly::res_bytes, &maps.exc, c0, b0, a0, bar);
  tma_load_3d(stage + Ly::res_bytes + Ly::exc_bytes, &maps.h, c0 - 4, b0 - 1, a0 - 1, bar);
}

// Neighbour-tile flag of a tile offset (dta, dtb, dtc) in {-1, 0, 1}^3:
// bit (dta + 1) * 9 + (dtb + 1) * 3 + (dtc + 1); bit 13 is the tile itself.
__device__ __forceinline__ unsigned nbr_bit3(int dta, int dtb, int dtc) {
  return 1u << ((dta + 1) * 9 + (dtb + 1) * 3 + (dtc + 1));
}

// One tile visit (see pr2d_tile for e0 / my_h and the flag word s_nbr).
template <int K, int TA, int TB>
__device__ __forceinline__ void pr3d_tile(const PoolPR<int>& p, const Geo& g, int hmax, int cur,
                                          int* s_res, int* s_exc, int* s_h, int tile,
                                          const int e0, int my_h, unsigned* s_nbr) {
  constexpr int NT = TA * TB * 32;
  constexpr int HW = kPr3dHaloW;
  constexpr int HB = TB + 2;
  const int t = threadIdx.x;
  const int ic = t & 31, ib = (t >> 5) % TB, ia = t / (32 * TB);
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  const int a0 = ta * TA, b0 = tb * TB, c0 = tc * 32;
  const long long plane_ab = (long long)g.Bp * g.Cp;
  const long long gi = (a0 + ia) * plane_ab + (long long)(b0 + ib) * g.Cp + (c0 + ic);
  const int hidx = ((ia + 1) * HB + (ib + 1)) * HW + (ic + 4);
  const int nxt = cur ^ 1;
  // directions that leave the tile
  unsigned outm = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int na = ia + s3_da<K>(k), nb = ib + s3_db<K>(k), nc = ic + s3_dc<K>(k);
    if (na < 0 || na >= TA || nb < 0 || nb >= TB || nc < 0 || nc >= 32) outm |= 1u << k;
  }
  unsigned nbr = 0;  // neighbour tiles this thread's pushes reached
  for (int it = 0; it < p.sweeps; ++it) {
    int e = s_exc[t];
    // a node parked at the epoch cap no longer relabels but still pushes
    // downhill (a lower neighbour may be a deficit)
    if (e > 0) {
      int sent = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int rem = e - sent;
        if (rem <= 0) break;
        const int r = s_res[k * NT + t];
        if (r <= 0) continue;
        constexpr int half = K / 2;
        const int da = s3_da<K>(k), db = s3_db<K>(k), dc = s3_dc<K>(k);
        if (s_h[hidx + (da * HB + db) * HW + dc] >= my_h) continue;
        const int d = rem < r ? rem : r;
        s_res[k * NT + t] = r - d;
        sent += d;
        const int rk = k < half ? k + half : k - half;
        if (!((outm >> k) & 1u)) {
          const int tn = t + (da * TB + db) * 32 + dc;
          atomicAdd(&s_exc[tn], d);
          s_res[rk * NT + tn] += d;
        } else {
          // across the tile edge: delivered at once with global atomics
          const long long dn = da * plane_ab + (long long)db * g.Cp + dc;
          atomicAdd(p.res + (long long)k * g.NP + gi, -d);
          atomicAdd(p.res + (long long)rk * g.NP + gi + dn, d);
          atomicAdd(p.exc + gi + dn, d);
          const int dta = (da < 0 && ia == 0) ? -1 : (da > 0 && ia == TA - 1) ? 1 : 0;
          const int dtb = (db < 0 && ib == 0) ? -1 : (db > 0 && ib == TB - 1) ? 1 : 0;
          const int dtc = (dc < 0 && ic == 0) ? -1 : (dc > 0 && ic == 31) ? 1 : 0;
          nbr |= nbr_bit3(dta, dtb, dtc);
        }
      }
      if (sent) atomicAdd(&s_exc[t], -sent);
    }
    __syncthreads();
    e = s_exc[t];
    int act = 0;
    if (e > 0 && my_h < hmax) {
      int hmin = kHInf;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (s_res[k * NT + t] > 0) {
          const int hn = s_h[hidx + (s3_da<K>(k) * HB + s3_db<K>(k)) * HW + s3_dc<K>(k)];
          hmin = hn < hmin ? hn : hmin;
        }
      }
      if (hmin >= my_h) {
        my_h = (hmin >= hmax - 1) ? hmax : hmin + 1;
        s_h[hidx] = my_h;
      }
      act = my_h < hmax;
    }
    // after the last sweep no vote and no barrier: the write-back below
    // reads only this node's own excess and residuals, final since the
    // barrier after the push phase (the relabel phase writes heights only)
    if (it + 1 == p.sweeps) break;
    if (!__syncthreads_or(act)) break;
  }
  const int ef = s_exc[t];
  if (outm) atomicAdd(&p.exc[gi], ef - e0);
  else p.exc[gi] = ef;
#pragma unroll
  for (int k = 0; k < K; ++k)  // edges across the tile edge were updated by their pushes
    if (!((outm >> k) & 1u)) p.res[(long long)k * g.NP + gi] = s_res[k * NT + t];
  p.h[gi] = my_h;
  nbr = __reduce_or_sync(0xffffffffu, nbr);
  if (ic == 0 && nbr) atomicOr(s_nbr, nbr);
  // the buffer's next contents come from the async proxy: order this
  // visit's shared-memory accesses before them
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const int still = ef > 0 && my_h < hmax;
  const bool again = __syncthreads_or(still);
  if (t < 27 && t != 13) {
    const unsigned f = *s_nbr;
    if ((f >> t) & 1u) {
      // a bit is set only by a push, which never leaves the lattice
      const int dta = t / 9 - 1, dtb = (t / 3) % 3 - 1, dtc = t % 3 - 1;
      enqueue_tile(p.q, nxt, ((ta + dta) * g.ntb + (tb + dtb)) * g.ntc + (tc + dtc));
    }
  }
  if (again && t == 0) enqueue_tile(p.q, nxt, tile);
}

// One 3-d lattice (the pool of one), no section mask, 32-bit capacities,
// one launch per pass.  `fault` (global) records a copy that did not land
// in time (1) or a queued tile id out of range (2).
template <int K, int TA, int TB>
__global__ void __launch_bounds__(TA * TB * 32, PR3dLayout<K, TA, TB>::min_blocks)
    k_pool_pr3d(const __grid_constant__ PR3dMaps maps, const __grid_constant__ PoolPR<int> p,
                unsigned long long* fault) {
  using Ly = PR3dLayout<K, TA, TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);  // two mbarriers, 8 bytes apart
  // neighbour-tile flags of the visit on each buffer: a word is cleared two
  // visits after its last readers, who have passed two barriers since
  unsigned* s_nbr = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const Geo& g = p.inst0.g;
  const int cur = p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  const int hmax = p.inst0.hmax;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = p.inst0.done != 0;
  if (threadIdx.x == 0 && !done) pr3d_issue<K, TA, TB>(maps, g, list[blockIdx.x], stage0, bar0);
  unsigned phases = 0;  // bit b: parity of the next phase of buffer b
  unsigned buf = 0;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x, buf ^= 1) {
    const int gt = list[i];
    if (threadIdx.x == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[0], 1ull);
      s_nbr[buf] = 0;
    }
    if (done) continue;
    // the next tile of this CTA: its copies fly while this one is worked on
    // (the other buffer was released by the barrier that ended its visit)
    const unsigned nx = i + gridDim.x;
    if (threadIdx.x == 0 && nx < n)
      pr3d_issue<K, TA, TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                            bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    // this node's excess and height as staged, read before the barrier that
    // opens the visit
    unsigned char* stg = smem + buf * Ly::stage_bytes;
    const int e0 = reinterpret_cast<const int*>(stg + Ly::res_bytes)[threadIdx.x];
    const int ia = threadIdx.x / (32 * TB), ib = (threadIdx.x >> 5) % TB, ic = threadIdx.x & 31;
    const int h0 = reinterpret_cast<const int*>(stg + Ly::res_bytes + Ly::exc_bytes)
        [((ia + 1) * Ly::HB + (ib + 1)) * kPr3dHaloW + ic + 4];
    if (__syncthreads_or(!ok)) {
      // a copy did not land: record it, wait (bounded) for the copies still
      // in flight so that none lands after the CTA is gone, and stop
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
    pr3d_tile<K, TA, TB>(p, g, hmax, cur, reinterpret_cast<int*>(stg),
                         reinterpret_cast<int*>(stg + Ly::res_bytes),
                         reinterpret_cast<int*>(stg + Ly::res_bytes + Ly::exc_bytes), gt, e0, h0,
                         s_nbr + buf);
  }
}

// ------------------------------------------------------------ 3-d BFS
//
// The relaxation of the 2-d staged BFS (lf_pool_bfs2d.cuh) on 4 x TB x 32
// tiles: exact distance to the nearest deficit along residual edges,
// iterated inside the tile until stable, rows (the c axis, directions 0 and
// K/2 of every 3-d stencil) relaxed whole by segmented warp min-scans.  One
// elected thread stages a visit with two bulk tensor copies: the heights
// with their halo (3-d box {40 x (TB + 2) x 6} from (c0 - 4, b0 - 1, a0 - 1))
// and the 64-bit masks (3-d box {32 x TB x 4}).  A changed node queues the
// tiles that hold its neighbours across the tile edge.

struct BFS3dMaps {
  CUtensorMap h;     // 3-d {Cp, Bp, Ap}, 32-bit
  CUtensorMap mask;  // 3-d {Cp, Bp, Ap}, 64-bit
};

template <int TA, int TB>
struct BFS3dLayout {
  static constexpr int NT = TA * TB * 32;
  static constexpr int HB = TB + 2;
  static constexpr int h_bytes = (TA + 2) * HB * kPr3dHaloW * 4;
  static constexpr int mask_off = (h_bytes + 127) / 128 * 128;
  static constexpr int mask_bytes = NT * 8;
  static constexpr int stage_bytes = (mask_off + mask_bytes + 127) / 128 * 128;
  static constexpr int tx_bytes = h_bytes + mask_bytes;
  // two stage buffers, two mbarriers, an edge-flag word per buffer, alignment slack
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
};

template <int TA, int TB>
__device__ __forceinline__ void bfs3d_issue(const BFS3dMaps& maps, const Geo& g, int tile,
                                            unsigned stage, unsigned bar) {
  using Ly = BFS3dLayout<TA, TB>;
  if (!tile_ok(tile, g.ntiles)) {
    mbar_expect_tx(bar, 0);
    return;
  }
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  const int a0 = ta * TA, b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_3d(stage, &maps.h, c0 - 4, b0 - 1, a0 - 1, bar);
  tma_load_3d(stage + Ly::mask_off, &maps.mask, c0, b0, a0, bar);
}

template <int K, int TA, int TB>
__device__ __forceinline__ void bfs3d_tile(const PoolBFS& p, const Geo& g, int cur,
                                           unsigned char* stage, unsigned* s_flags, int tile,
                                           int my_h, const uint64_t m) {
  constexpr int HW = kPr3dHaloW;
  constexpr int HB = TB + 2;
  int* s_h = reinterpret_cast<int*>(stage);
  const int t = threadIdx.x;
  const int ic = t & 31, ib = (t >> 5) % TB, ia = t / (32 * TB);
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  const long long gi = ((long long)(ta * TA + ia) * g.Bp + (tb * TB + ib)) * g.Cp + (tc * 32 + ic);
  const int hidx = ((ia + 1) * HB + (ib + 1)) * HW + (ic + 4);
  const int nxt = cur ^ 1;
  // the row directions of every 3-d stencil: (0, 0, 1) is entry 0,
  // (0, 0, -1) entry K/2
  constexpr int kr = 0, kl = K / 2;
  const bool can_l = (m >> kl) & 1, can_r = (m >> kr) & 1;
  bool changed = false;
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int best = my_h;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((m >> k) & 1) {
        const int hn = s_h[hidx + (s3_da<K>(k) * HB + s3_db<K>(k)) * HW + s3_dc<K>(k)] + 1;
        best = hn < best ? hn : best;
      }
    }
    // after the first iteration the row is consistent along its row edges,
    // and stays so while no node of the row improves
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
    if (!__syncthreads_or(c)) {
      converged = 1;
      break;
    }
  }
  if (changed) p.h[gi] = my_h;
  // tiles that hold the neighbours of changed nodes across the tile edge
  unsigned bits = 0;
  if (changed) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int da = s3_da<K>(k), db = s3_db<K>(k), dc = s3_dc<K>(k);
      const int dta = (da < 0 && ia == 0) ? -1 : (da > 0 && ia == TA - 1) ? 1 : 0;
      const int dtb = (db < 0 && ib == 0) ? -1 : (db > 0 && ib == TB - 1) ? 1 : 0;
      const int dtc = (dc < 0 && ic == 0) ? -1 : (dc > 0 && ic == 31) ? 1 : 0;
      if (dta || dtb || dtc) bits |= nbr_bit3(dta, dtb, dtc);
    }
  }
  bits = __reduce_or_sync(0xffffffffu, bits);
  if (ic == 0 && bits) atomicOr(s_flags, bits);
  // the buffer's next contents come from the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const unsigned f = *s_flags;
  if (t < 27 && t != 13 && ((f >> t) & 1u)) {
    const int a = ta + t / 9 - 1, b = tb + (t / 3) % 3 - 1, c = tc + t % 3 - 1;
    if (a >= 0 && a < g.nta && b >= 0 && b < g.ntb && c >= 0 && c < g.ntc)
      enqueue_tile(p.q, nxt, (a * g.ntb + b) * g.ntc + c);
  }
  if (t == 0) {
    if (f) *p.any_changed = 1;
    if (!converged) {
      enqueue_tile(p.q, nxt, tile);
      *p.any_changed = 1;
    }
  }
}

// One 3-d lattice (the pool of one), one launch per pass.  `fault` as for
// k_pool_pr3d.
template <int K, int TA, int TB>
__global__ void __launch_bounds__(TA * TB * 32, 1536 / (TA * TB * 32))
    k_pool_bfs3d(const __grid_constant__ BFS3dMaps maps, const __grid_constant__ PoolBFS p,
                 unsigned long long* fault) {
  using Ly = BFS3dLayout<TA, TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);  // two mbarriers, 8 bytes apart
  // edge flags of the visit on each buffer: a word is cleared two visits
  // after its last readers, who have passed two barriers since
  unsigned* s_flags = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const Geo& g = p.inst0.g;
  const int cur = p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = p.inst0.done != 0;
  if (threadIdx.x == 0 && !done) bfs3d_issue<TA, TB>(maps, g, list[blockIdx.x], stage0, bar0);
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
      bfs3d_issue<TA, TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                          bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    unsigned char* stg = smem + buf * Ly::stage_bytes;
    const int ia = threadIdx.x / (32 * TB), ib = (threadIdx.x >> 5) % TB, ic = threadIdx.x & 31;
    const int h0 = reinterpret_cast<const int*>(stg)[((ia + 1) * Ly::HB + (ib + 1)) * kPr3dHaloW +
                                                      ic + 4];
    const uint64_t m = reinterpret_cast<const uint64_t*>(stg + Ly::mask_off)[threadIdx.x];
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
    bfs3d_tile<K, TA, TB>(p, g, cur, stg, s_flags + buf, gt, h0, m);
  }
}

}  // namespace lfg
