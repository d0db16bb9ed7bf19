// Push/relabel tile pass specialised for one 2-d lattice with a 3x3
// neighbourhood (Full2d_4, Full2d_8) and 32-bit capacities, tiles staged
// into shared memory by TMA.
//
// Same algorithm as pr_tile (lf_pool_tile.cuh): up to `sweeps` rounds of a
// push phase with frozen heights and a relabel phase per tile visit, pushes
// across the tile edge delivered at once with global atomics.  What differs
// is how the work maps onto the SM:
//   * the stencil is a compile-time table (offsets become immediates in the
//     shared-memory addresses, the tile-edge tests fold to a few predicates);
//   * one elected thread stages a visit's tile with three bulk tensor copies
//     (cp.async.bulk.tensor): every residual plane as one 3-d box
//     {32 x TB x K}, the excess as a 2-d box {32 x TB}, the heights with
//     their one-node halo as a 2-d box {40 x (TB + 2)} starting at column
//     c0 - 4 (the innermost coordinate stays a multiple of 16 bytes; the
//     copy's zero fill stands in for nodes outside the lattice, whose
//     heights are never read because no residual leads there);
//   * two stage buffers: while the CTA works on one tile, the copies of the
//     next tile it will take from the queue are already in flight.
// A prefetched tile can only be staler than one loaded at the start of its
// visit, and staleness is safe: its excess and its residuals across the
// tile edge only grow through other tiles' pushes (the visit writes those
// back as deltas), and its interior belongs to this visit alone (a tile sits
// at most once in a pass's list).
//
// Every wait on a copy is bounded; a CTA whose copies do not land in time
// records the fault (the host turns it into an error) and returns once its
// copies have landed or a second bound has passed.
#pragma once

#include <cuda.h>

#include "lf_pool.cuh"
#include "lf_tile_common.cuh"

namespace lfg {

// Compile-time 2-d stencils, lattice order of the kernel registry: the
// positive half first, entry k + K/2 the reverse of entry k.  Each row /
// column offset (-1, 0, 1) is stored as offset + 1 in two bits.
template <int K> struct Stencil2d;
template <> struct Stencil2d<4> {  // (0,1) (1,0) (0,-1) (-1,0)
  static constexpr unsigned kDB = (1u << 0) | (2u << 2) | (1u << 4) | (0u << 6);
  static constexpr unsigned kDC = (2u << 0) | (1u << 2) | (0u << 4) | (1u << 6);
};
template <> struct Stencil2d<8> {  // (0,1) (1,-1) (1,0) (1,1) (0,-1) (-1,1) (-1,0) (-1,-1)
  static constexpr unsigned kDB = (1u << 0) | (2u << 2) | (2u << 4) | (2u << 6) |
                                  (1u << 8) | (0u << 10) | (0u << 12) | (0u << 14);
  static constexpr unsigned kDC = (2u << 0) | (0u << 2) | (1u << 4) | (2u << 6) |
                                  (0u << 8) | (2u << 10) | (1u << 12) | (0u << 14);
};
template <int K> __host__ __device__ constexpr int s2_db(int k) {
  return int((Stencil2d<K>::kDB >> (2 * k)) & 3u) - 1;
}
template <int K> __host__ __device__ constexpr int s2_dc(int k) {
  return int((Stencil2d<K>::kDC >> (2 * k)) & 3u) - 1;
}

constexpr int kPr2dHaloW = 40;  // staged height row: columns c0-4 .. c0+35

// tensor maps of one lattice's residual planes, excess and heights
struct PR2dMaps {
  CUtensorMap res;
  CUtensorMap exc;
  CUtensorMap h;
};

// Where a lattice lives in the pools, as the 2-d passes need it.
struct Lat2d {
  int ntc, ntb, Cp;  // tiles per tile row, tile rows, padded row length
  long long plane;   // elements between two of its residual planes
  long long node_base, res_base;
  int tile_base;
};

// The same fields of a lattice alone in its pool, read from its geometry
// (kernel parameters) where they are needed; every base is 0.
__device__ __forceinline__ int lat_ntc(const Geo& g) { return g.ntc; }
__device__ __forceinline__ int lat_ntb(const Geo& g) { return g.ntb; }
__device__ __forceinline__ int lat_Cp(const Geo& g) { return g.Cp; }
__device__ __forceinline__ long long lat_plane(const Geo& g) { return g.NP; }
__device__ __forceinline__ long long lat_node_base(const Geo&) { return 0; }
__device__ __forceinline__ long long lat_res_base(const Geo&) { return 0; }
__device__ __forceinline__ int lat_tile_base(const Geo&) { return 0; }
__device__ __forceinline__ int lat_ntc(const Lat2d& L) { return L.ntc; }
__device__ __forceinline__ int lat_ntb(const Lat2d& L) { return L.ntb; }
__device__ __forceinline__ int lat_Cp(const Lat2d& L) { return L.Cp; }
__device__ __forceinline__ long long lat_plane(const Lat2d& L) { return L.plane; }
__device__ __forceinline__ long long lat_node_base(const Lat2d& L) { return L.node_base; }
__device__ __forceinline__ long long lat_res_base(const Lat2d& L) { return L.res_base; }
__device__ __forceinline__ int lat_tile_base(const Lat2d& L) { return L.tile_base; }

__device__ __forceinline__ Lat2d lat2d_of(const InstDesc& I) {
  Lat2d L;
  L.ntc = I.g.ntc;
  L.ntb = I.g.ntb;
  L.Cp = I.g.Cp;
  L.plane = I.plane;
  L.node_base = I.node_base;
  L.res_base = I.res_base;
  L.tile_base = I.tile_base;
  return L;
}

template <int K, int TB>
struct PR2dLayout {
  static constexpr int NT = TB * 32;
  static constexpr int HR = TB + 2;
  static constexpr int res_bytes = K * NT * 4;
  static constexpr int exc_bytes = NT * 4;
  static constexpr int h_bytes = HR * kPr2dHaloW * 4;
  static constexpr int stage_bytes = (res_bytes + exc_bytes + h_bytes + 127) / 128 * 128;
  static constexpr int tx_bytes = res_bytes + exc_bytes + h_bytes;
  // two stage buffers, two mbarriers, a neighbour-tile flag word per buffer,
  // alignment slack
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
};

// ------------------------------------------------------------ PTX helpers

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap* map, int x, int y,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y,
                                            int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// ------------------------------------------------------------ the pass

constexpr int kPr2dWaitLimit = 1 << 20;  // try_wait rounds before a copy counts as lost

// A tile id taken from a queue must name a tile of the lattice; one that does
// not is recorded (fault flag 2) and skipped: its copies are not issued (the
// stage barrier's phase is completed by an arrival without bytes) and it is
// not visited.
__device__ __forceinline__ bool tile_ok(int gt, int ntiles) {
  return (unsigned)gt < (unsigned)ntiles;
}

// Neighbour-tile flag of a tile offset (dtb, dtc) in {-1, 0, 1}^2, not both
// 0: bit 0 up, 1 down, 2 left, 3 right, 4 up-left, 5 up-right, 6 down-left,
// 7 down-right (the layout of bfs2d_edge_bits).
__device__ __forceinline__ unsigned nbr_bit(int dtb, int dtc) {
  const int code = (dtb + 1) * 3 + (dtc + 1);  // 0..8, 4 = the tile itself
  // code: 0 (-1,-1) 1 (-1,0) 2 (-1,1) 3 (0,-1) 5 (0,1) 6 (1,-1) 7 (1,0) 8 (1,1)
  constexpr unsigned kBit = (4u << 0) | (0u << 3) | (5u << 6) | (2u << 9) | (0u << 12) |
                            (3u << 15) | (6u << 18) | (1u << 21) | (7u << 24);
  return code == 4 ? 0u : 1u << ((kBit >> (3 * code)) & 7u);
}

template <int K, int TB>
__device__ __forceinline__ void pr2d_issue(const PR2dMaps& maps, const Geo& g, int tile,
                                           unsigned stage, unsigned bar) {
  using Ly = PR2dLayout<K, TB>;
  if (!tile_ok(tile, g.ntiles)) {
    mbar_expect_tx(bar, 0);
    return;
  }
  const int tc = tile % g.ntc, tb = tile / g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_3d(stage, &maps.res, c0, b0, 0, bar);
  tma_load_2d(stage + Ly::res_bytes, &maps.exc, c0, b0, bar);
  tma_load_2d(stage + Ly::res_bytes + Ly::exc_bytes, &maps.h, c0 - 4, b0 - 1, bar);
}

// e0 / my_h: the node's staged excess and height, read by every thread
// before the barrier that opens the visit (once a visit runs, neighbours
// push into s_exc at once, and a later read would miss the flow they sent,
// which the delta write-back of the excess needs).
//
// LAT: Lat2d for a lattice that is one of many in the pools (its nodes,
// residual planes and tiles start at its bases; tile ids in the queue are
// global), Geo for a lattice alone in its pool (all bases 0).
//
// T: capacity type (int for binary cuts, long long for parametric / TV
// section solves); km: the node's staged section mask (bit k: direction k
// stays inside the node's section), or null when the pass has none.
//
// s_nbr: the visit's neighbour-tile flags (bit layout of bfs2d_edge_bits),
// zero at entry.  A push across the tile edge only sets the bit of the tile
// it reached; each flagged tile is queued once after the visit's last
// barrier, so no pushing thread waits on a global queue atomic.
template <int K, int TB, class LAT, class T = int>
__device__ __forceinline__ void pr2d_tile(const PoolPR<T>& p, const LAT& L, int hmax, int cur,
                                          T* s_res, T* s_exc, int* s_h, int tile,
                                          const T e0, int my_h, unsigned* s_nbr,
                                          const uint64_t* s_km = nullptr) {
  constexpr int NT = TB * 32;
  constexpr int HW = kPr2dHaloW;
  const int t = threadIdx.x;
  const int ic = t & 31, ib = t >> 5;
  const int tc = tile % lat_ntc(L), tb = tile / lat_ntc(L);
  const int b0 = tb * TB, c0 = tc * 32;
  const long long gi = (long long)(b0 + ib) * lat_Cp(L) + (c0 + ic) + lat_node_base(L);
  T* const res = p.res + (lat_res_base(L) - lat_node_base(L));  // res + k plane + gi
  const uint64_t km = s_km ? s_km[t] : ~0ull;
  const int tile_g = lat_tile_base(L) + tile;
  const int hidx = (ib + 1) * HW + (ic + 4);
  const int nxt = cur ^ 1;
  // directions that leave the tile
  unsigned outm = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int nb = ib + s2_db<K>(k), nc = ic + s2_dc<K>(k);
    if (nb < 0 || nb >= TB || nc < 0 || nc >= 32) outm |= 1u << k;
  }
  unsigned nbr = 0;  // neighbour tiles this thread's pushes reached
  for (int it = 0; it < p.sweeps; ++it) {
    T e = s_exc[t];
    // a node parked at the epoch cap no longer relabels but still pushes
    // downhill (a lower neighbour may be a deficit)
    if (e > 0) {
      T sent = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const T rem = e - sent;
        if (rem <= 0) break;
        if (!((km >> k) & 1)) continue;
        const T r = s_res[k * NT + t];
        if (r <= 0) continue;
        if (s_h[hidx + s2_db<K>(k) * HW + s2_dc<K>(k)] >= my_h) continue;
        const T d = rem < r ? rem : r;
        s_res[k * NT + t] = r - d;
        sent += d;
        constexpr int half = K / 2;
        const int rk = k < half ? k + half : k - half;
        if (!((outm >> k) & 1u)) {
          const int tn = t + s2_db<K>(k) * 32 + s2_dc<K>(k);
          atom_add(&s_exc[tn], d);
          s_res[rk * NT + tn] += d;
        } else {
          // across the tile edge: delivered at once with global atomics
          T* r0 = res + gi;
          atom_add(r0 + (long long)k * lat_plane(L), (T)-d);
          const long long dn = (long long)s2_db<K>(k) * lat_Cp(L) + s2_dc<K>(k);
          atom_add(r0 + (long long)rk * lat_plane(L) + dn, d);
          atom_add(p.exc + gi + dn, d);
          // the neighbour's tile: one tile row / column over where the
          // neighbour leaves this tile's rows / columns
          const int dtb = (s2_db<K>(k) < 0 && ib == 0) ? -1 : (s2_db<K>(k) > 0 && ib == TB - 1) ? 1 : 0;
          const int dtc = (s2_dc<K>(k) < 0 && ic == 0) ? -1 : (s2_dc<K>(k) > 0 && ic == 31) ? 1 : 0;
          nbr |= nbr_bit(dtb, dtc);
        }
      }
      if (sent) atom_add(&s_exc[t], (T)-sent);
    }
    __syncthreads();
    e = s_exc[t];
    int act = 0;
    if (e > 0 && my_h < hmax) {
      int hmin = kHInf;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (((km >> k) & 1) && s_res[k * NT + t] > 0) {
          const int hn = s_h[hidx + s2_db<K>(k) * HW + s2_dc<K>(k)];
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
  const T ef = s_exc[t];
  if (outm) atom_add(&p.exc[gi], (T)(ef - e0));
  else p.exc[gi] = ef;
#pragma unroll
  for (int k = 0; k < K; ++k)  // edges across the tile edge were updated by their pushes
    if (!((outm >> k) & 1u)) res[(long long)k * lat_plane(L) + gi] = s_res[k * NT + t];
  p.h[gi] = my_h;
  nbr = __reduce_or_sync(0xffffffffu, nbr);
  if (ic == 0 && nbr) atomicOr(s_nbr, nbr);
  // the buffer's next contents come from the async proxy: order this
  // visit's shared-memory accesses before them
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const int still = ef > 0 && my_h < hmax;
  const bool again = __syncthreads_or(still);
  if (t < 8) {
    const unsigned f = *s_nbr;
    if ((f >> t) & 1u) {
      const int dtb = (t == 0 || t == 4 || t == 5) ? -1 : (t == 1 || t == 6 || t == 7) ? 1 : 0;
      const int dtc = (t == 2 || t == 4 || t == 6) ? -1 : (t == 3 || t == 5 || t == 7) ? 1 : 0;
      // a bit is set only by a push, which never leaves the lattice
      enqueue_tile(p.q, nxt, tile_g + dtb * lat_ntc(L) + dtc);
    }
  }
  if (again && t == 0) enqueue_tile(p.q, nxt, tile_g);
}

// One lattice (the pool of one), no section mask, 32-bit capacities.
// `fault` (global) records a copy that did not land in time.  REGS caps the
// registers per thread: 40 keeps three 512-thread tiles on an SM without
// spills, 32 fits four (with a few spilled values for 8 directions).
// ctl: null for a launch of its own (list, height cap and finished flag from
// the parameters); else the pass runs inside a device-side loop of passes
// (a CUDA graph) and reads the list to consume from ctl[0] and the height
// cap and finished flag from the lattice's descriptor in device memory.
template <int K, int TB, int REGS>
__global__ void __maxnreg__(REGS)
    k_pool_pr2d(const __grid_constant__ PR2dMaps maps, PoolPR<int> p,
                unsigned long long* fault, const int* ctl) {
  using Ly = PR2dLayout<K, TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);  // two mbarriers, 8 bytes apart
  // neighbour-tile flags of the visit on each buffer: a word is cleared two
  // visits after its last readers, who have passed two barriers since
  unsigned* s_nbr = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const Geo& g = p.inst0.g;
  const int cur = ctl ? *ctl : p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  const int hmax = ctl ? p.inst[0].hmax : p.inst0.hmax;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = (ctl ? p.inst[0].done : p.inst0.done) != 0;
  if (threadIdx.x == 0 && !done) pr2d_issue<K, TB>(maps, g, list[blockIdx.x], stage0, bar0);
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
      pr2d_issue<K, TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                        bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    // this node's excess and height as staged (see pr2d_tile)
    unsigned char* st = smem + buf * Ly::stage_bytes;
    const int e0 = reinterpret_cast<const int*>(st + Ly::res_bytes)[threadIdx.x];
    const int h0 = reinterpret_cast<const int*>(st + Ly::res_bytes + Ly::exc_bytes)
        [((threadIdx.x >> 5) + 1) * kPr2dHaloW + (threadIdx.x & 31) + 4];
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
    pr2d_tile<K, TB>(p, g, hmax, cur, reinterpret_cast<int*>(st),
                            reinterpret_cast<int*>(st + Ly::res_bytes),
                            reinterpret_cast<int*>(st + Ly::res_bytes + Ly::exc_bytes), gt, e0, h0,
                            s_nbr + buf);
  }
}

// ------------------------------------------------ one warp per tile
//
// The same pass with a whole tile per warp: lane c owns column c of the tile
// (TB nodes, one per row), the phases of a sweep are separated by warp
// syncs instead of block barriers, and the warps of a block work on
// different tiles, each with its own two stage buffers and mbarriers.  A
// warp's stalls then hold up only its own tile.  Pushes inside the tile go
// to nodes of the same lane (vertical) or of the lanes beside it, by
// shared-memory atomics on the excess; as in pr2d_tile, a push from j to a
// lower neighbour is the only write of that neighbour's reverse residual in
// the phase (the neighbour pushes only further down).

template <int K, int TB>
struct PR2dWarpLayout {
  using Ly = PR2dLayout<K, TB>;
  // two stage buffers, then two mbarriers (8 bytes each); 128-aligned
  static constexpr int per_warp = (2 * Ly::stage_bytes + 16 + 127) / 128 * 128;
};

template <int K, int TB>
__device__ __forceinline__ void pr2d_tile_warp(const PoolPR<int>& p, const Geo& g, int hmax,
                                               int cur, int* s_res, int* s_exc, int* s_h,
                                               int tile, const int* e0) {
  constexpr int NT = TB * 32;
  constexpr int HW = kPr2dHaloW;
  constexpr int half = K / 2;
  const int lane = threadIdx.x & 31;
  const int tc = tile % g.ntc, tb = tile / g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  const int nxt = cur ^ 1;
  unsigned nbr = 0;  // neighbour tiles this lane's pushes reached
  // a node's own height sits in its staged slot: only its lane writes it
  for (int it = 0; it < p.sweeps; ++it) {
    // push phase (heights frozen)
#pragma unroll 1
    for (int r = 0; r < TB; ++r) {
      const int t = r * 32 + lane;
      const int e = s_exc[t];
      if (e <= 0) continue;
      const int hidx = (r + 1) * HW + (lane + 4);
      const int hr = s_h[hidx];
      int sent = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int rem = e - sent;
        if (rem <= 0) break;
        const int rv = s_res[k * NT + t];
        if (rv <= 0) continue;
        if (s_h[hidx + s2_db<K>(k) * HW + s2_dc<K>(k)] >= hr) continue;
        const int d = rem < rv ? rem : rv;
        s_res[k * NT + t] = rv - d;
        sent += d;
        const int rk = k < half ? k + half : k - half;
        const int nb = r + s2_db<K>(k), nc = lane + s2_dc<K>(k);
        if (nb >= 0 && nb < TB && nc >= 0 && nc < 32) {
          const int tn = nb * 32 + nc;
          atomicAdd(&s_exc[tn], d);
          s_res[rk * NT + tn] += d;
        } else {
          // across the tile edge: delivered at once with global atomics
          const long long gi = (long long)(b0 + r) * g.Cp + (c0 + lane);
          const long long dn = (long long)s2_db<K>(k) * g.Cp + s2_dc<K>(k);
          atomicAdd(p.res + (long long)k * g.NP + gi, -d);
          atomicAdd(p.res + (long long)rk * g.NP + gi + dn, d);
          atomicAdd(p.exc + gi + dn, d);
          const int dtb = nb < 0 ? -1 : nb >= TB ? 1 : 0;
          const int dtc = nc < 0 ? -1 : nc >= 32 ? 1 : 0;
          nbr |= nbr_bit(dtb, dtc);
        }
      }
      if (sent) atomicAdd(&s_exc[t], -sent);
    }
    __syncwarp();
    // relabel phase
    int act = 0;
#pragma unroll 1
    for (int r = 0; r < TB; ++r) {
      const int t = r * 32 + lane;
      const int hidx = (r + 1) * HW + (lane + 4);
      int hr = s_h[hidx];
      if (s_exc[t] <= 0 || hr >= hmax) continue;
      int hmin = kHInf;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (s_res[k * NT + t] > 0) {
          const int hn = s_h[hidx + s2_db<K>(k) * HW + s2_dc<K>(k)];
          hmin = hn < hmin ? hn : hmin;
        }
      }
      if (hmin >= hr) {
        hr = (hmin >= hmax - 1) ? hmax : hmin + 1;
        s_h[hidx] = hr;
      }
      act |= hr < hmax;
    }
    __syncwarp();
    if (it + 1 == p.sweeps) break;
    if (!__any_sync(0xffffffffu, act)) break;
  }
  // write-back: interior excess and residuals as staged, edge excess as a
  // delta (other tiles' pushes arrive there by atomics), heights
  int still = 0;
#pragma unroll
  for (int r = 0; r < TB; ++r) {
    const int t = r * 32 + lane;
    const long long gi = (long long)(b0 + r) * g.Cp + (c0 + lane);
    const int ef = s_exc[t];
    const int hr = s_h[(r + 1) * HW + (lane + 4)];
    const bool edge = r == 0 || r == TB - 1 || lane == 0 || lane == 31;
    if (edge) atomicAdd(p.exc + gi, ef - e0[r]);
    else p.exc[gi] = ef;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int nb = r + s2_db<K>(k), nc = lane + s2_dc<K>(k);
      if (nb >= 0 && nb < TB && nc >= 0 && nc < 32) p.res[(long long)k * g.NP + gi] = s_res[k * NT + t];
    }
    p.h[gi] = hr;
    still |= ef > 0 && hr < hmax;
  }
  nbr = __reduce_or_sync(0xffffffffu, nbr);
  const bool again = __any_sync(0xffffffffu, still);
  // the buffer's next contents come from the async proxy: order this
  // visit's shared-memory accesses before them
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncwarp();
  if (lane < 8 && ((nbr >> lane) & 1u)) {
    const int dtb = (lane == 0 || lane == 4 || lane == 5) ? -1 : (lane == 1 || lane == 6 || lane == 7) ? 1 : 0;
    const int dtc = (lane == 2 || lane == 4 || lane == 6) ? -1 : (lane == 3 || lane == 5 || lane == 7) ? 1 : 0;
    // a bit is set only by a push, which never leaves the lattice
    enqueue_tile(p.q, nxt, tile + dtb * g.ntc + dtc);
  }
  if (again && lane == 0) enqueue_tile(p.q, nxt, tile);
}

// One lattice (the pool of one), 32-bit capacities, no section mask; W
// warps per block, each taking the queued tiles gw, gw + warps, ... in turn.
template <int K, int TB, int W>
__global__ void __launch_bounds__(W * 32)
    k_pool_pr2d_warp(const __grid_constant__ PR2dMaps maps, PoolPR<int> p,
                     unsigned long long* fault) {
  using Ly = PR2dLayout<K, TB>;
  using WL = PR2dWarpLayout<K, TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* mine = smem + warp * WL::per_warp;
  const unsigned stage0 = smem_addr(mine);
  const unsigned bar0 = smem_addr(mine + 2 * Ly::stage_bytes);
  const Geo& g = p.inst0.g;
  const int cur = p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  const unsigned gw = blockIdx.x * W + warp, nw = gridDim.x * W;
  if (gw >= n) return;  // the whole warp: no block barrier follows
  const int hmax = p.inst0.hmax;
  const bool done = p.inst0.done != 0;
  if (lane == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (lane == 0 && !done) pr2d_issue<K, TB>(maps, g, list[gw], stage0, bar0);
  unsigned phases = 0, buf = 0;
  for (unsigned i = gw; i < n; i += nw, buf ^= 1) {
    const int gt = list[i];
    if (lane == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[0], 1ull);
    }
    if (done) continue;
    const unsigned nx = i + nw;
    if (lane == 0 && nx < n)
      pr2d_issue<K, TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                        bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(bar, par, kPr2dWaitLimit));
    phases ^= 1u << buf;
    if (!ok) {
      // a copy did not land: record it, wait (bounded) for the copies still
      // in flight so that none lands after the warp is gone, and stop
      if (lane == 0) atomicExch(fault, 1ull);
      mbar_wait_bounded(bar, par, kPr2dWaitLimit);
      if (nx < n) mbar_wait_bounded(bar0 + (buf ^ 1) * 8, (phases >> (buf ^ 1)) & 1u, kPr2dWaitLimit);
      return;
    }
    if (!tile_ok(gt, g.ntiles)) {
      if (lane == 0) atomicExch(fault, 2ull);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      continue;
    }
    unsigned char* st = mine + buf * Ly::stage_bytes;
    int* s_res = reinterpret_cast<int*>(st);
    int* s_exc = reinterpret_cast<int*>(st + Ly::res_bytes);
    int* s_h = reinterpret_cast<int*>(st + Ly::res_bytes + Ly::exc_bytes);
    int e0[TB];
#pragma unroll
    for (int r = 0; r < TB; ++r) e0[r] = s_exc[r * 32 + lane];
    __syncwarp();  // every lane has read its staged excess before any push
    pr2d_tile_warp<K, TB>(p, g, hmax, cur, s_res, s_exc, s_h, gt, e0);
  }
}

// ------------------------------------------------ 64-bit, section mask

// tensor maps of one lattice for the 64-bit pass: residual planes, excess
// (int64), heights (int32), section masks (uint64)
struct PR2dMaps64 {
  CUtensorMap res;
  CUtensorMap exc;
  CUtensorMap h;
  CUtensorMap km;
};

template <int K, int TB>
struct PR2dLayout64 {
  static constexpr int NT = TB * 32;
  static constexpr int res_bytes = K * NT * 8;
  static constexpr int exc_off = res_bytes;
  static constexpr int h_off = exc_off + NT * 8;
  static constexpr int h_bytes = (TB + 2) * kPr2dHaloW * 4;
  static constexpr int km_off = (h_off + h_bytes + 127) / 128 * 128;
  static constexpr int stage_bytes = km_off + NT * 8;
  static constexpr int tx_bytes = res_bytes + NT * 8 + h_bytes + NT * 8;
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
};

template <int K, int TB>
__device__ __forceinline__ void pr2d64_issue(const PR2dMaps64& maps, const Geo& g, int tile,
                                             unsigned stage, unsigned bar) {
  using Ly = PR2dLayout64<K, TB>;
  if (!tile_ok(tile, g.ntiles)) {
    mbar_expect_tx(bar, 0);
    return;
  }
  const int tc = tile % g.ntc, tb = tile / g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, Ly::tx_bytes);
  tma_load_3d(stage, &maps.res, c0, b0, 0, bar);
  tma_load_2d(stage + Ly::exc_off, &maps.exc, c0, b0, bar);
  tma_load_2d(stage + Ly::h_off, &maps.h, c0 - 4, b0 - 1, bar);
  tma_load_2d(stage + Ly::km_off, &maps.km, c0, b0, bar);
}

// One lattice, 64-bit capacities, section mask (the parametric / TV section
// solves): the pass of k_pool_pr2d with the mask staged beside the tile.
template <int K, int TB>
__global__ void __launch_bounds__(TB * 32)
    k_pool_pr2d64(const __grid_constant__ PR2dMaps64 maps, PoolPR<long long> p,
                  unsigned long long* fault, const int* ctl) {
  using Ly = PR2dLayout64<K, TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);
  unsigned* s_nbr = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
  const unsigned stage0 = smem_addr(smem);
  const Geo& g = p.inst0.g;
  const int cur = ctl ? *ctl : p.cur;
  const unsigned n = queued_count(p.q, cur);
  const int* list = p.q.list[cur];
  if (blockIdx.x >= n) return;
  const int hmax = ctl ? p.inst[0].hmax : p.inst0.hmax;
  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar0 + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool done = (ctl ? p.inst[0].done : p.inst0.done) != 0;
  if (threadIdx.x == 0 && !done) pr2d64_issue<K, TB>(maps, g, list[blockIdx.x], stage0, bar0);
  unsigned phases = 0;
  unsigned buf = 0;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x, buf ^= 1) {
    const int gt = list[i];
    if (threadIdx.x == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[0], 1ull);
      s_nbr[buf] = 0;
    }
    if (done) continue;
    const unsigned nx = i + gridDim.x;
    if (threadIdx.x == 0 && nx < n)
      pr2d64_issue<K, TB>(maps, g, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                          bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    unsigned char* st = smem + buf * Ly::stage_bytes;
    long long* s_res = reinterpret_cast<long long*>(st);
    long long* s_exc = reinterpret_cast<long long*>(st + Ly::exc_off);
    int* s_h = reinterpret_cast<int*>(st + Ly::h_off);
    const uint64_t* s_km = reinterpret_cast<const uint64_t*>(st + Ly::km_off);
    const long long e0 = s_exc[threadIdx.x];  // before the opening barrier (see pr2d_tile)
    const int h0 = s_h[((threadIdx.x >> 5) + 1) * kPr2dHaloW + (threadIdx.x & 31) + 4];
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
    pr2d_tile<K, TB, Geo, long long>(p, g, hmax, cur, s_res, s_exc, s_h, gt, e0, h0, s_nbr + buf,
                                     s_km);
  }
}

// ------------------------------------------------------------ pools

// Stage layout of the pool pass: room for 8 residual planes whatever the
// tile's lattice has, so the excess and heights sit at fixed offsets.
template <int TB>
struct PR2dPoolLayout {
  static constexpr int NT = TB * 32;
  static constexpr int res_bytes = 8 * NT * 4;
  static constexpr int exc_off = res_bytes;
  static constexpr int h_off = exc_off + NT * 4;
  static constexpr int h_bytes = (TB + 2) * kPr2dHaloW * 4;
  static constexpr int stage_bytes = (h_off + h_bytes + 127) / 128 * 128;
  static constexpr int smem_bytes = 2 * stage_bytes + 32 + 128;
};

// A lattice's three tensor maps (residual planes, excess, heights) in the
// pool's map array (global memory, written before the launch).
template <int TB>
__device__ __forceinline__ void pr2d_pool_issue(const PoolPR<int>& p, const CUtensorMap* maps,
                                                int gt, unsigned stage, unsigned bar) {
  using Ly = PR2dPoolLayout<TB>;
  const int ii = p.tile_inst[gt];
  const InstDesc& I = p.inst[ii];
  const int K = I.st.K;
  const int tile = gt - I.tile_base;
  const int tc = tile % I.g.ntc, tb = tile / I.g.ntc;
  const int b0 = tb * TB, c0 = tc * 32;
  mbar_expect_tx(bar, K * Ly::NT * 4 + Ly::NT * 4 + Ly::h_bytes);
  tma_load_3d(stage, &maps[3 * ii], c0, b0, 0, bar);
  tma_load_2d(stage + Ly::exc_off, &maps[3 * ii + 1], c0, b0, bar);
  tma_load_2d(stage + Ly::h_off, &maps[3 * ii + 2], c0 - 4, b0 - 1, bar);
}

// Many 2-d lattices (Full2d_4 / Full2d_8, one tile height) in one pool,
// 32-bit capacities, no section mask: the same pass as k_pool_pr2d, each
// tile with its own lattice's placement, stencil, height cap and tensor
// maps.  ctl as for k_pool_pr2d (the height caps and finished flags always
// come from the descriptors in device memory).
template <int TB, int REGS>
__global__ void __maxnreg__(REGS)
    k_pool_pr2d_pool(const CUtensorMap* maps, PoolPR<int> p, unsigned long long* fault,
                     const int* ctl) {
  using Ly = PR2dPoolLayout<TB>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<unsigned long long>(smem_raw) + 127) & ~127ull);
  const unsigned bar0 = smem_addr(smem + 2 * Ly::stage_bytes);
  unsigned* s_nbr = reinterpret_cast<unsigned*>(smem + 2 * Ly::stage_bytes + 16);
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
  if (threadIdx.x == 0) pr2d_pool_issue<TB>(p, maps, list[blockIdx.x], stage0, bar0);
  unsigned phases = 0;
  unsigned buf = 0;
  for (unsigned i = blockIdx.x; i < n; i += gridDim.x, buf ^= 1) {
    const int gt = list[i];
    if (threadIdx.x == 0) {
      p.q.flag[cur][gt] = 0;
      atomicAdd(&p.counters[0], 1ull);
      s_nbr[buf] = 0;
    }
    const unsigned nx = i + gridDim.x;
    if (threadIdx.x == 0 && nx < n)
      pr2d_pool_issue<TB>(p, maps, list[nx], stage0 + (buf ^ 1) * Ly::stage_bytes,
                          bar0 + (buf ^ 1) * 8);
    const unsigned bar = bar0 + buf * 8;
    const unsigned par = (phases >> buf) & 1u;
    const bool ok = mbar_wait_bounded(bar, par, kPr2dWaitLimit);
    phases ^= 1u << buf;
    unsigned char* st = smem + buf * Ly::stage_bytes;
    int* s_res = reinterpret_cast<int*>(st);
    int* s_exc = reinterpret_cast<int*>(st + Ly::exc_off);
    int* s_h = reinterpret_cast<int*>(st + Ly::h_off);
    // this node's staged excess and height (see pr2d_tile)
    const int e0 = s_exc[threadIdx.x];
    const int h0 = s_h[((threadIdx.x >> 5) + 1) * kPr2dHaloW + (threadIdx.x & 31) + 4];
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
      pr2d_tile<8, TB>(p, L, I.hmax, cur, s_res, s_exc, s_h, tile, e0, h0, s_nbr + buf);
    else
      pr2d_tile<4, TB>(p, L, I.hmax, cur, s_res, s_exc, s_h, tile, e0, h0, s_nbr + buf);
  }
}

}  // namespace lfg
