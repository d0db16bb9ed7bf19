// Host side of the instance pool and its node-level kernels.
//
// PoolRunner::maxflow solves every lattice of the pool to a maximum preflow:
//   repeat {
//     global relabel of every unfinished lattice (BFS passes draining the
//       tile queue until no tile changes);
//     count active nodes per lattice; a lattice with none is finished;
//       the others get their epoch height cap (BFS depth + slack) and their
//       active tiles queued;
//     stop when no lattice has active nodes;
//     `launches_per_relabel` push/relabel passes draining the tile queue
//   }
// Node pools hold all lattices back to back (node_base), residual planes
// likewise (res_base); the persistent kernels take whatever tile is queued
// next, from any lattice.  Passes: the TMA-staged 2-d kernels
// (lf_pool_pr2d.cuh, lf_pool_bfs2d.cuh) for lattices with 3x3
// neighbourhoods, the generic tile kernels otherwise; one launch per pass,
// or (device_loops) the passes of a relabel / an epoch in one CUDA graph.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "lf_pool_runner.h"
#include "lf_pool_tile.cuh"

namespace lfg {

namespace {

inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

// tuning value pr_kernel -> variant of the TMA-staged push/relabel pass:
// 0 block per tile (40 registers), 1 the same with 32, 2 warp per tile
inline int pr2d_variant(int pr_kernel) {
  return pr_kernel == 2 ? 1 : pr_kernel == 3 ? 2 : 0;
}

// lattice of pool node i (node_base ascending, n entries + sentinel)
__device__ __forceinline__ int inst_of(const long long* nbase, int n, long long i) {
  int lo = 0, hi = n;  // nbase[lo] <= i < nbase[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (nbase[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

struct NodeRef {
  int inst;
  long long li;
  int a, b, c;
};

__device__ __forceinline__ NodeRef node_ref(const InstDesc* insts, const long long* nbase, int n,
                                            long long i) {
  NodeRef r;
  r.inst = inst_of(nbase, n, i);
  r.li = i - nbase[r.inst];
  const Geo& g = insts[r.inst].g;
  r.c = int(r.li % g.Cp);
  r.b = int((r.li / g.Cp) % g.Bp);
  r.a = int(r.li / ((long long)g.Cp * g.Bp));
  return r;
}

template <typename T>
__global__ void k_pool_init_heights(const InstDesc* insts, const long long* nbase, int n,
                                    long long NP, const T* exc, const uint64_t* kmask, int* h) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int in = inst_of(nbase, n, i);
  if (insts[in].done || !insts[in].active) return;
  bool part = !kmask || (kmask[i] >> 63);
  h[i] = (part && exc[i] < 0) ? 0 : kHInf;
}

template <typename T>
__global__ void k_pool_mask(const InstDesc* insts, const long long* nbase, int n, long long NP,
                            const T* res, const uint64_t* kmask, uint64_t* mask) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int in = inst_of(nbase, n, i);
  const InstDesc& I = insts[in];
  if (I.done || !I.active) return;
  long long li = i - nbase[in];
  const T* r = res + I.res_base;
  uint64_t m = 0;
  for (int k = 0; k < I.st.K; ++k)
    if (r[(long long)k * I.plane + li] > 0) m |= 1ull << k;
  if (kmask) m &= kmask[i];
  mask[i] = m;
}

// The set-up of a global relabel for a pool of one lattice in one pass:
// initial heights (0 at deficits of the lattice's sections, else kHInf),
// residual masks, and every tile queued in list 0.  Four nodes (32-bit) or
// two (64-bit) per thread, one 16-byte load per residual plane.
template <typename T>
__global__ void k_relabel_init1(const InstDesc* insts, long long NP, const T* res, const T* exc,
                                const uint64_t* kmask, int* h, uint64_t* mask, TileQueue q,
                                int tiles) {
  constexpr int VW = 16 / sizeof(T);
  using V = typename std::conditional<sizeof(T) == 4, int4, longlong2>::type;
  const InstDesc& I = insts[0];
  if (I.done || !I.active) return;
  const int K = I.st.K;
  const long long plane = I.plane;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v * VW < NP; v += stride) {
    const long long i0 = v * VW;
    uint64_t m[VW];
#pragma unroll
    for (int j = 0; j < VW; ++j) m[j] = 0;
    for (int k = 0; k < K; ++k) {
      const V r = *reinterpret_cast<const V*>(res + (long long)k * plane + i0);
      const T* rv = reinterpret_cast<const T*>(&r);
#pragma unroll
      for (int j = 0; j < VW; ++j)
        if (rv[j] > 0) m[j] |= 1ull << k;
    }
    const V e = *reinterpret_cast<const V*>(exc + i0);
    const T* ev = reinterpret_cast<const T*>(&e);
#pragma unroll
    for (int j = 0; j < VW; ++j) {
      bool part = true;
      if (kmask) {
        const uint64_t km = kmask[i0 + j];
        m[j] &= km;
        part = (km >> 63) != 0;
      }
      mask[i0 + j] = m[j];
      h[i0 + j] = (part && ev[j] < 0) ? 0 : kHInf;
    }
  }
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tiles; t += stride) {
    q.flag[0][t] = 1;
    q.list[0][t] = (int)t;
  }
  if (blockIdx.x == 0 && threadIdx.x < 4) q.ctr[threadIdx.x] = threadIdx.x == q_count_idx(0) ? tiles : 0;
}

// every tile of every unfinished lattice into list 0
__global__ void k_pool_queue_all(const InstDesc* insts, const int* tile_inst, int tiles,
                                 TileQueue q) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tiles) return;
  const InstDesc& I = insts[tile_inst[t]];
  if (I.done || !I.active) return;
  enqueue_tile(q, 0, t);
}

// Lanes of a warp that belong to the same lattice combine their count and
// maximum height first, so each warp issues one atomic per lattice it spans.
template <typename T>
__global__ void k_pool_active(const InstDesc* insts, const long long* nbase, int n, long long NP,
                              const T* exc, const int* h, TileQueue q,
                              unsigned long long* cnt, unsigned* hmx) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int inst = -1;
  unsigned hv = 0, act = 0;
  if (i < NP) {
    NodeRef r = node_ref(insts, nbase, n, i);
    const InstDesc& I = insts[r.inst];
    if (!I.done && I.active) {
      inst = r.inst;
      int hh = h[i];
      if (hh < kHInf) hv = (unsigned)hh;
      if (exc[i] > 0 && hh < kHInf) {
        act = 1;
        enqueue_tile(q, 0, I.tile_base + tile_of(I.g, r.a, r.b, r.c));
      }
    }
  }
  const unsigned peers = __match_any_sync(0xffffffffu, inst);
  const unsigned hm = __reduce_max_sync(peers, hv);
  const unsigned na = __reduce_add_sync(peers, act);
  if (inst >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) {
    if (hm) atomicMax(&hmx[inst], hm);
    if (na) atomicAdd(&cnt[inst], (unsigned long long)na);
  }
}

// The same for a pool of one lattice: no lattice lookup per node, the
// active tiles queued once per warp (a warp's 32 nodes are one tile row),
// count and maximum height combined per block.
template <typename T>
__global__ void k_pool_active1(const InstDesc* insts, long long NP, const T* exc, const int* h,
                               TileQueue q, unsigned long long* cnt, unsigned* hmx) {
  __shared__ unsigned s_max[32];
  __shared__ unsigned long long s_cnt[32];
  const InstDesc& I = insts[0];
  const bool on = !I.done && I.active;
  const Geo& g = I.g;
  unsigned hv = 0, na = 0;
  const int lane = threadIdx.x & 31;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; on && i < NP;
       i += (long long)gridDim.x * blockDim.x) {
    const int hh = h[i];
    if (hh < kHInf && (unsigned)hh > hv) hv = (unsigned)hh;
    const bool a = exc[i] > 0 && hh < kHInf;
    na += a ? 1u : 0u;
    if (__ballot_sync(0xffffffffu, a) && lane == 0) {
      const int c = int(i % g.Cp);
      const long long r = i / g.Cp;
      enqueue_tile(q, 0, I.tile_base + tile_of(g, int(r / g.Bp), int(r % g.Bp), c));
    }
  }
  hv = __reduce_max_sync(0xffffffffu, hv);
  na = __reduce_add_sync(0xffffffffu, na);
  if (lane == 0) {
    s_max[threadIdx.x >> 5] = hv;
    s_cnt[threadIdx.x >> 5] = na;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool w = threadIdx.x < (blockDim.x >> 5);
    unsigned m = w ? s_max[threadIdx.x] : 0u;
    unsigned long long c = w ? s_cnt[threadIdx.x] : 0ull;
    m = __reduce_max_sync(0xffffffffu, m);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) {
      if (m) atomicMax(hmx, m);
      if (c) atomicAdd(cnt, c);
    }
  }
}

// a lattice with no active node is finished; the others get their cap
__global__ void k_pool_update(InstDesc* insts, int n, const unsigned long long* cnt,
                              const unsigned* hmx, long long cap, int slack,
                              unsigned long long* total) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  InstDesc& I = insts[i];
  if (I.done || !I.active) return;
  if (cnt[i] == 0) {
    I.done = 1;
    return;
  }
  long long hm = (long long)hmx[i] + slack;
  long long c = cap < I.g.NP + 2 ? cap : I.g.NP + 2;
  I.hmax = int(hm < c ? hm : c);
  atomicAdd(total, cnt[i]);
}

__global__ void k_pool_reset(InstDesc* insts, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) insts[i].done = 0;
}

template <typename T>
__global__ void k_pool_init_marks(const InstDesc* insts, const long long* nbase, int n,
                                  long long NP, const T* exc, int* mark) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int in = inst_of(nbase, n, i);
  if (!insts[in].active) return;
  mark[i] = exc[i] > 0 ? 1 : 0;
}

__global__ void k_pool_queue_active(const InstDesc* insts, const int* tile_inst, int tiles,
                                    TileQueue q) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tiles) return;
  if (!insts[tile_inst[t]].active) return;
  enqueue_tile(q, 0, t);
}

// per-lattice sum of max(exc, 0), combined per warp and lattice first
template <typename T>
__global__ void k_pool_sum_pos(const InstDesc* insts, const long long* nbase, int n, long long NP,
                               const T* exc, long long* sums) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int inst = -1;
  long long v = 0;
  if (i < NP) {
    int in = inst_of(nbase, n, i);
    if (insts[in].active) {
      inst = in;
      T a = exc[i];
      v = a > 0 ? (long long)a : 0;
    }
  }
  const unsigned peers = __match_any_sync(0xffffffffu, inst);
  long long sum = 0;
  for (unsigned m = peers; m; m &= m - 1) sum += __shfl_sync(peers, v, __ffs(m) - 1);
  if (inst >= 0 && sum && (threadIdx.x & 31) == __ffs(peers) - 1) atom_add(&sums[inst], sum);
}


}  // namespace

size_t pool_smem_head_bytes() { return sizeof(PoolSmemHead); }

// Launchers of the node-level pool kernels (used by PoolRunner and by the
// allocation-free single-lattice driver).
template <typename T>
cudaError_t pool_init_heights(const InstDesc* insts, const long long* nbase, int n, long long NP,
                              const T* exc, const uint64_t* kmask, int* h, cudaStream_t s) {
  k_pool_init_heights<T><<<nblk(NP, 256), 256, 0, s>>>(insts, nbase, n, NP, exc, kmask, h);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pool_mask(const InstDesc* insts, const long long* nbase, int n, long long NP,
                      const T* res, const uint64_t* kmask, uint64_t* mask, cudaStream_t s) {
  k_pool_mask<T><<<nblk(NP, 256), 256, 0, s>>>(insts, nbase, n, NP, res, kmask, mask);
  return cudaGetLastError();
}
cudaError_t pool_queue_all(const InstDesc* insts, const int* tile_inst, int tiles, TileQueue q,
                           cudaStream_t s) {
  if (tiles > 0) k_pool_queue_all<<<nblk(tiles, 256), 256, 0, s>>>(insts, tile_inst, tiles, q);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pool_active(const InstDesc* insts, const long long* nbase, int n, long long NP,
                        const T* exc, const int* h, TileQueue q, unsigned long long* cnt,
                        unsigned* hmx, cudaStream_t s) {
  k_pool_active<T><<<nblk(NP, 256), 256, 0, s>>>(insts, nbase, n, NP, exc, h, q, cnt, hmx);
  return cudaGetLastError();
}
cudaError_t pool_update(InstDesc* insts, int n, const unsigned long long* cnt, const unsigned* hmx,
                        long long cap, int slack, unsigned long long* total, cudaStream_t s) {
  k_pool_update<<<nblk(n, 256), 256, 0, s>>>(insts, n, cnt, hmx, cap, slack, total);
  return cudaGetLastError();
}
cudaError_t pool_reset(InstDesc* insts, int n, cudaStream_t s) {
  k_pool_reset<<<nblk(n, 256), 256, 0, s>>>(insts, n);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pool_init_marks(const InstDesc* insts, const long long* nbase, int n, long long NP,
                            const T* exc, int* mark, cudaStream_t s) {
  k_pool_init_marks<T><<<nblk(NP, 256), 256, 0, s>>>(insts, nbase, n, NP, exc, mark);
  return cudaGetLastError();
}
cudaError_t pool_queue_active(const InstDesc* insts, const int* tile_inst, int tiles, TileQueue q,
                              cudaStream_t s) {
  if (tiles > 0) k_pool_queue_active<<<nblk(tiles, 256), 256, 0, s>>>(insts, tile_inst, tiles, q);
  return cudaGetLastError();
}
template <typename T>
cudaError_t pool_sum_pos(const InstDesc* insts, const long long* nbase, int n, long long NP,
                         const T* exc, long long* sums, cudaStream_t s) {
  k_pool_sum_pos<T><<<nblk(NP, 256), 256, 0, s>>>(insts, nbase, n, NP, exc, sums);
  return cudaGetLastError();
}
template cudaError_t pool_init_heights<int>(const InstDesc*, const long long*, int, long long,
                                            const int*, const uint64_t*, int*, cudaStream_t);
template cudaError_t pool_mask<int>(const InstDesc*, const long long*, int, long long, const int*,
                                    const uint64_t*, uint64_t*, cudaStream_t);
template cudaError_t pool_active<int>(const InstDesc*, const long long*, int, long long, const int*,
                                      const int*, TileQueue, unsigned long long*, unsigned*,
                                      cudaStream_t);
template cudaError_t pool_init_marks<int>(const InstDesc*, const long long*, int, long long,
                                          const int*, int*, cudaStream_t);
template cudaError_t pool_sum_pos<int>(const InstDesc*, const long long*, int, long long,
                                       const int*, long long*, cudaStream_t);

// ------------------------------------------------------------------ runner

void PoolRunner::check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? 5 : 6;
    throw LfError{code, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

void PoolRunner::release() {
  cudaFree(d_inst); d_inst = nullptr;
  cudaFree(d_nbase); d_nbase = nullptr;
  cudaFree(d_tile_inst); d_tile_inst = nullptr;
  for (int b = 0; b < 2; ++b) {
    cudaFree(q.flag[b]); q.flag[b] = nullptr;
    cudaFree(q.list[b]); q.list[b] = nullptr;
  }
  cudaFree(q.ctr); q.ctr = nullptr;
  cudaFree(d_cnt); d_cnt = nullptr;
  cudaFree(d_hmx); d_hmx = nullptr;
  cudaFree(d_sum); d_sum = nullptr;
  cudaFree(d_flag); d_flag = nullptr;
  cudaFree(d_counters); d_counters = nullptr;
  cudaFree(d_ctl); d_ctl = nullptr;
  if (loop_pr) pass_loop_free(loop_pr);
  if (loop_bfs) pass_loop_free(loop_bfs);
  loop_pr = loop_bfs = nullptr;
  if (pool_maps) pool_maps_free(pool_maps);
  pool_maps = nullptr;
  if (h_pin) { cudaFreeHost(h_pin); h_pin = nullptr; }
  free_tail();
}

void PoolRunner::free_tail() {
  cudaFree(tail.vis);
  cudaFree(tail.node);
  cudaFree(tail.par);
  cudaFree(tail.dir);
  cudaFree(tail.dem);
  cudaFree(tail.rem);
  cudaFree(tail.lvl);
  cudaFree(tail.list);
  cudaFree(tail.count);
  tail = TailScratch();
  tail_stamp = 1;
}

// Tail scratch, allocated at the first tail step of this pool.
void PoolRunner::alloc_tail() {
  const long long want = std::min<long long>(
      std::max<long long>(NP, 1), tune.tail_tree_nodes > 0 ? tune.tail_tree_nodes : 65536);
  if (tail.vis && tail.cap == want) return;
  if (tail.vis) free_tail();
  TailScratch t;
  t.cap = int(want);
  t.lvl_cap = 1 << 16;
  t.max_active = 64;
  check(cudaMalloc(&t.vis, std::max<long long>(NP, 1) * sizeof(int)), "cudaMalloc tail");
  check(cudaMalloc(&t.node, t.cap * sizeof(long long)), "cudaMalloc tail");
  check(cudaMalloc(&t.par, t.cap * sizeof(int)), "cudaMalloc tail");
  check(cudaMalloc(&t.dir, t.cap), "cudaMalloc tail");
  check(cudaMalloc(&t.dem, t.cap * sizeof(long long)), "cudaMalloc tail");
  check(cudaMalloc(&t.rem, t.cap * sizeof(long long)), "cudaMalloc tail");
  check(cudaMalloc(&t.lvl, (t.lvl_cap + 2) * sizeof(int)), "cudaMalloc tail");
  check(cudaMalloc(&t.list, t.max_active * sizeof(long long)), "cudaMalloc tail");
  check(cudaMalloc(&t.count, sizeof(unsigned)), "cudaMalloc tail");
  check(cudaMemsetAsync(t.vis, 0, std::max<long long>(NP, 1) * sizeof(int), stream), "memset");
  tail = t;
  tail_stamp = 1;
}

PoolRunner::~PoolRunner() { release(); }

void PoolRunner::setup(const std::vector<InstDesc>& insts, cudaStream_t s) {
  stream = s;
  grid_bfs = grid_reach = 0;
  host = insts;
  n = int(insts.size());
  tiles = 0;
  NP = 0;
  for (const InstDesc& I : insts) {
    tiles += I.g.ntiles;
    NP += I.g.NP;
  }
  release();
  std::vector<long long> nb(n + 1, 0);
  std::vector<int> ti(std::max(tiles, 1), 0);
  for (int i = 0; i < n; ++i) {
    nb[i] = host[i].node_base;
    for (int t = 0; t < host[i].g.ntiles; ++t) ti[host[i].tile_base + t] = i;
  }
  nb[n] = NP;
  size_t T = std::max(tiles, 1);
  check(cudaMalloc(&d_inst, std::max(n, 1) * sizeof(InstDesc)), "cudaMalloc");
  check(cudaMalloc(&d_nbase, (n + 1) * sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_tile_inst, T * sizeof(int)), "cudaMalloc");
  for (int b = 0; b < 2; ++b) {
    check(cudaMalloc(&q.flag[b], T * sizeof(int)), "cudaMalloc");
    check(cudaMalloc(&q.list[b], T * sizeof(int)), "cudaMalloc");
    check(cudaMemsetAsync(q.flag[b], 0, T * sizeof(int), stream), "memset");
  }
  check(cudaMalloc(&q.ctr, 4 * sizeof(unsigned)), "cudaMalloc");
  check(cudaMalloc(&d_cnt, std::max(n, 1) * sizeof(unsigned long long)), "cudaMalloc");
  check(cudaMalloc(&d_hmx, std::max(n, 1) * sizeof(unsigned)), "cudaMalloc");
  check(cudaMalloc(&d_sum, 2 * std::max(n, 1) * sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_flag, sizeof(int)), "cudaMalloc");
  check(cudaMalloc(&d_counters, 16 * sizeof(unsigned long long)), "cudaMalloc");
  check(cudaMalloc(&d_ctl, 4 * sizeof(int)), "cudaMalloc");
  check(cudaMallocHost(&h_pin, 4096), "cudaMallocHost");
  check(cudaMemcpyAsync(d_inst, host.data(), n * sizeof(InstDesc), cudaMemcpyHostToDevice, stream), "memcpy");
  check(cudaMemcpyAsync(d_nbase, nb.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, stream), "memcpy");
  check(cudaMemcpyAsync(d_tile_inst, ti.data(), T * sizeof(int), cudaMemcpyHostToDevice, stream), "memcpy");
  check(cudaMemsetAsync(d_counters, 0, 16 * sizeof(unsigned long long), stream), "memset");
  check(cudaStreamSynchronize(stream), "sync");
  // kernel sizes of the pool (at most two distinct) and launch shapes
  ka = kb = 0;
  for (const InstDesc& I : host) {
    if (!ka) ka = I.st.K;
    else if (I.st.K != ka && !kb) kb = I.st.K;
    else if (I.st.K != ka && I.st.K != kb) throw LfError{2, "a pool mixes at most two kernel sizes"};
  }
  if (!kb) kb = ka;
  if (ka > kb) std::swap(ka, kb);
  threads = 1;
  hv_max = 0;
  for (const InstDesc& I : host) {
    threads = std::max(threads, I.g.TA * I.g.TB * I.g.TC);
    hv_max = std::max(hv_max, (I.g.TA + 2 * I.st.HA) * (I.g.TB + 2 * I.st.HB) * (I.g.TC + 2 * I.st.HC));
  }
}

// empty both tile lists so the next relabel starts clean
void PoolRunner::drain_queue() {
  check(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), stream), "memset");
  for (int b = 0; b < 2; ++b)
    check(cudaMemsetAsync(q.flag[b], 0, std::max(tiles, 1) * sizeof(int), stream), "memset");
}

void PoolRunner::prep_pass(int cur) {
  int lo = cur ? 0 : 2;  // see TileQueue: count of the other list + this pass's head
  check(cudaMemsetAsync(q.ctr + lo, 0, 2 * sizeof(unsigned), stream), "memset");
}

void PoolRunner::sync_read(void* dst, const void* src, size_t bytes) {
  check(cudaMemcpyAsync(h_pin, src, bytes, cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  std::memcpy(dst, h_pin, bytes);
}

void PoolRunner::mark(int cat, bool end) {
  if (hooks && hooks->profiling) hooks->mark(cat, end);
}

void PoolRunner::count_launch() {
  if (hooks) ++hooks->launches;
}

template <typename T>
void PoolRunner::global_relabel(const T* res, const T* exc, int* h, uint64_t* mask,
                                const uint64_t* kmask, SolveStats& stats) {
  const int B = 256;
  if (n == 1) {  // NP is a multiple of 32 and every plane 16-byte aligned
    k_relabel_init1<T><<<std::min(nblk(NP / (16 / sizeof(T)), B), 152 * 8), B, 0, stream>>>(
        d_inst, NP, res, exc, kmask, h, mask, q, tiles);
    count_launch();
  } else {
    k_pool_init_heights<T><<<nblk(NP, B), B, 0, stream>>>(d_inst, d_nbase, n, NP, exc, kmask, h);
    count_launch();
    k_pool_mask<T><<<nblk(NP, B), B, 0, stream>>>(d_inst, d_nbase, n, NP, res, kmask, mask);
    count_launch();
    check(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), stream), "memset");
    k_pool_queue_all<<<nblk(tiles, B), B, 0, stream>>>(d_inst, d_tile_inst, tiles, q);
    count_launch();
  }
  check(cudaGetLastError(), "bfs setup");
  const size_t smem = sizeof(PoolSmemHead) + size_t(hv_max) * sizeof(int);
  const int grid = std::max(tiles, 1);
  const int chunk = tune.pass_chunk > 0 ? tune.pass_chunk : 6;
  const long long cap = 4LL * tiles + 64;
  const int k2d = tune.bfs_kernel != 1 ? lattice2d_kernel_size(host[0], n == 1) : 0;
  const int k3d = (!k2d && tune.bfs_kernel != 1) ? lattice3d_kernel_size(host[0], n == 1) : 0;
  if (k2d && tune.device_loops == 1) {
    // the whole relabel in one device-side loop: passes until no tile is
    // queued (a cap that ends it early is reported by activate())
    if (!loop_bfs) loop_bfs = pass_loop_new();
    PoolBFS p{host[0], d_inst, d_tile_inst, h, mask, q, 0, 64, d_flag, d_counters};
    mark(1, false);
    check(loop_pool_bfs2d(loop_bfs, p, k2d, d_counters + 4, grid, d_ctl, (unsigned)cap,
                          d_counters + 5, d_counters + 7, stream),
          "bfs loop (TMA)");
    mark(1, true);
    // kernels of the loop are counted from its pass counter
    return;
  }
  // a pool of 2-d lattices: the TMA-staged pass with each lattice's maps
  const int tb_pool = (!k2d && n > 1 && tune.bfs_kernel != 1) ? pool2d_tile_rows(host) : 0;
  const void* maps = nullptr;
  if (tb_pool) {
    if (!pool_maps) pool_maps = pool_maps_new();
    maps = pool_maps_bfs(pool_maps, host, h, mask, stream);
  }
  if (maps && tune.device_loops == 1) {
    if (!loop_bfs) loop_bfs = pass_loop_new();
    PoolBFS p{host[0], d_inst, d_tile_inst, h, mask, q, 0, 64, d_flag, d_counters};
    mark(1, false);
    check(pool_bfs2d(loop_bfs, maps, p, tb_pool, d_counters + 4, grid, d_ctl, (unsigned)cap,
                     d_counters + 5, d_counters + 7, stream),
          "bfs loop (TMA, pool)");
    mark(1, true);
    // kernels of the loop are counted from its pass counter
    return;
  }
  int cur = 0;
  for (long long pass = 0;;) {
    if (pass > cap) throw LfError{4, "global relabel did not converge"};
    for (int c = 0; c < chunk; ++c, ++pass) {
      prep_pass(cur);
      check(cudaMemsetAsync(d_flag, 0, sizeof(int), stream), "memset");
      PoolBFS p{host[0], d_inst, d_tile_inst, h, mask, q, cur, 64, d_flag, d_counters};
      mark(1, false);
      if (k2d) check(launch_pool_bfs2d(p, k2d, d_counters + 4, grid, stream), "bfs pass (TMA)");
      else if (k3d)
        check(launch_pool_bfs3d(p, k3d, d_counters + 4, grid, stream), "bfs pass (TMA, 3-d)");
      else if (maps)
        check(pool_bfs2d(nullptr, maps, p, tb_pool, d_counters + 4, grid, nullptr, 0, nullptr,
                         nullptr, stream),
              "bfs pass (TMA, pool)");
      else check(launch_pool_bfs(p, ka, kb, n == 1, grid, threads, smem, stream), "bfs pass");
      check(cudaGetLastError(), "bfs pass");
      mark(1, true);
      count_launch();
      ++stats.bfs_passes;
      cur ^= 1;
    }
    int changed = 0;
    sync_read(&changed, d_flag, sizeof(int));
    if (!changed) break;
  }
}

template <typename T>
unsigned long long PoolRunner::activate(const T* exc, const int* h) {
  const int B = 256;
  check(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), stream), "memset");
  check(cudaMemsetAsync(d_cnt, 0, n * sizeof(unsigned long long), stream), "memset");
  check(cudaMemsetAsync(d_hmx, 0, n * sizeof(unsigned), stream), "memset");
  check(cudaMemsetAsync(d_counters + 3, 0, sizeof(unsigned long long), stream), "memset");
  if (n == 1)  // NP is a whole number of 32-node tile rows
    k_pool_active1<T><<<std::min(nblk(NP, B), 152 * 8), B, 0, stream>>>(d_inst, NP, exc, h, q,
                                                                        d_cnt, d_hmx);
  else
    k_pool_active<T><<<nblk(NP, B), B, 0, stream>>>(d_inst, d_nbase, n, NP, exc, h, q, d_cnt, d_hmx);
  count_launch();
  const long long hcap = (long long)kHInf - 2;
  const int slack = tune.height_slack > 0 ? tune.height_slack : 16;
  k_pool_update<<<nblk(n, B), B, 0, stream>>>(d_inst, n, d_cnt, d_hmx, hcap, slack, d_counters + 3);
  count_launch();
  check(cudaGetLastError(), "activate");
  unsigned long long total = 0;
  if (n == 1) {
    // a pool of one passes its descriptor by value: refresh cap / finished
    // flag, in the same synchronisation as the count (and the cap flag of a
    // device-side BFS loop, counters[7])
    unsigned char* hp = static_cast<unsigned char*>(h_pin);
    check(cudaMemcpyAsync(hp, d_counters + 3, 5 * sizeof(total), cudaMemcpyDeviceToHost, stream),
          "memcpy");
    check(cudaMemcpyAsync(hp + 64, d_inst, sizeof(InstDesc), cudaMemcpyDeviceToHost, stream), "memcpy");
    check(cudaStreamSynchronize(stream), "sync");
    unsigned long long c[5];
    std::memcpy(c, hp, sizeof(c));
    std::memcpy(&host[0], hp + 64, sizeof(InstDesc));
    if (c[4]) throw LfError{4, "global relabel did not converge"};
    total = c[0];
  } else {
    sync_read(&total, d_counters + 3, sizeof(total));
  }
  return total;
}

// Solves with device-side pass loops run one at a time in the process: the
// loops stay single-threaded by construction (they are opt-in, and a GPU
// fault was once seen with eight host threads each running their own loop
// graphs at once).  The lock is held until the solve's work on the stream
// has finished, on error paths too.
namespace {
std::mutex g_device_loop_lock;
}

template <typename T>
void PoolRunner::maxflow(T* res, T* exc, int* h, uint64_t* mask, const uint64_t* kmask, int* markv,
                         SolveStats& stats, bool sets) {
  if (tune.device_loops != 1) {
    maxflow_epochs<T>(res, exc, h, mask, kmask, markv, stats, sets);
    return;
  }
  std::lock_guard<std::mutex> lk(g_device_loop_lock);
  try {
    maxflow_epochs<T>(res, exc, h, mask, kmask, markv, stats, sets);
  } catch (...) {
    cudaStreamSynchronize(stream);  // nothing of this solve stays in flight
    throw;
  }
  check(cudaStreamSynchronize(stream), "sync");
}

template <typename T>
void PoolRunner::maxflow_epochs(T* res, T* exc, int* h, uint64_t* mask, const uint64_t* kmask,
                                int* markv, SolveStats& stats, bool sets) {
  const int B = 256;
  k_pool_reset<<<nblk(n, B), B, 0, stream>>>(d_inst, n);
  count_launch();
  for (InstDesc& I : host) I.done = 0;
  check(cudaMemsetAsync(d_counters, 0, 3 * sizeof(unsigned long long), stream), "memset");
  check(cudaMemsetAsync(d_counters + 4, 0, 4 * sizeof(unsigned long long), stream), "memset");
  const int M = tune.launches_per_relabel > 0 ? tune.launches_per_relabel : 4;
  const int R = tune.sweeps > 0 ? tune.sweeps : 4;
  const int KA = ka, KB = kb;
  const int NTmax = threads;
  const size_t smem = pool_pr_smem<T>(KB, NTmax, hv_max);
  const long long max_epochs = tune.max_epochs > 0 ? tune.max_epochs : 1000000;
  const auto t0 = std::chrono::steady_clock::now();
  const bool trace = std::getenv("LF_PR_TRACE") != nullptr;  // diagnostic: one line per epoch
  // tail steps per solve at most (each moves at least one unit; this bounds
  // a run of steps that each move little), then the tile passes finish
  const int kMaxTailSteps = 256;
  int tail_steps = 0;
  for (long long epoch = 0;; ++epoch) {
    if (epoch >= max_epochs) throw LfError{4, "push-relabel did not converge"};
    if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(300))
      throw LfError{4, "push-relabel exceeded its time limit"};
    const long long bfs0 = stats.bfs_passes;
    global_relabel<T>(res, exc, h, mask, kmask, stats);
    ++stats.epochs;
    const unsigned long long act = activate<T>(exc, h);
    if (trace) {
      unsigned long long c[2];
      sync_read(c, d_counters, sizeof(c));
      std::fprintf(stderr, "pr epoch %lld active %llu bfs %lld tiles %llu hmax0 %d\n", epoch, act,
                   stats.bfs_passes - bfs0, c[0], n == 1 ? host[0].hmax : -1);
    }
    if (act == 0) break;
    // few active nodes: route their excess along BFS trees to deficits
    const int tail_max = tune.tail_active == 0 ? 64 : tune.tail_active;
    if (tail_max > 0 && act <= (unsigned long long)tail_max && tail_steps < kMaxTailSteps) {
      ++tail_steps;
      alloc_tail();
      if (tail_stamp > INT_MAX - 2 * tail.max_active) {  // restart the stamps
        check(cudaMemsetAsync(tail.vis, 0, NP * sizeof(int), stream), "memset");
        tail_stamp = 1;
      }
      mark(0, false);
      check(launch_pool_tail<T>(d_inst, d_nbase, n, NP, res, exc, h, kmask, tail, tail_stamp,
                                d_counters + 2, stream), "tail step");
      mark(0, true);
      count_launch();
      count_launch();
      tail_stamp += tail.max_active;
      ++stats.tail_steps;
      unsigned long long moved = 0;
      sync_read(&moved, d_counters + 2, sizeof(moved));
      if (moved > 0) {  // relabel again; else fall back to the tile passes
        drain_queue();
        continue;
      }
    }
    if constexpr (std::is_same<T, long long>::value) {
      // 64-bit capacities with section masks on one 2-d lattice (parametric /
      // TV section solves): the TMA-staged pass, one launch per pass (or a
      // device-side loop of passes when device_loops is set)
      PoolPR<long long> p{host[0], d_inst, d_tile_inst, res, exc, h, kmask, q, 0, R, d_counters};
      const int k64 = tune.pr_kernel != 1 ? pr2d64_kernel_size(p, n == 1) : 0;
      if (k64) {
        if (!loop_pr) loop_pr = pass_loop_new();
        mark(0, false);
        if (tune.device_loops == 1) {
          check(pr2d64(loop_pr, p, k64, d_counters + 4, std::max(tiles, 1), d_ctl, (unsigned)M,
                       d_counters + 6, stream),
                "push-relabel loop (TMA, 64-bit)");
        } else {
          int cur = 0;
          for (int l = 0; l < M; ++l) {
            prep_pass(cur);
            p.cur = cur;
            check(pr2d64(nullptr, p, k64, d_counters + 4, std::max(tiles, 1), nullptr, 0, nullptr,
                         stream),
                  "push-relabel pass (TMA, 64-bit)");
            count_launch();
            ++stats.pr_launches;
            cur ^= 1;
          }
        }
        mark(0, true);
        drain_queue();
        continue;
      }
    }
    const void* pmaps = nullptr;  // pool of 2-d lattices: the TMA-staged pass
    int tb_pool = 0;
    if constexpr (std::is_same<T, int>::value) {
      PoolPR<int> p{host[0], d_inst, d_tile_inst, res, exc, h, kmask, q, 0, R, d_counters};
      const int k2d = tune.pr_kernel != 1 ? pr2d_kernel_size(p, n == 1) : 0;
      tb_pool = (!k2d && n > 1 && !kmask && tune.pr_kernel != 1) ? pool2d_tile_rows(host) : 0;
      if (tb_pool) {
        if (!pool_maps) pool_maps = pool_maps_new();
        pmaps = pool_maps_pr(pool_maps, host, res, exc, h, stream);
      }
      if (pmaps && tune.device_loops == 1) {
        if (!loop_pr) loop_pr = pass_loop_new();
        mark(0, false);
        check(pool_pr2d(loop_pr, pmaps, p, tb_pool, pr2d_variant(tune.pr_kernel), d_counters + 4,
                        std::max(tiles, 1), d_ctl, (unsigned)M, d_counters + 6, stream),
              "push-relabel loop (TMA, pool)");
        mark(0, true);
        // kernels of the loop are counted from its pass counter
        drain_queue();
        continue;
      }
      if (k2d && tune.device_loops == 1) {
        // M passes (fewer when the queue runs dry) in one device-side loop
        if (!loop_pr) loop_pr = pass_loop_new();
        mark(0, false);
        check(loop_pool_pr2d(loop_pr, p, k2d, pr2d_variant(tune.pr_kernel), d_counters + 4,
                             std::max(tiles, 1), d_ctl, (unsigned)M, d_counters + 6, stream),
              "push-relabel loop (TMA)");
        mark(0, true);
        // kernels of the loop are counted from its pass counter
        drain_queue();
        continue;
      }
    }
    int cur = 0;
    for (int l = 0; l < M; ++l) {
      prep_pass(cur);
      PoolPR<T> p{host[0], d_inst, d_tile_inst, res, exc, h, kmask, q, cur, R, d_counters};
      mark(0, false);
      int k2d = 0, k3d = 0;
      if constexpr (std::is_same<T, int>::value)
        if (tune.pr_kernel != 1) {
          k2d = pr2d_kernel_size(p, n == 1);
          if (!k2d && !pmaps) k3d = pr3d_kernel_size(p, n == 1);
        }
      if (k3d) {
        if constexpr (std::is_same<T, int>::value)
          check(launch_pool_pr3d(p, k3d, d_counters + 4, std::max(tiles, 1), stream),
                "push-relabel pass (TMA, 3-d)");
      } else if (k2d) {
        if constexpr (std::is_same<T, int>::value)
          check(launch_pool_pr2d(p, k2d, pr2d_variant(tune.pr_kernel), d_counters + 4,
                                 std::max(tiles, 1), stream),
                "push-relabel pass (TMA)");
      } else if (pmaps) {
        if constexpr (std::is_same<T, int>::value)
          check(pool_pr2d(nullptr, pmaps, p, tb_pool, pr2d_variant(tune.pr_kernel), d_counters + 4,
                          std::max(tiles, 1), nullptr, 0, nullptr, stream),
                "push-relabel pass (TMA, pool)");
      } else {
        check(launch_pool_pr<T>(p, KA, KB, NTmax, smem, n == 1, std::max(tiles, 1), stream),
              "push-relabel pass");
      }
      mark(0, true);
      count_launch();
      ++stats.pr_launches;
      cur ^= 1;
    }
    drain_queue();
  }
  if (sets) reach<T>(exc, mask, markv, stats);
  unsigned long long c[8];
  sync_read(c, d_counters, sizeof(c));
  stats.tiles_processed += c[0];
  stats.bfs_tiles += c[1];
  stats.bfs_passes += (long long)c[5];
  stats.pr_launches += (long long)c[6];
  if (hooks) hooks->launches += 2 * (long long)(c[5] + c[6]);  // pass + control kernel per pass
  if (c[4] == 2) throw LfError{6, "a queued tile id was out of range"};
  if (c[4]) throw LfError{6, "a tile's staging copy did not complete in time"};
  if (c[7]) throw LfError{4, "global relabel did not converge"};
}

template <typename T>
void PoolRunner::reach(const T* exc, const uint64_t* mask, int* markv, SolveStats& stats) {
  const int B = 256;
  k_pool_init_marks<T><<<nblk(NP, B), B, 0, stream>>>(d_inst, d_nbase, n, NP, exc, markv);
  count_launch();
  check(cudaMemsetAsync(q.ctr, 0, 4 * sizeof(unsigned), stream), "memset");
  k_pool_queue_active<<<nblk(tiles, B), B, 0, stream>>>(d_inst, d_tile_inst, tiles, q);
  count_launch();
  check(cudaGetLastError(), "reach setup");
  int NTmax = threads;
  const size_t smem = sizeof(PoolSmemHead) + size_t(NTmax) * sizeof(int);
  const int grid = std::max(tiles, 1);
  const int chunk = tune.pass_chunk > 0 ? tune.pass_chunk : 6;
  const long long cap = 4LL * tiles + 64;
  int cur = 0;
  for (long long pass = 0;;) {
    if (pass > cap) throw LfError{4, "cut-set closure did not converge"};
    for (int c = 0; c < chunk; ++c, ++pass) {
      prep_pass(cur);
      check(cudaMemsetAsync(d_flag, 0, sizeof(int), stream), "memset");
      PoolReach p{host[0], d_inst, d_tile_inst, markv, mask, q, cur, 256, d_flag};
      mark(2, false);
      check(launch_pool_reach(p, ka, kb, n == 1, grid, threads, smem, stream), "reach pass");
      check(cudaGetLastError(), "reach pass");
      mark(2, true);
      count_launch();
      ++stats.reach_passes;
      cur ^= 1;
    }
    int changed = 0;
    sync_read(&changed, d_flag, sizeof(int));
    if (!changed) break;
  }
}

template <typename T>
void PoolRunner::stuck_excess(const T* exc, long long* out_host) {
  const int B = 256;
  check(cudaMemsetAsync(d_sum, 0, n * sizeof(long long), stream), "memset");
  k_pool_sum_pos<T><<<nblk(NP, B), B, 0, stream>>>(d_inst, d_nbase, n, NP, exc, d_sum);
  count_launch();
  check(cudaGetLastError(), "sum");
  check(cudaMemcpyAsync(out_host, d_sum, n * sizeof(long long), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
}

void PoolRunner::set_active(const std::vector<int>& act) {
  for (int i = 0; i < n; ++i) host[i].active = act[i];
  check(cudaMemcpyAsync(d_inst, host.data(), n * sizeof(InstDesc), cudaMemcpyHostToDevice, stream), "memcpy");
}

template void PoolRunner::maxflow<int>(int*, int*, int*, uint64_t*, const uint64_t*, int*, SolveStats&, bool);
template void PoolRunner::maxflow<long long>(long long*, long long*, int*, uint64_t*, const uint64_t*, int*, SolveStats&, bool);
template void PoolRunner::stuck_excess<int>(const int*, long long*);
template void PoolRunner::stuck_excess<long long>(const long long*, long long*);


}  // namespace lfg
