// CUDA kernels of the lattice max-flow engine (sm_103a).
//
// The reference solves one lattice with a sequential highest-label
// push-relabel (network_flow/push_relabel.hpp:1069-1278).  Here the same
// preflow problem is solved by synchronous tile sweeps:
//   * k_pr_tile     stages one tile (all residual planes, excess, heights with
//                   a halo) in shared memory and runs up to `sweeps` local
//                   push / relabel rounds; flow pushed across the tile edge is
//                   delivered to the neighbour tile with global atomics at the
//                   end of the launch.
//   * k_bfs_tile    global relabel: exact distance to the nearest deficit
//                   node along residual edges (the reference's hotStart BFS,
//                   push_relabel.hpp:306-415), tile-local wavefronts repeated
//                   until no tile changes.  Nodes left at kHInf cannot reach a
//                   deficit: the reference flips exactly those
//                   (push_relabel.hpp:394-402, gap flip :692-711).
//   * k_reach_tile  forward residual closure of the excess nodes (the unique
//                   minimal on-set).
// All capacities are integers; results are exact.
#include <cstdint>
#include <cuda_runtime.h>

#include "lf_tile_common.cuh"

namespace lfg {

// ------------------------------------------------------------------ fill

// Energy form (interface.hpp:49-60).  One thread per (node, filling edge);
// edge 0 also adds the node's unary term.  Decomposition of a submodular
// pairwise table [[A, B], [C, D]] (rows: source node off/on):
//   node cost A (off) / D (on), then f(0,1) = B - A, f(1,0) = C - D as two
//   directed capacities, moving a negative one into the unary terms.
// exc = cost(off) - cost(on): > 0 prefers on (supply), < 0 prefers off.
__global__ void k_fill_energy(Geo g, Stencil st, int nd, long long N, const int64_t* unary,
                              const int64_t* binary, long long* exc, long long* cap,
                              long long* c0sum, int* err) {
  const int Kp = st.K / 2;
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = N * Kp;
  long long c0 = 0;
  if (tid < total) {
    long long b = tid / Kp;
    int e = int(tid % Kp);
    int a, bb, c;
    if (nd == 2) { a = 0; bb = int(b / g.C); c = int(b % g.C); }
    else { c = int(b % g.C); bb = int((b / g.C) % g.B); a = int(b / ((long long)g.C * g.B)); }
    long long u = ((long long)a * g.Bp + bb) * g.Cp + c;
    if (e == 0) {
      int64_t E0 = unary[2 * b], E1 = unary[2 * b + 1];
      atom_add(&exc[u], (long long)(E0 - E1));
      c0 += E0;
    }
    int na = a + st.da[e], nb = bb + st.db[e], nc = c + st.dc[e];
    if (na >= 0 && na < g.A && nb >= 0 && nb < g.B && nc >= 0 && nc < g.C) {
      long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
      const int64_t* q = binary + (b * Kp + e) * 4;
      long long A = q[0], B = q[1], C = q[2], D = q[3];
      c0 += A;
      long long du = A - D, dv = 0;
      long long Bq = B - A, Cq = C - D;
      if (Bq + Cq < 0) atomicExch(err, 1);
      int rv = st.rev[e];
      if (Bq < 0) {
        dv -= Bq; du += Bq;
        atom_add(&cap[(long long)e * g.NP + u], Bq + Cq);
      } else if (Cq < 0) {
        du -= Cq; dv += Cq;
        atom_add(&cap[(long long)rv * g.NP + v], Bq + Cq);
      } else {
        if (Cq) atom_add(&cap[(long long)e * g.NP + u], Cq);
        if (Bq) atom_add(&cap[(long long)rv * g.NP + v], Bq);
      }
      if (du) atom_add(&exc[u], du);
      if (dv) atom_add(&exc[v], dv);
    }
  }
  // block-reduce the constant part of the energy
  __shared__ long long red[32];
  for (int o = 16; o > 0; o >>= 1) c0 += __shfl_down_sync(0xffffffffu, c0, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c0;
  __syncthreads();
  if (threadIdx.x < 32) {
    long long v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atom_add(c0sum, v);
  }
}

// Capacity form: source = cost off, sink = cost on, edge = symmetric capacity.
// pf2x: the parametric solver's 2x-scaled form (reduction += 2 (sink - source),
// alpha += 2 w both ways).
__global__ void k_fill_caps(Geo g, Stencil st, int nd, long long N, const int32_t* src,
                            const int32_t* snk, const int32_t* edge, long long* exc,
                            long long* cap, long long* c0sum, int* err, int pf2x) {
  const long long mul = pf2x ? 2 : 1;
  const int Kp = st.K / 2;
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long c0 = 0;
  if (tid < N * Kp) {
    long long b = tid / Kp;
    int e = int(tid % Kp);
    int a, bb, c;
    if (nd == 2) { a = 0; bb = int(b / g.C); c = int(b % g.C); }
    else { c = int(b % g.C); bb = int((b / g.C) % g.B); a = int(b / ((long long)g.C * g.B)); }
    long long u = ((long long)a * g.Bp + bb) * g.Cp + c;
    if (e == 0) {
      long long s = src ? src[b] : 0, t = snk ? snk[b] : 0;
      if (s < 0 || t < 0) atomicExch(err, 1);
      if (s - t) atom_add(&exc[u], mul * (s - t));
      c0 += s;
    }
    if (edge) {
      long long w = edge[b * Kp + e];
      int na = a + st.da[e], nb = bb + st.db[e], nc = c + st.dc[e];
      if (w < 0) atomicExch(err, 1);
      if (w > 0 && na >= 0 && na < g.A && nb >= 0 && nb < g.B && nc >= 0 && nc < g.C) {
        long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
        atom_add(&cap[(long long)e * g.NP + u], mul * w);
        atom_add(&cap[(long long)st.rev[e] * g.NP + v], mul * w);
      }
    }
  }
  __shared__ long long red[32];
  for (int o = 16; o > 0; o >>= 1) c0 += __shfl_down_sync(0xffffffffu, c0, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c0;
  __syncthreads();
  if (threadIdx.x < 32) {
    long long v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atom_add(c0sum, v);
  }
}

// Range bound used to choose 32- or 64-bit working arrays: for every node
// |exc| + sum of outgoing and incoming capacities, i.e. the largest value an
// excess or a residual of that node can reach.
__global__ void k_range_bound(Geo g, Stencil st, const long long* exc, const long long* cap,
                              unsigned long long* out_max) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m = 0;
  if (i < g.NP) {
    int c = int(i % g.Cp), b = int((i / g.Cp) % g.Bp), a = int(i / ((long long)g.Cp * g.Bp));
    long long e = exc[i];
    unsigned long long s = (unsigned long long)(e < 0 ? -e : e);
    for (int k = 0; k < st.K; ++k) {
      s += (unsigned long long)cap[(long long)k * g.NP + i];
      int na = a + st.da[k], nb = b + st.db[k], nc = c + st.dc[k];
      if (na >= 0 && na < g.Ap && nb >= 0 && nb < g.Bp && nc >= 0 && nc < g.Cp) {
        long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
        s += (unsigned long long)cap[(long long)st.rev[k] * g.NP + v];
      }
    }
    m = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_down_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out_max, m);
}

template <typename T>
__global__ void k_convert(long long n, const long long* src, T* dst) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (T)src[i];
}

// sum of max(x, 0) over n values (int64 result)
template <typename T>
__global__ void k_sum_pos(long long n, const T* x, long long* out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long v = 0;
  if (i < n) { T a = x[i]; v = a > 0 ? (long long)a : 0; }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atom_add(out, v);
}

// ------------------------------------------------------------ epoch setup

// Deficit nodes are the BFS roots.  With sections (kmask non-null) only
// nodes whose bit 63 is set take part; the rest stay at kHInf.
template <typename T>
__global__ void k_init_heights(Geo g, const T* exc, const uint64_t* kmask, int* h) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.NP) return;
  bool part = !kmask || (kmask[i] >> 63);
  h[i] = (part && exc[i] < 0) ? 0 : kHInf;
}

// mask[i] bit k = res[k][i] > 0 (and the edge is inside the node's section)
template <typename T, int K>
__global__ void k_mask(Geo g, const T* res, const uint64_t* kmask, uint64_t* mask) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.NP) return;
  uint64_t m = 0;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (res[(long long)k * g.NP + i] > 0) m |= 1ull << k;
  if (kmask) m &= kmask[i];
  mask[i] = m;
}

// Count active nodes (excess > 0 and a finite height), flag their tiles and
// record the largest finite height (count[0], count[1]).
template <typename T>
__global__ void k_active(Geo g, const T* exc, const int* h, int* act, unsigned long long* count) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int a = 0;
  unsigned hm = 0;
  if (i < g.NP) {
    int hh = h[i];
    if (hh < kHInf) hm = (unsigned)hh;
    if (exc[i] > 0 && hh < kHInf) {
      a = 1;
      int c = int(i % g.Cp), b = int((i / g.Cp) % g.Bp), aa = int(i / ((long long)g.Cp * g.Bp));
      act[tile_of(g, aa, b, c)] = 1;
    }
  }
  unsigned bal = __ballot_sync(0xffffffffu, a);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(count, (unsigned long long)__popc(bal));
  for (int o = 16; o > 0; o >>= 1) {
    unsigned x = __shfl_down_sync(0xffffffffu, hm, o);
    hm = x > hm ? x : hm;
  }
  if ((threadIdx.x & 31) == 0 && hm) atomicMax(count + 1, (unsigned long long)hm);
}

// ---------------------------------------------------------------- BFS

template <int K>
__global__ void __launch_bounds__(1024) k_bfs_tile(BFSParams p) {
  const int tile = blockIdx.x;
  if (!p.dirty_cur[tile]) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const Geo& g = p.g;
  const TileCtx x = tile_ctx(g, p.st, tile);
  int* s_h = reinterpret_cast<int*>(smem);
  int* s_hoff = s_h + x.HV;
  const int t = threadIdx.x;
  if (t < K) s_hoff[t] = (p.st.da[t] * x.HBB + p.st.db[t]) * x.HCC + p.st.dc[t];
  load_halo_heights(g, p.st, x, p.h, s_h);
  const uint64_t m = p.mask[x.gi];
  bool boundary = false;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int na = x.ia + p.st.da[k], nb = x.ib + p.st.db[k], nc = x.ic + p.st.dc[k];
    if (na < 0 || na >= g.TA || nb < 0 || nb >= g.TB || nc < 0 || nc >= g.TC) boundary = true;
  }
  __syncthreads();
  int my_h = s_h[x.hidx];
  bool changed = false;
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int best = my_h;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((m >> k) & 1) {
        const int hn = s_h[x.hidx + s_hoff[k]] + 1;
        best = hn < best ? hn : best;
      }
    }
    const int c = best < my_h;
    if (c) {
      my_h = best;
      s_h[x.hidx] = best;
      changed = true;
    }
    if (!__syncthreads_or(c)) { converged = 1; break; }
  }
  if (changed) p.h[x.gi] = my_h;
  const int bch = changed && boundary;
  const int any_b = __syncthreads_or(bch);
  if (t == 0) {
    if (any_b) { mark_neighbour_tiles(g, tile, p.dirty_next); *p.any_changed = 1; }
    if (!converged) { p.dirty_next[tile] = 1; *p.any_changed = 1; }
    p.dirty_cur[tile] = 0;
    atomicAdd(&p.counters[1], 1ull);
  }
}

// ----------------------------------------------------- forward closure

template <int K>
__global__ void __launch_bounds__(1024) k_reach_tile(ReachParams p) {
  const int tile = blockIdx.x;
  if (!p.dirty_cur[tile]) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const Geo& g = p.g;
  const TileCtx x = tile_ctx(g, p.st, tile);
  int* s_mark = reinterpret_cast<int*>(smem);
  int* s_toff = s_mark + x.NT;
  const int t = threadIdx.x;
  if (t < K) s_toff[t] = (p.st.da[t] * g.TB + p.st.db[t]) * g.TC + p.st.dc[t];
  const int m0 = p.mark[x.gi];
  s_mark[t] = m0;
  const uint64_t m = p.mask[x.gi];
  uint64_t outm = 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int na = x.ia + p.st.da[k], nb = x.ib + p.st.db[k], nc = x.ic + p.st.dc[k];
    if (na < 0 || na >= g.TA || nb < 0 || nb >= g.TB || nc < 0 || nc >= g.TC) outm |= 1ull << k;
  }
  __syncthreads();
  int converged = 0;
  for (int it = 0; it < p.max_local; ++it) {
    int c = 0;
    if (s_mark[t]) {
      uint64_t in = m & ~outm;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if ((in >> k) & 1) {
          const int tn = t + s_toff[k];
          if (!s_mark[tn]) { s_mark[tn] = 1; c = 1; }
        }
      }
    }
    if (!__syncthreads_or(c)) { converged = 1; break; }
  }
  const int mine = s_mark[t];
  if (mine && !m0) p.mark[x.gi] = 1;
  int sent = 0;
  if (mine) {
    uint64_t out = m & outm;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if ((out >> k) & 1) {
        const int A_ = x.a0 + x.ia + p.st.da[k], B_ = x.b0 + x.ib + p.st.db[k],
                  C_ = x.c0 + x.ic + p.st.dc[k];
        const long long gn = ((long long)A_ * g.Bp + B_) * g.Cp + C_;
        if (!p.mark[gn]) {
          p.mark[gn] = 1;
          p.dirty_next[tile_of(g, A_, B_, C_)] = 1;
          sent = 1;
        }
      }
    }
  }
  const int any_sent = __syncthreads_or(sent);
  if (t == 0) {
    if (any_sent) *p.any_changed = 1;
    if (!converged) { p.dirty_next[tile] = 1; *p.any_changed = 1; }
    p.dirty_cur[tile] = 0;
  }
}

template <typename T>
__global__ void k_init_marks(long long n, const T* exc, int* mark) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mark[i] = exc[i] > 0 ? 1 : 0;
}

// Bounded (row-major) outputs: cut_min from marks, cut_max from h == kHInf.
__global__ void k_extract_cuts(Geo g, int nd, long long N, const int* mark, const int* h,
                               int* cut_min, int* cut_max) {
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= N) return;
  int a, bb, c;
  if (nd == 2) { a = 0; bb = int(b / g.C); c = int(b % g.C); }
  else { c = int(b % g.C); bb = int((b / g.C) % g.B); a = int(b / ((long long)g.C * g.B)); }
  long long i = ((long long)a * g.Bp + bb) * g.Cp + c;
  if (cut_min) cut_min[b] = mark[i] ? 1 : 0;
  if (cut_max) cut_max[b] = h[i] >= kHInf ? 1 : 0;
}

// ------------------------------------------------------------ launchers

int sm_count();

size_t pr_smem_bytes_for(const Geo& g, const Stencil& st, int elem_bytes) {
  return elem_bytes == 4 ? pr_smem_bytes<int>(g, st) : pr_smem_bytes<long long>(g, st);
}

cudaError_t launch_bfs_tile(const BFSParams& p, cudaStream_t s) {
  int HV = (p.g.TA + 2 * p.st.HA) * (p.g.TB + 2 * p.st.HB) * (p.g.TC + 2 * p.st.HC);
  size_t smem = size_t(HV + p.st.K) * sizeof(int);
  int threads = p.g.TA * p.g.TB * p.g.TC;
  switch (p.st.K) {
#define X(KK)                                                   \
  case KK:                                                      \
    k_bfs_tile<KK><<<p.g.ntiles, threads, smem, s>>>(p); \
    break;
    LF_K_LIST(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_reach_tile(const ReachParams& p, cudaStream_t s) {
  int NT = p.g.TA * p.g.TB * p.g.TC;
  size_t smem = size_t(NT + p.st.K) * sizeof(int);
  switch (p.st.K) {
#define X(KK)                                                  \
  case KK:                                                     \
    k_reach_tile<KK><<<p.g.ntiles, NT, smem, s>>>(p); \
    break;
    LF_K_LIST(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_mask(const Geo& g, int K, const T* res, const uint64_t* kmask, uint64_t* mask,
                        cudaStream_t s) {
  int blocks = int((g.NP + 255) / 256);
  switch (K) {
#define X(KK)                                                      \
  case KK:                                                         \
    k_mask<T, KK><<<blocks, 256, 0, s>>>(g, res, kmask, mask); \
    break;
    LF_K_LIST(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template cudaError_t launch_mask<int>(const Geo&, int, const int*, const uint64_t*, uint64_t*,
                                      cudaStream_t);
template cudaError_t launch_mask<long long>(const Geo&, int, const long long*, const uint64_t*,
                                            uint64_t*, cudaStream_t);

static inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

cudaError_t launch_fill_energy(const Geo& g, const Stencil& st, int nd, long long N,
                               const int64_t* u, const int64_t* b, long long* exc,
                               long long* cap, long long* c0, int* err, cudaStream_t s) {
  long long n = N * (st.K / 2);
  if (n > 0) k_fill_energy<<<nblk(n, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
  return cudaGetLastError();
}

cudaError_t launch_fill_caps(const Geo& g, const Stencil& st, int nd, long long N,
                             const int32_t* src, const int32_t* snk, const int32_t* edge,
                             long long* exc, long long* cap, long long* c0, int* err,
                             int pf2x, cudaStream_t s) {
  long long n = N * (st.K / 2);
  if (n > 0)
    k_fill_caps<<<nblk(n, 256), 256, 0, s>>>(g, st, nd, N, src, snk, edge, exc, cap, c0, err,
                                             pf2x);
  return cudaGetLastError();
}

cudaError_t launch_range_bound(const Geo& g, const Stencil& st, const long long* exc,
                               const long long* cap, unsigned long long* out, cudaStream_t s) {
  k_range_bound<<<nblk(g.NP, 256), 256, 0, s>>>(g, st, exc, cap, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_convert(long long n, const long long* src, T* dst, cudaStream_t s) {
  if (n > 0) k_convert<T><<<nblk(n, 256), 256, 0, s>>>(n, src, dst);
  return cudaGetLastError();
}
template cudaError_t launch_convert<int>(long long, const long long*, int*, cudaStream_t);
template cudaError_t launch_convert<long long>(long long, const long long*, long long*,
                                               cudaStream_t);

template <typename T>
cudaError_t launch_sum_pos(long long n, const T* x, long long* out, cudaStream_t s) {
  if (n > 0) k_sum_pos<T><<<nblk(n, 256), 256, 0, s>>>(n, x, out);
  return cudaGetLastError();
}
template cudaError_t launch_sum_pos<int>(long long, const int*, long long*, cudaStream_t);
template cudaError_t launch_sum_pos<long long>(long long, const long long*, long long*,
                                               cudaStream_t);

template <typename T>
cudaError_t launch_init_heights(const Geo& g, const T* exc, const uint64_t* kmask, int* h,
                                cudaStream_t s) {
  k_init_heights<T><<<nblk(g.NP, 256), 256, 0, s>>>(g, exc, kmask, h);
  return cudaGetLastError();
}
template cudaError_t launch_init_heights<int>(const Geo&, const int*, const uint64_t*, int*,
                                              cudaStream_t);
template cudaError_t launch_init_heights<long long>(const Geo&, const long long*,
                                                    const uint64_t*, int*, cudaStream_t);

template <typename T>
cudaError_t launch_active(const Geo& g, const T* exc, const int* h, int* act,
                          unsigned long long* count, cudaStream_t s) {
  k_active<T><<<nblk(g.NP, 256), 256, 0, s>>>(g, exc, h, act, count);
  return cudaGetLastError();
}
template cudaError_t launch_active<int>(const Geo&, const int*, const int*, int*,
                                        unsigned long long*, cudaStream_t);
template cudaError_t launch_active<long long>(const Geo&, const long long*, const int*, int*,
                                              unsigned long long*, cudaStream_t);

template <typename T>
cudaError_t launch_init_marks(long long n, const T* exc, int* mark, cudaStream_t s) {
  k_init_marks<T><<<nblk(n, 256), 256, 0, s>>>(n, exc, mark);
  return cudaGetLastError();
}
template cudaError_t launch_init_marks<int>(long long, const int*, int*, cudaStream_t);
template cudaError_t launch_init_marks<long long>(long long, const long long*, int*,
                                                  cudaStream_t);

cudaError_t launch_extract_cuts(const Geo& g, int nd, long long N, const int* mark, const int* h,
                                int* cmin, int* cmax, cudaStream_t s) {
  if (N > 0) k_extract_cuts<<<nblk(N, 256), 256, 0, s>>>(g, nd, N, mark, h, cmin, cmax);
  return cudaGetLastError();
}

}  // namespace lfg
