// Per-lattice element kernels: energy / capacity fill, range bound, type
// conversion, reductions and cut extraction.  The solve itself runs on the
// pool kernels (lf_pool_tile.cuh, lf_pool.cu).
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "lf_fill.cuh"
#include "lf_pool_runner.h"
#include "lf_tile_common.cuh"

namespace lfg {

// ------------------------------------------------------------------ fill

// Energy form (interface.hpp:49-60).  One thread per (node, filling edge);
// edge 0 also adds the node's unary term.  Decomposition of a submodular
// pairwise table [[A, B], [C, D]] (rows: source node off/on):
//   node cost A (off) / D (on), then f(0,1) = B - A, f(1,0) = C - D as two
//   directed capacities, moving a negative one into the unary terms.
// exc = cost(off) - cost(on): > 0 prefers on (supply), < 0 prefers off.
// VEC: the caller's arrays are 16-byte aligned, so each pairwise table (32
// bytes) is read with two 16-byte loads and each unary pair with one; fewer,
// wider requests matter when the arrays are pinned host memory read in place.
template <bool VEC>
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
      int64_t E0, E1;
      if (VEC) {
        const longlong2 ue = reinterpret_cast<const longlong2*>(unary)[b];
        E0 = ue.x;
        E1 = ue.y;
      } else {
        E0 = unary[2 * b];
        E1 = unary[2 * b + 1];
      }
      atom_add(&exc[u], (long long)(E0 - E1));
      c0 += E0;
    }
    int na = a + st.da[e], nb = bb + st.db[e], nc = c + st.dc[e];
    if (na >= 0 && na < g.A && nb >= 0 && nb < g.B && nc >= 0 && nc < g.C) {
      long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
      const int64_t* q = binary + (b * Kp + e) * 4;
      long long A, B, C, D;
      if (VEC) {
        const longlong2 q0 = reinterpret_cast<const longlong2*>(q)[0];
        const longlong2 q1 = reinterpret_cast<const longlong2*>(q)[1];
        A = q0.x; B = q0.y; C = q1.x; D = q1.y;
      } else {
        A = q[0]; B = q[1]; C = q[2]; D = q[3];
      }
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

__device__ __forceinline__ void fill_node_coords(const Geo& g, int nd, long long r, int& a, int& b,
                                                 int& c) {
  if (nd == 2) { a = 0; b = int(r / g.C); c = int(r % g.C); }
  else { c = int(r % g.C); b = int((r / g.C) % g.B); a = int(r / ((long long)g.C * g.B)); }
}

// Block sum of the constant term, one atomic per block.
__device__ __forceinline__ void fill_add_c0(long long c0, long long* c0sum) {
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

// One thread per node (k_fill_energy's gather form): no atomics on the
// accumulators.  Used for device-resident energies whose Kp does not divide
// a warp; pinned host energies read in place keep the scatter, which reads
// each pairwise table once.
template <bool VEC>
__global__ void k_fill_energy_gather(Geo g, Stencil st, int nd, long long N,
                                     const int64_t* unary, const int64_t* binary, long long* exc,
                                     long long* cap, long long* c0sum, int* err) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long c0 = 0;
  if (r < N) {
    int a, b, c;
    fill_node_coords(g, nd, r, a, b, c);
    bool bad = false;
    c0 = fill_gather_node<VEC>(g, st, r, a, b, c, unary, binary, exc, cap, &bad);
    if (bad) atomicExch(err, 1);
  }
  fill_add_c0(c0, c0sum);
}

// The gather with one lane per filling edge: KP (a power of two, dividing
// 32) adjacent lanes of a warp share node r = t / KP, lane e = t % KP takes
// direction e, so a warp's own-table reads are one contiguous span; the
// node's excess share is summed across its lanes with shuffles and written
// by lane 0 of the group.  Same words, same writers per word as the node
// form.
template <bool VEC, int KP>
__global__ void k_fill_energy_lanes(Geo g, Stencil st, int nd, long long N,
                                    const int64_t* unary, const int64_t* binary, long long* exc,
                                    long long* cap, long long* c0sum, int* err) {
  static_assert(KP >= 1 && KP <= 32 && (32 % KP) == 0, "lanes per node must divide a warp");
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long r = t / KP;
  const int e = int(t % KP);
  long long c0 = 0, x = 0, w = 0;
  if (r < N) {
    int a, b, c;
    fill_node_coords(g, nd, r, a, b, c);
    w = ((long long)a * g.Bp + b) * g.Cp + c;
    bool bad = false;
    x = fill_gather_edge<VEC>(g, st, r, a, b, c, w, e, binary, cap, &bad, &c0);
    if (e == 0) x += fill_gather_unary<VEC>(unary, r, &c0);
    if (bad) atomicExch(err, 1);
  }
#pragma unroll
  for (int o = KP / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if (r < N && e == 0 && x) exc[w] += x;
  fill_add_c0(c0, c0sum);
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

// 32-bit working arrays written at once, with a looser range bound than
// k_range_bound: |exc| <= mx_exc and every capacity <= mx_cap give any
// node's excess or residual at most mx_exc + 2 K mx_cap.  When that bound
// stays below 2^31 the copies are the working arrays; otherwise the exact
// per-node bound decides (and the copies are discarded or redone).
__global__ void k_convert_bounded(long long NP, int K, const long long* exc64,
                                  const long long* cap64, int* exc, int* res,
                                  unsigned long long* mx /* [0] |exc|, [1] cap */) {
  __shared__ unsigned long long s_e[32], s_c[32];
  unsigned long long me = 0, mc = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < NP;
       i += (long long)gridDim.x * blockDim.x) {
    const long long e = exc64[i];
    const unsigned long long ae = (unsigned long long)(e < 0 ? -e : e);
    me = ae > me ? ae : me;
    exc[i] = (int)e;
    for (int k = 0; k < K; ++k) {
      const long long c = cap64[(long long)k * NP + i];
      mc = (unsigned long long)c > mc ? (unsigned long long)c : mc;
      res[(long long)k * NP + i] = (int)c;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long xe = __shfl_down_sync(0xffffffffu, me, o);
    const unsigned long long xc = __shfl_down_sync(0xffffffffu, mc, o);
    me = xe > me ? xe : me;
    mc = xc > mc ? xc : mc;
  }
  if ((threadIdx.x & 31) == 0) {
    s_e[threadIdx.x >> 5] = me;
    s_c[threadIdx.x >> 5] = mc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) {
      me = s_e[w] > me ? s_e[w] : me;
      mc = s_c[w] > mc ? s_c[w] : mc;
    }
    if (me) atomicMax(&mx[0], me);
    if (mc) atomicMax(&mx[1], mc);
  }
}

template <typename T>
__global__ void k_convert(long long n, const long long* src, T* dst) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (T)src[i];
}

// sum of max(x, 0) over n values (int64 result)
template <typename T>
__global__ void k_sum_pos(long long n, const T* x, long long* out) {
  // grid-stride partial sums, one atomic per block (not per warp: a
  // lattice-wide sum otherwise queues ~N/32 atomics on one address)
  __shared__ long long part[32];
  long long v = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const T a = x[i];
    if (a > 0) v += (long long)a;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atom_add(out, v);
  }
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

size_t pr_smem_bytes_for(const Geo& g, const Stencil& st, int elem_bytes) {
  int NT = g.TA * g.TB * g.TC;
  int HV = (g.TA + 2 * st.HA) * (g.TB + 2 * st.HB) * (g.TC + 2 * st.HC);
  return elem_bytes == 4 ? pool_pr_smem<int>(st.K, NT, HV) : pool_pr_smem<long long>(st.K, NT, HV);
}

static inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

cudaError_t launch_fill_energy(const Geo& g, const Stencil& st, int nd, long long N,
                               const int64_t* u, const int64_t* b, long long* exc,
                               long long* cap, long long* c0, int* err, int form,
                               cudaStream_t s) {
  long long n = N * (st.K / 2);
  const bool vec = (reinterpret_cast<uintptr_t>(u) % 16 == 0) && (reinterpret_cast<uintptr_t>(b) % 16 == 0);
  // form: 0 = lanes (where Kp divides a warp, else per node), 1 = per node,
  // 2 = scatter
  const int Kp = st.K / 2;
  const bool gather = form == 0 || form == 1;
  if (form == 0 && N > 0 && (Kp == 2 || Kp == 4 || Kp == 8)) {
#define LF_FILL_LANES(KP)                                                                      \
  if (vec) k_fill_energy_lanes<true, KP><<<nblk(N * KP, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err); \
  else k_fill_energy_lanes<false, KP><<<nblk(N * KP, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
    if (Kp == 2) { LF_FILL_LANES(2) }
    else if (Kp == 4) { LF_FILL_LANES(4) }
    else { LF_FILL_LANES(8) }
#undef LF_FILL_LANES
  } else if (gather && N > 0) {
    if (vec) k_fill_energy_gather<true><<<nblk(N, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
    else k_fill_energy_gather<false><<<nblk(N, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
  } else if (n > 0) {
    if (vec) k_fill_energy<true><<<nblk(n, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
    else k_fill_energy<false><<<nblk(n, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, c0, err);
  }
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

cudaError_t launch_convert_bounded(long long NP, int K, const long long* exc64,
                                  const long long* cap64, int* exc, int* res,
                                  unsigned long long* mx, cudaStream_t s) {
  if (NP > 0)
    k_convert_bounded<<<std::min(nblk(NP, 256), 152 * 8), 256, 0, s>>>(NP, K, exc64, cap64, exc,
                                                                       res, mx);
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
  if (n > 0) k_sum_pos<T><<<std::min(nblk(n, 256), 152 * 8), 256, 0, s>>>(n, x, out);
  return cudaGetLastError();
}
template cudaError_t launch_sum_pos<int>(long long, const int*, long long*, cudaStream_t);
template cudaError_t launch_sum_pos<long long>(long long, const long long*, long long*,
                                               cudaStream_t);

cudaError_t launch_extract_cuts(const Geo& g, int nd, long long N, const int* mark, const int* h,
                                int* cmin, int* cmax, cudaStream_t s) {
  if (N > 0) k_extract_cuts<<<nblk(N, 256), 256, 0, s>>>(g, nd, N, mark, h, cmin, cmax);
  return cudaGetLastError();
}

}  // namespace lfg
