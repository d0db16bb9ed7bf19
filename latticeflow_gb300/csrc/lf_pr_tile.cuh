// Tile push/relabel kernel (template; instantiated in lf_pr32.cu / lf_pr64.cu).
//
// One CTA stages one tile in shared memory: every residual plane, the excess
// and the heights with a halo.  Up to `sweeps` rounds of
//   push: each node with excess sends flow to lower neighbours with residual
//         capacity, lowest index first (heights are frozen during the phase,
//         so an edge carries flow in one direction only and the only shared
//         update is the atomic excess add);
//   relabel: a node that still has excess and no lower residual neighbour
//         moves to one above its lowest residual neighbour
// run until no node of the tile is active.  Flow pushed across the tile edge
// is delivered at the end with global atomics (residual of the reverse edge
// and the neighbour's excess) and flags the neighbour tile for the next
// launch; edge nodes write back their excess as a delta for the same reason.
// Stale halo heights can leave labels invalid; the next global relabel
// recomputes them exactly, and the final answer depends only on the residual
// graph, never on the labels.
#pragma once
#include "lf_tile_common.cuh"

namespace lfg {

// ------------------------------------------------------- push / relabel

template <typename T, int K>
__global__ void __launch_bounds__(1024) k_pr_tile(PRParams<T> p) {
  const int tile = blockIdx.x;
  if (!p.act_cur[tile]) return;
  extern __shared__ __align__(16) unsigned char smem[];
  const Geo& g = p.g;
  const TileCtx x = tile_ctx(g, p.st, tile);
  const int NT = x.NT;
  T* s_res = reinterpret_cast<T*>(smem);
  T* s_exc = s_res + (size_t)K * NT;
  int* s_h = reinterpret_cast<int*>(s_exc + NT);
  int* s_hoff = s_h + x.HV;
  int* s_toff = s_hoff + K;
  const int t = threadIdx.x;
  if (t < K) {
    s_hoff[t] = (p.st.da[t] * x.HBB + p.st.db[t]) * x.HCC + p.st.dc[t];
    s_toff[t] = (p.st.da[t] * g.TB + p.st.db[t]) * g.TC + p.st.dc[t];
  }
  load_halo_heights(g, p.st, x, p.h, s_h);
  uint64_t outm = 0;
  T r0[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    r0[k] = p.res[(long long)k * g.NP + x.gi];
    s_res[k * NT + t] = r0[k];
    int na = x.ia + p.st.da[k], nb = x.ib + p.st.db[k], nc = x.ic + p.st.dc[k];
    if (na < 0 || na >= g.TA || nb < 0 || nb >= g.TB || nc < 0 || nc >= g.TC) outm |= 1ull << k;
  }
  const T e0 = p.exc[x.gi];
  s_exc[t] = e0;
  const uint64_t km = p.kmask ? p.kmask[x.gi] : ~0ull;
  __syncthreads();

  int my_h = s_h[x.hidx];
  for (int it = 0; it < p.sweeps; ++it) {
    // push phase: heights are fixed, so an edge is used in one direction only
    T e = s_exc[t];
    if (e > 0 && my_h < p.hmax) {
      T sent = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (!((km >> k) & 1)) continue;
        const T rem = e - sent;
        if (rem <= 0) break;
        const T r = s_res[k * NT + t];
        if (r <= 0) continue;
        if (s_h[x.hidx + s_hoff[k]] >= my_h) continue;
        const T d = rem < r ? rem : r;
        s_res[k * NT + t] = r - d;
        sent += d;
        if (!((outm >> k) & 1)) {
          const int tn = t + s_toff[k];
          atom_add(&s_exc[tn], d);
          s_res[p.st.rev[k] * NT + tn] += d;
        }
      }
      if (sent) atom_add(&s_exc[t], (T)-sent);
    }
    __syncthreads();
    // relabel phase
    e = s_exc[t];
    int act = 0;
    if (e > 0 && my_h < p.hmax) {
      int hmin = kHInf;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (((km >> k) & 1) && s_res[k * NT + t] > 0) {
          const int hn = s_h[x.hidx + s_hoff[k]];
          hmin = hn < hmin ? hn : hmin;
        }
      }
      if (hmin >= my_h) {
        my_h = (hmin >= p.hmax - 1) ? p.hmax : hmin + 1;
        s_h[x.hidx] = my_h;
      }
      act = my_h < p.hmax;
    }
    if (!__syncthreads_or(act)) break;
  }
  __syncthreads();

  // write back; flow that left the tile is delivered to the neighbour
  const T ef = s_exc[t];
  if (outm) atom_add(&p.exc[x.gi], (T)(ef - e0));
  else p.exc[x.gi] = ef;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const T rf = s_res[k * NT + t];
    if ((outm >> k) & 1) {
      const T d = r0[k] - rf;
      if (d != 0) {
        atom_add(&p.res[(long long)k * g.NP + x.gi], (T)-d);
        const int A_ = x.a0 + x.ia + p.st.da[k], B_ = x.b0 + x.ib + p.st.db[k],
                  C_ = x.c0 + x.ic + p.st.dc[k];
        const long long gn = ((long long)A_ * g.Bp + B_) * g.Cp + C_;
        atom_add(&p.res[(long long)p.st.rev[k] * g.NP + gn], d);
        atom_add(&p.exc[gn], d);
        p.act_next[tile_of(g, A_, B_, C_)] = 1;
      }
    } else {
      p.res[(long long)k * g.NP + x.gi] = rf;
    }
  }
  p.h[x.gi] = my_h;
  const int still = ef > 0 && my_h < p.hmax;
  if (__syncthreads_or(still) && t == 0) p.act_next[tile] = 1;
  if (t == 0) {
    p.act_cur[tile] = 0;
    atomicAdd(&p.counters[0], 1ull);
  }
}

template <typename T>
cudaError_t launch_pr_tile(const PRParams<T>& p, cudaStream_t s) {
  size_t smem = pr_smem_bytes<T>(p.g, p.st);
  int threads = p.g.TA * p.g.TB * p.g.TC;
  switch (p.st.K) {
#define X(KK)                                                                             \
  case KK: {                                                                              \
    static bool attr_set = false;                                                         \
    if (!attr_set) {                                                                      \
      cudaFuncSetAttribute(k_pr_tile<T, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                           227 * 1024);                                                   \
      cudaFuncSetAttribute(k_pr_tile<T, KK>,                                              \
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);          \
      attr_set = true;                                                                    \
    }                                                                                     \
    k_pr_tile<T, KK><<<p.g.ntiles, threads, smem, s>>>(p);                                \
    break;                                                                                \
  }
    LF_K_LIST(X)
#undef X
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}


}  // namespace lfg
