// Device helpers shared by the tile kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lf_device.cuh"

namespace lfg {

#define LF_K_LIST(X) X(4) X(6) X(8) X(12) X(16) X(18) X(20) X(24) X(26) X(28) X(32) X(36) X(40) X(48)

__device__ __forceinline__ int atom_add(int* p, int v) { return atomicAdd(p, v); }
__device__ __forceinline__ long long atom_add(long long* p, long long v) {
  return (long long)atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

__device__ __forceinline__ int tile_of(const Geo& g, int a, int b, int c) {
  return ((a / g.TA) * g.ntb + (b / g.TB)) * g.ntc + (c / g.TC);
}

// --------------------------------------------------------- tile geometry

struct TileCtx {
  int NT, HAA, HBB, HCC, HV;
  int ia, ib, ic, a0, b0, c0;
  long long gi;
  int hidx;
};

__device__ __forceinline__ TileCtx tile_ctx(const Geo& g, const Stencil& st, int tile) {
  TileCtx x;
  x.NT = g.TA * g.TB * g.TC;
  x.HAA = g.TA + 2 * st.HA;
  x.HBB = g.TB + 2 * st.HB;
  x.HCC = g.TC + 2 * st.HC;
  x.HV = x.HAA * x.HBB * x.HCC;
  const int t = threadIdx.x;
  x.ic = t % g.TC;
  x.ib = (t / g.TC) % g.TB;
  x.ia = t / (g.TC * g.TB);
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  x.a0 = ta * g.TA;
  x.b0 = tb * g.TB;
  x.c0 = tc * g.TC;
  x.gi = ((long long)(x.a0 + x.ia) * g.Bp + (x.b0 + x.ib)) * g.Cp + (x.c0 + x.ic);
  x.hidx = ((x.ia + st.HA) * x.HBB + (x.ib + st.HB)) * x.HCC + (x.ic + st.HC);
  return x;
}

// Loads the heights of the tile plus halo into s_h (kHInf outside the array).
__device__ __forceinline__ void load_halo_heights(const Geo& g, const Stencil& st,
                                                  const TileCtx& x, const int* h, int* s_h) {
  for (int i = threadIdx.x; i < x.HV; i += blockDim.x) {
    int hc = i % x.HCC, hb = (i / x.HCC) % x.HBB, ha = i / (x.HCC * x.HBB);
    int A_ = x.a0 + ha - st.HA, B_ = x.b0 + hb - st.HB, C_ = x.c0 + hc - st.HC;
    int v = kHInf;
    if (A_ >= 0 && A_ < g.Ap && B_ >= 0 && B_ < g.Bp && C_ >= 0 && C_ < g.Cp)
      v = h[((long long)A_ * g.Bp + B_) * g.Cp + C_];
    s_h[i] = v;
  }
}

__device__ __forceinline__ void mark_neighbour_tiles(const Geo& g, int tile, int* flags) {
  const int tc = tile % g.ntc, tb = (tile / g.ntc) % g.ntb, ta = tile / (g.ntc * g.ntb);
  for (int da = -1; da <= 1; ++da)
    for (int db = -1; db <= 1; ++db)
      for (int dc = -1; dc <= 1; ++dc) {
        int a = ta + da, b = tb + db, c = tc + dc;
        if (a < 0 || a >= g.nta || b < 0 || b >= g.ntb || c < 0 || c >= g.ntc) continue;
        if (da == 0 && db == 0 && dc == 0) continue;
        flags[(a * g.ntb + b) * g.ntc + c] = 1;
      }
}

template <typename T>
static inline size_t pr_smem_bytes(const Geo& g, const Stencil& st) {
  int NT = g.TA * g.TB * g.TC;
  int HV = (g.TA + 2 * st.HA) * (g.TB + 2 * st.HB) * (g.TC + 2 * st.HC);
  return size_t(st.K + 1) * NT * sizeof(T) + size_t(HV + 2 * st.K) * sizeof(int);
}

}  // namespace lfg
