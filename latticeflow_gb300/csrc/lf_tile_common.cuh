// Device helpers shared by the tile kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lf_device.cuh"

namespace lfg {


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

}  // namespace lfg
