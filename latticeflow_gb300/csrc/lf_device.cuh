// Device-side data structures and kernels of the lattice max-flow engine.
//
// Layout in HBM (one lattice):
//   every lattice is viewed as 3-d (A, B, C), C fastest; a 2-d (nx, ny)
//   lattice is (1, nx, ny).  Extents are padded up to whole tiles
//   (Ap, Bp, Cp); padding nodes carry zero capacity and never become active.
//   res[k * NP + i]  residual capacity of node i in direction k (SoA, one
//                    plane per kernel direction, lattice order)
//   exc[i]           net excess: > 0 excess, < 0 remaining sink capacity
//   h[i]             height (distance label), kHInf = cannot reach a sink
//   mask[i]          bit k set iff res[k][i] > 0 and the edge is usable
//   kmask[i]         (sections only) bit k set iff both ends share a section
// Tiles are TA x TB x TC boxes with TC = 32 so that a warp covers one row.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lfg {

constexpr int kHInf = 0x3fffffff;
constexpr int kMaxKDev = 48;

struct Geo {
  int A, B, C;          // logical extents
  int TA, TB, TC;       // tile extents
  int Ap, Bp, Cp;       // padded extents
  int nta, ntb, ntc;    // tiles per axis
  long long NP;         // Ap * Bp * Cp
  int ntiles;
};

struct Stencil {
  int K;
  int HA, HB, HC;                 // halo width per axis
  signed char da[kMaxKDev], db[kMaxKDev], dc[kMaxKDev];
  unsigned char rev[kMaxKDev];
};

template <typename T>
struct PRParams {
  Geo g;
  Stencil st;
  T* res;
  T* exc;
  int* h;
  const uint64_t* kmask;   // may be null
  int* act_cur;
  int* act_next;
  unsigned long long* counters;  // [0] processed tiles, [1] processed tile launches
  int hmax;
  int sweeps;
};

struct BFSParams {
  Geo g;
  Stencil st;
  int* h;
  uint64_t* mask;
  int* dirty_cur;
  int* dirty_next;
  int* any_changed;
  int max_local;
  unsigned long long* counters;  // [1] processed tiles
};

struct ReachParams {
  Geo g;
  Stencil st;
  int* mark;
  const uint64_t* mask;
  int* dirty_cur;
  int* dirty_next;
  int* any_changed;
  int max_local;
};

}  // namespace lfg
