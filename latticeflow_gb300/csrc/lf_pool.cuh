// Instance pool: any number of lattices of any shape in shared device pools,
// worked on by persistent kernels that drain device-side tile queues.
//
// A plain solve is a pool of one lattice; a batch is a pool of many.  Every
// lattice keeps its own padded layout (see lf_device.cuh) at an offset in the
// pools; tiles of all lattices share one global tile numbering.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lf_device.cuh"

namespace lfg {

struct InstDesc {
  Geo g;
  Stencil st;
  long long node_base;  // first node of the lattice in the node pools
  long long res_base;   // first element of its residual planes
  long long plane;      // elements between two residual planes (g.NP, or the
                        // enclosing lattice's NP for a lattice stacked in it)
  int tile_base;        // global id of its tile 0
  int hmax;             // height cap of the current epoch
  int done;             // no node can push any more: excluded from relabels
  int active;           // lattice takes part in this solve
};

// Work queue of global tile ids, double buffered over passes.
//   flag[b][t] = 1 while tile t sits in list b
//   ctr[2b] = entries in list b; ctr[3] / ctr[1] = pop head of a pass that
//   reads list 0 / 1.  Before a pass reading list `cur` the host zeroes the
//   count of the other list and this pass's head, which is ONE contiguous
//   pair (ctr[2..3] for cur = 0, ctr[0..1] for cur = 1).
__host__ __device__ __forceinline__ int q_count_idx(int b) { return 2 * b; }
__host__ __device__ __forceinline__ int q_head_idx(int cur) { return cur ? 1 : 3; }

struct TileQueue {
  int* flag[2];
  int* list[2];
  unsigned* ctr;
};

template <typename T>
struct PoolPR {
  InstDesc inst0;         // the lattice itself when the pool holds one
  InstDesc* inst;
  const int* tile_inst;
  T* res;
  T* exc;
  int* h;
  const uint64_t* kmask;  // may be null
  TileQueue q;
  int cur;                // list consumed by this pass; the other is filled
  int sweeps;
  unsigned long long* counters;  // [0] processed tiles
};

struct PoolBFS {
  InstDesc inst0;
  InstDesc* inst;
  const int* tile_inst;
  int* h;
  const uint64_t* mask;
  TileQueue q;
  int cur;
  int max_local;
  int* any_changed;
  unsigned long long* counters;  // [1] processed tiles
};

struct PoolReach {
  InstDesc inst0;
  InstDesc* inst;
  const int* tile_inst;
  int* mark;
  const uint64_t* mask;
  TileQueue q;
  int cur;
  int max_local;
  int* any_changed;
};

#ifdef __CUDACC__
__device__ __forceinline__ void enqueue_tile(const TileQueue& q, int nxt, int t) {
  if (atomicExch(&q.flag[nxt][t], 1) == 0) {
    unsigned pos = atomicAdd(&q.ctr[q_count_idx(nxt)], 1u);
    q.list[nxt][pos] = t;
  }
}

// Number of tiles queued for the pass reading list `cur` (written by the
// previous pass); the blocks of a pass stride over the list.
__device__ __forceinline__ unsigned queued_count(const TileQueue& q, int cur) {
  return *((volatile unsigned*)&q.ctr[q_count_idx(cur)]);
}
#endif  // __CUDACC__

}  // namespace lfg
