// Tail of a push/relabel solve: few active nodes left.
//
// When a handful of nodes still hold excess, the tile passes spend most of
// their launches on one excess that has just filled its nearest deficit: the
// exact distances of the last global relabel now point at a node that is no
// longer a deficit, and the excess climbs the heights around it pass after
// pass until the next relabel (one small deficit filled per epoch).  Here
// each active node instead sends its excess along a breadth-first tree of
// residual edges to as many deficits as it needs:
//   1. BFS from the active node u over edges with residual > 0 (within the
//      section mask, skipping nodes the relabel found cut off), until the
//      deficits met cover exc(u), the tree holds `cap` nodes or the level
//      list is full;
//   2. bottom-up, each tree node's demand = its own deficit + its children's
//      contributions, and its contribution to its parent = min(demand,
//      residual of the tree edge parent -> node);
//   3. top-down, u sends min(exc(u), demand(u)); every node keeps up to
//      its own deficit of what it receives and passes the rest to its
//      children, each child taking at most its contribution.
// Every edge carries at most its residual and every node ends with what it
// held plus what it kept, so the result is again a preflow; the solve then
// continues with a global relabel as usual.  The final cut sets do not depend
// on which preflow reaches the maximum.  One block handles the active nodes
// one after another (each tree stops as soon as its own excess is covered;
// trees of different nodes built at once would race on shared edges).  Every
// loop is bounded; the block reports the excess that left the roots.
#include <climits>

#include "lf_pool_runner.h"

namespace lfg {

namespace {

__device__ __forceinline__ int tail_inst_of(const long long* nbase, int n, long long i) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (nbase[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// take up to `want` from *rem (other children of the same parent take from
// it too); gives up (returns 0) after a bounded number of retries
__device__ __forceinline__ long long take_bounded(long long* rem, long long want) {
  long long old = *((volatile long long*)rem);
  for (int it = 0; it < 256; ++it) {
    if (old <= 0 || want <= 0) return 0;
    const long long t = want < old ? want : old;
    const long long seen = (long long)atomicCAS((unsigned long long*)rem,
                                                (unsigned long long)old,
                                                (unsigned long long)(old - t));
    if (seen == old) return t;
    old = seen;
  }
  return 0;
}

template <typename T>
__global__ void __launch_bounds__(1024)
k_pool_tail(const InstDesc* insts, const long long* nbase, int n, T* res, T* exc, const int* h,
            const uint64_t* kmask, const long long* act, const unsigned* nact_p, TailScratch s,
            int stamp0, unsigned long long* moved) {
  __shared__ int sh_tail, sh_nlev, sh_stop;
  __shared__ long long sh_coll;
  __shared__ unsigned long long sh_moved;
  const int tid = threadIdx.x, NT = blockDim.x;
  const int nact = int(*nact_p < (unsigned)s.max_active ? *nact_p : (unsigned)s.max_active);
  if (tid == 0) sh_moved = 0;
  __syncthreads();
  for (int a = 0; a < nact; ++a) {
    const long long u = act[a];
    const T eu = exc[u];  // every thread reads it after the last barrier
    if (eu <= 0 || h[u] >= kHInf) continue;
    const int in = tail_inst_of(nbase, n, u);
    const InstDesc& I = insts[in];
    const Geo& g = I.g;
    const long long base = nbase[in];
    const int stamp = stamp0 + a;
    if (tid == 0) {
      s.node[0] = u;
      s.par[0] = -1;
      s.dir[0] = 0;
      s.dem[0] = 0;
      s.vis[u] = stamp;
      sh_tail = 1;
      sh_nlev = 0;
      sh_stop = 0;
      sh_coll = 0;
    }
    __syncthreads();
    // 1. BFS, one level per round
    int head = 0;
    for (int round = 0; round < s.lvl_cap; ++round) {
      const int lo = head, hi = sh_tail < s.cap ? sh_tail : s.cap;
      __syncthreads();  // everyone has read sh_tail before it grows
      if (lo >= hi) break;
      if (tid == 0) s.lvl[sh_nlev++] = lo;
      for (int pos = lo + tid; pos < hi; pos += NT) {
        const long long v = s.node[pos];
        const long long li = v - base;
        const int c = int(li % g.Cp), b = int((li / g.Cp) % g.Bp),
                  a3 = int(li / ((long long)g.Cp * g.Bp));
        const uint64_t km = kmask ? kmask[v] : ~0ull;
        for (int k = 0; k < I.st.K; ++k) {
          if (!((km >> k) & 1)) continue;
          if (res[I.res_base + (long long)k * I.plane + li] <= 0) continue;
          const int na = a3 + I.st.da[k], nb = b + I.st.db[k], nc = c + I.st.dc[k];
          if (na < 0 || na >= g.A || nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) continue;
          const long long w = base + ((long long)na * g.Bp + nb) * g.Cp + nc;
          if (h[w] >= kHInf) continue;
          if (atomicMax(&s.vis[w], stamp) >= stamp) continue;  // already in this tree
          const int p = atomicAdd(&sh_tail, 1);
          if (p >= s.cap) continue;
          s.node[p] = w;
          s.par[p] = pos;
          s.dir[p] = (unsigned char)k;
          s.dem[p] = 0;
          const T e = exc[w];
          if (e < 0) atomicAdd((unsigned long long*)&sh_coll, (unsigned long long)(-(long long)e));
        }
      }
      __syncthreads();
      head = hi;
      if (tid == 0 && (sh_coll >= (long long)eu || sh_tail >= s.cap || sh_nlev >= s.lvl_cap - 1))
        sh_stop = 1;
      __syncthreads();
      if (sh_stop) break;
    }
    const int total = sh_tail < s.cap ? sh_tail : s.cap;
    // the children of the last expanded level form one more level
    if (tid == 0) {
      if (head < total) s.lvl[sh_nlev++] = head;
      s.lvl[sh_nlev] = total;
    }
    __syncthreads();
    const int nlev = sh_nlev;
    // 2. bottom-up contributions (levels nlev-1 .. 1)
    for (int L = nlev - 1; L >= 1; --L) {
      const int lo = s.lvl[L], hi = s.lvl[L + 1];
      for (int pos = lo + tid; pos < hi; pos += NT) {
        const long long v = s.node[pos];
        const T e = exc[v];
        long long d = s.dem[pos] + (e < 0 ? -(long long)e : 0);
        const int pp = s.par[pos];
        const long long pv = s.node[pp];
        const long long r = (long long)res[I.res_base + (long long)s.dir[pos] * I.plane + (pv - base)];
        if (d > r) d = r;
        s.dem[pos] = d;  // now: this node's contribution to its parent
        if (d > 0) atomicAdd((unsigned long long*)&s.dem[pp], (unsigned long long)d);
      }
      __syncthreads();
    }
    // 3. top-down
    if (tid == 0) {
      long long F = s.dem[0] < (long long)eu ? s.dem[0] : (long long)eu;
      if (F < 0) F = 0;
      s.rem[0] = F;
      exc[u] = (T)((long long)eu - F);
    }
    __syncthreads();
    for (int L = 1; L < nlev; ++L) {
      const int lo = s.lvl[L], hi = s.lvl[L + 1];
      for (int pos = lo + tid; pos < hi; pos += NT) {
        const int pp = s.par[pos];
        const long long got = take_bounded(&s.rem[pp], s.dem[pos]);
        long long keep = 0;
        if (got > 0) {
          const long long v = s.node[pos], pv = s.node[pp];
          const int k = s.dir[pos];
          res[I.res_base + (long long)k * I.plane + (pv - base)] -= (T)got;
          res[I.res_base + (long long)I.st.rev[k] * I.plane + (v - base)] += (T)got;
          const T e = exc[v];
          const long long own = e < 0 ? -(long long)e : 0;
          keep = got < own ? got : own;
          if (keep) exc[v] = (T)((long long)e + keep);
          if (L == 1) atomicAdd(&sh_moved, (unsigned long long)got);  // left the root
        }
        s.rem[pos] = got - keep;
      }
      __syncthreads();
    }
    // what a node could not pass on (only if a bounded take gave up) stays
    // with it as excess
    for (int pos = tid; pos < total; pos += NT) {
      const long long left = s.rem[pos];
      if (left > 0) {
        const long long v = s.node[pos];
        exc[v] = (T)((long long)exc[v] + left);
      }
    }
    __syncthreads();
  }
  if (tid == 0) *moved = sh_moved;
}

// active nodes (exc > 0, finite height) of unfinished lattices, up to `cap`
template <typename T>
__global__ void k_pool_list_active(const InstDesc* insts, const long long* nbase, int n,
                                   long long NP, const T* exc, const int* h, long long* list,
                                   unsigned* count, int cap) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  if (!(exc[i] > 0 && h[i] < kHInf)) return;
  const InstDesc& I = insts[tail_inst_of(nbase, n, i)];
  if (I.done || !I.active) return;
  unsigned p = atomicAdd(count, 1u);
  if (p < (unsigned)cap) list[p] = i;
}

}  // namespace

template <typename T>
cudaError_t launch_pool_tail(const InstDesc* insts, const long long* nbase, int n, long long NP,
                             T* res, T* exc, const int* h, const uint64_t* kmask,
                             const TailScratch& s, int stamp0, unsigned long long* moved,
                             cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(s.count, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  const int B = 256;
  k_pool_list_active<T><<<int((NP + B - 1) / B), B, 0, st>>>(insts, nbase, n, NP, exc, h, s.list,
                                                              s.count, s.max_active);
  k_pool_tail<T><<<1, 1024, 0, st>>>(insts, nbase, n, res, exc, h, kmask, s.list, s.count, s,
                                     stamp0, moved);
  return cudaGetLastError();
}

template cudaError_t launch_pool_tail<int>(const InstDesc*, const long long*, int, long long, int*,
                                           int*, const int*, const uint64_t*, const TailScratch&,
                                           int, unsigned long long*, cudaStream_t);
template cudaError_t launch_pool_tail<long long>(const InstDesc*, const long long*, int, long long,
                                                 long long*, long long*, const int*,
                                                 const uint64_t*, const TailScratch&, int,
                                                 unsigned long long*, cudaStream_t);

}  // namespace lfg
