// The reference's TV regularisation path on the GPU:
// calculate2dTV<Kernel, int64>(nx, ny, f, vector<double> lambdas)
// (tv/tv_solver.hpp:657-681).
//
// The reference solves the parametric flow once at the largest lambda, makes
// one path segment per level set, and then walks down in lambda with an event
// heap (tv_solver.hpp:300-564): two neighbouring segments whose lines r(lambda)
// meet join; a segment splits where a region max-flow probe finds a cut
// (tv_regpath_node.hpp:416-744), located by a closed form and integer
// bisection; a split's cut edges are saturated and both parts become new
// segments.  The output at each requested lambda is every pixel's segment
// line, traced down the segment tree (tv_solver.hpp:566-642).
//
// Here the event heap, the segment lines and every integer rule of the
// reference run on the host (they are sequential and O(1) per event); the
// lattice state lives on the device and every node-level step is a kernel:
//   * the initial parametric flow: engine_run_parametric (level sets in the
//     reference's order);
//   * a segment's region sums (128-bit), offsets and scale
//     (PFFlowNode::setOffsetAndScale, pf_flow_node.hpp:293-309;
//     TV_PRFlow::setRegionToLambda, tv_push_relabel.hpp:414-468);
//   * a region probe (TV_PRFlow::runPartitionedSection,
//     tv_push_relabel.hpp:84-237): the engine's max-flow restricted to the
//     region by the section mask, the region split by its maximal on-set,
//     the per-side sums and the cut value read off in one pass;
//   * a split's cut saturation (applyPartioningCut, tv_push_relabel.hpp:239-248).
// The region probes differ from the reference's only in the max-flow (push
// order), which changes flows inside a region but not the region's sums:
// those depend only on the flows across region boundaries, which every split
// saturates (edge sums are invariant), and on the cut, which is unique for
// the probes of any input without exact ties.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <queue>
#include <set>
#include <unordered_set>
#include <vector>

#include "lf_engine.h"

namespace lfg {

namespace {

typedef long long dtype;
typedef __int128 comp_type;

constexpr int kScaleBits = 48;   // n_bits_scale_precision for int64 (pf_flow_node.hpp:106)
constexpr int kAdjustBits = 16;  // n_bits_function_room for int64 (pf_flow_node.hpp:110)
constexpr dtype kDtMax = LLONG_MAX;

inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

// ------------------------------------------------------------ integer rules

inline comp_type iabs(comp_type x) { return x >= 0 ? x : -x; }
// products formed in the reference's dtype: two's-complement wrap
inline dtype wmul(dtype a, dtype b) { return dtype((unsigned long long)a * (unsigned long long)b); }

// PFFlowNode::multFVScale (pf_flow_node.hpp:160-176): round-half-away of
// fv * lm / 2^48, the division truncating toward zero
__host__ __device__ inline dtype mult_fv_scale(comp_type fv, dtype lm) {
  fv *= lm;
  fv += (fv > 0 ? 1 : -1) * (comp_type(1) << (kScaleBits - 1));
  // truncating division by 2^48
  const comp_type q = fv >= 0 ? (fv >> kScaleBits) : -((-fv) >> kScaleBits);
  return dtype(q);
}

// PFFlowNode::getScaleFromQuotient_T (pf_flow_node.hpp:178-203)
dtype scale_from_quotient(comp_type numer, comp_type denom) {
  if (denom == 0) return kDtMax;
  numer *= (comp_type(1) << kScaleBits);
  numer /= denom;
  return numer > kDtMax ? kDtMax : dtype(numer);
}

// floorAverage (common/type_processing.hpp:58-70)
dtype floor_average(comp_type sum, long n) {
  if (sum < 0) sum -= (n - 1);
  sum /= n;
  return dtype(sum);
}

dtype to_scale(double lm) { return dtype(std::round(lm * double(int64_t(1) << kScaleBits))); }

// ---------------------------------------------------------------- kernels

// 128-bit accumulators: (lo, hi) words, added with carry
__device__ __forceinline__ void atomic_add_i128(unsigned long long* acc, comp_type v) {
  const unsigned long long lo = (unsigned long long)v;
  const unsigned long long hi = (unsigned long long)(v >> 64);
  const unsigned long long old = atomicAdd(&acc[0], lo);
  const unsigned long long carry = (old + lo) < old ? 1ull : 0ull;
  if (hi + carry) atomicAdd(&acc[1], hi + carry);
}

__device__ __forceinline__ comp_type warp_sum_i128(comp_type v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long lo = __shfl_down_sync(0xffffffffu, (unsigned long long)v, o);
    const unsigned long long hi = __shfl_down_sync(0xffffffffu, (unsigned long long)(v >> 64), o);
    v += (comp_type)(((unsigned __int128)hi << 64) | lo);
  }
  return v;
}

// one 128-bit sum per warp into acc (lane 0)
__device__ __forceinline__ void warp_add(unsigned long long* acc, comp_type v) {
  v = warp_sum_i128(v);
  if ((threadIdx.x & 31) == 0 && v != 0) atomic_add_i128(acc, v);
}

// The segment's nodes at scale lm with offset 0 and its key
// (TVRegPathSegment::syncInformation, tv_regpath_node.hpp:216-224), summing
// r - lm_qii (the segment's gamma) into acc[0..1].
__global__ void k_seg_sync(const int* nodes, int n, dtype lm, int key, const dtype* base,
                           dtype* cur, dtype* off, dtype* exc, int* keys,
                           unsigned long long* acc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  comp_type g = 0;
  if (j < n) {
    const int i = nodes[j];
    const dtype fv = mult_fv_scale(base[i], lm);
    const dtype delta = fv - (cur[i] - off[i]);
    const dtype e = exc[i] - delta;  // reduction += delta
    exc[i] = e;
    cur[i] = fv;
    off[i] = 0;
    keys[i] = key;
    g = comp_type(-e) - fv;  // r - lm_qii with offset 0
  }
  warp_add(acc, g);
}

// influence sum of a region: sum of r - lm_qii (tv_push_relabel.hpp:428-434)
__global__ void k_seg_gamma(const int* nodes, int n, const dtype* cur, const dtype* off,
                            const dtype* exc, unsigned long long* acc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  comp_type g = 0;
  if (j < n) {
    const int i = nodes[j];
    g = comp_type(-exc[i]) + off[i] - cur[i];
  }
  warp_add(acc, g);
}

// TV_PRFlow::setRegionToLambda's per-node step (tv_push_relabel.hpp:456-465)
__global__ void k_seg_offset(const int* nodes, int n, dtype lm, dtype fv_offset, int pull,
                             const dtype* base, dtype* cur, dtype* off, dtype* exc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int i = nodes[j];
  const dtype fv = mult_fv_scale(base[i], lm);
  const dtype o = fv_offset + ((pull && fv > fv_offset) ? 1 : 0);
  const dtype delta = (fv - o) - (cur[i] - off[i]);
  exc[i] -= delta;
  cur[i] = fv;
  off[i] = o;
}

// section mask of a region: bit 63 (the node solves) and bit k for every
// neighbour k in the same region; clear = 0 everywhere on the region
__global__ void k_seg_kmask(const int* nodes, int n, int key, const int* keys, Geo g, Stencil st,
                            uint64_t* kmask, int set) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int i = nodes[j];
  uint64_t m = 0;
  if (set) {
    m = 1ull << 63;
    const int c = i % g.Cp, b = i / g.Cp;
    for (int k = 0; k < st.K; ++k) {
      const int nb = b + st.db[k], nc = c + st.dc[k];
      if (nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) continue;
      if (keys[nb * g.Cp + nc] == key) m |= 1ull << k;
    }
  }
  kmask[i] = m;
}

// Read a probe off the solved region: lab[j] = 1 for nodes of the maximal
// on-set (cannot reach a deficit); acc[0..1] / acc[2..3]: r - lm_qii summed
// over the off / on nodes; acc[4..5]: the cut value (for every off node the
// residual towards each on neighbour, halved: edgeCapacityFromSaturatedOffNodeToOnNode,
// network_flow_node.hpp:192-196); cnt[0]: on nodes.
__global__ void k_seg_probe(const int* nodes, int n, int key, const int* keys, const int* h,
                            const dtype* res, const dtype* exc, const dtype* off,
                            const dtype* cur, Geo g, Stencil st, unsigned char* lab,
                            unsigned long long* acc, unsigned long long* cnt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  comp_type g0 = 0, g1 = 0, cv = 0;
  bool on = false;
  if (j < n) {
    const int i = nodes[j];
    on = h[i] >= kHInf;
    lab[j] = on ? 1 : 0;
    const comp_type gam = comp_type(-exc[i]) + off[i] - cur[i];
    if (on) {
      g1 = gam;
    } else {
      g0 = gam;
      const int c = i % g.Cp, b = i / g.Cp;
      for (int k = 0; k < st.K; ++k) {
        const int nb = b + st.db[k], nc = c + st.dc[k];
        if (nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) continue;
        const int v = nb * g.Cp + nc;
        if (keys[v] == key && h[v] >= kHInf) {
          const dtype a = res[(long long)k * g.NP + i];
          cv += (a < 0 ? -a : a) >> 1;
        }
      }
    }
  }
  warp_add(acc, g0);
  warp_add(acc + 2, g1);
  warp_add(acc + 4, cv);
  const unsigned ons = __popc(__ballot_sync(0xffffffffu, on));
  if ((threadIdx.x & 31) == 0 && ons) atomicAdd(cnt, (unsigned long long)ons);
}

// ------------------------------------------------ fused small-region probe
//
// setRegionToLambda and runPartitionedSection of one region of at most
// kSmallRegion nodes in ONE block: the region's influence sum, the offset
// (floorAverage of a 128-bit sum), every node's new offset and scale, a
// push/relabel max-flow on the region alone (exact BFS relabels from the
// deficits, synchronous pushes along admissible edges, local relabels
// between them), and the probe's read-out -- labels of the maximal on-set
// (nodes that cannot reach a deficit), the per-side influence sums and the
// cut value -- with no host round trip in between.  Residuals stay in the
// lattice arrays (a small region is cache resident); excess, heights and the
// region's local neighbour table live in shared memory.
constexpr int kSmallRegion = 2048;
constexpr int kHUnreached = 0x3fffffff;

// truncating 128-bit / positive 32-bit division by 32-bit limbs
__device__ __forceinline__ comp_type div_i128(comp_type x, long long n) {
  const bool neg = x < 0;
  unsigned __int128 a = neg ? (unsigned __int128)(-x) : (unsigned __int128)x;
  unsigned long long rem = 0;
  unsigned __int128 q = 0;
  for (int i = 3; i >= 0; --i) {
    const unsigned long long cur = (rem << 32) | (unsigned long long)((a >> (32 * i)) & 0xffffffffull);
    q |= (unsigned __int128)(cur / (unsigned long long)n) << (32 * i);
    rem = cur % (unsigned long long)n;
  }
  return neg ? -(comp_type)q : (comp_type)q;
}

__device__ __forceinline__ comp_type block_sum_i128(comp_type v, comp_type* red) {
  v = warp_sum_i128(v);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  comp_type t = 0;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

// local index of padded node v in the sorted region list, or -1
__device__ __forceinline__ int local_index(const int* sn, int n, int v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (sn[mid] < v) lo = mid + 1; else hi = mid;
  }
  return (lo < n && sn[lo] == v) ? lo : -1;
}

// status[0]: 0 done, 1 the epoch cap ended the max-flow (the caller probes
// again with the lattice-wide solver); status[1] / [2] count the epochs and
// BFS levels run (summed over launches); acc as k_seg_probe.  Shared memory:
// excess, inflow and the residuals of every node in each direction (local
// layout j * K + k), then the 128-bit reduction slots, the padded ids, the
// heights and the local neighbour table.
__global__ void __launch_bounds__(1024)
    k_region_probe(const int* nodes, int n, int key, const int* keys, Geo g, Stencil st, dtype lm,
                   int pull, unsigned long long qii_lo, unsigned long long qii_hi,
                   const dtype* base, dtype* cur, dtype* off, dtype* exc, dtype* res,
                   unsigned char* lab, unsigned long long* acc, int* status, int max_epochs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int K = st.K;
  const int n2 = (n + 1) & ~1;
  dtype* e = reinterpret_cast<dtype*>(smem);                  // [n2] excess
  dtype* inflow = e + n2;                                     // [n2]
  dtype* rs = inflow + n2;                                    // [n2 * K] residuals
  comp_type* red = reinterpret_cast<comp_type*>(rs + (size_t)n2 * K);  // [32]
  int* sn = reinterpret_cast<int*>(red + 32);                 // [n2] padded ids, ascending
  int* h = sn + n2;                                           // [n2] heights
  short* nbr = reinterpret_cast<short*>(h + n2);              // [n2 * K] local neighbours or -1
  __shared__ dtype s_off;
  const int T = blockDim.x;

  // 1. the region, its influence sum and the offset (setRegionToLambda).
  // Every node id is checked against the lattice: a bad one sets
  // status[3] and the block stops before touching anything.
  comp_type gsum = 0;
  int bad = 0;
  for (int j = threadIdx.x; j < n; j += T) {
    const int i = nodes[j];
    if (i < 0 || (long long)i >= g.NP || (j > 0 && nodes[j - 1] >= i)) {
      bad = 1;
      sn[j] = 0;
      continue;
    }
    sn[j] = i;
    gsum += comp_type(-exc[i]) + off[i] - cur[i];
  }
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) status[3] = 1;
    return;
  }
  gsum = block_sum_i128(gsum, red);
  if (threadIdx.x == 0) {
    const comp_type qii = (comp_type)(((unsigned __int128)qii_hi << 64) | qii_lo);
    comp_type t = comp_type(mult_fv_scale(qii, lm)) + gsum;
    if (t < 0) t -= (n - 1);  // floorAverage
    s_off = dtype(div_i128(t, n));
  }
  __syncthreads();
  const dtype fv_offset = s_off;
  for (int j = threadIdx.x; j < n; j += T) {
    const int i = sn[j];
    const dtype fv = mult_fv_scale(base[i], lm);
    const dtype o = fv_offset + ((pull && fv > fv_offset) ? 1 : 0);
    const dtype ex = exc[i] - ((fv - o) - (cur[i] - off[i]));
    cur[i] = fv;
    off[i] = o;
    e[j] = ex;
    inflow[j] = 0;
    const int c = i % g.Cp, b = i / g.Cp;
    for (int k = 0; k < K; ++k) {
      const int nb = b + st.db[k], nc = c + st.dc[k];
      int loc = -1;
      if (nb >= 0 && nb < g.B && nc >= 0 && nc < g.C) {
        const int v = nb * g.Cp + nc;
        if (keys[v] == key) loc = local_index(sn, n, v);
      }
      nbr[j * K + k] = short(loc >= 0 && loc < n ? loc : -1);
      rs[j * K + k] = res[(long long)k * g.NP + i];
    }
  }
  __syncthreads();

  // 2. the region's max-flow on the staged residuals
  int epoch = 0, levels = 0;
  for (;; ++epoch) {
    // exact distance to the nearest deficit along residual edges (a node
    // found on a level is set to lvl + 1, which no other test of the same
    // level matches, so a level needs no barrier inside)
    for (int j = threadIdx.x; j < n; j += T) h[j] = e[j] < 0 ? 0 : kHUnreached;
    __syncthreads();
    for (int lvl = 0; lvl < n; ++lvl) {
      int changed = 0;
      for (int j = threadIdx.x; j < n; j += T) {
        if (h[j] != kHUnreached) continue;
        for (int k = 0; k < K; ++k) {
          const int v = nbr[j * K + k];
          if (v >= 0 && h[v] == lvl && rs[j * K + k] > 0) {
            h[j] = lvl + 1;
            changed = 1;
            break;
          }
        }
      }
      ++levels;
      if (!__syncthreads_or(changed)) break;
    }
    int act = 0;
    for (int j = threadIdx.x; j < n; j += T) act |= (e[j] > 0 && h[j] < kHUnreached);
    if (!__syncthreads_or(act)) break;
    if (epoch >= max_epochs) {
      if (threadIdx.x == 0) status[0] = 1;
      break;
    }
    // push / relabel sweeps on these labels until no node below height n
    // holds excess (a label of n or more cannot lead to a deficit), at most
    // 64 per exact relabel.  A push goes from j to a neighbour one level
    // down; that neighbour pushes only further down, so the reverse
    // residual is written by j alone.
    for (int sweep = 0; sweep < 64; ++sweep) {
      for (int j = threadIdx.x; j < n; j += T) {
        dtype rem = e[j];
        const int hj = h[j];
        if (rem <= 0 || hj >= n) continue;
        for (int k = 0; k < K && rem > 0; ++k) {
          const int v = nbr[j * K + k];
          if (v < 0 || h[v] != hj - 1) continue;
          const dtype r = rs[j * K + k];
          if (r <= 0) continue;
          const dtype a = r < rem ? r : rem;
          rs[j * K + k] = r - a;
          rs[v * K + st.rev[k]] += a;
          atomicAdd(reinterpret_cast<unsigned long long*>(&inflow[v]), (unsigned long long)a);
          rem -= a;
        }
        e[j] = rem;
      }
      __syncthreads();
      // take the inflow, then relabel: a node still holding excess with no
      // admissible edge moves one above its lowest residual neighbour
      // (neighbours' labels may be read while they rise: a stale, lower
      // label keeps the labelling valid)
      int busy = 0;
      for (int j = threadIdx.x; j < n; j += T) {
        const dtype ej = e[j] + inflow[j];
        e[j] = ej;
        inflow[j] = 0;
        const int hj = h[j];
        if (ej <= 0 || hj >= n) continue;  // (a filled deficit at 0 rises too)
        int hm = kHUnreached;
        for (int k = 0; k < K; ++k) {
          const int v = nbr[j * K + k];
          if (v >= 0 && rs[j * K + k] > 0) hm = min(hm, h[v]);
        }
        if (hm != hj - 1) h[j] = hm >= n ? n : hm + 1;
        busy |= h[j] < n;
      }
      if (!__syncthreads_or(busy)) break;
    }
  }

  // 3. read-out: labels, per-side sums, cut value; excess and residuals back
  comp_type g0 = 0, g1 = 0, cv = 0;
  int ons = 0;
  for (int j = threadIdx.x; j < n; j += T) {
    const int i = sn[j];
    exc[i] = e[j];
    for (int k = 0; k < K; ++k) res[(long long)k * g.NP + i] = rs[j * K + k];
    const bool on = h[j] >= kHUnreached;
    lab[j] = on ? 1 : 0;
    const comp_type gam = comp_type(-e[j]) + off[i] - cur[i];
    if (on) {
      g1 += gam;
      ++ons;
    } else {
      g0 += gam;
      for (int k = 0; k < K; ++k) {
        const int v = nbr[j * K + k];
        if (v >= 0 && h[v] >= kHUnreached) {
          const dtype a = rs[j * K + k];
          cv += (a < 0 ? -a : a) >> 1;
        }
      }
    }
  }
  g0 = block_sum_i128(g0, red);
  g1 = block_sum_i128(g1, red);
  cv = block_sum_i128(cv, red);
  const comp_type on_total = block_sum_i128(comp_type(ons), red);
  if (threadIdx.x == 0) {
    status[1] += epoch;
    status[2] += levels;
    acc[0] = (unsigned long long)g0;
    acc[1] = (unsigned long long)(g0 >> 64);
    acc[2] = (unsigned long long)g1;
    acc[3] = (unsigned long long)(g1 >> 64);
    acc[4] = (unsigned long long)cv;
    acc[5] = (unsigned long long)(cv >> 64);
    acc[6] = (unsigned long long)on_total;
  }
}

constexpr size_t kRegionProbeSmem = 200 * 1024;

size_t region_probe_smem(int n, int K) {
  const size_t n2 = size_t((n + 1) & ~1);
  return n2 * (8 + 8 + 8 * size_t(K) + 4 + 4 + 2 * size_t(K)) + 32 * sizeof(comp_type) + 16;
}

__global__ void k_seg_setkey(const int* nodes, int n, int key, int* keys) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) keys[nodes[j]] = key;
}

// applyPartioningCut (tv_push_relabel.hpp:239-248): every edge from a node of
// the on part (`nodes`) to a node of the off part (key `key_off`) is
// saturated: its residual moves to the reverse direction, the flow from the
// on node's excess to the off node's.
__global__ void k_seg_saturate(const int* nodes, int n, int key_off, const int* keys, Geo g,
                               Stencil st, dtype* res, dtype* exc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int u = nodes[j];
  const int c = u % g.Cp, b = u / g.Cp;
  dtype sent = 0;
  for (int k = 0; k < st.K; ++k) {
    const int nb = b + st.db[k], nc = c + st.dc[k];
    if (nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) continue;
    const int v = nb * g.Cp + nc;
    if (keys[v] != key_off) continue;
    const dtype a = res[(long long)k * g.NP + u];
    if (a <= 0) continue;
    res[(long long)k * g.NP + u] = 0;
    res[(long long)st.rev[k] * g.NP + v] += a;
    atomicAdd(reinterpret_cast<unsigned long long*>(&exc[v]), (unsigned long long)a);
    sent += a;
  }
  if (sent) exc[u] -= sent;
}

// ------------------------------------------------------------- the tracker

// TV_PRFlow::CutInfo (tv_push_relabel.hpp:44-55): the two parts of a probe
// (padded node ids, region order) and the cut value
struct Cut {
  bool any_cut = false;
  std::vector<int> part[2];
  dtype cut_value = 0;
};
typedef std::shared_ptr<Cut> CutPtr;

class PathGPU {
 public:
  PathGPU(Engine& e, const std::vector<int64_t>& base_rowmajor, const std::vector<long long>& pwf2,
          double fmean, double fscale, double max_lambda);
  ~PathGPU();
  void run();
  int output(const std::vector<double>& lams, double* out);
  // [0] segments, [1] probes, [2] events, [3] initial level sets, [4] probes
  // on the lattice-wide solver, [5] microseconds in them, [6] microseconds in
  // fused probes, [7] microseconds in segment set-ups, [8] [9] epochs and BFS
  // levels of the fused probes
  static constexpr int kStats = 10;
  int64_t stats[kStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};

 private:
  enum Mode { Unset, Initial, Join, Split };
  enum Event { EvJoin, EvSplit, EvSplitUB };

  struct Seg {
    Mode rhs_mode = Unset, lhs_mode = Unset;
    dtype rhs_lambda = 0, lhs_lambda = -1;
    dtype ar1 = 0, ar0 = 0;  // adjusted_r_at_1 / adjusted_r_at_0
    size_t n_nodes = 0;
    std::vector<int> nodeset;  // kept after deactivation (Split / Initial)
    int lhs_nodes[2] = {-1, -1};
    // construction information (tv_regpath_node.hpp:249-277), while active
    int key = 0;
    std::set<int> neighbors;
    std::multimap<dtype, int> join_points;
    std::vector<int> ci_nodes;  // padded ids, ascending
    int* d_nodes = nullptr;     // device copy of ci_nodes
    comp_type qii_sum = 0;      // sum of the nodes' base values
    CutPtr split_info;
  };

  struct DSI {
    bool occurs = false, exact = false;
    dtype lam = 0;
    CutPtr cut;
  };

  struct SplitInfo {
    bool occurs;
    dtype split_lambda, split_ub;
  };

  struct FunPoint {
    dtype lambda;
    Event mode;
    int r1, r2;
    bool operator<(const FunPoint& o) const { return lambda < o.lambda; }
  };

  Engine& E;
  Geo g;
  Stencil st;
  cudaStream_t s;
  int K;
  double fmean, fscale, max_lambda;
  std::vector<dtype> base;       // padded: base value of every node (host mirror)
  std::vector<int> keys;         // padded: key of every node (host mirror)
  std::vector<unsigned char> edge_ok;  // per direction: the kernel's edge has capacity
  dtype *d_base = nullptr, *d_cur = nullptr, *d_off = nullptr;
  int* d_keys = nullptr;
  unsigned char* d_lab = nullptr;
  unsigned long long* d_acc = nullptr;  // [0..5] 128-bit sums, [6] count
  unsigned long long* h_acc = nullptr;  // pinned
  unsigned char* h_lab = nullptr;       // pinned, N bytes
  std::deque<Seg> segs;
  std::vector<int> node_map;  // padded: segment at the largest lambda
  dtype calculated_lambda = -1;

  void ck(cudaError_t e, const char* what) { E.check(e, what); }
  int new_seg();
  void upload_nodes(Seg& sg);
  void free_nodes(Seg& sg);
  comp_type host_qii(const std::vector<int>& nodes) const {
    comp_type q = 0;
    for (int i : nodes) q += base[i];
    return q;
  }
  comp_type read_i128(int slot) const {
    return (comp_type)(((unsigned __int128)h_acc[2 * slot + 1] << 64) | h_acc[2 * slot]);
  }
  void read_acc();
  void sync_information(Seg& sg, dtype lambda);
  dtype r_at_lambda(const Seg& sg, dtype lambda) const;
  comp_type region_gamma(const Seg& sg);
  void set_region_to_lambda(Seg& sg, dtype lambda, bool pull);
  CutPtr probe(Seg& sg);
  // setRegionToLambda + runPartitionedSection: one fused launch for a small
  // region, else the lattice-wide solver
  CutPtr region_probe(Seg& sg, dtype lambda, bool pull);
  CutPtr read_probe(Seg& sg);
  int* d_status = nullptr;
  int small_cap = 0;  // largest region the fused probe takes
  dtype lambda_of_join(int a, int b, dtype cur) const;
  dtype calculate_joins(int a, int b, dtype cur);
  dtype first_join_point(const Seg& sg) const {
    return sg.join_points.empty() ? 0 : sg.join_points.rbegin()->first;
  }
  DSI bisection_check(Seg& sg, dtype lb, dtype ub);
  DSI single_split(Seg& sg, dtype lambda_lb, dtype lambda_ub);
  SplitInfo calculate_split(int si, dtype cur);
  void apply_split(int si, int d0, int d1, dtype lambda);
  void setup_from_join(int ni, int a, int b, dtype lambda);
  void deactivate(int si);
  std::set<int> neighborhood_keys(const std::vector<int>& nodes, int key) const;
  bool edge(int i, int k, int* v) const {
    const int c = i % g.Cp, b = i / g.Cp;
    const int nb = b + st.db[k], nc = c + st.dc[k];
    if (nb < 0 || nb >= g.B || nc < 0 || nc >= g.C || !edge_ok[k]) return false;
    *v = nb * g.Cp + nc;
    return true;
  }
};

PathGPU::PathGPU(Engine& e, const std::vector<int64_t>& base_rowmajor,
                 const std::vector<long long>& pwf2, double fm, double fs, double ml)
    : E(e), g(e.g), st(e.st), s(e.stream), K(e.st.K), fmean(fm), fscale(fs), max_lambda(ml) {
  const long long NP = g.NP;
  base.assign(NP, 0);
  keys.assign(NP, -1);
  for (int b = 0; b < g.B; ++b)
    for (int c = 0; c < g.C; ++c) base[b * g.Cp + c] = base_rowmajor[(size_t)b * g.C + c];
  edge_ok.assign(K, 0);
  for (int k = 0; k < K; ++k) edge_ok[k] = pwf2[k] > 0;
  ck(cudaMalloc(&d_base, NP * sizeof(dtype)), "cudaMalloc");
  ck(cudaMalloc(&d_cur, NP * sizeof(dtype)), "cudaMalloc");
  ck(cudaMalloc(&d_off, NP * sizeof(dtype)), "cudaMalloc");
  ck(cudaMalloc(&d_keys, NP * sizeof(int)), "cudaMalloc");
  ck(cudaMalloc(&d_lab, std::max<long long>(E.N, 1)), "cudaMalloc");
  ck(cudaMalloc(&d_acc, 8 * sizeof(unsigned long long)), "cudaMalloc");  // [7] unused
  ck(cudaMalloc(&d_status, 4 * sizeof(int)), "cudaMalloc");
  ck(cudaMemsetAsync(d_status, 0, 4 * sizeof(int), s), "memset");
  {
    // the fused probe's region bound: what fits the shared memory of a block
    small_cap = kSmallRegion;
    while (small_cap > 32 && region_probe_smem(small_cap, K) > kRegionProbeSmem) small_cap /= 2;
    // one value for every kernel size, so that concurrent paths agree
    ck(cudaFuncSetAttribute(k_region_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            int(kRegionProbeSmem)),
       "cudaFuncSetAttribute");
  }
  // [0..6] probe sums, [8..9] the probe's status words
  ck(cudaMallocHost(&h_acc, 10 * sizeof(unsigned long long)), "cudaMallocHost");
  ck(cudaMallocHost(&h_lab, std::max<long long>(E.N, 1)), "cudaMallocHost");
  ck(cudaMemcpyAsync(d_base, base.data(), NP * sizeof(dtype), cudaMemcpyHostToDevice, s), "memcpy");
  // after the parametric flow: scale 1 (current value = base), offsets 0
  ck(cudaMemcpyAsync(d_cur, base.data(), NP * sizeof(dtype), cudaMemcpyHostToDevice, s), "memcpy");
  ck(cudaMemsetAsync(d_off, 0, NP * sizeof(dtype), s), "memset");
  ck(cudaMemsetAsync(d_keys, 0xff, NP * sizeof(int), s), "memset");
  // no node solves until a probe marks its region
  ck(cudaMemsetAsync(E.d_kmask, 0, NP * sizeof(uint64_t), s), "memset");
  // a region probe moves flow within one region, a small part of the
  // lattice: a short pass cadence between relabels (the parametric flow's
  // 64 passes are for sections that span the lattice)
  E.tune.launches_per_relabel = 8;
  // region probes too large for one block run on the staged 64-bit passes
  // with the section mask (pr_kernel / bfs_kernel 0; measured at 256^2:
  // 17.1 s of large probes against 19.5 s on the generic tile passes),
  // without the tail step
  E.tune.pr_kernel = 0;
  E.tune.bfs_kernel = 0;
  E.tune.tail_active = -1;
  ck(cudaStreamSynchronize(s), "sync");
}

PathGPU::~PathGPU() {
  cudaStreamSynchronize(s);
  for (Seg& sg : segs)
    if (sg.d_nodes) cudaFree(sg.d_nodes);
  cudaFree(d_base);
  cudaFree(d_cur);
  cudaFree(d_off);
  cudaFree(d_keys);
  cudaFree(d_lab);
  cudaFree(d_acc);
  cudaFree(d_status);
  cudaFreeHost(h_acc);
  cudaFreeHost(h_lab);
}

int PathGPU::new_seg() {
  segs.emplace_back();
  segs.back().key = int(segs.size());
  ++stats[0];
  return int(segs.size()) - 1;
}

void PathGPU::upload_nodes(Seg& sg) {
  free_nodes(sg);
  const size_t n = sg.ci_nodes.size();
  // every kernel over a region indexes the lattice with these ids
  for (size_t j = 0; j < n; ++j)
    if (sg.ci_nodes[j] < 0 || sg.ci_nodes[j] >= g.NP || (j > 0 && sg.ci_nodes[j - 1] >= sg.ci_nodes[j]))
      throw LfError{6, "TV path: a region's node list is not a sorted list of lattice nodes"};
  if (n == 0) throw LfError{6, "TV path: empty region"};
  ck(cudaMallocAsync(&sg.d_nodes, std::max<size_t>(n, 1) * sizeof(int), s), "cudaMallocAsync");
  ck(cudaMemcpyAsync(sg.d_nodes, sg.ci_nodes.data(), n * sizeof(int), cudaMemcpyHostToDevice, s),
     "memcpy");
  for (int i : sg.ci_nodes) keys[i] = sg.key;
  sg.qii_sum = host_qii(sg.ci_nodes);
}

void PathGPU::free_nodes(Seg& sg) {
  if (sg.d_nodes) cudaFreeAsync(sg.d_nodes, s);
  sg.d_nodes = nullptr;
}

void PathGPU::read_acc() {
  ck(cudaMemcpyAsync(h_acc, d_acc, 7 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
     "memcpy");
  ck(cudaStreamSynchronize(s), "sync");
}

// TVRegPathSegment::syncInformation (tv_regpath_node.hpp:216-245): the
// line's end points from the segment's sums.  Its gamma is the difference
// of two int64 sums (getRegionInfo, tv_regpath_node.hpp:176-206), i.e. the
// exact sum taken modulo 2^64.
void PathGPU::sync_information(Seg& sg, dtype lambda) {
  const auto t0 = std::chrono::steady_clock::now();
  const int n = int(sg.ci_nodes.size());
  sg.n_nodes = size_t(n);
  ck(cudaMemsetAsync(d_acc, 0, 7 * sizeof(unsigned long long), s), "memset");
  k_seg_sync<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, lambda, sg.key, d_base, d_cur, d_off,
                                          (dtype*)E.d_exc, d_keys, d_acc);
  ck(E.counted(cudaGetLastError()), "segment sync");
  read_acc();
  const comp_type gamma = comp_type(dtype(read_i128(0)));
  const comp_type adj = comp_type(1) << kAdjustBits;
  sg.ar0 = dtype((gamma * adj) / comp_type(n));
  sg.ar1 = dtype(((sg.qii_sum + gamma) * adj) / comp_type(n));
  stats[7] += (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(
                  std::chrono::steady_clock::now() - t0).count();
}

// TVRegPathSegment::get_r_AtLambda (tv_regpath_node.hpp:131-148)
dtype PathGPU::r_at_lambda(const Seg& sg, dtype lambda) const {
  dtype v = sg.ar0 + mult_fv_scale(comp_type(dtype(sg.ar1 - sg.ar0)), lambda);
  v += (v < 0 ? -1 : 1) * (dtype(1) << (kAdjustBits - 1));
  return v / (dtype(1) << kAdjustBits);
}

comp_type PathGPU::region_gamma(const Seg& sg) {
  const int n = int(sg.ci_nodes.size());
  ck(cudaMemsetAsync(d_acc, 0, 7 * sizeof(unsigned long long), s), "memset");
  k_seg_gamma<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, d_cur, d_off, (const dtype*)E.d_exc,
                                           d_acc);
  ck(E.counted(cudaGetLastError()), "segment gamma");
  read_acc();
  return read_i128(0);
}

// TV_PRFlow::setRegionToLambda (tv_push_relabel.hpp:414-468)
void PathGPU::set_region_to_lambda(Seg& sg, dtype lambda, bool pull) {
  const int n = int(sg.ci_nodes.size());
  const comp_type gamma = region_gamma(sg);
  const dtype fv_offset =
      floor_average(comp_type(mult_fv_scale(sg.qii_sum, lambda)) + gamma, long(n));
  k_seg_offset<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, lambda, fv_offset, pull ? 1 : 0,
                                            d_base, d_cur, d_off, (dtype*)E.d_exc);
  ck(E.counted(cudaGetLastError()), "segment offsets");
}

// TV_PRFlow::runPartitionedSection (tv_push_relabel.hpp:84-237): the region's
// max-flow, split by its maximal on-set.
CutPtr PathGPU::probe(Seg& sg) {
  ++stats[1];
  const int n = int(sg.ci_nodes.size());
  k_seg_kmask<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, sg.key, d_keys, g, st, E.d_kmask, 1);
  ck(E.counted(cudaGetLastError()), "segment mask");
  E.maxflow<long long>(false);
  ck(cudaMemsetAsync(d_acc, 0, 7 * sizeof(unsigned long long), s), "memset");
  k_seg_probe<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, sg.key, d_keys, E.d_h,
                                           (const dtype*)E.d_res, (const dtype*)E.d_exc, d_off,
                                           d_cur, g, st, d_lab, d_acc, d_acc + 6);
  ck(E.counted(cudaGetLastError()), "segment probe");
  k_seg_kmask<<<nblk(n, 256), 256, 0, s>>>(sg.d_nodes, n, sg.key, d_keys, g, st, E.d_kmask, 0);
  ck(E.counted(cudaGetLastError()), "segment mask");
  return read_probe(sg);
}

CutPtr PathGPU::read_probe(Seg& sg) {
  const int n = int(sg.ci_nodes.size());
  ck(cudaMemcpyAsync(h_lab, d_lab, (size_t)n, cudaMemcpyDeviceToHost, s), "memcpy");
  read_acc();
  CutPtr cut = std::make_shared<Cut>();
  const long long on = (long long)h_acc[6];
  if (on == 0 || on == n) return cut;
  cut->any_cut = true;
  cut->part[0].reserve(size_t(n - on));
  cut->part[1].reserve(size_t(on));
  for (int j = 0; j < n; ++j) cut->part[h_lab[j] ? 1 : 0].push_back(sg.ci_nodes[j]);
  cut->cut_value = dtype(read_i128(2));
  return cut;
}

CutPtr PathGPU::region_probe(Seg& sg, dtype lambda, bool pull) {
  const int n = int(sg.ci_nodes.size());
  const auto t0 = std::chrono::steady_clock::now();
  auto us = [&]() {
    return (int64_t)std::chrono::duration_cast<std::chrono::microseconds>(
               std::chrono::steady_clock::now() - t0).count();
  };
  if (n > small_cap) {
    set_region_to_lambda(sg, lambda, pull);
    CutPtr c = probe(sg);
    ++stats[4];
    stats[5] += us();
    return c;
  }
  ++stats[1];
  ck(cudaMemsetAsync(d_status, 0, sizeof(int), s), "memset");  // the cap flag; [1], [2] count on
  const int threads = std::min(1024, std::max(32, (n + 31) / 32 * 32));
  k_region_probe<<<1, threads, region_probe_smem(n, K), s>>>(
      sg.d_nodes, n, sg.key, d_keys, g, st, lambda, pull ? 1 : 0,
      (unsigned long long)sg.qii_sum, (unsigned long long)(sg.qii_sum >> 64), d_base, d_cur,
      d_off, (dtype*)E.d_exc, (dtype*)E.d_res, d_lab, d_acc, d_status, 4 * n + 64);
  ck(E.counted(cudaGetLastError()), "region probe");
  int status[4] = {0, 0, 0, 0};
  ck(cudaMemcpyAsync(&h_acc[8], d_status, 4 * sizeof(int), cudaMemcpyDeviceToHost, s), "memcpy");
  CutPtr cut = read_probe(sg);
  std::memcpy(status, &h_acc[8], sizeof(status));
  if (status[3]) throw LfError{6, "TV path: a region probe met an invalid node id"};
  if (status[0]) {  // the epoch cap ended it: finish on the lattice-wide solver
    --stats[1];
    ++stats[4];
    cut = probe(sg);
    stats[5] += us();
    return cut;
  }
  stats[6] += us();
  return cut;
}

// TV_PRFlow::getNeighborhoodKeySet (tv_push_relabel.hpp:367-391).  The
// residuals of an edge sum to its capacity in both directions whatever the
// flow, so an edge counts exactly when the kernel gives it capacity.
std::set<int> PathGPU::neighborhood_keys(const std::vector<int>& nodes, int key) const {
  std::set<int> out;
  for (int i : nodes)
    for (int k = 0; k < K; ++k) {
      int v;
      if (edge(i, k, &v) && keys[v] != key) out.insert(keys[v]);
    }
  return out;
}

// TVRegPathSegment::lambdaOfJoin (tv_regpath_node.hpp:927-966)
dtype PathGPU::lambda_of_join(int a, int b, dtype cur) const {
  const Seg& r1 = segs[a];
  const Seg& r2 = segs[b];
  if (r1.rhs_mode == Split && r2.rhs_mode == Split && r1.rhs_lambda == cur && r2.rhs_lambda == cur)
    return -1;
  const dtype numer = r2.ar0 - r1.ar0;
  const dtype denom = (r1.ar1 - r1.ar0) - (r2.ar1 - r2.ar0);
  const dtype jl = ((numer < 0) != (denom < 0)) ? -1 : scale_from_quotient(numer, denom);
  return (0 < jl && jl <= cur) ? jl : -1;
}

// TVRegPathSegment::calculateJoins (tv_regpath_node.hpp:968-992)
dtype PathGPU::calculate_joins(int a, int b, dtype cur) {
  const dtype jl = lambda_of_join(a, b, cur);
  if (jl != -1) {
    segs[a].join_points.insert({jl, b});
    segs[b].join_points.insert({jl, a});
  }
  return jl;
}

// TVRegPathSegment::BisectionCheck (tv_regpath_node.hpp:416-455)
PathGPU::DSI PathGPU::bisection_check(Seg& sg, dtype lb, dtype ub) {
  int rate = 4;
  CutPtr best;
  bool occurred = false;
  while (lb + 1 < ub) {
    const dtype t = rate != 1 ? (lb + 1) + ((ub - (lb + 1)) / (dtype(1) << rate)) : (ub + lb) / 2;
    CutPtr cut = region_probe(sg, t, true);
    if (!cut->any_cut) {
      ub = t;
    } else {
      lb = t;
      best = cut;
      occurred = true;
      if (rate > 1) --rate;
    }
  }
  DSI d;
  d.occurs = d.exact = occurred;
  d.lam = lb;
  d.cut = occurred ? best : nullptr;
  return d;
}

// TVRegPathSegment::_calculateSingleSplit (tv_regpath_node.hpp:457-633)
PathGPU::DSI PathGPU::single_split(Seg& sg, const dtype lambda_lb, const dtype lambda_ub) {
  CutPtr cut = region_probe(sg, lambda_lb, false);
  DSI d;
  if (!cut->any_cut) return d;
  const dtype s0 = dtype(cut->part[0].size()), s1 = dtype(cut->part[1].size());
  const comp_type c = cut->cut_value;
  if (c == 0) {
    d.occurs = d.exact = true;
    d.cut = cut;
    d.lam = lambda_ub;
    return d;
  }
  // getRegionInfo of both parts: gamma as an int64 difference (see
  // sync_information), from the probe's per-side sums
  const comp_type gam0 = comp_type(dtype(read_i128(0)));
  const comp_type gam1 = comp_type(dtype(read_i128(1)));
  const comp_type g0 = gam0 - c, g1 = gam1 + c;
  const comp_type q0 = host_qii(cut->part[0]), q1 = host_qii(cut->part[1]);
  const dtype sn = s0 + s1;
  const comp_type intercept = iabs((s1 * g0 - s0 * g1) + c * sn);
  const comp_type denom = iabs(q1 * s0 - q0 * s1);
  const dtype denom_pm = sn;
  dtype lb = scale_from_quotient(intercept - comp_type(wmul(std::max(s1, s0), sn)), denom + denom_pm);
  dtype ub = scale_from_quotient(intercept, denom - denom_pm);
  if (ub < lambda_lb) return bisection_check(sg, lambda_lb, lambda_ub);
  d.occurs = true;
  d.cut = cut;
  if (lb > lambda_ub) {
    d.lam = lambda_ub;
    return d;
  }
  lb = std::max(lb, lambda_lb);
  ub = std::min(ub, lambda_ub);
  const comp_type gs = g0 + g1;
  auto value = [&](dtype lm) -> comp_type {
    comp_type lmq0 = 0, lmq1 = 0;
    if (s0 > 32) lmq0 = mult_fv_scale(q0, lm);
    else for (int i : cut->part[0]) lmq0 += mult_fv_scale(base[i], lm);
    if (s1 > 32) lmq1 = mult_fv_scale(q1, lm);
    else for (int i : cut->part[1]) lmq1 += mult_fv_scale(base[i], lm);
    const dtype fl_avg = floor_average(gs + lmq0 + lmq1, long(sn));
    return std::min(lmq1 + g1 - c - comp_type(wmul(s1, fl_avg)),
                    lmq0 + g0 + c - comp_type(wmul(s0, fl_avg)));
  };
  comp_type value_lb = value(lb);
  comp_type value_ub = value(ub);
  if (value_lb >= 0) {
    d.lam = lb;
    return d;
  }
  if (value_ub < 0) {
    d.lam = ub;
    return d;
  }
  while (lb + 1 < ub) {
    if (value_ub == 0) break;
    const dtype mid = (lb + ub) / 2;
    const comp_type v = value(mid);
    if (v < 0) { lb = mid; value_lb = v; } else { ub = mid; value_ub = v; }
  }
  d.lam = ub;
  return d;
}

// TVRegPathSegment::calculateSplit (tv_regpath_node.hpp:647-744)
PathGPU::SplitInfo PathGPU::calculate_split(int si, dtype cur) {
  Seg& sg = segs[si];
  if (sg.n_nodes == 1) return {false, -1, 0};
  dtype lambda_calc_lb = 0;
  for (auto it = sg.join_points.begin(); it != sg.join_points.end();) {
    const dtype join_lm = it->first;
    const int o = it->second;
    if (join_lm >= cur || segs[o].lhs_mode != Unset) {
      it = sg.join_points.erase(it);
      continue;
    }
    // (an empty map's last key reads as 0 in the reference build)
    if (join_lm == first_join_point(segs[o])) lambda_calc_lb = std::max(join_lm, lambda_calc_lb);
    ++it;
  }
  DSI dsi, last;
  dtype lambda_calc = lambda_calc_lb;
  bool cut_exists = false;
  while (true) {
    dsi = single_split(sg, lambda_calc, cur);
    if (!dsi.occurs) break;
    cut_exists = true;
    last = dsi;
    if (dsi.exact) {
      lambda_calc = dsi.lam;
      break;
    }
    lambda_calc = dsi.lam + (dtype(1) << std::max(0, kScaleBits - 24));
    if (lambda_calc >= cur) {
      lambda_calc = cur;
      break;
    }
  }
  if (cut_exists) {
    sg.split_info = last.cut;
    return {true, lambda_calc, lambda_calc_lb};
  }
  return {false, -1, lambda_calc_lb};
}

// TVRegPathSegment::applySplit (tv_regpath_node.hpp:747-814)
void PathGPU::apply_split(int si, int d0, int d1, dtype lambda) {
  CutPtr cut = segs[si].split_info;
  const int dest[2] = {d0, d1};
  for (int i = 0; i < 2; ++i) {
    Seg& d = segs[dest[i]];
    d.ci_nodes = std::move(cut->part[i]);
    d.rhs_lambda = lambda;
    d.rhs_mode = Split;
    upload_nodes(d);
    const int n = int(d.ci_nodes.size());
    k_seg_setkey<<<nblk(n, 256), 256, 0, s>>>(d.d_nodes, n, d.key, d_keys);
    ck(E.counted(cudaGetLastError()), "segment keys");
  }
  // the cut's edges, on part -> off part, saturated before the new sums
  {
    const Seg& on = segs[d1];
    const int n = int(on.ci_nodes.size());
    k_seg_saturate<<<nblk(n, 256), 256, 0, s>>>(on.d_nodes, n, segs[d0].key, d_keys, g, st,
                                                 (dtype*)E.d_res, (dtype*)E.d_exc);
    ck(E.counted(cudaGetLastError()), "cut saturation");
  }
  for (int i = 0; i < 2; ++i) sync_information(segs[dest[i]], lambda);
  for (int i = 0; i < 2; ++i) {
    const std::set<int> ks = neighborhood_keys(segs[dest[i]].ci_nodes, segs[dest[i]].key);
    for (int k : ks) {
      const int o = k - 1;
      segs[o].neighbors.insert(dest[i]);
      segs[dest[i]].neighbors.insert(o);
    }
  }
  for (int o : segs[si].neighbors) segs[o].neighbors.erase(si);
  Seg& sg = segs[si];
  sg.lhs_lambda = lambda;
  sg.lhs_mode = Split;
  sg.lhs_nodes[0] = d0;
  sg.lhs_nodes[1] = d1;
  if (segs[d0].ci_nodes.size() > segs[d1].ci_nodes.size()) std::swap(sg.lhs_nodes[0], sg.lhs_nodes[1]);
}

// TVRegPathSegment::setupFromJoin (tv_regpath_node.hpp:820-921)
void PathGPU::setup_from_join(int ni, int a, int b, dtype lambda) {
  Seg& n = segs[ni];
  Seg& r1 = segs[a];
  Seg& r2 = segs[b];
  n.ci_nodes.resize(r1.ci_nodes.size() + r2.ci_nodes.size());
  std::merge(r1.ci_nodes.begin(), r1.ci_nodes.end(), r2.ci_nodes.begin(), r2.ci_nodes.end(),
             n.ci_nodes.begin());
  n.rhs_mode = Join;
  n.rhs_lambda = lambda;
  const bool big1 = r1.neighbors.size() > r2.neighbors.size();
  std::set<int>& nb_big = big1 ? r1.neighbors : r2.neighbors;
  std::set<int>& nb_small = big1 ? r2.neighbors : r1.neighbors;
  n.neighbors = std::move(nb_big);
  nb_big.clear();
  n.neighbors.insert(nb_small.begin(), nb_small.end());
  n.neighbors.erase(a);
  n.neighbors.erase(b);
  for (int o : n.neighbors) {
    segs[o].neighbors.insert(ni);
    segs[o].neighbors.erase(a);
    segs[o].neighbors.erase(b);
  }
  r1.lhs_mode = Join;
  r1.lhs_lambda = lambda;
  r1.lhs_nodes[0] = ni;
  r2.lhs_mode = Join;
  r2.lhs_lambda = lambda;
  r2.lhs_nodes[0] = ni;
  upload_nodes(n);
  sync_information(n, lambda);
}

// TVRegPathSegment::deactivate (tv_regpath_node.hpp:300-373)
void PathGPU::deactivate(int si) {
  Seg& sg = segs[si];
  if (sg.rhs_mode == Split || sg.rhs_mode == Initial) {
    sg.nodeset.swap(sg.ci_nodes);
    std::sort(sg.nodeset.begin(), sg.nodeset.end());
  }
  free_nodes(sg);
  std::set<int>().swap(sg.neighbors);
  std::multimap<dtype, int>().swap(sg.join_points);
  std::vector<int>().swap(sg.ci_nodes);
  sg.split_info.reset();
}

// TVSolver::run + _constructInitialRegPathsFromSolvedLattice (tv_solver.hpp:114-136,300-564)
void PathGPU::run() {
  const dtype solved_lambda = to_scale(1);
  // level sets of the parametric flow, in the reference's order
  int n_sets = 0;
  for (int v : E.level_sets_host) n_sets = std::max(n_sets, v + 1);
  std::vector<std::vector<int>> level_sets(n_sets);
  for (int b = 0; b < g.B; ++b)
    for (int c = 0; c < g.C; ++c) {
      const int v = E.level_sets_host[(size_t)b * g.C + c];
      if (v < 0) throw LfError{6, "parametric flow left a node without a level set"};
      level_sets[v].push_back(b * g.Cp + c);
    }
  stats[3] = n_sets;
  node_map.assign(g.NP, -1);
  std::vector<int> initial;
  for (auto& nv : level_sets) {
    const int si = new_seg();
    Seg& sg = segs[si];
    sg.ci_nodes = std::move(nv);
    sg.rhs_lambda = solved_lambda;
    sg.rhs_mode = Initial;
    upload_nodes(sg);
    sync_information(sg, solved_lambda);
    initial.push_back(si);
    for (int i : sg.ci_nodes) node_map[i] = si;
  }
  // TV_PRFlow::constructNeighborhoodKeyPairs (tv_push_relabel.hpp:339-365)
  {
    std::unordered_set<uint64_t> seen;
    auto gen_key = [](int k1, int k2) {
      return (uint64_t(std::min(k1, k2)) << 32) | uint64_t(std::max(k1, k2));
    };
    for (int b = 0; b < g.B; ++b)
      for (int c = 0; c < g.C; ++c) {
        const int i = b * g.Cp + c;
        seen.insert(gen_key(keys[i], keys[i]));
        for (int k = 0; k < K / 2; ++k) {
          int v;
          if (edge(i, k, &v) && seen.insert(gen_key(keys[i], keys[v])).second) {
            const int a = node_map[i], bb = node_map[v];
            segs[a].neighbors.insert(bb);
            segs[bb].neighbors.insert(a);
          }
        }
      }
  }
  std::priority_queue<FunPoint> heap;
  auto register_join = [&](int a, int b, dtype lambda_start) {
    const dtype jl = calculate_joins(a, b, lambda_start);
    if (jl > 0) heap.push(FunPoint{jl, EvJoin, a, b});
  };
  auto register_split = [&](int a, dtype lambda_start) {
    const SplitInfo sp = calculate_split(a, lambda_start);
    if (sp.occurs) heap.push(FunPoint{sp.split_lambda, EvSplit, a, -1});
    else if (sp.split_ub != 0) heap.push(FunPoint{sp.split_ub, EvSplitUB, a, -1});
  };
  for (int a : initial) {
    const std::set<int> nb = segs[a].neighbors;
    for (int b : nb)
      if (a < b) register_join(a, b, solved_lambda);
  }
  for (int a : initial) register_split(a, solved_lambda);
  auto activate = [&](int a, dtype lambda_start) {
    const std::set<int> nb = segs[a].neighbors;
    for (int b : nb) register_join(a, b, lambda_start);
    register_split(a, lambda_start);
  };
  const auto t0 = std::chrono::steady_clock::now();
  while (!heap.empty()) {
    const FunPoint fp = heap.top();
    heap.pop();
    const dtype cur = fp.lambda;
    if (segs[fp.r1].lhs_mode != Unset || (fp.r2 >= 0 && segs[fp.r2].lhs_mode != Unset)) continue;
    ++stats[2];
    if ((stats[2] & 1023) == 0 &&
        std::chrono::steady_clock::now() - t0 > std::chrono::seconds(3600))
      throw LfError{4, "TV path exceeded its time limit"};
    switch (fp.mode) {
      case EvJoin: {
        const int ni = new_seg();
        setup_from_join(ni, fp.r1, fp.r2, cur);
        deactivate(fp.r1);
        deactivate(fp.r2);
        activate(ni, cur);
        break;
      }
      case EvSplit: {
        const int d0 = new_seg();
        const int d1 = new_seg();
        apply_split(fp.r1, d0, d1, cur);
        deactivate(fp.r1);
        activate(d0, cur);
        activate(d1, cur);
        break;
      }
      case EvSplitUB:
        register_split(fp.r1, cur);
        break;
    }
  }
  {
    int cnt[4] = {0, 0, 0, 0};
    ck(cudaMemcpyAsync(cnt, d_status, sizeof(cnt), cudaMemcpyDeviceToHost, s), "memcpy");
    ck(cudaStreamSynchronize(s), "sync");
    stats[8] = cnt[1];
    stats[9] = cnt[2];
  }
  Seg& last = segs.back();
  last.lhs_lambda = 0;
  last.lhs_mode = Initial;
  deactivate(int(segs.size()) - 1);
  for (Seg& sg : segs) free_nodes(sg);
  ck(cudaStreamSynchronize(s), "sync");
  calculated_lambda = solved_lambda;
}

// TVSolver::getRegularizationPath + traceRegularizationPath
// (tv_solver.hpp:174-244, 566-642); out[n_lambda][nx][ny]
int PathGPU::output(const std::vector<double>& lams, double* out) {
  const size_t nl = lams.size();
  struct LambdaIdx {
    dtype value;
    size_t index;
    bool operator<(const LambdaIdx& o) const { return value > o.value; }
  };
  std::vector<LambdaIdx> li(nl);
  std::vector<dtype> calc(nl);
  for (size_t i = 0; i < nl; ++i) li[i] = {to_scale(lams[i] / max_lambda), i};
  std::sort(li.begin(), li.end());
  for (size_t i = 0; i < nl; ++i) calc[i] = li[i].value;
  if (calculated_lambda == -1 || calc.front() > calculated_lambda || calc.back() < 0)
    throw LfError{3, "Given lambda values not in calculated range."};
  const size_t N = (size_t)g.B * g.C;
  std::vector<double> sums(nl, 0);
  std::vector<dtype> rv(nl);
  const double fs = double(int64_t(1) << 40);
  for (int b = 0; b < g.B; ++b)
    for (int c = 0; c < g.C; ++c) {
      const int n = b * g.Cp + c;
      int cur = node_map[n];
      size_t idx = 0;
      while (idx < nl) {
        while (segs[cur].lhs_lambda > calc[idx]) {
          const Seg& sg = segs[cur];
          int nxt;
          if (sg.lhs_mode == Split) {
            const int a = sg.lhs_nodes[0], bb = sg.lhs_nodes[1];
            const auto& ns = segs[a].nodeset;
            nxt = std::binary_search(ns.begin(), ns.end(), n) ? a : bb;
          } else {
            nxt = sg.lhs_nodes[0];
          }
          if (nxt < 0) throw LfError{6, "TV path: a segment has no successor"};
          cur = nxt;
        }
        while (idx < nl && segs[cur].lhs_lambda <= calc[idx]) {
          rv[idx] = r_at_lambda(segs[cur], calc[idx]);
          ++idx;
        }
      }
      const size_t pix = (size_t)b * g.C + c;
      for (size_t i = 0; i < nl; ++i) {
        // TVSolver::toFValue (tv_solver.hpp:281-285)
        const double v = (double(rv[i]) / fs - 0.5) * fscale + fmean;
        out[li[i].index * N + pix] = v;
        sums[li[i].index] += v;
      }
    }
  for (size_t i = 0; i < nl; ++i) {
    const double mean = sums[i] / double(N);
    for (size_t p = 0; p < N; ++p) {
      double& v = out[i * N + p];
      v = (v - mean) * fscale + fmean;
    }
  }
  return 0;
}

}  // namespace

int tv_2d_path(const KernelDef* kd, size_t nx, size_t ny, const double* f, size_t n_lambda,
               const double* lambdas, double* out, int64_t* stats) {
  if (n_lambda == 0 || nx * ny == 0) return 0;
  if (nx * ny > size_t(INT_MAX / 2)) throw LfError{2, "lattice too large for the TV path"};
  std::vector<double> lams(lambdas, lambdas + n_lambda);
  for (double& l : lams)
    if (!(l >= 0)) l = 0;  // tv_solver.hpp:669-674
  const double lam_max = *std::max_element(lams.begin(), lams.end());
  const double max_lambda = std::max(lam_max, 1e-8);
  size_t dims[2] = {nx, ny};
  Engine E("GPULevelReductions", kd, 2, dims);
  double fmean = 0, fscale = 0;
  std::vector<int64_t> base;
  std::vector<long long> pwf2;
  tv_fill_single(E, f, max_lambda, &fmean, &fscale, &base, &pwf2);
  engine_run_parametric(E);
  if ((long long)E.g.NP > (long long)INT_MAX) throw LfError{2, "lattice too large for the TV path"};
  PathGPU P(E, base, pwf2, fmean, fscale, max_lambda);
  P.run();
  const int rc = P.output(lams, out);
  if (stats)
    for (int i = 0; i < PathGPU::kStats; ++i) stats[i] = P.stats[i];
  return rc;
}

}  // namespace lfg
