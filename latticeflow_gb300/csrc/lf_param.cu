// Parametric flow (LatticeLevelReductions) and single-lambda TV on the GPU.
//
// Reference: ParametricFlowSolver::run (parametricflow/pf_solver.hpp:33-208)
// processes a FIFO of node ranges; for each range it
//   1. computes r_sum (128-bit), r_min, r_max of r = reduction + offset and
//      stops when r_max - r_min <= 1, else moves the range's offset to
//      r_new = ceil(double(r_sum) / count), minus one if that equals r_max
//      (pf_flow_node.hpp:330-396);
//   2. solves a key-restricted max-flow on the range (push_relabel.hpp:1360-1463);
//   3. splits the range by the partition of every node and requeues both parts.
// Ranges never exchange flow (edges between different keys are inert), so
// every range of one queue generation is independent.  Here a whole
// generation is one step: the statistics are reduced per section on the
// device, the offsets are decided on the host with the reference's exact
// integer / double rule, all sections are solved by ONE lattice-wide max-flow
// with the cross-section edges masked out (kmask), and each section is split
// by its maximal on-set (nodes that cannot reach a deficit node).
//
// Values use the reference's 2x-scaled representation (network_flow_node.hpp:
// 420-485): exc = -(reduction) = -(r - offset).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <climits>
#include <cstring>
#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "lf_engine.h"
#include "lf_tile_common.cuh"

namespace lfg {

namespace {

inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

__device__ __forceinline__ void bounded_coords(const Geo& g, int nd, long long b, int& a, int& bb,
                                               int& c) {
  if (nd == 2) { a = 0; bb = int(b / g.C); c = int(b % g.C); }
  else { c = int(b % g.C); bb = int((b / g.C) % g.B); a = int(b / ((long long)g.C * g.B)); }
}

// NodeFiller::addE1 / addE2 in 2x mode: reduction += 2(E1 - E0);
// pairwise q1 = E10 - E00, q2 = E01 - E00, q12 = E00 + E11 - E01 - E10:
// reduction1 += 2 q1 + q12, reduction2 += 2 q2 + q12, alpha both ways += -q12.
__global__ void k_fill_energy_pf(Geo g, Stencil st, int nd, long long N, const int64_t* unary,
                                 const int64_t* binary, long long* exc, long long* cap, int* err) {
  const int Kp = st.K / 2;
  long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= N * Kp) return;
  long long b = tid / Kp;
  int e = int(tid % Kp);
  int a, bb, c;
  bounded_coords(g, nd, b, a, bb, c);
  long long u = ((long long)a * g.Bp + bb) * g.Cp + c;
  if (e == 0) atom_add(&exc[u], -2LL * (unary[2 * b + 1] - unary[2 * b]));
  int na = a + st.da[e], nb = bb + st.db[e], nc = c + st.dc[e];
  if (na < 0 || na >= g.A || nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) return;
  long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
  const int64_t* q = binary + (b * Kp + e) * 4;
  long long q1 = q[2] - q[0], q2 = q[1] - q[0], q12 = q[0] + q[3] - q[1] - q[2];
  if (q12 > 0) atomicExch(err, 1);
  atom_add(&exc[u], -(2 * q1 + q12));
  atom_add(&exc[v], -(2 * q2 + q12));
  if (q12) {
    atom_add(&cap[(long long)e * g.NP + u], -q12);
    atom_add(&cap[(long long)st.rev[e] * g.NP + v], -q12);
  }
}

// TV setup (tv/tv_solver.hpp:71-112): node value uf (fixed point) enters as
// reduction 2 uf; every in-lattice edge of direction k gets 2 pwf[k].
// Several problems of one shape may be stacked along the rows: problem p holds
// `nx` real rows starting at row p*rows, its values at uf + p*uf_stride
// (uf_stride 0: one image shared by all problems) and its edge weights at
// pwf2 + p*K; edges leaving a problem get no capacity.  N = problems*nx*C.
__global__ void k_fill_tv(Geo g, Stencil st, long long N, int nx, int rows, long long uf_stride,
                          const int64_t* uf, const long long* pwf2, long long* exc,
                          long long* cap) {
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= N) return;
  const long long per = (long long)nx * g.C;
  const int p = int(b / per);
  const long long q = b - p * per;
  const int lo = p * rows, hi = lo + nx;
  const int bb = lo + int(q / g.C), c = int(q % g.C);
  long long u = (long long)bb * g.Cp + c;
  exc[u] = -2LL * uf[p * uf_stride + q];
  for (int k = 0; k < st.K; ++k) {
    int nb = bb + st.db[k], nc = c + st.dc[k];
    bool in = st.da[k] == 0 && nb >= lo && nb < hi && nc >= 0 && nc < g.C;
    cap[(long long)k * g.NP + u] = in ? pwf2[(long long)p * st.K + k] : 0;
  }
}

// Section of every in-lattice node = its problem's index (problems every
// `rows` rows along the second axis, the first `real` of them in the
// lattice), padding = -1.
__global__ void k_pf_init_keys(Geo g, int rows, int real, int* key) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.NP) return;
  int c = int(i % g.Cp), b = int((i / g.Cp) % g.Bp), a = int(i / ((long long)g.Cp * g.Bp));
  key[i] = (a < g.A && b < g.B && c < g.C && b % rows < real) ? b / rows : -1;
}

// Per-section r statistics: 128-bit sum (lo, hi), count, min, max.
// Lanes holding the same section are combined in the warp first.
__global__ void k_pf_stats(long long NP, const int* key, const long long* exc,
                           const long long* off, unsigned long long* lo, unsigned long long* hi,
                           unsigned long long* cnt, long long* rmin, long long* rmax) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int s = -1;
  long long r = 0;
  if (i < NP) {
    s = key[i];
    if (s >= 0) r = off[s] - exc[i];
  }
  unsigned peers = __match_any_sync(0xffffffffu, s);
  int leader = __ffs(peers) - 1;
  int lane = threadIdx.x & 31;
  long long sum = 0, mn = r, mx = r;
  unsigned n = 0;
  for (unsigned m = peers; m; m &= m - 1) {
    int l = __ffs(m) - 1;
    long long v = __shfl_sync(peers, r, l);
    sum += v;
    mn = v < mn ? v : mn;
    mx = v > mx ? v : mx;
    ++n;
  }
  if (s >= 0 && lane == leader) {
    unsigned long long x = (unsigned long long)sum;
    unsigned long long old = atomicAdd(&lo[s], x);
    unsigned long long carry = (old + x) < old ? 1ull : 0ull;
    unsigned long long hadd = (sum < 0 ? ~0ull : 0ull) + carry;
    if (hadd) atomicAdd(&hi[s], hadd);
    atomicAdd(&cnt[s], (unsigned long long)n);
    atomicMin(&rmin[s], mn);
    atomicMax(&rmax[s], mx);
  }
}

// Sections marked finished fold their offset into the node (offset 0, as the
// reference's final setOffset(0)) and leave the computation (key -2),
// recording the level set they end in (leaf[s]); the others move their
// offset: exc += off_new - off_old.
__global__ void k_pf_apply(long long NP, int* key, long long* exc, const long long* off_old,
                           const long long* off_new, const unsigned char* finished,
                           const int* leaf, int* lset) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int s = key[i];
  if (s < 0) return;
  if (finished[s]) {
    exc[i] -= off_old[s];
    key[i] = -2;
    lset[i] = leaf[s];
  } else {
    exc[i] += off_new[s] - off_old[s];
  }
}

// bit k: neighbour k shares the node's (solving) section; bit 63: node solves.
__global__ void k_pf_kmask(Geo g, Stencil st, const int* key, uint64_t* kmask) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.NP) return;
  int s = key[i];
  uint64_t m = 0;
  if (s >= 0) {
    m = 1ull << 63;
    int c = int(i % g.Cp), b = int((i / g.Cp) % g.Bp), a = int(i / ((long long)g.Cp * g.Bp));
    for (int k = 0; k < st.K; ++k) {
      int na = a + st.da[k], nb = b + st.db[k], nc = c + st.dc[k];
      if (na < 0 || na >= g.Ap || nb < 0 || nb >= g.Bp || nc < 0 || nc >= g.Cp) continue;
      if (key[((long long)na * g.Bp + nb) * g.Cp + nc] == s) m |= 1ull << k;
    }
  }
  kmask[i] = m;
}

// side = 1 for the maximal on-set (cannot reach a deficit), else 0.
__global__ void k_pf_count(long long NP, const int* key, const int* h, unsigned long long* cnt2) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int s = key[i];
  if (s < 0) return;
  int side = h[i] >= kHInf ? 1 : 0;
  atomicAdd(&cnt2[2 * s + side], 1ull);
}

__global__ void k_pf_remap(long long NP, int* key, const int* h, const int* child) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  int s = key[i];
  if (s < 0) return;
  int side = h[i] >= kHInf ? 1 : 0;
  key[i] = child[2 * s + side];
}

__global__ void k_pf_levels(Geo g, int nd, long long N, const long long* exc, const int* lset,
                            int64_t* r, int* ls) {
  long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= N) return;
  int a, bb, c;
  bounded_coords(g, nd, b, a, bb, c);
  const long long i = ((long long)a * g.Bp + bb) * g.Cp + c;
  r[b] = -exc[i];
  ls[b] = lset[i];
}

}  // namespace

cudaError_t launch_fill_energy_pf(const Geo& g, const Stencil& st, int nd, long long N,
                                  const int64_t* u, const int64_t* b, long long* exc,
                                  long long* cap, int* err, cudaStream_t s) {
  long long n = N * (st.K / 2);
  if (n > 0) k_fill_energy_pf<<<nblk(n, 256), 256, 0, s>>>(g, st, nd, N, u, b, exc, cap, err);
  return cudaGetLastError();
}

// The parametric driver over an engine whose accumulators hold the 2x-scaled
// reductions (exc64 = -reduction) and alphas (cap64).  An engine holding
// stacked lattices (sub_count > 1) starts with one section per lattice.
void engine_run_parametric(Engine& E) {
  // Section solves move small excess over long distances through
  // high-capacity regions: more local sweeps per tile visit and more passes
  // between global relabels than the binary cut (measured on 256^2-1024^2 TV
  // problems: 6.7x fewer milliseconds at 1024^2 than the binary-cut setting).
  if (E.tune.sweeps <= 0) E.tune.sweeps = 16;
  if (E.tune.launches_per_relabel <= 0) E.tune.launches_per_relabel = 64;
  // 16-row tiles: with the TMA-staged 64-bit pass, 1024^2 TV solves ran
  // 10-20% faster than with 32-row tiles (lambda 1e-3 and 0.05)
  if (E.tune.tile_rows <= 0) E.tune.tile_rows = 16;
  // Tail step only when a single node is still active, with trees as large
  // as a section: after a generation's flow the remainder can sit in one
  // node beside a million nodes short of one unit each, which the tile
  // passes fill a few hundred per relabel.  With more roots the trees of a
  // section solve cost more than the passes they save.  Measured at 1024^2:
  // lambda = 1e-3 2.7 s -> 0.55 s, 0.05 1.58 -> 1.34 s, 1: 0.9 s either way;
  // 64 lambdas 25.9 -> 20.8 s (4 roots: 22.9 s, 64 roots: 169 s).
  if (E.tune.tail_active == 0) E.tune.tail_active = 1;
  if (E.tune.tail_tree_nodes == 0) E.tune.tail_tree_nodes = 1 << 22;
  E.alloc_accumulators();
  E.stats = SolveStats();
  E.prepare_working(8);
  const Geo& g = E.g;
  cudaStream_t s = E.stream;
  long long* exc = (long long*)E.d_exc;
  const long long NP = g.NP;
  const int problems = std::max(E.sub_count, 1);
  const int rows = problems > 1 ? E.sub_rows : std::max(E.g.B, 1);
  const int real = problems > 1 ? E.sub_real_rows : rows;
  const long long cap_sections = std::max<long long>(E.N, 1) + problems;

  DevBuf<int> key;
  DevBuf<long long> off_old, off_new, rmin, rmax;
  DevBuf<unsigned long long> lo, hi, cnt, cnt2;
  DevBuf<unsigned char> fin;
  DevBuf<int> child, leaf, lset;
  key.alloc(NP, s);
  off_old.alloc(cap_sections, s);
  off_new.alloc(cap_sections, s);
  rmin.alloc(cap_sections, s);
  rmax.alloc(cap_sections, s);
  lo.alloc(cap_sections, s);
  hi.alloc(cap_sections, s);
  cnt.alloc(cap_sections, s);
  cnt2.alloc(2 * cap_sections, s);
  fin.alloc(cap_sections, s);
  child.alloc(2 * cap_sections, s);
  leaf.alloc(cap_sections, s);
  lset.alloc(NP, s);
  if (!E.d_kmask) E.check(cudaMalloc(&E.d_kmask, NP * sizeof(uint64_t)), "cudaMalloc kmask");
  // (the section mask stays allocated with the engine for its next solve)

  E.check(cudaEventRecord(E.ev0, s), "event");
  k_pf_init_keys<<<nblk(NP, 256), 256, 0, s>>>(g, rows, real, key.p);
  E.check(E.counted(cudaGetLastError()), "init keys");
  E.check(cudaMemsetAsync(off_old.p, 0, problems * sizeof(long long), s), "memset");

  long long S = E.N > 0 ? problems : 0;  // sections of the current generation, ids 0..S-1
  std::vector<unsigned long long> h_lo, h_hi, h_cnt, h_cnt2;
  std::vector<long long> h_min, h_max, h_off, h_new;
  std::vector<unsigned char> h_fin;
  std::vector<int> h_child, h_leaf;
  // Level sets in the reference's order: the reference partitions one node
  // list in place, the lower (off) part of a range before its upper (on)
  // part, and returns the final ranges by position (pf_solver.hpp:101-203).
  // pos[s] = first position of section s in that list; a finished section
  // is a level set (leaf), ordered by its position.
  std::vector<long long> pos(S, 0), leaf_pos;
  for (long long p = 0; p < S; ++p) pos[p] = p * (long long)real * std::max(E.g.C, 1);
  const long long max_rounds = 20000;
  const bool trace = std::getenv("LF_PF_TRACE") != nullptr;  // diagnostic: one line per generation
  for (long long round = 0; S > 0; ++round) {
    const auto tr0 = std::chrono::steady_clock::now();
    const SolveStats st0 = E.stats;
    if (round > max_rounds) throw LfError{4, "parametric flow did not converge"};
    // 1. statistics of every section
    E.check(cudaMemsetAsync(lo.p, 0, S * 8, s), "memset");
    E.check(cudaMemsetAsync(hi.p, 0, S * 8, s), "memset");
    E.check(cudaMemsetAsync(cnt.p, 0, S * 8, s), "memset");
    E.check(cudaMemsetAsync(rmin.p, 0x7f, S * 8, s), "memset");
    E.check(cudaMemsetAsync(rmax.p, 0x80, S * 8, s), "memset");
    k_pf_stats<<<nblk(NP, 256), 256, 0, s>>>(NP, key.p, exc, off_old.p, lo.p, hi.p, cnt.p,
                                             rmin.p, rmax.p);
    E.check(E.counted(cudaGetLastError()), "pf stats");
    h_lo.resize(S); h_hi.resize(S); h_cnt.resize(S); h_min.resize(S); h_max.resize(S);
    h_off.resize(S); h_new.resize(S); h_fin.assign(S, 0);
    E.check(cudaMemcpyAsync(h_lo.data(), lo.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(h_hi.data(), hi.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(h_cnt.data(), cnt.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(h_min.data(), rmin.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(h_max.data(), rmax.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(h_off.data(), off_old.p, S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaStreamSynchronize(s), "sync");
    // 2. the reference's offset rule, exactly (pf_flow_node.hpp:364-374)
    long long solving = 0;
    h_leaf.assign(S, -1);
    for (long long i = 0; i < S; ++i) {
      if (h_max[i] - h_min[i] <= 1) {
        h_fin[i] = 1;
        h_new[i] = h_off[i];
        h_leaf[i] = int(leaf_pos.size());
        leaf_pos.push_back(pos[i]);
        continue;
      }
      __int128 sum = (__int128)(((unsigned __int128)h_hi[i] << 64) | h_lo[i]);
      double count = double(h_cnt[i]);
      long long r_new = (long long)std::ceil(double(sum) / count);
      if (r_new == h_max[i]) --r_new;
      // The double quotient rounds to r_min when the mean exceeds r_min by
      // less than its resolution (sections of more than ~2^12 nodes at
      // 41-bit values); no node then holds excess, nothing moves, and the
      // reference requeues the same range for ever.  The exact ceiling is
      // then r_min + 1 (the mean is above r_min whenever r_max > r_min).
      if (r_new <= h_min[i]) r_new = h_min[i] + 1;
      h_new[i] = r_new;
      ++solving;
    }
    E.check(cudaMemcpyAsync(off_new.p, h_new.data(), S * 8, cudaMemcpyHostToDevice, s), "memcpy");
    E.check(cudaMemcpyAsync(fin.p, h_fin.data(), S, cudaMemcpyHostToDevice, s), "memcpy");
    E.check(cudaMemcpyAsync(leaf.p, h_leaf.data(), S * sizeof(int), cudaMemcpyHostToDevice, s),
            "memcpy");
    k_pf_apply<<<nblk(NP, 256), 256, 0, s>>>(NP, key.p, exc, off_old.p, off_new.p, fin.p, leaf.p,
                                             lset.p);
    E.check(E.counted(cudaGetLastError()), "pf apply");
    if (solving == 0) { E.check(cudaStreamSynchronize(s), "sync"); break; }
    // 3. one max-flow for every solving section
    k_pf_kmask<<<nblk(NP, 256), 256, 0, s>>>(g, E.st, key.p, E.d_kmask);
    E.check(E.counted(cudaGetLastError()), "pf kmask");
    E.maxflow<long long>(false);
    // 4. split each section by its maximal on-set
    E.check(cudaMemsetAsync(cnt2.p, 0, 2 * S * 8, s), "memset");
    k_pf_count<<<nblk(NP, 256), 256, 0, s>>>(NP, key.p, E.d_h, cnt2.p);
    E.check(E.counted(cudaGetLastError()), "pf count");
    h_cnt2.resize(2 * S);
    E.check(cudaMemcpyAsync(h_cnt2.data(), cnt2.p, 2 * S * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaStreamSynchronize(s), "sync");
    h_child.assign(2 * S, -1);
    std::vector<long long> next_off, next_pos;
    long long S2 = 0;
    for (long long i = 0; i < S; ++i) {
      if (h_fin[i]) continue;
      for (int side = 0; side < 2; ++side)
        if (h_cnt2[2 * i + side] > 0) {
          h_child[2 * i + side] = int(S2++);
          next_off.push_back(h_new[i]);
          next_pos.push_back(pos[i] + (side ? (long long)h_cnt2[2 * i] : 0));
        }
    }
    pos.swap(next_pos);
    if (S2 > cap_sections) throw LfError{4, "section count overflow"};
    E.check(cudaMemcpyAsync(child.p, h_child.data(), 2 * S * sizeof(int), cudaMemcpyHostToDevice, s), "memcpy");
    k_pf_remap<<<nblk(NP, 256), 256, 0, s>>>(NP, key.p, E.d_h, child.p);
    E.check(E.counted(cudaGetLastError()), "pf remap");
    if (S2 > 0)
      E.check(cudaMemcpyAsync(off_old.p, next_off.data(), S2 * 8, cudaMemcpyHostToDevice, s), "memcpy");
    E.check(cudaStreamSynchronize(s), "sync");
    if (trace) {
      double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tr0).count();
      std::fprintf(stderr, "pf gen %lld sections %lld solving %lld next %lld epochs %lld bfs %lld pr %lld tiles %llu ms %.2f\n",
                   round, S, solving, S2, E.stats.epochs - st0.epochs, E.stats.bfs_passes - st0.bfs_passes,
                   E.stats.pr_launches - st0.pr_launches, E.stats.tiles_processed - st0.tiles_processed, ms);
    }
    S = S2;
  }
  E.check(cudaEventRecord(E.ev1, s), "event");
  E.levels_host.assign((size_t)E.N, 0);
  E.level_sets_host.assign((size_t)E.N, 0);
  if (E.N > 0) {
    DevBuf<int64_t> r;
    DevBuf<int> ls;
    r.alloc(E.N, s);
    ls.alloc(E.N, s);
    k_pf_levels<<<nblk(E.N, 256), 256, 0, s>>>(g, E.nd, E.N, exc, lset.p, r.p, ls.p);
    E.check(E.counted(cudaGetLastError()), "pf levels");
    E.check(cudaMemcpyAsync(E.levels_host.data(), r.p, E.N * 8, cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaMemcpyAsync(E.level_sets_host.data(), ls.p, E.N * sizeof(int),
                            cudaMemcpyDeviceToHost, s), "memcpy");
    E.check(cudaStreamSynchronize(s), "sync");
    // leaf ids -> level-set index in the reference's order (by position)
    std::vector<int> order(leaf_pos.size()), rank(leaf_pos.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = int(i);
    std::sort(order.begin(), order.end(),
              [&](int a, int b) { return leaf_pos[a] < leaf_pos[b]; });
    for (size_t i = 0; i < order.size(); ++i) rank[order[i]] = int(i);
    for (int& v : E.level_sets_host) v = v >= 0 && size_t(v) < rank.size() ? rank[v] : -1;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, E.ev0, E.ev1);
  E.run_time = ms * 1e-3;
  E.prof_ms[3] = ms;
  E.solved = true;
}

namespace {

// TV setup of one image (tv/tv_solver.hpp:71-112), sequential double
// arithmetic as the reference: mean, scale = 2 max |f - mean|, node values in
// 40-bit fixed point (n_bits_function_precision for int64,
// pf_flow_node.hpp:103-115).
struct TVImage {
  double mean = 0, scale = 0;
  std::vector<int64_t> uf;
};
constexpr int kTVBits = 40;

TVImage tv_setup(const double* f, size_t N) {
  TVImage t;
  const double fscale = double(int64_t(1) << kTVBits);
  double v_min = f[0], v_max = f[0], v_sum = f[0];
  for (size_t i = 1; i < N; ++i) {
    v_min = std::min(v_min, f[i]);
    v_max = std::max(v_max, f[i]);
    v_sum += f[i];
  }
  t.mean = v_sum / double(N);
  v_min -= t.mean;
  v_max -= t.mean;
  t.scale = 2 * std::max(v_max, -v_min);
  t.uf.resize(N);
  for (size_t i = 0; i < N; ++i)
    t.uf[i] = int64_t(std::round((0.5 + (f[i] - t.mean) / t.scale) * fscale));
  return t;
}

// Edge values 2 pwf[k] for one lambda (tv_solver.hpp:90-110, max_lambda = lambda).
void tv_edges(const KernelDef* kd, double scale, double lambda, long long* pwf2) {
  const double fscale = double(int64_t(1) << kTVBits);
  const double gsv = 0.5 / (scale * std::max(lambda, 1e-8));
  for (int k = 0; k < kd->K; ++k)
    pwf2[k] = 2LL * (long long)std::round((gsv * kd->weight[k]) / scale * fscale);
}

}  // namespace

// `count` single-lambda TV problems of one shape nx x ny solved together on
// an engine of shape (count * nx, ny): problem p is image f + p * f_stride
// (f_stride 0: every problem uses the same image) at lambdas[p]
// (calculate2dTV<Kernel, int64>(nx, ny, f, lambda), tv/tv_solver.hpp:650-655,
// once per problem).  The problems never share a section, so each one's
// levels equal its own single solve.
int tv_2d_stack_on(Engine& E, size_t nx, size_t ny, size_t count, const double* f,
                   size_t f_stride, const double* lambdas, double* out, int64_t* levels_out) {
  const KernelDef* kd = E.kd;
  const size_t N = nx * ny;
  if (N == 0 || count == 0) return 0;
  const size_t rows = count > 1 ? size_t(E.sub_rows) : nx;
  if (E.nd != 2 || E.dims[1] != ny || (count > 1 && (size_t(E.sub_count) != count ||
                                                     size_t(E.sub_real_rows) != nx)) ||
      (count == 1 && (E.sub_count > 1 || E.dims[0] != nx)))
    throw LfError{2, "engine shape does not match the stacked problems"};
  const double fscale = double(int64_t(1) << kTVBits);
  const size_t n_images = f_stride ? count : 1;
  std::vector<TVImage> img(n_images);
  for (size_t p = 0; p < n_images; ++p) img[p] = tv_setup(f + p * f_stride, N);
  std::vector<long long> pwf2(count * kd->K);
  for (size_t p = 0; p < count; ++p)
    tv_edges(kd, img[f_stride ? p : 0].scale, lambdas[p], &pwf2[p * kd->K]);

  E.alloc_accumulators();
  DevBuf<int64_t> d_uf;
  DevBuf<long long> d_pwf;
  d_uf.alloc(n_images * N, E.stream);
  d_pwf.alloc(pwf2.size(), E.stream);
  for (size_t p = 0; p < n_images; ++p)
    E.check(cudaMemcpyAsync(d_uf.p + p * N, img[p].uf.data(), N * 8, cudaMemcpyHostToDevice,
                            E.stream), "memcpy");
  E.check(cudaMemcpyAsync(d_pwf.p, pwf2.data(), pwf2.size() * 8, cudaMemcpyHostToDevice,
                          E.stream), "memcpy");
  const long long NT = (long long)(N * count);
  k_fill_tv<<<nblk(NT, 256), 256, 0, E.stream>>>(E.g, E.st, NT, int(nx), int(rows),
                                                  f_stride ? (long long)N : 0LL, d_uf.p, d_pwf.p,
                                                  E.d_exc64, E.d_cap64);
  E.check(cudaGetLastError(), "fill tv");
  // the image values are no longer needed once filled
  for (auto& t : img) std::vector<int64_t>().swap(t.uf);
  engine_run_parametric(E);
  // output (tv_solver.hpp:159-175): value of r/2 in the fixed point, mean removed
  std::vector<double> R(N);
  for (size_t p = 0; p < count; ++p) {
    const TVImage& t = img[f_stride ? p : 0];
    // levels_host: the engine's logical rows, problem p from row p * rows
    const int64_t* lv = E.levels_host.data() + p * rows * ny;
    double sum = 0;
    for (size_t i = 0; i < N; ++i) {
      int64_t r = lv[i];
      if (levels_out) levels_out[p * N + i] = r;
      double x = double(r / 2) / fscale;
      double v = (x - 0.5) * t.scale + t.mean;
      R[i] = v;
      sum += v;
    }
    double* o = out + p * N;
    for (size_t i = 0; i < N; ++i) o[i] = (R[i] - sum / double(N)) * t.scale + t.mean;
  }
  return 0;
}

// TV setup of one image on a single-problem parametric engine of shape
// (nx, ny) (tv/tv_solver.hpp:71-112, max_lambda = lambda): fills the
// engine's accumulators, returns the image mean and scale and, per node in
// row-major order, the base value 2 uf (PFFlowNode::base_fv after
// pullBaseFunctionValueFromLattice, pf_flow_node.hpp:398-406).
void tv_fill_single(Engine& E, const double* f, double lambda, double* mean, double* scale,
                    std::vector<int64_t>* base_fv, std::vector<long long>* pwf2_out) {
  const KernelDef* kd = E.kd;
  const size_t nx = E.dims[0], ny = E.dims[1], N = nx * ny;
  if (E.nd != 2 || E.sub_count > 1) throw LfError{2, "TV fill takes one 2-d lattice"};
  TVImage t = tv_setup(f, N);
  std::vector<long long> pwf2(kd->K);
  tv_edges(kd, t.scale, lambda, pwf2.data());
  E.alloc_accumulators();
  DevBuf<int64_t> d_uf;
  DevBuf<long long> d_pwf;
  d_uf.alloc(N, E.stream);
  d_pwf.alloc(pwf2.size(), E.stream);
  E.check(cudaMemcpyAsync(d_uf.p, t.uf.data(), N * 8, cudaMemcpyHostToDevice, E.stream), "memcpy");
  E.check(cudaMemcpyAsync(d_pwf.p, pwf2.data(), pwf2.size() * 8, cudaMemcpyHostToDevice,
                          E.stream), "memcpy");
  k_fill_tv<<<nblk((long long)N, 256), 256, 0, E.stream>>>(E.g, E.st, (long long)N, int(nx),
                                                           int(nx), 0LL, d_uf.p, d_pwf.p,
                                                           E.d_exc64, E.d_cap64);
  E.check(cudaGetLastError(), "fill tv");
  E.check(cudaStreamSynchronize(E.stream), "sync");
  *mean = t.mean;
  *scale = t.scale;
  if (base_fv) {
    base_fv->resize(N);
    for (size_t i = 0; i < N; ++i) (*base_fv)[i] = 2 * t.uf[i];
  }
  if (pwf2_out) *pwf2_out = pwf2;
}

// calculate2dTV<Kernel, int64>(nx, ny, f, lambda)  (tv/tv_solver.hpp:650-655)
// on an existing parametric engine of shape (nx, ny) (its buffers are reused).
int tv_2d_on(Engine& E, const double* f, double lambda, double* out, int64_t* levels_out) {
  return tv_2d_stack_on(E, E.dims[0], E.dims[1], 1, f, 0, &lambda, out, levels_out);
}

int tv_2d(const KernelDef* kd, size_t nx, size_t ny, const double* f, double lambda, double* out,
          int64_t* levels_out, int32_t* sets_out) {
  if (nx * ny == 0) return 0;
  size_t dims[2] = {nx, ny};
  Engine E("GPULevelReductions", kd, 2, dims);
  const int rc = tv_2d_on(E, f, lambda, out, levels_out);
  if (sets_out)
    std::memcpy(sets_out, E.level_sets_host.data(), nx * ny * sizeof(int32_t));
  return rc;
}

Engine* new_tv_stack_engine(const KernelDef* kd, size_t nx, size_t ny, size_t count) {
  if (count <= 1) {
    size_t dims[2] = {nx, ny};
    return new Engine("GPULevelReductions", kd, 2, dims);
  }
  const size_t rows = (nx + 31) / 32 * 32;  // the padded rows of one lattice
  if (rows * count > size_t(INT_MAX / 2)) throw LfError{2, "stack too tall"};
  size_t dims[2] = {rows * count, ny};
  Engine* E = new Engine("GPULevelReductions", kd, 2, dims);
  E->sub_count = int(count);
  E->sub_rows = int(rows);
  E->sub_real_rows = int(nx);
  return E;
}

// Problems per stacked solve: as many as keep the stack within max_nodes.
size_t tv_stack_size(size_t nx, size_t ny, size_t count, size_t max_nodes) {
  const size_t N = std::max<size_t>(nx * ny, 1);
  size_t per = std::max<size_t>(max_nodes / N, 1);
  per = std::min(per, count);
  // INT_MAX / 2 rows at most in one engine
  per = std::min(per, std::max<size_t>(size_t(INT_MAX / 2) / ((nx + 31) / 32 * 32), 1));
  return std::max<size_t>(per, 1);
}

// Many single-lambda TV problems of one shape.  Stacked problems advance in
// lockstep generations (every generation waits for its slowest member), so
// only small problems are stacked -- up to max_nodes lattice nodes per stack
// (0: 2^18), where launch and synchronisation costs dominate -- and the
// stacks run as independent solves on `workers` host threads (0: 8), each
// with its own engine and CUDA stream, whose kernels overlap on the device.
int tv_2d_batch(const KernelDef* kd, size_t nx, size_t ny, size_t count, const double* f,
                size_t f_stride, const double* lambdas, double* out, int64_t* levels_out,
                size_t max_nodes, int workers) {
  const size_t N = nx * ny;
  if (N == 0 || count == 0) return 0;
  if (max_nodes == 0) max_nodes = kTVStackNodes;
  if (workers <= 0) workers = 8;
  const size_t per = tv_stack_size(nx, ny, count, max_nodes);
  const size_t stacks = (count + per - 1) / per;
  const int W = int(std::min<size_t>(size_t(workers), stacks));
  int device = 0;
  cudaGetDevice(&device);
  std::atomic<size_t> next{0};
  std::mutex mu;
  LfError first{0, ""};
  bool failed = false;
  auto work = [&]() {
    cudaSetDevice(device);
    std::unique_ptr<Engine> E;
    size_t E_count = 0;
    for (;;) {
      const size_t s = next.fetch_add(1);
      if (s >= stacks) return;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (failed) return;
      }
      const size_t p0 = s * per, m = std::min(per, count - p0);
      try {
        if (!E || E_count != m) {
          E.reset();
          E.reset(new_tv_stack_engine(kd, nx, ny, m));
          E_count = m;
        }
        tv_2d_stack_on(*E, nx, ny, m, f + p0 * f_stride, f_stride, lambdas + p0, out + p0 * N,
                       levels_out ? levels_out + p0 * N : nullptr);
      } catch (const LfError& e) {
        std::lock_guard<std::mutex> lk(mu);
        if (!failed) { failed = true; first = e; }
        return;
      } catch (const std::exception& e) {
        std::lock_guard<std::mutex> lk(mu);
        if (!failed) { failed = true; first = LfError{7, e.what()}; }
        return;
      }
    }
  };
  if (W <= 1) {
    work();
  } else {
    std::vector<std::thread> th;
    for (int w = 0; w < W; ++w) th.emplace_back(work);
    for (auto& t : th) t.join();
  }
  if (failed) throw first;
  return 0;
}

}  // namespace lfg
