// CPU restatement of latticeflow's lattice push-relabel, parametric flow and
// single-lambda TV solver.
//
// TEST INFRASTRUCTURE ONLY: this is the oracle.  It is loaded by tests, by
// the smoke check and by the benchmark's CPU-baseline leg; the GPU product
// never links or calls it.
//
// Each routine restates the reference algorithm step for step (same node
// order, same queue discipline, same tie order), so that on the same inputs
// it produces the same final state as the reference build:
//   lattice layout ............ lattices/lattice.hpp:102-111, kernellattice.hpp:61-96
//   node state / flips ........ network_flow/network_flow_node.hpp:112-126,171-190,313-402
//   energy fill ............... network_flow/network_flow_node.hpp:420-485
//   PRFlow .................... network_flow/push_relabel.hpp:306-745,1069-1487
//   PF driver / offsets ....... parametricflow/pf_solver.hpp:33-208, pf_flow_node.hpp:291-396
//   TV setup / output ......... tv/tv_solver.hpp:71-112,151-176,270-285
// The sorting step of the discharge loop is the bitonic network for arbitrary
// n (push_relabel.hpp:1145, make_sorting_functions.py:16-54), comparing
// heights only (pr_auxilary_structures.hpp:13-15).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <climits>
#include <deque>
#include <map>
#include <memory>
#include <queue>
#include <set>
#include <unordered_set>
#include <vector>

namespace {

typedef int64_t dtype;
typedef __int128 comp_type;

// ---------------------------------------------------------------- sorting net
struct CmpEx { int lo, hi; };

int largest_pow2_below(int n) { int k = 1; while (k < n) k *= 2; return k / 2; }

void merge_steps(std::vector<CmpEx>& out, int s, int n, bool up) {
  if (n <= 1) return;
  int m = largest_pow2_below(n);
  for (int i = s; i < s + n - m; ++i) out.push_back(up ? CmpEx{i, i + m} : CmpEx{i + m, i});
  merge_steps(out, s, m, up);
  merge_steps(out, s + m, n - m, up);
}

void sort_steps(std::vector<CmpEx>& out, int s, int n, bool up) {
  if (n <= 1) return;
  int m = n / 2;
  sort_steps(out, s, m, !up);
  sort_steps(out, s + m, n - m, up);
  merge_steps(out, s, n, up);
}

// ---------------------------------------------------------------- lattice
struct Lattice {
  int nd = 0;
  int64_t dims[4] = {0, 0, 0, 0};
  int64_t full[4] = {0, 0, 0, 0};
  int64_t stride[4] = {0, 0, 0, 0};
  int64_t begin = 0, end = 0, size_all = 0;
  int K = 0;
  std::vector<int64_t> jump;  // lattice order: [0, K/2) positive ascending, i+K/2 reverse of i
  std::vector<int> delta;     // K*nd

  void init(int _nd, const int64_t* d, int _K, const int* offs) {
    nd = _nd; K = _K;
    delta.assign(offs, offs + K * nd);
    int64_t b[4] = {0, 0, 0, 0};
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < nd; ++i) b[i] = std::max<int64_t>(b[i], std::abs(offs[k * nd + i]));
    for (int i = 0; i < nd; ++i) { dims[i] = d[i]; full[i] = d[i] + b[i]; }
    full[0] += 3 * b[0];
    stride[nd - 1] = 1;
    for (int i = nd - 2; i >= 0; --i) stride[i] = stride[i + 1] * full[i + 1];
    size_all = stride[0] * full[0];
    begin = 2 * b[0] * stride[0];
    end = size_all - 2 * b[0] * stride[0];
    jump.resize(K);
    for (int k = 0; k < K; ++k) {
      int64_t j = 0;
      for (int i = 0; i < nd; ++i) j += int64_t(offs[k * nd + i]) * stride[i];
      jump[k] = j;
    }
  }
  int rev(int k) const { return k < K / 2 ? k + K / 2 : k - K / 2; }
  // padded index of bounded (row-major, last dim fastest) node index
  int64_t padded(int64_t bidx) const {
    int64_t p = begin;
    for (int i = nd - 1; i >= 0; --i) { int64_t c = bidx % dims[i]; bidx /= dims[i]; p += c * stride[i]; }
    return p;
  }
  bool within(int64_t p) const {
    if (p < begin || p >= end) return false;
    int64_t q = p - begin;
    for (int i = 0; i < nd; ++i) { int64_t c = q / stride[i]; q %= stride[i]; if (c >= dims[i]) return false; }
    return true;
  }
  int64_t n_bounded() const { int64_t n = 1; for (int i = 0; i < nd; ++i) n *= dims[i]; return n; }
};

struct Node {
  uint32_t key_state = 0;
  uint32_t height = 0;
  uint32_t level_index = 0;
  dtype reduction = 0;
};

// ---------------------------------------------------------------- PR engine
// PRFlow<dtype, Lattice, 0> with NFNodeDefaultPolicy-style keys (push_relabel.hpp:45-1487)
struct PR {
  Lattice& L;
  std::vector<Node>& nodes;
  std::vector<dtype>& alpha;  // size_all * K
  int K;
  uint32_t key = 0;
  size_t top_level = 1, tlwe = 0;
  struct Level { std::vector<int64_t> nodes, active; };
  std::vector<Level> levels;
  std::vector<CmpEx> net;
  std::vector<int64_t> node_buffer;

  PR(Lattice& l, std::vector<Node>& n, std::vector<dtype>& a) : L(l), nodes(n), alpha(a), K(l.K) {
    int64_t mx = 0;
    for (int i = 0; i < L.nd; ++i) mx = std::max(mx, L.dims[i]);
    levels.resize(size_t(2 * mx + 25));
    sort_steps(net, 0, K, true);
  }

  dtype& al(int64_t n, int k) { return alpha[size_t(n) * K + k]; }
  bool eligible(int64_t n) const { return nodes[n].key_state == key; }
  dtype excess(int64_t n) const { return -nodes[n].reduction; }
  dtype sinkFlow(int64_t n) const { return nodes[n].reduction; }
  dtype pushCap(int64_t n, int k) { dtype a = al(n, k); return a > 0 ? a : 0; }

  // network_flow_node.hpp:313-354 (start state 0 -> 1, or 1 -> 0)
  void nodeFlip(int64_t n, int start_state) {
    for (int i = 0; i < K; ++i) al(n + L.jump[i], L.rev(i)) *= -1;
    if (start_state == 0) nodes[n].key_state |= 1u; else nodes[n].key_state &= ~1u;
  }
  // network_flow_node.hpp:357-402, partition 0
  void pushExcess(int64_t src, int64_t dst, int ei, dtype amount) {
    nodes[src].reduction += amount;
    al(src, ei) -= amount;
    nodes[dst].reduction -= amount;
    al(dst, L.rev(ei)) += amount;
  }

  void ensureLevel(size_t lv) {
    if (lv >= levels.size()) levels.resize(2 * levels.size());
  }

  void addToLevel(int64_t n, size_t new_level, int status /*0 no,1 has,2 check*/) {
    bool has = status == 2 ? excess(n) > 0 : status == 1;
    if (new_level > top_level) { ++top_level; ensureLevel(top_level); }
    nodes[n].height = uint32_t(new_level);
    Level& lv = levels[new_level];
    nodes[n].level_index = uint32_t(lv.nodes.size());
    lv.nodes.push_back(n);
    if (has) { lv.active.push_back(n); if (tlwe < new_level) tlwe = new_level; }
  }

  void nodeNowHasExcess(int64_t n) {
    levels[nodes[n].height].active.push_back(n);
    if (tlwe < nodes[n].height) tlwe = nodes[n].height;
  }

  void push(int64_t src, int64_t dst, int ei, dtype amount, bool may_have_excess) {
    if (amount == 0) return;
    pushExcess(src, dst, ei, amount);
    dtype de = excess(dst);
    if (may_have_excess && de > 0 && de <= amount) nodeNowHasExcess(dst);
  }

  void raiseAndFlip(size_t level) {
    for (size_t lv = level; lv <= top_level; ++lv) {
      for (int64_t n : levels[lv].nodes) flipNode(n, false);
      levels[lv].nodes.clear();
    }
    top_level = level - 1;
  }

  void flipNode(int64_t n, bool check_top) {
    if (check_top && levels[nodes[n].height].nodes.empty()) {
      if (top_level > nodes[n].height) raiseAndFlip(nodes[n].height);
      else top_level = nodes[n].height - 1;
    }
    nodes[n].height = 0;
    nodeFlip(n, 0);
  }

  void initQueue() { top_level = 1; tlwe = 0; }

  // push_relabel.hpp:306-415
  template <class It>
  void hotStart(It start, It end) {
    initQueue();
    std::vector<int64_t>& orig = node_buffer;
    orig.clear();
    for (It it = start; it != end; ++it) {
      int64_t n = *it;
      if (sinkFlow(n) > 0) { orig.push_back(n); nodes[n].height = 1; }
    }
    std::deque<int64_t> q;
    auto addNeighbors = [&](int64_t n, size_t cur) {
      for (int i = 0; i < K; ++i) {
        int64_t nn = n + L.jump[i];
        if (eligible(nn) && nodes[nn].height == 0 && pushCap(nn, L.rev(i)) > 0) {
          addToLevel(nn, cur + 1, 2);
          q.push_back(nn);
        }
      }
    };
    for (int64_t n : orig) addNeighbors(n, 0);
    size_t cur = 0;
    while (!q.empty()) {
      int64_t n = q.front(); q.pop_front();
      if (nodes[n].height != cur) { ++cur; ensureLevel(cur + 1); }
      addNeighbors(n, cur);
    }
    for (It it = start; it != end; ++it) {
      int64_t n = *it;
      if (nodes[n].height == 0) flipNode(n, false);
    }
    for (int64_t n : orig) nodes[n].height = 0;
    orig.clear();
  }

  // push_relabel.hpp:417-509
  void quickFlow() {
    for (size_t level = top_level; level != 1; --level) {
      Level& lv = levels[level];
      for (size_t idx = 0; idx < lv.active.size(); ++idx) {
        int64_t n = lv.active[idx];
        if (!eligible(n) || nodes[n].height != level || excess(n) <= 0) continue;
        dtype rem = excess(n);
        for (int i = 0; i < K; ++i) {
          int64_t nn = n + L.jump[i];
          dtype cap = pushCap(n, i);
          if (cap != 0 && eligible(nn) && nodes[nn].height == level - 1) {
            dtype amount = std::min(rem, cap);
            rem -= amount;
            push(n, nn, i, amount, true);
            if (rem == 0) {
              std::swap(lv.active[idx], lv.active.back());
              lv.active.pop_back();
              --idx;
              break;
            }
          }
        }
      }
      if (tlwe == level && lv.active.empty()) --tlwe;
    }
    Level& lv = levels[1];
    for (size_t idx = 0; idx < lv.active.size(); ++idx) {
      int64_t n = lv.active[idx];
      if (!eligible(n) || nodes[n].height != 1 || excess(n) <= 0) continue;
      dtype rem = excess(n);
      for (int i = 0; i < K; ++i) {
        int64_t nn = n + L.jump[i];
        dtype cap = pushCap(n, i), sf;
        if (cap != 0 && eligible(nn) && nodes[nn].height == 0 && (sf = sinkFlow(nn)) > 0) {
          dtype amount = std::min(std::min(rem, cap), sf);
          rem -= amount;
          push(n, nn, i, amount, false);
          if (rem == 0) {
            std::swap(lv.active[idx], lv.active.back());
            lv.active.pop_back();
            --idx;
            break;
          }
        }
      }
    }
    if (tlwe == 1 && lv.active.empty()) --tlwe;
  }

  // push_relabel.hpp:532-587
  bool nextInQueue(int64_t& out, bool& base_empty) {
    for (;;) {
      if (tlwe == 0) return true;
      while (levels[tlwe].active.empty()) { --tlwe; if (tlwe == 0) return true; }
      Level& lv = levels[tlwe];
      int64_t n = lv.active.back();
      lv.active.pop_back();
      if (excess(n) <= 0) continue;
      uint32_t li = nodes[n].level_index;
      std::swap(lv.nodes[li], lv.nodes.back());
      nodes[lv.nodes[li]].level_index = li;
      lv.nodes.pop_back();
      base_empty = lv.nodes.empty();
      out = n;
      return false;
    }
  }

  void finish() {
    for (size_t level = 1; level <= top_level; ++level) {
      for (int64_t n : levels[level].nodes) nodes[n].height = 0;
      levels[level].nodes.clear();
    }
    top_level = 1;
  }

  // push_relabel.hpp:1069-1278
  void runLoop() {
    if (levels[1].nodes.empty()) return;
    struct PN { uint32_t h; int idx; };
    std::vector<PN> hl(K);
    std::vector<int64_t> nl(K);
    bool base_empty = false;
    int64_t n = 0;
    for (;;) {
    next_iteration:
      if (nextInQueue(n, base_empty)) break;
      uint32_t base_height = nodes[n].height;
      dtype rem = excess(n);
      int first_nn = K, last_valid = 0;
      for (int i = 0; i < K; ++i) {
        int64_t nn = nl[i] = n + L.jump[i];
        bool valid = pushCap(n, i) != 0 && eligible(nn);
        hl[i].h = valid ? nodes[nn].height + 1 : 0;
        hl[i].idx = i;
        if (valid) { --first_nn; last_valid = i; }
      }
      if (first_nn == K) { flipNode(n, base_empty); continue; }
      if (first_nn == K - 1) {
        hl[first_nn] = hl[last_valid];
      } else if (K <= 48) {
        for (const CmpEx& c : net) if (hl[c.hi].h < hl[c.lo].h) std::swap(hl[c.lo], hl[c.hi]);
      } else {
        std::sort(hl.begin(), hl.end(), [](const PN& a, const PN& b) { return a.h < b.h; });
      }
      if (base_height == 1 && hl[first_nn].h == 1) {
        for (int i = first_nn; i < K && hl[i].h == 1; ++i) {
          int idx = hl[i].idx;
          int64_t nn = nl[idx];
          dtype pc = pushCap(n, idx);
          dtype amount = std::min(std::min(pc, rem), sinkFlow(nn));
          rem -= amount;
          push(n, nn, idx, amount, false);
          if (pc == amount) { std::swap(hl[i], hl[first_nn]); ++first_nn; }
          if (rem == 0) { addToLevel(n, 1, 0); goto next_iteration; }
        }
        for (int i = first_nn; i < K && hl[i].h == 1; ++i) {
          addToLevel(nl[hl[i].idx], 1, 2);
          ++hl[i].h;
        }
        base_empty = false;
      }
      for (int i = first_nn; i < K; ++i) {
        if (base_empty && hl[i].h > base_height) {
          raiseAndFlip(base_height);
          flipNode(n, false);
          goto next_iteration;
        }
        int idx = hl[i].idx;
        int64_t nn = nl[idx];
        dtype amount = std::min(pushCap(n, idx), rem);
        rem -= amount;
        push(n, nn, idx, amount, true);
        if (rem == 0) { addToLevel(n, hl[i].h, 0); goto next_iteration; }
      }
      flipNode(n, base_empty);
    }
    finish();
    top_level = 1;
    tlwe = 0;
  }

  // push_relabel.hpp:1303-1354 (whole lattice, key 0)
  void run() {
    key = 0;
    std::vector<int64_t> all;
    all.reserve(size_t(L.end - L.begin));
    for (int64_t p = L.begin; p < L.end; ++p) all.push_back(p);
    hotStart(all.begin(), all.end());
    quickFlow();
    runLoop();
  }

  // push_relabel.hpp:1360-1384, 1383-1463, 1468-1487
  template <class It> void prepareSection(It s, It e, uint32_t k) {
    key = k << 1;
    for (It it = s; it != e; ++it) nodes[*it].key_state = (k << 1);
  }
  template <class It> void runSection(It s, It e, uint32_t k) {
    key = k << 1;
    hotStart(s, e);
    quickFlow();
    runLoop();
  }
  template <class It> void cleanupSection(It s, It e) {
    for (It it = s; it != e; ++it) {
      int64_t n = *it;
      if ((nodes[n].key_state & 1u) != 0) nodeFlip(n, 1);
      nodes[n].key_state &= 1u;
    }
  }
};

// ---------------------------------------------------------------- problem
struct Problem {
  Lattice L;
  std::vector<Node> nodes;
  std::vector<dtype> alpha;
  std::vector<dtype> offset;  // PF current_fv_offset (pf_flow_node.hpp:125)

  void init(int nd, const int64_t* dims, int K, const int* offs) {
    L.init(nd, dims, K, offs);
    nodes.assign(size_t(L.size_all), Node());
    alpha.assign(size_t(L.size_all) * K, 0);
    offset.assign(size_t(L.size_all), 0);
  }
  // NodeFiller::addE1 / addE2 (network_flow_node.hpp:420-485), 2x-scaled mode
  void addE1(int64_t n, dtype e0, dtype e1) { nodes[n].reduction += 2 * (e1 - e0); }
  void addE2(int64_t n1, int ei, dtype e00, dtype e01, dtype e10, dtype e11) {
    int64_t n2 = n1 + L.jump[ei];
    dtype q1 = e10 - e00, q2 = e01 - e00, q12 = e00 + e11 - e01 - e10;
    nodes[n1].reduction += 2 * q1 + q12;
    nodes[n2].reduction += 2 * q2 + q12;
    alpha[size_t(n1) * L.K + ei] += -q12;
    alpha[size_t(n2) * L.K + L.rev(ei)] += -q12;
  }
  // LatticeFlowDirectInterface::addEnergyPotentials (direct_interface.hpp:60-95):
  // every node's unary, then every in-bounds positive edge.
  void fill(const int64_t* unary, const int64_t* binary) {
    int64_t N = L.n_bounded();
    int Kp = L.K / 2;
    for (int64_t b = 0; b < N; ++b) addE1(L.padded(b), unary[2 * b], unary[2 * b + 1]);
    for (int64_t b = 0; b < N; ++b) {
      int64_t p = L.padded(b);
      for (int e = 0; e < Kp; ++e) {
        if (!L.within(p + L.jump[e])) continue;
        const int64_t* q = binary + (size_t(b) * Kp + e) * 4;
        addE2(p, e, q[0], q[1], q[2], q[3]);
      }
    }
  }
  dtype r(int64_t n) const { return nodes[n].reduction + offset[n]; }
  // PFFlowNode::setOffset (pf_flow_node.hpp:310-319)
  void setOffset(int64_t n, dtype off) {
    nodes[n].reduction += offset[n] - off;
    offset[n] = off;
  }
};

// ParametricFlowSolver::run (pf_solver.hpp:33-208) + setToMeanReductionPoint
// (pf_flow_node.hpp:330-396).  Leaves final r() values in the lattice; with
// level_sets, also returns the level sets as the reference does (ranges of
// the partitioned node list between the sorted split boundaries, each sorted
// by node, pf_solver.hpp:180-203).
void run_pf(Problem& P, std::vector<std::vector<int64_t>>* level_sets = nullptr) {
  PR pr(P.L, P.nodes, P.alpha);
  std::vector<int64_t> pts;
  for (int64_t p = P.L.begin; p < P.L.end; ++p)
    if (P.L.within(p)) pts.push_back(p);
  struct Range { size_t s, e; };
  std::deque<Range> q;
  uint32_t key = 1;
  q.push_back({0, pts.size()});
  std::vector<size_t> boundaries(1, 0);
  while (!q.empty()) {
    Range rg = q.front(); q.pop_front();
    // setToMeanReductionPoint
    comp_type r_sum = 0;
    double count = 0;
    dtype r_min = P.r(pts[rg.s]), r_max = r_min;
    for (size_t i = rg.s; i < rg.e; ++i) {
      dtype r = P.r(pts[i]);
      r_sum += r;
      r_min = std::min(r_min, r);
      r_max = std::max(r_max, r);
      count += 1;
    }
    if (r_max - r_min <= 1) continue;
    dtype r_new = dtype(std::ceil(double(r_sum) / count));
    if (r_new == r_max) --r_new;
    for (size_t i = rg.s; i < rg.e; ++i) P.setOffset(pts[i], r_new);

    auto b = pts.begin() + rg.s, e = pts.begin() + rg.e;
    pr.prepareSection(b, e, key);
    pr.runSection(b, e, key);

    // two-pointer partition by state (pf_solver.hpp:101-152)
    size_t fwd = rg.s, bck = rg.e - 1;
    long mid = 0;
    auto st = [&](size_t i) { return (P.nodes[pts[i]].key_state & 1u) != 0; };
    for (;;) {
      bool done = false;
      while (!st(fwd)) { ++fwd; if (bck == fwd) { done = true; break; } }
      if (!done)
        while (st(bck)) { --bck; if (bck == fwd) { done = true; break; } }
      if (!done) {
        std::swap(pts[fwd], pts[bck]);
        ++fwd;
        if (fwd == bck) done = true;
      }
      if (done) {
        if (bck != rg.e && !st(bck)) ++bck;
        mid = long(bck - rg.s);
        break;
      }
    }
    long top = long(rg.e - rg.s);
    if (mid > 0) q.push_back({rg.s, rg.s + size_t(mid)});
    if (mid < top) {
      q.push_back({rg.s + size_t(mid), rg.e});
      for (size_t i = rg.s + size_t(mid); i < rg.e; ++i) pr.nodeFlip(pts[i], 1);
    }
    if (mid > 0 && mid < top) boundaries.push_back(rg.s + size_t(mid));
    pr.cleanupSection(b, e);
    ++key;
  }
  for (int64_t p : pts) P.setOffset(p, 0);
  if (level_sets) {
    const size_t n_sets = boundaries.size();
    boundaries.push_back(pts.size());
    std::sort(boundaries.begin(), boundaries.end());
    level_sets->assign(n_sets, {});
    for (size_t i = 0; i < n_sets; ++i) {
      auto& ls = (*level_sets)[i];
      ls.assign(pts.begin() + boundaries[i], pts.begin() + boundaries[i + 1]);
      std::sort(ls.begin(), ls.end());
    }
  }
}

// ---------------------------------------------------------------- TV path
//
// TVSolver<Kernel, int64>::run and getRegularizationPath (tv/tv_solver.hpp:
// 114-244, 300-642), TVRegPathSegment (tv/tv_regpath_node.hpp:62-1009) and
// the region operations of TV_PRFlow (tv/tv_push_relabel.hpp:84-237,
// 339-468), restated on the port's lattice.  Segments live in a deque and
// are named by index (key - 1).  The reference orders a segment's neighbour
// set by segment address; segments are allocated in creation order from its
// deque, so the restatement orders neighbour sets by creation index.

constexpr int kScaleBits = 48;   // n_bits_scale_precision for int64 (pf_flow_node.hpp:106)
constexpr int kAdjustBits = 16;  // n_bits_function_room for int64 (pf_flow_node.hpp:110)
constexpr dtype kDtMax = INT64_MAX;

inline comp_type iabs(comp_type x) { return x >= 0 ? x : -x; }
// int64 products and sums of the reference that are formed in dtype (two's
// complement wrap, as the reference build computes them)
inline dtype wmul(dtype a, dtype b) { return dtype(uint64_t(a) * uint64_t(b)); }
inline dtype wadd(dtype a, dtype b) { return dtype(uint64_t(a) + uint64_t(b)); }

// PFFlowNode::multFVScale (pf_flow_node.hpp:160-176)
dtype multFVScale(comp_type fv, dtype lm) {
  fv *= lm;
  fv += (fv > 0 ? 1 : -1) * (comp_type(1) << (kScaleBits - 1));
  fv /= (comp_type(1) << kScaleBits);
  return dtype(fv);
}

// PFFlowNode::getScaleFromQuotient_T (pf_flow_node.hpp:178-203)
dtype scaleFromQuotient(comp_type numer, comp_type denom) {
  if (denom == 0) return kDtMax;
  numer *= (comp_type(1) << kScaleBits);
  numer /= denom;
  return numer > kDtMax ? kDtMax : dtype(numer);
}

// floorAverage (common/type_processing.hpp:58-70)
dtype floorAverage(comp_type sum, long n) {
  if (sum < 0) sum -= (n - 1);
  sum /= n;
  return dtype(sum);
}

dtype toScaleDType(double lm) { return dtype(std::round(lm * double(int64_t(1) << kScaleBits))); }

// The lattice of TV nodes (TVFlowNode = PFFlowNode<..., PFScaledUnweightedNodePolicy>):
// base value qii, current value lm_qii = multFVScale(qii, lambda), offset.
struct TVLattice {
  Problem P;
  std::vector<dtype> base_fv, cur_fv;
  double fmean = 0, fscale = 0, max_lambda = 0;

  dtype fv(int64_t n, dtype lm) const { return multFVScale(base_fv[n], lm); }
  dtype r(int64_t n) const { return P.r(n); }
  uint32_t key(int64_t n) const { return P.nodes[n].key_state >> 1; }
  // PFFlowNode::setOffsetAndScale (pf_flow_node.hpp:293-309)
  void setOffsetAndScale(int64_t n, dtype off, dtype lm) {
    const dtype true_fv = fv(n, lm);
    const dtype delta = (true_fv - off) - (cur_fv[n] - P.offset[n]);
    P.nodes[n].reduction += delta;
    cur_fv[n] = true_fv;
    P.offset[n] = off;
  }

  // TVSolver::setup (tv_solver.hpp:71-112)
  void setup(int64_t nx, int64_t ny, int K, const int* offsets, const double* weights,
             const double* f, double lam_max) {
    const double fs = double(int64_t(1) << 40);  // n_bits_function_precision for int64
    int64_t dims[2] = {nx, ny};
    P.init(2, dims, K, offsets);
    base_fv.assign(size_t(P.L.size_all), 0);
    cur_fv.assign(size_t(P.L.size_all), 0);
    const int64_t N = nx * ny;
    double v_min = f[0], v_max = f[0], v_sum = f[0];
    for (int64_t i = 1; i < N; ++i) {
      v_min = std::min(v_min, f[i]);
      v_max = std::max(v_max, f[i]);
      v_sum += f[i];
    }
    fmean = v_sum / double(N);
    v_min -= fmean;
    v_max -= fmean;
    fscale = 2 * std::max(v_max, -v_min);
    max_lambda = std::max(lam_max, 1e-8);
    for (int64_t b = 0; b < N; ++b) {
      const int64_t p = P.L.padded(b);
      const double v = 0.5 + (f[b] - fmean) / fscale;
      P.addE1(p, 0, dtype(std::round(v * fs)));
      base_fv[p] = P.nodes[p].reduction;  // pullBaseFunctionValueFromLattice
      cur_fv[p] = base_fv[p];
      P.offset[p] = 0;
    }
    const double gsv = 0.5 / (fscale * max_lambda);
    for (int64_t b = 0; b < N; ++b) {
      const int64_t p = P.L.padded(b);
      for (int e = 0; e < K / 2; ++e) {
        if (!P.L.within(p + P.L.jump[e])) continue;
        const dtype pwf = dtype(std::round((gsv * weights[e]) / fscale * fs));
        P.addE2(p, e, 0, pwf, pwf, 0);
      }
    }
  }
  // TVSolver::toFValue (tv_solver.hpp:281-285)
  double toFValue(dtype x) const {
    return (double(x) / double(int64_t(1) << 40) - 0.5) * fscale + fmean;
  }
};

// TV_PRFlow::CutInfo (tv_push_relabel.hpp:44-55)
struct CutInfo {
  bool any_cut = false;
  std::vector<int64_t> part[2];  // [0] off nodes, [1] on nodes
  dtype cut_value = 0;
  std::vector<std::pair<int64_t, int>> cut_edges;
};
typedef std::shared_ptr<CutInfo> CutPtr;

struct TVPath {
  enum Mode { Unset, Initial, Join, Split };
  enum Event { EvJoin, EvSplit, EvSplitUB };

  struct Seg {
    Mode rhs_mode = Unset, lhs_mode = Unset;
    dtype rhs_lambda = 0, lhs_lambda = -1;
    dtype ar1 = 0, ar0 = 0;  // adjusted_r_at_1 / adjusted_r_at_0
    size_t n_nodes = 0;
    std::vector<int64_t> nodeset;  // kept after deactivation (Split / Initial segments)
    int rhs_nodes[2] = {-1, -1}, lhs_nodes[2] = {-1, -1};
    // ConstructionInfo (tv_regpath_node.hpp:249-277), alive while active
    uint32_t key = 0;
    bool active = true;
    std::set<int> neighbors;
    std::multimap<dtype, int> join_points;
    std::vector<int64_t> ci_nodes;
    dtype split_done_to = -1, lambda_of_split = -1;
    CutPtr split_info;
  };

  struct RegionInfo {
    dtype lm_qii_sum_d = 0, r_sum_d = 0, zero_reference = 0, partition_size = 0;
    comp_type qii_sum = 0, gamma_sum = 0;
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

  TVLattice& T;
  PR pr;  // TV_PRFlow: the one solver of every region probe
  const int K;
  std::deque<Seg> segs;
  std::vector<int> node_map;  // segment of every node at the largest lambda
  dtype calculated_lambda = -1;
  bool broken = false;        // a trace met a segment without a successor

  explicit TVPath(TVLattice& t) : T(t), pr(t.P.L, t.P.nodes, t.P.alpha), K(t.P.L.K) {}

  int newSeg() {
    segs.emplace_back();
    segs.back().key = uint32_t(segs.size());
    return int(segs.size()) - 1;
  }

  // TVRegPathSegment::getRegionInfo (tv_regpath_node.hpp:176-206)
  RegionInfo regionInfo(const std::vector<int64_t>& nodes) const {
    RegionInfo ri;
    ri.zero_reference = T.r(nodes[0]);
    for (int64_t n : nodes) {
      ri.lm_qii_sum_d = wadd(ri.lm_qii_sum_d, T.cur_fv[n] - ri.zero_reference);
      ri.r_sum_d = wadd(ri.r_sum_d, T.r(n) - ri.zero_reference);
      ri.qii_sum += T.base_fv[n];
      ++ri.partition_size;
    }
    ri.gamma_sum = comp_type(dtype(ri.r_sum_d - ri.lm_qii_sum_d));
    return ri;
  }

  // TVRegPathSegment::syncInformation (tv_regpath_node.hpp:216-245)
  void syncInformation(Seg& s, dtype lambda) {
    s.n_nodes = 0;
    for (int64_t n : s.ci_nodes) {
      T.setOffsetAndScale(n, 0, lambda);
      T.P.nodes[n].key_state = s.key << 1;  // setKey<0>
      ++s.n_nodes;
    }
    const RegionInfo ri = regionInfo(s.ci_nodes);
    const comp_type adj = comp_type(1) << kAdjustBits;
    s.ar0 = dtype((ri.gamma_sum * adj) / comp_type(ri.partition_size));
    s.ar1 = dtype(((ri.qii_sum + ri.gamma_sum) * adj) / comp_type(ri.partition_size));
  }

  // TVRegPathSegment::get_r_AtLambda / deadjust_r (tv_regpath_node.hpp:131-148)
  dtype rAtLambda(const Seg& s, dtype lambda) const {
    dtype v = s.ar0 + multFVScale(comp_type(dtype(s.ar1 - s.ar0)), lambda);
    v += (v < 0 ? -1 : 1) * (dtype(1) << (kAdjustBits - 1));
    return v / (dtype(1) << kAdjustBits);
  }

  // TV_PRFlow::runPartitionedSection (tv_push_relabel.hpp:84-237)
  CutPtr runPartitionedSection(const std::vector<int64_t>& nodes, uint32_t key) {
    pr.runSection(nodes.begin(), nodes.end(), key);
    bool any_on = false, any_off = false;
    for (int64_t n : nodes) {
      if (T.P.nodes[n].key_state & 1u) any_on = true; else any_off = true;
      if (any_on && any_off) break;
    }
    CutPtr cut = std::make_shared<CutInfo>();
    if (any_on && !any_off) {
      for (int64_t n : nodes) pr.nodeFlip(n, 1);
      return cut;
    }
    if (any_off && !any_on) return cut;
    cut->any_cut = true;
    const uint32_t on_state = (key << 1) | 1u;
    for (int64_t n : nodes) {
      const bool n_on = (T.P.nodes[n].key_state & 1u) != 0;
      cut->part[n_on ? 1 : 0].push_back(n);
      if (!n_on) {
        for (int ei = 0; ei < K; ++ei) {
          const int64_t nn = n + T.P.L.jump[ei];
          if (T.P.nodes[nn].key_state == on_state) {
            const dtype a = T.P.alpha[size_t(n) * K + ei];
            cut->cut_value += (a < 0 ? -a : a) >> 1;  // edgeCapacityFromSaturatedOffNodeToOnNode
            cut->cut_edges.push_back({nn, T.P.L.rev(ei)});
          }
        }
      }
    }
    for (int64_t n : cut->part[1]) pr.nodeFlip(n, 1);
    return cut;
  }

  // TV_PRFlow::applyPartioningCut (tv_push_relabel.hpp:239-248)
  void applyPartitioningCut(const CutInfo& cut) {
    for (const auto& ce : cut.cut_edges) {
      const int64_t n = ce.first;
      const int ei = ce.second;
      const dtype a = T.P.alpha[size_t(n) * K + ei];
      pr.pushExcess(n, n + T.P.L.jump[ei], ei, a > 0 ? a : 0);
    }
  }

  // TV_PRFlow::setRegionToLambda (tv_push_relabel.hpp:414-468)
  void setRegionToLambda(const std::vector<int64_t>& nodes, dtype lambda, bool pull_to_center) {
    comp_type qii_sum = 0, gamma_sum = 0;
    long psize = 0;
    for (int64_t n : nodes) {
      qii_sum += T.base_fv[n];
      gamma_sum += T.r(n) - T.cur_fv[n];  // influence()
      ++psize;
    }
    const dtype fv_offset = floorAverage(comp_type(multFVScale(qii_sum, lambda)) + gamma_sum, psize);
    for (int64_t n : nodes) {
      const dtype off = fv_offset + ((pull_to_center && T.fv(n, lambda) > fv_offset) ? 1 : 0);
      T.setOffsetAndScale(n, off, lambda);
    }
  }

  dtype pushCap(int64_t n, int ei) const {
    const dtype a = T.P.alpha[size_t(n) * K + ei];
    return a > 0 ? a : 0;
  }

  // TV_PRFlow::getNeighborhoodKeySet (tv_push_relabel.hpp:367-391)
  std::set<uint32_t> neighborhoodKeys(const std::vector<int64_t>& nodes, uint32_t key) const {
    std::set<uint32_t> keys;
    for (int64_t n : nodes)
      for (int ei = 0; ei < K; ++ei) {
        const int64_t nn = n + T.P.L.jump[ei];
        if (T.key(nn) != key && pushCap(n, ei) + pushCap(nn, T.P.L.rev(ei)) > 0)
          keys.insert(T.key(nn));
      }
    return keys;
  }

  // TVRegPathSegment::lambdaOfJoin (tv_regpath_node.hpp:927-966)
  dtype lambdaOfJoin(int a, int b, dtype cur) const {
    const Seg& r1 = segs[a];
    const Seg& r2 = segs[b];
    if (r1.rhs_mode == Split && r2.rhs_mode == Split && r1.rhs_lambda == cur &&
        r2.rhs_lambda == cur)
      return -1;
    const dtype numer = r2.ar0 - r1.ar0;
    const dtype denom = (r1.ar1 - r1.ar0) - (r2.ar1 - r2.ar0);
    const dtype jl = ((numer < 0) != (denom < 0)) ? -1 : scaleFromQuotient(numer, denom);
    return (0 < jl && jl <= cur) ? jl : -1;
  }

  // TVRegPathSegment::calculateJoins (tv_regpath_node.hpp:968-992)
  dtype calculateJoins(int a, int b, dtype cur) {
    const dtype jl = lambdaOfJoin(a, b, cur);
    if (jl != -1) {
      segs[a].join_points.insert({jl, b});
      segs[b].join_points.insert({jl, a});
    }
    return jl;
  }

  // TVRegPathSegment::firstJoinPoint (tv_regpath_node.hpp:295-298).  For an
  // empty map the reference reads the map header, whose key slot is the
  // element count (0) in the standard library it is built with.
  dtype firstJoinPoint(const Seg& s) const {
    return s.join_points.empty() ? 0 : s.join_points.rbegin()->first;
  }

  // TVRegPathSegment::BisectionCheck (tv_regpath_node.hpp:416-455)
  DSI bisectionCheck(Seg& s, dtype lb, dtype ub) {
    int rate = 4;
    CutPtr best;
    bool occurred = false;
    while (lb + 1 < ub) {
      const dtype t = rate != 1 ? (lb + 1) + ((ub - (lb + 1)) / (dtype(1) << rate)) : (ub + lb) / 2;
      setRegionToLambda(s.ci_nodes, t, true);
      CutPtr cut = runPartitionedSection(s.ci_nodes, s.key);
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
    d.occurs = occurred;
    d.exact = occurred;
    d.lam = lb;
    d.cut = occurred ? best : nullptr;
    return d;
  }

  // TVRegPathSegment::_calculateSingleSplit (tv_regpath_node.hpp:457-633)
  DSI calculateSingleSplit(Seg& s, const dtype lambda_lb, const dtype lambda_ub) {
    setRegionToLambda(s.ci_nodes, lambda_lb, false);
    CutPtr cut = runPartitionedSection(s.ci_nodes, s.key);
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
    const RegionInfo p0 = regionInfo(cut->part[0]), p1 = regionInfo(cut->part[1]);
    const comp_type g0 = p0.gamma_sum - c, g1 = p1.gamma_sum + c;
    const comp_type q0 = p0.qii_sum, q1 = p1.qii_sum;
    const dtype sn = s0 + s1;
    const comp_type intercept = iabs((s1 * g0 - s0 * g1) + c * sn);
    const comp_type denom = iabs(q1 * s0 - q0 * s1);
    const dtype denom_pm = sn;
    dtype lb = scaleFromQuotient(intercept - comp_type(wmul(std::max(s1, s0), sn)), denom + denom_pm);
    dtype ub = scaleFromQuotient(intercept, denom - denom_pm);
    if (ub < lambda_lb) return bisectionCheck(s, lambda_lb, lambda_ub);
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
      if (s0 > 32) lmq0 = multFVScale(q0, lm);
      else for (int64_t n : cut->part[0]) lmq0 += T.fv(n, lm);
      if (s1 > 32) lmq1 = multFVScale(q1, lm);
      else for (int64_t n : cut->part[1]) lmq1 += T.fv(n, lm);
      const dtype fl_avg = floorAverage(gs + lmq0 + lmq1, long(sn));
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
  SplitInfo calculateSplit(int si, dtype cur) {
    Seg& s = segs[si];
    if (s.n_nodes == 1) {
      s.split_done_to = 0;
      s.lambda_of_split = -1;
      return {false, -1, 0};
    }
    dtype lambda_calc_lb = 0;
    for (auto it = s.join_points.begin(); it != s.join_points.end();) {
      const dtype join_lm = it->first;
      const int o = it->second;
      if (join_lm >= cur || segs[o].lhs_mode != Unset) {
        it = s.join_points.erase(it);
        continue;
      }
      if (join_lm == firstJoinPoint(segs[o])) lambda_calc_lb = std::max(join_lm, lambda_calc_lb);
      ++it;
    }
    DSI dsi, last;
    dtype lambda_calc = lambda_calc_lb;
    bool cut_exists = false;
    while (true) {
      dsi = calculateSingleSplit(s, lambda_calc, cur);
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
      s.split_info = last.cut;
      s.lambda_of_split = last.lam;
      return {true, lambda_calc, lambda_calc_lb};
    }
    s.split_done_to = lambda_calc_lb;
    s.lambda_of_split = -1;
    return {false, -1, lambda_calc_lb};
  }

  // TVRegPathSegment::applySplit (tv_regpath_node.hpp:747-814)
  void applySplit(int si, int d0, int d1, dtype lambda) {
    CutPtr cut = segs[si].split_info;
    applyPartitioningCut(*cut);
    const int dest[2] = {d0, d1};
    for (int i = 0; i < 2; ++i) {
      Seg& d = segs[dest[i]];
      d.ci_nodes = std::move(cut->part[i]);
      d.rhs_lambda = lambda;
      d.rhs_mode = Split;
      d.rhs_nodes[0] = si;
      d.rhs_nodes[1] = -1;
      syncInformation(d, lambda);
    }
    for (int i = 0; i < 2; ++i) {
      const std::set<uint32_t> keys = neighborhoodKeys(segs[dest[i]].ci_nodes, segs[dest[i]].key);
      for (uint32_t k : keys) {
        const int o = int(k) - 1;
        segs[o].neighbors.insert(dest[i]);
        segs[dest[i]].neighbors.insert(o);
      }
    }
    for (int o : segs[si].neighbors) segs[o].neighbors.erase(si);
    Seg& s = segs[si];
    s.lhs_lambda = lambda;
    s.lhs_mode = Split;
    s.lhs_nodes[0] = d0;
    s.lhs_nodes[1] = d1;
    if (segs[d0].ci_nodes.size() > segs[d1].ci_nodes.size()) std::swap(s.lhs_nodes[0], s.lhs_nodes[1]);
  }

  // TVRegPathSegment::setupFromJoin (tv_regpath_node.hpp:820-921), release build
  void setupFromJoin(int ni, int a, int b, dtype lambda) {
    Seg& n = segs[ni];
    Seg& r1 = segs[a];
    Seg& r2 = segs[b];
    n.ci_nodes.resize(r1.ci_nodes.size() + r2.ci_nodes.size());
    std::merge(r1.ci_nodes.begin(), r1.ci_nodes.end(), r2.ci_nodes.begin(), r2.ci_nodes.end(),
               n.ci_nodes.begin());
    n.rhs_mode = Join;
    n.rhs_lambda = lambda;
    n.rhs_nodes[0] = a;
    n.rhs_nodes[1] = b;
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
    r1.lhs_nodes[1] = -1;
    r2.lhs_mode = Join;
    r2.lhs_lambda = lambda;
    r2.lhs_nodes[0] = ni;
    r2.lhs_nodes[1] = -1;
    syncInformation(n, lambda);
  }

  // TVRegPathSegment::deactivate (tv_regpath_node.hpp:300-373)
  void deactivate(int si) {
    Seg& s = segs[si];
    if (s.rhs_mode == Split || s.rhs_mode == Initial) {
      s.nodeset.swap(s.ci_nodes);
      std::sort(s.nodeset.begin(), s.nodeset.end());
    }
    s.active = false;
    std::set<int>().swap(s.neighbors);
    std::multimap<dtype, int>().swap(s.join_points);
    std::vector<int64_t>().swap(s.ci_nodes);
    s.split_info.reset();
  }

  // TVSolver::run + _constructInitialRegPathsFromSolvedLattice (tv_solver.hpp:114-136,300-564)
  void run() {
    const dtype solved_lambda = toScaleDType(1);
    std::vector<std::vector<int64_t>> level_sets;
    run_pf(T.P, &level_sets);
    node_map.assign(size_t(T.P.L.size_all), -1);
    std::vector<int> initial;
    for (auto& nv : level_sets) {
      const int si = newSeg();
      Seg& s = segs[si];
      s.ci_nodes = nv;
      s.rhs_lambda = solved_lambda;
      s.rhs_mode = Initial;
      syncInformation(s, solved_lambda);
      initial.push_back(si);
      for (int64_t n : nv) {
        T.P.nodes[n].key_state = s.key << 1;
        node_map[size_t(n)] = si;
      }
    }
    // TV_PRFlow::constructNeighborhoodKeyPairs (tv_push_relabel.hpp:339-365)
    {
      std::unordered_set<uint64_t> seen;
      auto gen_key = [](uint32_t k1, uint32_t k2) {
        return (uint64_t(std::min(k1, k2)) << 32) | uint64_t(std::max(k1, k2));
      };
      const Lattice& L = T.P.L;
      for (int64_t n = L.begin; n < L.end; ++n) {
        seen.insert(gen_key(T.key(n), T.key(n)));
        for (int ei = 0; ei < K / 2; ++ei) {
          const int64_t nn = n + L.jump[ei];
          if (pushCap(n, ei) + pushCap(nn, L.rev(ei)) > 0 &&
              seen.insert(gen_key(T.key(n), T.key(nn))).second) {
            const int a = node_map[size_t(n)], b = node_map[size_t(nn)];
            segs[a].neighbors.insert(b);
            segs[b].neighbors.insert(a);
          }
        }
      }
    }
    std::priority_queue<FunPoint> heap;
    auto registerPossibleJoin = [&](int a, int b, dtype lambda_start) {
      const dtype jl = calculateJoins(a, b, lambda_start);
      if (jl > 0) heap.push(FunPoint{jl, EvJoin, a, b});
    };
    auto registerPossibleSplit = [&](int a, dtype lambda_start) {
      const SplitInfo sp = calculateSplit(a, lambda_start);
      if (sp.occurs) heap.push(FunPoint{sp.split_lambda, EvSplit, a, -1});
      else if (sp.split_ub != 0) heap.push(FunPoint{sp.split_ub, EvSplitUB, a, -1});
    };
    for (int a : initial) {
      const std::set<int> nb = segs[a].neighbors;
      for (int b : nb)
        if (a < b) registerPossibleJoin(a, b, solved_lambda);
    }
    for (int a : initial) registerPossibleSplit(a, solved_lambda);
    auto activateNewLine = [&](int a, dtype lambda_start) {
      const std::set<int> nb = segs[a].neighbors;
      for (int b : nb) registerPossibleJoin(a, b, lambda_start);
      registerPossibleSplit(a, lambda_start);
    };
    while (!heap.empty()) {
      const FunPoint fp = heap.top();
      heap.pop();
      const dtype cur = fp.lambda;
      if (segs[fp.r1].lhs_mode != Unset || (fp.r2 >= 0 && segs[fp.r2].lhs_mode != Unset))
        continue;
      switch (fp.mode) {
        case EvJoin: {
          const int ni = newSeg();
          setupFromJoin(ni, fp.r1, fp.r2, cur);
          deactivate(fp.r1);
          deactivate(fp.r2);
          activateNewLine(ni, cur);
          break;
        }
        case EvSplit: {
          const int d0 = newSeg();
          const int d1 = newSeg();
          applySplit(fp.r1, d0, d1, cur);
          deactivate(fp.r1);
          activateNewLine(d0, cur);
          activateNewLine(d1, cur);
          break;
        }
        case EvSplitUB:
          registerPossibleSplit(fp.r1, cur);
          break;
      }
    }
    Seg& last = segs.back();
    last.lhs_lambda = 0;
    last.lhs_mode = Initial;
    deactivate(int(segs.size()) - 1);
    calculated_lambda = solved_lambda;
  }

  // TVSolver::traceRegularizationPath (tv_solver.hpp:566-642)
  void trace(int64_t n, const std::vector<dtype>& lambdas, std::vector<dtype>& out) {
    int cur = node_map[size_t(n)];
    size_t idx = 0;
    out.assign(lambdas.size(), 0);
    if (lambdas.empty() || cur < 0) return;
    for (;;) {
      while (segs[cur].lhs_lambda > lambdas[idx]) {
        const Seg& s = segs[cur];
        int nxt;
        if (s.lhs_mode == Split) {
          const int a = s.lhs_nodes[0], b = s.lhs_nodes[1];
          const auto& ns = segs[a].nodeset;
          nxt = std::binary_search(ns.begin(), ns.end(), n) ? a : b;
        } else {
          nxt = s.lhs_nodes[0];
        }
        if (nxt < 0) { broken = true; return; }
        cur = nxt;
      }
      while (segs[cur].lhs_lambda <= lambdas[idx]) {
        out[idx] = rAtLambda(segs[cur], lambdas[idx]);
        if (++idx == lambdas.size()) return;
      }
    }
  }

  // TVSolver::getRegularizationPath (tv_solver.hpp:174-244); out[n_lambda][nx][ny]
  int path(const double* lams, size_t n_lambda, double* out) {
    struct LambdaIdx {
      dtype value;
      size_t index;
      bool operator<(const LambdaIdx& o) const { return value > o.value; }
    };
    std::vector<LambdaIdx> li(n_lambda);
    std::vector<dtype> calc(n_lambda);
    for (size_t i = 0; i < n_lambda; ++i) li[i] = {toScaleDType(lams[i] / T.max_lambda), i};
    std::sort(li.begin(), li.end());
    for (size_t i = 0; i < n_lambda; ++i) calc[i] = li[i].value;
    if (calculated_lambda == -1 || calc.front() > calculated_lambda || calc.back() < 0) return -3;
    const int64_t N = T.P.L.n_bounded();
    std::vector<double> sums(n_lambda, 0);
    std::vector<dtype> pv;
    for (int64_t b = 0; b < N; ++b) {
      trace(T.P.L.padded(b), calc, pv);
      for (size_t i = 0; i < n_lambda; ++i) {
        const double v = T.toFValue(pv[i]);
        out[li[i].index * size_t(N) + size_t(b)] = v;
        sums[li[i].index] += v;
      }
    }
    for (size_t i = 0; i < n_lambda; ++i) {
      const double mean = sums[i] / double(N);
      for (int64_t b = 0; b < N; ++b) {
        double& v = out[i * size_t(N) + size_t(b)];
        v = (v - mean) * T.fscale + T.fmean;
      }
    }
    return broken ? -4 : 0;
  }
};

}  // namespace

extern "C" {

// Plain cut with the push-relabel restatement.  offsets: K*nd in lattice order
// (positive half ascending, then reverses).  cut_out[N]: 1 = on (partition 1).
int lfo_pr_solve(int nd, const int64_t* dims, int K, const int* offsets,
                 const int64_t* unary, const int64_t* binary, int32_t* cut_out,
                 double* seconds) {
  Problem P;
  P.init(nd, dims, K, offsets);
  P.fill(unary, binary);
  auto t0 = std::chrono::steady_clock::now();
  PR pr(P.L, P.nodes, P.alpha);
  pr.run();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  int64_t N = P.L.n_bounded();
  for (int64_t b = 0; b < N; ++b) cut_out[b] = (P.nodes[P.L.padded(b)].key_state & 1u) ? 1 : 0;
  return 0;
}

// Plain cut plus both canonical cut sets.  After the restated solve every
// flip is undone (flipping twice is the identity, network_flow_node.hpp:325-326),
// which leaves alpha[n][i] = residual capacity n -> n+jump[i] (2x units) and
// -reduction = excess.  cut_min = forward residual closure of excess nodes
// (the unique minimal on-set), cut_max = complement of the backward closure
// of deficit nodes (the unique maximal on-set).  cut_pr = the reference's own
// labelling (state bit), which is some minimum cut between the two.
int lfo_pr_canonical(int nd, const int64_t* dims, int K, const int* offsets,
                     const int64_t* unary, const int64_t* binary, int32_t* cut_pr,
                     int32_t* cut_min, int32_t* cut_max, double* seconds) {
  Problem P;
  P.init(nd, dims, K, offsets);
  P.fill(unary, binary);
  auto t0 = std::chrono::steady_clock::now();
  PR pr(P.L, P.nodes, P.alpha);
  pr.run();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  const Lattice& L = P.L;
  int64_t N = L.n_bounded();
  std::vector<int64_t> pad(static_cast<size_t>(N));
  for (int64_t b = 0; b < N; ++b) {
    pad[b] = L.padded(b);
    cut_pr[b] = (P.nodes[pad[b]].key_state & 1u) ? 1 : 0;
  }
  for (int64_t p = L.begin; p < L.end; ++p)
    if (P.nodes[p].key_state & 1u) pr.nodeFlip(p, 1);
  std::vector<uint8_t> inb(size_t(L.size_all), 0), mark(size_t(L.size_all), 0);
  for (int64_t b = 0; b < N; ++b) inb[pad[b]] = 1;
  std::vector<int64_t> stack;
  // forward closure of excess nodes
  for (int64_t b = 0; b < N; ++b)
    if (P.nodes[pad[b]].reduction < 0) { mark[pad[b]] = 1; stack.push_back(pad[b]); }
  while (!stack.empty()) {
    int64_t n = stack.back(); stack.pop_back();
    for (int i = 0; i < K; ++i) {
      int64_t m = n + L.jump[i];
      if (inb[m] && !mark[m] && P.alpha[size_t(n) * K + i] > 0) { mark[m] = 1; stack.push_back(m); }
    }
  }
  for (int64_t b = 0; b < N; ++b) cut_min[b] = mark[pad[b]];
  // backward closure of deficit nodes
  std::fill(mark.begin(), mark.end(), 0);
  for (int64_t b = 0; b < N; ++b)
    if (P.nodes[pad[b]].reduction > 0) { mark[pad[b]] = 1; stack.push_back(pad[b]); }
  while (!stack.empty()) {
    int64_t n = stack.back(); stack.pop_back();
    for (int i = 0; i < K; ++i) {
      int64_t m = n + L.jump[i];  // edge m -> n has index rev(i) at m
      if (inb[m] && !mark[m] && P.alpha[size_t(m) * K + L.rev(i)] > 0) { mark[m] = 1; stack.push_back(m); }
    }
  }
  for (int64_t b = 0; b < N; ++b) cut_max[b] = mark[pad[b]] ? 0 : 1;
  return 0;
}

// Parametric flow over the filled lattice (LatticeLevelReductions).  r_out[N]
// receives the final 2x-scaled reductions, cut_out[N] = (reduction < 0)
// (network_flow_node.hpp:50-55 with on_by_reduction), sets_out[N] (may be
// NULL) the index of every node's level set in the order run() returns them.
int lfo_pf_solve(int nd, const int64_t* dims, int K, const int* offsets,
                 const int64_t* unary, const int64_t* binary, int64_t* r_out,
                 int32_t* cut_out, double* seconds, int32_t* sets_out) {
  Problem P;
  P.init(nd, dims, K, offsets);
  P.fill(unary, binary);
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::vector<int64_t>> level_sets;
  run_pf(P, &level_sets);
  if (sets_out) {
    std::vector<int32_t> id(size_t(P.L.size_all), -1);
    for (size_t i = 0; i < level_sets.size(); ++i)
      for (int64_t p : level_sets[i]) id[size_t(p)] = int32_t(i);
    const int64_t N = P.L.n_bounded();
    for (int64_t b = 0; b < N; ++b) sets_out[b] = id[size_t(P.L.padded(b))];
  }
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  int64_t N = P.L.n_bounded();
  for (int64_t b = 0; b < N; ++b) {
    int64_t p = P.L.padded(b);
    if (r_out) r_out[b] = P.r(p);
    if (cut_out) cut_out[b] = P.nodes[p].reduction < 0 ? 1 : 0;
  }
  return 0;
}

// TVSolver<Kernel, int64>::runSingleLambda (tv_solver.hpp:71-112,151-176).
// weights: geocut weights in lattice order.  out[N] doubles, r_out[N] raw r(),
// sets_out[N] (may be NULL) the level set of every node (run()'s order).
int lfo_tv_single(int64_t nx, int64_t ny, int K, const int* offsets, const double* weights,
                  const double* f, double lam, double* out, int64_t* r_out, double* seconds,
                  int32_t* sets_out) {
  const int nbits = 40;  // n_bits_function_precision for int64 (pf_flow_node.hpp:111-113)
  const double fscale = double(int64_t(1) << nbits);
  Problem P;
  int64_t dims[2] = {nx, ny};
  P.init(2, dims, K, offsets);
  int64_t N = nx * ny;
  auto t0 = std::chrono::steady_clock::now();
  double v_min = f[0], v_max = f[0], v_sum = f[0];
  for (int64_t i = 1; i < N; ++i) {
    v_min = std::min(v_min, f[i]);
    v_max = std::max(v_max, f[i]);
    v_sum += f[i];
  }
  double mean = v_sum / double(N);
  v_min -= mean;
  v_max -= mean;
  double scale = 2 * std::max(v_max, -v_min);
  double max_lambda = std::max(lam, 1e-8);
  for (int64_t b = 0; b < N; ++b) {
    double v = 0.5 + (f[b] - mean) / scale;
    dtype uf = dtype(std::round(v * fscale));
    P.addE1(P.L.padded(b), 0, uf);
  }
  double gsv = 0.5 / (scale * max_lambda);
  int Kp = K / 2;
  for (int64_t b = 0; b < N; ++b) {
    int64_t p = P.L.padded(b);
    for (int e = 0; e < Kp; ++e) {
      if (!P.L.within(p + P.L.jump[e])) continue;
      dtype pwf = dtype(std::round((gsv * weights[e]) / scale * fscale));
      P.addE2(p, e, 0, pwf, pwf, 0);
    }
  }
  std::vector<std::vector<int64_t>> level_sets;
  run_pf(P, &level_sets);
  if (sets_out) {
    std::vector<int32_t> id(size_t(P.L.size_all), -1);
    for (size_t i = 0; i < level_sets.size(); ++i)
      for (int64_t p : level_sets[i]) id[size_t(p)] = int32_t(i);
    for (int64_t b = 0; b < N; ++b) sets_out[b] = id[size_t(P.L.padded(b))];
  }
  double sum = 0;
  std::vector<double> R(static_cast<size_t>(N));
  for (int64_t b = 0; b < N; ++b) {
    dtype r = P.r(P.L.padded(b));
    if (r_out) r_out[b] = r;
    double x = double(r / 2) / fscale;      // Node::toFValue(translateFromRaw(r))
    double v = (x - 0.5) * scale + mean;    // TVSolver::toFValue (tv_solver.hpp:281-285)
    R[b] = v;
    sum += v;
  }
  for (int64_t b = 0; b < N; ++b) out[b] = (R[b] - sum / double(N)) * scale + mean;
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  return 0;
}

}  // extern "C"

extern "C" {

// calculate2dTV<Kernel, int64>(nx, ny, f, vector<double> lambdas)
// (tv/tv_solver.hpp:657-681): the reference's regularisation path, out[n][nx][ny].
// Negative lambdas count as 0; n_lambda = 0 returns at once.  Returns 0, or
// -3 when the lambdas are outside the computed range (std::out_of_range in
// the reference), -4 when a trace met a segment without a successor.
// stats (may be NULL): [0] segments, [1] region probes.
int lfo_tv_path(int64_t nx, int64_t ny, int K, const int* offsets, const double* weights,
                const double* f, int64_t n_lambda, const double* lambdas, double* out,
                double* seconds, int64_t* stats) {
  if (n_lambda <= 0) return 0;
  std::vector<double> lams(lambdas, lambdas + n_lambda);
  for (double& l : lams) if (l < 0) l = 0;
  auto t0 = std::chrono::steady_clock::now();
  TVLattice T;
  T.setup(nx, ny, K, offsets, weights, f, *std::max_element(lams.begin(), lams.end()));
  TVPath tp(T);
  tp.run();
  const int rc = tp.path(lams.data(), lams.size(), out);
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (stats) {
    stats[0] = int64_t(tp.segs.size());
    stats[1] = 0;
  }
  return rc;
}

}  // extern "C"
