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
#include <deque>
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
// (pf_flow_node.hpp:330-396).  Leaves final r() values in the lattice.
void run_pf(Problem& P) {
  PR pr(P.L, P.nodes, P.alpha);
  std::vector<int64_t> pts;
  for (int64_t p = P.L.begin; p < P.L.end; ++p)
    if (P.L.within(p)) pts.push_back(p);
  struct Range { size_t s, e; };
  std::deque<Range> q;
  uint32_t key = 1;
  q.push_back({0, pts.size()});
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
    pr.cleanupSection(b, e);
    ++key;
  }
  for (int64_t p : pts) P.setOffset(p, 0);
}

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
// (network_flow_node.hpp:50-55 with on_by_reduction).
int lfo_pf_solve(int nd, const int64_t* dims, int K, const int* offsets,
                 const int64_t* unary, const int64_t* binary, int64_t* r_out,
                 int32_t* cut_out, double* seconds) {
  Problem P;
  P.init(nd, dims, K, offsets);
  P.fill(unary, binary);
  auto t0 = std::chrono::steady_clock::now();
  run_pf(P);
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
// weights: geocut weights in lattice order.  out[N] doubles, r_out[N] raw r().
int lfo_tv_single(int64_t nx, int64_t ny, int K, const int* offsets, const double* weights,
                  const double* f, double lam, double* out, int64_t* r_out, double* seconds) {
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
  run_pf(P);
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
