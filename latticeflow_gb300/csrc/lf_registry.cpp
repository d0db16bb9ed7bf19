// Kernel (neighbourhood) registry.
//
// Restates the rules of the reference's kernel generator
// (install/code_setup.py) as a table built once at load time:
//   * radius list: distinct norms of integer vectors with coordinates in
//     [0, R], 0 < norm <= R + 1e-8 (code_setup.py:84-88); R = 4 in 2-d and
//     R = 2 in 3-d (wscript:54-64, code_setup.py:13);
//   * Full: offsets x with 0 < |x|^2 <= radius^2 in double arithmetic, so the
//     3-d corners are not produced at radius sqrt(3) (code_setup.py:200-222);
//   * Star: Full minus every offset whose direction tuple
//     (atan2(x1, x0), atan2(x2, x0), ...) already appeared on a shorter offset
//     (code_setup.py:224-263);
//   * 2-d geocut weights: half the angle between the two angular neighbours
//     divided by 2|x| (code_setup.py:163-197), each weight paired with its own
//     offset;
//   * names "%s%dd_%d" (code_setup.py:40); a repeated offset set becomes an
//     alias of the first kernel that produced it (code_setup.py:369-399);
//   * the 1-d kernels of the reference's opt-in 1-d build (Full only, integer
//     radii 1 .. 7, code_setup.py:81-92).
// "Full3d_26" names the 3x3x3 neighbourhood (produced by the Star rule at
// radius 2 as "Star3d_26").
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "lf_internal.h"

namespace lfg {
namespace {

typedef std::vector<int> Vec;

std::vector<double> radius_list(int dim, int R) {
  std::set<double> vals;
  std::vector<int> c(dim, 0);
  for (;;) {
    long s = 0;
    for (int v : c) s += long(v) * v;
    vals.insert(std::sqrt(double(s)));
    int i = dim - 1;
    while (i >= 0 && c[i] == R) { c[i] = 0; --i; }
    if (i < 0) break;
    ++c[i];
  }
  std::vector<double> out;
  for (double d : vals)
    if (d > 0 && d <= R + 1e-8) out.push_back(d);
  return out;
}

std::vector<Vec> full_offsets(int dim, double radius) {
  int lo = int(std::floor(-radius)), hi = int(std::ceil(radius));
  std::vector<Vec> out;
  Vec c(dim, lo);
  for (;;) {
    long s = 0;
    for (int v : c) s += long(v) * v;
    if (s > 0 && double(s) <= radius * radius) out.push_back(c);
    int i = dim - 1;
    while (i >= 0 && c[i] == hi) { c[i] = lo; --i; }
    if (i < 0) break;
    ++c[i];
  }
  std::sort(out.begin(), out.end());
  return out;
}

long norm2(const Vec& v) { long s = 0; for (int x : v) s += long(x) * x; return s; }

std::vector<Vec> star_offsets(int dim, double radius) {
  std::vector<Vec> full = full_offsets(dim, radius);
  std::vector<Vec> by_len = full;
  std::stable_sort(by_len.begin(), by_len.end(),
                   [](const Vec& a, const Vec& b) { return norm2(a) < norm2(b); });
  std::set<std::vector<double>> seen;
  std::vector<Vec> keep;
  for (const Vec& e : by_len) {
    std::vector<double> ang;
    for (int i = 1; i < dim; ++i) ang.push_back(std::atan2(double(e[i]), double(e[0])));
    if (seen.count(ang)) continue;
    seen.insert(ang);
    keep.push_back(e);
  }
  std::sort(keep.begin(), keep.end());
  return keep;
}

bool geocut_weights(int dim, const std::vector<Vec>& edges, std::vector<double>& w) {
  w.assign(edges.size(), 1.0);
  if (dim != 2 || edges.size() < 4) return false;
  const double two_pi = 2 * M_PI;
  std::vector<std::pair<double, size_t>> info;
  std::set<double> uniq;
  for (size_t i = 0; i < edges.size(); ++i) {
    double a = std::fmod(std::atan2(double(edges[i][1]), double(edges[i][0])), two_pi);
    if (a < 0) a += two_pi;  // Python's % on floats is non-negative for a positive divisor
    info.push_back({a, i});
    uniq.insert(a);
  }
  if (uniq.size() != edges.size()) return false;
  std::sort(info.begin(), info.end(), [&](const std::pair<double, size_t>& x,
                                          const std::pair<double, size_t>& y) {
    if (x.first != y.first) return x.first < y.first;
    return edges[x.second] < edges[y.second];
  });
  size_t n = info.size();
  for (size_t i = 0; i < n; ++i) {
    double a1 = info[(i + n - 1) % n].first;
    double a2 = info[(i + 1) % n].first;
    if (a2 < a1) a2 += two_pi;
    double width = (a2 - a1) / 2;
    const Vec& e = edges[info[i].second];
    w[info[i].second] = width / (2.0 * std::sqrt(double(e[0] * e[0] + e[1] * e[1])));
  }
  return true;
}

// Put (offsets, weights) of a kernel into lattice order.
void to_lattice_order(const std::vector<Vec>& offs, const std::vector<double>& w, KernelDef& k) {
  std::vector<std::pair<Vec, double>> pos;
  for (size_t i = 0; i < offs.size(); ++i) {
    Vec zero(offs[i].size(), 0);
    if (offs[i] > zero) pos.push_back({offs[i], w[i]});
  }
  std::sort(pos.begin(), pos.end());
  std::map<Vec, double> wmap;
  for (size_t i = 0; i < offs.size(); ++i) wmap[offs[i]] = w[i];
  k.K = int(offs.size());
  k.delta.clear();
  k.weight.clear();
  for (auto& p : pos) { for (int v : p.first) k.delta.push_back(v); k.weight.push_back(p.second); }
  for (auto& p : pos) {
    Vec r = p.first;
    for (int& v : r) v = -v;
    for (int v : r) k.delta.push_back(v);
    k.weight.push_back(wmap[r]);
  }
}

std::vector<KernelDef> build_registry() {
  std::vector<KernelDef> out;
  std::map<std::set<Vec>, std::string> seen_sets;
  std::set<std::string> names;
  // The reference's opt-in 1-d build (--1d, wscript:49-67): Full kernels at
  // the integer radii 1 .. 7 (code_setup.py:81-92), Full1d_2 .. Full1d_14.
  for (int r = 1; r < 8; ++r) {
    std::vector<Vec> offs = full_offsets(1, double(r));
    char buf[64];
    std::snprintf(buf, sizeof(buf), "Full1d_%d", int(offs.size()));
    KernelDef k;
    k.name = buf;
    k.nd = 1;
    std::vector<double> w;
    k.geocut = geocut_weights(1, offs, w);
    to_lattice_order(offs, w, k);
    seen_sets[std::set<Vec>(offs.begin(), offs.end())] = k.name;
    names.insert(k.name);
    out.push_back(k);
  }
  const int max_r[4] = {0, 0, 4, 2};
  for (int dim = 2; dim <= 3; ++dim) {
    for (double r : radius_list(dim, max_r[dim])) {
      for (int kind = 0; kind < 2; ++kind) {
        std::vector<Vec> offs = kind == 0 ? full_offsets(dim, r) : star_offsets(dim, r);
        if (offs.empty()) continue;
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%s%dd_%d", kind == 0 ? "Full" : "Star", dim,
                      int(offs.size()));
        std::string name(buf);
        std::set<Vec> key(offs.begin(), offs.end());
        if (names.count(name)) continue;
        auto it = seen_sets.find(key);
        KernelDef k;
        k.name = name;
        k.nd = dim;
        if (it != seen_sets.end()) {
          for (const KernelDef& b : out)
            if (b.name == it->second) { k = b; break; }
          k.name = name;
          k.alias_of = it->second;
        } else {
          std::vector<double> w;
          k.geocut = geocut_weights(dim, offs, w);
          to_lattice_order(offs, w, k);
          seen_sets[key] = name;
        }
        names.insert(name);
        out.push_back(k);
      }
    }
  }
  // 3x3x3 neighbourhood under the name used by the 3-d volume workloads
  std::vector<Vec> n26;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c)
        if (a || b || c) n26.push_back({a, b, c});
  std::set<Vec> key26(n26.begin(), n26.end());
  auto it = seen_sets.find(key26);
  if (it != seen_sets.end()) {
    for (const KernelDef& b : out)
      if (b.name == it->second) {
        KernelDef k = b;
        k.name = "Full3d_26";
        k.alias_of = b.name;
        out.push_back(k);
        break;
      }
  }
  return out;
}

}  // namespace

const std::vector<KernelDef>& kernel_registry() {
  static std::vector<KernelDef> reg = build_registry();
  return reg;
}

const KernelDef* find_kernel(const std::string& name) {
  for (const KernelDef& k : kernel_registry())
    if (k.name == name) return &k;
  return nullptr;
}

const std::vector<std::string>& solver_names() {
  static std::vector<std::string> s = {"LatticeEnergyMinimizer", "LatticeLevelReductions",
                                       "GPUPushRelabel", "GPULevelReductions"};
  return s;
}

}  // namespace lfg
