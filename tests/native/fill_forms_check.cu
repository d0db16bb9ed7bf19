// Host check of the gathered energy fill (lf_fill.cuh): for every kernel of
// the registry and random lattices (2-d and 3-d, single rows, ragged edges),
// the per-node form and the per-edge (lane) composition give the same
// accumulators, constant term and submodularity flag as the scattered form,
// restated here on the host (k_fill_energy in lf_kernels.cu: one pass per
// filling edge adding into both ends).  Exit status 0 = all equal.
#include <cstdio>
#include <random>
#include <vector>

#include "lf_fill.cuh"
#include "lf_internal.h"

using namespace lfg;

static Stencil stencil_of(const KernelDef& kd) {  // the engine's make_stencil rule
  Stencil st{};
  st.K = kd.K;
  for (int i = 0; i < st.K; ++i) {
    st.da[i] = (signed char)(kd.nd == 3 ? kd.delta[i * kd.nd] : 0);
    st.db[i] = (signed char)kd.delta[i * kd.nd + (kd.nd == 3 ? 1 : 0)];
    st.dc[i] = (signed char)kd.delta[i * kd.nd + (kd.nd == 3 ? 2 : 1)];
    st.rev[i] = (unsigned char)(i < st.K / 2 ? i + st.K / 2 : i - st.K / 2);
  }
  return st;
}

static void coords(int nd, const Geo& g, long long r, int& a, int& b, int& c) {
  if (nd == 2) { a = 0; b = int(r / g.C); c = int(r % g.C); }
  else { c = int(r % g.C); b = int((r / g.C) % g.B); a = int(r / ((long long)g.C * g.B)); }
}

int main() {
  std::mt19937_64 rng(7);
  int cases = 0, fails = 0;
  for (const KernelDef& kd : kernel_registry()) {
    if (kd.K > kMaxKDev) continue;
    for (int trial = 0; trial < 3; ++trial) {
      Geo g{};
      g.A = kd.nd == 3 ? 1 + int(rng() % 7) : 1;
      g.B = trial == 2 ? 1 : 1 + int(rng() % 19);
      g.C = 1 + int(rng() % 45);
      g.Ap = kd.nd == 3 ? (g.A + 3) / 4 * 4 : 1;
      g.Bp = kd.nd == 3 ? (g.B + 7) / 8 * 8 : (g.B + 31) / 32 * 32;
      g.Cp = (g.C + 31) / 32 * 32;
      g.NP = (long long)g.Ap * g.Bp * g.Cp;
      const Stencil st = stencil_of(kd);
      const int Kp = st.K / 2;
      const long long N = (long long)g.A * g.B * g.C;
      std::vector<int64_t> un(2 * N), bi(N * Kp * 4);
      for (auto& v : un) v = (int64_t)(rng() % 2001) - 1000;
      for (long long i = 0; i < N * Kp; ++i) {
        int64_t A = int64_t(rng() % 1001) - 500, D = int64_t(rng() % 1001) - 500;
        int64_t B = int64_t(rng() % 1001) - 500, C = int64_t(rng() % 1001) - 500;
        if (rng() % 5 == 0) { B = A; C = D; }  // zero capacities
        bi[4 * i] = A; bi[4 * i + 1] = B; bi[4 * i + 2] = C; bi[4 * i + 3] = D;
      }
      std::vector<long long> e0(g.NP), c0v(g.NP * st.K);
      for (auto& v : e0) v = (long long)(rng() % 100);
      for (auto& v : c0v) v = (long long)(rng() % 100);
      // scattered form
      std::vector<long long> es = e0, cs = c0v;
      long long ks = 0;
      bool bs = false;
      for (long long t = 0; t < N * Kp; ++t) {
        const long long r = t / Kp;
        const int e = int(t % Kp);
        int a, b, c;
        coords(kd.nd, g, r, a, b, c);
        const long long u = ((long long)a * g.Bp + b) * g.Cp + c;
        if (e == 0) { es[u] += un[2 * r] - un[2 * r + 1]; ks += un[2 * r]; }
        const int na = a + st.da[e], nb = b + st.db[e], nc = c + st.dc[e];
        if (na < 0 || na >= g.A || nb < 0 || nb >= g.B || nc < 0 || nc >= g.C) continue;
        const long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
        const int64_t* q = &bi[(r * Kp + e) * 4];
        ks += q[0];
        long long du = q[0] - q[3], dv = 0;
        const long long Bq = q[1] - q[0], Cq = q[2] - q[3];
        if (Bq + Cq < 0) bs = true;
        if (Bq < 0) { dv -= Bq; du += Bq; cs[e * g.NP + u] += Bq + Cq; }
        else if (Cq < 0) { du -= Cq; dv += Cq; cs[st.rev[e] * g.NP + v] += Bq + Cq; }
        else { cs[e * g.NP + u] += Cq; cs[st.rev[e] * g.NP + v] += Bq; }
        es[u] += du;
        es[v] += dv;
      }
      // per-node form
      std::vector<long long> en = e0, cn = c0v;
      long long kn = 0;
      bool bn = false;
      for (long long r = 0; r < N; ++r) {
        int a, b, c;
        coords(kd.nd, g, r, a, b, c);
        kn += fill_gather_node<false>(g, st, r, a, b, c, un.data(), bi.data(), en.data(), cn.data(), &bn);
      }
      // lane form: edge shares in lane order, summed per node, lane 0 writes
      std::vector<long long> el = e0, cl = c0v;
      long long kl = 0;
      bool bl = false;
      for (long long r = 0; r < N; ++r) {
        int a, b, c;
        coords(kd.nd, g, r, a, b, c);
        const long long w = ((long long)a * g.Bp + b) * g.Cp + c;
        long long x = 0;
        for (int e = 0; e < Kp; ++e) {
          x += fill_gather_edge<false>(g, st, r, a, b, c, w, e, bi.data(), cl.data(), &bl, &kl);
          if (e == 0) x += fill_gather_unary<false>(un.data(), r, &kl);
        }
        if (x) el[w] += x;
      }
      ++cases;
      const bool ok = en == es && cn == cs && kn == ks && bn == bs && el == es && cl == cs &&
                      kl == ks && bl == bs;
      if (!ok) {
        ++fails;
        std::printf("mismatch: %s %dx%dx%d\n", kd.name.c_str(), g.A, g.B, g.C);
      }
    }
  }
  std::printf("%d cases, %d mismatches\n", cases, fails);
  return fails != 0 || cases == 0;
}
