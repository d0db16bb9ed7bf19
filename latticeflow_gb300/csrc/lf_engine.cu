// Host orchestration of one lattice solve.
//
// run() = reference LatticeEnergyBase::run + PRFlow::run
// (energy_minimization/energy_base.hpp:137-148, network_flow/push_relabel.hpp:1303-1354):
//   repeat { global relabel (BFS from the deficit nodes; unreachable nodes get
//            kHInf, the reference's flip); stop when no node with excess has a
//            finite height; otherwise run a batch of tile push/relabel launches }
// then the two canonical cut sets are read off the final residual graph.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <mutex>

#include "lf_engine.h"

namespace lfg {

void Engine::check(cudaError_t e, const char* what) const {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? 5 : 6;
    throw LfError{code, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (!n) n = 1;
  }
  return n;
}

Engine::Engine(const std::string& solver, const KernelDef* k, int _nd, const size_t* d)
    : solver_name(solver), kernel_name(k->name), kd(k), nd(_nd) {
  parametric = (solver == "LatticeLevelReductions" || solver == "GPULevelReductions");
  dims.assign(d, d + nd);
  N = 1;
  for (size_t v : dims) N *= (long long)v;
  if (nd != 2 && nd != 3) throw LfError{2, "only 2-d and 3-d lattices are supported"};
  for (size_t v : dims)
    if (v > (size_t)INT_MAX / 2) throw LfError{2, "lattice extent too large"};
  st.K = kd->K;
  st.HA = st.HB = st.HC = 0;
  for (int i = 0; i < st.K; ++i) {
    int a = nd == 3 ? kd->delta[i * nd + 0] : 0;
    int b = kd->delta[i * nd + (nd == 3 ? 1 : 0)];
    int c = kd->delta[i * nd + (nd == 3 ? 2 : 1)];
    st.da[i] = (signed char)a;
    st.db[i] = (signed char)b;
    st.dc[i] = (signed char)c;
    st.rev[i] = (unsigned char)(i < st.K / 2 ? i + st.K / 2 : i - st.K / 2);
    st.HA = std::max(st.HA, std::abs(a));
    st.HB = std::max(st.HB, std::abs(b));
    st.HC = std::max(st.HC, std::abs(c));
  }
  g.A = nd == 3 ? int(dims[0]) : 1;
  g.B = int(dims[nd == 3 ? 1 : 0]);
  g.C = int(dims[nd == 3 ? 2 : 1]);
  choose_geometry(4);
  check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  check(cudaEventCreate(&ev0), "cudaEventCreate");
  check(cudaEventCreate(&ev1), "cudaEventCreate");
  check(cudaMallocHost(&h_pinned, 64), "cudaMallocHost");
}

void Engine::free_working() {
  cudaFree(d_res); d_res = nullptr;
  cudaFree(d_exc); d_exc = nullptr;
  cudaFree(d_h); d_h = nullptr;
  cudaFree(d_mask); d_mask = nullptr;
  cudaFree(d_mark); d_mark = nullptr;
  for (int i = 0; i < 2; ++i) {
    cudaFree(d_act[i]); d_act[i] = nullptr;
    cudaFree(d_dirty[i]); d_dirty[i] = nullptr;
  }
}

Engine::~Engine() {
  if (stream) cudaStreamSynchronize(stream);
  for (cudaEvent_t e : pev) cudaEventDestroy(e);
  free_working();
  cudaFree(d_exc64);
  cudaFree(d_cap64);
  cudaFree(d_c0);
  cudaFree(d_err);
  cudaFree(d_flag);
  cudaFree(d_u64);
  cudaFree(d_sum);
  cudaFree(d_kmask);
  if (h_pinned) cudaFreeHost(h_pinned);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (stream) cudaStreamDestroy(stream);
}

// Padding is fixed at construction (multiples of the largest tile, so every
// smaller power-of-two tile also divides it); the tile extents are chosen per
// working element size: TC = 32 (one warp per row), 2-d: TA = 1 and TB rows,
// 3-d: TA x TB; the largest tile whose shared-memory footprint fits is used.
void Engine::choose_geometry(int elem) {
  if (g.Cp == 0) {
    g.Ap = nd == 3 ? (g.A + 3) / 4 * 4 : 1;
    g.Bp = nd == 3 ? (g.B + 7) / 8 * 8 : (g.B + 31) / 32 * 32;
    g.Cp = (g.C + 31) / 32 * 32;
    g.NP = (long long)g.Ap * g.Bp * g.Cp;
  }
  auto fits = [&](int ta, int tb) {
    Geo t{};
    t.TA = ta; t.TB = tb; t.TC = 32;
    return pr_smem_bytes_for(t, st, elem) <= 220 * 1024 && ta >= st.HA && tb >= st.HB;
  };
  int TA, TB;
  int want = tune.tile_rows > 0 ? tune.tile_rows : (nd == 2 ? 32 : 8);
  int tbmax = nd == 2 ? 32 : 8;
  TB = 1;
  while (TB * 2 <= std::min(want, tbmax)) TB *= 2;
  if (nd == 2) {
    TA = 1;
    while (TB > 1 && !fits(TA, TB)) TB /= 2;
  } else {
    TA = 4;
    while (TA > 1 && !fits(TA, TB)) TA /= 2;
    while (TB > 1 && !fits(TA, TB)) TB /= 2;
  }
  if (!fits(TA, TB)) throw LfError{2, "kernel too large for a shared-memory tile"};
  g.TA = TA; g.TB = TB; g.TC = 32;
  g.nta = g.Ap / TA; g.ntb = g.Bp / TB; g.ntc = g.Cp / 32;
  g.ntiles = g.nta * g.ntb * g.ntc;
}

void Engine::alloc_accumulators() {
  if (d_exc64) return;
  check(cudaMalloc(&d_exc64, g.NP * sizeof(long long)), "cudaMalloc exc");
  check(cudaMalloc(&d_cap64, (size_t)st.K * g.NP * sizeof(long long)), "cudaMalloc cap");
  check(cudaMalloc(&d_c0, sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc");
  check(cudaMalloc(&d_flag, 4 * sizeof(int)), "cudaMalloc");
  check(cudaMalloc(&d_u64, 8 * sizeof(unsigned long long)), "cudaMalloc");
  check(cudaMalloc(&d_sum, 4 * sizeof(long long)), "cudaMalloc");
  check(cudaMemsetAsync(d_exc64, 0, g.NP * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_cap64, 0, (size_t)st.K * g.NP * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_c0, 0, sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_err, 0, sizeof(int), stream), "memset");
}

void Engine::clear() {
  if (!d_exc64) return;
  check(cudaMemsetAsync(d_exc64, 0, g.NP * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_cap64, 0, (size_t)st.K * g.NP * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_c0, 0, sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_err, 0, sizeof(int), stream), "memset");
  solved = false;
}

// Records an event before (end = false) or after (end = true) a launch of
// category cat (0 push/relabel, 1 BFS, 2 closure).
void Engine::prof_mark(int cat, bool end) {
  if (!profiling) return;
  if (pev_used == pev.size()) {
    cudaEvent_t e;
    check(cudaEventCreate(&e), "cudaEventCreate");
    pev.push_back(e);
    pcat.push_back(0);
  }
  pcat[pev_used] = end ? -1 : cat;
  check(cudaEventRecord(pev[pev_used], stream), "cudaEventRecord");
  ++pev_used;
}

void Engine::prof_collect() {
  if (!profiling) return;
  check(cudaStreamSynchronize(stream), "sync");
  for (size_t i = 0; i + 1 < pev_used; i += 2) {
    float ms = 0;
    cudaEventElapsedTime(&ms, pev[i], pev[i + 1]);
    int c = pcat[i];
    if (c >= 0 && c < 3) prof_ms[c] += ms;
  }
  pev_used = 0;
}

void Engine::sync_read(void* host, const void* dev, size_t bytes) {
  check(cudaMemcpyAsync(h_pinned, dev, bytes, cudaMemcpyDeviceToHost, stream), "memcpy D2H");
  check(cudaStreamSynchronize(stream), "stream sync");
  std::memcpy(host, h_pinned, bytes);
}

void Engine::add_energy(const int64_t* unary, const int64_t* binary, bool device_ptrs) {
  alloc_accumulators();
  const int64_t *du = unary, *db = binary;
  int64_t *tu = nullptr, *tb = nullptr;
  size_t ub = (size_t)N * 2 * sizeof(int64_t), bb = (size_t)N * (st.K / 2) * 4 * sizeof(int64_t);
  if (!device_ptrs) {
    check(cudaMallocAsync(&tu, ub, stream), "cudaMallocAsync unary");
    check(cudaMallocAsync(&tb, bb, stream), "cudaMallocAsync binary");
    check(cudaMemcpyAsync(tu, unary, ub, cudaMemcpyHostToDevice, stream), "memcpy unary");
    check(cudaMemcpyAsync(tb, binary, bb, cudaMemcpyHostToDevice, stream), "memcpy binary");
    du = tu;
    db = tb;
  }
  if (parametric)  // the reference's 2x-scaled reparametrisation (network_flow_node.hpp:420-485)
    check(counted(launch_fill_energy_pf(g, st, nd, N, du, db, d_exc64, d_cap64, d_err, stream)),
          "fill energy");
  else
    check(counted(launch_fill_energy(g, st, nd, N, du, db, d_exc64, d_cap64, d_c0, d_err, stream)),
          "fill energy");
  if (tu) cudaFreeAsync(tu, stream);
  if (tb) cudaFreeAsync(tb, stream);
  int err = 0;
  sync_read(&err, d_err, sizeof(int));
  if (err) throw LfError{3, "pairwise term is not submodular (E00 + E11 > E01 + E10)"};
  solved = false;
}

void Engine::add_caps(const int32_t* src, const int32_t* snk, const int32_t* edge) {
  alloc_accumulators();
  int32_t* buf = nullptr;
  size_t nb = (size_t)N * sizeof(int32_t), eb = (size_t)N * (st.K / 2) * sizeof(int32_t);
  check(cudaMallocAsync(&buf, 2 * nb + eb, stream), "cudaMallocAsync caps");
  int32_t *ds = nullptr, *dt = nullptr, *de = nullptr;
  if (src) { ds = buf; check(cudaMemcpyAsync(ds, src, nb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  if (snk) { dt = buf + N; check(cudaMemcpyAsync(dt, snk, nb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  if (edge) { de = buf + 2 * N; check(cudaMemcpyAsync(de, edge, eb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  check(counted(launch_fill_caps(g, st, nd, N, ds, dt, de, d_exc64, d_cap64, d_c0, d_err, parametric ? 1 : 0, stream)),
        "fill caps");
  cudaFreeAsync(buf, stream);
  int err = 0;
  sync_read(&err, d_err, sizeof(int));
  if (err) throw LfError{3, "capacities must be non-negative"};
  solved = false;
}

void Engine::prepare_working(int elem) {
  if (elem != elem_bytes) {
    free_working();
    elem_bytes = elem;
  }
  choose_geometry(elem);
  size_t T = elem;
  if (!d_res) {
    check(cudaMalloc(&d_res, (size_t)st.K * g.NP * T), "cudaMalloc res");
    check(cudaMalloc(&d_exc, g.NP * T), "cudaMalloc exc");
    check(cudaMalloc(&d_h, g.NP * sizeof(int)), "cudaMalloc h");
    check(cudaMalloc(&d_mask, g.NP * sizeof(uint64_t)), "cudaMalloc mask");
    check(cudaMalloc(&d_mark, g.NP * sizeof(int)), "cudaMalloc mark");
    for (int i = 0; i < 2; ++i) {
      check(cudaMalloc(&d_act[i], g.ntiles * sizeof(int)), "cudaMalloc act");
      check(cudaMalloc(&d_dirty[i], g.ntiles * sizeof(int)), "cudaMalloc dirty");
    }
  }
  if (elem == 4) {
    check(counted(launch_convert<int>((long long)st.K * g.NP, d_cap64, (int*)d_res, stream)), "convert");
    check(counted(launch_convert<int>(g.NP, d_exc64, (int*)d_exc, stream)), "convert");
  } else {
    check(cudaMemcpyAsync(d_res, d_cap64, (size_t)st.K * g.NP * 8, cudaMemcpyDeviceToDevice, stream), "copy");
    check(cudaMemcpyAsync(d_exc, d_exc64, g.NP * 8, cudaMemcpyDeviceToDevice, stream), "copy");
  }
}

template <typename T>
void Engine::global_relabel() {
  check(counted(launch_init_heights<T>(g, (const T*)d_exc, d_kmask, d_h, stream)), "init heights");
  check(counted(launch_mask<T>(g, st.K, (const T*)d_res, d_kmask, d_mask, stream)), "mask");
  check(cudaMemsetAsync(d_dirty[0], 0x01, g.ntiles * sizeof(int), stream), "memset");
  check(cudaMemsetAsync(d_dirty[1], 0, g.ntiles * sizeof(int), stream), "memset");
  int cur = 0;
  const long long cap = 4LL * g.ntiles + 64;
  const int chunk = tune.pass_chunk > 0 ? tune.pass_chunk : 4;
  // passes run in chunks; a pass on a converged lattice finds no dirty tile
  // and exits at once, so only the last pass's flag needs reading
  for (long long pass = 0;;) {
    if (pass > cap) throw LfError{4, "global relabel did not converge"};
    for (int c = 0; c < chunk; ++c, ++pass) {
      BFSParams p{g, st, d_h, d_mask, d_dirty[cur], d_dirty[cur ^ 1], d_flag, 64, d_u64 + 2};
      check(cudaMemsetAsync(d_flag, 0, sizeof(int), stream), "memset");
      prof_mark(1, false);
      check(counted(launch_bfs_tile(p, stream)), "bfs tile");
      prof_mark(1, true);
      ++stats.bfs_passes;
      cur ^= 1;
    }
    int changed = 0;
    sync_read(&changed, d_flag, sizeof(int));
    if (!changed) break;
  }
}

template <typename T>
void Engine::reach() {
  check(counted(launch_init_marks<T>(g.NP, (const T*)d_exc, d_mark, stream)), "init marks");
  check(cudaMemsetAsync(d_dirty[0], 0x01, g.ntiles * sizeof(int), stream), "memset");
  check(cudaMemsetAsync(d_dirty[1], 0, g.ntiles * sizeof(int), stream), "memset");
  int cur = 0;
  const long long cap = 4LL * g.ntiles + 64;
  const int chunk = tune.pass_chunk > 0 ? tune.pass_chunk : 4;
  for (long long pass = 0;;) {
    if (pass > cap) throw LfError{4, "cut-set closure did not converge"};
    for (int c = 0; c < chunk; ++c, ++pass) {
      ReachParams p{g, st, d_mark, d_mask, d_dirty[cur], d_dirty[cur ^ 1], d_flag, 256};
      check(cudaMemsetAsync(d_flag, 0, sizeof(int), stream), "memset");
      prof_mark(2, false);
      check(counted(launch_reach_tile(p, stream)), "reach tile");
      prof_mark(2, true);
      ++stats.reach_passes;
      cur ^= 1;
    }
    int changed = 0;
    sync_read(&changed, d_flag, sizeof(int));
    if (!changed) break;
  }
}

template <typename T>
void Engine::maxflow(bool compute_sets) {
  const long long hcap = std::min<long long>(g.NP + 2, (long long)kHInf - 2);
  // defaults from a sweep of (sweeps, launches, slack) on the 256^2 Full2d_4
  // and 2048^2 Full2d_8 workloads
  int M = tune.launches_per_relabel > 0 ? tune.launches_per_relabel : 4;
  int R = tune.sweeps > 0 ? tune.sweeps : 4;
  const int slack = tune.height_slack > 0 ? tune.height_slack : 16;
  const long long max_epochs = 20000;
  const auto t_start = std::chrono::steady_clock::now();
  for (long long epoch = 0;; ++epoch) {
    if (epoch > max_epochs) throw LfError{4, "push-relabel did not converge"};
    if (std::chrono::steady_clock::now() - t_start > std::chrono::seconds(300))
      throw LfError{4, "push-relabel exceeded its time limit"};
    global_relabel<T>();
    ++stats.epochs;
    check(cudaMemsetAsync(d_act[0], 0, g.ntiles * sizeof(int), stream), "memset");
    check(cudaMemsetAsync(d_act[1], 0, g.ntiles * sizeof(int), stream), "memset");
    check(cudaMemsetAsync(d_u64, 0, 2 * sizeof(unsigned long long), stream), "memset");
    check(counted(launch_active<T>(g, (const T*)d_exc, d_h, d_act[0], d_u64, stream)), "active");
    unsigned long long act_h[2] = {0, 0};
    sync_read(act_h, d_u64, sizeof(act_h));
    if (act_h[0] == 0) break;
    // heights above the BFS depth plus a slack park until the next relabel:
    // a node that climbs that far is bouncing flow inside a saturated region
    const int hmax = (int)std::min<long long>(hcap, (long long)act_h[1] + slack);
    int cur = 0;
    for (int l = 0; l < M; ++l) {
      PRParams<T> p{g, st, (T*)d_res, (T*)d_exc, d_h, d_kmask, d_act[cur], d_act[cur ^ 1],
                    d_u64 + 2, hmax, R};
      prof_mark(0, false);
      check(counted(launch_pr_tile<T>(p, stream)), "push-relabel tile");
      prof_mark(0, true);
      ++stats.pr_launches;
      cur ^= 1;
    }
  }
  if (compute_sets) reach<T>();
}

void Engine::run() {
  if (parametric) {
    engine_run_parametric(*this);
    return;
  }
  alloc_accumulators();
  stats = SolveStats();
  for (int i = 0; i < 4; ++i) prof_ms[i] = 0;
  for (int i = 0; i < 6; ++i) prof_cnt[i] = 0;
  pev_used = 0;
  // choose 32-bit working arrays when every reachable value fits
  check(cudaMemsetAsync(d_u64 + 1, 0, sizeof(unsigned long long), stream), "memset");
  check(counted(launch_range_bound(g, st, d_exc64, d_cap64, d_u64 + 1, stream)), "range bound");
  unsigned long long bound = 0;
  sync_read(&bound, d_u64 + 1, sizeof(bound));
  if (bound >= (1ULL << 62)) throw LfError{3, "capacities exceed the 63-bit range"};
  int elem = bound < (unsigned long long)INT_MAX ? 4 : 8;
  prepare_working(elem);
  check(cudaMemsetAsync(d_sum, 0, 4 * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_u64 + 2, 0, 2 * sizeof(unsigned long long), stream), "memset");
  check(cudaEventRecord(ev0, stream), "event");
  if (elem == 4) {
    check(counted(launch_sum_pos<int>(g.NP, (const int*)d_exc, d_sum + 1, stream)), "sum");
    maxflow<int>(true);
    check(counted(launch_sum_pos<int>(g.NP, (const int*)d_exc, d_sum, stream)), "sum");
  } else {
    check(counted(launch_sum_pos<long long>(g.NP, (const long long*)d_exc, d_sum + 1, stream)), "sum");
    maxflow<long long>(true);
    check(counted(launch_sum_pos<long long>(g.NP, (const long long*)d_exc, d_sum, stream)), "sum");
  }
  check(cudaEventRecord(ev1, stream), "event");
  long long sums[2];
  sync_read(sums, d_sum, sizeof(sums));
  long long c0 = 0;
  sync_read(&c0, d_c0, sizeof(c0));
  unsigned long long tp[2] = {0, 0};
  sync_read(tp, d_u64 + 2, sizeof(tp));
  stats.tiles_processed = tp[0];
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  run_time = ms * 1e-3;
  flow = sums[1] - sums[0];
  energy = c0 - sums[0];
  prof_collect();
  prof_ms[3] = ms;
  prof_cnt[0] = stats.pr_launches;
  prof_cnt[1] = (long long)stats.tiles_processed;
  prof_cnt[2] = stats.bfs_passes;
  prof_cnt[3] = stats.reach_passes;
  prof_cnt[4] = launches;
  prof_cnt[5] = (long long)tp[1];
  fetch_cuts();
  solved = true;
}

void Engine::fetch_cuts() {
  cut_min_host.assign((size_t)N, 0);
  cut_max_host.assign((size_t)N, 0);
  if (N == 0) return;
  int* buf = nullptr;
  check(cudaMallocAsync(&buf, 2 * (size_t)N * sizeof(int), stream), "cudaMallocAsync");
  check(counted(launch_extract_cuts(g, nd, N, d_mark, d_h, buf, buf + N, stream)), "extract cuts");
  check(cudaMemcpyAsync(cut_min_host.data(), buf, N * sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaMemcpyAsync(cut_max_host.data(), buf + N, N * sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  cudaFreeAsync(buf, stream);
  check(cudaStreamSynchronize(stream), "sync");
}

void Engine::get_cut(int* out, bool maximal) const {
  if (!solved) throw LfError{8, "getCut called before run"};
  if (parametric) {
    for (long long i = 0; i < N; ++i) out[i] = levels_host[i] < 0 ? 1 : 0;
    return;
  }
  const std::vector<int>& v = maximal ? cut_max_host : cut_min_host;
  std::memcpy(out, v.data(), N * sizeof(int));
}

void Engine::get_levels(int64_t* out) const {
  if (!solved || !parametric) throw LfError{8, "levels are available after a parametric run"};
  std::memcpy(out, levels_host.data(), N * sizeof(int64_t));
}

template void Engine::maxflow<int>(bool);
template void Engine::maxflow<long long>(bool);
template void Engine::global_relabel<int>();
template void Engine::global_relabel<long long>();
template void Engine::reach<int>();
template void Engine::reach<long long>();

}  // namespace lfg
