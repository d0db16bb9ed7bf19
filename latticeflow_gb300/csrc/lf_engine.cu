// Host orchestration of one lattice solve.
//
// run() = reference LatticeEnergyBase::run + PRFlow::run
// (energy_minimization/energy_base.hpp:137-148, network_flow/push_relabel.hpp:1303-1354):
// the lattice is a pool of one for the pool runner (lf_pool.cu), which
// alternates global relabels (BFS from the deficit nodes; unreachable nodes
// get kHInf, the reference's flip) with push/relabel passes until no node
// with excess has a finite height.  The two canonical cut sets are then read
// off the final residual graph.
#include <algorithm>
#include <climits>
#include <cstring>

#include "lf_engine.h"

namespace lfg {

void Engine::check(cudaError_t e, const char* what) const {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? 5 : 6;
    throw LfError{code, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

Stencil make_stencil(const KernelDef* kd) {
  Stencil st{};
  const int nd = kd->nd;
  st.K = kd->K;
  // a 1-d lattice is one row of a 2-d one: its offsets run along the row
  for (int i = 0; i < st.K; ++i) {
    int a = nd == 3 ? kd->delta[i * nd + 0] : 0;
    int b = nd == 1 ? 0 : kd->delta[i * nd + (nd == 3 ? 1 : 0)];
    int c = kd->delta[i * nd + (nd == 3 ? 2 : nd - 1)];
    st.da[i] = (signed char)a;
    st.db[i] = (signed char)b;
    st.dc[i] = (signed char)c;
    st.rev[i] = (unsigned char)(i < st.K / 2 ? i + st.K / 2 : i - st.K / 2);
    st.HA = std::max(st.HA, std::abs(a));
    st.HB = std::max(st.HB, std::abs(b));
    st.HC = std::max(st.HC, std::abs(c));
  }
  return st;
}

// Padding is a multiple of the largest tile (1 x 32 x 32 in 2-d, 4 x 8 x 32
// in 3-d), so every smaller power-of-two tile also divides it; TC = 32 (one
// warp per row); the largest tile whose shared-memory footprint fits is used.
void lattice_geometry(int nd, const size_t* dims, const Stencil& st, int elem, int tile_rows,
                      Geo& g) {
  if (nd == 1) {  // one row of 1 x 32 tiles, no padding rows
    g.A = g.B = 1;
    g.C = int(dims[0]);
    g.Ap = g.Bp = 1;
    g.Cp = (g.C + 31) / 32 * 32;
    g.NP = g.Cp;
    g.TA = g.TB = 1;
    g.TC = 32;
    g.nta = g.ntb = 1;
    g.ntc = g.Cp / 32;
    g.ntiles = g.ntc;
    return;
  }
  g.A = nd == 3 ? int(dims[0]) : 1;
  g.B = int(dims[nd == 3 ? 1 : 0]);
  g.C = int(dims[nd == 3 ? 2 : 1]);
  g.Ap = nd == 3 ? (g.A + 3) / 4 * 4 : 1;
  g.Bp = nd == 3 ? (g.B + 7) / 8 * 8 : (g.B + 31) / 32 * 32;
  g.Cp = (g.C + 31) / 32 * 32;
  g.NP = (long long)g.Ap * g.Bp * g.Cp;
  auto fits = [&](int ta, int tb) {
    Geo t{};
    t.TA = ta; t.TB = tb; t.TC = 32;
    return pr_smem_bytes_for(t, st, elem) <= 220 * 1024 && ta >= st.HA && tb >= st.HB;
  };
  const int tbmax = nd == 2 ? 32 : 8;
  const int want = tile_rows > 0 ? tile_rows : tbmax;
  int TB = 1;
  while (TB * 2 <= std::min(want, tbmax)) TB *= 2;
  int TA = 1;
  if (nd == 2) {
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

Engine::Engine(const std::string& solver, const KernelDef* k, int _nd, const size_t* d)
    : solver_name(solver), kernel_name(k->name), kd(k), nd(_nd) {
  parametric = (solver == "LatticeLevelReductions" || solver == "GPULevelReductions");
  dims.assign(d, d + nd);
  N = 1;
  for (size_t v : dims) N *= (long long)v;
  if (nd < 1 || nd > 3) throw LfError{2, "only 1-d, 2-d and 3-d lattices are supported"};
  for (size_t v : dims)
    if (v > (size_t)INT_MAX / 2) throw LfError{2, "lattice extent too large"};
  st = make_stencil(kd);
  choose_geometry(4);
  check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  check(cudaEventCreate(&ev0), "cudaEventCreate");
  check(cudaEventCreate(&ev1), "cudaEventCreate");
  check(cudaMallocHost(&h_pinned, 64), "cudaMallocHost");
}

void Engine::choose_geometry(int elem) {
  lattice_geometry(nd, dims.data(), st, elem, tune.tile_rows, g);
}

void Engine::free_working() {
  cudaFree(d_res); d_res = nullptr;
  cudaFree(d_exc); d_exc = nullptr;
  cudaFree(d_h); d_h = nullptr;
  cudaFree(d_mask); d_mask = nullptr;
  cudaFree(d_mark); d_mark = nullptr;
  runner_ready = false;
}

Engine::~Engine() {
  if (stream) cudaStreamSynchronize(stream);
  for (cudaEvent_t e : pev) cudaEventDestroy(e);
  free_working();
  cudaFree(d_exc64);
  cudaFree(d_cap64);
  cudaFree(d_c0);
  cudaFree(d_err);
  cudaFree(d_u64);
  cudaFree(d_sum);
  cudaFree(d_kmask);
  cudaFree(d_cuts);
  cudaFree(d_stage);
  if (h_pinned) cudaFreeHost(h_pinned);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (stream) cudaStreamDestroy(stream);
}

void Engine::alloc_accumulators() {
  if (d_exc64) return;
  check(cudaMalloc(&d_exc64, g.NP * sizeof(long long)), "cudaMalloc exc");
  check(cudaMalloc(&d_cap64, (size_t)st.K * g.NP * sizeof(long long)), "cudaMalloc cap");
  check(cudaMalloc(&d_c0, sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc");
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
void Engine::mark(int cat, bool end) {
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

// Device address of host memory the GPU reads in place (pinned, mapped into
// the device's address space; on GB300 the reads go over NVLink-C2C), else
// null (pageable memory is copied first).
const void* mapped_host_ptr(const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void Engine::add_energy(const int64_t* unary, const int64_t* binary, bool device_ptrs) {
  alloc_accumulators();
  const int64_t *du = unary, *db = binary;
  DevBuf<int64_t> tu, tb;  // staging copies of pageable arrays
  size_t ub = (size_t)N * 2 * sizeof(int64_t), bb = (size_t)N * (st.K / 2) * 4 * sizeof(int64_t);
  // pinned caller arrays: the fill kernel reads them in place, so the
  // transfer overlaps the fill instead of preceding it
  const int64_t* mu = device_ptrs ? nullptr : (const int64_t*)mapped_host_ptr(unary);
  const int64_t* mb = device_ptrs ? nullptr : (const int64_t*)mapped_host_ptr(binary);
  // read over the host link: each table once (scatter); or staged by the
  // copy engine like pageable arrays, then filled from HBM
  const bool in_place = mu && mb && tune.host_stage != 1;
  if (in_place) {
    du = mu;
    db = mb;
    device_ptrs = true;
  } else if (mu && mb) {
    // host_stage: the copy engine moves the pinned tables into a device
    // buffer the engine keeps (no allocation per call), the fill reads HBM
    if (stage_bytes < ub + bb) {
      check(cudaStreamSynchronize(stream), "sync");
      cudaFree(d_stage);
      d_stage = nullptr;
      stage_bytes = 0;
      check(cudaMalloc(&d_stage, ub + bb), "cudaMalloc staging");
      stage_bytes = ub + bb;
    }
    int64_t* su = static_cast<int64_t*>(d_stage);
    int64_t* sb = su + ub / sizeof(int64_t);
    check(cudaMemcpyAsync(su, unary, ub, cudaMemcpyHostToDevice, stream), "memcpy unary");
    check(cudaMemcpyAsync(sb, binary, bb, cudaMemcpyHostToDevice, stream), "memcpy binary");
    du = su;
    db = sb;
    device_ptrs = true;
  }
  if (!device_ptrs) {
    tu.alloc(ub / sizeof(int64_t), stream);
    tb.alloc(bb / sizeof(int64_t), stream);
    check(cudaMemcpyAsync(tu.p, unary, ub, cudaMemcpyHostToDevice, stream), "memcpy unary");
    check(cudaMemcpyAsync(tb.p, binary, bb, cudaMemcpyHostToDevice, stream), "memcpy binary");
    du = tu.p;
    db = tb.p;
  }
  if (parametric)  // the reference's 2x-scaled reparametrisation (network_flow_node.hpp:420-485)
    check(counted(launch_fill_energy_pf(g, st, nd, N, du, db, d_exc64, d_cap64, d_err, stream)),
          "fill energy");
  else
    check(counted(launch_fill_energy(g, st, nd, N, du, db, d_exc64, d_cap64, d_c0, d_err,
                                          in_place ? 2 : tune.fill_kernel,
                                          stream)),
          "fill energy");
  int err = 0;
  sync_read(&err, d_err, sizeof(int));
  if (err) throw LfError{3, "pairwise term is not submodular (E00 + E11 > E01 + E10)"};
  solved = false;
}

void Engine::add_caps(const int32_t* src, const int32_t* snk, const int32_t* edge) {
  alloc_accumulators();
  size_t nb = (size_t)N * sizeof(int32_t), eb = (size_t)N * (st.K / 2) * sizeof(int32_t);
  DevBuf<int32_t> staging;  // staging copies of pageable arrays
  staging.alloc((2 * nb + eb) / sizeof(int32_t), stream);
  int32_t* buf = staging.p;
  int32_t *ds = nullptr, *dt = nullptr, *de = nullptr;
  // pinned caller arrays are read in place (see add_energy)
  auto in = [&](const int32_t* h, int32_t* stage, size_t bytes) -> int32_t* {
    if (!h) return nullptr;
    if (const void* m = mapped_host_ptr(h)) return (int32_t*)m;
    check(cudaMemcpyAsync(stage, h, bytes, cudaMemcpyHostToDevice, stream), "memcpy");
    return stage;
  };
  ds = in(src, buf, nb);
  dt = in(snk, buf + N, nb);
  de = in(edge, buf + 2 * N, eb);
  check(counted(launch_fill_caps(g, st, nd, N, ds, dt, de, d_exc64, d_cap64, d_c0, d_err,
                                 parametric ? 1 : 0, stream)),
        "fill caps");
  int err = 0;
  sync_read(&err, d_err, sizeof(int));
  if (err) throw LfError{3, "capacities must be non-negative"};
  solved = false;
}

// Working arrays in the chosen capacity type, converted from the int64
// accumulators, and the pool runner for this single lattice.
void Engine::prepare_working(int elem, bool convert) {
  if (elem != elem_bytes) {
    free_working();
    elem_bytes = elem;
  }
  Geo before = g;
  choose_geometry(elem);
  if (g.TA != before.TA || g.TB != before.TB) runner_ready = false;
  size_t T = elem;
  if (!d_res) {
    check(cudaMalloc(&d_res, (size_t)st.K * g.NP * T), "cudaMalloc res");
    check(cudaMalloc(&d_exc, g.NP * T), "cudaMalloc exc");
    check(cudaMalloc(&d_h, g.NP * sizeof(int)), "cudaMalloc h");
    check(cudaMalloc(&d_mask, g.NP * sizeof(uint64_t)), "cudaMalloc mask");
    check(cudaMalloc(&d_mark, g.NP * sizeof(int)), "cudaMalloc mark");
  }
  if (!runner_ready) {
    std::vector<InstDesc> insts;
    if (sub_count <= 1) {
      InstDesc I{};
      I.g = g;
      I.st = st;
      I.plane = g.NP;
      I.hmax = kHInf - 2;
      I.active = 1;
      insts.push_back(I);
    } else {
      // sub_count lattices of sub_real_rows real rows stacked along the
      // second axis every sub_rows rows: one pool instance each (own epoch
      // height cap, own finish), sharing this lattice's residual planes
      if (nd != 2 || g.Bp != (long long)sub_rows * sub_count || sub_rows % 32)
        throw LfError{2, "stacked lattices do not tile the padded rows"};
      size_t sd[2] = {(size_t)sub_real_rows, dims[1]};
      Geo gs{};
      lattice_geometry(2, sd, st, elem, tune.tile_rows, gs);
      if (gs.Bp != sub_rows || gs.Cp != g.Cp || gs.TB != g.TB || gs.TC != g.TC)
        throw LfError{2, "stacked lattice geometry mismatch"};
      for (int c = 0; c < sub_count; ++c) {
        InstDesc I{};
        I.g = gs;
        I.st = st;
        I.node_base = (long long)c * gs.NP;
        I.res_base = (long long)c * gs.NP;
        I.plane = g.NP;
        I.tile_base = c * gs.ntiles;
        I.hmax = kHInf - 2;
        I.active = 1;
        insts.push_back(I);
      }
    }
    runner.setup(insts, stream);
    runner_ready = true;
  }
  if (!convert) return;
  if (elem == 4) {
    check(counted(launch_convert<int>((long long)st.K * g.NP, d_cap64, (int*)d_res, stream)), "convert");
    check(counted(launch_convert<int>(g.NP, d_exc64, (int*)d_exc, stream)), "convert");
  } else {
    check(cudaMemcpyAsync(d_res, d_cap64, (size_t)st.K * g.NP * 8, cudaMemcpyDeviceToDevice, stream), "copy");
    check(cudaMemcpyAsync(d_exc, d_exc64, g.NP * 8, cudaMemcpyDeviceToDevice, stream), "copy");
  }
}

template <typename T>
void Engine::maxflow(bool compute_sets) {
  runner.tune = tune;
  runner.hooks = this;
  runner.maxflow<T>((T*)d_res, (T*)d_exc, d_h, d_mask, d_kmask, d_mark, stats, compute_sets);
}

void Engine::run() {
  if (parametric) {
    engine_run_parametric(*this);
    return;
  }
  alloc_accumulators();
  solved = false;  // a solve that fails leaves no result behind
  stats = SolveStats();
  for (int i = 0; i < 4; ++i) prof_ms[i] = 0;
  for (int i = 0; i < 6; ++i) prof_cnt[i] = 0;
  pev_used = 0;
  // choose 32-bit working arrays when every reachable value fits: first
  // the 32-bit copies with a loose bound in one pass; only when that bound
  // fails, the exact per-node bound (and the copies again, or 64-bit arrays)
  prepare_working(4, false);
  check(cudaMemsetAsync(d_u64 + 2, 0, 2 * sizeof(unsigned long long), stream), "memset");
  check(counted(launch_convert_bounded(g.NP, st.K, d_exc64, d_cap64, (int*)d_exc, (int*)d_res,
                                       d_u64 + 2, stream)), "convert");
  unsigned long long mx[2] = {0, 0};
  sync_read(mx, d_u64 + 2, sizeof(mx));
  const unsigned long long lim = (unsigned long long)INT_MAX;
  const bool loose_ok = mx[0] < lim && mx[1] < lim &&
                        mx[0] + 2ULL * (unsigned long long)st.K * mx[1] < lim;
  if (!loose_ok) {
    check(cudaMemsetAsync(d_u64 + 1, 0, sizeof(unsigned long long), stream), "memset");
    check(counted(launch_range_bound(g, st, d_exc64, d_cap64, d_u64 + 1, stream)), "range bound");
    unsigned long long bound = 0;
    sync_read(&bound, d_u64 + 1, sizeof(bound));
    if (bound >= (1ULL << 62)) throw LfError{3, "capacities exceed the 63-bit range"};
    prepare_working(bound < lim ? 4 : 8);
  }
  const int elem = elem_bytes;
  check(cudaMemsetAsync(d_sum, 0, 4 * sizeof(long long), stream), "memset");
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
  // flow and energy: both reads, one synchronisation
  long long* hp = reinterpret_cast<long long*>(h_pinned);
  check(cudaMemcpyAsync(hp, d_sum, 2 * sizeof(long long), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaMemcpyAsync(hp + 2, d_c0, sizeof(long long), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  const long long sums[2] = {hp[0], hp[1]};
  const long long c0 = hp[2];
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
  prof_cnt[5] = (long long)stats.bfs_tiles;
  extract_cuts();
  solved = true;
}

// Both cut sets, read off the final labels (closure marks and heights), stay
// in HBM (d_cuts, row-major); get_cut copies the requested one straight to
// the caller.
void Engine::extract_cuts() {
  if (N == 0) return;
  if (!d_cuts) check(cudaMalloc(&d_cuts, 2 * (size_t)N * sizeof(int)), "cudaMalloc cuts");
  check(counted(launch_extract_cuts(g, nd, N, d_mark, d_h, d_cuts, d_cuts + N, stream)),
        "extract cuts");
}

void Engine::get_cut(int* out, bool maximal) {
  if (!solved) throw LfError{8, "getCut called before run"};
  if (parametric) {
    for (long long i = 0; i < N; ++i) out[i] = levels_host[i] < 0 ? 1 : 0;
    return;
  }
  if (N == 0) return;
  check(cudaMemcpyAsync(out, d_cuts + (maximal ? N : 0), N * sizeof(int), cudaMemcpyDeviceToHost,
                        stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
}

void Engine::get_levels(int64_t* out) const {
  if (!solved || !parametric) throw LfError{8, "levels are available after a parametric run"};
  std::memcpy(out, levels_host.data(), N * sizeof(int64_t));
}

template void Engine::maxflow<int>(bool);
template void Engine::maxflow<long long>(bool);

}  // namespace lfg
