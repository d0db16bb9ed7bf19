// Batched solves: many lattices of uneven shapes (and up to two kernel
// sizes) in one instance pool, solved together by the pool runner.  Every
// pass of the solve is a single launch over the queued tiles of ALL lattices,
// so a batch of 512 lattices costs about as many launches and host round
// trips as one lattice.  Results are per lattice and identical to a plain
// solve of that lattice (both are the unique canonical cut sets).
#include <algorithm>
#include <climits>
#include <cstring>

#include "lf_batch.h"

namespace lfg {

void Batch::check(cudaError_t e, const char* what) const {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? 5 : 6;
    throw LfError{code, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

Batch::Batch() {
  check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  check(cudaEventCreate(&ev0), "cudaEventCreate");
  check(cudaEventCreate(&ev1), "cudaEventCreate");
}

Batch::~Batch() {
  if (stream) cudaStreamSynchronize(stream);
  release();
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (stream) cudaStreamDestroy(stream);
}

void Batch::release() {
  for (void* p : {(void*)d_exc64, (void*)d_cap64, (void*)d_c0, (void*)d_err, (void*)d_u64,
                  d_res, d_exc, (void*)d_h, (void*)d_mask, (void*)d_mark})
    cudaFree(p);
  d_exc64 = d_cap64 = d_c0 = nullptr;
  d_err = nullptr;
  d_u64 = nullptr;
  d_res = d_exc = nullptr;
  d_h = d_mark = nullptr;
  d_mask = nullptr;
  laid_out = false;
  elem_bytes = 0;
}

int Batch::add(const KernelDef* kd, int nd, const size_t* dims) {
  if (laid_out) throw LfError{8, "lattices must be added before the first fill or run"};
  if (nd != kd->nd) throw LfError{2, "dimension count does not match the kernel"};
  if (nd != 2 && nd != 3) throw LfError{2, "only 2-d and 3-d lattices are supported"};
  Member m;
  m.kd = kd;
  m.nd = nd;
  m.dims.assign(dims, dims + nd);
  m.N = 1;
  for (size_t v : m.dims) {
    if (v > (size_t)INT_MAX / 2) throw LfError{2, "lattice extent too large"};
    m.N *= (long long)v;
  }
  m.st = make_stencil(kd);
  int distinct = 0;
  std::vector<int> ks;
  for (const Member& o : members) if (std::find(ks.begin(), ks.end(), o.st.K) == ks.end()) ks.push_back(o.st.K);
  if (std::find(ks.begin(), ks.end(), m.st.K) == ks.end()) ks.push_back(m.st.K);
  distinct = int(ks.size());
  if (distinct > 2) throw LfError{2, "a batch mixes at most two kernel sizes"};
  if (distinct == 2) {
    int a = std::min(ks[0], ks[1]), b = std::max(ks[0], ks[1]);
    if (!(a == 4 && b == 8)) throw LfError{2, "mixed batches pair Full2d_4 and Full2d_8 kernels"};
  }
  members.push_back(m);
  return int(members.size()) - 1;
}

// Geometry of every member for the working element size, node / residual /
// tile offsets in the pools.
void Batch::layout(int elem) {
  long long nb = 0, rb = 0;
  int tb = 0;
  for (Member& m : members) {
    lattice_geometry(m.nd, m.dims.data(), m.st, elem, tune.tile_rows, m.g);
    m.node_base = nb;
    m.res_base = rb;
    m.tile_base = tb;
    nb += m.g.NP;
    rb += (long long)m.st.K * m.g.NP;
    tb += m.g.ntiles;
  }
  NP = nb;
  RES = rb;
  tiles = tb;
}

void Batch::alloc_accumulators() {
  if (laid_out) return;
  if (members.empty()) throw LfError{8, "empty batch"};
  layout(4);
  check(cudaMalloc(&d_exc64, std::max<long long>(NP, 1) * sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_cap64, std::max<long long>(RES, 1) * sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_c0, members.size() * sizeof(long long)), "cudaMalloc");
  check(cudaMalloc(&d_err, sizeof(int)), "cudaMalloc");
  check(cudaMalloc(&d_u64, 4 * sizeof(unsigned long long)), "cudaMalloc");
  laid_out = true;
  clear();
}

void Batch::clear() {
  if (!laid_out) return;
  check(cudaMemsetAsync(d_exc64, 0, std::max<long long>(NP, 1) * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_cap64, 0, std::max<long long>(RES, 1) * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_c0, 0, members.size() * sizeof(long long), stream), "memset");
  check(cudaMemsetAsync(d_err, 0, sizeof(int), stream), "memset");
  solved = false;
}

void Batch::check_err(const char* msg) {
  int err = 0;
  check(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  err = h_err;
  if (err) throw LfError{3, msg};
}

void Batch::add_caps(int i, const int32_t* src, const int32_t* snk, const int32_t* edge) {
  alloc_accumulators();
  Member& m = member(i);
  size_t nb = (size_t)m.N * sizeof(int32_t), eb = (size_t)m.N * (m.st.K / 2) * sizeof(int32_t);
  DevBuf<int32_t> stage;
  stage.alloc((2 * nb + eb) / sizeof(int32_t), stream);
  int32_t* buf = stage.p;
  int32_t *ds = nullptr, *dt = nullptr, *de = nullptr;
  if (src) { ds = buf; check(cudaMemcpyAsync(ds, src, nb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  if (snk) { dt = buf + m.N; check(cudaMemcpyAsync(dt, snk, nb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  if (edge) { de = buf + 2 * m.N; check(cudaMemcpyAsync(de, edge, eb, cudaMemcpyHostToDevice, stream), "memcpy"); }
  check(launch_fill_caps(m.g, m.st, m.nd, m.N, ds, dt, de, d_exc64 + m.node_base,
                         d_cap64 + m.res_base, d_c0 + i, d_err, 0, stream), "fill caps");
  solved = false;
  if (!defer_checks) check_err("capacities must be non-negative");
}

// Every lattice's capacities from three packed host arrays (lattices back to
// back in index order): one copy per array, then the fill kernels.
void Batch::add_caps_packed(const int32_t* src, const int32_t* snk, const int32_t* edge) {
  alloc_accumulators();
  long long nodes = 0, edges = 0;
  for (const Member& m : members) {
    nodes += m.N;
    edges += m.N * (m.st.K / 2);
  }
  // pinned caller arrays are read in place by the fill kernels (the transfer
  // overlaps the fills); pageable ones are copied to a staging buffer first
  DevBuf<int32_t> stage;
  const int32_t* ms = (const int32_t*)mapped_host_ptr(src);
  const int32_t* mt = (const int32_t*)mapped_host_ptr(snk);
  const int32_t* me = (const int32_t*)mapped_host_ptr(edge);
  if ((src && !ms) || (snk && !mt) || (edge && !me)) stage.alloc(size_t(2 * nodes + edges) + 1, stream);
  const int32_t* ds = nullptr;
  const int32_t* dt = nullptr;
  const int32_t* de = nullptr;
  if (src) {
    ds = ms;
    if (!ds) {
      check(cudaMemcpyAsync(stage.p, src, nodes * 4, cudaMemcpyHostToDevice, stream), "memcpy");
      ds = stage.p;
    }
  }
  if (snk) {
    dt = mt;
    if (!dt) {
      check(cudaMemcpyAsync(stage.p + nodes, snk, nodes * 4, cudaMemcpyHostToDevice, stream), "memcpy");
      dt = stage.p + nodes;
    }
  }
  if (edge) {
    de = me;
    if (!de) {
      check(cudaMemcpyAsync(stage.p + 2 * nodes, edge, edges * 4, cudaMemcpyHostToDevice, stream),
            "memcpy");
      de = stage.p + 2 * nodes;
    }
  }
  long long no = 0, eo = 0;
  for (size_t i = 0; i < members.size(); ++i) {
    Member& m = members[i];
    check(launch_fill_caps(m.g, m.st, m.nd, m.N, ds ? ds + no : nullptr, dt ? dt + no : nullptr,
                           de ? de + eo : nullptr, d_exc64 + m.node_base, d_cap64 + m.res_base,
                           d_c0 + i, d_err, 0, stream),
          "fill caps");
    no += m.N;
    eo += m.N * (m.st.K / 2);
  }
  solved = false;
  if (!defer_checks) check_err("capacities must be non-negative");
}

void Batch::add_energy(int i, const int64_t* unary, const int64_t* binary) {
  alloc_accumulators();
  Member& m = member(i);
  size_t ub = (size_t)m.N * 2 * sizeof(int64_t), bb = (size_t)m.N * (m.st.K / 2) * 4 * sizeof(int64_t);
  DevBuf<int64_t> stage;
  stage.alloc((ub + bb) / sizeof(int64_t), stream);
  int64_t* buf = stage.p;
  check(cudaMemcpyAsync(buf, unary, ub, cudaMemcpyHostToDevice, stream), "memcpy");
  check(cudaMemcpyAsync(buf + 2 * m.N, binary, bb, cudaMemcpyHostToDevice, stream), "memcpy");
  check(launch_fill_energy(m.g, m.st, m.nd, m.N, buf, buf + 2 * m.N, d_exc64 + m.node_base,
                           d_cap64 + m.res_base, d_c0 + i, d_err, tune.fill_kernel, stream), "fill energy");
  solved = false;
  if (!defer_checks) check_err("pairwise term is not submodular (E00 + E11 > E01 + E10)");
}

Member& Batch::member(int i) {
  if (i < 0 || i >= (int)members.size()) throw LfError{7, "lattice index out of range"};
  return members[i];
}

void Batch::run() {
  alloc_accumulators();
  if (defer_checks) check_err("invalid energies or capacities in the batch");
  stats = SolveStats();
  // 32-bit working arrays when every member fits
  check(cudaMemsetAsync(d_u64, 0, sizeof(unsigned long long), stream), "memset");
  for (Member& m : members)
    check(launch_range_bound(m.g, m.st, d_exc64 + m.node_base, d_cap64 + m.res_base, d_u64, stream),
          "range bound");
  unsigned long long bound = 0;
  check(cudaMemcpyAsync(&h_bound, d_u64, sizeof(h_bound), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  bound = h_bound;
  if (bound >= (1ULL << 62)) throw LfError{3, "capacities exceed the 63-bit range"};
  const int elem = bound < (unsigned long long)INT_MAX ? 4 : 8;
  if (elem != elem_bytes) {
    // working arrays (the accumulator layout is fixed by the 32-bit tiles;
    // 64-bit tiles of the kernels batched here keep the same padding)
    for (void* p : {d_res, d_exc, (void*)d_h, (void*)d_mask, (void*)d_mark}) cudaFree(p);
    d_res = d_exc = nullptr;
    check(cudaMalloc(&d_res, std::max<long long>(RES, 1) * elem), "cudaMalloc res");
    check(cudaMalloc(&d_exc, std::max<long long>(NP, 1) * elem), "cudaMalloc exc");
    check(cudaMalloc(&d_h, std::max<long long>(NP, 1) * sizeof(int)), "cudaMalloc h");
    check(cudaMalloc(&d_mask, std::max<long long>(NP, 1) * sizeof(uint64_t)), "cudaMalloc mask");
    check(cudaMalloc(&d_mark, std::max<long long>(NP, 1) * sizeof(int)), "cudaMalloc mark");
    elem_bytes = elem;
    runner_ready = false;
  }
  if (!runner_ready) {
    long long np0 = NP;
    layout(elem);
    if (NP != np0) throw LfError{2, "64-bit tiles change the batch layout"};
    std::vector<InstDesc> insts(members.size());
    for (size_t i = 0; i < members.size(); ++i) {
      InstDesc& I = insts[i];
      I = InstDesc{};
      I.g = members[i].g;
      I.st = members[i].st;
      I.node_base = members[i].node_base;
      I.res_base = members[i].res_base;
      I.plane = members[i].g.NP;
      I.tile_base = members[i].tile_base;
      I.hmax = kHInf - 2;
      I.active = 1;
    }
    runner.setup(insts, stream);
    runner_ready = true;
  }
  if (elem == 4) {
    check(launch_convert<int>(RES, d_cap64, (int*)d_res, stream), "convert");
    check(launch_convert<int>(NP, d_exc64, (int*)d_exc, stream), "convert");
  } else {
    check(cudaMemcpyAsync(d_res, d_cap64, RES * 8, cudaMemcpyDeviceToDevice, stream), "copy");
    check(cudaMemcpyAsync(d_exc, d_exc64, NP * 8, cudaMemcpyDeviceToDevice, stream), "copy");
  }
  runner.tune = tune;
  runner.hooks = nullptr;
  const size_t n = members.size();
  std::vector<long long> supply(n), stuck(n), c0(n);
  check(cudaEventRecord(ev0, stream), "event");
  if (elem == 4) {
    runner.stuck_excess<int>((const int*)d_exc, supply.data());
    runner.maxflow<int>((int*)d_res, (int*)d_exc, d_h, d_mask, nullptr, d_mark, stats, true);
    runner.stuck_excess<int>((const int*)d_exc, stuck.data());
  } else {
    runner.stuck_excess<long long>((const long long*)d_exc, supply.data());
    runner.maxflow<long long>((long long*)d_res, (long long*)d_exc, d_h, d_mask, nullptr, d_mark,
                              stats, true);
    runner.stuck_excess<long long>((const long long*)d_exc, stuck.data());
  }
  check(cudaEventRecord(ev1, stream), "event");
  check(cudaMemcpyAsync(c0.data(), d_c0, n * sizeof(long long), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  run_time = ms * 1e-3;
  for (size_t i = 0; i < n; ++i) {
    members[i].flow = supply[i] - stuck[i];
    members[i].energy = c0[i] - stuck[i];
  }
  solved = true;
  cuts_fetched = false;
}

void Batch::fetch_cuts() {
  if (cuts_fetched) return;
  long long total = 0;
  for (Member& m : members) total += m.N;
  DevBuf<int> stage;
  stage.alloc(2 * std::max<long long>(total, 1), stream);
  int* buf = stage.p;
  long long off = 0;
  for (Member& m : members) {
    check(launch_extract_cuts(m.g, m.nd, m.N, d_mark + m.node_base, d_h + m.node_base, buf + off,
                              buf + total + off, stream), "extract cuts");
    off += m.N;
  }
  host_cuts.resize(2 * total);
  check(cudaMemcpyAsync(host_cuts.data(), buf, 2 * total * sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  off = 0;
  for (Member& m : members) {
    m.cut_off = off;
    off += m.N;
  }
  cut_total = total;
  cuts_fetched = true;
}

// Every lattice's cut, back to back in index order.
// The requested set only, extracted on the device and copied straight into
// the caller's buffer (pinned memory makes it one DMA).
void Batch::get_cuts_packed(int* out, bool maximal) {
  if (!solved) throw LfError{8, "getCut called before run"};
  if (cuts_fetched) {
    std::memcpy(out, host_cuts.data() + (maximal ? cut_total : 0), cut_total * sizeof(int));
    return;
  }
  long long total = 0;
  for (Member& m : members) total += m.N;
  DevBuf<int> stage;
  stage.alloc(std::max<long long>(total, 1), stream);
  long long off = 0;
  for (Member& m : members) {
    check(launch_extract_cuts(m.g, m.nd, m.N, d_mark + m.node_base, d_h + m.node_base,
                              maximal ? nullptr : stage.p + off, maximal ? stage.p + off : nullptr,
                              stream),
          "extract cuts");
    off += m.N;
  }
  check(cudaMemcpyAsync(out, stage.p, total * sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
}

void Batch::get_cut(int i, int* out, bool maximal) {
  if (!solved) throw LfError{8, "getCut called before run"};
  Member& m = member(i);
  fetch_cuts();
  const int* src = host_cuts.data() + (maximal ? cut_total : 0) + m.cut_off;
  std::memcpy(out, src, m.N * sizeof(int));
}

}  // namespace lfg
