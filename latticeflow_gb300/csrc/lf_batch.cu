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
#include "lf_tile_common.cuh"

namespace lfg {

// ------------------------------------------------ batch-wide element kernels
//
// One launch over the elements of every lattice of the batch instead of one
// launch per lattice: a thread finds its lattice by binary search over the
// lattices' first elements (a table in device memory, rebuilt when the
// layout changes), then does what the per-lattice kernel does for that
// element.

struct BatchMember {
  Geo g;
  Stencil st;
  long long node_base, res_base;  // the lattice's first node / residual word in the pools
  long long node_off, edge_off;   // its first node / filling edge in packed host arrays
  int nd;
};

// largest i in [0, nm) with begin[i] <= x (begin ascending, begin[0] = 0)
__device__ __forceinline__ int batch_member_of(const long long* begin, int nm, long long x) {
  int lo = 0, hi = nm - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (begin[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ long long batch_local_node(const BatchMember& m, long long b) {
  int a, bb, c;
  if (m.nd == 2) { a = 0; bb = int(b / m.g.C); c = int(b % m.g.C); }
  else { c = int(b % m.g.C); bb = int((b / m.g.C) % m.g.B); a = int(b / ((long long)m.g.C * m.g.B)); }
  return ((long long)a * m.g.Bp + bb) * m.g.Cp + c;
}

// k_fill_caps (capacity form, plain scale) for every lattice: thread = one
// (node, filling edge) of the packed arrays; the constant term is summed per
// warp when the whole warp serves one lattice, else per thread.
__global__ void k_fill_caps_batch(const BatchMember* M, const long long* edge_begin, int nm,
                                  long long total, const int32_t* src, const int32_t* snk,
                                  const int32_t* edge, long long* exc, long long* cap,
                                  long long* c0sum, int* err) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int i = -1;
  long long c0 = 0;
  if (tid < total) {
    i = batch_member_of(edge_begin, nm, tid);
    const BatchMember& m = M[i];
    const int Kp = m.st.K / 2;
    const long long local = tid - edge_begin[i];
    const long long b = local / Kp;
    const int e = int(local % Kp);
    int a, bb, c;
    if (m.nd == 2) { a = 0; bb = int(b / m.g.C); c = int(b % m.g.C); }
    else { c = int(b % m.g.C); bb = int((b / m.g.C) % m.g.B); a = int(b / ((long long)m.g.C * m.g.B)); }
    const long long u = ((long long)a * m.g.Bp + bb) * m.g.Cp + c;
    if (e == 0) {
      const long long sv = src ? src[m.node_off + b] : 0, tv = snk ? snk[m.node_off + b] : 0;
      if (sv < 0 || tv < 0) atomicExch(err, 1);
      if (sv - tv) atom_add(&exc[m.node_base + u], sv - tv);
      c0 += sv;
    }
    if (edge) {
      const long long w = edge[m.edge_off + b * Kp + e];
      const int na = a + m.st.da[e], nb = bb + m.st.db[e], nc = c + m.st.dc[e];
      if (w < 0) atomicExch(err, 1);
      if (w > 0 && na >= 0 && na < m.g.A && nb >= 0 && nb < m.g.B && nc >= 0 && nc < m.g.C) {
        const long long v = ((long long)na * m.g.Bp + nb) * m.g.Cp + nc;
        atom_add(&cap[m.res_base + (long long)e * m.g.NP + u], w);
        atom_add(&cap[m.res_base + (long long)m.st.rev[e] * m.g.NP + v], w);
      }
    }
  }
  const int i0 = __shfl_sync(0xffffffffu, i, 0);
  if (__all_sync(0xffffffffu, i == i0)) {
    for (int o = 16; o > 0; o >>= 1) c0 += __shfl_down_sync(0xffffffffu, c0, o);
    if ((threadIdx.x & 31) == 0 && i0 >= 0 && c0) atom_add(&c0sum[i0], c0);
  } else if (i >= 0 && c0) {
    atom_add(&c0sum[i], c0);
  }
}

// k_range_bound for every lattice: thread = one padded node of the pools
__global__ void k_range_bound_batch(const BatchMember* M, const long long* node_begin, int nm,
                                    long long NP, const long long* exc, const long long* cap,
                                    unsigned long long* out_max) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long mx = 0;
  if (gi < NP) {
    const int i = batch_member_of(node_begin, nm, gi);
    const BatchMember& m = M[i];
    const long long li = gi - m.node_base;
    const Geo& g = m.g;
    const int c = int(li % g.Cp), b = int((li / g.Cp) % g.Bp), a = int(li / ((long long)g.Cp * g.Bp));
    const long long e = exc[gi];
    unsigned long long s = (unsigned long long)(e < 0 ? -e : e);
    const long long* cp = cap + m.res_base;
    for (int k = 0; k < m.st.K; ++k) {
      s += (unsigned long long)cp[(long long)k * g.NP + li];
      const int na = a + m.st.da[k], nb = b + m.st.db[k], nc = c + m.st.dc[k];
      if (na >= 0 && na < g.Ap && nb >= 0 && nb < g.Bp && nc >= 0 && nc < g.Cp) {
        const long long v = ((long long)na * g.Bp + nb) * g.Cp + nc;
        s += (unsigned long long)cp[(long long)m.st.rev[k] * g.NP + v];
      }
    }
    mx = s;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, mx, o);
    mx = x > mx ? x : mx;
  }
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(out_max, mx);
}

// k_extract_cuts for every lattice: thread = one node of the packed output
__global__ void k_extract_cuts_batch(const BatchMember* M, const long long* out_begin, int nm,
                                     long long total, const int* mark, const int* h, int* cut_min,
                                     int* cut_max) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= total) return;
  const int i = batch_member_of(out_begin, nm, x);
  const BatchMember& m = M[i];
  const long long gi = m.node_base + batch_local_node(m, x - out_begin[i]);
  if (cut_min) cut_min[x] = mark[gi] ? 1 : 0;
  if (cut_max) cut_max[x] = h[gi] >= kHInf ? 1 : 0;
}

static inline int bblk(long long n, int t) { return int((n + t - 1) / t); }

// The lattice table of the batch-wide kernels: members, then the first
// padded node, first packed output node and first packed filling edge of
// each lattice (three arrays of nm + 1 entries).
void Batch::upload_table() {
  if (table_ok) return;
  const int nm = int(members.size());
  std::vector<BatchMember> h(nm);
  std::vector<long long> begins(3 * (size_t)(nm + 1));
  long long no = 0, eo = 0;
  for (int i = 0; i < nm; ++i) {
    const Member& m = members[i];
    BatchMember& b = h[i];
    b.g = m.g;
    b.st = m.st;
    b.node_base = m.node_base;
    b.res_base = m.res_base;
    b.node_off = no;
    b.edge_off = eo;
    b.nd = m.nd;
    begins[i] = m.node_base;
    begins[(nm + 1) + i] = no;
    begins[2 * (nm + 1) + i] = eo;
    no += m.N;
    eo += m.N * (m.st.K / 2);
  }
  begins[nm] = NP;
  begins[(nm + 1) + nm] = no;
  begins[2 * (nm + 1) + nm] = eo;
  if (!d_table) {
    check(cudaMalloc(&d_table, nm * sizeof(BatchMember)), "cudaMalloc");
    check(cudaMalloc(&d_begins, begins.size() * sizeof(long long)), "cudaMalloc");
  }
  check(cudaMemcpyAsync(d_table, h.data(), nm * sizeof(BatchMember), cudaMemcpyHostToDevice, stream),
        "memcpy");
  check(cudaMemcpyAsync(d_begins, begins.data(), begins.size() * sizeof(long long),
                        cudaMemcpyHostToDevice, stream),
        "memcpy");
  // the host vectors go away with this call: the copies finish first
  check(cudaStreamSynchronize(stream), "sync");
  table_ok = true;
}

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
                  d_res, d_exc, (void*)d_h, (void*)d_mask, (void*)d_mark, d_table,
                  (void*)d_begins, d_stage})
    cudaFree(p);
  d_stage = nullptr;
  stage_bytes = 0;
  d_table = nullptr;
  d_begins = nullptr;
  table_ok = false;
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
  table_ok = false;
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
  // pinned caller arrays are read in place by the fill kernel (host_stage 0;
  // the transfer overlaps the fill) or moved by the copy engine into a
  // staging buffer the batch keeps (host_stage 1: whole-array copies instead
  // of the fill's 4-byte reads over the host link); pageable ones are always
  // copied into that buffer first
  const bool stage_pinned = tune.host_stage == 1;
  const int32_t* ms = stage_pinned ? nullptr : (const int32_t*)mapped_host_ptr(src);
  const int32_t* mt = stage_pinned ? nullptr : (const int32_t*)mapped_host_ptr(snk);
  const int32_t* me = stage_pinned ? nullptr : (const int32_t*)mapped_host_ptr(edge);
  int32_t* stage = nullptr;
  if ((src && !ms) || (snk && !mt) || (edge && !me)) {
    const size_t want = size_t(2 * nodes + edges + 1) * sizeof(int32_t);
    if (stage_bytes < want) {
      check(cudaStreamSynchronize(stream), "sync");
      cudaFree(d_stage);
      d_stage = nullptr;
      stage_bytes = 0;
      check(cudaMalloc(&d_stage, want), "cudaMalloc staging");
      stage_bytes = want;
    }
    stage = static_cast<int32_t*>(d_stage);
  }
  const int32_t* ds = nullptr;
  const int32_t* dt = nullptr;
  const int32_t* de = nullptr;
  if (src) {
    ds = ms;
    if (!ds) {
      check(cudaMemcpyAsync(stage, src, nodes * 4, cudaMemcpyHostToDevice, stream), "memcpy");
      ds = stage;
    }
  }
  if (snk) {
    dt = mt;
    if (!dt) {
      check(cudaMemcpyAsync(stage + nodes, snk, nodes * 4, cudaMemcpyHostToDevice, stream), "memcpy");
      dt = stage + nodes;
    }
  }
  if (edge) {
    de = me;
    if (!de) {
      check(cudaMemcpyAsync(stage + 2 * nodes, edge, edges * 4, cudaMemcpyHostToDevice, stream),
            "memcpy");
      de = stage + 2 * nodes;
    }
  }
  upload_table();
  const int nm = int(members.size());
  if (edges > 0)
    k_fill_caps_batch<<<bblk(edges, 256), 256, 0, stream>>>(
        static_cast<const BatchMember*>(d_table), d_begins + 2 * (nm + 1), nm, edges, ds, dt, de,
        d_exc64, d_cap64, d_c0, d_err);
  check(cudaGetLastError(), "fill caps");
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
  upload_table();
  if (NP > 0)
    k_range_bound_batch<<<bblk(NP, 256), 256, 0, stream>>>(
        static_cast<const BatchMember*>(d_table), d_begins, int(members.size()), NP, d_exc64,
        d_cap64, d_u64);
  check(cudaGetLastError(), "range bound");
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
  upload_table();
  const int nm = int(members.size());
  if (total > 0)
    k_extract_cuts_batch<<<bblk(total, 256), 256, 0, stream>>>(
        static_cast<const BatchMember*>(d_table), d_begins + (nm + 1), nm, total, d_mark, d_h, buf,
        buf + total);
  check(cudaGetLastError(), "extract cuts");
  host_cuts.resize(2 * total);
  check(cudaMemcpyAsync(host_cuts.data(), buf, 2 * total * sizeof(int), cudaMemcpyDeviceToHost, stream), "memcpy");
  check(cudaStreamSynchronize(stream), "sync");
  long long off = 0;
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
  upload_table();
  const int nm = int(members.size());
  if (total > 0)
    k_extract_cuts_batch<<<bblk(total, 256), 256, 0, stream>>>(
        static_cast<const BatchMember*>(d_table), d_begins + (nm + 1), nm, total, d_mark, d_h,
        maximal ? nullptr : stage.p, maximal ? stage.p : nullptr);
  check(cudaGetLastError(), "extract cuts");
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
