// C ABI (include/latticeflow_gpu.h) over the engine.
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/latticeflow_gpu.h"
#include "lf_batch.h"
#include "lf_serve.h"

struct lf_lattice {
  lfg::Engine* e;
};

struct lf_batch {
  lfg::Batch* b;
};

struct lf_server {
  lfg::Server* s;
};

namespace lfg {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
}  // namespace lfg

namespace {

template <class F>
int guarded(F&& f) {
  try {
    f();
    lfg::set_error("");
    return LF_OK;
  } catch (const lfg::LfError& e) {
    lfg::set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    lfg::set_error("host allocation failed");
    return LF_ERR_OOM;
  } catch (const std::exception& e) {
    lfg::set_error(e.what());
    return LF_ERR_INVALID;
  }
}

bool valid_solver(const char* s) {
  if (!s) return false;
  for (const std::string& n : lfg::solver_names())
    if (n == s) return true;
  return false;
}

size_t write_names(const std::vector<std::string>& names, char* buf, size_t len) {
  std::string all;
  for (size_t i = 0; i < names.size(); ++i) {
    if (i) all += '\n';
    all += names[i];
  }
  if (buf && len) {
    size_t n = std::min(len - 1, all.size());
    std::memcpy(buf, all.data(), n);
    buf[n] = 0;
  }
  return all.size() + 1;
}

}  // namespace

extern "C" {

const char* lf_last_error(void) { return lfg::g_last_error.c_str(); }

int lf_is_valid_solver(const char* name) { return valid_solver(name) ? 1 : 0; }
int lf_is_valid_kernel(const char* name) { return name && lfg::find_kernel(name) ? 1 : 0; }

int lf_kernel_dimension(const char* kernel) {
  const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
  return k ? k->nd : -1;
}

size_t lf_valid_kernel_names(char* buf, size_t len) {
  std::vector<std::string> names;
  for (const lfg::KernelDef& k : lfg::kernel_registry()) names.push_back(k.name);
  return write_names(names, buf, len);
}

size_t lf_valid_solver_names(char* buf, size_t len) {
  return write_names(lfg::solver_names(), buf, len);
}

int lf_kernel_info(const char* kernel, int* nd, int* deltas, double* w, int* geocut) {
  const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
  if (!k) {
    lfg::set_error(std::string("Bad Kernel or Solver Name: ") + (kernel ? kernel : "(null)"));
    return -1;
  }
  if (nd) *nd = k->nd;
  if (deltas) std::memcpy(deltas, k->delta.data(), k->delta.size() * sizeof(int));
  if (w) std::memcpy(w, k->weight.data(), k->weight.size() * sizeof(double));
  if (geocut) *geocut = k->geocut ? 1 : 0;
  return k->K;
}

int lf_create(const char* solver, const char* kernel, int nd, const size_t* dims,
              lf_lattice** out) {
  return guarded([&] {
    if (!out) throw lfg::LfError{LF_ERR_INVALID, "null output handle"};
    *out = nullptr;
    if (!valid_solver(solver) || !kernel || !lfg::find_kernel(kernel))
      throw lfg::LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                              (solver ? solver : "(null)") + ", " +
                                              (kernel ? kernel : "(null)")};
    const lfg::KernelDef* k = lfg::find_kernel(kernel);
    if (!dims || nd != k->nd)
      throw lfg::LfError{LF_ERR_SHAPE, "Kernel '" + std::string(kernel) + "' is " +
                                           std::to_string(k->nd) + "-dimensional; a shape of " +
                                           std::to_string(nd) + " dimensions was provided."};
    lf_lattice* h = new lf_lattice;
    try {
      h->e = new lfg::Engine(solver, k, nd, dims);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

void lf_destroy(lf_lattice* h) {
  if (!h) return;
  delete h->e;
  delete h;
}

int lf_n_dimensions(const lf_lattice* h) { return h ? h->e->nd : -1; }

int lf_shape(const lf_lattice* h, size_t* dims_out) {
  if (!h || !dims_out) return LF_ERR_INVALID;
  for (int i = 0; i < h->e->nd; ++i) dims_out[i] = h->e->dims[i];
  return LF_OK;
}

size_t lf_n_nodes(const lf_lattice* h) { return h ? (size_t)h->e->N : 0; }
int lf_n_filling_edges(const lf_lattice* h) { return h ? h->e->st.K / 2 : -1; }

int lf_edge_deltas(const lf_lattice* h, int* out) {
  if (!h || !out) return LF_ERR_INVALID;
  const lfg::KernelDef* k = h->e->kd;
  std::memcpy(out, k->delta.data(), (k->K / 2) * k->nd * sizeof(int));
  return LF_OK;
}

int lf_add_energy_potentials(lf_lattice* h, const int64_t* unary, const int64_t* binary) {
  return guarded([&] {
    if (!h || !unary || !binary) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    h->e->add_energy(unary, binary, false);
  });
}

int lf_add_energy_potentials_device(lf_lattice* h, const int64_t* unary, const int64_t* binary) {
  return guarded([&] {
    if (!h || !unary || !binary) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    h->e->add_energy(unary, binary, true);
  });
}

int lf_add_capacities(lf_lattice* h, const int32_t* src, const int32_t* snk, const int32_t* edge) {
  return guarded([&] {
    if (!h) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    h->e->add_caps(src, snk, edge);
  });
}

int lf_run(lf_lattice* h) {
  return guarded([&] {
    if (!h) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    h->e->run();
  });
}

double lf_run_time(const lf_lattice* h) { return h ? h->e->run_time : 0.0; }

int lf_get_cut(const lf_lattice* h, int* out) {
  return guarded([&] {
    if (!h || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    h->e->get_cut(out, false);
  });
}

int lf_get_cut_max(const lf_lattice* h, int* out) {
  return guarded([&] {
    if (!h || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    h->e->get_cut(out, true);
  });
}

int lf_get_flow(const lf_lattice* h, int64_t* flow, int64_t* energy) {
  return guarded([&] {
    if (!h) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (!h->e->solved) throw lfg::LfError{LF_ERR_STATE, "no solution yet"};
    if (flow) *flow = h->e->flow;
    if (energy) *energy = h->e->energy;
  });
}

int lf_get_levels(const lf_lattice* h, int64_t* out) {
  return guarded([&] {
    if (!h || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    h->e->get_levels(out);
  });
}

int lf_get_level_sets(const lf_lattice* h, int32_t* out) {
  return guarded([&] {
    if (!h || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    const lfg::Engine& e = *h->e;
    if (!e.solved || !e.parametric)
      throw lfg::LfError{LF_ERR_STATE, "level sets are available after a parametric run"};
    std::memcpy(out, e.level_sets_host.data(), e.N * sizeof(int32_t));
  });
}

int lf_get_stats(const lf_lattice* h, int64_t* epochs, int64_t* pr, int64_t* bfs) {
  if (!h) return LF_ERR_INVALID;
  if (epochs) *epochs = h->e->stats.epochs;
  if (pr) *pr = h->e->stats.pr_launches;
  if (bfs) *bfs = h->e->stats.bfs_passes;
  return LF_OK;
}

int lf_set_tuning(lf_lattice* h, int tile_rows, int sweeps, int launches) {
  if (!h) return LF_ERR_INVALID;
  if (tile_rows > 0) h->e->tune.tile_rows = tile_rows;
  if (sweeps > 0) h->e->tune.sweeps = sweeps;
  if (launches > 0) h->e->tune.launches_per_relabel = launches;
  return LF_OK;
}

int lf_set_param(lf_lattice* h, const char* name, int value) {
  return guarded([&] {
    if (!h || !name) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    std::string n(name);
    lfg::Tuning& t = h->e->tune;
    if (n == "tile_rows") t.tile_rows = value;
    else if (n == "local_sweeps") t.sweeps = value;
    else if (n == "launches_per_relabel") t.launches_per_relabel = value;
    else if (n == "height_slack") t.height_slack = value;
    else if (n == "pass_chunk") t.pass_chunk = value;
    else if (n == "tail_active") t.tail_active = value;
    else if (n == "max_epochs") t.max_epochs = value;
    else if (n == "tail_tree_nodes") t.tail_tree_nodes = value;
    else if (n == "pr_kernel") t.pr_kernel = value;
    else if (n == "bfs_kernel") t.bfs_kernel = value;
    else if (n == "device_loops") t.device_loops = value;
    else if (n == "fill_kernel") t.fill_kernel = value;
    else if (n == "host_stage") t.host_stage = value;
    else throw lfg::LfError{LF_ERR_INVALID, "unknown parameter " + n};
  });
}

int lf_clear(lf_lattice* h) {
  return guarded([&] {
    if (!h) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    h->e->clear();
  });
}

int lf_set_profiling(lf_lattice* h, int enable) {
  if (!h) return LF_ERR_INVALID;
  h->e->profiling = enable != 0;
  return LF_OK;
}

int lf_get_profile(const lf_lattice* h, double* ms, int64_t* counts) {
  if (!h) return LF_ERR_INVALID;
  for (int i = 0; i < 4; ++i)
    if (ms) ms[i] = h->e->prof_ms[i];
  for (int i = 0; i < 6; ++i)
    if (counts) counts[i] = h->e->prof_cnt[i];
  return LF_OK;
}

int lf_get_layout(const lf_lattice* h, int* tile, size_t* padded, int* elem) {
  if (!h) return LF_ERR_INVALID;
  const lfg::Geo& g = h->e->g;
  if (tile) { tile[0] = g.TA; tile[1] = g.TB; tile[2] = g.TC; }
  if (padded) { padded[0] = g.Ap; padded[1] = g.Bp; padded[2] = g.Cp; }
  if (elem) *elem = h->e->elem_bytes;
  return LF_OK;
}

int lf_get_stream(const lf_lattice* h, void** out) {
  if (!h || !out) return LF_ERR_INVALID;
  *out = (void*)h->e->stream;
  return LF_OK;
}

namespace {
const lfg::KernelDef* tv_kernel(const char* kernel) {
  const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
  if (!k) throw lfg::LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                                  (kernel ? kernel : "(null)")};
  if (k->nd != 2 || !k->geocut)
    throw lfg::LfError{LF_ERR_BAD_NAME, "Kernel is not valid for GeoCuts or TV Minimization."};
  return k;
}
}  // namespace

int lf_tv_2d_level_sets(const char* kernel, size_t nx, size_t ny, const double* f,
                        double lambda, double* out, int64_t* levels_out, int32_t* sets_out) {
  return guarded([&] {
    const lfg::KernelDef* k = tv_kernel(kernel);
    if (!f || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    int rc = lfg::tv_2d(k, nx, ny, f, lambda, out, levels_out, sets_out);
    if (rc) throw lfg::LfError{rc, "tv solve failed"};
  });
}

int lf_tv_2d(const char* kernel, size_t nx, size_t ny, const double* f, double lambda,
             double* out, int64_t* levels_out) {
  return lf_tv_2d_level_sets(kernel, nx, ny, f, lambda, out, levels_out, nullptr);
}

int lf_tv_2d_path_stats(const char* kernel, size_t nx, size_t ny, const double* f,
                        size_t n_lambda, const double* lambdas, double* out, int64_t* stats) {
  return guarded([&] {
    const lfg::KernelDef* k = tv_kernel(kernel);
    if (n_lambda == 0 || nx * ny == 0) return;
    if (!f || !out || !lambdas) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    int rc = lfg::tv_2d_path(k, nx, ny, f, n_lambda, lambdas, out, stats);
    if (rc) throw lfg::LfError{rc, "tv path failed"};
  });
}

int lf_tv_2d_path(const char* kernel, size_t nx, size_t ny, const double* f, size_t n_lambda,
                  const double* lambdas, double* out) {
  return lf_tv_2d_path_stats(kernel, nx, ny, f, n_lambda, lambdas, out, nullptr);
}

int lf_tv_2d_batch(const char* kernel, size_t nx, size_t ny, size_t count, const double* f,
                   size_t f_stride, const double* lambdas, double* out, int64_t* levels_out,
                   size_t max_nodes) {
  return guarded([&] {
    const lfg::KernelDef* k = tv_kernel(kernel);
    if (count == 0 || nx * ny == 0) return;
    if (!f || !out || !lambdas) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    int rc = lfg::tv_2d_batch(k, nx, ny, count, f, f_stride, lambdas, out, levels_out, max_nodes);
    if (rc) throw lfg::LfError{rc, "tv batch failed"};
  });
}

// ------------------------------------------------------------------ serving

int lf_server_create(int workers, size_t budget, lf_server** out) {
  return guarded([&] {
    if (!out) throw lfg::LfError{LF_ERR_INVALID, "null output handle"};
    *out = nullptr;
    lf_server* h = new lf_server;
    try {
      h->s = new lfg::Server(workers, budget);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

void lf_server_destroy(lf_server* s) {
  if (!s) return;
  delete s->s;
  delete s;
}

int lf_server_submit_tv(lf_server* s, const char* kernel, size_t nx, size_t ny, const double* f,
                        double lambda, int64_t* ticket) {
  return guarded([&] {
    if (!s || !f || !ticket) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
    if (!k) throw lfg::LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                                    (kernel ? kernel : "(null)")};
    *ticket = s->s->submit_tv(k, nx, ny, f, lambda);
  });
}

int lf_server_submit_cut(lf_server* s, const char* kernel, size_t nx, size_t ny,
                         const int32_t* src, const int32_t* snk, const int32_t* edge,
                         int64_t* ticket) {
  return guarded([&] {
    if (!s || !src || !snk || !edge || !ticket) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
    if (!k) throw lfg::LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                                    (kernel ? kernel : "(null)")};
    *ticket = s->s->submit_cut(k, nx, ny, src, snk, edge);
  });
}

int lf_server_wait(lf_server* s, int64_t ticket, double timeout_s, double* latency_s) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (!s->s->wait(ticket, timeout_s, latency_s))
      throw lfg::LfError{LF_ERR_STATE, "request not finished within the timeout"};
  });
}

int lf_server_get_tv(lf_server* s, int64_t ticket, double* out, int64_t* levels) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    s->s->get_tv(ticket, out, levels);
  });
}

int lf_server_get_cut(lf_server* s, int64_t ticket, int* cut, int64_t* flow, int64_t* energy) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    long long f = 0, e = 0;
    s->s->get_cut(ticket, cut, &f, &e);
    if (flow) *flow = f;
    if (energy) *energy = e;
  });
}

int lf_server_release(lf_server* s, int64_t ticket) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    s->s->release(ticket);
  });
}

int lf_server_cancel(lf_server* s, int64_t ticket) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (!s->s->cancel(ticket))
      throw lfg::LfError{LF_ERR_STATE, "request already admitted; it cannot be cancelled"};
  });
}

int lf_server_inject_alloc_failures(lf_server* s, int count) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    s->s->inject_alloc_failures(count);
  });
}

int lf_server_stats(lf_server* s, double* p50, double* p99, double* sps, int64_t* completed,
                    int64_t* max_in_flight) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    long long c = 0, m = 0;
    s->s->stats(p50, p99, sps, &c, &m);
    if (completed) *completed = c;
    if (max_in_flight) *max_in_flight = m;
  });
}

int lf_server_set_max_group(lf_server* s, int max_group) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (max_group < 1) throw lfg::LfError{LF_ERR_INVALID, "max_group must be at least 1"};
    s->s->set_max_group(max_group);
  });
}

int lf_server_group_stats(lf_server* s, int64_t* groups, int64_t* grouped) {
  return guarded([&] {
    if (!s) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    long long a = 0, b = 0;
    s->s->group_stats(&a, &b);
    if (groups) *groups = a;
    if (grouped) *grouped = b;
  });
}

// ------------------------------------------------------------ no allocation

int lf_cut_2d_noalloc(const char* kernel, size_t nx, size_t ny, const int32_t* src,
                      const int32_t* snk, const int32_t* edge, int32_t* cut, int64_t* fe,
                      void* stream) {
  return guarded([&] {
    lfg::cut_2d_noalloc(kernel, nx, ny, src, snk, edge, cut, fe, (cudaStream_t)stream);
  });
}

// ----------------------------------------------------------------- batches

int lf_batch_create(lf_batch** out) {
  return guarded([&] {
    if (!out) throw lfg::LfError{LF_ERR_INVALID, "null output handle"};
    *out = nullptr;
    lf_batch* h = new lf_batch;
    try {
      h->b = new lfg::Batch();
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

void lf_batch_destroy(lf_batch* b) {
  if (!b) return;
  delete b->b;
  delete b;
}

int lf_batch_add(lf_batch* b, const char* kernel, int nd, const size_t* dims, int* index_out) {
  return guarded([&] {
    if (!b || !dims) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    const lfg::KernelDef* k = kernel ? lfg::find_kernel(kernel) : nullptr;
    if (!k) throw lfg::LfError{LF_ERR_BAD_NAME, std::string("Bad Kernel or Solver Name: ") +
                                                    (kernel ? kernel : "(null)")};
    int i = b->b->add(k, nd, dims);
    if (index_out) *index_out = i;
  });
}

int lf_batch_size(const lf_batch* b) { return b ? int(b->b->members.size()) : -1; }

int lf_batch_add_energy_potentials(lf_batch* b, int index, const int64_t* unary,
                                   const int64_t* binary) {
  return guarded([&] {
    if (!b || !unary || !binary) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    b->b->add_energy(index, unary, binary);
  });
}

int lf_batch_add_capacities(lf_batch* b, int index, const int32_t* src, const int32_t* snk,
                            const int32_t* edge) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    b->b->add_caps(index, src, snk, edge);
  });
}

int lf_batch_add_capacities_packed(lf_batch* b, const int32_t* src, const int32_t* snk,
                                   const int32_t* edge) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    b->b->add_caps_packed(src, snk, edge);
  });
}

int lf_batch_get_cuts_packed(lf_batch* b, int* cuts_out, int maximal) {
  return guarded([&] {
    if (!b || !cuts_out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    b->b->get_cuts_packed(cuts_out, maximal != 0);
  });
}

int lf_batch_get_flows(lf_batch* b, int64_t* flows, int64_t* energies) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (!b->b->solved) throw lfg::LfError{LF_ERR_STATE, "flows are available after run"};
    for (size_t i = 0; i < b->b->members.size(); ++i) {
      if (flows) flows[i] = b->b->members[i].flow;
      if (energies) energies[i] = b->b->members[i].energy;
    }
  });
}

int lf_batch_clear(lf_batch* b) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    b->b->clear();
  });
}

int lf_batch_run(lf_batch* b) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    b->b->run();
  });
}

double lf_batch_run_time(const lf_batch* b) { return b ? b->b->run_time : 0.0; }

int lf_batch_get_cut(lf_batch* b, int index, int* out) {
  return guarded([&] {
    if (!b || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    b->b->get_cut(index, out, false);
  });
}

int lf_batch_get_cut_max(lf_batch* b, int index, int* out) {
  return guarded([&] {
    if (!b || !out) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    b->b->get_cut(index, out, true);
  });
}

int lf_batch_get_flow(lf_batch* b, int index, int64_t* flow, int64_t* energy) {
  return guarded([&] {
    if (!b) throw lfg::LfError{LF_ERR_INVALID, "null handle"};
    if (!b->b->solved) throw lfg::LfError{LF_ERR_STATE, "no solution yet"};
    lfg::Member& m = b->b->member(index);
    if (flow) *flow = m.flow;
    if (energy) *energy = m.energy;
  });
}

int lf_batch_set_param(lf_batch* b, const char* name, int value) {
  return guarded([&] {
    if (!b || !name) throw lfg::LfError{LF_ERR_INVALID, "null argument"};
    std::string n(name);
    lfg::Tuning& t = b->b->tune;
    if (n == "tile_rows") { t.tile_rows = value; b->b->relayout(); }
    else if (n == "local_sweeps") t.sweeps = value;
    else if (n == "launches_per_relabel") t.launches_per_relabel = value;
    else if (n == "height_slack") t.height_slack = value;
    else if (n == "pass_chunk") t.pass_chunk = value;
    else if (n == "tail_active") t.tail_active = value;
    else if (n == "max_epochs") t.max_epochs = value;
    else if (n == "tail_tree_nodes") t.tail_tree_nodes = value;
    else if (n == "pr_kernel") t.pr_kernel = value;
    else if (n == "bfs_kernel") t.bfs_kernel = value;
    else if (n == "device_loops") t.device_loops = value;
    else if (n == "fill_kernel") t.fill_kernel = value;
    else if (n == "host_stage") t.host_stage = value;
    else if (n == "defer_checks") b->b->defer_checks = value != 0;
    else throw lfg::LfError{LF_ERR_INVALID, "unknown parameter " + n};
  });
}

int lf_batch_get_stats(const lf_batch* b, int64_t* epochs, int64_t* pr, int64_t* bfs) {
  if (!b) return LF_ERR_INVALID;
  if (epochs) *epochs = b->b->stats.epochs;
  if (pr) *pr = b->b->stats.pr_launches;
  if (bfs) *bfs = b->b->stats.bfs_passes;
  return LF_OK;
}

}  // extern "C"
