// Request server: TV-denoise and graph-cut requests of any size, admitted as
// they arrive, solved concurrently on one GPU.
//
//   * submit() copies the request's inputs and queues it (FIFO);
//   * a request is admitted when a worker is idle AND its device footprint
//     fits in the HBM budget still free (a request larger than the whole
//     budget runs alone);
//   * every worker owns a CUDA stream (inside its engines) and keeps the
//     engines of the shapes it has served, so admitted requests run at the
//     same time on different streams and their kernels overlap on the device;
//     a request arriving while others run is admitted as soon as a worker and
//     memory free up;
//   * small TV requests of one kernel and shape waiting together are solved
//     as one stacked problem (continuous batching): the worker that admits a
//     TV request also takes up to max_group - 1 more of the same shape from
//     the queue (a power-of-two group, so that few engine shapes are cached;
//     the stack stays within kTVStackNodes nodes, since stacked problems
//     advance in lockstep), within the HBM budget; each result equals the
//     request's own solve;
//   * latency = completion time - submission time (queueing included).
// No reference counterpart (the reference solves one request per call).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "lf_serve.h"

namespace lfg {

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0, Clock::time_point t) {
  return std::chrono::duration<double>(t - t0).count();
}

}  // namespace

// Device bytes a request needs beyond the engines already cached: an upper
// estimate from the padded node count (accumulators, working arrays, heights,
// masks, marks, section arrays of the parametric solver).
size_t request_footprint(const KernelDef* kd, size_t nx, size_t ny, bool tv) {
  const size_t np = (nx + 31) / 32 * 32 * ((ny + 31) / 32 * 32);
  const size_t K = kd->K;
  size_t per = 8 * (K + 1) + (tv ? 8 : 4) * (K + 1) + 4 + 8 + 4;
  if (tv) per += 8 + 4 + 12 * 8;
  return np * per + (size_t(1) << 20);
}

struct Server::Impl {
  struct Req {
    int64_t id = 0;
    bool tv = false;
    const KernelDef* kd = nullptr;
    size_t nx = 0, ny = 0;
    double lambda = 0;
    std::vector<double> f;
    std::vector<int32_t> src, snk, edge;
    size_t bytes = 0;
    Clock::time_point t_submit, t_start, t_end;
    bool done = false;
    int status = 0;
    std::string error;
    std::vector<double> out;
    std::vector<int64_t> levels;
    std::vector<int> cut;
    long long flow = 0, energy = 0;
  };

  struct Worker {
    std::thread th;
    std::map<std::tuple<bool, std::string, size_t, size_t, size_t>, std::unique_ptr<Engine>> engines;
  };

  size_t budget = 0, in_flight_bytes = 0;
  int max_group = 8;
  long long groups = 0, grouped = 0;
  int in_flight = 0, max_in_flight = 0;
  bool stop = false;
  int64_t next_id = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Req>> queue;
  std::unordered_map<int64_t, std::shared_ptr<Req>> reqs;
  std::vector<std::unique_ptr<Worker>> workers;
  std::vector<double> latencies;
  Clock::time_point t0 = Clock::now();
  Clock::time_point first_submit, last_end;
  bool any = false;
  int device = 0;
  int fail_allocs = 0;  // engine creations still to fail (host-side fault injection)

  bool admissible(const Req& r) const {
    if (in_flight == 0) return true;  // a request larger than the budget runs alone
    return in_flight_bytes + r.bytes <= budget;
  }

  static bool same_shape(const Req& a, const Req& b) {
    return a.tv && b.tv && a.kd == b.kd && a.nx == b.nx && a.ny == b.ny;
  }

  // With `mu` held: the front request plus, for a TV request, the queued TV
  // requests of its shape that fit the budget (power-of-two group size).
  std::vector<std::shared_ptr<Req>> take_group() {
    std::vector<std::shared_ptr<Req>> g{queue.front()};
    queue.pop_front();
    size_t bytes = g[0]->bytes;
    // stacked problems advance in lockstep generations: only small ones
    const size_t n0 = g[0]->nx * g[0]->ny;
    const int cap = int(std::min<size_t>(size_t(std::max(max_group, 1)),
                                         std::max<size_t>(kTVStackNodes / std::max<size_t>(n0, 1), 1)));
    if (g[0]->tv && cap > 1) {
      std::vector<size_t> idx;
      for (size_t i = 0; i < queue.size() && int(idx.size()) + 1 < cap; ++i) {
        if (!same_shape(*g[0], *queue[i])) continue;
        if (in_flight_bytes + bytes + queue[i]->bytes > budget) break;
        bytes += queue[i]->bytes;
        idx.push_back(i);
      }
      size_t G = 1;
      while (G * 2 <= idx.size() + 1) G *= 2;
      idx.resize(G - 1);
      for (size_t k = idx.size(); k-- > 0;) {
        g.push_back(queue[idx[k]]);
        queue.erase(queue.begin() + idx[k]);
      }
      std::reverse(g.begin() + 1, g.end());
    }
    return g;
  }

  void work(Worker* w) {
    cudaSetDevice(device);
    for (;;) {
      std::vector<std::shared_ptr<Req>> grp;
      size_t grp_bytes = 0;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || (!queue.empty() && admissible(*queue.front())); });
        if (stop && queue.empty()) return;
        if (queue.empty() || !admissible(*queue.front())) continue;
        grp = take_group();
        const auto now = Clock::now();
        for (auto& r : grp) {
          grp_bytes += r->bytes;
          r->t_start = now;
        }
        in_flight_bytes += grp_bytes;
        in_flight += int(grp.size());
        max_in_flight = std::max(max_in_flight, in_flight);
        if (grp.size() > 1) {
          ++groups;
          grouped += (long long)grp.size();
        }
      }
      if (grp.size() == 1) solve(w, *grp[0]);
      else solve_group(w, grp);
      {
        std::lock_guard<std::mutex> lk(mu);
        const auto now = Clock::now();
        for (auto& r : grp) {
          r->t_end = now;
          r->done = true;
          latencies.push_back(std::chrono::duration<double>(r->t_end - r->t_submit).count());
        }
        in_flight_bytes -= grp_bytes;
        in_flight -= int(grp.size());
        last_end = now;
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }

  // the worker's engine for `count` stacked TV problems (count 1 for a cut)
  Engine& engine_for(Worker* w, bool tv, const KernelDef* kd, size_t nx, size_t ny,
                     size_t count = 1) {
    auto key = std::make_tuple(tv, kd->name, nx, ny, count);
    auto it = w->engines.find(key);
    if (it == w->engines.end()) {
      {
        std::lock_guard<std::mutex> lk(mu);
        if (fail_allocs > 0) {
          --fail_allocs;
          throw LfError{5, "device allocation failed (injected)"};
        }
      }
      size_t dims[2] = {nx, ny};
      std::unique_ptr<Engine> e(tv ? new_tv_stack_engine(kd, nx, ny, count)
                                   : new Engine("GPUPushRelabel", kd, 2, dims));
      it = w->engines.emplace(key, std::move(e)).first;
    }
    return *it->second;
  }

  // TV requests of one shape as one stacked solve.
  void solve_group(Worker* w, std::vector<std::shared_ptr<Req>>& grp) {
    const Req& r0 = *grp[0];
    const size_t G = grp.size(), N = r0.nx * r0.ny;
    try {
      Engine& E = engine_for(w, true, r0.kd, r0.nx, r0.ny, G);
      std::vector<double> f(G * N), lam(G), out(G * N);
      std::vector<int64_t> lv(G * N);
      for (size_t p = 0; p < G; ++p) {
        std::copy(grp[p]->f.begin(), grp[p]->f.end(), f.begin() + p * N);
        lam[p] = grp[p]->lambda;
      }
      tv_2d_stack_on(E, r0.nx, r0.ny, G, f.data(), N, lam.data(), out.data(), lv.data());
      for (size_t p = 0; p < G; ++p) {
        Req& r = *grp[p];
        r.out.assign(out.begin() + p * N, out.begin() + (p + 1) * N);
        r.levels.assign(lv.begin() + p * N, lv.begin() + (p + 1) * N);
        r.status = 0;
      }
    } catch (const LfError& e) {
      for (auto& r : grp) { r->status = e.code; r->error = e.msg; }
    } catch (const std::exception& e) {
      for (auto& r : grp) { r->status = 7; r->error = e.what(); }
    }
  }

  void solve(Worker* w, Req& r) {
    try {
      Engine& E = engine_for(w, r.tv, r.kd, r.nx, r.ny);
      if (r.tv) {
        r.out.resize(r.nx * r.ny);
        r.levels.resize(r.nx * r.ny);
        tv_2d_on(E, r.f.data(), r.lambda, r.out.data(), r.levels.data());
      } else {
        E.clear();
        E.add_caps(r.src.data(), r.snk.data(), r.edge.data());
        E.run();
        r.cut.resize(r.nx * r.ny);
        E.get_cut(r.cut.data(), false);
        r.flow = E.flow;
        r.energy = E.energy;
      }
      r.status = 0;
    } catch (const LfError& e) {
      r.status = e.code;
      r.error = e.msg;
    } catch (const std::exception& e) {
      r.status = 7;
      r.error = e.what();
    }
  }

  int64_t push(std::shared_ptr<Req> r) {
    {
      std::lock_guard<std::mutex> lk(mu);
      r->id = next_id++;
      r->t_submit = Clock::now();
      if (!any) { first_submit = r->t_submit; any = true; }
      reqs[r->id] = r;
      queue.push_back(r);
    }
    cv_work.notify_all();
    return r->id;
  }
};

Server::Server(int workers, size_t budget_bytes) : impl(new Impl) {
  if (workers < 1) throw LfError{7, "a server needs at least one worker"};
  cudaGetDevice(&impl->device);
  if (budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    budget_bytes = free_b / 2;
  }
  impl->budget = budget_bytes;
  for (int i = 0; i < workers; ++i) {
    impl->workers.emplace_back(new Impl::Worker);
    Impl::Worker* w = impl->workers.back().get();
    w->th = std::thread([this, w] { impl->work(w); });
  }
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(impl->mu);
    impl->stop = true;
  }
  impl->cv_work.notify_all();
  for (auto& w : impl->workers)
    if (w->th.joinable()) w->th.join();
}

int64_t Server::submit_tv(const KernelDef* kd, size_t nx, size_t ny, const double* f,
                          double lambda) {
  if (kd->nd != 2 || !kd->geocut) throw LfError{1, "Kernel is not valid for GeoCuts or TV Minimization."};
  if (nx == 0 || ny == 0) throw LfError{2, "empty image"};
  auto r = std::make_shared<Impl::Req>();
  r->tv = true;
  r->kd = kd;
  r->nx = nx;
  r->ny = ny;
  r->lambda = lambda;
  r->f.assign(f, f + nx * ny);
  r->bytes = request_footprint(kd, nx, ny, true);
  return impl->push(r);
}

int64_t Server::submit_cut(const KernelDef* kd, size_t nx, size_t ny, const int32_t* src,
                           const int32_t* snk, const int32_t* edge) {
  if (kd->nd != 2) throw LfError{2, "the server takes 2-d lattices"};
  if (nx == 0 || ny == 0) throw LfError{2, "empty lattice"};
  auto r = std::make_shared<Impl::Req>();
  r->kd = kd;
  r->nx = nx;
  r->ny = ny;
  const size_t n = nx * ny, ne = n * (kd->K / 2);
  r->src.assign(src, src + n);
  r->snk.assign(snk, snk + n);
  r->edge.assign(edge, edge + ne);
  r->bytes = request_footprint(kd, nx, ny, false);
  return impl->push(r);
}

bool Server::wait(int64_t id, double timeout_s, double* latency_s) {
  std::unique_lock<std::mutex> lk(impl->mu);
  auto it = impl->reqs.find(id);
  if (it == impl->reqs.end()) throw LfError{7, "unknown ticket"};
  auto r = it->second;
  bool ok = impl->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                   [&] { return r->done; });
  if (!ok) return false;
  if (latency_s) *latency_s = std::chrono::duration<double>(r->t_end - r->t_submit).count();
  if (r->status) throw LfError{r->status, r->error};
  return true;
}

bool Server::cancel(int64_t id) {
  {
    std::lock_guard<std::mutex> lk(impl->mu);
    auto it = impl->reqs.find(id);
    if (it == impl->reqs.end()) throw LfError{7, "unknown ticket"};
    auto q = std::find(impl->queue.begin(), impl->queue.end(), it->second);
    if (q == impl->queue.end()) return false;  // admitted already (or finished)
    impl->queue.erase(q);
    Impl::Req& r = *it->second;
    r.t_start = r.t_end = Clock::now();
    r.status = 8;
    r.error = "request cancelled";
    r.done = true;
  }
  impl->cv_done.notify_all();
  impl->cv_work.notify_all();
  return true;
}

void Server::inject_alloc_failures(int n) {
  std::lock_guard<std::mutex> lk(impl->mu);
  impl->fail_allocs = std::max(0, n);
}

namespace {
std::shared_ptr<Server::Impl::Req> finished(Server::Impl* impl, int64_t id) {
  std::lock_guard<std::mutex> lk(impl->mu);
  auto it = impl->reqs.find(id);
  if (it == impl->reqs.end()) throw LfError{7, "unknown ticket"};
  if (!it->second->done) throw LfError{8, "request not finished"};
  if (it->second->status) throw LfError{it->second->status, it->second->error};
  return it->second;
}
}  // namespace

void Server::get_tv(int64_t id, double* out, int64_t* levels) {
  auto r = finished(impl.get(), id);
  if (!r->tv) throw LfError{8, "not a TV request"};
  if (out) std::memcpy(out, r->out.data(), r->out.size() * sizeof(double));
  if (levels) std::memcpy(levels, r->levels.data(), r->levels.size() * sizeof(int64_t));
}

void Server::get_cut(int64_t id, int* cut, long long* flow, long long* energy) {
  auto r = finished(impl.get(), id);
  if (r->tv) throw LfError{8, "not a cut request"};
  if (cut) std::memcpy(cut, r->cut.data(), r->cut.size() * sizeof(int));
  if (flow) *flow = r->flow;
  if (energy) *energy = r->energy;
}

void Server::release(int64_t id) {
  std::lock_guard<std::mutex> lk(impl->mu);
  auto it = impl->reqs.find(id);
  if (it != impl->reqs.end() && it->second->done) impl->reqs.erase(it);
}

void Server::set_max_group(int g) {
  std::lock_guard<std::mutex> lk(impl->mu);
  impl->max_group = std::max(1, g);
}

void Server::group_stats(long long* groups, long long* grouped) {
  std::lock_guard<std::mutex> lk(impl->mu);
  if (groups) *groups = impl->groups;
  if (grouped) *grouped = impl->grouped;
}

void Server::stats(double* p50_ms, double* p99_ms, double* solves_per_s, long long* completed,
                   long long* max_in_flight) {
  std::lock_guard<std::mutex> lk(impl->mu);
  std::vector<double> l = impl->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double q) {
    if (l.empty()) return 0.0;
    size_t i = std::min(l.size() - 1, size_t(q * (l.size() - 1) + 0.5));
    return 1e3 * l[i];
  };
  if (p50_ms) *p50_ms = pct(0.50);
  if (p99_ms) *p99_ms = pct(0.99);
  double span = impl->any ? std::chrono::duration<double>(impl->last_end - impl->first_submit).count() : 0;
  if (solves_per_s) *solves_per_s = span > 0 ? double(l.size()) / span : 0;
  if (completed) *completed = (long long)l.size();
  if (max_in_flight) *max_in_flight = impl->max_in_flight;
}

}  // namespace lfg
