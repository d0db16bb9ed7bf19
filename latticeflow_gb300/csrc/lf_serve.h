// Request server over the engine (see lf_serve.cpp).
#pragma once

#include <cstdint>
#include <memory>

#include "lf_engine.h"

namespace lfg {

size_t request_footprint(const KernelDef* kd, size_t nx, size_t ny, bool tv);

class Server {
 public:
  Server(int workers, size_t budget_bytes);
  ~Server();
  int64_t submit_tv(const KernelDef* kd, size_t nx, size_t ny, const double* f, double lambda);
  int64_t submit_cut(const KernelDef* kd, size_t nx, size_t ny, const int32_t* src,
                     const int32_t* snk, const int32_t* edge);
  // true when finished within timeout_s (throws the request's error if it failed)
  bool wait(int64_t id, double timeout_s, double* latency_s);
  void get_tv(int64_t id, double* out, int64_t* levels);
  void get_cut(int64_t id, int* cut, long long* flow, long long* energy);
  void release(int64_t id);
  // a request still waiting in the queue is dropped: its wait reports it
  // cancelled (LF_ERR_STATE); false once it has been admitted
  bool cancel(int64_t id);
  // host-side fault injection: the next n engine creations of the workers
  // fail as a failed device allocation would (the request gets LF_ERR_OOM)
  void inject_alloc_failures(int n);
  // largest group of same-shape TV requests solved together (1 = none)
  void set_max_group(int g);
  void group_stats(long long* groups, long long* grouped);
  void stats(double* p50_ms, double* p99_ms, double* solves_per_s, long long* completed,
             long long* max_in_flight);

  struct Impl;
  std::unique_ptr<Impl> impl;
};

}  // namespace lfg
